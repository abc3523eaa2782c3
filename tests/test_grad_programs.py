"""The fused gradient kernel's generated programs (four weighted contraction grids, six
HRR sub-programs) emulated on the CPU against the straight-line generated code applied to
raised (l+1, coefficients times 2 alpha) and lowered (l-1) shells."""
import os
import sys

import numpy as np
import pytest

import oracle
from conftest import ROOT
from gaussium_gb300.basis import ShellBasis
import hostcheck

sys.path.insert(0, os.path.join(ROOT, "gaussium_gb300", "csrc"))
import gen_eri  # noqa: E402
import gen_grad  # noqa: E402


def _shell(rng, l, k, centre):
    return dict(l=l, centre=centre, expo=np.exp(rng.uniform(np.log(0.1), np.log(20), k)),
                coef=rng.standard_normal(k))


def emulate(cls, pr, pd, alpha_bra, alpha_ket):
    p = gen_grad.grad_program(cls)
    L = p["L"]
    B, K = pr[0], pr[1]
    acc = np.zeros(p["nacc"])
    for i in range(B["nprim"]):
        P = pd[B["prim_off"] + i]
        for j in range(K["nprim"]):
            Q = pd[K["prim_off"] + j]
            pq = P[0] + Q[0]
            PQ = Q[2:5] - P[2:5]
            wq, wp = Q[0] / pq, P[0] / pq
            t = P[0] * wq * PQ @ PQ
            F = np.array([oracle.boys_exact(m, t) for m in range(L + 1)]) * P[8] * Q[8] / np.sqrt(pq)
            c = np.zeros(36)
            c[0:3] = P[5:8]; c[3:6] = wq * PQ; c[6:9] = Q[5:8]; c[9:12] = -wp * PQ
            for k in range(1, 5):
                c[11 + k] = k * P[1]; c[15 + k] = -k * wq * P[1]; c[19 + k] = k * Q[1]
                c[23 + k] = -k * wp * Q[1]; c[27 + k] = k * 0.5 / pq
            a, gmm = alpha_bra[i // K["nprim"]] if False else P[9], Q[9]
            c[32], c[33], c[34], c[35] = 2 * P[9], 2 * (P[0] - P[9]), 2 * Q[9], 5 * 0.5 / pq
            node = np.zeros(p["nvslot"])
            node[:L + 1] = F
            rec = p["vrec"]
            for noff, _, cnt, nt, lv, sync in p["vseg"]:
                new = {}
                for n in range(cnt):
                    w = rec[8 * (noff + n): 8 * (noff + n) + 8]
                    new[w[0] & 0xffff] = sum(c[w[1 + tt] >> 16] * node[w[1 + tt] & 0xffff] for tt in range(nt))
                for kk, val in new.items():
                    node[kk] = val
            for q in range(p["nacc"]):
                wgt = 1.0 if p["acc_kind"][q] == 0 else c[31 + p["acc_kind"][q]]
                acc[q] += wgt * node[p["acc_slot"][q]]
    H = np.zeros(p["hsize"])
    H[np.array(p["acc_pos"])] = acc
    dv = [*B["AB"], *K["AB"]]
    for lv in range(len(p["hlev"]) - 1):
        new = {}
        for e in range(p["hlev"][lv], p["hlev"][lv + 1]):
            out, x, y, d = p["hops"][e]
            new[out] = H[x] + dv[d] * H[y]
        for kk, val in new.items():
            H[kk] = val
    return [None if o is None else H[np.array(o)] for o in p["outs"]]


@pytest.mark.parametrize("cls", gen_eri.canonical_classes(1))
def test_grad_program_blocks(cls):
    rng = np.random.default_rng(sum(cls) + 11)
    cents = rng.uniform(-1.0, 1.0, size=(4, 3))
    shells = [_shell(rng, l, int(rng.integers(1, 3)), cents[i]) for i, l in enumerate(cls)]
    sb = ShellBasis.from_shell_dicts(shells)
    pr, pd, _ = hostcheck.make_pairs(sb, [(0, 1), (2, 3)])
    pd[:, 9] = [sb.expo[sb.prim_off[0] + i // sb.nprim[1]] for i in range(sb.nprim[0] * sb.nprim[1])] + \
        [sb.expo[sb.prim_off[2] + i // sb.nprim[3]] for i in range(sb.nprim[2] * sb.nprim[3])]
    outs = emulate(cls, pr, pd, None, None)
    # reference blocks from the generated thread code on modified shells
    for which, (cen, raised) in enumerate([(0, True), (1, True), (2, True), (0, False), (1, False), (2, False)]):
        if outs[which] is None:
            continue
        mod = []
        for s in range(4):
            k0, k1 = sb.prim_off[s], sb.prim_off[s + 1]
            l = int(sb.l[s])
            cf = sb.coef[k0:k1].copy()
            if s == cen:
                l = l + 1 if raised else l - 1
                if raised:
                    cf = cf * 2 * sb.expo[k0:k1]
            mod.append((l, sb.centre[s], sb.expo[k0:k1], cf))
        msb = ShellBasis([m[0] for m in mod], np.array([m[1] for m in mod]),
                         np.concatenate([[0], np.cumsum([len(m[2]) for m in mod])]),
                         np.concatenate([m[2] for m in mod]), np.concatenate([m[3] for m in mod]),
                         np.ones((4, 6)))
        blk, canon = hostcheck.canonical_block(msb, (0, 1, 2, 3), 64)
        inv = np.argsort(canon)                 # canonical position of original shell k
        ref = blk.transpose(inv).ravel()
        assert np.max(np.abs(outs[which] - ref)) <= 1e-12 * max(1.0, np.max(np.abs(ref))), which


@pytest.mark.parametrize("cls", [(2, 0, 0, 0), (2, 1, 1, 0), (2, 2, 1, 0), (2, 1, 2, 1),
                                 (2, 2, 2, 2)])
def test_grad_program_blocks_d_shells(cls):
    """d classes, whose raised shells are f: the six derivative blocks from the program
    against the oracle's Obara-Saika integrals of the modified shells (any l)."""
    rng = np.random.default_rng(sum(cls) + 41)
    cents = rng.uniform(-1.0, 1.0, size=(4, 3))
    shells = [_shell(rng, l, int(rng.integers(1, 3)), cents[i]) for i, l in enumerate(cls)]
    sb = ShellBasis.from_shell_dicts(shells)
    pr, pd, _ = hostcheck.make_pairs(sb, [(0, 1), (2, 3)])
    pd[:, 9] = [sb.expo[sb.prim_off[0] + i // sb.nprim[1]] for i in range(sb.nprim[0] * sb.nprim[1])] + \
        [sb.expo[sb.prim_off[2] + i // sb.nprim[3]] for i in range(sb.nprim[2] * sb.nprim[3])]
    outs = emulate(cls, pr, pd, None, None)
    for which, (cen, raised) in enumerate([(0, True), (1, True), (2, True), (0, False), (1, False), (2, False)]):
        if outs[which] is None:
            continue
        centre, lmn, prims, first = [], [], [], []
        for s in range(4):
            k0, k1 = sb.prim_off[s], sb.prim_off[s + 1]
            l = int(sb.l[s])
            cf = sb.coef[k0:k1].copy()
            if s == cen:
                l = l + 1 if raised else l - 1
                if raised:
                    cf = cf * 2 * sb.expo[k0:k1]
            first.append(len(centre))
            for comp in gen_eri.cart(l):
                centre.append(sb.centre[s]); lmn.append(comp)
                prims.append(list(zip(cf, sb.expo[k0:k1], np.ones(k1 - k0))))
        table = oracle.FunctionTable(np.array(centre), np.array(lmn), np.ones(len(centre)), prims)
        n = [len(gen_eri.cart(sum(lmn[first[s]]))) for s in range(4)]
        fq = np.stack(np.meshgrid(*[first[s] + np.arange(n[s]) for s in range(4)], indexing="ij"),
                      -1).reshape(-1, 4)
        ref = oracle.eri_functions(table, fq, boys_mode=1)
        assert np.max(np.abs(outs[which] - ref)) <= 1e-12 * max(1.0, np.max(np.abs(ref))), which


def _body(code, fn):
    """Statements of a generated thread-code function, as Python (they are plain
    assignments over arrays with fma)."""
    text = code.split(f"void {fn}(")[1]
    text = text[text.index("{") + 1:]
    out = []
    for ln in text.split("\n")[1:]:
        if ln.startswith("  }"):
            break
        ln = ln.strip()
        if ln and not ln.startswith("double "):
            out.append(ln.rstrip(";"))
    return compile("\n".join(out), fn, "exec")


def _fma(a, b, c):
    return a * b + c


@pytest.mark.parametrize("cls", [c for c in gen_eri.canonical_classes(2) if sum(c) <= gen_grad.THREAD_LMAX])
def test_thread_gradient_code_matches_program(cls):
    rng = np.random.default_rng(sum(cls) + 29)
    cents = rng.uniform(-1.0, 1.0, size=(4, 3))
    shells = [_shell(rng, l, int(rng.integers(1, 3)), cents[i]) for i, l in enumerate(cls)]
    sb = ShellBasis.from_shell_dicts(shells)
    pr, pd, _ = hostcheck.make_pairs(sb, [(0, 1), (2, 3)])
    pd[:, 9] = [sb.expo[sb.prim_off[0] + i // sb.nprim[1]] for i in range(sb.nprim[0] * sb.nprim[1])] + \
        [sb.expo[sb.prim_off[2] + i // sb.nprim[3]] for i in range(sb.nprim[2] * sb.nprim[3])]
    outs = emulate(cls, pr, pd, None, None)
    p = gen_grad.grad_program(cls)
    code = gen_grad.emit_grad_thread(cls, p)
    prim, hrr, contract = _body(code, "prim"), _body(code, "hrr"), _body(code, "contract")
    L = p["L"]
    B, K = pr[0], pr[1]
    H = np.zeros(p["hsize"])
    for i in range(B["nprim"]):
        P = pd[B["prim_off"] + i]
        for j in range(K["nprim"]):
            Q = pd[K["prim_off"] + j]
            pq = P[0] + Q[0]
            PQ = Q[2:5] - P[2:5]
            wq, wp = Q[0] / pq, P[0] / pq
            t = P[0] * wq * PQ @ PQ
            c = np.zeros(36)
            c[0:3] = P[5:8]; c[3:6] = wq * PQ; c[6:9] = Q[5:8]; c[9:12] = -wp * PQ
            for k in range(1, 5):
                c[11 + k] = k * P[1]; c[15 + k] = -k * wq * P[1]; c[19 + k] = k * Q[1]
                c[23 + k] = -k * wp * Q[1]; c[27 + k] = k * 0.5 / pq
            c[32], c[33], c[34] = 2 * P[9], 2 * (P[0] - P[9]), 2 * Q[9]
            n = np.zeros(p["nvslot"])
            n[:L + 1] = np.array([oracle.boys_exact(m, t) for m in range(L + 1)]) * P[8] * Q[8] / np.sqrt(pq)
            exec(prim, {"fma": _fma, "c": c, "n": n, "H": H})
    exec(hrr, {"fma": _fma, "H": H, "dv": [*B["AB"], *K["AB"]]})
    for which, o in enumerate(p["outs"]):
        if o is not None:
            assert np.max(np.abs(H[np.array(o)] - outs[which])) <= 1e-13 * max(1.0, np.max(np.abs(outs[which])))
    # contraction against a direct loop over the blocks
    nc = [gen_eri.ncart(x) for x in cls]
    dens = {k: rng.standard_normal(nc[a] * nc[b]) for k, (a, b) in
            {"pab": (0, 1), "pcd": (2, 3), "pac": (0, 2), "pbd": (1, 3), "pad": (0, 3), "pbc": (1, 2)}.items()}
    cs = [rng.uniform(0.5, 2.0, nc[k]) for k in range(4)]
    g = np.zeros(9)
    exec(contract, {"fma": _fma, "H": H, "w": 0.5, **dens, "cs0": cs[0], "cs1": cs[1], "cs2": cs[2],
                    "cs3": cs[3], "g": g})
    ref = np.zeros(9)
    for ia in range(nc[0]):
        for ib in range(nc[1]):
            for ic in range(nc[2]):
                for idd in range(nc[3]):
                    idx = [ia, ib, ic, idd]
                    gam = 0.5 * (0.5 * dens["pab"][ia * nc[1] + ib] * dens["pcd"][ic * nc[3] + idd] -
                                 0.125 * (dens["pac"][ia * nc[2] + ic] * dens["pbd"][ib * nc[3] + idd] +
                                          dens["pad"][ia * nc[3] + idd] * dens["pbc"][ib * nc[2] + ic]))
                    for cen in range(3):
                        ex = gen_eri.cart(cls[cen])[idx[cen]]
                        for x in range(3):
                            up = list(ex); up[x] += 1
                            ii = list(idx); nn = list(nc)
                            ii[cen] = gen_eri.cart(cls[cen] + 1).index(tuple(up)); nn[cen] = gen_eri.ncart(cls[cen] + 1)
                            v = outs[cen][((ii[0] * nn[1] + ii[1]) * nn[2] + ii[2]) * nn[3] + ii[3]]
                            if ex[x] > 0:
                                dn = list(ex); dn[x] -= 1
                                jj = list(idx); mm = list(nc)
                                jj[cen] = gen_eri.cart(cls[cen] - 1).index(tuple(dn)); mm[cen] = gen_eri.ncart(cls[cen] - 1)
                                v -= ex[x] * outs[3 + cen][((jj[0] * mm[1] + jj[1]) * mm[2] + jj[2]) * mm[3] + jj[3]]
                            scale = cs[0][ia] * cs[1][ib] * cs[2][ic] * cs[3][idd]
                            ref[3 * cen + x] += gam * scale * v
    assert np.max(np.abs(g - ref)) <= 1e-12 * max(1.0, np.max(np.abs(ref)))
