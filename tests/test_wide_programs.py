"""The warp-cooperative kernels' generated programs (VRR node levels, HRR element
operations on the planned shared buffer, output slots) emulated on the CPU and compared
with the straight-line generated code, for every class that uses them."""
import os
import sys

import numpy as np
import pytest

import oracle
from conftest import synthetic_shells, golden, ROOT
from gaussium_gb300.basis import ShellBasis
import hostcheck

sys.path.insert(0, os.path.join(ROOT, "gaussium_gb300", "csrc"))
import gen_eri  # noqa: E402


def emulate(cls, pr, pd, bra, ket, grouped=False):
    """Run the warp program of `cls` (the grouped form's with ``grouped``) for quartet
    (bra|ket) with numpy.  Writes of a synchronisation step become visible only at the
    next step, as on the GPU, where the lanes of one step run in no fixed order."""
    p = gen_eri.wide_program(cls)
    if grouped:
        pv = gen_eri.vrr_group(cls)[1]
        p = dict(p, vrec=pv["vrec"], vseg=pv["vseg"], vtgt=pv["vtgt"], nvslot=pv["nvslot"])
    L = p["L"]
    B, K = pr[bra], pr[ket]
    acc = np.zeros(p["nacc"])
    for i in range(B["nprim"]):
        P = pd[B["prim_off"] + i]
        for j in range(K["nprim"]):
            Q = pd[K["prim_off"] + j]
            pq = P[0] + Q[0]
            PQ = Q[2:5] - P[2:5]
            wq, wp = Q[0] / pq, P[0] / pq
            t = P[0] * wq * PQ @ PQ
            pref = P[8] * Q[8] / np.sqrt(pq)
            F = np.array([oracle.boys_exact(m, t) for m in range(L + 1)]) * pref
            c = np.zeros(32)
            c[0:3] = P[5:8]; c[3:6] = wq * PQ; c[6:9] = Q[5:8]; c[9:12] = -wp * PQ
            i2p, i2q = P[1], Q[1]
            for k in range(1, 5):
                c[11 + k] = k * i2p; c[15 + k] = -k * wq * i2p; c[19 + k] = k * i2q
                c[23 + k] = -k * wp * i2q; c[27 + k] = k * 0.5 / pq
            c[gen_eri.ZERO_COEF] = 0.0          # padding terms of short nodes in a wave
            node = np.zeros(p["nvslot"])
            node[:L + 1] = F
            rec = p["vrec"]
            new, reads = {}, set()
            for noff, _, cnt, nt_max, lv, sync in p["vseg"]:
                if sync:
                    # no lane of a step may overwrite a slot another lane of it still reads
                    assert not (reads & set(new))
                    for k, val in new.items():
                        node[k] = val
                    new, reads = {}, set()
                for n in range(cnt):
                    w = rec[8 * (noff + n): 8 * (noff + n) + 8]
                    nt = w[0] >> 16                    # the record's wave term count
                    assert 2 <= nt <= nt_max
                    r = 0.0
                    for tt in range(nt):
                        x = w[1 + tt]
                        reads.add(x & 0xffff)
                        r += c[x >> 16] * node[x & 0xffff]
                    assert (w[0] & 0xffff) not in new     # one writer per slot and step
                    new[w[0] & 0xffff] = r
            assert not (reads & set(new))
            for k, val in new.items():
                node[k] = val
            acc += node[np.array(p["vtgt"])]
    H = np.zeros(p["hsize"])
    H[:p["nacc"]] = acc
    dv = [B["AB"][0], B["AB"][1], B["AB"][2], K["AB"][0], K["AB"][1], K["AB"][2]]
    for lv in range(len(p["hlev"]) - 1):
        new, reads = {}, set()
        for e in range(p["hlev"][lv], p["hlev"][lv + 1]):
            out, x, y, d = p["hops"][e]
            reads.update((x, y))
            assert out not in new                  # one writer per slot and level
            new[out] = H[x] + dv[d] * H[y]
        # the kernel loads the next element's operands before storing the current one:
        # no element of a level may write a slot the level reads
        assert not (reads & set(new))
        for k, v in new.items():
            H[k] = v
    return H[np.array(p["outslot"])]


@pytest.mark.parametrize("grouped", [False, True])
@pytest.mark.parametrize("cls", [c for c in gen_eri.canonical_classes(2) if sum(c) >= 2])
def test_wide_program_matches_generated_code(cls, grouped):
    shells = synthetic_shells()
    sb = ShellBasis.from_shell_dicts(shells)
    g = golden("synthetic")
    done = 0
    for q in g["quartets"]:
        a, b, c, d = (int(x) for x in q)
        ls = tuple(int(sb.l[x]) for x in (a, b, c, d))
        if ls != cls:
            continue
        pr, pd, _ = hostcheck.make_pairs(sb, [(a, b), (c, d)])
        got = emulate(cls, pr, pd, 0, 1, grouped)
        blk, _ = hostcheck.canonical_block(sb, q, 64)
        s = [sb.comp_scale[x][:n] for x, n in zip((a, b, c, d), blk.shape)]
        blk = blk / (s[0][:, None, None, None] * s[1][None, :, None, None] *
                     s[2][None, None, :, None] * s[3][None, None, None, :])
        assert np.max(np.abs(got - blk.ravel())) <= 1e-13 + 1e-11 * np.max(np.abs(blk))
        done += 1
        if done == 2:
            break
    assert done > 0


@pytest.mark.parametrize("grouped", [False, True])
@pytest.mark.parametrize("cls", [(1, 1, 1, 1), (2, 0, 1, 0), (2, 1, 2, 1), (2, 2, 2, 1), (2, 2, 2, 2)])
def test_bank_spread_keeps_slots_and_cuts_conflicts(cls, grouped):
    """The slot renaming keeps the Boys value slots, maps slots one to one within the
    slot count, and lowers the shared-memory wavefronts of the operand loads (FP32: 1
    ideal; FP64: 2).  The grouped program's slot count is padded to ``wave`` mod 32, so
    that the groups' buffers start ``wave`` banks apart."""
    wave = 32 // gen_eri.vrr_group(cls)[0] if grouped else 32
    if wave == 32 and grouped:
        pytest.skip("class has no grouped form")
    real = gen_eri.bank_spread
    try:
        gen_eri.bank_spread = lambda vrec, vseg, vtgt, nvslot, L, wave=32: (vrec, vtgt, nvslot)
        p0 = gen_eri.wide_program(cls, wave)
    finally:
        gen_eri.bank_spread = real
    p1 = gen_eri.wide_program(cls, wave)
    if wave == 32:
        assert p1["nvslot"] == p0["nvslot"]
    else:
        assert p0["nvslot"] <= p1["nvslot"] < p0["nvslot"] + 32
        assert p1["nvslot"] % 32 == wave % 32
    L = p1["L"]
    ren = {}
    for r in range(len(p0["vrec"]) // 8):
        w0, w1 = p0["vrec"][8 * r: 8 * r + 8], p1["vrec"][8 * r: 8 * r + 8]
        assert w0[0] >> 16 == w1[0] >> 16
        for t in range(1 + (w0[0] >> 16)):
            a, b = w0[t] & 0xffff, w1[t] & 0xffff
            assert ren.setdefault(a, b) == b
            assert w0[t] >> 16 == w1[t] >> 16
    for a, b in zip(p0["vtgt"], p1["vtgt"]):
        assert ren.setdefault(a, b) == b
    assert len(set(ren.values())) == len(ren)              # one to one
    assert all(ren.get(m, m) == m for m in range(L + 1))   # Boys values stay put
    assert max(ren.values()) < p0["nvslot"]
    for eb in (4, 8):
        w0 = gen_eri.bank_wavefronts(p0["vrec"], p0["vseg"], eb, wave, p0["nvslot"])
        w1 = gen_eri.bank_wavefronts(p1["vrec"], p1["vseg"], eb, wave, p1["nvslot"])
        ideal = eb / 4                                     # 1 (FP32) or 2 (FP64)
        assert w1 <= w0 and (w1 < 0.9 * w0 or w0 <= ideal + 1e-9), (eb, w0, w1)


@pytest.mark.parametrize("cls", [(1, 1, 1, 1), (2, 2, 2, 1)])
def test_vrr_l1_wavefront_model(cls):
    """The L1 model of the ungrouped VRR program: FMAs are the nodes' terms; every term of
    a wave costs at least one operand and one coefficient wavefront per quartet (a wave
    holds at most 32 nodes); stacking shares only the record loads, and no 8-byte load
    takes fewer wavefronts than the 4-byte one (a bank shared within a half-warp is
    shared within the warp)."""
    p = gen_eri.wide_program(cls)
    terms = sum(p["vrec"][8 * r] >> 16 for r in range(len(p["vrec"]) // 8))
    f1, w1 = gen_eri.vrr_l1_wavefronts(cls, 1, 4)
    f4, w4 = gen_eri.vrr_l1_wavefronts(cls, 4, 4)
    _, w8 = gen_eri.vrr_l1_wavefronts(cls, 1, 8)
    assert f1 == f4 == terms
    assert w4 >= 2 * terms / 32
    nwaves = sum(-(-s[2] // 32) for s in p["vseg"])
    assert w1 - w4 == pytest.approx(8 * nwaves * (1 - 1 / 4))
    assert w8 >= w1
