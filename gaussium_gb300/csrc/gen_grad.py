"""Warp programs for the fused ERI-gradient (adjoint) kernel, one per input class.

For a canonical class (la lb | lc ld) the program evaluates, per primitive quartet, the
Obara-Saika VRR to the union of four target grids and accumulates each grid with its own
primitive weight:
    w = 1      e in [la-1, la+lb],   f in [lc-1, lc+ld]    (lowered A, B and C blocks)
    w = 2alpha e in [la+1, la+lb+1], f in [lc, lc+ld]      (A raised)
    w = 2beta  e in [la, la+lb+1],   f in [lc, lc+ld]      (B raised)
    w = 2gamma e in [la, la+lb],     f in [lc+1, lc+ld+1]  (C raised)
then six HRR sub-programs turn the contracted grids into the blocks
(la+1 lb|lc ld), (la lb+1|..), (la lb|lc+1 ld) and the lowered (la-1 ..), (.. lb-1|..),
(..|lc-1 ld), whose combination d/dR_x (ab|cd) = (a+1x ..)_{2alpha} - a_x (a-1x ..) the
kernel contracts with the density weights.
"""
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
import gen_eri  # noqa: E402
from gen_eri import HrrGen, VrrGen, cart, ncart, _alloc, _release  # noqa: E402

WEIGHT_SLOT = {0: None, 1: 32, 2: 33, 3: 34}    # coefficient slots holding 2alpha, 2beta, 2gamma
NCOEF_G = 36
# the ERI programs' coefficient slots, plus 5/(2(p+q)) in slot 35: the raised bra of a
# (dd|..) class reaches e_i = 5 in the electron-transfer term
COEF_ID = dict(gen_eri.COEF_ID, i2pq_5=35)


def _range(lo, hi):
    return [e for L in range(max(lo, 0), hi + 1) for e in cart(L)]


def grad_program(cls):
    la, lb, lc, ld = cls
    L = la + lb + lc + ld + 1
    regions = [  # (weight kind, e list, f list)
        (0, _range(la - 1, la + lb), _range(lc - 1, lc + ld)),
        (1, _range(la + 1, la + lb + 1), _range(lc, lc + ld)),
        (2, _range(la, la + lb + 1), _range(lc, lc + ld)),
        (3, _range(la, la + lb), _range(lc + 1, lc + ld + 1)),
    ]
    v = VrrGen((la, lb, lc, ld))
    names = {}
    acc_entries = []          # (region index, element index, node name)
    rbase = []
    off = 0
    for r, (w, es, fs) in enumerate(regions):
        rbase.append(off)
        for ie, e in enumerate(es):
            for jf, f in enumerate(fs):
                nm = v.node(e, f, 0)
                acc_entries.append((r, ie * len(fs) + jf, nm))
        off += len(es) * len(fs)
    nacc = off

    # ---- VRR node program (levels, term groups, liveness-planned slots)
    def slot(opnd):
        if opnd.startswith("F["):
            return int(opnd[2:-1])
        return L + 1 + int(opnd[1:])

    level = {m: 0 for m in range(L + 1)}
    nodes = []
    for idx, terms in enumerate(v.struct):
        ts = [(COEF_ID[c], slot(x)) for c, x in terms]
        lv = 1 + max(level[s] for _, s in ts)
        level[L + 1 + idx] = lv
        nodes.append((lv, len(ts), L + 1 + idx, ts))
    nodes.sort(key=lambda n: (n[0], n[1], n[2]))
    tslots = set(slot(nm) for _, _, nm in acc_entries)
    maxlv = max((n[0] for n in nodes), default=0)
    last = {}
    for lv, nt, out, ts in nodes:
        for _, sl in ts:
            last[sl] = max(last.get(sl, 0), lv)
    for sl in tslots:
        last[sl] = maxlv + 1
    phys = {m: m for m in range(L + 1)}
    free, top, by_level = [], L + 1, {}
    for n in nodes:
        by_level.setdefault(n[0], []).append(n)
    for lv in sorted(by_level):
        for n in by_level[lv]:
            if free:
                phys[n[2]] = free.pop()
            else:
                phys[n[2]] = top
                top += 1
        for sl, lu in last.items():
            if lu == lv and sl > L:
                free.append(phys[sl])
        free.sort(reverse=True)
    vrec, vseg = [], []
    i = 0
    while i < len(nodes):
        j = i
        while j < len(nodes) and nodes[j][:2] == nodes[i][:2]:
            j += 1
        lv, nt = nodes[i][:2]
        sync = 1 if (not vseg or vseg[-1][4] != lv) else 0
        vseg.append([len(vrec) // 8, 0, j - i, nt, lv, sync])
        for n in nodes[i:j]:
            words = [phys[n[2]] | (nt << 16)] + [(cid << 16) | phys[sl] for cid, sl in n[3]]
            vrec.extend(words + [0] * (8 - len(words)))
        i = j
    acc_slot = [phys[slot(nm)] for _, _, nm in acc_entries]
    acc_kind = [regions[r][0] for r, _, _ in acc_entries]
    acc_pos = [rbase[r] + k for r, k, _ in acc_entries]       # position in the H buffer
    nvslot = top

    # ---- six HRR sub-programs on the H buffer (acc grids at the front)
    subs = [  # (name, centre, raised?, region, modified class)
        ("A+", 0, True, 1, (la + 1, lb, lc, ld)),
        ("B+", 1, True, 2, (la, lb + 1, lc, ld)),
        ("C+", 2, True, 3, (la, lb, lc + 1, ld)),
        ("A-", 0, False, 0, (la - 1, lb, lc, ld)),
        ("B-", 1, False, 0, (la, lb - 1, lc, ld)),
        ("C-", 2, False, 0, (la, lb, lc - 1, ld)),
    ]
    free = [(nacc, 1 << 20)]
    peak = nacc
    hops, hlev = [], []
    outs = []
    for sname, cen, raised, reg, mcls in subs:
        if min(mcls) < 0:
            outs.append(None)
            continue
        _, es, fs = regions[reg]
        h = HrrGen(mcls, es, fs).build()
        nf = len(fs)
        ma, mb, mc, md = (ncart(x) for x in mcls)
        nab = ma * mb
        base = {}
        for r in range(len(es)):
            base[f"(acc + {r * nf})"] = rbase[reg] + r * nf
        lvl = {k: 0 for k in base}
        ops = []
        for name, x, y, d in h.bra_ops:
            lv = 1 + max(lvl[x], lvl[y])
            lvl[name] = lv
            ops.append((lv, 0, name, x, y, d, nf))
        nbra = max([o[0] for o in ops], default=0)

        def kl(n):
            return nbra if isinstance(n, tuple) else lvl[n]
        for name, x, y, d in h.ket_ops:
            lv = 1 + max(kl(x), kl(y))
            lvl[name] = lv
            ops.append((lv, 1, name, x, y, d, nab))
        nlev = max([o[0] for o in ops], default=0)
        lastu = {}

        def touch(n, lv):
            if isinstance(n, tuple):
                for ab in range(nab):
                    rn = h.bra_final[(ab // mb, ab % mb)]
                    lastu[rn] = max(lastu.get(rn, 0), lv)
            else:
                lastu[n] = max(lastu.get(n, 0), lv)
        for o in ops:
            touch(o[3], o[0])
            touch(o[4], o[0])
        keep = set()
        for n in h.ket_final.values():
            if isinstance(n, tuple):
                for ab in range(nab):
                    keep.add(h.bra_final[(ab // mb, ab % mb)])
            else:
                keep.add(n)
        if not h.ket_ops:
            keep.update(h.bra_final.values())
        sizes = {o[2]: o[6] for o in ops}
        for lv in range(1, nlev + 1):
            for o in ops:
                if o[0] == lv:
                    base[o[2]] = _alloc(free, sizes[o[2]])
                    peak = max(peak, base[o[2]] + sizes[o[2]])
            for n, lu in list(lastu.items()):
                if lu == lv and n in sizes and n not in keep:
                    _release(free, base[n], sizes[n])

        def eslot(n, k):
            if isinstance(n, tuple):
                rn = h.bra_final[(k // mb, k % mb)]
                return base[rn] + n[1]
            return base[n] + k
        for lv in range(1, nlev + 1):
            hlev.append(len(hops))
            for o in ops:
                if o[0] != lv:
                    continue
                _, ph, name, x, y, d, n = o
                for k in range(n):
                    hops.append((base[name] + k, eslot(x, k), eslot(y, k), d + 3 * ph))
        # the sub-program's levels end with a barrier; record its output slots
        outslot = []
        for ab in range(nab):
            for cd in range(mc * md):
                src = h.ket_final[(cd // md, cd % md)]
                if isinstance(src, tuple):
                    outslot.append(base[h.bra_final[(ab // mb, ab % mb)]] + src[1])
                else:
                    outslot.append(base[src] + ab)
        outs.append(outslot)
    hlev.append(len(hops))
    assert peak < 65536 and nvslot < 65536
    return dict(L=L, nacc=nacc, nvslot=nvslot, vrec=vrec, vseg=vseg, acc_slot=acc_slot,
                acc_kind=acc_kind, acc_pos=acc_pos, hsize=peak, hops=hops, hlev=hlev, outs=outs,
                regions=[(w, len(es), len(fs)) for w, es, fs in regions])


def emit_grad(cls):
    p = grad_program(cls)
    tag = "".join(map(str, cls))
    la, lb, lc, ld = cls

    def arr(ctype, name, vals):
        body = ",".join(str(x) for x in vals) if vals else "0"
        return f"__device__ const {ctype} {name}[{max(1, len(vals))}] = {{{body}}};"
    segs = [x for s in p["vseg"] for x in (s[0], s[2], s[3], s[5])]
    hop = [x for o in p["hops"] for x in (o[0] | (o[1] << 16), o[2] | (o[3] << 16))]
    acc = [s | (k << 16) for s, k in zip(p["acc_slot"], p["acc_kind"])]
    out_all, out_off = [], []
    for o in p["outs"]:
        out_off.append(len(out_all) if o is not None else -1)
        if o is not None:
            out_all.extend(o)
    lines = [f"// generated by gen_grad.py -- gradient warp program of class ({la}{lb}|{lc}{ld})",
             "#pragma once", "namespace gs {",
             arr("unsigned int __align__(16)", f"g{tag}_vrec", p["vrec"]),
             arr("int", f"g{tag}_vseg", segs),
             arr("unsigned int", f"g{tag}_acc", acc),
             arr("unsigned short", f"g{tag}_accpos", p["acc_pos"]),
             arr("unsigned int", f"g{tag}_hop", hop),
             arr("int", f"g{tag}_hlev", p["hlev"]),
             arr("unsigned short", f"g{tag}_out", out_all),
             arr("int", f"g{tag}_outoff", out_off),
             f"template <> struct GradProg<{la}, {lb}, {lc}, {ld}> {{",
             f"  static constexpr int L = {p['L']}, NACC = {p['nacc']}, NVSLOT = {p['nvslot']};",
             f"  static constexpr int NVSEG = {len(p['vseg'])}, HSIZE = {p['hsize']}, "
             f"NHLEV = {len(p['hlev']) - 1};",
             f"  static __device__ const int* out_off() {{ return g{tag}_outoff; }}",
             f"  static __device__ const uint4* vrec() {{ return reinterpret_cast<const uint4*>(g{tag}_vrec); }}",
             f"  static __device__ const int* vseg() {{ return g{tag}_vseg; }}",
             f"  static __device__ const unsigned int* acc() {{ return g{tag}_acc; }}",
             f"  static __device__ const unsigned short* accpos() {{ return g{tag}_accpos; }}",
             f"  static __device__ const unsigned int* hop() {{ return g{tag}_hop; }}",
             f"  static __device__ const int* hlev() {{ return g{tag}_hlev; }}",
             f"  static __device__ const unsigned short* out() {{ return g{tag}_out; }}",
             "};", "}  // namespace gs", ""]
    return "\n".join(lines), p


THREAD_LMAX = 3       # classes with la+lb+lc+ld <= this also get a thread-per-quartet form


def emit_grad_thread(cls, p=None):
    """Straight-line thread-per-quartet form of the same program: per primitive quartet the
    VRR node program and the weighted accumulation into H[0 .. NACC), then the six HRR
    sub-programs on H and the contraction with the density weights, all with
    compile-time indices so that the node values and accumulators live in registers."""
    p = p or grad_program(cls)
    la, lb, lc, ld = cls
    tag = "".join(map(str, cls))
    L, nacc = p["L"], p["nacc"]
    vr = p["vrec"]
    body = []
    # VRR: records of 8 words: out | nt << 16, then (cid << 16 | slot) per term
    for r in range(len(vr) // 8):
        w = vr[8 * r: 8 * r + 8]
        out, nt = w[0] & 0xffff, w[0] >> 16
        terms = [(x >> 16, x & 0xffff) for x in w[1:1 + nt]]
        e = f"c[{terms[0][0]}] * n[{terms[0][1]}]"
        for cid, sl in terms[1:]:
            e = f"fma(c[{cid}], n[{sl}], {e})"
        body.append(f"    n[{out}] = {e};")
    acc = []
    for k, (sl, kind, pos) in enumerate(zip(p["acc_slot"], p["acc_kind"], p["acc_pos"])):
        if kind == 0:
            acc.append(f"    H[{pos}] += n[{sl}];")
        else:
            acc.append(f"    H[{pos}] = fma(c[{31 + kind}], n[{sl}], H[{pos}]);")
    hrr = [f"    H[{d}] = fma(dv[{dd}], H[{y}], H[{x}]);" for d, x, y, dd in p["hops"]]
    # contraction: g[3 cen + x] += gamma_e s_cen (H[raised] - e_x H[lowered])
    ls = [la, lb, lc, ld]
    n = [ncart(x) for x in ls]
    con = []
    for ia in range(n[0]):
        for ib in range(n[1]):
            for ic in range(n[2]):
                for idd in range(n[3]):
                    idx = [ia, ib, ic, idd]
                    con.append(f"    gam = w * (0.5 * pab[{ia * n[1] + ib}] * pcd[{ic * n[3] + idd}] - "
                               f"0.125 * (pac[{ia * n[2] + ic}] * pbd[{ib * n[3] + idd}] + "
                               f"pad[{ia * n[3] + idd}] * pbc[{ib * n[2] + ic}]));")
                    # unscaled HRR blocks: the element carries all four component scales
                    con.append(f"    s = gam * cs0[{ia}] * cs1[{ib}] * cs2[{ic}] * cs3[{idd}];")
                    for cen in range(3):
                        ex = cart(ls[cen])[idx[cen]]
                        for x in range(3):
                            up = list(ex)
                            up[x] += 1
                            ii = list(idx)
                            nn = list(n)
                            ii[cen] = cart(ls[cen] + 1).index(tuple(up))
                            nn[cen] = ncart(ls[cen] + 1)
                            e_up = ((ii[0] * nn[1] + ii[1]) * nn[2] + ii[2]) * nn[3] + ii[3]
                            h_up = p["outs"][cen][e_up]
                            term = f"H[{h_up}]"
                            if ex[x] > 0:
                                dn = list(ex)
                                dn[x] -= 1
                                jj = list(idx)
                                mm = list(n)
                                jj[cen] = cart(ls[cen] - 1).index(tuple(dn))
                                mm[cen] = ncart(ls[cen] - 1)
                                e_dn = ((jj[0] * mm[1] + jj[1]) * mm[2] + jj[2]) * mm[3] + jj[3]
                                h_dn = p["outs"][3 + cen][e_dn]
                                term = f"(H[{h_up}] - {ex[x]}.0 * H[{h_dn}])"
                            con.append(f"    g[{3 * cen + x}] = fma(s, {term}, g[{3 * cen + x}]);")
    lines = [f"// generated by gen_grad.py -- thread-per-quartet gradient code of class ({la}{lb}|{lc}{ld})",
             "#pragma once", "namespace gs {",
             f"template <> struct GradThread<{la}, {lb}, {lc}, {ld}> {{",
             f"  static constexpr int L = {L}, NACC = {nacc}, NVSLOT = {p['nvslot']}, HSIZE = {p['hsize']};",
             "  template <typename T>",
             "  static __device__ __forceinline__ void prim(const T* __restrict__ c, T* n, T* H) {",
             *body, *acc, "  }",
             "  static __device__ __forceinline__ void hrr(double* H, const double* dv) {",
             *hrr, "  }",
             "  static __device__ __forceinline__ void contract(const double* H, double w, const double* pab,",
             "      const double* pcd, const double* pac, const double* pbd, const double* pad,",
             "      const double* pbc, const double* cs0, const double* cs1, const double* cs2,",
             "      const double* cs3, double* g) {",
             "    double gam, s;", *con, "  }", "};", "}  // namespace gs", ""]
    return "\n".join(lines)


def main():
    out = sys.argv[1]
    lmax = int(sys.argv[2]) if len(sys.argv) > 2 else 1
    os.makedirs(out, exist_ok=True)
    classes = gen_eri.canonical_classes(lmax)
    for cls in classes:
        code, prog = emit_grad(cls)
        path = os.path.join(out, "eri_grad_%s.h" % "".join(map(str, cls)))
        if not os.path.exists(path) or open(path).read() != code:
            with open(path, "w") as f:
                f.write(code)
        if sum(cls) <= THREAD_LMAX:
            code = emit_grad_thread(cls, prog)
            path = os.path.join(out, "eri_gradt_%s.h" % "".join(map(str, cls)))
            if not os.path.exists(path) or open(path).read() != code:
                with open(path, "w") as f:
                    f.write(code)
    lst = ("// generated by gen_grad.py\n#pragma once\n#define GS_FOR_EACH_GRAD(X) " +
           " ".join("X(%d, %d, %d, %d)" % c for c in classes) + "\n")
    path = os.path.join(out, "eri_grad_list.h")
    if not os.path.exists(path) or open(path).read() != lst:
        with open(path, "w") as f:
            f.write(lst)


if __name__ == "__main__":
    main()
