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
from gen_eri import COEF_ID, HrrGen, VrrGen, cart, ncart, _alloc, _release  # noqa: E402

WEIGHT_SLOT = {0: None, 1: 32, 2: 33, 3: 34}    # coefficient slots holding 2alpha, 2beta, 2gamma
NCOEF_G = 36


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


def main():
    out = sys.argv[1]
    lmax = int(sys.argv[2]) if len(sys.argv) > 2 else 1
    os.makedirs(out, exist_ok=True)
    classes = gen_eri.canonical_classes(lmax)
    for cls in classes:
        code, _ = emit_grad(cls)
        path = os.path.join(out, "eri_grad_%s.h" % "".join(map(str, cls)))
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
