"""Code generator for the shell-quartet ERI classes (la lb | lc ld).

For each canonical class it emits a C++ template specialisation ``ClassGen<LA,LB,LC,LD>``
with ``__host__ __device__`` members, usable for T = double and T = float:

* ``vrr(F, c, acc)``  one primitive quartet: Obara-Saika vertical recursion from the
  scaled Boys values ``F[m] = [00|00]^(m)`` to the targets [e0|f0]^(0),
  la <= |e| <= la+lb and lc <= |f| <= lc+ld, added into the contraction accumulator
  ``acc[ie * NF + if]``.  Bra step (x_i is the chosen direction):
      [e+1_i|0]^(m) = PA_i [e]^(m) + WP_i [e]^(m+1) + e_i/(2p) ([e-1_i]^(m) - rho/p [e-1_i]^(m+1))
  ket (electron-transfer free) step:
      [e|f+1_i]^(m) = QC_i [e|f]^(m) + WQ_i [e|f]^(m+1)
                      + f_i/(2q) ([e|f-1_i]^(m) - rho/q [e|f-1_i]^(m+1))
                      + e_i/(2(p+q)) [e-1_i|f]^(m+1)
  (Obara & Saika, J. Chem. Phys. 84, 3963 (1986); Head-Gordon & Pople, J. Chem. Phys.
  89, 5777 (1988)).  The direction of each step is chosen to drop terms (components
  equal to one) and to reuse nodes already built.
* ``hrr(acc, AB, CD, blk)``  once per contracted quartet: horizontal recursion
      (a, b+1_i| = (a+1_i, b| + AB_i (a, b|     and the same on the ket with CD,
  giving the Cartesian block blk[((ia*NB+ib)*NC+ic)*ND+id] in the reference's
  component order (s; x,y,z; xx,yy,zz,xy,xz,yz -- factory/primitive_basis_factory.py:5-86).

It also writes ``opcount.json``: floating-point operations per primitive quartet (VRR and
its set-up, Boys included) and per contracted quartet (HRR), FMA counted as two.  These
are the algorithmic FLOP figures the roofline uses.

Usage: python gen_eri.py OUTDIR [LMAX]
"""
import itertools
import json
import os
import sys

XYZ = "xyz"


def cart(L):
    if L == 0:
        return [(0, 0, 0)]
    if L == 1:
        return [(1, 0, 0), (0, 1, 0), (0, 0, 1)]
    if L == 2:
        return [(2, 0, 0), (0, 2, 0), (0, 0, 2), (1, 1, 0), (1, 0, 1), (0, 1, 1)]
    return [(lx, ly, L - lx - ly) for lx in range(L, -1, -1) for ly in range(L - lx, -1, -1)]


def ncart(L):
    return (L + 1) * (L + 2) // 2


def shift(v, i, k):
    t = list(v)
    t[i] += k
    return tuple(t)


PAIR_ORDER = [(0, 0), (1, 0), (1, 1), (2, 0), (2, 1), (2, 2), (3, 0), (3, 1), (3, 2), (3, 3)]


def pair_class(la, lb):
    return PAIR_ORDER.index((la, lb))


def canonical_classes(lmax):
    pairs = [p for p in PAIR_ORDER if p[0] <= lmax]
    out = []
    for i, (la, lb) in enumerate(pairs):
        for (lc, ld) in pairs[:i + 1]:
            out.append((la, lb, lc, ld))
    return out


class Emitter:
    def __init__(self):
        self.lines = []
        self.flops = 0

    def line(self, s):
        self.lines.append(s)


class VrrGen:
    """Builds the VRR DAG for one class and emits it in dependency order."""

    def __init__(self, cls):
        self.la, self.lb, self.lc, self.ld = cls
        self.names = {}
        self.em = Emitter()
        self.coefs = set()
        self.count = 0
        self.e_targets = [e for L in range(self.la, self.la + self.lb + 1) for e in cart(L)]
        self.f_targets = [f for L in range(self.lc, self.lc + self.ld + 1) for f in cart(L)]

    def exists(self, e, f, m):
        return (e == (0, 0, 0) and f == (0, 0, 0)) or (e, f, m) in self.names

    def coef(self, kind, k=1):
        if k == 1:
            self.coefs.add((kind, 1))
            return kind
        self.coefs.add((kind, k))
        return f"{kind}_{k}"

    def node(self, e, f, m):
        if e == (0, 0, 0) and f == (0, 0, 0):
            return f"F[{m}]"
        key = (e, f, m)
        if key in self.names:
            return self.names[key]
        terms = []
        if f == (0, 0, 0):
            cands = []
            for i in range(3):
                if e[i] == 0:
                    continue
                e1 = shift(e, i, -1)
                nterm = 2 + (2 if e1[i] > 0 else 0)
                reuse = self.exists(e1, f, m) + self.exists(e1, f, m + 1)
                cands.append((nterm, -reuse, i))
            _, _, i = min(cands)
            e1 = shift(e, i, -1)
            terms.append((f"PA{XYZ[i]}", self.node(e1, f, m)))
            terms.append((f"WP{XYZ[i]}", self.node(e1, f, m + 1)))
            if e1[i] > 0:
                e2 = shift(e1, i, -1)
                terms.append((self.coef("i2p", e1[i]), self.node(e2, f, m)))
                terms.append(("-" + self.coef("rp2", e1[i]), self.node(e2, f, m + 1)))
        else:
            cands = []
            for i in range(3):
                if f[i] == 0:
                    continue
                f1 = shift(f, i, -1)
                nterm = 2 + (2 if f1[i] > 0 else 0) + (1 if e[i] > 0 else 0)
                reuse = self.exists(e, f1, m) + self.exists(e, f1, m + 1)
                cands.append((nterm, -reuse, i))
            _, _, i = min(cands)
            f1 = shift(f, i, -1)
            terms.append((f"QC{XYZ[i]}", self.node(e, f1, m)))
            terms.append((f"WQ{XYZ[i]}", self.node(e, f1, m + 1)))
            if f1[i] > 0:
                f2 = shift(f1, i, -1)
                terms.append((self.coef("i2q", f1[i]), self.node(e, f2, m)))
                terms.append(("-" + self.coef("rq2", f1[i]), self.node(e, f2, m + 1)))
            if e[i] > 0:
                terms.append((self.coef("i2pq", e[i]), self.node(shift(e, i, -1), f1, m + 1)))
        name = f"v{self.count}"
        self.count += 1
        expr = " + ".join(f"{c} * {x}" if not c.startswith("-") else f"-{c[1:]} * {x}"
                          for c, x in terms).replace("+ -", "- ")
        self.em.line(f"    const T {name} = {expr};")
        self.em.flops += 1 + 2 * (len(terms) - 1)
        self.names[key] = name
        return name

    def build(self):
        nf = len(self.f_targets)
        for ie, e in enumerate(self.e_targets):
            for jf, f in enumerate(self.f_targets):
                x = self.node(e, f, 0)
                self.em.line(f"    acc[{ie * nf + jf}] += {x};")
                self.em.flops += 1
        return self


class HrrGen:
    """Bra then ket horizontal recursion on contracted [e0|f0] values."""

    def __init__(self, cls, e_targets, f_targets):
        self.la, self.lb, self.lc, self.ld = cls
        self.e_index = {e: i for i, e in enumerate(e_targets)}
        self.f_index = {f: i for i, f in enumerate(f_targets)}
        self.nf = len(f_targets)
        self.em = Emitter()
        self.bra_names = {}
        self.ket_names = {}
        self.count = 0

    # bra nodes are arrays over the ket VRR targets (length NF)
    def bra(self, a, b):
        if b == (0, 0, 0):
            return f"(acc + {self.e_index[a] * self.nf})"
        key = (a, b)
        if key in self.bra_names:
            return self.bra_names[key]
        cands = []
        for i in range(3):
            if b[i] == 0:
                continue
            reuse = ((shift(a, i, 1), shift(b, i, -1)) in self.bra_names) + \
                    ((a, shift(b, i, -1)) in self.bra_names)
            cands.append((-reuse, i))
        _, i = min(cands)
        x = self.bra(shift(a, i, 1), shift(b, i, -1))
        y = self.bra(a, shift(b, i, -1))
        name = f"hb{self.count}"
        self.count += 1
        self.em.line(f"    T {name}[{self.nf}];")
        self.em.line(f"    GS_UNROLL for (int k = 0; k < {self.nf}; ++k) "
                     f"{name}[k] = {x}[k] + AB{XYZ[i]} * {y}[k];")
        self.em.flops += 2 * self.nf
        self.bra_names[(a, b)] = name
        return name

    def build(self):
        na, nb, nc, nd = ncart(self.la), ncart(self.lb), ncart(self.lc), ncart(self.ld)
        nab = na * nb
        # bra HRR into G[ab * NF + f]
        self.em.line(f"    T G[{nab * self.nf}];")
        for ia, a in enumerate(cart(self.la)):
            for ib, b in enumerate(cart(self.lb)):
                src = self.bra(a, b)
                self.em.line(f"    GS_UNROLL for (int k = 0; k < {self.nf}; ++k) "
                             f"G[{(ia * nb + ib) * self.nf} + k] = {src}[k];")
        # ket HRR: arrays over ab (length NAB)
        kn = {}

        def ket(c, d):
            if d == (0, 0, 0):
                return ("G", self.f_index[c])
            if (c, d) in kn:
                return kn[(c, d)]
            cands = []
            for i in range(3):
                if d[i] == 0:
                    continue
                reuse = ((shift(c, i, 1), shift(d, i, -1)) in kn) + ((c, shift(d, i, -1)) in kn)
                cands.append((-reuse, i))
            _, i = min(cands)
            x = ket(shift(c, i, 1), shift(d, i, -1))
            y = ket(c, shift(d, i, -1))
            name = f"hk{self.count}"
            self.count += 1

            def ref(n):
                if isinstance(n, tuple):
                    return f"G[k * {self.nf} + {n[1]}]"
                return f"{n}[k]"
            self.em.line(f"    T {name}[{nab}];")
            self.em.line(f"    GS_UNROLL for (int k = 0; k < {nab}; ++k) "
                         f"{name}[k] = {ref(x)} + CD{XYZ[i]} * {ref(y)};")
            self.em.flops += 2 * nab
            kn[(c, d)] = name
            return name

        for ic, c in enumerate(cart(self.lc)):
            for id_, d in enumerate(cart(self.ld)):
                src = ket(c, d)
                off = ic * nd + id_
                if isinstance(src, tuple):
                    self.em.line(f"    GS_UNROLL for (int k = 0; k < {nab}; ++k) "
                                 f"blk[k * {nc * nd} + {off}] = G[k * {self.nf} + {src[1]}];")
                else:
                    self.em.line(f"    GS_UNROLL for (int k = 0; k < {nab}; ++k) "
                                 f"blk[k * {nc * nd} + {off}] = {src}[k];")
        return self


COEF_DEF = {
    "i2p": "i2p", "rp2": "rp2", "i2q": "i2q", "rq2": "rq2", "i2pq": "i2pq",
}


def gen_class(cls):
    la, lb, lc, ld = cls
    v = VrrGen(cls).build()
    h = HrrGen(cls, v.e_targets, v.f_targets).build()
    L = la + lb + lc + ld
    ne, nf = len(v.e_targets), len(v.f_targets)
    na, nb, nc, nd = ncart(la), ncart(lb), ncart(lc), ncart(ld)
    uses = set(c for c, _ in v.coefs)
    src = []
    src.append(f"// generated by gen_eri.py -- class ({la}{lb}|{lc}{ld})")
    src.append("#pragma once")
    src.append("namespace gs {")
    src.append(f"template <> struct ClassGen<{la}, {lb}, {lc}, {ld}> {{")
    src.append(f"  static constexpr int L = {L};")
    src.append(f"  static constexpr int NE = {ne}, NF = {nf}, NACC = {ne * nf};")
    src.append(f"  static constexpr int NA = {na}, NB = {nb}, NC = {nc}, ND = {nd};")
    src.append(f"  static constexpr int NBLK = {na * nb * nc * nd};")
    src.append(f"  static constexpr int VRR_FLOPS = {v.em.flops};")
    src.append(f"  static constexpr int HRR_FLOPS = {h.em.flops};")
    src.append("  template <typename T>")
    src.append("  GS_HD GS_INLINE static void vrr(const T* __restrict__ F, const VrrCoef<T>& c, "
               "T* __restrict__ acc) {")
    for name in ("PAx", "PAy", "PAz", "WPx", "WPy", "WPz", "QCx", "QCy", "QCz", "WQx", "WQy", "WQz",
                 "i2p", "rp2", "i2q", "rq2", "i2pq"):
        src.append(f"    const T {name} = c.{name}; (void){name};")
    for kind, k in sorted(v.coefs):
        if k != 1:
            src.append(f"    const T {kind}_{k} = T({k}) * {kind};")
    src.extend(v.em.lines)
    src.append("  }")
    src.append("  template <typename T>")
    src.append("  GS_HD GS_INLINE static void hrr(const T* __restrict__ acc, T ABx, T ABy, T ABz, "
               "T CDx, T CDy, T CDz, T* __restrict__ blk) {")
    src.append("    (void)ABx; (void)ABy; (void)ABz; (void)CDx; (void)CDy; (void)CDz;")
    src.extend(h.em.lines)
    src.append("  }")
    src.append("};")
    src.append("}  // namespace gs")
    coef_flops = sum(1 for kind, k in v.coefs if k != 1)
    return "\n".join(src) + "\n", dict(L=L, ne=ne, nf=nf, nblk=na * nb * nc * nd,
                                       vrr_flops=v.em.flops + coef_flops, hrr_flops=h.em.flops,
                                       vrr_nodes=v.count)


def main():
    out = sys.argv[1]
    lmax = int(sys.argv[2]) if len(sys.argv) > 2 else 2
    os.makedirs(out, exist_ok=True)
    classes = canonical_classes(lmax)
    counts = {}
    names = []
    for cls in classes:
        code, info = gen_class(cls)
        tag = "".join(map(str, cls))
        fn = f"eri_class_{tag}.h"
        names.append(fn)
        counts[tag] = info
        path = os.path.join(out, fn)
        if not os.path.exists(path) or open(path).read() != code:
            with open(path, "w") as f:
                f.write(code)
    agg = "// generated by gen_eri.py\n#pragma once\n" + "".join(f'#include "{n}"\n' for n in names)
    agg += "#define GS_FOR_EACH_CLASS(X) " + " ".join(
        "X(%d, %d, %d, %d)" % c for c in classes) + "\n"
    path = os.path.join(out, "eri_classes.h")
    if not os.path.exists(path) or open(path).read() != agg:
        with open(path, "w") as f:
            f.write(agg)
    lst = "// generated by gen_eri.py\n#pragma once\n#define GS_FOR_EACH_CLASS(X) " + " ".join(
        "X(%d, %d, %d, %d)" % c for c in classes) + "\n"
    path = os.path.join(out, "eri_class_list.h")
    if not os.path.exists(path) or open(path).read() != lst:
        with open(path, "w") as f:
            f.write(lst)
    with open(os.path.join(out, "opcount.json"), "w") as f:
        json.dump(counts, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
