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
        self.struct = []      # per node: list of (coefficient name, operand)
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
        self.struct.append(terms)
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
        self.bra_ops = []     # (name, x, y, dir): name[k] = x[k] + AB_dir * y[k], k < NF
        self.ket_ops = []     # (name, x, y, dir): arrays over ab, x/y may be ("G", f)
        self.bra_final = {}   # (ia, ib) -> array name (or "(acc + off)")
        self.ket_final = {}   # (ic, id) -> array name or ("G", f)

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
        self.bra_ops.append((name, x, y, i))
        return name

    def build(self):
        na, nb, nc, nd = ncart(self.la), ncart(self.lb), ncart(self.lc), ncart(self.ld)
        nab = na * nb
        # bra HRR into G[ab * NF + f]
        self.em.line(f"    T G[{nab * self.nf}];")
        for ia, a in enumerate(cart(self.la)):
            for ib, b in enumerate(cart(self.lb)):
                src = self.bra(a, b)
                self.bra_final[(ia, ib)] = src
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
            self.ket_ops.append((name, x, y, i))
            return name

        for ic, c in enumerate(cart(self.lc)):
            for id_, d in enumerate(cart(self.ld)):
                src = ket(c, d)
                self.ket_final[(ic, id_)] = src
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
    for cls in classes:
        code, _ = emit_wide(cls)
        path = os.path.join(out, "eri_wide_%s.h" % "".join(map(str, cls)))
        if not os.path.exists(path) or open(path).read() != code:
            with open(path, "w") as f:
                f.write(code)
    with open(os.path.join(out, "opcount.json"), "w") as f:
        json.dump(counts, f, indent=1, sort_keys=True)



# ---------------------------------------------------------------------- warp programs
COEF_ID = {}
for _i, _n in enumerate(["PAx", "PAy", "PAz", "WPx", "WPy", "WPz", "QCx", "QCy", "QCz",
                         "WQx", "WQy", "WQz"]):
    COEF_ID[_n] = _i
for _base, _kind in ((12, "i2p"), (16, "-rp2"), (20, "i2q"), (24, "-rq2"), (28, "i2pq")):
    for _k in range(1, 5):
        COEF_ID[_kind if _k == 1 else f"{_kind}_{_k}"] = _base + _k - 1
NCOEF = 32


def _alloc(free, size):
    """First fit in a sorted free list of [start, end) intervals; returns start."""
    for i, (a, b) in enumerate(free):
        if b - a >= size:
            if b - a == size:
                free.pop(i)
            else:
                free[i] = (a + size, b)
            return a
    raise RuntimeError("allocator exhausted")


def _release(free, start, size):
    free.append((start, start + size))
    free.sort()
    merged = []
    for a, b in free:
        if merged and merged[-1][1] == a:
            merged[-1] = (merged[-1][0], b)
        else:
            merged.append((a, b))
    free[:] = merged


# Coefficient slot that the warp kernels set to zero: the term a node is padded with when
# its wave holds nodes with more terms.  It is the i2p_4 slot, which no class up to
# (dd|dd) reads (the bra step uses (e-1_i)_i <= la+lb-1 <= 3).
ZERO_COEF = 15


def vrr_waves(nodes, L, target_slots, wave=32):
    """Schedule the VRR nodes of one primitive quartet for a warp.

    ``nodes``: (virtual slot, [(coefficient id, operand slot), ...]) in dependency order;
    slots 0..L are the scaled Boys values.  Returns (vrec, vseg, phys, nvslot).

    The warp evaluates the nodes in waves of at most ``wave`` nodes, one node per lane (or
    per lane group of the grouped form, which runs 32/wave primitive quartets at once).
    Each wave costs as many FP64 instructions as its largest term count whatever its
    active lanes, so the scheduler fills waves completely: at each step it takes the nodes
    whose operands are all done, most critical (longest path to a target) first, and
    emits as many full waves as it can, a partial one only when nothing else is ready.
    Nodes of a wave with fewer terms are padded with (ZERO_COEF x node 0).  Waves of one
    step read only values of earlier steps, so the kernel synchronises the warp at the
    first wave of each step only.  Slots are assigned by liveness over steps: a slot last
    read in step s is reused from step s+1 on; targets and Boys values live to the end."""
    import collections
    byout = {o: ts for o, ts in nodes}
    users = collections.defaultdict(list)
    for o, ts in nodes:
        for _, s in ts:
            users[s].append(o)
    height = {}
    for o, ts in reversed(nodes):
        height[o] = 1 + max((height[u] for u in users[o]), default=0)
    done = set(range(L + 1))
    pending = set(byout)
    steps = []
    while pending:
        ready = [o for o in pending if all(s in done for _, s in byout[o])]
        ready.sort(key=lambda o: (-height[o], -len(byout[o]), o))
        nfull = len(ready) // wave
        take = ready[:nfull * wave] if nfull else ready
        take.sort(key=lambda o: (-len(byout[o]), o))
        steps.append([take[i:i + wave] for i in range(0, len(take), wave)])
        done |= set(take)
        pending -= set(take)
    step_of = {o: k for k, st in enumerate(steps) for w in st for o in w}
    last = {}
    for o, ts in nodes:
        for _, s in ts:
            last[s] = max(last.get(s, 0), step_of[o])
    for s in target_slots:
        last[s] = len(steps)
    phys = {m: m for m in range(L + 1)}
    free, top = [], L + 1
    for k, st in enumerate(steps):
        for w in st:
            for o in w:
                if free:
                    phys[o] = free.pop()
                else:
                    phys[o] = top
                    top += 1
        for s, lu in last.items():
            if lu == k and s > L:
                free.append(phys[s])
        free.sort(reverse=True)
    # one segment per step: its waves are consecutive runs of ``wave`` records, each padded
    # to the wave's largest term count, which every record of the wave carries
    vrec, vseg = [], []
    for k, st in enumerate(steps):
        seg = [len(vrec) // 8, 0, sum(len(w) for w in st), 0, k, 1 if k > 0 else 0]
        for w in st:
            nt = max(len(byout[o]) for o in w)
            seg[3] = max(seg[3], nt)
            for o in w:
                ts = byout[o]
                assert all(cid != ZERO_COEF for cid, _ in ts), "zero slot in use"
                words = [phys[o] | (nt << 16)] + [(cid << 16) | phys[s] for cid, s in ts]
                words += [(ZERO_COEF << 16)] * (nt - len(ts))
                words += [0] * (8 - len(words))
                vrec.extend(words)
        vseg.append(seg)
    return vrec, vseg, phys, top


def bank_spread(vrec, vseg, vtgt, nvslot, L, wave=32):
    """Rename the node slots of a program so that the slots one instruction touches across
    the warp fall in different shared-memory banks.

    Waves of 32 (the ungrouped program): each wave's operands of one term, its outputs,
    and each run of 32 targets.  A slot s sits in bank s mod 32 (FP32 words; an FP64 slot
    spans banks 2s, 2s+1, so FP64 lanes of one half-warp conflict when their slots agree
    mod 16).  Waves of 32/VG (the grouped program): lane g*wave + j runs record j on group
    g's buffer, at g*NVS + slot.  With the wave's slots distinct mod ``wave`` and NVS = wave
    (mod 32), the groups' copies land ``wave`` banks apart, so the warp (FP32) and each
    half-warp (FP64) read distinct banks; the slot count is padded to that residue.

    Greedy colouring: slots in order of the weight of their groups take the class (with
    room left) least shared with the slots already placed in their groups, FP64 half-warp
    pairs counted too for waves of 32; then class b's slots become b, b + M, b + 2M, ...
    (M = 32 or ``wave``).  The Boys value slots 0..L stay where the kernel writes them.  A
    renaming changes no value's lifetime, so the schedule's hazard rules hold.  Returns
    (vrec, vtgt, nvslot)."""
    import collections
    M = 32 if wave == 32 else wave
    groups = []
    for noff, _, cnt, _, _, _ in vseg:
        for w0 in range(0, cnt, wave):
            recs = [vrec[8 * (noff + n): 8 * (noff + n) + 8] for n in range(w0, min(cnt, w0 + wave))]
            nt = recs[0][0] >> 16
            groups.append([r[0] & 0xffff for r in recs])
            for t in range(nt):
                groups.append([r[1 + t] & 0xffff for r in recs])
    if wave == 32:
        for k in range(0, len(vtgt), 32):
            groups.append(list(vtgt[k:k + 32]))
    w32 = collections.defaultdict(collections.Counter)      # same wave: avoid equal mod M
    w16 = collections.defaultdict(collections.Counter)      # same half-warp: equal mod 16
    for g in groups:
        u = sorted(set(g))
        for i, a in enumerate(u):
            for b in u[i + 1:]:
                w32[a][b] += 1
                w32[b][a] += 1
        if wave < 32:
            continue
        for half in (g[:16], g[16:]):
            u = sorted(set(half))
            for i, a in enumerate(u):
                for b in u[i + 1:]:
                    w16[a][b] += 1
                    w16[b][a] += 1
    cap = [len(range(b, nvslot, M)) for b in range(M)]      # ids stay below nvslot
    bank = {}
    fill = [0] * M
    for s in range(L + 1):                       # Boys slots keep their ids
        bank[s] = s % M
        fill[s % M] += 1
    order = sorted((s for s in range(L + 1, nvslot)),
                   key=lambda s: (-(sum(w32[s].values()) + sum(w16[s].values())), s))
    for s in order:
        cost = [0] * M
        for n, c in w32[s].items():
            if n in bank:
                cost[bank[n]] += 2 * c
        for n, c in w16[s].items():
            if n in bank:
                b = bank[n] % 16
                cost[b] += c
                cost[b + 16] += c
        best = min((b for b in range(M) if fill[b] < cap[b]), key=lambda b: (cost[b], fill[b], b))
        bank[s] = best
        fill[best] += 1
    rank = [0] * M
    new = {}
    for s in range(nvslot):                      # Boys slots first, then in slot order
        b = bank[s]
        new[s] = M * rank[b] + b
        rank[b] += 1
    out = list(vrec)
    for r in range(len(vrec) // 8):
        w = vrec[8 * r: 8 * r + 8]
        nt = w[0] >> 16
        out[8 * r] = (w[0] & ~0xffff) | new[w[0] & 0xffff]
        for t in range(nt):
            x = w[1 + t]
            out[8 * r + 1 + t] = (x & ~0xffff) | new[x & 0xffff]
    if wave < 32:
        nvslot += (wave - nvslot) % 32
    return out, [new[t] for t in vtgt], nvslot


def bank_wavefronts(vrec, vseg, elem_bytes, wave=32, nvs=0):
    """Average shared-memory wavefronts per warp-wide operand load of a program (1 ideal
    for 4-byte, 2 for 8-byte elements): the distinct addresses of each bank, per warp
    (4 B) or per half-warp (8 B).  Lane g*wave + j reads record j's slot in group g's
    buffer, at g*nvs + slot (one group for waves of 32)."""
    vg = 32 // wave
    tot = wf = 0
    for noff, _, cnt, _, _, _ in vseg:
        for w0 in range(0, cnt, wave):
            recs = [vrec[8 * (noff + n): 8 * (noff + n) + 8] for n in range(w0, min(cnt, w0 + wave))]
            for t in range(recs[0][0] >> 16):
                slots = [r[1 + t] & 0xffff for r in recs]
                lanes = {g * wave + j: g * nvs + x for g in range(vg) for j, x in enumerate(slots)}
                parts = ([list(lanes.values())] if elem_bytes == 4 else
                         [[a for ln, a in lanes.items() if ln < 16],
                          [a for ln, a in lanes.items() if ln >= 16]])
                n = 0
                for part in parts:
                    if part:
                        banks = _bank_sets(part, 32 if elem_bytes == 4 else 16)
                        n += max(len(v) for v in banks.values())
                tot += 1
                wf += n
    return wf / tot if tot else 1.0


def vrr_l1_wavefronts(cls, rq=1, elem_bytes=4):
    """L1 wavefronts and FMAs per primitive quartet of the ungrouped VRR program run by the
    warp form (rq = 1) or the stacked form (rq primitive quartets per record decode).
    Counted per wave: the two 16-byte record loads of every lane (8 wavefronts, shared
    by the rq quartets); per quartet and term, the operand load (its bank conflicts
    included, per warp for 4-byte and per half-warp for 8-byte elements) and the
    coefficient load (a gather from the quartet's 32 contiguous coefficients: 1
    wavefront, or 2 for 8-byte elements); per quartet, the output store.  FMAs are the
    nodes' terms, padding excluded.  Returns (fma, wavefronts) per primitive quartet."""
    p = wide_program(cls)
    vrec, vseg = p["vrec"], p["vseg"]
    nb = 32 if elem_bytes == 4 else 16

    def wf(slots):
        parts = [slots] if elem_bytes == 4 else [slots[:16], slots[16:]]
        return sum(max(len(v) for v in _bank_sets(x, nb).values()) for x in parts if x)
    fma = 0
    per_q = 0
    rec = 0
    for noff, _, cnt, _, _, _ in vseg:
        for w0 in range(0, cnt, 32):
            recs = [vrec[8 * (noff + n): 8 * (noff + n) + 8] for n in range(w0, min(cnt, w0 + 32))]
            fma += sum(r[0] >> 16 for r in recs)
            rec += 8
            per_q += wf([r[0] & 0xffff for r in recs])
            for t in range(recs[0][0] >> 16):
                per_q += wf([r[1 + t] & 0xffff for r in recs]) + elem_bytes // 4
    return fma, per_q + rec / rq


def _bank_sets(slots, nbanks):
    """Distinct slots per bank (slot mod nbanks)."""
    out = {}
    for a in set(slots):
        out.setdefault(a % nbanks, set()).add(a)
    return out


def wave_efficiency(vrec, vseg, lanes_per_node=1):
    """Useful FMA lane-slots over issued lane-slots of a scheduled VRR program whose
    waves are ``32 // lanes_per_node`` records long."""
    wave = 32 // lanes_per_node
    useful = issued = 0
    for noff, _, cnt, _, _, _ in vseg:
        for w0 in range(0, cnt, wave):
            nt = vrec[8 * (noff + w0)] >> 16
            for n in range(w0, min(cnt, w0 + wave)):
                r = 8 * (noff + n)
                assert vrec[r] >> 16 == nt
                useful += sum(1 for w in vrec[r + 1: r + 1 + nt] if (w >> 16) != ZERO_COEF)
            issued += 32 * nt
    return useful * lanes_per_node / issued if issued else 1.0


def wide_program(cls, wave=32):
    """Tables for the warp-cooperative kernel of one class: VRR node descriptors packed
    into waves of ``wave`` independent nodes (vrr_waves), the targets' slots, and the HRR
    element operations on a liveness-planned shared buffer."""
    la, lb, lc, ld = cls
    v = VrrGen(cls).build()
    h = HrrGen(cls, v.e_targets, v.f_targets).build()
    L = la + lb + lc + ld
    nf = len(v.f_targets)
    nacc = len(v.e_targets) * nf
    na, nb, nc, nd = ncart(la), ncart(lb), ncart(lc), ncart(ld)
    nab, ncd = na * nb, nc * nd

    # ---- VRR
    def slot(opnd):
        if opnd.startswith("F["):
            return int(opnd[2:-1])
        return L + 1 + int(opnd[1:])

    nodes = [(L + 1 + idx, [(COEF_ID[c], slot(x)) for c, x in terms])
             for idx, terms in enumerate(v.struct)]
    tgt = [v.names[(e, f, 0)] if not (e == (0, 0, 0) and f == (0, 0, 0)) else "F[0]"
           for e in v.e_targets for f in v.f_targets]
    vrec, vseg, phys, nvslot = vrr_waves(nodes, L, [slot(t) for t in tgt], wave)
    vtgt = [phys[slot(t)] for t in tgt]
    vrec, vtgt, nvslot = bank_spread(vrec, vseg, vtgt, nvslot, L, wave)
    vout, vdesc = [], []
    # ---- HRR: arrays, levels, liveness
    arrays = {}          # name -> (size, producer level)
    lvl = {}
    for r in range(len(v.e_targets)):
        lvl[f"(acc + {r * nf})"] = 0
    ops = []             # (level, phase, name, x, y, dir)
    for name, x, y, d in h.bra_ops:
        lv = 1 + max(lvl[x], lvl[y])
        lvl[name] = lv
        arrays[name] = nf
        ops.append((lv, 0, name, x, y, d))
    nbra = max([o[0] for o in ops], default=0)

    def kl(n):
        return nbra if isinstance(n, tuple) else lvl[n]
    for name, x, y, d in h.ket_ops:
        lv = 1 + max(kl(x), kl(y))
        lvl[name] = lv
        arrays[name] = nab
        ops.append((lv, 1, name, x, y, d))
    nlev = max([o[0] for o in ops], default=0)
    # last level each array is read at (finals live to the end)
    last = {}

    def touch(n, lv):
        if isinstance(n, tuple):
            for ab in range(nab):
                rn = h.bra_final[(ab // nb, ab % nb)]
                last[rn] = max(last.get(rn, 0), lv)
        else:
            last[n] = max(last.get(n, 0), lv)
    for lv, ph, name, x, y, d in ops:
        touch(x, lv)
        touch(y, lv)
    for n in h.bra_final.values():
        last[n] = max(last.get(n, 0), nbra + 1 if h.ket_ops else nlev + 1)
    for n in h.ket_final.values():
        if isinstance(n, tuple):
            touch(n, nlev + 1)
        else:
            last[n] = nlev + 1
    if not h.ket_ops:
        for n in h.bra_final.values():
            last[n] = nlev + 1
    base = {}
    big = 1 << 20
    free = [(nacc, big)]
    for r in range(len(v.e_targets)):
        base[f"(acc + {r * nf})"] = r * nf
    # acc rows are freed after their last read
    acc_rows = [f"(acc + {r * nf})" for r in range(len(v.e_targets))]
    peak = nacc
    for lv in range(1, nlev + 2):
        for o in ops:
            if o[0] == lv:
                base[o[2]] = _alloc(free, arrays[o[2]])
                peak = max(peak, base[o[2]] + arrays[o[2]])
        for n in list(base):
            if last.get(n, 0) == lv and n not in ("",):
                size = nf if n in acc_rows else arrays[n]
                _release(free, base[n], size)
    hsize = peak

    def eslot(n, k):
        """slot of element k of array n (k over f for bra arrays, over ab for ket arrays)."""
        if isinstance(n, tuple):
            rn = h.bra_final[(k // nb, k % nb)]
            return base[rn] + n[1]
        return base[n] + k
    hops, hlev = [], []
    for lv in range(1, nlev + 1):
        hlev.append(len(hops))
        for o in ops:
            if o[0] != lv:
                continue
            _, ph, name, x, y, d = o
            n = nf if ph == 0 else nab
            for k in range(n):
                hops.append((base[name] + k, eslot(x, k), eslot(y, k), d + 3 * ph))
    hlev.append(len(hops))
    outslot = []
    for ab in range(nab):
        for cd in range(ncd):
            src = h.ket_final[(cd // nd, cd % nd)]
            if isinstance(src, tuple):
                rn = h.bra_final[(ab // nb, ab % nb)]
                outslot.append(base[rn] + src[1])
            else:
                outslot.append(base[src] + ab)
    assert max(outslot) < hsize and hsize < 65536 and nvslot < 65536
    return dict(L=L, nacc=nacc, nvslot=nvslot, vrec=vrec, vseg=vseg, vtgt=vtgt,
                hsize=hsize, hops=hops, hlev=hlev, outslot=outslot,
                vrr_flops=v.em.flops, hrr_flops=h.em.flops)


VGROUP_SLOT_BUDGET = 2600     # node slots (doubles) the grouped VRR buffers may take per warp


def vrr_group(cls):
    """Primitive quartets the grouped warp form runs through the VRR at once, with its
    program (waves of 32/VG nodes, so a wave of VG quartets fills the warp): the smallest
    of 2, 4, 8 whose program fills at least 95 % of the lanes, or the best within the
    buffer budget.  Returns (VG, program), VG = 1 when no grouped form pays."""
    base = wide_program(cls, 32)
    best, best_eff, best_p = 1, wave_efficiency(base["vrec"], base["vseg"]), base
    if best_eff >= 0.95:
        return 1, base
    for g in (2, 4, 8):
        p = wide_program(cls, 32 // g)
        if g * p["nvslot"] > VGROUP_SLOT_BUDGET:
            break
        e = wave_efficiency(p["vrec"], p["vseg"], g)
        if e > best_eff + 0.02:
            best, best_eff, best_p = g, e, p
        if e >= 0.95:
            break
    return best, best_p


def emit_wide(cls):
    p = wide_program(cls)
    vg, pg = vrr_group(cls)
    tag = "".join(map(str, cls))
    la, lb, lc, ld = cls

    def arr(ctype, name, vals):
        body = ",".join(str(x) for x in vals) if vals else "0"
        return f"__device__ const {ctype} {name}[{max(1, len(vals))}] = {{{body}}};"

    def segs(q):
        return [x for s in q["vseg"] for x in (s[0], s[2], s[3], s[5])]
    hop = [x for o in p["hops"] for x in (o[0] | (o[1] << 16), o[2] | (o[3] << 16))]
    out = [f"// generated by gen_eri.py -- warp program of class ({la}{lb}|{lc}{ld})",
           "#pragma once", "namespace gs {",
           arr("unsigned int __align__(16)", f"w{tag}_vrec", p["vrec"]),
           arr("int", f"w{tag}_vseg", segs(p)),
           arr("unsigned short", f"w{tag}_vtgt", p["vtgt"]),
           arr("unsigned int __align__(16)", f"w{tag}_vrecg", pg["vrec"]),
           arr("int", f"w{tag}_vsegg", segs(pg)),
           arr("unsigned short", f"w{tag}_vtgtg", pg["vtgt"]),
           arr("unsigned int", f"w{tag}_hop", hop),
           arr("int", f"w{tag}_hlev", p["hlev"]),
           arr("unsigned short", f"w{tag}_out", p["outslot"]),
           f"template <> struct WideProg<{la}, {lb}, {lc}, {ld}> {{",
           f"  static constexpr int NVSLOT = {p['nvslot']}, NVSEG = {len(p['vseg'])}, "
           f"VGROUP = {vg};",
           f"  static constexpr int NVSLOT_G = {pg['nvslot']}, NVSEG_G = {len(pg['vseg'])};",
           f"  static constexpr int HSIZE = {p['hsize']}, NHLEV = {len(p['hlev']) - 1};",
           f"  static __device__ const uint4* vrec() {{ return reinterpret_cast<const uint4*>(w{tag}_vrec); }}",
           f"  static __device__ const int* vseg() {{ return w{tag}_vseg; }}",
           f"  static __device__ const unsigned short* vtgt() {{ return w{tag}_vtgt; }}",
           f"  static __device__ const uint4* vrec_g() {{ return reinterpret_cast<const uint4*>(w{tag}_vrecg); }}",
           f"  static __device__ const int* vseg_g() {{ return w{tag}_vsegg; }}",
           f"  static __device__ const unsigned short* vtgt_g() {{ return w{tag}_vtgtg; }}",
           f"  static __device__ const unsigned int* hop() {{ return w{tag}_hop; }}",
           f"  static __device__ const int* hlev() {{ return w{tag}_hlev; }}",
           f"  static __device__ const unsigned short* outslot() {{ return w{tag}_out; }}",
           "};", "}  // namespace gs", ""]
    return "\n".join(out), p


if __name__ == "__main__":
    main()
