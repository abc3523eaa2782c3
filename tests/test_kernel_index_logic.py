"""Index arithmetic of the data-movement kernels, walked on the CPU exactly as the device
code does it (no GPU): the spin-orbital expansion kernels of csrc/transform.cu and the
element decomposition of csrc/symmetry.cu, against the oracle.  Every address the walk
forms is checked against its buffer, so a change to the kernels' indexing is caught here
before it runs on a GPU."""
import numpy as np
import pytest

import oracle
from conftest import golden

THREADS = 256


def slab_of(mo, h, mode, r, s):
    """stage_slab: (live, slab with odd row pitch, pitch); asserts the reads stay in mo."""
    pitch = h | 1
    flat = mo.ravel()
    h2, h3 = h * h, h * h * h
    if mode == 0:
        live, src, si = (r & 1) == (s & 1), (r >> 1) * h3 + (s >> 1) * h2, h
    elif mode == 1:
        live, src, si = (r < h) == (s < h), (r % h) * h3 + (s % h) * h2, h
    else:
        live, src, si = True, (r >> 1) * h3 + (s >> 1) * h, h2
    slab = np.full(h * pitch, np.nan)
    if live:
        for i in range(h):
            idx = src + i * si + np.arange(h)
            assert idx.min() >= 0 and idx.max() < h ** 4
            slab[i * pitch:i * pitch + h] = flat[idx]
    return live, slab, pitch


def pairs_kernel(mo, h, mode):
    """k_spin_expand_pairs, modes 0 and 2, with its (t, k) carry instead of a division."""
    n = 2 * h
    out = np.full(n ** 4, np.nan)
    sign = lambda x: -x if x != 0 else np.copysign(0.0, -np.copysign(1.0, x))  # noqa: E731
    for blk in range(n * n):
        r, s = blk // n, blk % n
        live, slab, pitch = slab_of(mo, h, mode, r, s)
        sp, rp = s & 1, r & 1
        npairs = 2 * h * h
        dt, dk = THREADS // h, THREADS - (THREADS // h) * h
        for tid in range(min(THREADS, npairs)):
            t, k, e = tid // h, tid - (tid // h) * h, tid
            while e < npairs:
                assert t * h + k == e and 0 <= k < h and 0 <= t < n
                tp = t & 1
                if mode == 0:
                    a = slab[(t >> 1) * pitch + k] if live else 0.0
                    x, y = (0.0, a) if tp else (a, 0.0)
                elif sp == rp:
                    d = slab[(t >> 1) * pitch + k] - slab[(t >> 1) + k * pitch] if tp == sp else 0.0
                    x, y = (0.0, d) if sp else (d, 0.0)
                else:
                    a = slab[(t >> 1) * pitch + k] if tp == rp else 0.0
                    b = sign(slab[(t >> 1) + k * pitch]) if tp == sp else 0.0
                    x, y = (b, a) if sp else (a, b)
                o = blk * n * n + 2 * e
                assert o + 1 < n ** 4
                out[o], out[o + 1] = x, y
                k += dk
                t += dt
                if k >= h:
                    k -= h
                    t += 1
                e += THREADS
    return out.reshape((n,) * 4)


def scalar_kernel(mo, h, mode):
    """k_spin_expand (any mode): one warp per output row."""
    n = 2 * h
    out = np.full(n ** 4, np.nan)
    for blk in range(n * n):
        r, s = blk // n, blk % n
        live, slab, pitch = slab_of(mo, h, mode, r, s)
        for t in range(n):
            row = blk * n * n + t * n
            for u in range(n):
                if mode == 0:
                    v = slab[(t >> 1) * pitch + (u >> 1)] if live and (u & 1) == (t & 1) else 0.0
                elif mode == 1:
                    tlo = t < h
                    v = slab[(t if tlo else t - h) * pitch + (u if u < h else u - h)] \
                        if live and (u < h) == tlo else 0.0
                else:
                    a = slab[(t >> 1) * pitch + (u >> 1)] if (r & 1) == (t & 1) and (u & 1) == (s & 1) else 0.0
                    b = slab[(t >> 1) + (u >> 1) * pitch] if (u & 1) == (r & 1) and (s & 1) == (t & 1) else 0.0
                    v = a - b
                out[row + u] = v
    return out.reshape((n,) * 4)


REF = {0: oracle.spin_basis_set, 1: oracle.blocked_spin_basis_set, 2: oracle.spin_basis_anti_physicist}


@pytest.mark.parametrize("h", [1, 2, 3, 5, 17])
def test_spin_pair_kernel_walk(h):
    mo = np.random.default_rng(h).standard_normal((h,) * 4)
    for mode in (0, 2):
        assert np.array_equal(pairs_kernel(mo, h, mode), REF[mode](mo)), mode


@pytest.mark.parametrize("h", [1, 2, 3, 4])
def test_spin_scalar_kernel_walk(h):
    mo = np.random.default_rng(10 + h).standard_normal((h,) * 4)
    for mode in (0, 1, 2):
        assert np.array_equal(scalar_kernel(mo, h, mode), REF[mode](mo)), mode


def test_symmetry_kernel_element_decomposition():
    """k_symmetry_zero's e -> (i, j, k, l) split and test, over every element of O2/STO-3G
    (10 functions), against the oracle on the canonical keys."""
    g = golden("symmetry")
    table, flip = g["o2_table"], g["o2_flip"]
    cid = oracle.centre_ids(g["o2_centre"])
    par = oracle.parity_bits(g["o2_lmn"])
    n, nops = table.shape
    n2 = n * n
    zero = np.zeros(n ** 4, dtype=bool)
    for e in range(n ** 4):
        ij, kl = divmod(e, n2)
        i, j = divmod(ij, n)
        k, l = divmod(kl, n)
        p = par[i] ^ par[j] ^ par[k] ^ par[l]
        if cid[i] == cid[j] == cid[k] == cid[l]:
            zero[e] = p != 0
            continue
        for m in range(nops):
            a, b, c, d = table[i, m], table[j, m], table[k, m], table[l, m]
            if a == 0 or b == 0 or c == 0 or d == 0:
                continue
            w, x, y, z = abs(a) - 1, abs(b) - 1, abs(c) - 1, abs(d) - 1
            if ((i == w and j == x) or (i == x and j == w)) and \
                    ((k == y and l == z) or (k == z and l == y)) and flip[m, p]:
                zero[e] = True
                break
    zero = zero.reshape((n,) * 4)
    keys = oracle.canonical_keys(g["o2_table"].shape[0])
    assert np.array_equal(~zero[keys[:, 0], keys[:, 1], keys[:, 2], keys[:, 3]], g["o2_nonzero"])


def test_pair_queue_compaction():
    """k_pairs_build_compact's queue restated: a warp pushes each chunk's kept candidates
    (ballot-ranked) and evaluates full batches of 32 off the front, then the rest; every
    kept candidate is evaluated exactly once, at its own record slot, and the queue never
    holds more than its 64 entries."""
    rng = np.random.default_rng(11)
    for trial in range(200):
        chunks = [rng.random(32) < rng.uniform(0.05, 0.95) for _ in range(rng.integers(1, 12))]
        q, evaluated, slot, peak = [], [], 0, 0
        for keep in chunks:
            for lane in range(32):           # q[len + rank] = candidate, for kept lanes
                if keep[lane]:
                    q.append(slot)
                    slot += 1
            peak = max(peak, len(q))
            if len(q) >= 32:                 # lane l evaluates q[l]; q[l] = q[l + 32]
                evaluated += q[:32]
                q = q[32:]
            assert len(q) < 32
        evaluated += q                       # the last partial batch
        assert sorted(evaluated) == list(range(slot))
        assert peak <= 64


def test_packed_pair_build_lane_mapping():
    """The grouped pair build's lane mapping restated lane by lane: every primitive pair of every shell pair
    is taken by exactly one lane, and the kept ones land at the same record slots, in the
    same order, as the one-pair-per-warp form (rank among the pair's kept lanes)."""
    from gaussium_gb300.engine import pair_groups
    rng = np.random.default_rng(5)
    ka = rng.integers(1, 7, 400)
    kb = rng.integers(1, 7, 400)
    sizes = ka * kb
    groups = pair_groups(sizes)
    keep = rng.random(int(sizes.sum())) < 0.4
    first_rec = np.concatenate([[0], np.cumsum(sizes)[:-1]])
    got = {}
    for g in range(len(groups) - 1):
        first, np_ = groups[g], groups[g + 1] - groups[g]
        if np_ == 1:
            continue                         # one-pair groups run the one-pair loop
        size = np.zeros(32, dtype=int)
        size[:np_] = sizes[first:first + np_]
        off = np.cumsum(size) - size         # exclusive scan
        total = off[31] + size[31]
        assert total <= 32
        ballot = 0
        lanes = []
        for lane in range(32):
            j = max([q for q in range(np_) if off[q] <= lane] or [0])
            if lane < total:
                k = lane - off[j]
                assert 0 <= k < size[j]
                kp = keep[first_rec[first + j] + k]
                if kp:
                    ballot |= 1 << lane
                lanes.append((lane, j, k, kp))
        for lane, j, k, kp in lanes:
            mask = ((1 << int(size[j])) - 1) << int(off[j])
            if kp:
                rank = bin(ballot & mask & ((1 << lane) - 1)).count("1")
                got[(first + j, rank)] = k
    # the one-pair-per-warp form: kept primitive pairs in increasing k
    for p in range(len(sizes)):
        g = np.searchsorted(groups, p, side="right") - 1
        if groups[g + 1] - groups[g] == 1:
            continue
        ks = np.flatnonzero(keep[first_rec[p]:first_rec[p] + sizes[p]])
        for rank, k in enumerate(ks):
            assert got.pop((p, rank)) == k
    assert not got


def test_heavy_threshold_every_class():
    """The split-form threshold is defined for every built class: at least 32 primitive
    quartets and twice the class's contraction accumulators (its generated NACC)."""
    import os
    import sys
    from gaussium_gb300 import engine
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                                    "gaussium_gb300", "csrc"))
    import gen_eri
    for cls in gen_eri.canonical_classes(2):
        v = gen_eri.VrrGen(cls)
        nacc = len(v.e_targets) * len(v.f_targets)
        assert engine.heavy_threshold(cls) == max(engine.HEAVY_PRIM_QUARTETS, 2 * nacc)


def test_device_pair_groups_match_host():
    """pair_groups_device (torch, here on the CPU) gives the host pair_groups' starts."""
    import torch
    from gaussium_gb300.engine import pair_groups, pair_groups_device
    rng = np.random.default_rng(13)
    for n in (0, 1, 2, 3, 4, 5, 7, 8, 1001, 40000):
        s = rng.integers(1, 40, n)
        got = pair_groups_device(torch.as_tensor(s)).numpy()
        assert np.array_equal(got, pair_groups(s)), n


def _dense_expand_sources(l, quartets):
    """k_dense_expand (csrc/dense.cu) on the CPU, each block element standing for its own
    function quartet: per tensor position, the set of source elements written there."""
    ncart = lambda x: (x + 1) * (x + 2) // 2
    func_off = np.concatenate([[0], np.cumsum([ncart(x) for x in l])])
    n = int(func_off[-1])
    src = {}
    for s in quartets:
        A, B, C, D = (int(x) for x in s)
        na, nb, nc, nd = (ncart(l[x]) for x in (A, B, C, D))
        for e in range(na * nb * nc * nd):
            id_, ic = e % nd, (e // nd) % nc
            ib, ia = (e // (nd * nc)) % nb, e // (nd * nc * nb)
            a, b, c, d = func_off[A] + ia, func_off[B] + ib, func_off[C] + ic, func_off[D] + id_
            if (A == B and a < b) or (C == D and c < d) or \
                    (A == C and B == D and (a < c or (a == c and b < d))):
                continue
            for p in ((a, b, c, d), (b, a, c, d), (a, b, d, c), (b, a, d, c),
                      (c, d, a, b), (d, c, a, b), (c, d, b, a), (d, c, b, a)):
                src.setdefault(tuple(int(x) for x in p), set()).add((a, b, c, d))
    return n, src


def test_dense_expand_one_writer_per_index_orbit():
    """The 8-fold fill of the dense tensor (the reference's create_repulsion_matrix fills
    every position from its canonical key, Symmetry.sort_index, common/symmetry.py:186-197):
    over the unique shell quartets of shells with repeated angular momenta, every position
    is written, by one source element only, from the position's own orbit, and all
    positions of an orbit by the same element."""
    from gaussium_gb300.dropin import unique_shell_quartets
    l = [0, 1, 2, 1, 0]
    n, src = _dense_expand_sources(l, unique_shell_quartets(len(l)))
    assert len(src) == n ** 4
    writer = {}
    for pos, s in src.items():
        assert len(s) == 1, (pos, s)
        (e,) = s
        key = oracle.sort_index(*pos)
        assert oracle.sort_index(*e) == key
        assert writer.setdefault(key, e) == e
