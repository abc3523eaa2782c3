"""Test helper: ctypes front end of the CPU build of the generated recursions
(gaussium_gb300/csrc/hostcheck.cpp), plus canonical-block reference data from the oracle."""
import ctypes

import numpy as np

from gaussium_gb300 import build
from gaussium_gb300.basis import COMPONENTS
from gaussium_gb300.engine import PAIR_ORDER

PAIR = np.dtype([("AB", "f8", 3), ("prim_off", "i4"), ("nprim", "i4"), ("sa", "i4"), ("sb", "i4"),
                 ("qmax", "f4"), ("pad", "i4")])
_hc = None


def hc():
    global _hc
    if _hc is None:
        L = ctypes.CDLL(build.build_hostcheck())
        V, I = ctypes.c_void_p, ctypes.c_int
        L.hc_make_pairs.argtypes = [I] + [V] * 10
        L.hc_eri_block.argtypes = [I] * 5 + [V, V, I, I, V]
        L.hc_boys.argtypes = [I, I, ctypes.c_double, V]
        _hc = L
    return _hc


def make_pairs(sb, pairs):
    pairs = np.ascontiguousarray(pairs, dtype=np.int32)
    npp = sb.nprim[pairs[:, 0]] * sb.nprim[pairs[:, 1]]
    off = np.concatenate([[0], np.cumsum(npp)[:-1]]).astype(np.int32)
    pr = np.zeros(len(pairs), dtype=PAIR)
    pd = np.zeros((int(npp.sum()), 10))
    pf = np.zeros((int(npp.sum()), 12), dtype=np.float32)
    hc().hc_make_pairs(len(pairs), pairs.ctypes.data, off.ctypes.data, sb.centre.ctypes.data,
                       sb.l.ctypes.data, sb.prim_off.ctypes.data, sb.expo.ctypes.data,
                       sb.coef.ctypes.data, pr.ctypes.data, pd.ctypes.data, pf.ctypes.data)
    return pr, pd, pf


def canonical_block(sb, quartet, precision):
    """Canonical block of one shell quartet through the generated code on the CPU, scaled
    by the per-component factors; returns (block, canonical shells)."""
    a, b, c, d = (int(x) for x in quartet)
    la, lb, lc, ld = (int(sb.l[x]) for x in (a, b, c, d))
    if la < lb:
        a, b, la, lb = b, a, lb, la
    if lc < ld:
        c, d, lc, ld = d, c, ld, lc
    if PAIR_ORDER.index((lc, ld)) > PAIR_ORDER.index((la, lb)):
        a, b, c, d, la, lb, lc, ld = c, d, a, b, lc, ld, la, lb
    pr, pd, pf = make_pairs(sb, [(a, b), (c, d)])
    n = [len(COMPONENTS[x]) for x in (la, lb, lc, ld)]
    out = np.zeros(int(np.prod(n)))
    rc = hc().hc_eri_block(la, lb, lc, ld, precision, pr.ctypes.data,
                           (pd if precision == 64 else pf).ctypes.data, 0, 1, out.ctypes.data)
    assert rc == 0
    blk = out.reshape(n)
    s = [sb.comp_scale[x][:k] for x, k in zip((a, b, c, d), n)]
    blk = blk * s[0][:, None, None, None] * s[1][None, :, None, None] * \
        s[2][None, None, :, None] * s[3][None, None, None, :]
    return blk, (a, b, c, d)


def function_quartets(sb, shells):
    fo = [int(sb.func_off[x]) for x in shells]
    n = [len(COMPONENTS[int(sb.l[x])]) for x in shells]
    return np.array([(fo[0] + i, fo[1] + j, fo[2] + k, fo[3] + l) for i in range(n[0])
                     for j in range(n[1]) for k in range(n[2]) for l in range(n[3])])
