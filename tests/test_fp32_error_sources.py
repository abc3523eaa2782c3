"""Where the FP32 quartets' error comes from, on the CPU build of the generated recursions.

The FP32 path evaluates the Boys function below its asymptotic threshold (series and
downward recursion) in FP64 and every other stage in FP32.  Over a seeded sample of the
microbench's shell quartets (l uniform over s/p/d, K 1-6, exponents 0.05-1e4, centres in a
10 A cube), the errors against the FP64 blocks, scaled by the sample's largest integral,
are compared across variants that change one stage at a time:
  * the library's FP32 path;
  * the same with the horizontal recursion in FP64 (HRR's share);
  * the same with the Boys function in FP32 as well (the FP64 Boys' gain);
  * FP64 arithmetic on the FP32-rounded primitive-pair records (input rounding only).
At the 99.9th percentile the vertical recursion's FP32 arithmetic carries the error:
moving the HRR or the Boys function to the other precision changes it by a few per cent,
and the rounding of the inputs alone is two orders of magnitude smaller."""
import ctypes

import numpy as np

import hostcheck
from gaussium_gb300.basis import COMPONENTS
from gaussium_gb300.engine import PAIR_ORDER
from gaussium_gb300.workloads import random_shell_quartets


def _blocks(n, seed):
    L = hostcheck.hc()
    f = L.hc_eri_block_f32_mode
    f.argtypes = [ctypes.c_int] * 5 + [ctypes.c_void_p] * 2 + [ctypes.c_int] * 2 + [ctypes.c_void_p]
    sb, q, _ = random_shell_quartets(n, seed=seed)
    ref, outs = [], {m: [] for m in range(4)}
    for quart in q:
        a, b, c, d = (int(x) for x in quart)
        la, lb, lc, ld = (int(sb.l[x]) for x in (a, b, c, d))
        if la < lb:
            a, b, la, lb = b, a, lb, la
        if lc < ld:
            c, d, lc, ld = d, c, ld, lc
        if PAIR_ORDER.index((lc, ld)) > PAIR_ORDER.index((la, lb)):
            a, b, c, d, la, lb, lc, ld = c, d, a, b, lc, ld, la, lb
        pr, pd, pf = hostcheck.make_pairs(sb, [(a, b), (c, d)])
        o = np.zeros(int(np.prod([len(COMPONENTS[x]) for x in (la, lb, lc, ld)])))
        assert L.hc_eri_block(la, lb, lc, ld, 64, pr.ctypes.data, pd.ctypes.data, 0, 1,
                              o.ctypes.data) == 0
        ref.append(o.copy())
        for m in range(4):
            assert f(la, lb, lc, ld, m, pr.ctypes.data, pf.ctypes.data, 0, 1, o.ctypes.data) == 0
            outs[m].append(o.copy())
    ref = np.concatenate(ref)
    return ref, {m: np.concatenate(v) for m, v in outs.items()}


def test_fp32_error_sources():
    ref, outs = _blocks(6000, seed=3)
    scale = np.abs(ref).max()
    p999 = {m: float(np.quantile(np.abs(o - ref) / scale, 0.999)) for m, o in outs.items()}
    lib, hrr64, boys32, inputs = p999[0], p999[1], p999[2], p999[3]
    assert lib < 1e-6
    assert abs(hrr64 - lib) < 0.2 * lib          # HRR in FP64: a few per cent
    assert abs(boys32 - lib) < 0.2 * lib         # Boys in FP32: a few per cent
    assert inputs < 0.05 * lib                   # input rounding alone: far below
