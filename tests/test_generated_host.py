"""The generated VRR/HRR code and the Boys function compiled for the CPU (same sources as
the sm_103a kernels) against the oracle.  Catches generator errors without a GPU."""
import numpy as np
import pytest

import oracle
from conftest import synthetic_shells, golden
from gaussium_gb300.basis import ShellBasis
import hostcheck


@pytest.fixture(scope="module")
def synth():
    shells = synthetic_shells()
    return ShellBasis.from_shell_dicts(shells), oracle.FunctionTable.from_shells(shells), golden("synthetic")


@pytest.mark.parametrize("precision,rtol,atol", [(64, 1e-11, 1e-13), (32, 1e-4, 1e-8)])
def test_every_class_matches_oracle(synth, precision, rtol, atol):
    sb, table, g = synth
    seen = set()
    for q in g["quartets"]:
        blk, canon = hostcheck.canonical_block(sb, q, precision)
        ref = oracle.eri_functions(table, hostcheck.function_quartets(sb, canon), boys_mode=1)
        ref = ref.reshape(blk.shape)
        tol = atol + rtol * np.max(np.abs(ref))
        assert np.max(np.abs(blk - ref)) <= tol
        seen.add(tuple(int(sb.l[x]) for x in canon))
    assert len(seen) == 21


def test_boys_host_matches_exact():
    g = golden("boys")
    h = hostcheck.hc()
    for M in (0, 3, 8, 10):
        F = np.zeros(M + 1)
        for x in g["x"]:
            h.hc_boys(M, 64, float(x), F.ctypes.data)
            ex = np.array([oracle.boys_exact(m, x) for m in range(M + 1)])
            assert np.max(np.abs(F - ex) / ex) < 5e-14, (M, x)


def test_boys_host_fp32_matches_exact():
    """The FP32 quartets' Boys function: FP64 grid expansion and downward recursion below
    the order's asymptotic threshold, FP32 asymptotic form above it; every order within
    2e-6 relative (1e-30 absolute, for values below float range) of the exact value at the
    double argument, as the device test asks."""
    g = golden("boys")
    h = hostcheck.hc()
    for M in range(11):
        F = np.zeros(M + 1)
        for x in g["x"]:
            h.hc_boys(M, 32, float(x), F.ctypes.data)
            ex = np.array([oracle.boys_exact(m, x) for m in range(M + 1)])
            assert np.all(np.abs(F - ex) <= 1e-30 + 2e-6 * np.abs(ex)), (M, x)
