"""Point-group zero screening on the GPU (``gs_symmetry_zero`` through the drop-in) against
the reference's own none_zero_integral on every canonical key (tests/golden/symmetry.npz,
made by tests/golden/make_symmetry_golden.py)."""
import numpy as np
import pytest
import torch

import oracle
from conftest import golden
from molecules import functions
from test_symmetry_logic import fake_reference_symmetry

pytestmark = pytest.mark.gpu


def system_functions(g, name):
    keys = ("centre", "lmn", "norm", "nprim", "coef", "expo", "pnorm")
    return functions({k: g[f"{name}_{k}"] for k in keys})


@pytest.mark.parametrize("name", ["ethene", "water", "o2"])
def test_kernel_zeroes_exactly_the_reference_zeros(gpu_lib, name):
    from gaussium_gb300 import dropin
    g = golden("symmetry")
    sym, funcs = fake_reference_symmetry(g, name)
    n = len(funcs)
    t = torch.ones((n, n, n, n), dtype=torch.float64, device="cuda")
    dropin.symmetry_zero(t, *dropin.symmetry_tables(sym, funcs))
    keys = torch.as_tensor(oracle.canonical_keys(g[f"{name}_table"].shape[0]).astype(np.int64)).cuda()
    got = t[keys[:, 0], keys[:, 1], keys[:, 2], keys[:, 3]].cpu().numpy()
    assert np.array_equal(got == 1.0, g[f"{name}_nonzero"])
    # every permutation of a key agrees with the key (the reference's 8-fold expansion)
    for perm in ((1, 0, 2, 3), (0, 1, 3, 2), (2, 3, 0, 1)):
        assert torch.equal(t, t.permute(*perm))
    assert int((t == 0).sum()) > 0


def test_drop_in_tensor_with_symmetry(gpu_lib):
    """TwoElectronRepulsionGPU with the reference's Symmetry (ethene/3-21G, D2h): the
    screened tensor is the unscreened one with exactly the reference's zeros."""
    from gaussium_gb300.dropin import TwoElectronRepulsionGPU
    g = golden("symmetry")
    sym, _ = fake_reference_symmetry(g, "ethene")
    funcs = system_functions(g, "ethene")
    full = TwoElectronRepulsionGPU(funcs, None, None, 1).create_repulsion_matrix()
    screened = TwoElectronRepulsionGPU(funcs, None, sym, 1).create_repulsion_matrix()
    k = oracle.canonical_keys(g["ethene_table"].shape[0])
    nz = g["ethene_nonzero"]
    vals = screened[k[:, 0], k[:, 1], k[:, 2], k[:, 3]]
    assert np.all(vals[~nz] == 0.0)
    assert np.array_equal(vals[nz], full[k[nz, 0], k[nz, 1], k[nz, 2], k[nz, 3]])
    # what the screen removes is zero by symmetry indeed, to the integrals' accuracy
    assert np.max(np.abs(full[k[~nz, 0], k[~nz, 1], k[~nz, 2], k[~nz, 3]])) < 1e-10
