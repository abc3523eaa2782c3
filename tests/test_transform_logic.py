"""The AO -> MO transform's algebra on host tensors (no GPU): the pair index maps and the
pair-packed and quarter-transform GEMM sequences against the oracle's restatement of
matrixelements/transformations.py:5-26.  The public entry points refuse host tensors; these
internal functions are the same torch operations the device path runs."""
import numpy as np
import pytest
import torch

import oracle
from gaussium_gb300 import transform


def symmetric_eri(n, seed):
    x = np.random.default_rng(seed).standard_normal((n, n, n, n))
    x = x + x.transpose(1, 0, 2, 3)
    x = x + x.transpose(0, 1, 3, 2)
    return x + x.transpose(2, 3, 0, 1)


def test_pair_index_maps():
    packed, full = transform._pair_index(5, "cpu")
    assert packed.numel() == 15 and full.numel() == 25
    i, j = packed // 5, packed % 5
    assert torch.all(i >= j)
    f = full.view(5, 5)
    assert torch.equal(f, f.T) and set(f.flatten().tolist()) == set(range(15))
    assert torch.equal(f[i, j], torch.arange(15))


@pytest.mark.parametrize("n,m", [(1, 1), (6, 6), (9, 4)])
def test_pair_packed_and_general_forms_match_oracle(n, m):
    ao = symmetric_eri(n, n)
    c = np.random.default_rng(50 + n).standard_normal((n, m)) / np.sqrt(n)
    ref = np.einsum("abcd,ap,bq,cr,ds->pqrs", ao, c, c, c, c, optimize=True)
    if n == m:
        assert np.max(np.abs(oracle.molecular_orbitals(ao, c) - ref)) <= 1e-12 * np.max(np.abs(ref))
    scale = max(1.0, np.max(np.abs(ref)))
    for form in (transform.transform_pair_symmetric, transform.transform_general):
        got = form(torch.tensor(ao), torch.tensor(c)).numpy()
        assert np.max(np.abs(got - ref)) <= 1e-12 * scale, form.__name__
    got = transform.transform_pair_symmetric(torch.tensor(ao), torch.tensor(c)).numpy()
    assert np.array_equal(got, got.transpose(0, 1, 3, 2))      # mirrored from one triangle


def test_pair_packed_form_needs_only_pair_symmetry():
    """(ab|cd) = (ba|cd) = (ab|dc) without (ab|cd) = (cd|ab) is enough."""
    x = np.random.default_rng(3).standard_normal((5,) * 4)
    x = x + x.transpose(1, 0, 2, 3)
    x = x + x.transpose(0, 1, 3, 2)
    c = np.random.default_rng(4).standard_normal((5, 5))
    got = transform.transform_pair_symmetric(torch.tensor(x), torch.tensor(c)).numpy()
    ref = oracle.molecular_orbitals(x, c)
    assert np.max(np.abs(got - ref)) <= 1e-12 * np.max(np.abs(ref))
