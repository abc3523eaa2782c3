"""One-electron integrals (S, T, V) on the GPU against the reference's own matrices."""
import numpy as np
import pytest

from conftest import golden
from molecules import functions

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["h2o_sto3g", "h2o_631gs", "heh_sto3g", "o2_sto3g"])
def test_overlap_kinetic_nuclear_match_reference(gpu_lib, name):
    from gaussium_gb300.basis import ShellBasis
    from gaussium_gb300.hamiltonian import one_electron
    g = golden(name)
    sb = ShellBasis.from_functions(functions(g))
    S, T, V = one_electron(sb, g["coords"], g["charges"])
    assert np.max(np.abs(S - g["overlap"])) < 1e-12
    assert np.max(np.abs(T - g["kinetic"])) < 1e-11
    # the reference's V uses its Boys series (error ~1e-11 relative, times Z)
    assert np.max(np.abs(V - g["nuclear"])) < 1e-8
