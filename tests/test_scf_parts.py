"""The restated SCF host functions (``gaussium_gb300.scf``) against the reference's own
outputs on the HeH+ STO-3G inputs of its unit tests (``tests/golden/scf_parts.npz``, made
by ``tests/golden/make_scf_parts.py``).  The reference's tests pin these values to 3-6
significant figures.  The restatement is held to rounding: the total energy, density
and orbital energies to 1e-13, the orthogonaliser and orbital coefficients to 1e-12.
Columns are compared up to sign, since an eigenvector's sign is arbitrary."""
import numpy as np

from conftest import golden
from gaussium_gb300 import scf


def _same_up_to_column_sign(a, b, tol):
    for j in range(a.shape[1]):
        s = 1.0 if np.dot(a[:, j], b[:, j]) >= 0 else -1.0
        if np.max(np.abs(a[:, j] - s * b[:, j])) > tol:
            return False
    return True


def test_total_energy_restricted():
    """hartreefock/total_energy.py:16-35 on test_total_energy.py's P, H and F."""
    g = golden("scf_parts")
    e = scf.total_energy_restricted(g["H"], g["P"], g["F"])
    assert abs(e - float(g["energy"])) < 1e-13
    assert abs(e - (-4.14186)) < 5e-6                    # the reference test's 6 figures


def test_canonical_orthogonalisation_and_diagonalisation():
    """hartreefock/linear_algebra.py:6-25 on test_linear_algebra.py's S and H."""
    g = golden("scf_parts")
    la = scf.LinearAlgebra(g["S"])
    assert _same_up_to_column_sign(la.transformation_matrix, g["X"], 1e-12)
    eps, c = la.diagonalize(g["H"])
    assert np.max(np.abs(eps - g["eps"])) < 1e-13
    assert _same_up_to_column_sign(c, g["Cd"], 1e-12)
    # orthonormal in the overlap metric, as any canonical orthogonaliser must be
    assert np.allclose(c.T @ g["S"] @ c, np.eye(2), atol=1e-13)


def test_density_matrix_restricted():
    """matrixelements/density_matrix.py:4-9 on test_density_matrix.py's coefficients."""
    g = golden("scf_parts")
    d = scf.density_matrix_restricted(g["C"], 2)
    assert np.max(np.abs(d - g["D"])) < 1e-13


def test_nuclear_repulsion_two_nuclei():
    """common/nuclear_repulsion.py:5-24 on the two pairs of the reference's
    tests/testsfast/common/test_nuclear_repulsion.py:9-21 (H2 and HeH at +-z, bohr): the
    sum over pairs equals the one pair's Z_a Z_b / r, which the reference pins to 4 and 7
    figures."""
    for z, half, want, digits in (((1.0, 1.0), (0.70, -0.70), 0.7143, 4),
                                  ((1.0, 2.0), (0.7316, -0.7316), 1.366867, 7)):
        coords = np.array([[0.0, 0.0, half[0]], [0.0, 0.0, half[1]]])
        e = scf.nuclear_repulsion(np.array(z), coords)
        assert abs(e - z[0] * z[1] / (half[0] - half[1])) < 1e-15
        assert abs(e - want) <= 0.5 * 10.0 ** (np.floor(np.log10(abs(want))) - digits + 1)
