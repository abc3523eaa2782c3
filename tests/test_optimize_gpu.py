"""Gradient-driven optimisation and the restated Nelder-Mead reach the same minimum."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_h2_bfgs_and_nelder_mead_agree(gpu_lib):
    from gaussium_gb300.molecules import Molecule
    from gaussium_gb300.optimize import NelderMead, optimize_bfgs
    from gaussium_gb300.gradient import rhf_energy_gradient
    mol = Molecule(["H", "H"], np.array([[0.0, 0.0, 0.0], [0.0, 0.0, 1.6]]))
    e_b, x_b, n_b, g_b = optimize_bfgs(mol, "6-31G", gtol=1e-6)
    nm = NelderMead(mol.symbols, mol.coords, lambda m: rhf_energy_gradient(m, "6-31G", want_gradient=False)[0],
                    threshold=1e-9)
    e_n, x_n = nm.optimize()
    r_b = np.linalg.norm(x_b[1] - x_b[0])
    r_n = np.linalg.norm(x_n[1] - x_n[0])
    assert abs(e_b - e_n) < 1e-7
    assert abs(r_b - r_n) < 1e-3
    assert n_b < nm.evals
