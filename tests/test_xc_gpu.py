"""LDA exchange-correlation on the GPU (``gs_basis_on_grid``, ``gs_lda_xc`` and the
``ExchangeCorrelationGPU`` drop-in) against the reference's own outputs
(tests/golden/xc.npz, made by tests/golden/make_xc_golden.py) and the oracle's
restatement of kohnsham/."""
import numpy as np
import pytest
import torch

import oracle
from conftest import golden
from molecules import load

pytestmark = pytest.mark.gpu


def lda(gpu_lib, rho, alpha, vwn):
    from gaussium_gb300 import _lib
    r = torch.tensor(rho, dtype=torch.float64, device="cuda")
    w = torch.ones_like(r)
    wv, we = torch.empty_like(r), torch.empty_like(r)
    a, x0, b, c = vwn if vwn is not None else (0.0, 0.0, 0.0, 1.0)
    _lib.check(gpu_lib.gs_lda_xc(len(rho), _lib.ptr(r), _lib.ptr(w), alpha, int(vwn is not None),
                                 a, x0, b, c, _lib.ptr(wv), _lib.ptr(we), _lib.stream()), "lda")
    return wv.cpu().numpy(), we.cpu().numpy()


@pytest.mark.parametrize("alpha,vwn,tags", [
    (2 / 3, None, ("slater_s",)), (0.7, None, ("slater_xa",)),
    (0.0, oracle.VWN3, ("vwn3",)), (0.0, oracle.VWN5, ("vwn5",)),
    (2 / 3, oracle.VWN3, ("slater_s", "vwn3")), (0.7, oracle.VWN5, ("slater_xa", "vwn5"))])
def test_functionals_match_reference(gpu_lib, alpha, vwn, tags):
    g = golden("xc")
    d = g["density"]
    v, e = lda(gpu_lib, d, alpha, vwn)
    v_ref = sum(g[f"{t}_potential"] for t in tags)
    e_ref = d * sum(g[f"{t}_energy"] for t in tags)
    # VWN subtracts nearly equal log / arctan terms: one ulp in one of them moves the result
    # by up to 1.9e-14 relative (measured on the host over these densities), and CUDA's
    # log, atan and cbrt differ from numpy's by a few ulp, hence 2e-12
    m = d > 0
    for got, ref in ((v, v_ref), (e, e_ref)):
        rel = np.max(np.abs(got[m] - ref[m]) / np.abs(ref[m]))
        assert rel < 2e-12, rel
    assert v[0] == 0.0 and e[0] == 0.0           # zero density contributes nothing


def test_functionals_edge_densities(gpu_lib):
    """Negative (rounding) and subnormal densities contribute nothing and stay finite."""
    v, e = lda(gpu_lib, np.array([-1e-18, 5e-320, 1e-299, 1e-20]), 2 / 3, oracle.VWN5)
    assert np.all(np.isfinite(v)) and np.all(np.isfinite(e))
    assert v[0] == v[1] == 0.0 and e[0] == e[1] == 0.0
    assert v[2] != 0.0 and v[3] != 0.0


def test_bad_vwn_fit_is_rejected(gpu_lib):
    from gaussium_gb300 import _lib
    x = torch.ones(4, dtype=torch.float64, device="cuda")
    rc = gpu_lib.gs_lda_xc(4, _lib.ptr(x), _lib.ptr(x), 0.0, 1, 0.06, -0.1, 10.0, 1.0,
                           _lib.ptr(x), _lib.ptr(x), _lib.stream())
    assert rc == 1


@pytest.mark.parametrize("name", ["h2o_sto3g", "h2o_631gs"])
def test_basis_on_grid_matches_oracle(gpu_lib, name):
    from gaussium_gb300.basis import ShellBasis
    from gaussium_gb300.kohnsham import ExchangeCorrelationGPU
    _, funcs, table = load(name)
    xc = ExchangeCorrelationGPU(ShellBasis.from_functions(funcs), params=(2 / 3, None), radial=4)
    pts = np.random.default_rng(5).uniform(-4, 4, size=(3000, 3))
    got = xc.basis_on(torch.tensor(pts, device="cuda")).cpu().numpy()
    ref = oracle.basis_values(table, pts)
    assert np.max(np.abs(got - ref)) <= 1e-14 * max(1.0, np.max(np.abs(ref)))


def test_electron_density_matches_reference(gpu_lib):
    from gaussium_gb300.kohnsham import ExchangeCorrelationGPU
    g = golden("xc")
    _, funcs, _ = load("h2o_sto3g")
    xc = ExchangeCorrelationGPU(funcs, params=(2 / 3, None), radial=4)
    got = np.array([xc.electron_density(g["pmat"], *p) for p in g["points"]])
    assert np.max(np.abs(got - g["rho"])) < 1e-14          # rho up to 0.19; GEMM vs loop order


def he_functions(basis):
    from gaussium_gb300.molecules import Molecule, basis_functions
    return basis_functions(Molecule(["He"], np.zeros((1, 3))), basis)


@pytest.mark.parametrize("vwn,key", [(None, "he_energy_s"), (oracle.VWN3, "he_energy_svwn3")])
def test_he_dft_energy_matches_reference(gpu_lib, vwn, key):
    """The reference's own DFT test values (He/STO-3G, 6 s.f.); the oracle gets 4e-10."""
    from gaussium_gb300 import kohnsham
    from gaussium_gb300.molecules import Molecule
    res = kohnsham.rks(Molecule(["He"], np.zeros((1, 3))), "STO-3G", 2 / 3, vwn)
    assert res["converged"]
    assert abs(res["energy"] - float(golden("xc")[key])) < 1e-8


@pytest.mark.parametrize("symbol,basis,vwn", [("He", "6-31G*", oracle.VWN5), ("O", "STO-3G", oracle.VWN3)])
def test_xc_matrix_and_energy_match_oracle_quadrature(gpu_lib, symbol, basis, vwn):
    """Atom at the origin (the reference's use), a non-spherical density matrix: the GPU's
    fixed radial grid against the oracle's adaptive quad with the same angular rule."""
    from gaussium_gb300.basis import ShellBasis
    from gaussium_gb300.kohnsham import ExchangeCorrelationGPU
    from gaussium_gb300.molecules import Molecule, basis_functions
    funcs = basis_functions(Molecule([symbol], np.zeros((1, 3))), basis)
    sb = ShellBasis.from_functions(funcs)
    table = oracle.FunctionTable(
        np.array([f.coordinates for f in funcs]), np.array([f.integral_exponents for f in funcs]),
        np.array([f.normalisation for f in funcs]),
        [[(p.contraction, p.exponent, p.normalisation) for p in f.primitive_gaussian_array]
         for f in funcs])
    n = sb.nbf
    a = np.random.default_rng(n).standard_normal((n, n)) * 0.4
    P = a @ a.T
    xc = ExchangeCorrelationGPU(sb, params=(2 / 3, vwn))
    V, E = xc.evaluate(P)
    V_ref = oracle.xc_potential_matrix(table, P, 2 / 3, vwn)
    E_ref = oracle.xc_energy(table, P, 2 / 3, vwn)
    assert np.max(np.abs(V - V_ref)) < 1e-8 * max(1.0, np.max(np.abs(V_ref)))
    assert abs(E - E_ref) < 1e-8 * max(1.0, abs(E_ref))
    assert np.array_equal(V, V.T)
    # the reference's element-wise surface reads the same matrix
    assert xc.integrate_potential(P, 0, n - 1) == V[0, n - 1]
    assert xc.integrate_energy(P) == E


def test_ks_hamiltonian_drop_in_uses_whole_matrix(gpu_lib):
    from gaussium_gb300.fock import RestrictedKohnShamHamiltonianGPU
    from gaussium_gb300.kohnsham import ExchangeCorrelationGPU
    from gaussium_gb300.molecules import Molecule, basis_functions
    funcs = basis_functions(Molecule(["O"], np.zeros((1, 3))), "STO-3G")
    n = len(funcs)
    P = np.eye(n) * 0.5
    xc = ExchangeCorrelationGPU(funcs, params=(2 / 3, oracle.VWN5))
    h = RestrictedKohnShamHamiltonianGPU(np.zeros((n, n)), funcs, xc)
    core, J, XC = h.create(P)
    assert np.array_equal(XC, xc.potential_matrix(P))
    assert J.shape == (n, n)
