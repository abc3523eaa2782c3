"""Host logic of the Kohn-Sham exchange-correlation drop-in (no GPU): the quadrature
rules, the functional parameters read from the reference's objects, and install()."""
import math
import types

import numpy as np
import pytest

from gaussium_gb300 import kohnsham


def test_radial_rule_integrates_gaussian_moments():
    r, w = kohnsham.radial_rule(200)
    # int_0^inf r^2 exp(-a r^2) dr = sqrt(pi) / (4 a^1.5)
    for a in (0.3, 1.0, 6.4):
        assert abs(np.sum(w * np.exp(-a * r * r)) - math.sqrt(math.pi) / (4 * a ** 1.5)) < 1e-12


def test_angular_rule_has_degree_35():
    dirs, w = kohnsham.angular_rule()
    assert dirs.shape == (648, 3) and abs(w.sum() - 4 * math.pi) < 1e-13
    assert np.allclose(np.linalg.norm(dirs, axis=1), 1.0)
    x, y, z = dirs.T
    # monomials of even degree up to 34 in each variable: int x^2a y^2b z^2c over the sphere
    def exact(a, b, c):
        g = math.gamma
        return 2 * g(a + .5) * g(b + .5) * g(c + .5) / g(a + b + c + 1.5)
    for a, b, c in ((1, 0, 0), (2, 1, 0), (4, 4, 4), (10, 4, 3), (17, 0, 0), (0, 8, 9)):
        assert abs(np.dot(w, x ** (2 * a) * y ** (2 * b) * z ** (2 * c)) - exact(a, b, c)) < 1e-14
    assert abs(np.dot(w, x * y ** 2 * z ** 3)) < 1e-14


def test_single_centre_grid_is_centred():
    pts, w = kohnsham.single_centre_grid(centre=(1.0, -2.0, 0.5), radial=10)
    assert pts.shape == (6480, 3) and w.shape == (6480,)
    assert np.allclose(np.average(pts, axis=0, weights=w), [1.0, -2.0, 0.5])


def test_functional_params_from_reference_objects():
    slater = types.SimpleNamespace(alpha=0.7)
    vwn = types.SimpleNamespace(a=0.0621814, x_0=-0.10498, b=3.72744, c=12.9352)
    assert kohnsham.functional_params(slater, vwn) == (0.7, kohnsham.VWN5)
    assert kohnsham.functional_params(object(), object()) == (0.0, None)


def test_install_swaps_exchange_correlation():
    from gaussium_gb300 import fock
    hf = types.ModuleType("gaussium.hartreefock.hartree_fock")
    for name in ("TwoElectronRepulsionMatrixOS", "FockMatrixRestricted", "FockMatrixUnrestricted",
                 "BlockedFockMatrixUnrestricted", "blocked_spin_basis_set"):
        setattr(hf, name, object())
    ks = types.ModuleType("gaussium.kohnsham.kohn_sham")
    ks.RestrictedKohnShamHamiltonian = object()
    ks.ExchangeCorrelation = before = object()
    g = types.SimpleNamespace(hartreefock=types.SimpleNamespace(hartree_fock=hf),
                              kohnsham=types.SimpleNamespace(kohn_sham=ks))
    orig = fock.install(g)
    assert ks.ExchangeCorrelation is kohnsham.ExchangeCorrelationGPU
    assert orig[("gaussium.kohnsham.kohn_sham", "ExchangeCorrelation")] is before


def test_xc_drop_in_fails_loudly_without_gpu(monkeypatch):
    import torch
    from gaussium_gb300 import _lib
    monkeypatch.setattr(torch.cuda, "is_available", lambda: False)
    monkeypatch.setattr(_lib, "_LIB", None)
    with pytest.raises((_lib.GsError, RuntimeError, AssertionError)):
        kohnsham.ExchangeCorrelationGPU.__new__(kohnsham.ExchangeCorrelationGPU).functionals(
            torch.zeros(3, dtype=torch.float64), torch.zeros(3, dtype=torch.float64))


def test_ks_scf_loop_reproduces_reference_he_energies():
    """scf.ks_restricted_scf (the product's restatement of KSRestrictedSCF with DIIS) driven
    by the oracle's J and XC on the host reaches the reference's He/STO-3G DFT energies."""
    import oracle
    from conftest import golden
    from gaussium_gb300 import scf
    he = oracle.FunctionTable.from_shells([dict(
        l=0, centre=np.zeros(3), expo=np.array([6.36242139, 1.15892300, 0.31364979]),
        coef=np.array([0.15432897, 0.53532814, 0.44463454]))])
    S, T, V = oracle.one_centre_s(he, 2.0)
    eri = oracle.dense_tensor(he)
    g = golden("xc")
    for vwn, key in ((None, "he_energy_s"), (oracle.VWN3, "he_energy_svwn3")):
        class XC:
            @staticmethod
            def evaluate(p, vwn=vwn):
                return (oracle.xc_potential_matrix(he, p, 2 / 3, vwn),
                        oracle.xc_energy(he, p, 2 / 3, vwn))
        res = scf.ks_restricted_scf(S, T + V, 2, lambda p: oracle.coulomb(eri, p), XC())
        assert res["converged"]
        assert abs(res["energy"] - float(g[key])) < 1e-8, key
