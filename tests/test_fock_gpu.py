"""Integral-direct J/K and the Fock-builder drop-ins on the GPU against the oracle and
the reference's own Fock matrices and SCF energies."""
import numpy as np
import pytest
import torch

import oracle
from conftest import golden
from molecules import load, random_density, functions

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def water631():
    from gaussium_gb300.engine import JKEngine
    from gaussium_gb300.basis import ShellBasis
    g, funcs, table = load("h2o_631gs")
    eri = oracle.dense_tensor(table, boys_mode=1)
    eng = JKEngine(ShellBasis.from_functions(funcs), schwarz_thr=0.0)
    return g, funcs, eri, eng


def _jk_ref(eri, p):
    return np.einsum("kl,ijkl->ij", p, eri), np.einsum("kl,ikjl->ij", p, eri)


@pytest.mark.parametrize("precision,tol", [(64, 1e-12), (32, 2e-5)])
def test_jk_matches_oracle(gpu_lib, water631, precision, tol):
    g, funcs, eri, eng = water631
    p = random_density(eng.sb.nbf, 11)
    pt = torch.tensor(p, device="cuda")
    J, (K,) = eng.jk(pt, [pt], precision=precision)
    jr, kr = _jk_ref(eri, p)
    assert np.max(np.abs(J.cpu().numpy() - jr)) < tol * max(1, np.abs(jr).max())
    assert np.max(np.abs(K.cpu().numpy() - kr)) < tol * max(1, np.abs(kr).max())


def test_jk_two_exchange_densities(gpu_lib, water631):
    g, funcs, eri, eng = water631
    pa, pb = random_density(eng.sb.nbf, 1), random_density(eng.sb.nbf, 2)
    ta, tb = torch.tensor(pa, device="cuda"), torch.tensor(pb, device="cuda")
    J, (Ka, Kb) = eng.jk(ta + tb, [ta, tb])
    jr, ka = _jk_ref(eri, pa + pb)
    _, kb = _jk_ref(eri, pb)
    _, ka = _jk_ref(eri, pa)
    assert np.max(np.abs(J.cpu().numpy() - jr)) < 1e-12
    assert np.max(np.abs(Ka.cpu().numpy() - ka)) < 1e-12
    assert np.max(np.abs(Kb.cpu().numpy() - kb)) < 1e-12


def test_screening_and_mixed_precision_bounds(gpu_lib, water631):
    g, funcs, eri, eng = water631
    p = random_density(eng.sb.nbf, 5) * 0.1
    pt = torch.tensor(p, device="cuda")
    jr, kr = _jk_ref(eri, p)
    J, (K,) = eng.jk(pt, [pt], screen_thr=1e-12)
    assert np.max(np.abs(J.cpu().numpy() - jr)) < 1e-9
    assert np.max(np.abs(K.cpu().numpy() - kr)) < 1e-9
    J, (K,) = eng.jk(pt, [pt], screen_thr=1e-14, mixed_cut=1e-3)
    assert np.max(np.abs(J.cpu().numpy() - jr)) < 1e-7
    assert np.max(np.abs(K.cpu().numpy() - kr)) < 1e-7


def test_fock_dropins_match_reference_fock(gpu_lib):
    from gaussium_gb300.fock import (FockMatrixRestrictedGPU, FockMatrixUnrestrictedGPU,
                                     BlockedFockMatrixUnrestrictedGPU,
                                     RestrictedKohnShamHamiltonianGPU)
    g, funcs, table = load("h2o_sto3g")
    n = len(funcs)
    pa, pb = g["density_a"], g["density_b"]
    h = np.zeros((n, n))
    f = FockMatrixRestrictedGPU(h, funcs).create(pa)
    assert np.max(np.abs(f - g["fock_rhf"])) < 1e-10
    fa, fb = FockMatrixUnrestrictedGPU(h, funcs).create(pa, pb)
    assert np.max(np.abs(fa - g["fock_uhf_a"])) < 1e-10
    assert np.max(np.abs(fb - g["fock_uhf_b"])) < 1e-10
    big = np.block([[pa, np.zeros((n, n))], [np.zeros((n, n)), pb]])
    f2 = BlockedFockMatrixUnrestrictedGPU(np.zeros((2 * n, 2 * n)), funcs).create(big)
    assert np.max(np.abs(f2 - g["fock_guhf"])) < 1e-10
    hc, J, xc = RestrictedKohnShamHamiltonianGPU(h, funcs).create(pa)
    assert np.max(np.abs(J - g["coulomb_ks"])) < 1e-10


def _rhf(name, **kw):
    from gaussium_gb300.fock import FockMatrixRestrictedGPU
    from gaussium_gb300 import scf
    g = golden(name)
    funcs = functions(g)
    hcore = g["kinetic"] + g["nuclear"]
    fb = FockMatrixRestrictedGPU(hcore, funcs, **kw)
    res = scf.restricted_scf(g["overlap"], hcore, int(g["electrons"]), fb, threshold=1e-12)
    return res.energy + scf.nuclear_repulsion(g["charges"], g["coords"]), res, g


@pytest.mark.parametrize("name", ["h2o_sto3g", "h2o_631gs", "heh_sto3g", "heh_6311pgss",
                                  "ethene_321g"])
def test_rhf_energy_matches_reference(gpu_lib, name):
    e, res, g = _rhf(name)
    ref = float(golden("energies")["heh_sto3g_rhf"]) if name == "heh_sto3g" else float(g["energy"])
    assert res.converged
    assert abs(e - ref) < 1e-8


def test_rhf_mixed_incremental_within_1e6(gpu_lib):
    e64, _, _ = _rhf("h2o_631gs")
    em, res, _ = _rhf("h2o_631gs", mixed_cut=1e-4, screen_thr=1e-13, incremental=True)
    assert res.converged
    assert abs(em - e64) < 1e-6


@pytest.mark.parametrize("method", ["uhf", "guhf"])
def test_o2_open_shell_energy(gpu_lib, method):
    from gaussium_gb300.fock import FockMatrixUnrestrictedGPU
    from gaussium_gb300 import scf
    g = golden("o2_sto3g")
    funcs = functions(g)
    hcore = g["kinetic"] + g["nuclear"]
    fb = FockMatrixUnrestrictedGPU(hcore, funcs)
    res = scf.unrestricted_scf(g["overlap"], hcore, int(g["electrons"]), int(g["multiplicity"]), fb)
    e = res.energy + scf.nuclear_repulsion(g["charges"], g["coords"])
    assert abs(e - float(golden("energies")["o2_sto3g_" + method])) < 1e-8
