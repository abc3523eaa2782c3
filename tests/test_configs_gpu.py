"""The parity bars of the workloads the engine is measured on, each on its own workload:

  * the 2,000,000-quartet microbench: every ERI of a seeded sample of 4,096 of its shell
    quartets within 1e-10 absolute of the exact-Boys oracle (K up to 6 per shell);
  * the synthetic K = 1-6 golden: the reference's own ObaraSaika values;
  * (H2O)8 / 6-31G* RHF: mixed-precision incremental Fock builds within 1e-6 Eh of the
    all-FP64 energy, with and without a final FP64 build;
  * (H2O)8 / 6-31G: analytic gradient against central finite differences (h = 1e-4 bohr)
    of the FP64 energy on 12 seeded coordinates, to 1e-6 Eh/bohr;
  * water / 6-31G and 6-31G*: analytic gradient against the reference's own energy
    differentiated numerically (tests/golden/make_golden.py, gradient_fd);
  * 256 seeded C/H/N/O chain molecules / 6-31G*, batched mixed-precision SCF: 32 of them
    against one-molecule-at-a-time FP64 RHF, within 1e-6 Eh.

Reference anchors: matrixelements/electron_repulsion_matrix.py:18-47 (ERIs),
hartreefock/fock_matrix.py:12-22 and hartreefock/scf_procedure.py:24-42 (Fock builds and
SCF), geometryoptimization/nelder_mead.py:126-144 (the energies the gradient replaces)."""
import os

import numpy as np
import pytest
import torch

import oracle
from conftest import golden, synthetic_shells

pytestmark = pytest.mark.gpu


def _function_table(sb, shells):
    from gaussium_gb300.basis import COMPONENTS
    centre, lmn, cnorm, prims, row = [], [], [], [], {}
    for s in shells:
        k0, k1 = sb.prim_off[s], sb.prim_off[s + 1]
        row[int(s)] = len(centre)
        for ci, c in enumerate(COMPONENTS[int(sb.l[s])]):
            centre.append(sb.centre[s]); lmn.append(c); cnorm.append(sb.comp_scale[s, ci])
            prims.append(list(zip(sb.coef[k0:k1], sb.expo[k0:k1], np.ones(k1 - k0))))
    return oracle.FunctionTable(np.array(centre), np.array(lmn), np.array(cnorm), prims), row


def test_microbench_4096_quartets_within_1e10_absolute(gpu_lib):
    """4,096 seeded quartets of the 2M microbench batch, every element against the
    exact-Boys oracle: |GPU - oracle| <= 1e-10 absolute."""
    from gaussium_gb300 import engine
    from gaussium_gb300.basis import COMPONENTS
    from gaussium_gb300.workloads import random_shell_quartets
    sb, q, _ = random_shell_quartets(2_000_000, seed=0)
    pick = np.sort(np.random.default_rng(12).choice(len(q), size=4096, replace=False))
    ds = engine.DeviceShells(sb)
    batch = engine.QuartetBatch(ds, q[pick], want32=False, max_exp=engine.PRIM_SCREEN)
    out = torch.empty(batch.total, dtype=torch.float64, device="cuda")
    batch.run(out, 64)
    got = out.cpu().numpy()
    table, row = _function_table(sb, np.unique(q[pick].ravel()))
    fq = []
    for a, b, c, d in q[pick]:
        n = [len(COMPONENTS[int(sb.l[x])]) for x in (a, b, c, d)]
        fq.append(np.stack(np.meshgrid(*[row[int(x)] + np.arange(k) for x, k in
                                         zip((a, b, c, d), n)], indexing="ij"), -1).reshape(-1, 4))
    ref = oracle.eri_functions(table, np.concatenate(fq), boys_mode=1)
    err = np.abs(got - ref)
    kmax = int(sb.nprim[q[pick]].max())
    print(f"\n4096 microbench quartets ({len(ref)} integrals, K up to {kmax}): "
          f"max |err| {err.max():.3e}, max |ERI| {np.abs(ref).max():.3e}")
    assert kmax == 6
    assert err.max() <= 1e-10


@pytest.mark.parametrize("precision", [64, 32])
def test_synthetic_k6_golden(gpu_lib, precision):
    """The reference's ObaraSaika values for K = 1-6 (and K = 6 on all four shells) in
    every canonical class: FP64 within the reference's own Boys error (its series stops
    at a term below 1e-10) and within 1e-10 absolute of the exact-Boys oracle; FP32
    within 1e-4 of the golden's largest value (the tolerance of every FP32 class test)."""
    from gaussium_gb300 import engine
    from gaussium_gb300.basis import ShellBasis
    g = golden("synthetic_k6")
    shells = synthetic_shells("synthetic_k6")
    sb = ShellBasis.from_shell_dicts(shells)
    table = oracle.FunctionTable.from_shells(shells)
    out, off = engine.eri_blocks(sb, g["quartets"], precision=precision)
    ncomp = [len(oracle.COMPONENTS[s["l"]]) for s in shells]
    got = []
    for si, qi in enumerate(g["sample_quartet"]):
        q = g["quartets"][qi]
        n = [ncomp[x] for x in q]
        c = g["sample_comp"][si]
        got.append(out[off[qi] + ((c[0] * n[1] + c[1]) * n[2] + c[2]) * n[3] + c[3]])
    got = np.array(got)
    if precision == 64:
        assert np.max(np.abs(got - g["os"])) < 1e-9
        fo = np.concatenate([[0], np.cumsum(ncomp)])
        fq = np.array([[fo[g["quartets"][qi][k]] + g["sample_comp"][si][k] for k in range(4)]
                       for si, qi in enumerate(g["sample_quartet"])])
        assert np.max(np.abs(got - oracle.eri_functions(table, fq, boys_mode=1))) < 1e-10
    else:
        assert np.max(np.abs(got - g["os"])) < 1e-4 * np.abs(g["os"]).max()


@pytest.fixture(scope="module")
def water8_631gs():
    from gaussium_gb300 import driver, molecules
    from gaussium_gb300.engine import JKEngine
    mol = molecules.water_cluster(8, seed=8)
    eng = JKEngine(molecules.shell_basis(mol, "6-31G*"), schwarz_thr=1e-12)
    r64 = driver.rhf(mol, engine=eng, threshold=1e-10)
    return mol, eng, r64


@pytest.mark.parametrize("final_fp64", [True, False])
def test_water8_mixed_incremental_within_1e6(gpu_lib, water8_631gs, final_fp64):
    """(H2O)8 / 6-31G* (152 functions), Schwarz 1e-12: mixed FP32/FP64 incremental builds
    with density screening at 1e-12 against the all-FP64 SCF.  Without the final FP64
    build the reported energy is that of the mixed builds themselves, so their FP32 error
    shows in full."""
    from gaussium_gb300 import driver
    mol, eng, r64 = water8_631gs
    rmx = driver.rhf(mol, engine=eng, threshold=1e-10, mixed_cut=1e-2, screen_thr=1e-12,
                     incremental=True, final_fp64=final_fp64)
    de = abs(rmx["energy"] - r64["energy"])
    print(f"\n(H2O)8/6-31G* mixed incremental (final FP64 build: {final_fp64}): "
          f"|dE| = {de:.3e} Eh over {len(rmx['fock_seconds'])} builds")
    assert r64["converged"] and rmx["converged"]
    assert de <= 1e-6


def test_water8_gradient_against_finite_differences(gpu_lib):
    """(H2O)8 / 6-31G (104 functions): the analytic gradient (one-electron derivative
    kernel, ERI adjoint kernels, nuclear repulsion) on 12 seeded coordinates against
    central differences of the converged FP64 energy, h = 1e-4 bohr."""
    from gaussium_gb300 import molecules
    from gaussium_gb300.gradient import rhf_energy_gradient
    from gaussium_gb300.molecules import Molecule
    mol = molecules.water_cluster(8, seed=8)
    _, g, _ = rhf_energy_gradient(mol, "6-31G", threshold=1e-12)
    rng = np.random.default_rng(8)
    coords = rng.choice(mol.coords.size, size=12, replace=False)
    h, worst = 1e-4, 0.0
    for c in coords:
        a, x = divmod(int(c), 3)
        e = []
        for sign in (1.0, -1.0):
            xyz = mol.coords.copy()
            xyz[a, x] += sign * h
            e.append(rhf_energy_gradient(Molecule(mol.symbols, xyz), "6-31G", threshold=1e-12,
                                         want_gradient=False)[0])
        worst = max(worst, abs(g[a, x] - (e[0] - e[1]) / (2 * h)))
    print(f"\n(H2O)8/6-31G gradient vs central differences on 12 coordinates: max {worst:.2e}")
    assert worst <= 1e-6


@pytest.mark.parametrize("basis", ["6-31G", "6-31G*"])
def test_water_gradient_against_reference_energy_differences(gpu_lib, basis):
    """Water off equilibrium: the analytic gradient against the reference's own RHF
    energies at +-1e-4 bohr per coordinate, differentiated numerically."""
    from gaussium_gb300.gradient import rhf_energy_gradient
    from gaussium_gb300.molecules import Molecule
    g = golden("gradient_fd")
    tag = basis.replace("*", "s").replace("-", "")
    e, grad, _ = rhf_energy_gradient(Molecule(["O", "H", "H"], g["coords"]), basis,
                                     threshold=1e-12)
    assert abs(e - float(g[f"energy_{tag}"])) < 1e-8
    err = np.max(np.abs(grad - g[f"fd_gradient_{tag}"]))
    print(f"\nwater/{basis} gradient vs the reference's energy differences: max {err:.2e}")
    assert err <= 1e-6


def test_batch256_sample_against_single_molecule_fp64(gpu_lib):
    """256 seeded C/H/N/O chains / 6-31G*, batched SCF with graph-captured mixed-precision
    incremental Fock builds; 32 of them (every 8th) against one-molecule FP64 RHF."""
    from gaussium_gb300 import batch, driver, molecules
    mols = [molecules.random_chain(s) for s in range(256)]
    eng = batch.BatchedRHF(mols)
    e, _ = eng.run(threshold=1e-10, mixed_cut=1e-2, screen_thr=1e-12, incremental=True,
                   guess="sad")
    conv = eng.converged.copy()
    checked, worst = 0, 0.0
    for i in range(0, 256, 8):
        r = driver.rhf(mols[i], threshold=1e-10, max_iter=200)
        if not (r["converged"] and conv[i]):
            continue
        checked += 1
        worst = max(worst, abs(e[i] - r["energy"]))
    print(f"\n256-molecule batch: {int(conv.sum())} converged; {checked} of 32 sampled "
          f"molecules checked, max |dE| vs single FP64 {worst:.2e} Eh")
    assert checked >= 28
    assert worst <= 1e-6
