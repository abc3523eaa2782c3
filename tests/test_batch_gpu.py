"""Batched SCF of several molecules in one engine (graph-captured Fock builds) against
one-molecule-at-a-time RHF."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def batch_case():
    from gaussium_gb300 import batch, driver, molecules
    mols = [molecules.water_cluster(1, seed=1), molecules.random_chain(3),
            molecules.random_chain(1), molecules.water_cluster(2, seed=5)]
    single = np.array([driver.rhf(m, threshold=1e-11)["energy"] for m in mols])
    return batch.BatchedRHF(mols), single


def test_batched_energies_match_single(gpu_lib, batch_case):
    b, single = batch_case
    e, it = b.run(threshold=1e-11)
    assert b.converged.all() and it < 60
    assert np.max(np.abs(e - single)) < 1e-8
    e2, _ = b.run(threshold=1e-11, use_graph=False)
    assert np.max(np.abs(e2 - e)) < 1e-9


def test_batched_mixed_incremental_within_target(gpu_lib, batch_case):
    b, single = batch_case
    e, it = b.run(threshold=1e-10, mixed_cut=1e-2, screen_thr=1e-12, incremental=True)
    assert b.converged.all()
    assert np.max(np.abs(e - single)) < 1e-6


def test_batched_task_list_matches_engine_count(gpu_lib, batch_case):
    from gaussium_gb300.engine import JKEngine
    b, _ = batch_case
    total = sum(JKEngine(sb, schwarz_thr=1e-12).ntasks for sb in b.sbs)
    assert b.ntasks == total


def test_batched_sad_guess_same_energies(gpu_lib, batch_case):
    b, single = batch_case
    e, it = b.run(threshold=1e-11, guess="sad")
    assert b.converged.all()
    assert np.max(np.abs(e - single)) < 1e-8


@pytest.mark.parametrize("mixed_cut,screen_thr", [(None, 0.0), (1e-2, 1e-12)])
def test_persistent_launch_matches_per_class_launches(gpu_lib, batch_case, mixed_cut, screen_thr):
    """One persistent launch per precision over every class and molecule gives the Fock
    matrices of the per-class launches (same quartets, same precision split)."""
    import torch
    b, _ = batch_case
    rng = np.random.default_rng(3)
    P = torch.tensor(rng.standard_normal(b.mat_stride) * 0.1, device="cuda")
    g1 = b.fock_packed(P, mixed_cut=mixed_cut, screen_thr=screen_thr)
    g2 = b.fock_packed(P, mixed_cut=mixed_cut, screen_thr=screen_thr, persistent=True)
    scale = float(g1.abs().max())
    tol = 1e-12 if mixed_cut is None else 1e-6
    assert float((g1 - g2).abs().max()) <= tol * scale


def test_persistent_batched_scf(gpu_lib, batch_case):
    b, single = batch_case
    e, it = b.run(threshold=1e-10, mixed_cut=1e-2, screen_thr=1e-12, incremental=True,
                  persistent=True)
    assert b.converged.all()
    assert np.max(np.abs(e - single)) < 1e-6
