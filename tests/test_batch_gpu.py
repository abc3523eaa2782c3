"""Batched SCF of several molecules in one engine (graph-captured Fock builds) against
one-molecule-at-a-time RHF."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_batched_energies_match_single(gpu_lib):
    from gaussium_gb300 import batch, driver, molecules
    mols = [molecules.water_cluster(1, seed=1), molecules.random_chain(3),
            molecules.random_chain(1), molecules.water_cluster(2, seed=5)]
    single = [driver.rhf(m, threshold=1e-11)["energy"] for m in mols]
    b = batch.BatchedRHF(mols)
    e, it = b.run(threshold=1e-11)
    assert np.max(np.abs(e - np.array(single))) < 1e-7
    e2, _ = b.run(threshold=1e-11, use_graph=False)
    assert np.max(np.abs(e2 - e)) < 1e-9
