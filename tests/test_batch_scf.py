"""The batched SCF loop (padded matrices, per-molecule DIIS and convergence) on the CPU,
with the oracle's dense-tensor Fock builds standing in for the GPU J/K, against the
one-molecule restated SCF loop on the same Fock builds."""
import numpy as np
import pytest
import torch

import oracle
from conftest import golden
from gaussium_gb300 import scf
from gaussium_gb300.batch import batched_rhf_iterations, padded_system


class _OracleFock:
    def __init__(self, hcore, eri):
        self.hcore, self.eri = hcore, eri

    def create(self, p):
        return oracle.fock_restricted(self.hcore, self.eri, p)


def _system(name):
    g = golden(name)
    table = oracle.FunctionTable.from_arrays(g)
    n = len(g["norm"])
    if "dense" in g.files:
        eri = g["dense"]
    elif "keys" in g.files:
        eri = oracle.expand_dense(n, g["keys"], g["eri"])
    else:
        eri = oracle.dense_tensor(table, boys_mode=1)
    hcore = g["kinetic"] + g["nuclear"]
    return g["overlap"], hcore, eri, int(g["electrons"])


@pytest.fixture(scope="module")
def systems():
    return [_system(n) for n in ("h2o_sto3g", "heh_sto3g", "o2_sto3g", "h2o_631gs")]


def test_batched_loop_matches_single_loop(systems):
    single = []
    for S, H, eri, ne in systems:
        r = scf.restricted_scf(S, H, ne, _OracleFock(H, eri), threshold=1e-12)
        assert r.converged
        single.append(r.energy)
    Sb, Hb, X, occ, pad = padded_system([s[0] for s in systems], [s[1] for s in systems],
                                        [s[3] // 2 for s in systems], "cpu")
    N = Sb.shape[1]

    def two_electron(Pb, active=None):
        out = torch.zeros_like(Pb)
        for m, (S, H, eri, ne) in enumerate(systems):
            n = S.shape[0]
            p = Pb[m, :n, :n].numpy()
            out[m, :n, :n] = torch.as_tensor(oracle.fock_restricted(np.zeros_like(H), eri, p))
        return out

    e, it, done, _ = batched_rhf_iterations(Sb, Hb, X, occ, pad, two_electron, threshold=1e-12,
                                         max_iter=100)
    assert done.all()
    assert it < 100
    assert np.max(np.abs(e.numpy() - np.array(single))) < 1e-9
    assert N == 19


def test_reference_energy_of_water_sto3g_through_batched_loop(systems):
    S, H, eri, ne = systems[0]
    g = golden("h2o_sto3g")
    Sb, Hb, X, occ, pad = padded_system([S], [H], [ne // 2], "cpu")
    two = lambda Pb, active=None: torch.as_tensor(oracle.fock_restricted(np.zeros_like(H), eri,
                                                            Pb[0].numpy()))[None]
    e, it, done, _ = batched_rhf_iterations(Sb, Hb, X, occ, pad, two, threshold=1e-12)
    e_nuc = scf.nuclear_repulsion(g["charges"], g["coords"])
    assert abs(float(e[0]) + e_nuc - float(g["energy"])) < 1e-8


def _task_list_loops(q, pc, pair_mol, nprim, thr, nclass):
    """Plain-loop statement of the batched task list (per molecule, per class pair)."""
    from gaussium_gb300.engine import PAIR_ORDER
    out = {}
    for m in np.unique(pair_mol):
        pm = np.flatnonzero(pair_mol == m)
        for cb in range(nclass):
            for ck in range(cb + 1):
                for b in pm[pc[pm] == cb]:
                    for k in pm[pc[pm] == ck]:
                        if q[b] * q[k] >= thr and (cb != ck or b >= k):
                            out.setdefault((cb, ck), []).append((nprim[b], nprim[k], b, k))
    segs, rows = [], []
    for (cb, ck), lst in sorted(out.items()):
        # most primitive quartets first, then (K_bra, K_ket) descending; stable
        lst = sorted(lst, key=lambda r: (-(r[0] * r[1]), -r[0], -r[1]))
        (la, lb), (lc, ld) = PAIR_ORDER[cb], PAIR_ORDER[ck]
        segs.append(((la, lb, lc, ld), len(rows), len(rows) + len(lst)))
        rows.extend((b, k) for _, _, b, k in lst)
    return segs, np.array(rows, dtype=np.int32).reshape(-1, 2)


def test_batched_task_list_matches_loops():
    from gaussium_gb300.batch import batched_task_list
    rng = np.random.default_rng(7)
    npair = 300
    pair_mol = np.sort(rng.integers(0, 9, npair))
    pair_mol[pair_mol == 4] = 5                                # a molecule with no pairs
    pc = rng.integers(0, 6, npair)
    q = 10.0 ** rng.uniform(-9, 1, npair)
    nprim = rng.integers(1, 37, npair)
    segs, tasks = batched_task_list(torch.tensor(q), torch.tensor(pc), torch.tensor(pair_mol),
                                    torch.tensor(nprim), 1e-9, 6, 9)
    segs_ref, tasks_ref = _task_list_loops(q, pc, pair_mol, nprim, 1e-9, 6)
    assert segs == segs_ref
    assert np.array_equal(tasks.numpy(), tasks_ref)


def test_level_shifted_loop_reaches_the_same_energies(systems):
    """With the level shift switched on from the second iteration the loop converges to
    the same energies (the shift changes the path, not the fixed point)."""
    single = [scf.restricted_scf(S, H, ne, _OracleFock(H, eri), threshold=1e-12).energy
              for S, H, eri, ne in systems]
    Sb, Hb, X, occ, pad = padded_system([s[0] for s in systems], [s[1] for s in systems],
                                        [s[3] // 2 for s in systems], "cpu")

    def two_electron(Pb, active=None):
        out = torch.zeros_like(Pb)
        for m, (S, H, eri, ne) in enumerate(systems):
            n = S.shape[0]
            out[m, :n, :n] = torch.as_tensor(oracle.fock_restricted(np.zeros_like(H), eri,
                                                                    Pb[m, :n, :n].numpy()))
        return out

    e, it, done, _ = batched_rhf_iterations(Sb, Hb, X, occ, pad, two_electron, threshold=1e-12,
                                            max_iter=200, shift_after=2)
    assert done.all()
    assert np.max(np.abs(e.numpy() - np.array(single))) < 1e-9


def test_fractional_occupations():
    from gaussium_gb300.guess import fractional_occupations
    eps = np.array([-11.0, -0.7, -0.3, -0.3, -0.3, 0.2])
    occ = fractional_occupations(eps, 6)          # carbon-like: 1s2 2s2 2p(2/3 x 3)
    assert np.allclose(occ, [2, 2, 2 / 3, 2 / 3, 2 / 3, 0])
    assert np.isclose(fractional_occupations(eps, 1).sum(), 1.0)


def test_starting_density_reaches_the_same_energy(systems):
    """Block-diagonal 'atomic' starting densities (fractional-occupation SCF on each atom's
    own functions) lead the batched loop to the same energies as the core guess."""
    from gaussium_gb300.guess import atomic_density
    g = golden("h2o_sto3g")
    S, H, eri, ne = systems[0]
    centre = g["centre"]
    # functions of each atom (the golden lists them atom by atom)
    atom_of = np.argmin(np.linalg.norm(centre[:, None, :] - g["coords"][None], axis=-1), axis=1)
    P0 = np.zeros_like(S)
    for a in range(len(g["coords"])):
        f = np.flatnonzero(atom_of == a)
        sub = np.ix_(f, f)
        e4 = eri[np.ix_(f, f, f, f)]
        nel = int(round(g["charges"][a]))
        P0[sub] = atomic_density(S[sub], H[sub], lambda p: oracle.fock_restricted(np.zeros_like(p), e4, p), nel)
    assert np.isclose(np.sum(P0 * S), ne, atol=1e-6)        # electrons conserved
    Sb, Hb, X, occ, pad = padded_system([S], [H], [ne // 2], "cpu")
    two = lambda Pb, active=None: torch.as_tensor(oracle.fock_restricted(np.zeros_like(H), eri,
                                                                        Pb[0].numpy()))[None]
    e_core, it_core, _, _ = batched_rhf_iterations(Sb, Hb, X, occ, pad, two, threshold=1e-12)
    e_sad, it_sad, done, _ = batched_rhf_iterations(Sb, Hb, X, occ, pad, two, threshold=1e-12,
                                                    P_init=torch.as_tensor(P0)[None])
    assert done.all()
    assert abs(float(e_sad[0]) - float(e_core[0])) < 1e-9
