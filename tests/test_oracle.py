"""The oracle (C restatement of the reference ERI path) against the golden vectors that
tests/golden/make_golden.py produced by running the reference itself."""
import numpy as np
import pytest

import oracle
from conftest import golden, synthetic_shells


def test_boys_reference_port_matches_reference():
    g = golden("boys")
    got = np.array([[oracle.boys_reference(v, x) for x in g["x"]] for v in g["v"]])
    ref = g["reference"]
    assert np.max(np.abs(got - ref) / np.maximum(np.abs(ref), 1e-300)) < 1e-13


def test_boys_exact_matches_mpmath():
    g = golden("boys")
    got = np.array([[oracle.boys_exact(v, x) for x in g["x"]] for v in g["v"]])
    assert np.max(np.abs(got - g["exact"]) / np.abs(g["exact"])) < 1e-14


def test_reference_boys_error_is_the_known_one():
    # the reference's series stops at a term < 1e-10 (boys_function.py:34,48)
    g = golden("boys")
    err = np.max(np.abs(g["reference"] - g["exact"]))
    assert 1e-12 < err < 1e-10


@pytest.mark.parametrize("memo", [True, False])
def test_heh_unit_test_quartets(memo):
    g = golden("eri_heh")
    he_r, h_r = (0, 0, 0.7316), (0, 0, -0.7316)
    he = [(0.15432897, 9.75393461, 3.9336432656254527), (0.53532814, 1.77669115, 1.0967787981767012),
          (0.44463454, 0.48084429, 0.41154131374122654)]
    h = [(0.15432897, 3.42525091, 1.794441832218435), (0.53532814, 0.62391373, 0.5003264923314032),
         (0.44463454, 0.16885540, 0.18773545851092535)]
    t = oracle.FunctionTable(np.array([he_r, h_r]), np.zeros((2, 3)), np.ones(2), [he, h])
    got = oracle.eri_functions(t, g["keys"], boys_mode=0, memo=memo)
    np.testing.assert_allclose(got, g["os"], rtol=0, atol=1e-15)
    # the reference test file's own values, to its 4 significant figures
    for v, want in zip(got, g["test_values"]):
        np.testing.assert_approx_equal(v, want, 4)


@pytest.mark.parametrize("name", ["h2o_sto3g", "h2o_631gs"])
def test_molecule_eris_match_reference(name):
    g = golden(name)
    t = oracle.FunctionTable.from_arrays(g)
    got = oracle.eri_functions(t, g["keys"], boys_mode=0)
    assert np.max(np.abs(got - g["eri"])) < 1e-14
    exact = oracle.eri_functions(t, g["keys"], boys_mode=1)
    # exact-Boys oracle differs from the as-is reference by the reference's Boys error only
    assert np.max(np.abs(exact - g["eri"])) < 1e-10


def test_dense_tensor_and_fock_restatements():
    g = golden("h2o_sto3g")
    t = oracle.FunctionTable.from_arrays(g)
    dense = oracle.dense_tensor(t, boys_mode=0)
    assert np.max(np.abs(dense - g["dense"])) < 1e-14
    eri = g["dense"]
    pa, pb = g["density_a"], g["density_b"]
    h = np.zeros_like(pa)
    np.testing.assert_allclose(oracle.fock_restricted(h, eri, pa), g["fock_rhf"], atol=1e-13)
    fa, fb = oracle.fock_unrestricted(h, eri, pa, pb)
    np.testing.assert_allclose(fa, g["fock_uhf_a"], atol=1e-13)
    np.testing.assert_allclose(fb, g["fock_uhf_b"], atol=1e-13)
    np.testing.assert_allclose(oracle.coulomb(eri, pa), g["coulomb_ks"], atol=1e-13)


def test_synthetic_quartets_and_normalisation():
    g = golden("synthetic")
    shells = synthetic_shells()
    t = oracle.FunctionTable.from_shells(shells)
    ncomp = [len(oracle.COMPONENTS[s["l"]]) for s in shells]
    off = np.concatenate([[0], np.cumsum(ncomp)])
    cn = np.concatenate([g["contracted_norm"][i, :ncomp[i]] for i in range(len(shells))])
    np.testing.assert_allclose(t.cnorm, cn, rtol=1e-14)
    q = g["quartets"][g["sample_quartet"]]
    fq = np.array([[off[q[i, k]] + g["sample_comp"][i, k] for k in range(4)] for i in range(len(q))])
    got = oracle.eri_functions(t, fq, boys_mode=0)
    assert np.max(np.abs(got - g["os"])) < 1e-15
    # HGP agrees with OS in the reference itself; Cook calls the (inexact) reference Boys
    # series once per order instead of recursing down, so it differs by that error
    m = ~np.isnan(g["hgp"])
    assert np.max(np.abs(g["hgp"][m] - g["os"][m])) < 1e-15
    m = ~np.isnan(g["cook"])
    assert np.max(np.abs(g["cook"][m] - g["os"][m])) < 5e-9


def test_synthetic_k6_quartets():
    """The microbench's contraction range (K = 1-6, and K = 6 on all four shells) for every
    canonical class: the oracle against the reference's ObaraSaika values."""
    g = golden("synthetic_k6")
    assert g["shell_k"].max() == 6 and g["shell_k"].min() == 1
    shells = synthetic_shells("synthetic_k6")
    t = oracle.FunctionTable.from_shells(shells)
    ncomp = [len(oracle.COMPONENTS[s["l"]]) for s in shells]
    off = np.concatenate([[0], np.cumsum(ncomp)])
    q = g["quartets"][g["sample_quartet"]]
    fq = np.array([[off[q[i, k]] + g["sample_comp"][i, k] for k in range(4)] for i in range(len(q))])
    got = oracle.eri_functions(t, fq, boys_mode=0)
    assert np.max(np.abs(got - g["os"])) < 1e-15


def test_ao_to_mo_restatements_match_reference():
    """The oracle's restatements of matrixelements/transformations.py against the
    reference's own outputs (tests/golden/make_mo_golden.py)."""
    g = golden("mo_transform")
    mo = oracle.molecular_orbitals(g["ao"], g["coefficients"])
    assert np.max(np.abs(mo - g["mo"])) < 1e-14
    assert np.max(np.abs(oracle.spin_basis_set(g["mo"]) - g["spin"])) == 0.0
    assert np.max(np.abs(oracle.blocked_spin_basis_set(g["mo"]) - g["blocked"])) == 0.0
    assert np.max(np.abs(oracle.spin_basis_anti_physicist(g["mo"]) - g["anti"])) == 0.0


def test_lda_functionals_and_density_match_reference():
    """The oracle's Slater / VWN restatements and electron density against the reference's
    own outputs (tests/golden/make_xc_golden.py)."""
    from molecules import load
    g = golden("xc")
    d = g["density"]
    for tag, alpha in (("s", 2 / 3), ("xa", 0.7)):
        assert np.allclose(oracle.slater_energy(d, alpha), g[f"slater_{tag}_energy"], rtol=1e-14, atol=0)
        assert np.allclose(oracle.slater_potential(d, alpha), g[f"slater_{tag}_potential"], rtol=1e-14, atol=0)
    for tag, prm in (("vwn3", oracle.VWN3), ("vwn5", oracle.VWN5)):
        assert np.allclose(oracle.vwn_energy(d, *prm), g[f"{tag}_energy"], rtol=1e-13, atol=0)
        assert np.allclose(oracle.vwn_potential(d, *prm), g[f"{tag}_potential"], rtol=1e-13, atol=0)
    _, _, table = load("h2o_sto3g")
    rho = oracle.electron_density(table, g["pmat"], g["points"])
    assert np.max(np.abs(rho - g["rho"])) < 1e-15


def he_sto3g():
    return oracle.FunctionTable.from_shells([dict(
        l=0, centre=np.zeros(3), expo=np.array([6.36242139, 1.15892300, 0.31364979]),
        coef=np.array([0.15432897, 0.53532814, 0.44463454]))])


def test_ks_oracle_reproduces_reference_he_dft_energies():
    """The oracle's Kohn-Sham restatement (quad radially, degree-35 product rule in angle)
    against the reference's own He/STO-3G DFT energies (test_start.py, 6 s.f.)."""
    g = golden("xc")
    he = he_sto3g()
    S, T, V = oracle.one_centre_s(he, 2.0)
    eri = oracle.dense_tensor(he)
    for alpha, vwn, key in ((2 / 3, None, "he_energy_s"), (2 / 3, oracle.VWN3, "he_energy_svwn3")):
        e = oracle.ks_restricted_scf(S, T + V, eri, 2, he, alpha, vwn)
        assert abs(e - float(g[key])) < 1e-8, key


def test_symmetry_screen_restatement_matches_reference():
    """The oracle's point-group screen against the reference's none_zero_integral on every
    canonical key of three systems (tests/golden/make_symmetry_golden.py), and invariance
    under the 8 index permutations the dense tensor expands each key to."""
    g = golden("symmetry")
    rng = np.random.default_rng(0)
    for name in ("ethene", "water", "o2"):
        table, flip = g[f"{name}_table"], g[f"{name}_flip"]
        cid = oracle.centre_ids(g[f"{name}_centre"])
        par = oracle.parity_bits(g[f"{name}_lmn"])
        keys, ref = oracle.canonical_keys(g[f"{name}_table"].shape[0]), g[f"{name}_nonzero"]
        got = np.array([oracle.symmetry_nonzero(table, flip, cid, par, k) for k in keys])
        assert np.array_equal(got, ref), name
        for t in rng.choice(len(keys), 300, replace=False):
            a, b, c, d = keys[t]
            for perm in ((b, a, c, d), (a, b, d, c), (c, d, a, b), (d, c, b, a)):
                assert oracle.symmetry_nonzero(table, flip, cid, par, perm) == ref[t]


def test_sort_index_known_answers():
    """oracle.sort_index against the reference's own cases
    (tests/testsfast/common/test_symmetry.py:14-48 within the reference project)."""
    cases = [((6, 2, 1, 0), (0, 1, 2, 6)), ((0, 0, 1, 0), (0, 0, 0, 1)),
             ((1, 0, 0, 0), (0, 0, 0, 1)), ((1, 0, 1, 0), (0, 1, 0, 1)),
             ((2, 2, 1, 0), (0, 1, 2, 2)), ((2, 1, 1, 0), (0, 1, 1, 2)),
             ((1, 1, 1, 0), (0, 1, 1, 1)), ((2, 1, 2, 0), (0, 2, 1, 2)),
             ((1, 1, 0, 2), (0, 2, 1, 1))]
    for key, want in cases:
        assert tuple(oracle.sort_index(*key)) == want, key


@pytest.mark.parametrize("name", ["heh_6311pgss", "ethene_321g"])
def test_start_rhf_energies_through_the_oracle(name):
    """HeH+/6-311+G** and ethene/3-21G (the reference's test_start.py:15-25 systems): the
    restated SCF loop over the oracle's ERI tensor and Fock builder reproduces the
    reference's RHF total energy to 1e-8 Eh."""
    from molecules import load
    from gaussium_gb300 import scf
    g, _, table = load(name)
    eri = oracle.dense_tensor(table, boys_mode=1)
    hcore = g["kinetic"] + g["nuclear"]

    class Fock:
        core_hamiltonian = hcore

        def create(self, p):
            return oracle.fock_restricted(hcore, eri, p)
    res = scf.restricted_scf(g["overlap"], hcore, int(g["electrons"]), Fock(), threshold=1e-12)
    e = res.energy + scf.nuclear_repulsion(g["charges"], g["coords"])
    assert res.converged
    assert abs(e - float(g["energy"])) < 1e-8, (e, float(g["energy"]))


def test_co_mp2_energy_through_the_oracle():
    """Carbon monoxide / STO-3G (the reference's test_start.py:45-49): the restated SCF
    over the oracle's ERI tensor, the oracle's AO->MO transform and its MP2 sum reproduce
    the reference's RHF and MP2 total energies to 1e-8 Eh."""
    from molecules import load
    from gaussium_gb300 import scf
    g, _, table = load("co_sto3g")
    eri = oracle.dense_tensor(table, boys_mode=1)
    hcore = g["kinetic"] + g["nuclear"]

    class Fock:
        core_hamiltonian = hcore

        def create(self, p):
            return oracle.fock_restricted(hcore, eri, p)
    res = scf.restricted_scf(g["overlap"], hcore, int(g["electrons"]), Fock(), threshold=1e-12)
    e_nuc = scf.nuclear_repulsion(g["charges"], g["coords"])
    assert res.converged
    assert abs(res.energy + e_nuc - float(g["energy_rhf"])) < 1e-8
    mo = oracle.molecular_orbitals(eri, res.coefficients)
    corr = oracle.mp2_correlation(mo, res.orbital_energies, int(g["electrons"]) // 2)
    assert abs(res.energy + e_nuc + corr - float(g["energy_mp2"])) < 1e-8
