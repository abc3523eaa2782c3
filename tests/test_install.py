"""install() rebinds the reference's SCF module attributes to the drop-ins (checked on a
stand-in package with the reference's module layout; no GPU needed)."""
import types

from gaussium_gb300 import fock


def _fake_gaussium():
    hf = types.ModuleType("gaussium.hartreefock.hartree_fock")
    for name in ("TwoElectronRepulsionMatrixOS", "FockMatrixRestricted", "FockMatrixUnrestricted",
                 "BlockedFockMatrixUnrestricted", "blocked_spin_basis_set"):
        setattr(hf, name, object())
    ks = types.ModuleType("gaussium.kohnsham.kohn_sham")
    ks.RestrictedKohnShamHamiltonian = object()
    mp = types.ModuleType("gaussium.moellerplesset.moeller_plesset")
    mp.molecular_orbitals = object()
    cc = types.ModuleType("gaussium.coupledcluster.coupled_cluster")
    cc.molecular_orbitals, cc.spin_basis_anti_physicist = object(), object()
    td = types.ModuleType("gaussium.tdhartreefock.td_hartree_fock")
    td.molecular_orbitals, td.spin_basis_set = object(), object()
    g = types.SimpleNamespace(hartreefock=types.SimpleNamespace(hartree_fock=hf),
                              kohnsham=types.SimpleNamespace(kohn_sham=ks),
                              moellerplesset=types.SimpleNamespace(moeller_plesset=mp),
                              coupledcluster=types.SimpleNamespace(coupled_cluster=cc),
                              tdhartreefock=types.SimpleNamespace(td_hartree_fock=td))
    return g


def test_install_rebinds_and_returns_originals():
    g = _fake_gaussium()
    before = dict(vars(g.hartreefock.hartree_fock))
    orig = fock.install(g, mixed_cut=1e-3)
    hf = g.hartreefock.hartree_fock
    assert hf.TwoElectronRepulsionMatrixOS is fock._BasisOnly
    assert hf.FockMatrixRestricted.func is fock.FockMatrixRestrictedGPU
    assert hf.FockMatrixRestricted.keywords == {"mixed_cut": 1e-3}
    assert hf.FockMatrixUnrestricted.func is fock.FockMatrixUnrestrictedGPU
    assert hf.BlockedFockMatrixUnrestricted.func is fock.BlockedFockMatrixUnrestrictedGPU
    assert g.kohnsham.kohn_sham.RestrictedKohnShamHamiltonian.func is fock.RestrictedKohnShamHamiltonianGPU
    basis = ["f1", "f2"]
    assert hf.TwoElectronRepulsionMatrixOS(basis, None, 4).create_repulsion_matrix() is basis
    assert hf.blocked_spin_basis_set(basis) is basis
    assert orig[("gaussium.hartreefock.hartree_fock", "FockMatrixRestricted")] is before["FockMatrixRestricted"]


def test_install_reroutes_post_scf_transforms():
    from gaussium_gb300 import transform
    g = _fake_gaussium()
    before = g.coupledcluster.coupled_cluster.spin_basis_anti_physicist
    orig = fock.install(g)
    assert g.moellerplesset.moeller_plesset.molecular_orbitals is fock._mo_from_source
    assert g.coupledcluster.coupled_cluster.molecular_orbitals is fock._mo_from_source
    assert g.coupledcluster.coupled_cluster.spin_basis_anti_physicist is transform.spin_basis_anti_physicist
    assert g.tdhartreefock.td_hartree_fock.spin_basis_set is transform.spin_basis_set
    assert not hasattr(g.tdhartreefock.td_hartree_fock, "spin_basis_anti_physicist")
    assert orig[("gaussium.coupledcluster.coupled_cluster", "spin_basis_anti_physicist")] is before


def test_install_on_the_real_reference_package():
    """Acceptance on the reference itself (when its source tree is given by the
    GAUSSIUM_REFERENCE environment variable; skipped without it): install() rebinds
    hartreefock/hartree_fock.py:14,39-41 and kohnsham/kohn_sham.py:1-2 of the real package,
    the reference's own HartreeFock constructor then takes the basis list instead of
    building the N^4 tensor, and uninstall() restores every original."""
    import contextlib
    import io
    import os
    import sys
    if not os.environ.get("GAUSSIUM_REFERENCE"):
        import pytest
        pytest.skip("GAUSSIUM_REFERENCE (the reference source tree) is not set")
    here = os.path.dirname(os.path.abspath(__file__))
    sys.path.insert(0, os.path.join(here, "golden"))
    import ref_harness
    g = ref_harness.load()
    import gaussium.hartreefock.hartree_fock as hf
    import gaussium.kohnsham.kohn_sham as ks
    from gaussium.common import read_mol_file, read_basis_set_file
    before = {n: getattr(hf, n) for n in ("TwoElectronRepulsionMatrixOS", "FockMatrixRestricted",
                                          "FockMatrixUnrestricted", "BlockedFockMatrixUnrestricted",
                                          "blocked_spin_basis_set")}
    ks_before = ks.RestrictedKohnShamHamiltonian
    orig = fock.install(g)
    try:
        assert hf.TwoElectronRepulsionMatrixOS is fock._BasisOnly
        assert hf.FockMatrixRestricted.func is fock.FockMatrixRestrictedGPU
        assert hf.FockMatrixUnrestricted.func is fock.FockMatrixUnrestrictedGPU
        assert hf.BlockedFockMatrixUnrestricted.func is fock.BlockedFockMatrixUnrestrictedGPU
        assert ks.RestrictedKohnShamHamiltonian.func is fock.RestrictedKohnShamHamiltonianGPU
        root = ref_harness.reference_root()
        nuclei, electrons, _ = read_mol_file(os.path.join(root, "examples", "molfiles", "H2O.mol"))
        basis = read_basis_set_file(os.path.join(root, "examples", "basissets", "STO-3G.gbs"), nuclei)
        with contextlib.redirect_stdout(io.StringIO()):
            obj = hf.Restricted(nuclei, basis, electrons, ref_harness.c1_symmetry(basis), 1)
        assert obj.repulsion is basis           # no tensor: the Fock drop-in takes the shells
    finally:
        fock.uninstall(orig)
    for n, v in before.items():
        assert getattr(hf, n) is v
    assert ks.RestrictedKohnShamHamiltonian is ks_before
