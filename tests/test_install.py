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
