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
    g = types.SimpleNamespace(hartreefock=types.SimpleNamespace(hartree_fock=hf),
                              kohnsham=types.SimpleNamespace(kohn_sham=ks))
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
