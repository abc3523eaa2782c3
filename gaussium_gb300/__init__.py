"""GB300-native two-electron-integral and Fock-build engine with the call surface of the
reference Gaussium's ERI path (integral objects, ERI-matrix builder, Fock builders)."""
from .basis import Basis, PrimitiveBasis, Nuclei, ShellBasis, read_basis_set_file, read_mol_file

__all__ = ["Basis", "PrimitiveBasis", "Nuclei", "ShellBasis", "read_basis_set_file",
           "read_mol_file"]
