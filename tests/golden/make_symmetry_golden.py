"""Generate ``symmetry.npz`` by running the reference's point-group screening here.

Run from this directory:  ``python make_symmetry_golden.py``.  It needs the reference source
tree (the GAUSSIUM_REFERENCE environment variable); it writes only ``symmetry.npz`` beside itself.

For each system the reference's ``MoleculeFactory(symmetry=True).create`` orients the
nuclei and finds the point group (``factory/molecule_factory.py``), ``read_basis_set_file``
builds the basis on the oriented nuclei, and ``Symmetry(point_group, basis)``
(``common/symmetry.py:10-16``) builds its tables.  Stored per system (prefix ``<name>_``):
the basis arrays (as make_golden.py's ``basis_arrays``), the function-image table
``symmetry_matrix[1:, 1:]`` (signed 1-based images, 0 = no image), the parity-flip table
``flip[m - 1, p] = (p != int_operate_dict[(m, p)])`` for the 8 parity vectors p (bit 0 x,
bit 1 y, bit 2 z), the point-group label, and the reference's
``none_zero_integral`` (``common/symmetry.py:18-47``) for every canonical key
a <= b, c <= d, (a, b) <= (c, d), in the order create_repulsion_matrix enumerates them
(lexicographic; ``oracle.canonical_keys`` regenerates the list, so it is not stored).

Systems: ethene/3-21G (the reference's own symmetry test, test_start.py:27-31), water/
6-311+G** (d functions) and O2/STO-3G (test_start.py:33-43), all from the reference's
test inputs; water uses make_golden.py's geometry.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import ref_harness  # noqa: E402
import make_golden  # noqa: E402

START = os.path.join(make_golden.ref_harness.reference_root(), "tests", "testslow", "start")
PARITIES = [(p & 1, (p >> 1) & 1, (p >> 2) & 1) for p in range(8)]


def system(mol_path, gbs):
    ref_harness.load()
    from gaussium.common import read_mol_file, read_basis_set_file, Symmetry
    from gaussium.factory import MoleculeFactory
    nuclei, electrons, mult = read_mol_file(mol_path)
    nuclei, point_group = MoleculeFactory(True).create(nuclei)
    basis = read_basis_set_file(os.path.join(START, gbs), nuclei)
    sym = Symmetry(point_group, basis)
    n = len(basis)
    nops = sym.symmetry_matrix.shape[1] - 1
    table = np.array([[int(sym.symmetry_matrix[i + 1, m + 1]) for m in range(nops)]
                      for i in range(n)], dtype=np.int32).reshape(n, nops)
    flip = np.array([[PARITIES[p] != tuple(sym.int_operate_dict[(m + 1, PARITIES[p])])
                      for p in range(8)] for m in range(nops)], dtype=bool).reshape(nops, 8)
    keys = []
    for a in range(n):
        for b in range(a, n):
            for c in range(a, n):
                for d in range(c, n):
                    if a == c and b > d:
                        continue
                    keys.append((a, b, c, d))
    keys = np.array(keys, dtype=np.int32)
    mask = np.array([bool(sym.none_zero_integral(tuple(int(x) for x in k))) for k in keys])
    out = {"table": table, "flip": flip, "label": np.array(point_group.label),
           "nonzero": mask}
    out.update(make_golden.basis_arrays(basis))
    return out


def main():
    water = make_golden.write_tmp("water.mol", make_golden.water_mol_text())
    systems = {"ethene": (os.path.join(START, "C2H4.mol"), "3-21G.gbs"),
               "water": (water, "6-311+GPP.gbs"),
               "o2": (os.path.join(START, "O2.mol"), "STO-3G.gbs")}
    out = {}
    for name, (mol, gbs) in systems.items():
        for k, v in make_golden.quiet(system, mol, gbs).items():
            out[f"{name}_{k}"] = v
    np.savez_compressed(os.path.join(HERE, "symmetry.npz"), **out)


if __name__ == "__main__":
    main()
