"""Molecules and basis sets for the SCF workloads.

``water_cluster(n, seed)``: (H2O)n with TIP3P monomer geometry (r_OH 0.9572 A, HOH 104.52
deg), seeded random rigid rotations and positions in a cube sized for 1 g/cm^3, no O-O
distance below 2.6 A.  ``random_chain(seed)``: a neutral closed-shell C/N/O chain of 3-30
atoms (bonds 1.0-1.5 A) saturated with hydrogens.  ``basis_functions`` expands a basis set
from gaussium_gb300/data/basis_sets.json into reference-ordered functions
(factory/primitive_basis_factory.py:5-86 order, reference normalisation).  Coordinates are
in bohr, as the reference's .mol files are (common/file_input.py:59-88).
"""
import json
import math
import os

import numpy as np

from .basis import Nuclei, ShellBasis, expand_shell

BOHR_PER_ANGSTROM = 1.0 / 0.529177210903
Z = {"H": 1, "He": 2, "C": 6, "N": 7, "O": 8}
NAME = {"H": "HYDROGEN", "He": "HELIUM", "C": "CARBON", "N": "NITROGEN", "O": "OXYGEN"}
VALENCE = {"C": 4, "N": 3, "O": 2}
_DATA = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "basis_sets.json")
_BASIS = None


class Molecule:
    def __init__(self, symbols, coords_bohr, charge=0, multiplicity=1):
        self.symbols = list(symbols)
        self.coords = np.asarray(coords_bohr, dtype=np.float64).reshape(-1, 3)
        self.charges = np.array([Z[s] for s in self.symbols], dtype=np.float64)
        self.electrons = int(self.charges.sum()) - charge
        self.multiplicity = multiplicity

    @property
    def nuclei(self):
        return [Nuclei(NAME[s], float(Z[s]), 0.0, tuple(c)) for s, c in zip(self.symbols, self.coords)]

    def nuclear_repulsion(self):
        d = self.coords[:, None, :] - self.coords[None, :, :]
        r = np.sqrt((d ** 2).sum(-1))
        iu = np.triu_indices(len(self.symbols), 1)
        return float(np.sum(self.charges[iu[0]] * self.charges[iu[1]] / r[iu]))


def basis_functions(mol, basis="6-31G*"):
    global _BASIS
    if _BASIS is None:
        with open(_DATA) as f:
            _BASIS = json.load(f)
    table = _BASIS[basis]
    out = []
    for s, c in zip(mol.symbols, mol.coords):
        for sh in table[s]:
            out.extend(expand_shell(sh["type"], sh["rows"], tuple(float(x) for x in c)))
    return out


def shell_basis(mol, basis="6-31G*"):
    return ShellBasis.from_functions(basis_functions(mol, basis))


def _rotation(rng):
    q = rng.standard_normal(4)
    q /= np.linalg.norm(q)
    a, b, c, d = q
    return np.array([[a * a + b * b - c * c - d * d, 2 * (b * c - a * d), 2 * (b * d + a * c)],
                     [2 * (b * c + a * d), a * a - b * b + c * c - d * d, 2 * (c * d - a * b)],
                     [2 * (b * d - a * c), 2 * (c * d + a * b), a * a - b * b - c * c + d * d]])


def water_cluster(n, seed=None, min_oo=2.6, density=1.0):
    rng = np.random.default_rng(n if seed is None else seed)
    r, ang = 0.9572, math.radians(104.52)
    mono = np.array([[0.0, 0.0, 0.0],
                     [r * math.sin(ang / 2), r * math.cos(ang / 2), 0.0],
                     [-r * math.sin(ang / 2), r * math.cos(ang / 2), 0.0]])
    mono -= mono.mean(0)
    side = (n * 18.015 / (6.02214076e23 * density)) ** (1 / 3) * 1e8   # cm -> A
    oxy, coords = [], []
    tries = 0
    while len(oxy) < n:
        tries += 1
        if tries > 200000:
            raise RuntimeError("could not place the water molecules")
        pos = rng.uniform(0, side, size=3)
        m = mono @ _rotation(rng).T + pos
        if any(np.linalg.norm(m[0] - o) < min_oo for o in oxy):
            continue
        oxy.append(m[0])
        coords.extend(m)
    return Molecule(["O", "H", "H"] * n, np.array(coords) * BOHR_PER_ANGSTROM)


def perturbed(mol, amplitude_angstrom=0.1, seed=4):
    """Every nucleus moved by ``amplitude_angstrom`` in a seeded random direction."""
    rng = np.random.default_rng(seed)
    d = rng.standard_normal(mol.coords.shape)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return Molecule(mol.symbols, mol.coords + amplitude_angstrom * BOHR_PER_ANGSTROM * d)


def random_chain(seed, min_heavy=2, max_atoms=30):
    """Random bonded C/N/O chain with hydrogens filling free valences; even electron count."""
    rng = np.random.default_rng(seed)
    while True:
        nheavy = int(rng.integers(min_heavy, 11))
        heavy = list(rng.choice(["C", "N", "O"], size=nheavy, p=[0.6, 0.2, 0.2]))
        for i in range(1, nheavy - 1):
            if heavy[i] == "O":
                heavy[i] = "C"          # divalent O only at the chain ends
        nh = sum(VALENCE[h] for h in heavy) - 2 * (nheavy - 1)
        natoms = nheavy + nh
        if natoms < 3 or natoms > max_atoms:
            continue
        electrons = sum(Z[h] for h in heavy) + nh
        if electrons % 2:
            continue
        pos = [np.zeros(3)]
        direction = np.array([1.0, 0.0, 0.0])
        for i in range(1, nheavy):
            bond = rng.uniform(1.0, 1.5)
            turn = rng.standard_normal(3) * 0.6
            direction = direction + turn
            direction /= np.linalg.norm(direction)
            pos.append(pos[-1] + bond * direction)
        sym = list(heavy)
        coords = list(pos)
        for i, h in enumerate(heavy):
            free = VALENCE[h] - (1 if i > 0 else 0) - (1 if i < nheavy - 1 else 0)
            for _ in range(free):
                for _t in range(50):
                    v = rng.standard_normal(3)
                    v /= np.linalg.norm(v)
                    cand = pos[i] + rng.uniform(1.0, 1.1) * v
                    if all(np.linalg.norm(cand - c) > 0.9 for j, c in enumerate(coords) if j != i):
                        break
                sym.append("H")
                coords.append(cand)
        coords = np.array(coords)
        d = np.linalg.norm(coords[:, None] - coords[None], axis=-1) + np.eye(len(coords)) * 9
        if d.min() < 0.75:
            continue
        return Molecule(sym, coords * BOHR_PER_ANGSTROM)
