"""Seeded synthetic workloads.

``random_shell_quartets(n, seed)``: n shell quartets of four independent shells each:
angular momentum uniform over {s, p, d} (6 Cartesian d), contraction degree uniform 1..6,
exponents log-uniform in [0.05, 1e4], raw coefficients N(0, 1) normalised with the
reference's conventions (objects/primitive_basis_function.py:26-42 and
objects/basis_function.py:22-53: no contracted normalisation for a single primitive),
centres uniform in a 10 A cube (converted to bohr).  Vectorised; returns a ShellBasis and
the (n, 4) quartet index array.
"""
import math

import numpy as np

from .basis import ShellBasis

BOHR_PER_ANGSTROM = 1.0 / 0.529177210903
_DFACT = np.array([1.0, 1.0, 3.0])          # (2l-1)!! for l = 0, 1, 2 (first component)


def normalised_shells(l, nprim, expo, coef):
    """Effective coefficients (first component) and component scales of shells given as
    flat primitive arrays; l and nprim per shell."""
    l = np.asarray(l)
    nprim = np.asarray(nprim)
    owner = np.repeat(np.arange(len(l)), nprim)
    L = l[owner]
    # primitive normalisation of the first component (L,0,0)
    pw = np.where(L == 0, 1.0, np.where(L == 1, 4 * expo, 16 * expo * expo))   # (4a)^L
    t = np.pi / (2 * expo)
    npr = 1.0 / np.sqrt(_DFACT[L] * t * np.sqrt(t) / pw)
    # contracted normalisation: sum over primitive pairs within each shell, done per
    # contraction degree k on (shells, k, k) blocks
    off = np.concatenate([[0], np.cumsum(nprim)])
    s = np.zeros(len(l))
    for k in np.unique(nprim):
        sh = np.flatnonzero(nprim == k)
        idx = off[:-1][sh][:, None] + np.arange(k)[None, :]          # (ns, k)
        e = expo[idx]
        w = coef[idx] * npr[idx]
        sab = e[:, :, None] + e[:, None, :]
        Ls = l[sh][:, None, None]
        t = np.pi / sab
        pw = np.where(Ls == 0, 1.0, np.where(Ls == 1, 2 * sab, 4 * sab * sab))   # (2s)^L
        s[sh] = np.einsum("ni,nj,nij->n", w, w, t * np.sqrt(t) / pw) * _DFACT[l[sh]]
    cn = np.where(nprim == 1, 1.0, 1.0 / np.sqrt(np.where(s > 0, s, 1.0)))
    eff = coef * npr * cn[owner]
    scale = np.ones((len(l), 6))
    scale[l == 2, 3:] = math.sqrt(3.0)
    return eff, scale


def random_shell_quartets(n, seed=0, box_angstrom=10.0, lmax=2, kmax=6):
    rng = np.random.default_rng(seed)
    ns = 4 * n
    l = rng.integers(0, lmax + 1, size=ns)
    nprim = rng.integers(1, kmax + 1, size=ns)
    npt = int(nprim.sum())
    expo = np.exp(rng.uniform(np.log(0.05), np.log(1e4), size=npt))
    coef = rng.standard_normal(npt)
    centre = rng.uniform(0.0, box_angstrom, size=(ns, 3)) * BOHR_PER_ANGSTROM
    eff, scale = normalised_shells(l, nprim, expo, coef)
    off = np.concatenate([[0], np.cumsum(nprim)])
    sb = ShellBasis(l, centre, off, expo, eff, scale)
    return sb, np.arange(ns, dtype=np.int64).reshape(n, 4), dict(raw_coef=coef)
