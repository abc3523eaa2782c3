"""Superposition-of-atomic-densities (SAD) starting density for RHF.

The reference starts every SCF from the core Hamiltonian (hartreefock/scf_procedure.py:
24-42, orbitals of H).  For molecules of tens of atoms that guess is far from the answer
and costs SCF iterations; the usual remedy is to start from the sum of the densities of
the free atoms.  Each element's density is computed once per basis set by a small
fractional-occupation SCF of the neutral atom (the electrons of a partly filled level
spread evenly over its degenerate orbitals, so the density is spherical), on the same GPU
engine as the molecules, and placed on the diagonal block of every atom of that element
(functions are generated atom by atom, so an atom's functions are contiguous).  The
converged SCF does not depend on the guess; only the number of iterations does.
"""
import numpy as np

from . import scf

_CACHE = {}


def fractional_occupations(eps, nelec, tol=1e-4):
    """Aufbau occupations (at most 2 per orbital) of ``nelec`` electrons over orbital
    energies ``eps`` (ascending), with the partly filled level shared evenly by the
    orbitals within ``tol`` of it."""
    n = len(eps)
    occ = np.zeros(n)
    left = float(nelec)
    i = 0
    while left > 1e-12 and i < n:
        j = i
        while j + 1 < n and abs(eps[j + 1] - eps[i]) < tol:
            j += 1
        deg = j - i + 1
        put = min(left, 2.0 * deg)
        occ[i:j + 1] = put / deg
        left -= put
        i = j + 1
    return occ


def atomic_density(overlap, hcore, two_electron, nelec, max_iter=60, threshold=1e-9, damping=0.3):
    """Density of a fractionally occupied atom: ``two_electron(P) -> J - K/2``.  Canonical
    orthogonalisation, then damped Roothaan steps (the fractional occupations make DIIS
    unnecessary for a single atom) until the energy changes by less than ``threshold``."""
    la = scf.LinearAlgebra(overlap)
    eps, c = la.diagonalize(hcore)
    occ = fractional_occupations(eps, nelec)
    p = (c * occ) @ c.T
    e_prev = None
    for _ in range(max_iter):
        f = hcore + two_electron(p)
        e = 0.5 * float(np.sum(p * (hcore + f)))
        if e_prev is not None and abs(e - e_prev) < threshold:
            break
        e_prev = e
        eps, c = la.diagonalize(f)
        occ = fractional_occupations(eps, nelec)
        p = (1.0 - damping) * ((c * occ) @ c.T) + damping * p
    return p


def element_density(symbol, basis="6-31G*"):
    """Cached spherical density of the neutral atom ``symbol`` in ``basis`` (GPU engine)."""
    key = (symbol, basis)
    if key not in _CACHE:
        import torch
        from .engine import JKEngine
        from .hamiltonian import one_electron
        from .molecules import Z, Molecule, shell_basis
        atom = Molecule([symbol], np.zeros((1, 3)))
        sb = shell_basis(atom, basis)
        S, T, V = one_electron(sb, atom.coords, atom.charges)
        eng = JKEngine(sb, schwarz_thr=1e-14)

        def g(p):
            pt = torch.tensor(p, device=eng.dev)
            J, (K,) = eng.jk(pt, [pt])
            return (J - 0.5 * K).cpu().numpy()

        _CACHE[key] = atomic_density(S, T + V, g, Z[symbol])
    return _CACHE[key]


def sad_density(mol, basis="6-31G*", densities=None):
    """Block-diagonal starting density of ``mol``: each atom's element density on its own
    functions.  ``densities`` maps symbol -> density (default: ``element_density``)."""
    dens = densities or {}
    blocks = [dens[s] if s in dens else element_density(s, basis) for s in mol.symbols]
    n = sum(b.shape[0] for b in blocks)
    P = np.zeros((n, n))
    o = 0
    for b in blocks:
        k = b.shape[0]
        P[o:o + k, o:o + k] = b
        o += k
    return P
