"""Host-side SCF driver (FP64 numpy) with the reference's algorithm, for use where the
reference package itself is not installed (it is not a dependency of this library).

Restated from the reference (file:line within the reference project):
  LinearAlgebra           hartreefock/linear_algebra.py:4-30   canonical orthogonalisation, eigh
  DIIS                    diismethod/diis.py:4-112             Pulay DIIS, subspace 8
  TotalEnergy             hartreefock/total_energy.py:4-52
  density matrices        matrixelements/density_matrix.py:4-36
  RestrictedSCF           hartreefock/scf_procedure.py:15-42
  PopleNesbetBerthier     hartreefock/scf_procedure.py:45-86
  coulomb_matrix          common/nuclear_repulsion.py:5-24

Additions: ``max_iter`` (the reference loops forever on non-convergence) and a
``converged`` flag and iteration count in the result.
"""
import numpy as np


class LinearAlgebra:
    # smallest overlap eigenvalue accepted: below it the basis is linearly dependent and
    # the symmetric orthogonalisation S^-1/2 would amplify rounding without bound
    MIN_OVERLAP_EIGENVALUE = 1e-10

    def __init__(self, orbital_overlap):
        s, u = np.linalg.eigh(orbital_overlap)
        if not np.all(np.isfinite(s)) or s.min() <= self.MIN_OVERLAP_EIGENVALUE:
            raise ValueError(f"overlap matrix is singular or not positive definite (smallest "
                             f"eigenvalue {s.min():.3e}): the basis is linearly dependent")
        order = np.argsort(s)
        s, u = s[order], u[:, order]
        self.transformation_matrix = u @ np.diag(s ** -0.5)

    def diagonalize(self, fock_matrix):
        x = self.transformation_matrix
        e, c = np.linalg.eigh(x.T @ fock_matrix @ x)
        order = np.argsort(e)
        return e[order], x @ c[:, order]

    def orthonormalize(self, matrix):
        x = self.transformation_matrix
        return x.T @ matrix @ x


class DIIS:
    def __init__(self, overlap, linear_algebra, diis_subspace=8):
        self.n = overlap.shape[0]
        self.overlap = overlap
        self.linear_algebra = linear_algebra
        self.fock_array = []
        self.error_array = []
        self.diis_subspace = diis_subspace
        self.begin = False

    def fock_matrix(self, fock, density):
        error = self.overlap @ density @ fock - fock @ density @ self.overlap
        error = self.linear_algebra.orthonormalize(error)
        if np.any(error < 0.1):
            self.begin = True
        if np.all(error < 1e-6):
            self.begin = False
        if self.begin:
            self.error_array.append(error)
            self.fock_array.append(fock)
            if len(self.fock_array) > self.diis_subspace:
                self.fock_array = []
                self.error_array = []
                return fock
            if len(self.fock_array) > 1:
                c = self._coefficients()
                fock = np.zeros((self.n, self.n))
                for k in range(len(self.fock_array)):
                    fock = fock + c[k] * self.fock_array[k]
        return fock

    def _coefficients(self):
        while True:
            m = len(self.fock_array)
            b = np.zeros((m + 1, m + 1))
            b[:m, m] = 1
            b[m, :m] = 1
            for i in range(m):
                for j in range(m):
                    b[i, j] = np.trace(self.error_array[i] @ self.error_array[j].T)
            rhs = np.zeros(m + 1)
            rhs[m] = 1
            try:
                return np.linalg.solve(b, rhs)
            except np.linalg.LinAlgError:
                self.fock_array.pop(0)
                self.error_array.pop(0)


def density_matrix_restricted(c, electrons):
    occ = c[:, :electrons // 2]
    return 2 * occ @ occ.T


def density_matrix_unrestricted(c, electrons):
    occ = c[:, :electrons]
    return occ @ occ.T


def total_energy_restricted(hcore, density, fock):
    return 0.5 * float(np.sum(density * (hcore + fock)))


def total_energy_unrestricted(hcore, pa, pb, fa, fb):
    return 0.5 * float(np.sum((pa + pb) * hcore + pa * fa + pb * fb))


def nuclear_repulsion(charges, coords):
    charges = np.asarray(charges, dtype=np.float64)
    coords = np.asarray(coords, dtype=np.float64)
    e = 0.0
    for i in range(len(charges)):
        for j in range(i + 1, len(charges)):
            e += charges[i] * charges[j] / np.linalg.norm(coords[i] - coords[j])
    return e


class SCFResult(dict):
    __getattr__ = dict.__getitem__


def restricted_scf(overlap, hcore, electrons, fock_builder, threshold=1e-12, max_iter=100,
                   callback=None):
    """RestrictedSCF.begin_iterations: core-Hamiltonian guess, density, Fock, energy,
    DIIS, diagonalise; stop when |dE| < threshold."""
    la = LinearAlgebra(overlap)
    diis = DIIS(overlap, la)
    e_orb, c = la.diagonalize(hcore)
    previous = 0.0
    energies = []
    for it in range(1, max_iter + 1):
        p = density_matrix_restricted(c, electrons)
        f = fock_builder.create(p)
        e = total_energy_restricted(hcore, p, f)
        energies.append(e)
        if callback:
            callback(it, e, p, f)
        if abs(previous - e) < threshold:
            return SCFResult(energy=e, orbital_energies=e_orb, coefficients=c, iterations=it,
                             converged=True, energies=energies, density=p, fock=f)
        previous = e
        f = diis.fock_matrix(f, p)
        e_orb, c = la.diagonalize(f)
    return SCFResult(energy=e, orbital_energies=e_orb, coefficients=c, iterations=max_iter,
                     converged=False, energies=energies, density=p, fock=f)


def ks_restricted_scf(overlap, hcore, electrons, coulomb, exchange_correlation, threshold=1e-12,
                      max_iter=100):
    """KSRestrictedSCF.begin_iterations (kohnsham/kohn_sham_scf.py:14-38) with
    KSEnergy.restricted (kohnsham/kohn_sham_energy.py:10-18): core-Hamiltonian guess; per
    iteration P, J = coulomb(P), (V_xc, E_xc) = exchange_correlation.evaluate(P), the
    energy 2 sum(eps_occ) - sum P (J/2 + V_xc) + E_xc from the previous orbital energies,
    DIIS on H + J + V_xc, diagonalise; stop when |dE| < threshold."""
    la = LinearAlgebra(overlap)
    diis = DIIS(overlap, la)
    e_orb, c = la.diagonalize(hcore)
    previous = 0.0
    energies = []
    nocc = electrons // 2
    for it in range(1, max_iter + 1):
        p = density_matrix_restricted(c, electrons)
        j = coulomb(p)
        v, exc = exchange_correlation.evaluate(p)
        ks = hcore + j + v
        e = 2 * float(np.sum(e_orb[:nocc])) - float(np.sum(p * (0.5 * j + v))) + exc
        energies.append(e)
        if abs(previous - e) < threshold:
            return SCFResult(energy=e, orbital_energies=e_orb, coefficients=c, iterations=it,
                             converged=True, energies=energies, density=p, fock=ks)
        previous = e
        ks = diis.fock_matrix(ks, p)
        e_orb, c = la.diagonalize(ks)
    return SCFResult(energy=e, orbital_energies=e_orb, coefficients=c, iterations=max_iter,
                     converged=False, energies=energies, density=p, fock=ks)


def unrestricted_scf(overlap, hcore, electrons, multiplicity, fock_builder, threshold=1e-12,
                     max_iter=200):
    """PopleNesbetBerthier.begin_iterations (first density from all alpha orbitals as the
    reference does at total_energy == 0)."""
    la = LinearAlgebra(overlap)
    ea_n = (electrons + multiplicity - 1) // 2
    eb_n = (electrons - multiplicity + 1) // 2
    e_orb, c = la.diagonalize(hcore)
    ca = cb = c
    total = previous = 0.0
    for it in range(1, max_iter + 1):
        if total == 0:
            pa = density_matrix_unrestricted(ca, ca.shape[0])
            pb = density_matrix_unrestricted(cb, 0)
        else:
            pa = density_matrix_unrestricted(ca, ea_n)
            pb = density_matrix_unrestricted(cb, eb_n)
        fa, fb = fock_builder.create(pa, pb)
        total = total_energy_unrestricted(hcore, pa, pb, fa, fb)
        if abs(previous - total) < threshold:
            return SCFResult(energy=total, iterations=it, converged=True)
        previous = total
        _, ca = la.diagonalize(fa)
        _, cb = la.diagonalize(fb)
    return SCFResult(energy=total, iterations=max_iter, converged=False)
