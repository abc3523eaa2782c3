"""Geometry optimisation: the reference's Nelder-Mead driver restated over the GPU energy,
and a gradient-driven optimiser over the analytic gradient.

``NelderMead`` follows geometryoptimization/nelder_mead.py:11-187: internal frame (first
nucleus at the origin, second on the z axis, third in the yz plane), m = 3N-6 variables
(1 for a diatomic),
initial simplex by +tau on each variable, adaptive coefficients alpha = 1,
beta = 2 + 2/m, gamma = 0.75 + 1/(2m), delta = 0.5 - 1/m, and the stop when the standard
deviation of the simplex energies is <= threshold.

``optimize_bfgs`` minimises the RHF energy with scipy's BFGS on the analytic gradient
(gaussium_gb300.gradient), over the same internal-frame variables.
"""
import numpy as np

from .gradient import rhf_energy_gradient
from .molecules import Molecule


def _internal_frame(coords):
    c = np.asarray(coords, dtype=np.float64) - coords[0]
    if len(c) >= 2:
        v = c[1] / np.linalg.norm(c[1])
        z = np.array([0.0, 0.0, 1.0])
        axis = np.cross(v, z)
        s, cth = np.linalg.norm(axis), float(v @ z)
        if s > 1e-12:
            axis /= s
            ang = np.arctan2(s, cth)
            K = np.array([[0, -axis[2], axis[1]], [axis[2], 0, -axis[0]], [-axis[1], axis[0], 0]])
            R = np.eye(3) + np.sin(ang) * K + (1 - np.cos(ang)) * K @ K
            c = c @ R.T
    if len(c) >= 3:
        x, y = c[2, 0], c[2, 1]
        ang = np.arctan2(x, y)              # rotate about z so the third lies in yz (x = 0)
        R = np.array([[np.cos(ang), -np.sin(ang), 0], [np.sin(ang), np.cos(ang), 0], [0, 0, 1]])
        c = c @ R.T
    return c


class NelderMead:
    def __init__(self, symbols, coords, energy_fn, tau=0.25, threshold=1e-6, max_evals=100000):
        self.symbols = list(symbols)
        self.frame = _internal_frame(coords)
        n = len(self.symbols)
        self.m = 1 if n <= 2 else 3 * n - 6
        self.alpha = 1
        self.beta = 2 + 2 / self.m
        self.gamma = 0.75 + 1 / (2 * self.m)
        self.delta = 0.5 - 1 / self.m
        self.tau = tau
        self.threshold = threshold
        self.energy_fn = energy_fn
        self.evals = 0
        self.max_evals = max_evals

    def _vector(self, c):
        v = []
        for i in range(1, len(c)):
            if i == 1:
                v.append(c[1, 2])
            elif i == 2:
                v.extend([c[2, 1], c[2, 2]])
            else:
                v.extend(c[i])
        return np.array(v) if len(c) > 1 else np.array([c[0, 2]])

    def coordinates(self, v):
        n = len(self.symbols)
        c = np.zeros((n, 3))
        if n == 1:
            c[0, 2] = v[0]
            return c
        j = 0
        for i in range(1, n):
            if i == 1:
                c[1, 2] = v[j]; j += 1
            elif i == 2:
                c[2, 1], c[2, 2] = v[j], v[j + 1]; j += 2
            else:
                c[i] = v[j:j + 3]; j += 3
        return c

    def energy(self, v):
        self.evals += 1
        return self.energy_fn(Molecule(self.symbols, self.coordinates(v)))

    def optimize(self):
        x0 = self._vector(self.frame)
        m = len(x0)
        simplex = [x0.copy()] + [x0 + self.tau * np.eye(m)[i] for i in range(m)]
        energies = [self.energy(p) for p in simplex]
        while np.std(energies) > self.threshold and self.evals < self.max_evals:
            order = np.argsort(energies)
            imax = int(order[-1])
            e_max, e_second, e_min = energies[imax], energies[int(order[-2])], energies[int(order[0])]
            centroid = (np.sum(simplex, axis=0) - simplex[imax]) / m
            refl = centroid + self.alpha * (centroid - simplex[imax])
            e_r = self.energy(refl)
            if e_min <= e_r < e_second:
                simplex[imax], energies[imax] = refl, e_r
            elif e_r < e_min:
                exp_ = centroid + self.beta * (refl - centroid)
                e_e = self.energy(exp_)
                simplex[imax], energies[imax] = (exp_, e_e) if e_e < e_r else (refl, e_r)
            elif e_second <= e_r < e_max:
                oc = centroid + self.gamma * (refl - centroid)
                e_oc = self.energy(oc)
                if e_oc <= e_r:
                    simplex[imax], energies[imax] = oc, e_oc
                else:
                    simplex, energies = self._shrink(simplex, energies)
            else:
                ic = centroid - self.gamma * (refl - centroid)
                e_ic = self.energy(ic)
                if e_ic < e_max:
                    simplex[imax], energies[imax] = ic, e_ic
                else:
                    simplex, energies = self._shrink(simplex, energies)
        best = int(np.argmin(energies))
        return energies[best], self.coordinates(simplex[best])

    def _shrink(self, simplex, energies):
        best = simplex[int(np.argmin(energies))]
        simplex = [best + self.delta * (p - best) for p in simplex]
        return simplex, [self.energy(p) for p in simplex]


def optimize_bfgs(mol, basis="6-31G", gtol=1e-5, max_iter=500, energy_gradient=None,
                  method="L-BFGS-B"):
    """Gradient-driven minimisation in the Nelder-Mead driver's internal frame (first nucleus
    at the origin, second on z, third in the yz plane: 3N-6 variables, so the six zero
    modes of overall translation and rotation are not searched).  The energy is invariant
    under those motions, so the derivative with respect to each free variable is the
    Cartesian gradient component that variable sets.  Returns (energy, coordinates,
    evaluations, max |gradient| at the end).  ``energy_gradient(molecule) -> (E, dE/dR)``
    defaults to the RHF energy and analytic gradient in ``basis``.  ``method`` is a scipy
    quasi-Newton method: "L-BFGS-B" (default; its initial Hessian is scaled from the first
    step, which matters for the soft intermolecular modes of clusters) or "BFGS"."""
    from scipy.optimize import minimize
    symbols = mol.symbols
    frame = NelderMead(symbols, mol.coords, None)
    count = [0]

    def fg(v):
        count[0] += 1
        c = frame.coordinates(v)
        if energy_gradient is None:
            e, g, _ = rhf_energy_gradient(Molecule(symbols, c), basis)
        else:
            e, g = energy_gradient(Molecule(symbols, c))
        return e, frame._vector(np.asarray(g))

    x0 = frame._vector(frame.frame)
    if method == "L-BFGS-B":
        opts = {"gtol": gtol, "maxiter": max_iter, "maxcor": 30, "ftol": 1e-14}
    else:
        opts = {"gtol": gtol, "maxiter": max_iter}
    r = minimize(fg, x0, jac=True, method=method, options=opts)
    return float(r.fun), frame.coordinates(r.x), count[0], float(np.abs(r.jac).max())
