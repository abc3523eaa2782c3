"""LDA Kohn-Sham exchange-correlation on the GPU, behind the reference's
``ExchangeCorrelation(basis_set, exchange, correlation)`` (kohnsham/integration.py:7-61).

The reference evaluates every XC matrix element and the XC energy by its own adaptive
quadrature: scipy's ``quad`` on [0, inf) in r around the origin, and at every radial node a
degree-35 Lebedev rule (quadpy) over the sphere, re-evaluating the electron density
function by function at each point.  Here the quadrature is a fixed grid built once:

* radial: Gauss-Chebyshev of the second kind mapped to [0, inf) by r = R (1+x)/(1-x)
  (Becke, J. Chem. Phys. 88, 2547 (1988)), ``radial`` nodes (default 200, R = 1 bohr);
* angular: the product rule of degree 35 (18 Gauss-Legendre nodes in cos(theta) times 36
  equally spaced phi; 648 points, weights summing to 4 pi), the same degree as the
  reference's Lebedev rule, so both integrate the reference's use -- atoms at the origin,
  whose integrands are radial functions times polynomials of degree <= 4 in the direction
  -- exactly in angle.

The grid is centred where the reference centres it, the origin (``centre`` moves it).
Per evaluation: basis values on the grid (``gs_basis_on_grid``, cached across SCF
iterations), rho = diag(Phi P Phi^T) (one GEMM), the functionals per point
(``gs_lda_xc``), V = Phi^T diag(w v) Phi (one GEMM) and E = sum w rho eps.  The GEMMs are
cuBLAS through torch.matmul.
"""
import numpy as np
import torch

from . import _lib
from .basis import ShellBasis
from .engine import DeviceShells

VWN3 = (0.0621814, -0.409286, 13.0720, 42.7198)     # kohnsham/kohn_sham.py:21-28
VWN5 = (0.0621814, -0.10498, 3.72744, 12.9352)


def radial_rule(n=200, scale=1.0):
    """Nodes r (bohr) and weights of int_0^inf f(r) r^2 dr."""
    i = np.arange(1, n + 1)
    t = i * np.pi / (n + 1)
    x = np.cos(t)
    r = scale * (1 + x) / (1 - x)
    w = (np.pi / (n + 1)) * np.sin(t) * 2 * scale / (1 - x) ** 2 * r * r
    return r, w


def angular_rule():
    """Unit vectors (648, 3) and weights (sum 4 pi) of the degree-35 product rule."""
    ct, wt = np.polynomial.legendre.leggauss(18)
    phi = 2 * np.pi * np.arange(36) / 36
    st = np.sqrt(1 - ct * ct)
    dirs = np.stack([np.outer(st, np.cos(phi)), np.outer(st, np.sin(phi)),
                     np.outer(ct, np.ones_like(phi))], axis=-1).reshape(-1, 3)
    return dirs, np.outer(wt, np.full(36, 2 * np.pi / 36)).reshape(-1)


def single_centre_grid(centre=(0.0, 0.0, 0.0), radial=200, scale=1.0):
    """Points (G, 3) and weights (G,) of the spherical grid about ``centre``."""
    r, wr = radial_rule(radial, scale)
    dirs, wa = angular_rule()
    pts = (r[:, None, None] * dirs[None]).reshape(-1, 3) + np.asarray(centre, dtype=np.float64)
    return pts, np.outer(wr, wa).reshape(-1)


def functional_params(exchange, correlation):
    """(slater_alpha, vwn fit or None) from the reference's functional objects, by their
    attributes: SlaterExchange has ``alpha``, VoskoWilkNusair ``a, x_0, b, c``; the base
    Exchange / Correlation (zero functionals) have neither."""
    alpha = float(getattr(exchange, "alpha", 0.0) or 0.0)
    vwn = None
    if correlation is not None and all(hasattr(correlation, k) for k in ("a", "x_0", "b", "c")):
        vwn = (float(correlation.a), float(correlation.x_0), float(correlation.b),
               float(correlation.c))
    return alpha, vwn


class ExchangeCorrelationGPU:
    """Drop-in for the reference's ExchangeCorrelation.  ``basis_set`` is the reference's
    function list (or a ShellBasis); ``exchange``/``correlation`` the reference's functional
    objects, or (alpha, vwn-fit) through ``params``."""

    def __init__(self, basis_set, exchange=None, correlation=None, params=None, radial=200,
                 scale=1.0, centre=(0.0, 0.0, 0.0), device="cuda"):
        self.basis_set = basis_set
        self.exchange = exchange
        self.correlation = correlation
        self.alpha, self.vwn = params if params is not None else functional_params(exchange,
                                                                                    correlation)
        if torch.device(device).type != "cuda":
            raise _lib.GsError("the exchange-correlation quadrature runs on a CUDA device only")
        self.sb = basis_set if isinstance(basis_set, ShellBasis) else ShellBasis.from_functions(basis_set)
        self.ds = DeviceShells(self.sb, device)
        self.device = self.ds.device
        pts, w = single_centre_grid(centre, radial, scale)
        self.points = torch.as_tensor(pts).to(self.device)
        self.weights = torch.as_tensor(w).to(self.device)
        self._phi = None
        self._key = None
        self._result = None

    # ------------------------------------------------------------------ device pieces
    def basis_on(self, points):
        """Phi (G x nbf) at device points (G, 3)."""
        L = _lib.lib()
        points = points.contiguous()
        phi = torch.empty((points.shape[0], self.sb.nbf), dtype=torch.float64, device=self.device)
        ds = self.ds
        _lib.check(L.gs_basis_on_grid(_lib.ptr(ds.centre), _lib.ptr(ds.l), _lib.ptr(ds.prim_off),
                                      _lib.ptr(ds.expo), _lib.ptr(ds.coef), _lib.ptr(ds.comp_scale),
                                      _lib.ptr(ds.func_off), ds.nshell, ds.nbf, points.shape[0],
                                      _lib.ptr(points), _lib.ptr(phi), _lib.stream()),
                   "gs_basis_on_grid")
        return phi

    def phi(self):
        if self._phi is None:
            self._phi = self.basis_on(self.points)
        return self._phi

    def functionals(self, rho, weights):
        """(w v_xc, w rho eps_xc) per point."""
        L = _lib.lib()
        wv = torch.empty_like(rho)
        we = torch.empty_like(rho)
        a, x0, b, c = self.vwn if self.vwn is not None else (0.0, 0.0, 0.0, 1.0)
        _lib.check(L.gs_lda_xc(rho.shape[0], _lib.ptr(rho), _lib.ptr(weights), self.alpha,
                               int(self.vwn is not None), a, x0, b, c, _lib.ptr(wv),
                               _lib.ptr(we), _lib.stream()), "gs_lda_xc")
        return wv, we

    def evaluate_device(self, p):
        """(V_xc matrix, E_xc) for a device density matrix."""
        phi = self.phi()
        rho = ((phi @ p) * phi).sum(dim=1).contiguous()
        wv, we = self.functionals(rho, self.weights)
        v = phi.transpose(0, 1) @ (phi * wv[:, None])
        v = 0.5 * (v + v.transpose(0, 1))
        return v, we.sum()

    def evaluate(self, density_matrix):
        p = np.ascontiguousarray(density_matrix, dtype=np.float64)
        key = p.tobytes()
        if key != self._key:
            v, e = self.evaluate_device(torch.as_tensor(p).to(self.device))
            self._result = (v.cpu().numpy(), float(e.item()))
            self._key = key
        return self._result

    # ------------------------------------------------------------------ reference surface
    def potential_matrix(self, density_matrix):
        """All of integrate_potential(P, i, j) at once (a copy: the cached matrix stays
        intact if the caller updates the returned one in place)."""
        return self.evaluate(density_matrix)[0].copy()

    def integrate_potential(self, density_matrix, i, j):
        return float(self.evaluate(density_matrix)[0][i, j])

    def integrate_energy(self, density_matrix):
        return self.evaluate(density_matrix)[1]

    def electron_density(self, density_matrix, x, y, z):
        pts = torch.tensor([[x, y, z]], dtype=torch.float64, device=self.device)
        phi = self.basis_on(pts)
        p = torch.as_tensor(np.asarray(density_matrix, dtype=np.float64)).to(self.device)
        return float(((phi @ p) * phi).sum().item())


def rks(mol, basis="STO-3G", exchange_alpha=2 / 3, vwn=VWN3, threshold=1e-12, radial=200):
    """Restricted Kohn-Sham energy as the reference's RestrictedKohnSham computes it
    (kohnsham/kohn_sham.py, kohn_sham_scf.py, kohn_sham_energy.py): ERIs (J) from the
    integral engine, XC on the GPU grid about the origin, plus the nuclear repulsion."""
    from . import scf
    from .engine import JKEngine
    from .hamiltonian import one_electron
    from .molecules import shell_basis
    sb = shell_basis(mol, basis)
    S, T, V = one_electron(sb, mol.coords, mol.charges)
    eng = JKEngine(sb, schwarz_thr=1e-14)
    xc = ExchangeCorrelationGPU(sb, params=(exchange_alpha, vwn), radial=radial)

    def coulomb(p):
        J, _ = eng.jk(torch.as_tensor(p).to(eng.dev), [], precision=64)
        return J.cpu().numpy()

    res = scf.ks_restricted_scf(S, T + V, mol.electrons, coulomb, xc, threshold=threshold)
    res["energy"] += scf.nuclear_repulsion(mol.charges, mol.coords)
    return res
