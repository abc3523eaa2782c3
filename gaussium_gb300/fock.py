"""Integral-direct Fock builders with the reference's call surface.

  FockMatrixRestrictedGPU        for FockMatrixRestricted          hartreefock/fock_matrix.py:5-22
  FockMatrixUnrestrictedGPU      for FockMatrixUnrestricted        hartreefock/fock_matrix.py:25-53
  BlockedFockMatrixUnrestrictedGPU for BlockedFockMatrixUnrestricted hartreefock/fock_matrix.py:56-81
  RestrictedKohnShamHamiltonianGPU for RestrictedKohnShamHamiltonian kohnsham/kohn_sham_hamiltonian.py:5-24

Each takes ``(core_hamiltonian, source)`` where ``source`` is a JKEngine, a ShellBasis or
the reference-style list of basis functions (in place of the stored N^4 tensor the
reference passes), keeps ``.core_hamiltonian``, and returns host numpy matrices from
``create`` exactly as the reference does, so the reference's SCF loops
(hartreefock/scf_procedure.py) run unchanged on top.

Options beyond the reference (all off by default, giving the plain FP64 build):
  schwarz_thr   Schwarz threshold for the quartet list (1e-12)
  screen_thr    density-weighted screening threshold per build
  mixed_cut     quartets with density-weighted bound below it run in FP32 (FP64 accumulation)
  incremental   build G[P_n - P_{n-1}] and add it to the previous G; a full build every
                ``reset_every`` calls
"""
import numpy as np
import torch

from .basis import ShellBasis
from .engine import JKEngine


def _engine(source, device, schwarz_thr):
    if isinstance(source, JKEngine):
        return source
    sb = source if isinstance(source, ShellBasis) else ShellBasis.from_functions(source)
    return JKEngine(sb, device=device, schwarz_thr=schwarz_thr)


class _Base:
    def __init__(self, core_hamiltonian, source, device="cuda", schwarz_thr=1e-12,
                 screen_thr=0.0, mixed_cut=None, incremental=False, reset_every=8):
        self.core_hamiltonian = core_hamiltonian
        self.engine = _engine(source, device, schwarz_thr)
        self.matrix_size = self.engine.sb.nbf
        self.device = self.engine.dev
        self.screen_thr = screen_thr
        self.mixed_cut = mixed_cut
        self.incremental = incremental
        self.reset_every = reset_every
        self._prev = None
        self._count = 0
        self.builds = []   # (kind, seconds) per build, for reporting

    def _t(self, m):
        return torch.as_tensor(np.asarray(m), dtype=torch.float64).to(self.device)

    def _jk(self, pj, pk):
        return self.engine.jk(pj, pk, precision=64, screen_thr=self.screen_thr,
                              mixed_cut=self.mixed_cut)

    def _two_electron(self, dens, fn):
        """G for the given densities, incrementally if enabled: fn(densities) -> tuple of G."""
        full = (not self.incremental or self._prev is None or
                (self.reset_every and self._count % self.reset_every == 0))
        self._count += 1
        if full:
            g = fn(dens)
        else:
            pd, pg = self._prev
            dg = fn([d - p for d, p in zip(dens, pd)])
            g = tuple(a + b for a, b in zip(pg, dg))
        if self.incremental:
            self._prev = ([d.clone() for d in dens], tuple(x.clone() for x in g))
        return g

    def reset(self):
        self._prev = None
        self._count = 0


class FockMatrixRestrictedGPU(_Base):
    def create(self, density_matrix):
        p = self._t(density_matrix)

        def g(d):
            J, (K,) = self._jk(d[0], [d[0]])
            return (J - 0.5 * K,)

        (G,) = self._two_electron([p], g)
        return self.core_hamiltonian + G.cpu().numpy()


class FockMatrixUnrestrictedGPU(_Base):
    def create(self, density_matrix_alph, density_matrix_beta):
        pa, pb = self._t(density_matrix_alph), self._t(density_matrix_beta)

        def g(d):
            J, (Ka, Kb) = self._jk(d[0] + d[1], [d[0], d[1]])
            return (J - Ka, J - Kb)

        Ga, Gb = self._two_electron([pa, pb], g)
        return self.core_hamiltonian + Ga.cpu().numpy(), self.core_hamiltonian + Gb.cpu().numpy()


class BlockedFockMatrixUnrestrictedGPU(_Base):
    """GUHF in the spin-blocked 2N basis.  The reference builds the 2N^4 spin-orbital
    tensor (matrixelements/transformations.py:29-70); here the alpha-alpha and beta-beta
    blocks of P give J[Paa + Pbb] on both diagonal blocks and -K[Paa], -K[Pbb].  Densities
    with alpha-beta coupling (never produced by the reference's block-diagonal
    coefficients, hartreefock/linear_algebra.py:34-61) are rejected."""

    def __init__(self, core_hamiltonian, source, **kw):
        super().__init__(core_hamiltonian, source, **kw)
        self.matrix_size = 2 * self.engine.sb.nbf

    def create(self, density_matrix):
        n = self.engine.sb.nbf
        p = np.asarray(density_matrix)
        if p.shape != (2 * n, 2 * n):
            raise ValueError(f"blocked density must be {2 * n}x{2 * n}")
        if np.any(p[:n, n:] != 0) or np.any(p[n:, :n] != 0):
            raise NotImplementedError("alpha-beta blocks of the density must be zero")
        pa, pb = self._t(p[:n, :n]), self._t(p[n:, n:])

        def g(d):
            J, (Ka, Kb) = self._jk(d[0] + d[1], [d[0], d[1]])
            return (J - Ka, J - Kb)

        Ga, Gb = self._two_electron([pa, pb], g)
        G = np.zeros((2 * n, 2 * n))
        G[:n, :n] = Ga.cpu().numpy()
        G[n:, n:] = Gb.cpu().numpy()
        return self.core_hamiltonian + G


class RestrictedKohnShamHamiltonianGPU(_Base):
    """Returns (core_hamiltonian, J, XC) like the reference's create; J comes from the
    engine, XC from the caller's exchange-correlation object: the whole matrix at once from
    ``kohnsham.ExchangeCorrelationGPU``, element by element (as the reference evaluates it)
    from any other object."""

    def __init__(self, core_hamiltonian, source, exchange_correlation=None, **kw):
        super().__init__(core_hamiltonian, source, **kw)
        self.exchange_correlation = exchange_correlation

    def create(self, density_matrix):
        p = self._t(density_matrix)

        def g(d):
            J, _ = self.engine.jk(d[0], [], precision=64, screen_thr=self.screen_thr,
                                  mixed_cut=self.mixed_cut)
            return (J,)

        (J,) = self._two_electron([p], g)
        xc = None
        if hasattr(self.exchange_correlation, "potential_matrix"):
            # the GPU exchange-correlation object builds the whole matrix in one pass
            xc = self.exchange_correlation.potential_matrix(density_matrix)
        elif self.exchange_correlation is not None:
            n = self.matrix_size
            xc = np.zeros((n, n))
            for i in range(n):
                for j in range(i, n):
                    xc[i, j] = xc[j, i] = self.exchange_correlation.integrate_potential(
                        density_matrix, i, j)
        return self.core_hamiltonian, J.cpu().numpy(), xc


class _BasisOnly:
    """Stands in for TwoElectronRepulsionMatrixOS inside HartreeFock.__init__
    (hartreefock/hartree_fock.py:38-41): instead of the N^4 tensor it hands on the
    basis-function list, which the drop-in Fock builders take as their source."""

    def __init__(self, basis_set_array, symmetry=None, processes=1):
        self.basis_set_array = basis_set_array

    def create_repulsion_matrix(self):
        return self.basis_set_array


def _mo_from_source(repulsion, coefficients):
    """``molecular_orbitals`` for callers of an installed package, whose
    ``hartree_fock.repulsion`` is the basis-function list (``_BasisOnly``): the MO tensor
    is built from the shells on the device; a dense tensor goes through the drop-in."""
    from . import transform
    from .basis import ShellBasis
    if isinstance(repulsion, (list, tuple)):
        sb = ShellBasis.from_functions(repulsion)
        return transform.mo_integrals(sb, coefficients).cpu().numpy()
    return transform.molecular_orbitals(repulsion, coefficients)


# post-SCF modules of the reference and the transform names each imports
# (moellerplesset/moeller_plesset.py:2, coupledcluster/coupled_cluster.py:5-6,
# tdhartreefock/td_hartree_fock.py:3-4)
_POST_SCF = (("moellerplesset", "moeller_plesset"), ("coupledcluster", "coupled_cluster"),
             ("tdhartreefock", "td_hartree_fock"))


def install(gaussium, **options):
    """Route a loaded reference package's SCF through this engine: in
    ``gaussium.hartreefock.hartree_fock`` the tensor builder becomes ``_BasisOnly``, the
    three Fock builders become the GPU drop-ins, and the spin-blocking of the tensor
    (``blocked_spin_basis_set``) passes the basis list through (the blocked drop-in builds
    the spin blocks itself); in ``gaussium.kohnsham.kohn_sham`` the Kohn-Sham Hamiltonian
    and the exchange-correlation quadrature become their drop-ins.  In the post-SCF modules (MP2, CCSD, TDHF) that are loaded,
    ``molecular_orbitals`` builds the MO tensor from the basis list on the device and
    ``spin_basis_set`` / ``spin_basis_anti_physicist`` become the GPU drop-ins.
    ``options`` (e.g. ``mixed_cut``, ``incremental``) go to every builder.  Returns the
    replaced originals, keyed by module attribute, for undoing."""
    import functools
    from . import transform
    hf = gaussium.hartreefock.hartree_fock
    swaps = [(hf, "TwoElectronRepulsionMatrixOS", _BasisOnly),
             (hf, "FockMatrixRestricted", functools.partial(FockMatrixRestrictedGPU, **options)),
             (hf, "FockMatrixUnrestricted", functools.partial(FockMatrixUnrestrictedGPU, **options)),
             (hf, "BlockedFockMatrixUnrestricted",
              functools.partial(BlockedFockMatrixUnrestrictedGPU, **options)),
             (hf, "blocked_spin_basis_set", lambda basis: basis)]
    ks = getattr(getattr(gaussium, "kohnsham", None), "kohn_sham", None)
    if ks is not None:
        from .kohnsham import ExchangeCorrelationGPU
        swaps.append((ks, "RestrictedKohnShamHamiltonian",
                      functools.partial(RestrictedKohnShamHamiltonianGPU, **options)))
        if hasattr(ks, "ExchangeCorrelation"):
            swaps.append((ks, "ExchangeCorrelation", ExchangeCorrelationGPU))
    for pkg, modname in _POST_SCF:
        mod = getattr(getattr(gaussium, pkg, None), modname, None)
        if mod is None:
            continue
        for name, new in (("molecular_orbitals", _mo_from_source),
                          ("spin_basis_set", transform.spin_basis_set),
                          ("spin_basis_anti_physicist", transform.spin_basis_anti_physicist)):
            if hasattr(mod, name):
                swaps.append((mod, name, new))
    originals = {}
    for mod, name, new in swaps:
        originals[(mod.__name__, name)] = getattr(mod, name)
        setattr(mod, name, new)
    return originals


def uninstall(originals):
    """Undo ``install``: put back the attributes it replaced (its return value)."""
    import sys
    for (modname, name), value in originals.items():
        setattr(sys.modules[modname], name, value)
