"""ORACLE — test infrastructure only.

ctypes front end of ``eri_oracle.c`` (the CPU restatement of the reference's
Obara-Saika ERI and Boys function) plus numpy restatements of the reference's Fock
builders and SCF loop.  Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU legs of
``bench.py`` import this module: the tests and smoke compare the GPU results with it, the
CPU legs time it on the host cores.  The product path never calls it.

Restated reference functions (file:line within the reference project):
  FockMatrixRestricted.create            hartreefock/fock_matrix.py:12-22
  FockMatrixUnrestricted.create          hartreefock/fock_matrix.py:32-53
  BlockedFockMatrixUnrestricted.create   hartreefock/fock_matrix.py:63-81
  RestrictedKohnShamHamiltonian J part   kohnsham/kohn_sham_hamiltonian.py:15-19
  TwoElectronRepulsion.create_repulsion_matrix  matrixelements/electron_repulsion_matrix.py:28-47
  Symmetry.sort_index                    common/symmetry.py:186-197
  MoellerPlesset.second_order            moellerplesset/moeller_plesset.py:14-22
                                         (index loops: common/indices.py:30-32, 70-80)
"""
import ctypes
import itertools
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIBPATH = os.path.join(BUILD, "liberi_oracle.so")

COMPONENTS = {0: [(0, 0, 0)],
              1: [(1, 0, 0), (0, 1, 0), (0, 0, 1)],
              2: [(2, 0, 0), (0, 2, 0), (0, 0, 2), (1, 1, 0), (1, 0, 1), (0, 1, 1)]}

_lib = None


def build(force=False):
    """Compile eri_oracle.c with gcc into oracle/_build (no reference files involved)."""
    src = os.path.join(HERE, "eri_oracle.c")
    os.makedirs(BUILD, exist_ok=True)
    if not force and os.path.exists(LIBPATH) and os.path.getmtime(LIBPATH) >= os.path.getmtime(src):
        return LIBPATH
    tmp = LIBPATH + ".tmp%d" % os.getpid()
    subprocess.check_call(["gcc", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-o", tmp,
                           src, "-lm", "-lpthread"])
    os.replace(tmp, LIBPATH)
    return LIBPATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIBPATH)
        L.oracle_boys_reference.restype = ctypes.c_double
        L.oracle_boys_reference.argtypes = [ctypes.c_int, ctypes.c_double]
        L.oracle_boys_exact.restype = ctypes.c_double
        L.oracle_boys_exact.argtypes = [ctypes.c_int, ctypes.c_double]
        L.oracle_eri_functions.restype = ctypes.c_int
        P = ctypes.c_void_p
        L.oracle_eri_functions.argtypes = [ctypes.c_int, P, P, P, P, P, P, P, ctypes.c_long, P,
                                           ctypes.c_int, ctypes.c_int, ctypes.c_int, P]
        _lib = L
    return _lib


def boys_reference(v, x):
    return lib().oracle_boys_reference(int(v), float(x))


def boys_exact(v, x):
    return lib().oracle_boys_exact(int(v), float(x))


class FunctionTable:
    """Contracted Cartesian functions in the reference's per-function layout
    (objects/basis_function.py, objects/primitive_basis_function.py): centre, integral
    exponents, contracted normalisation, and per primitive (contraction, exponent,
    primitive normalisation)."""

    def __init__(self, centre, lmn, cnorm, prims):
        self.centre = np.ascontiguousarray(centre, dtype=np.float64).reshape(-1, 3)
        self.lmn = np.ascontiguousarray(lmn, dtype=np.int32).reshape(-1, 3)
        self.cnorm = np.ascontiguousarray(cnorm, dtype=np.float64)
        starts = [0]
        coef, expo, pnorm = [], [], []
        for plist in prims:
            for c, e, n in plist:
                coef.append(c); expo.append(e); pnorm.append(n)
            starts.append(len(coef))
        self.pstart = np.array(starts, dtype=np.int32)
        self.coef = np.array(coef, dtype=np.float64)
        self.expo = np.array(expo, dtype=np.float64)
        self.pnorm = np.array(pnorm, dtype=np.float64)

    def __len__(self):
        return len(self.cnorm)

    @classmethod
    def from_arrays(cls, d):
        """From the ``basis_arrays`` layout of the golden fixtures."""
        prims = []
        for i in range(len(d["norm"])):
            k = int(d["nprim"][i])
            prims.append(list(zip(d["coef"][i, :k], d["expo"][i, :k], d["pnorm"][i, :k])))
        return cls(d["centre"], d["lmn"], d["norm"], prims)

    @classmethod
    def from_shells(cls, shells):
        """Expand shells (dict l, centre, expo, coef) into reference-normalised Cartesian
        functions, in the reference's component order (factory/primitive_basis_factory.py:5-86)
        with the reference's normalisation formulas (objects/primitive_basis_function.py:26-42,
        objects/basis_function.py:22-53)."""
        centre, lmn, cnorm, prims = [], [], [], []
        for sh in shells:
            for comp in COMPONENTS[int(sh["l"])]:
                pn = [primitive_norm(e, comp) for e in sh["expo"]]
                centre.append(sh["centre"]); lmn.append(comp)
                cnorm.append(contracted_norm(sh["coef"], sh["expo"], pn, comp))
                prims.append(list(zip(sh["coef"], sh["expo"], pn)))
        return cls(np.array(centre), np.array(lmn), np.array(cnorm), prims)


def _fact2(n):
    r = 1.0
    while n > 1:
        r *= n
        n -= 2
    return r


def primitive_norm(alpha, lmn):
    """PrimitiveBasis.normalisation, objects/primitive_basis_function.py:26-42
    (factorial2(n <= 0) = 1 as in scipy < 1.11)."""
    l, m, n = lmn
    out1 = _fact2(2 * l - 1) * _fact2(2 * m - 1) * _fact2(2 * n - 1)
    out2 = (np.pi / (2 * alpha)) ** (3 / 2)
    out3 = (4 * alpha) ** (l + m + n)
    return 1 / np.sqrt((out1 * out2) / out3)


def contracted_norm(coef, expo, pnorm, lmn):
    """Basis.normalisation, objects/basis_function.py:22-53 (1 for a single primitive)."""
    if len(coef) == 1:
        return 1.0
    l, m, n = lmn
    ans = 0.0
    for (c1, a1, n1), (c2, a2, n2) in itertools.product(list(zip(coef, expo, pnorm)), repeat=2):
        out1 = _fact2(2 * l - 1) * _fact2(2 * m - 1) * _fact2(2 * n - 1)
        out2 = (np.pi / (a1 + a2)) ** (3 / 2)
        out3 = (2 * (a1 + a2)) ** (l + m + n)
        ans += (c1 * c2 * n1 * n2 * out1 * out2) / out3
    return 1 / np.sqrt(ans)


def eri_functions(table, quartets, boys_mode=1, memo=True, threads=None):
    """ERIs of function quartets (n x 4 indices into ``table``) by the restated
    ObaraSaika.integrate.  boys_mode 0: the reference's Boys series; 1: accurate Boys."""
    q = np.ascontiguousarray(quartets, dtype=np.int32).reshape(-1, 4)
    out = np.zeros(len(q))
    if threads is None:
        threads = os.cpu_count() or 1
    t = table
    rc = lib().oracle_eri_functions(
        len(t), t.centre.ctypes.data, t.lmn.ctypes.data, t.cnorm.ctypes.data, t.pstart.ctypes.data,
        t.coef.ctypes.data, t.expo.ctypes.data, t.pnorm.ctypes.data, len(q), q.ctypes.data,
        int(boys_mode), int(bool(memo)), int(threads), out.ctypes.data)
    if rc != 0:
        raise ValueError("oracle_eri_functions rejected its arguments")
    return out


def sort_index(a, b, c, d):
    """Symmetry.sort_index, common/symmetry.py:186-197."""
    if a > b:
        a, b = b, a
    if c > d:
        c, d = d, c
    if a > c:
        a, c = c, a
        b, d = d, b
    if a == c and b > d:
        a, c = c, a
        b, d = d, b
    return a, b, c, d


def canonical_keys(n):
    """The key list of create_repulsion_matrix, electron_repulsion_matrix.py:30-33."""
    return np.array([(a, b, c, d) for a, b, c, d in itertools.product(range(n), repeat=4)
                     if not (a > b or c > d or a > c or (a == c and b > d))], dtype=np.int32)


def dense_tensor(table, boys_mode=1, threads=None):
    """create_repulsion_matrix: canonical keys, evaluated, expanded 8-fold (dense N^4)."""
    n = len(table)
    keys = canonical_keys(n)
    vals = eri_functions(table, keys, boys_mode=boys_mode, threads=threads)
    return expand_dense(n, keys, vals)


def expand_dense(n, keys, vals):
    t = np.zeros((n, n, n, n))
    for (a, b, c, d), v in zip(keys.tolist(), vals.tolist()):
        for (i, j, k, l) in ((a, b, c, d), (b, a, c, d), (a, b, d, c), (b, a, d, c),
                             (c, d, a, b), (d, c, a, b), (c, d, b, a), (d, c, b, a)):
            t[i, j, k, l] = v
    return t


# ---------------------------------------------------------------- Fock restatements
def fock_restricted(hcore, eri, p):
    """FockMatrixRestricted.create: F = H + sum_ab P_ab [(ij|ab) - 1/2 (ib|aj)]."""
    return hcore + np.einsum("ab,ijab->ij", p, eri) - 0.5 * np.einsum("ab,ibaj->ij", p, eri)


def fock_unrestricted(hcore, eri, pa, pb):
    """FockMatrixUnrestricted.create: J from Pa+Pb, exchange per spin."""
    j = np.einsum("ab,ijab->ij", pa + pb, eri)
    return (hcore + j - np.einsum("ab,ibaj->ij", pa, eri),
            hcore + j - np.einsum("ab,ibaj->ij", pb, eri))


def fock_blocked(hcore2, eri2, p2):
    """BlockedFockMatrixUnrestricted.create on the spin-blocked 2N tensor."""
    return hcore2 + np.einsum("ab,ijab->ij", p2, eri2) - np.einsum("ab,ibaj->ij", p2, eri2)


def coulomb(eri, p):
    """RestrictedKohnShamHamiltonian.create, calculate_elst: J_ij = sum_ab P_ab (ij|ab)."""
    return np.einsum("ab,ijab->ij", p, eri)


# ---------------------------------------------------------------------- AO -> MO transforms
# Restatements of matrixelements/transformations.py (test infrastructure, like the rest of
# this file): the reference's loops, in numpy.

def molecular_orbitals(repulsion, coefficients):
    """transformations.py:5-26: C^T X C over the last index pair for every (r, s), then over
    the first pair for every (t, u)."""
    x = np.array(repulsion, dtype=np.float64, copy=True)
    c = np.asarray(coefficients)
    n = c.shape[0]
    for r in range(n):
        for s in range(n):
            x[r, s, :, :] = c.T @ x[r, s, :, :] @ c
    for t in range(n):
        for u in range(n):
            x[:, :, t, u] = c.T @ x[:, :, t, u] @ c
    return x


def blocked_spin_basis_set(repulsion):
    """transformations.py:29-70: alpha block first, beta second; (r s| only within a spin."""
    h = repulsion.shape[0]
    out = np.zeros((2 * h,) * 4)
    for r in range(2 * h):
        for s in range(2 * h):
            if (r < h) == (s < h):
                blk = repulsion[r % h, s % h]
                out[r, s, :h, :h] = blk
                out[r, s, h:, h:] = blk
    return out


def spin_basis_set(repulsion):
    """transformations.py:73-92: interleaved spins, (rs|tu) = (r/2 s/2|t/2 u/2) when r, s share
    a spin and t, u share a spin."""
    n = 2 * repulsion.shape[0]
    out = np.zeros((n,) * 4)
    for r in range(n):
        for s in range(n):
            if r % 2 != s % 2:
                continue
            for t in range(n):
                for u in range(n):
                    if t % 2 == u % 2:
                        out[r, s, t, u] = repulsion[r // 2, s // 2, t // 2, u // 2]
    return out


def spin_basis_anti_physicist(repulsion):
    """transformations.py:114-136: <rs||tu> = [rt|su] d(r,t) d(s,u) - [ru|st] d(r,u) d(s,t)
    over interleaved spins."""
    n = 2 * repulsion.shape[0]
    out = np.zeros((n,) * 4)
    for r in range(n):
        for s in range(n):
            for t in range(n):
                for u in range(n):
                    a = (r % 2 == t % 2) * (s % 2 == u % 2) * repulsion[r // 2, t // 2, s // 2, u // 2]
                    b = (r % 2 == u % 2) * (s % 2 == t % 2) * repulsion[r // 2, u // 2, s // 2, t // 2]
                    out[r, s, t, u] = a - b
    return out


def mp2_correlation(mo, orbital_energies, occupied):
    """MoellerPlesset.second_order: for occupied i, j and unoccupied a, b, the sum of
    [2 (ia|jb)^2 - (ia|jb)(ib|ja)] / (e_i + e_j - e_a - e_b) over the MO tensor in
    chemists' order (the reference's molecular_orbitals)."""
    e = np.asarray(orbital_energies, dtype=np.float64)
    o, v = slice(0, occupied), slice(occupied, len(e))
    iajb = np.asarray(mo)[o, v, o, v]
    ibja = iajb.transpose(0, 3, 2, 1)
    denom = (e[o, None, None, None] + e[None, None, o, None]
             - e[None, v, None, None] - e[None, None, None, v])
    return float(np.sum((2.0 * iajb * iajb - iajb * ibja) / denom))


# ---------------------------------------------------------------------- LDA exchange-correlation
# Restatements of kohnsham/ (test infrastructure, like the rest of this file).  The
# reference's angular rule is quadpy's Lebedev rule of degree 35 (kohnsham/integration.py:
# 53-61; quadpy is not installed here).  The oracle uses a product rule of the same degree
# instead: 18 Gauss-Legendre nodes in cos(theta) times 36 equally spaced phi (exact for
# spherical harmonics up to degree 35, weights summing to 4 pi).  On the reference's own
# use, atoms at the origin, every integrand is a radial function times a polynomial of
# degree <= 4 in the direction, which both rules integrate exactly.  Radial: scipy's
# adaptive quad on [0, inf) with its default tolerances, as the reference.

def slater_energy(rho, alpha):
    """SlaterExchange.energy, kohnsham/exchange/slater_exchange.py (per electron)."""
    return -(9 / 8) * alpha * (3 / np.pi) ** (1 / 3) * np.cbrt(rho)


def slater_potential(rho, alpha):
    """SlaterExchange.potential."""
    return -(3 / 2) * alpha * (3 / np.pi) ** (1 / 3) * np.cbrt(rho)


def _vwn_terms(rho, a, x0, b, c):
    rs = (3 / (4 * np.pi * rho)) ** (1 / 3)
    x = np.sqrt(rs)
    xx = x * x + b * x + c
    xx0 = x0 * x0 + b * x0 + c
    q = np.sqrt(4 * c - b * b)
    at = np.arctan(q / (2 * x + b))
    e = (a / 2) * (np.log(x * x / xx) + (2 * b / q) * at
                   - (b * x0 / xx0) * (np.log((x - x0) ** 2 / xx) + (2 * (b + 2 * x0) / q) * at))
    return x, xx, e


def vwn_energy(rho, a, x0, b, c):
    """VoskoWilkNusair._energy, kohnsham/correlation/local_density.py (a in Rydberg, halved
    to Hartree; 0 at zero density)."""
    rho = np.asarray(rho, dtype=np.float64)
    out = np.zeros_like(rho)
    m = rho != 0
    out[m] = _vwn_terms(rho[m], a, x0, b, c)[2]
    return out


def vwn_potential(rho, a, x0, b, c):
    """VoskoWilkNusair._potential."""
    rho = np.asarray(rho, dtype=np.float64)
    out = np.zeros_like(rho)
    m = rho != 0
    x, xx, e = _vwn_terms(rho[m], a, x0, b, c)
    out[m] = e - (a / 2 / 3) * ((c * (x - x0) - b * x0 * x) / ((x - x0) * xx))
    return out


VWN3 = (0.0621814, -0.409286, 13.0720, 42.7198)     # kohnsham/kohn_sham.py:21-28
VWN5 = (0.0621814, -0.10498, 3.72744, 12.9352)


def basis_values(table, pts):
    """Basis.value / PrimitiveBasis.value (objects/basis_function.py, objects/
    primitive_basis_function.py:44-60) of every function at points (n, 3)."""
    pts = np.asarray(pts, dtype=np.float64).reshape(-1, 3)
    out = np.zeros((len(pts), len(table)))
    for f in range(len(table)):
        d = pts - table.centre[f]
        r2 = np.sum(d * d, axis=1)
        poly = np.prod(d ** table.lmn[f], axis=1)
        s = np.zeros(len(pts))
        for k in range(table.pstart[f], table.pstart[f + 1]):
            s += table.pnorm[k] * table.coef[k] * np.exp(-table.expo[k] * r2)
        out[:, f] = table.cnorm[f] * poly * s
    return out


def electron_density(table, p, pts):
    """ExchangeCorrelation.electron_density, kohnsham/integration.py:14-24."""
    phi = basis_values(table, pts)
    return np.einsum("ga,ab,gb->g", phi, p, phi)


def angular_rule():
    """Product rule of degree 35 on the unit sphere: unit vectors (648, 3), weights."""
    ct, wt = np.polynomial.legendre.leggauss(18)
    phi = 2 * np.pi * np.arange(36) / 36
    st = np.sqrt(1 - ct * ct)
    dirs = np.stack([np.outer(st, np.cos(phi)), np.outer(st, np.sin(phi)),
                     np.outer(ct, np.ones_like(phi))], axis=-1).reshape(-1, 3)
    w = np.outer(wt, np.full(36, 2 * np.pi / 36)).reshape(-1)
    return dirs, w


def _xc_parts(rho, alpha, vwn):
    e = np.zeros_like(rho)
    v = np.zeros_like(rho)
    if alpha:
        e += slater_energy(rho, alpha)
        v += slater_potential(rho, alpha)
    if vwn is not None:
        e += vwn_energy(rho, *vwn)
        v += vwn_potential(rho, *vwn)
    return e, v


def xc_integrate(fn):
    """ExchangeCorrelation.integrate, kohnsham/integration.py:53-61: radial quad of the
    spherical integral of fn(points (n, 3)) r^2 about the origin."""
    from scipy import integrate
    dirs, w = angular_rule()
    return integrate.quad(lambda r: float(np.dot(w, fn(r * dirs))) * r * r, 0.0, np.inf)[0]


def xc_potential_matrix(table, p, alpha, vwn):
    """ExchangeCorrelation.integrate_potential (kohnsham/integration.py:26-40) for every
    (i, j), i <= j mirrored, as RestrictedKohnShamHamiltonian.create builds it
    (kohnsham/kohn_sham_hamiltonian.py:21-24)."""
    n = len(table)
    out = np.zeros((n, n))
    for i in range(n):
        for j in range(i, n):
            def f(pts, i=i, j=j):
                phi = basis_values(table, pts)
                rho = np.einsum("ga,ab,gb->g", phi, p, phi)
                return phi[:, i] * _xc_parts(rho, alpha, vwn)[1] * phi[:, j]
            out[i, j] = out[j, i] = xc_integrate(f)
    return out


def xc_energy(table, p, alpha, vwn):
    """ExchangeCorrelation.integrate_energy, kohnsham/integration.py:42-51."""
    def f(pts):
        rho = electron_density(table, p, pts)
        return rho * _xc_parts(rho, alpha, vwn)[0]
    return xc_integrate(f)


def ks_restricted_scf(overlap, hcore, eri, electrons, table, alpha, vwn, threshold=1e-12,
                      max_iter=60):
    """KSRestrictedSCF.begin_iterations (kohnsham/kohn_sham_scf.py:14-38) with
    KSEnergy.restricted (kohnsham/kohn_sham_energy.py:10-18): core guess, then
    P -> (H, J, XC), E = 2 sum(eps_occ) - sum P (J/2 + XC) + Exc, until |dE| < threshold.
    Plain Roothaan steps (the reference's DIIS changes the path, not the fixed point)."""
    s_eval, s_vec = np.linalg.eigh(overlap)
    x = s_vec / np.sqrt(s_eval)
    eps, c = np.linalg.eigh(x.T @ hcore @ x)
    c = x @ c
    previous = 0.0
    for _ in range(max_iter):
        occ = c[:, :electrons // 2]
        p = 2 * occ @ occ.T
        j = coulomb(eri, p)
        v = xc_potential_matrix(table, p, alpha, vwn)
        e = 2 * np.sum(eps[:electrons // 2]) - np.sum(p * (0.5 * j + v)) + xc_energy(table, p, alpha, vwn)
        if abs(previous - e) < threshold:
            return e
        previous = e
        eps, c = np.linalg.eigh(x.T @ (hcore + j + v) @ x)
        c = x @ c
    return e


def one_centre_s(table, charge):
    """S, T, V of s functions that all sit on one nucleus of the given charge (closed forms
    of integrals/orbital_overlap_integral.py, matrixelements/kinetic_energy_matrix.py and
    integrals/nuclear_attraction_integral.py for l = 0, |AB| = |AC| = 0)."""
    n = len(table)
    S, T, V = (np.zeros((n, n)) for _ in range(3))
    for i in range(n):
        for j in range(n):
            for a in range(table.pstart[i], table.pstart[i + 1]):
                for b in range(table.pstart[j], table.pstart[j + 1]):
                    pa, pb = table.expo[a], table.expo[b]
                    k = (table.cnorm[i] * table.cnorm[j] * table.coef[a] * table.coef[b]
                         * table.pnorm[a] * table.pnorm[b])
                    p = pa + pb
                    s = (np.pi / p) ** 1.5
                    S[i, j] += k * s
                    T[i, j] += k * 3 * pa * pb / p * s
                    V[i, j] += -k * charge * 2 * np.pi / p
    return S, T, V


# ---------------------------------------------------------------------- point-group screening
def symmetry_nonzero(table, flip, centre_id, parity, key):
    """Symmetry.none_zero_integral (common/symmetry.py:18-47) for a non-C1 group, from its
    tables: table[f, m-1] = signed 1-based image of function f under operation m (0: none,
    basis_set_symmetry_matrix), flip[m-1, p] = whether operation m changes the parity vector
    p (symmetry_exponent_dict), centre_id[f] (functions on one centre share it),
    parity[f] = bits (l mod 2, m mod 2, n mod 2) of the integral exponents."""
    i, j, k, l = (int(x) for x in key)
    p = parity[i] ^ parity[j] ^ parity[k] ^ parity[l]
    if centre_id[i] == centre_id[j] == centre_id[k] == centre_id[l]:
        return p == 0
    for m in range(table.shape[1]):
        a, b, c, d = table[i, m], table[j, m], table[k, m], table[l, m]
        if a == 0 or b == 0 or c == 0 or d == 0:
            continue
        w, x, y, z = abs(a) - 1, abs(b) - 1, abs(c) - 1, abs(d) - 1
        if ((i == w and j == x) or (i == x and j == w)) and \
                ((k == y and l == z) or (k == z and l == y)) and flip[m, p]:
            return False
    return True


def centre_ids(centres):
    """Functions whose coordinates are exactly equal share an id (the reference compares
    coordinate tuples with ==, common/symmetry.py:28)."""
    ids = {}
    return np.array([ids.setdefault(tuple(float(v) for v in c), len(ids)) for c in centres],
                    dtype=np.int32)


def parity_bits(lmn):
    lmn = np.asarray(lmn)
    return ((lmn[:, 0] % 2) | ((lmn[:, 1] % 2) << 1) | ((lmn[:, 2] % 2) << 2)).astype(np.int32)
