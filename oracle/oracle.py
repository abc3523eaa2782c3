"""ORACLE — test infrastructure only.

ctypes front end of ``eri_oracle.c`` (the CPU restatement of the reference's
Obara-Saika ERI and Boys function) plus numpy restatements of the reference's Fock
builders and SCF loop.  Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU legs of
``bench.py`` import this module, always as the checker and never as the measured path.

Restated reference functions (file:line within the reference project):
  FockMatrixRestricted.create            hartreefock/fock_matrix.py:12-22
  FockMatrixUnrestricted.create          hartreefock/fock_matrix.py:32-53
  BlockedFockMatrixUnrestricted.create   hartreefock/fock_matrix.py:63-81
  RestrictedKohnShamHamiltonian J part   kohnsham/kohn_sham_hamiltonian.py:15-19
  TwoElectronRepulsion.create_repulsion_matrix  matrixelements/electron_repulsion_matrix.py:28-47
  Symmetry.sort_index                    common/symmetry.py:186-197
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
