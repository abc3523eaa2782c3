"""Basis-set data model and the shell packer.

The reference describes a basis as a list of contracted Cartesian *functions*
(``objects/basis_function.py:6-71``), each with its own primitives
(``objects/primitive_basis_function.py:6-61``) and its own normalisation.  The engine works
on *shells*: all Cartesian components of one angular momentum on one centre sharing one
primitive set.  ``ShellBasis.from_functions`` regroups reference-ordered functions into
shells (s; x,y,z; xx,yy,zz,xy,xz,yz as ``factory/primitive_basis_factory.py:5-86`` emits
them) and folds every normalisation into

    coef[k]        = contraction_k * primitive_norm_k(first component) * Basis.normalisation(first)
    comp_scale[i]  = (primitive_norm_k(comp i) * Basis.normalisation(comp i)) /
                     (primitive_norm_k(first) * Basis.normalisation(first))

which must not depend on k (it holds for the reference's own normalisation formulas; the
packer checks it).  Only attributes are read -- ``primitive_gaussian_array``,
``coordinates``, ``integral_exponents``, ``normalisation``; per primitive ``contraction``,
``exponent``, ``normalisation`` -- so duck-typed objects work as they do in the
reference's tests.
"""
import itertools
import math
import re

import numpy as np

COMPONENTS = {0: [(0, 0, 0)],
              1: [(1, 0, 0), (0, 1, 0), (0, 0, 1)],
              2: [(2, 0, 0), (0, 2, 0), (0, 0, 2), (1, 1, 0), (1, 0, 1), (0, 1, 1)]}
LMAX = 2


def _fact2(n):
    r = 1.0
    while n > 1:
        r *= n
        n -= 2
    return r


class PrimitiveBasis:
    """Primitive Cartesian Gaussian with the reference's normalisation
    (objects/primitive_basis_function.py:26-42; double factorial of n <= 0 is 1)."""

    def __init__(self, contraction, exponent, coordinates, integral_exponents):
        self.contraction = contraction
        self.exponent = exponent
        self.coordinates = coordinates
        self.integral_exponents = integral_exponents
        self._norm = None

    @property
    def normalisation(self):
        if self._norm is None:
            l, m, n = self.integral_exponents
            out1 = _fact2(2 * l - 1) * _fact2(2 * m - 1) * _fact2(2 * n - 1)
            out2 = (math.pi / (2 * self.exponent)) ** 1.5
            out3 = (4 * self.exponent) ** (l + m + n)
            self._norm = 1.0 / math.sqrt(out1 * out2 / out3)
        return self._norm


class Basis:
    """Contracted Cartesian function with the reference's normalisation
    (objects/basis_function.py:22-53: 1 for a single primitive)."""

    def __init__(self, primitive_gaussian_array, coordinates, integral_exponents):
        self.primitive_gaussian_array = primitive_gaussian_array
        self.coordinates = coordinates
        self.integral_exponents = integral_exponents
        self._norm = None

    @property
    def normalisation(self):
        if self._norm is None:
            prims = self.primitive_gaussian_array
            if len(prims) == 1:
                self._norm = 1
            else:
                l, m, n = self.integral_exponents
                out1 = _fact2(2 * l - 1) * _fact2(2 * m - 1) * _fact2(2 * n - 1)
                ans = 0.0
                for pa, pb in itertools.product(prims, repeat=2):
                    s = pa.exponent + pb.exponent
                    ans += (pa.contraction * pb.contraction * pa.normalisation * pb.normalisation
                            * out1 * (math.pi / s) ** 1.5) / (2 * s) ** (l + m + n)
                self._norm = 1.0 / math.sqrt(ans)
        return self._norm


class Nuclei:
    def __init__(self, element, charge, mass, coordinates):
        self.element = element
        self.charge = charge
        self.mass = mass
        self.coordinates = coordinates


def expand_shell(kind, rows, coordinates):
    """S/L/P/D shell of a GAMESS-UK basis file -> Basis objects, in the reference order."""
    out = []

    def block(lmn_list, coef_col):
        for lmn in lmn_list:
            prims = [PrimitiveBasis(r[coef_col], r[1], coordinates, lmn) for r in rows]
            out.append(Basis(prims, coordinates, lmn))

    if kind == "S":
        block(COMPONENTS[0], 0)
    elif kind == "L":
        block(COMPONENTS[0], 0)
        block(COMPONENTS[1], 2)
    elif kind == "P":
        block(COMPONENTS[1], 0)
    elif kind == "D":
        block(COMPONENTS[2], 0)
    else:
        raise ValueError(f"unsupported shell type {kind!r}")
    return out


def read_basis_set_file(path, nuclei_array):
    """GAMESS-UK basis file -> functions for each nucleus in order (the format
    common/file_input.py:6-56 reads: an element-name header line, then shell lines
    'S|L|P|D  X' followed by 'coef exponent [coef_p]' rows)."""
    with open(path) as f:
        text = f.read()
    blocks = {}
    current = None
    for raw in text.splitlines():
        line = raw.strip()
        if not line:
            continue
        if line.startswith("#"):
            name = line[1:].strip().split()
            if name and name[0].isalpha():
                current = name[0].upper()
                blocks.setdefault(current, [])
            continue
        if current is None:
            continue
        parts = line.split()
        if parts[0] in ("S", "L", "P", "D", "F", "SP") and (len(parts) == 1 or not _isnum(parts[0])):
            blocks[current].append([parts[0], []])
        elif _isnum(parts[0]) and blocks[current]:
            blocks[current][-1][1].append([float(x) for x in parts])
    out = []
    for nuc in nuclei_array:
        key = nuc.element.upper()
        if key not in blocks:
            raise KeyError(f"element {nuc.element} not in {path}")
        for kind, rows in blocks[key]:
            out.extend(expand_shell(kind, rows, tuple(nuc.coordinates)))
    return out


def _isnum(s):
    return re.match(r"^[-+]?(\d+\.?\d*|\.\d+)([eEdD][-+]?\d+)?$", s) is not None


def read_mol_file(path):
    """'charge multiplicity' then 'ELEMENT Z mass x y z' (bohr) -- common/file_input.py:59-88."""
    with open(path) as f:
        lines = [l for l in f.read().splitlines() if l.strip()]
    charge, mult = (int(x) for x in lines[0].split()[:2])
    nuclei, total = [], 0
    for line in lines[1:]:
        a = line.split()
        total += int(a[1])
        nuclei.append(Nuclei(a[0], float(a[1]), float(a[2]), (float(a[3]), float(a[4]), float(a[5]))))
    return nuclei, total - charge, mult


class ShellBasis:
    """Shells in the reference's function order (host numpy arrays).

    l[s], centre[s] (bohr), func_off[s] (first function index), prim_off[s..s+1],
    expo[k], coef[k] (effective, see module docstring), comp_scale[s, i].
    """

    def __init__(self, l, centre, prim_off, expo, coef, comp_scale):
        self.l = np.ascontiguousarray(l, dtype=np.int32)
        self.centre = np.ascontiguousarray(centre, dtype=np.float64).reshape(-1, 3)
        self.prim_off = np.ascontiguousarray(prim_off, dtype=np.int32)
        self.expo = np.ascontiguousarray(expo, dtype=np.float64)
        self.coef = np.ascontiguousarray(coef, dtype=np.float64)
        cs = np.ones((len(self.l), 6))
        cs[:, :] = np.asarray(comp_scale, dtype=np.float64).reshape(len(self.l), -1)[:, :6] \
            if np.asarray(comp_scale).size == 6 * len(self.l) else 1.0
        self.comp_scale = np.ascontiguousarray(cs)
        self._validate()
        nfun = np.array([1, 3, 6], dtype=np.int32)[self.l]
        self.nfunc = nfun
        self.func_off = np.concatenate([[0], np.cumsum(nfun)[:-1]]).astype(np.int32)
        self.nbf = int(nfun.sum())
        self.nprim = np.diff(self.prim_off).astype(np.int32)

    def _validate(self):
        """Reject shell data a kernel would turn into garbage or out-of-range reads, before
        anything reaches the device."""
        ns = len(self.l)
        if int(self.l.max(initial=0)) > LMAX or int(self.l.min(initial=0)) < 0:
            raise ValueError(f"angular momentum outside 0..{LMAX}")
        if self.centre.shape != (ns, 3) or not np.all(np.isfinite(self.centre)):
            raise ValueError("shell centres must be finite, one (x, y, z) per shell")
        po = self.prim_off
        if len(po) != ns + 1 or (ns and po[0] != 0) or np.any(np.diff(po) < 1) or \
                po[-1] != len(self.expo) or len(self.coef) != len(self.expo):
            raise ValueError("prim_off must start at 0, increase by at least one primitive per "
                             "shell and end at the number of exponents (= coefficients)")
        if not np.all(np.isfinite(self.expo)) or np.any(self.expo <= 0):
            raise ValueError("primitive exponents must be finite and positive")
        if not np.all(np.isfinite(self.coef)) or not np.all(np.isfinite(self.comp_scale)):
            raise ValueError("contraction coefficients and component scales must be finite")

    @property
    def nshell(self):
        return len(self.l)

    # ---------------------------------------------------------------- constructors
    @classmethod
    def from_shell_dicts(cls, shells):
        """Shells given as dict(l, centre, expo, coef) with raw contraction coefficients,
        normalised by the reference's conventions."""
        funcs = []
        for sh in shells:
            c = tuple(float(x) for x in sh["centre"])
            for lmn in COMPONENTS[int(sh["l"])]:
                prims = [PrimitiveBasis(float(cf), float(ex), c, lmn)
                         for cf, ex in zip(sh["coef"], sh["expo"])]
                funcs.append(Basis(prims, c, lmn))
        return cls.from_functions(funcs)

    @classmethod
    def from_functions(cls, funcs):
        """Group reference-ordered functions (duck-typed Basis objects) into shells."""
        ls, centres, offs, expo, coef, scales = [], [], [0], [], [], []
        i = 0
        n = len(funcs)
        while i < n:
            f0 = funcs[i]
            lmn0 = tuple(int(x) for x in f0.integral_exponents)
            L = sum(lmn0)
            if L > LMAX:
                raise ValueError(f"function {i}: angular momentum {L} above {LMAX}")
            comps = COMPONENTS[L]
            if lmn0 != comps[0]:
                raise ValueError(f"function {i}: components of an l={L} shell must start with "
                                 f"{comps[0]} (reference order), got {lmn0}")
            group = funcs[i:i + len(comps)]
            if len(group) != len(comps):
                raise ValueError(f"function {i}: incomplete l={L} shell")
            p0 = f0.primitive_gaussian_array
            ex0 = [float(p.exponent) for p in p0]
            r0 = tuple(float(x) for x in f0.coordinates)
            d = np.zeros((len(comps), len(p0)))
            for ci, (f, lmn) in enumerate(zip(group, comps)):
                if tuple(int(x) for x in f.integral_exponents) != lmn:
                    raise ValueError(f"function {i + ci}: expected component {lmn}")
                if tuple(float(x) for x in f.coordinates) != r0:
                    raise ValueError(f"function {i + ci}: centre differs within the shell")
                prims = f.primitive_gaussian_array
                if [float(p.exponent) for p in prims] != ex0:
                    raise ValueError(f"function {i + ci}: exponents differ within the shell")
                norm = float(f.normalisation)
                for k, p in enumerate(prims):
                    d[ci, k] = float(p.contraction) * float(p.normalisation) * norm
            u = d[0]
            scale = np.ones(6)
            for ci in range(1, len(comps)):
                nz = np.abs(u) > 0
                if not nz.any():
                    continue
                ratios = d[ci, nz] / u[nz]
                if np.max(np.abs(ratios - ratios[0])) > 1e-12 * abs(ratios[0]) + 1e-300:
                    raise ValueError(f"function {i + ci}: normalisation is not a per-component "
                                     "factor times a per-primitive one")
                scale[ci] = ratios[0]
            ls.append(L)
            centres.append(r0)
            expo.extend(ex0)
            coef.extend(u.tolist())
            offs.append(len(expo))
            scales.append(scale)
            i += len(comps)
        return cls(ls, centres, offs, expo, coef, np.array(scales))

    @classmethod
    def single_function(cls, f):
        """One contracted function as its own shell (for the per-function integral API):
        the shell has l = l+m+n with all normalisation folded into the coefficients, and
        the caller picks component ``component_index(f)`` of the block."""
        lmn = tuple(int(x) for x in f.integral_exponents)
        L = sum(lmn)
        if L > LMAX:
            raise ValueError(f"angular momentum {L} above {LMAX}")
        prims = f.primitive_gaussian_array
        norm = float(f.normalisation)
        coef = [float(p.contraction) * float(p.normalisation) * norm for p in prims]
        expo = [float(p.exponent) for p in prims]
        return cls([L], [tuple(float(x) for x in f.coordinates)], [0, len(expo)], expo, coef,
                   np.ones((1, 6)))


def component_index(lmn):
    lmn = tuple(int(x) for x in lmn)
    return COMPONENTS[sum(lmn)].index(lmn)
