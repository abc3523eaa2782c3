"""Drop-in replacements for the reference's ERI call surface, running on the GPU engine.

Integral objects (``.integrate(basis_i, basis_j, basis_k, basis_l) -> float``):
  GpuObaraSaika          for ObaraSaika         integrals/twoelectronrepulsion/obara_saika_scheme.py:10-82
  GpuHeadGordonPople     for HeadGordonPople    integrals/twoelectronrepulsion/head_gordon_pople.py:11-91
  GpuElectronRepulsion   for ElectronRepulsion  integrals/twoelectronrepulsion/cook_integral.py:10-99
All three evaluate the same exact integral (the schemes differ only in recursion order),
through the sm_103a class kernels.  A call packs its four functions as single-function
shells (all normalisation folded into the coefficients, read from the objects' attributes
exactly as the reference does) and returns one component of the shell block -- slow per
call, present for API and test parity.

ERI-matrix builders (``.create_repulsion_matrix() -> ndarray[N,N,N,N]``,
``.calculate_integral(i,j,k,l) -> float``):
  TwoElectronRepulsionGPU (basis_set_array, integral, symmetry, processes)
      for TwoElectronRepulsion  matrixelements/electron_repulsion_matrix.py:9-47
  TwoElectronRepulsionMatrixOSGPU / HGPGPU / CookGPU (basis_set_array, symmetry, processes)
      for the three subclasses, electron_repulsion_matrix.py:50-65
The dense tensor is computed from unique shell quartets on the device and expanded 8-fold
there; ``processes`` is accepted and ignored.  A ``symmetry`` object whose point group is
not C1 is honoured by zeroing the keys its ``none_zero_integral`` rejects, as
``calculate_integral`` does in the reference (electron_repulsion_matrix.py:19-26).
"""
import numpy as np
import torch

from . import _lib, engine
from .basis import COMPONENTS, ShellBasis, component_index


class GpuObaraSaika:
    def __init__(self, device="cuda"):
        self.device = device

    def integrate(self, basis_i, basis_j, basis_k, basis_l):
        funcs = (basis_i, basis_j, basis_k, basis_l)
        shells = [ShellBasis.single_function(f) for f in funcs]
        sb = _concat(shells)
        out, off = engine.eri_blocks(sb, np.array([[0, 1, 2, 3]]), precision=64, device=self.device)
        n = [len(COMPONENTS[int(x)]) for x in sb.l]
        idx = [component_index(f.integral_exponents) for f in funcs]
        return float(out[:off[1]].reshape(n)[tuple(idx)])


class GpuHeadGordonPople(GpuObaraSaika):
    pass


class GpuElectronRepulsion(GpuObaraSaika):
    pass


def _concat(shells):
    l = np.concatenate([s.l for s in shells])
    centre = np.concatenate([s.centre for s in shells])
    expo = np.concatenate([s.expo for s in shells])
    coef = np.concatenate([s.coef for s in shells])
    off = np.concatenate([[0], np.cumsum([len(s.expo) for s in shells])])
    scale = np.concatenate([s.comp_scale for s in shells])
    return ShellBasis(l, centre, off, expo, coef, scale)


def unique_shell_quartets(nshell):
    """(a,b,c,d) with a >= b, c >= d and pair(ab) >= pair(cd)."""
    i, j = np.tril_indices(nshell)
    pairs = np.stack([i, j], axis=1)
    pi, pj = np.tril_indices(len(pairs))
    return np.concatenate([pairs[pi], pairs[pj]], axis=1)


def dense_eri(sb: ShellBasis, device="cuda", precision=64):
    """Dense N^4 ERI tensor (torch f64 on the device) from unique shell quartets."""
    ds = engine.DeviceShells(sb, device)
    q = unique_shell_quartets(sb.nshell)
    batch = engine.QuartetBatch(ds, q, want32=precision == 32)
    n = sb.nbf
    if n ** 4 * 8 > 64 * 2 ** 30:
        raise MemoryError(f"dense ERI tensor of {n} functions does not fit")
    vals = torch.zeros(max(1, batch.total), dtype=torch.float64, device=ds.device)
    batch.run(vals, precision)
    dev = ds.device
    # the 8-fold expansion on the device (gs_dense_expand): one warp per unique block
    qt = torch.as_tensor(np.ascontiguousarray(q, dtype=np.int32)).to(dev)
    offs = torch.as_tensor(np.ascontiguousarray(batch.offsets[:-1], dtype=np.int64)).to(dev)
    t = torch.empty((n, n, n, n), dtype=torch.float64, device=dev)
    _lib.check(_lib.lib().gs_dense_expand(len(q), _lib.ptr(qt), _lib.ptr(offs), _lib.ptr(vals),
                                          _lib.ptr(ds.l), _lib.ptr(ds.func_off), n, _lib.ptr(t),
                                          _lib.stream()), "gs_dense_expand")
    return t


_PARITIES = [(p & 1, (p >> 1) & 1, (p >> 2) & 1) for p in range(8)]


def symmetry_tables(symmetry, basis_set_array):
    """Device-kernel tables of the reference's Symmetry object (common/symmetry.py:10-16):
    (table, flip, centre_id, parity) as numpy arrays, or None when the object does not
    carry the reference's ``symmetry_matrix`` / ``int_operate_dict``."""
    sm = getattr(symmetry, "symmetry_matrix", None)
    ops = getattr(symmetry, "int_operate_dict", None)
    n = len(basis_set_array)
    if not isinstance(sm, np.ndarray) or not isinstance(ops, dict) or sm.ndim != 2 \
            or sm.shape[0] != n + 1:
        return None
    nops = sm.shape[1] - 1
    table = np.array([[int(sm[f + 1, m + 1]) for m in range(nops)] for f in range(n)],
                     dtype=np.int32).reshape(n, nops)
    flip = np.array([[_PARITIES[p] != tuple(ops[(m + 1, _PARITIES[p])]) for p in range(8)]
                     for m in range(nops)], dtype=np.uint8).reshape(nops, 8)
    ids = {}
    centre = np.array([ids.setdefault(tuple(float(v) for v in b.coordinates), len(ids))
                       for b in basis_set_array], dtype=np.int32)
    lmn = np.array([b.integral_exponents for b in basis_set_array], dtype=np.int64).reshape(n, 3)
    parity = ((lmn[:, 0] % 2) | ((lmn[:, 1] % 2) << 1) | ((lmn[:, 2] % 2) << 2)).astype(np.int32)
    return table, flip, centre, parity


def symmetry_zero(tensor, table, flip, centre_id, parity):
    """Zero in place the elements of a dense device tensor that the point group makes
    vanish (``gs_symmetry_zero``)."""
    n = tensor.shape[0]
    if not tensor.is_cuda or tensor.dtype != torch.float64 or not tensor.is_contiguous() \
            or tuple(tensor.shape) != (n, n, n, n):
        raise _lib.GsError("gs_symmetry_zero takes a contiguous float64 CUDA tensor of n^4 elements")
    dev = tensor.device
    tb = torch.as_tensor(np.ascontiguousarray(table, dtype=np.int32)).to(dev)
    fl = torch.as_tensor(np.ascontiguousarray(flip, dtype=np.uint8)).to(dev)
    ci = torch.as_tensor(np.ascontiguousarray(centre_id, dtype=np.int32)).to(dev)
    pa = torch.as_tensor(np.ascontiguousarray(parity, dtype=np.int32)).to(dev)
    L = _lib.lib()
    _lib.check(L.gs_symmetry_zero(n, tb.shape[1] if tb.dim() == 2 else 0, _lib.ptr(tb), _lib.ptr(fl),
                                  _lib.ptr(ci), _lib.ptr(pa), _lib.ptr(tensor), _lib.stream()),
               "gs_symmetry_zero")
    return tensor


class TwoElectronRepulsionGPU:
    def __init__(self, basis_set_array, integral=None, symmetry=None, processes=1, device="cuda"):
        self.basis_set_array = basis_set_array
        self.matrix_size = len(basis_set_array)
        self.integral = integral
        self.symmetry = symmetry
        self.processes = processes
        self.device = device
        self._single = GpuObaraSaika(device)

    def _nonzero(self, key):
        s = self.symmetry
        if s is None:
            return True
        pg = getattr(s, "point_group", None)
        if pg is not None and getattr(pg, "label", None) == "C_{1}":
            return True
        return bool(s.none_zero_integral(key))

    def calculate_integral(self, i, j, k, l):
        if self._nonzero((i, j, k, l)):
            b = self.basis_set_array
            return self._single.integrate(b[i], b[j], b[k], b[l])
        return 0.0

    def create_repulsion_matrix(self, as_tensor=False):
        sb = ShellBasis.from_functions(self.basis_set_array)
        t = dense_eri(sb, self.device)
        s = self.symmetry
        pg = getattr(s, "point_group", None) if s is not None else None
        if s is not None and not (pg is not None and getattr(pg, "label", None) == "C_{1}"):
            tables = symmetry_tables(s, self.basis_set_array)
            if tables is not None:
                symmetry_zero(t, *tables)
                return t if as_tensor else t.cpu().numpy()
            # a symmetry object without the reference's tables (e.g. a test double):
            # ask it key by key, as the reference does
            n = self.matrix_size
            mask = torch.ones((n, n, n, n), dtype=torch.bool)
            for a in range(n):
                for b in range(a, n):
                    for c in range(a, n):
                        for d in range(c, n):
                            if (a == c and b > d):
                                continue
                            if not s.none_zero_integral((a, b, c, d)):
                                for key in ((a, b, c, d), (b, a, c, d), (a, b, d, c), (b, a, d, c),
                                            (c, d, a, b), (d, c, a, b), (c, d, b, a), (d, c, b, a)):
                                    mask[key] = False
            t = t * mask.to(t.device)
        return t if as_tensor else t.cpu().numpy()


class TwoElectronRepulsionMatrixOSGPU(TwoElectronRepulsionGPU):
    def __init__(self, basis_set_array, symmetry_matrix, processes, device="cuda"):
        super().__init__(basis_set_array, GpuObaraSaika(device), symmetry_matrix, processes, device)


class TwoElectronRepulsionMatrixHGPGPU(TwoElectronRepulsionGPU):
    def __init__(self, basis_set_array, symmetry_matrix, processes, device="cuda"):
        super().__init__(basis_set_array, GpuHeadGordonPople(device), symmetry_matrix, processes,
                         device)


class TwoElectronRepulsionMatrixCookGPU(TwoElectronRepulsionGPU):
    def __init__(self, basis_set_array, symmetry_matrix, processes, device="cuda"):
        super().__init__(basis_set_array, GpuElectronRepulsion(device), symmetry_matrix, processes,
                         device)
