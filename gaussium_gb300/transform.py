"""AO -> MO transformation of the two-electron integrals on the GPU, with the reference's
call surface (matrixelements/transformations.py):

  molecular_orbitals(repulsion, coefficients)   transformations.py:5-26
  blocked_spin_basis_set(repulsion)             transformations.py:29-70
  spin_basis_set(repulsion)                     transformations.py:73-92
  spin_basis_anti_physicist(repulsion)          transformations.py:114-136

The reference transforms with 2 N^2 small matrix products in Python loops and expands to
spin orbitals element by element.  Here the four-index transform is FP64 GEMMs over the
whole tensor (cuBLAS through torch.matmul, the only library call on this path).  A tensor
with the pair symmetries of real integrals ((ab|cd) = (ba|cd) = (ab|dc), checked exactly)
is transformed over its unique pairs only: C^T X C for every pair a >= b, then the same
over (a, b) for every pair r >= s, about 4 N^5 flops.  Any other tensor takes four quarter
transforms with no transposition copies (8 N^5 flops).  The spin-orbital expansions are
the library's ``gs_spin_expand`` kernel (one pass, every output element written once).

``molecular_orbitals`` overwrites its input array with the MO integrals and returns it,
as the reference does (the reference's callers keep using the argument); the others
return new arrays.  The ``*_device`` forms take and return device tensors, for callers
that keep the tensors resident.
"""
import numpy as np
import torch

from . import _lib

SPIN_INTERLEAVED, SPIN_BLOCKED, SPIN_ANTI_PHYSICIST = 0, 1, 2


def _dev(x, device):
    if device != "cuda" and not str(device).startswith("cuda"):
        raise _lib.GsError("the AO -> MO transform runs on a CUDA device only")
    _lib.lib()   # raises without a GPU or without the built library
    return torch.as_tensor(np.asarray(x), dtype=torch.float64).to(device).contiguous()


def _pair_index(n, device):
    """Unique pairs i >= j of n indices and the n x n map of every (i, j) to its pair."""
    i, j = torch.tril_indices(n, n, device=device)
    full = torch.empty((n, n), dtype=torch.long, device=device)
    k = torch.arange(i.numel(), device=device)
    full[i, j] = k
    full[j, i] = k
    return i * n + j, full.reshape(-1)


def transform_general(ao, c):
    """Four quarter transforms, each one GEMM over the whole tensor: 8 N^4 M flops."""
    n, m = c.shape
    ct = c.transpose(0, 1).contiguous()
    x = ao.reshape(n * n * n, n) @ c                                  # [a b c s]
    x = ct @ x.reshape(n, n * n * m)                                  # [p b c s]
    x = torch.matmul(ct, x.reshape(m, n, n * m))                      # [p q c s]
    x = torch.matmul(ct, x.reshape(m * m, n, m))                      # [p q r s]
    return x.reshape(m, m, m, m)


def transform_pair_symmetric(ao, c):
    """The same transform for a tensor with (ab|cd) = (ba|cd) = (ab|dc), as every real
    two-electron tensor has: the (c, d) half runs only over the pairs a >= b, and the
    (a, b) half only over the pairs r >= s, so the GEMMs do about 4 N^5 flops; the result
    is mirrored from one triangle of (r, s).  Each half is two large GEMMs: the (c, d)
    half transforms d, then c on the transposed intermediate, whose (r, s) symmetry makes
    transposing back unnecessary."""
    n, m = c.shape
    ct = c.transpose(0, 1).contiguous()
    ab, ab_full = _pair_index(n, ao.device)
    rs, rs_full = _pair_index(m, ao.device)
    x = ao.reshape(n * n, n, n)[ab]                                   # [ab c d], a >= b
    y = x.reshape(-1, n) @ c                                          # [ab c s]
    y = y.reshape(-1, n, m).transpose(1, 2).reshape(-1, n) @ c        # [ab s r] = [ab r s]
    w = y.reshape(-1, m * m)[:, rs]                                   # [ab rs], one triangle
    z = w[ab_full]                                                    # [a b rs]
    z = ct @ z.reshape(n, -1)                                         # [p b rs]
    z = torch.matmul(ct, z.reshape(m, n, -1))                         # [p q rs]
    return z[:, :, rs_full].reshape(m, m, m, m)


def transform_device(ao, c):
    """(pq|rs) = sum_abcd C_ap C_bq C_cr C_ds (ab|cd) for a device tensor ``ao`` (N^4,
    float64, row-major) and coefficients ``c`` (N x M, columns = orbitals).  A tensor that
    is exactly symmetric in a <-> b and c <-> d takes the pair-packed form; any other
    tensor the general one."""
    n, m = c.shape
    if ao.shape != (n, n, n, n):
        raise ValueError(f"repulsion tensor {tuple(ao.shape)} does not match {n} basis functions")
    if not (ao.is_cuda and c.is_cuda):
        raise _lib.GsError("the AO -> MO transform runs on CUDA tensors only")
    ao = ao.contiguous()
    if torch.equal(ao, ao.transpose(0, 1)) and torch.equal(ao, ao.transpose(2, 3)):
        return transform_pair_symmetric(ao, c)
    return transform_general(ao, c)


def spin_expand_device(mo, mode):
    """(2h)^4 spin-orbital tensor from an h^4 MO tensor on the device (``gs_spin_expand``)."""
    if mo.dim() != 4 or len(set(mo.shape)) != 1:
        raise ValueError(f"expected an h^4 tensor, got {tuple(mo.shape)}")
    if not mo.is_cuda:
        raise _lib.GsError("gs_spin_expand takes a CUDA tensor")
    mo = mo.to(torch.float64).contiguous()
    h = mo.shape[0]
    out = torch.empty((2 * h,) * 4, dtype=torch.float64, device=mo.device)
    L = _lib.lib()
    _lib.check(L.gs_spin_expand(_lib.ptr(mo), h, mode, _lib.ptr(out), _lib.stream()),
               "gs_spin_expand")
    return out


def max_spatial_orbitals():
    return _lib.lib().gs_spin_expand_max_orbitals()


def _to_host(t):
    """A device tensor as a new numpy array, copied into page-locked memory (torch's
    pinned-host cache reuses the block once the array is freed), which the copy engine
    fills at full link speed instead of staging through pageable pages."""
    out = torch.empty(t.shape, dtype=t.dtype, pin_memory=True)
    out.copy_(t)
    return out.numpy()


def molecular_orbitals(repulsion, coefficients, device="cuda"):
    c = _dev(coefficients, device)
    mo = transform_device(_dev(repulsion, device), c)
    if isinstance(repulsion, np.ndarray) and repulsion.shape == tuple(mo.shape) \
            and repulsion.dtype == np.float64 and repulsion.flags.writeable \
            and repulsion.flags.c_contiguous:
        torch.from_numpy(repulsion).copy_(mo)       # straight into the caller's array
        return repulsion
    out = _to_host(mo)
    if isinstance(repulsion, np.ndarray) and repulsion.shape == out.shape \
            and repulsion.dtype == np.float64 and repulsion.flags.writeable:
        repulsion[...] = out
        return repulsion
    return out


def spin_basis_set(repulsion, device="cuda"):
    return _to_host(spin_expand_device(_dev(repulsion, device), SPIN_INTERLEAVED))


def blocked_spin_basis_set(repulsion, device="cuda"):
    return _to_host(spin_expand_device(_dev(repulsion, device), SPIN_BLOCKED))


def spin_basis_anti_physicist(repulsion, device="cuda"):
    return _to_host(spin_expand_device(_dev(repulsion, device), SPIN_ANTI_PHYSICIST))


def mo_integrals(sb, coefficients, device="cuda"):
    """MO-basis (pq|rs) of a ShellBasis as a device tensor: the dense AO tensor is built by
    the integral engine and transformed without leaving the device."""
    from .dropin import dense_eri
    return transform_device(dense_eri(sb, device=device), _dev(coefficients, device))
