"""Core Hamiltonian pieces on the device: S, T, V through the one-electron kernel."""
import numpy as np
import torch

from . import _lib
from .engine import DeviceShells


def one_electron(sb, coords, charges, device="cuda"):
    """Overlap, kinetic and nuclear-attraction matrices (host numpy, FP64) of a ShellBasis
    for point charges ``charges`` at ``coords`` (bohr)."""
    ds = sb if isinstance(sb, DeviceShells) else DeviceShells(sb, device)
    h = ds.host
    i, j = np.tril_indices(h.nshell)
    pairs = torch.as_tensor(np.stack([i, j], 1).astype(np.int32)).to(ds.device)
    n = h.nbf
    S = torch.zeros((n, n), dtype=torch.float64, device=ds.device)
    T = torch.zeros_like(S)
    V = torch.zeros_like(S)
    xyz = torch.as_tensor(np.ascontiguousarray(coords, dtype=np.float64)).to(ds.device)
    z = torch.as_tensor(np.ascontiguousarray(charges, dtype=np.float64)).to(ds.device)
    L = _lib.lib()
    _lib.check(L.gs_one_electron(_lib.ptr(ds.centre), _lib.ptr(ds.l), _lib.ptr(ds.prim_off),
                                 _lib.ptr(ds.expo), _lib.ptr(ds.coef), _lib.ptr(ds.comp_scale),
                                 _lib.ptr(ds.func_off), len(i), _lib.ptr(pairs), n, len(charges),
                                 _lib.ptr(xyz), _lib.ptr(z), _lib.ptr(S), _lib.ptr(T), _lib.ptr(V),
                                 _lib.stream()), "gs_one_electron")
    return S.cpu().numpy(), T.cpu().numpy(), V.cpu().numpy()
