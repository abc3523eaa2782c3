"""ctypes binding of ``libgaussium_gb300.so`` (the C ABI in include/gaussium_gb300.h).

The library is the only compute path: there is no CPU fallback.  ``lib()`` raises when
no CUDA device is visible or the library has not been built.
"""
import ctypes
import os

from . import build as _build

_LIB = None

P = ctypes.c_void_p
I = ctypes.c_int
D = ctypes.c_double

_SIGS = {
    "gs_version": (I, []),
    "gs_status_string": (ctypes.c_char_p, [I]),
    "gs_record_sizes": (I, [P]),
    "gs_class_available": (I, [I, I, I, I]),
    "gs_pairs_build": (I, [P, P, P, P, P, I, P, P, P, P, P, D, P, I, P, P]),
    "gs_schwarz": (I, [I, I, P, P, P, I, P, P, I, P]),
    "gs_eri_blocks": (I, [I, I, I, I, I, P, P, P, I, P, P, P]),
    "gs_fock_jk": (I, [I, I, I, I, I, P, P, P, P, I, I, I, P, P, P, I, P, P, P, D, D, D, P]),
    "gs_fock_jk_batched": (I, [I, I, I, I, I, P, P, P, P, P, P, P, P, ctypes.c_longlong, I, P,
                               P, P, I, P, P, D, D, D, P]),
    "gs_fock_jk_batched_mixed": (I, [I, I, I, I, P, P, P, P, P, P, P, P, P, P, P, P,
                                     ctypes.c_longlong, I, P, P, P, I, P, P, D, D, P,
                                     ctypes.c_longlong, P]),
    "gs_fock_jk_mixed_workspace": (ctypes.c_longlong, [I]),
    "gs_fock_jk_persistent_workspace": (ctypes.c_longlong, [I]),
    "gs_fock_jk_batched_persistent": (I, [P, P, P, P, P, P, P, P, P, P, P, P, ctypes.c_longlong,
                                          P, I, P, P, P, I, P, P, D, D, P, ctypes.c_longlong, P]),
    "gs_fock_jk_mixed": (I, [I, I, I, I, P, P, P, P, P, I, I, I, P, P, P, I, P, P, P, D, D, P,
                             ctypes.c_longlong, P]),
    "gs_fock_jk_mixed_noalloc": (I, [I, I, I, I, P, P, P, P, P, I, I, I, P, P, P, I, P, P, P, D,
                                     D, P]),
    "gs_fock_jk_mixed_noalloc_max_tasks": (I, []),
    "gs_class_variants": (I, [I, I, I, I, I]),
    "gs_class_form": (I, [I, I, I, I, I]),
    "gs_set_class_variant": (I, [I, I, I, I, I, I]),
    "gs_boys_eval": (I, [I, I, I, P, P, P]),
    "gs_fma_probe": (I, [I, I, I, I, P, P]),
    "gs_fma_probe_lanes": (I, [I, I, I, I, I, P, P]),
    "gs_one_electron": (I, [P, P, P, P, P, P, P, I, P, I, I, P, P, P, P, P, P]),
    "gs_eri_grad_contract": (I, [I, P, P, P, P, P, P, P, I, P, P, P]),
    "gs_eri_grad": (I, [I, I, I, I, P, P, P, P, P, I, P, I, I, P, P, P]),
    "gs_eri_grad_form": (I, [I, I, I, I, I, P, P, P, P, P, I, P, I, I, P, P, P]),
    "gs_eri_grad_band": (I, [I, I, I, I, I, I, P, P, P, P, P, I, P, I, I, P, I, P, D, D, D, P, P]),
    "gs_eri_grad_class_form": (I, [I, I, I, I]),
    "gs_eri_grad_variants": (I, [I, I, I, I]),
    "gs_set_eri_grad_variant": (I, [I, I, I, I, I]),
    "gs_one_electron_grad": (I, [P, P, P, P, P, P, P, P, I, P, I, I, P, P, P, P, P, P]),
    "gs_spin_expand": (I, [P, I, I, P, P]),
    "gs_spin_expand_max_orbitals": (I, []),
    "gs_basis_on_grid": (I, [P, P, P, P, P, P, P, I, I, ctypes.c_longlong, P, P, P]),
    "gs_lda_xc": (I, [ctypes.c_longlong, P, P, D, I, D, D, D, D, P, P, P]),
    "gs_symmetry_zero": (I, [I, I, P, P, P, P, P, P]),
    "gs_dense_expand": (I, [ctypes.c_longlong, P, P, P, P, P, I, P, P]),
}


class GsError(RuntimeError):
    pass


def _bind(L):
    for name, (res, args) in _SIGS.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    return L


def load_library(path=None):
    """Load and bind the shared library without touching the GPU."""
    return _bind(ctypes.CDLL(path or _build.LIB))


def lib():
    global _LIB
    if _LIB is None:
        import torch
        if not torch.cuda.is_available():
            raise GsError("gaussium_gb300 runs on a CUDA GPU only; no device is visible "
                          "(there is no CPU fallback)")
        if not os.path.exists(_build.LIB):
            raise GsError(f"CUDA library {_build.LIB} is missing: run gaussium_gb300.build.build()")
        _LIB = load_library()
    return _LIB


def check(rc, what):
    if rc != 0:
        msg = lib().gs_status_string(rc).decode()
        raise GsError(f"{what} failed: {msg} (status {rc})")


def ptr(t):
    """Device (or host) address of a tensor, or None."""
    if t is None:
        return None
    return ctypes.c_void_p(t.data_ptr())


def stream(s=None):
    import torch
    s = s or torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)
