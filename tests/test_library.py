"""The C-ABI library builds for sm_103a, loads, and exports every entry point that
include/gaussium_gb300.h declares (no GPU calls)."""
import os
import re
import shutil

import pytest

from conftest import ROOT


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "gaussium_gb300.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|long long|const char\*)\s+(gs_\w+)\s*\(", text, re.M)))


def test_header_declares_entry_points():
    names = declared_symbols()
    for n in ("gs_pairs_build", "gs_eri_blocks", "gs_fock_jk", "gs_schwarz", "gs_boys_eval"):
        assert n in names


@pytest.mark.parametrize("lang,cc", [("c", "gcc"), ("c++", "g++")])
def test_header_compiles_as_c_and_cxx(lang, cc, tmp_path):
    """A foreign-function binding (cgo, cffi, a C host) includes the header as plain C."""
    if shutil.which(cc) is None:
        pytest.skip(f"{cc} not available")
    import subprocess
    src = tmp_path / ("use." + ("c" if lang == "c" else "cpp"))
    src.write_text('#include "gaussium_gb300.h"\nint main(void) { return gs_version() == 1 ? 0 : 1; }\n')
    r = subprocess.run([cc, "-fsyntax-only", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                        str(src)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


@pytest.mark.skipif(shutil.which("nvcc") is None, reason="nvcc not available")
def test_library_exports_every_declared_symbol():
    from gaussium_gb300 import build, _lib
    path = build.build()
    L = _lib.load_library(path)
    for name in declared_symbols():
        assert hasattr(L, name), name
    assert L.gs_version() == 1
    assert L.gs_status_string(0) == b"ok"
    from gaussium_gb300 import engine
    engine.check_record_sizes(L)              # host record layouts equal the library's
    limit = L.gs_status_string(6)
    assert b"no-allocation" in limit and b"gs_spin_expand_max_orbitals" in limit


def test_product_path_fails_loudly_without_gpu(monkeypatch):
    import torch
    from gaussium_gb300 import _lib
    monkeypatch.setattr(torch.cuda, "is_available", lambda: False)
    monkeypatch.setattr(_lib, "_LIB", None)
    with pytest.raises(_lib.GsError):
        _lib.lib()


def test_transform_fails_loudly_without_gpu(monkeypatch):
    """The AO -> MO drop-ins have no CPU path: no device (or a CPU device) is an error."""
    import numpy as np
    import torch
    from gaussium_gb300 import _lib, transform
    monkeypatch.setattr(torch.cuda, "is_available", lambda: False)
    monkeypatch.setattr(_lib, "_LIB", None)
    x = np.zeros((2, 2, 2, 2))
    for call in (lambda: transform.spin_basis_set(x),
                 lambda: transform.molecular_orbitals(x, np.eye(2)),
                 lambda: transform.spin_basis_anti_physicist(x, device="cpu")):
        with pytest.raises(_lib.GsError):
            call()


def test_new_drop_ins_refuse_cpu_tensors():
    """CPU tensors never reach a kernel: the transform, the spin expansion, the symmetry
    screen and the XC quadrature raise instead of passing host pointers or computing on
    the host."""
    import numpy as np
    import torch
    from gaussium_gb300 import _lib, dropin, kohnsham, transform
    x = torch.zeros((2, 2, 2, 2), dtype=torch.float64)
    with pytest.raises(_lib.GsError):
        transform.transform_device(x, torch.eye(2, dtype=torch.float64))
    with pytest.raises(_lib.GsError):
        transform.spin_expand_device(x, 0)
    with pytest.raises(_lib.GsError):
        dropin.symmetry_zero(x, np.zeros((2, 1), np.int32), np.zeros((1, 8), np.uint8),
                             np.zeros(2, np.int32), np.zeros(2, np.int32))
    with pytest.raises(_lib.GsError):
        kohnsham.ExchangeCorrelationGPU([], params=(2 / 3, None), device="cpu")


def test_every_entry_point_is_documented_for_integrators():
    """Each C-ABI symbol the header declares has its row in the integration guide at the
    repository root."""
    doc = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    assert [n for n in declared_symbols() if n not in doc] == []


def test_record_size_mismatch_is_refused(monkeypatch):
    """A host record layout that differs from the library's is refused, not packed."""
    from gaussium_gb300 import build, engine, _lib
    L = _lib.load_library(build.build())
    monkeypatch.setattr(engine, "PRIM64", engine.PRIM64 + 8)
    with pytest.raises(_lib.GsError):
        engine.check_record_sizes(L)
