"""The no-allocation mixed J/K entry point (gs_fock_jk_mixed_noalloc), for callers that
cannot allocate device memory, called through the C ABI and compared with the
workspace-taking entry point (gs_fock_jk_mixed) on the same inputs, twice in a row (the
fixed scratch array keeps the previous call's contents, which must not leak into the next
result)."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _setup():
    from gaussium_gb300.engine import JKEngine
    from gaussium_gb300.basis import ShellBasis
    from molecules import load, random_density
    g, funcs, table = load("h2o_631gs")
    eng = JKEngine(ShellBasis.from_functions(funcs), schwarz_thr=1e-14)
    return eng, random_density(eng.sb.nbf, 21) * 0.3


def _run(eng, L, p, noalloc, mixed_cut=1e-3):
    from gaussium_gb300 import _lib
    n = eng.sb.nbf
    pt = torch.tensor(p, device="cuda").contiguous()
    pk = pt.unsqueeze(0).contiguous()
    dmax = eng.shell_dmax([pt])
    J = torch.zeros((n, n), dtype=torch.float64, device="cuda")
    K = torch.zeros((1, n, n), dtype=torch.float64, device="cuda")
    base = eng.tasks.data_ptr()
    ws = None
    for cls, s, e in eng.segments:
        common = (*cls, _lib.ptr(eng.pairs.rec), _lib.ptr(eng.pairs.p64), _lib.ptr(eng.pairs.p32),
                  _lib.ptr(eng.ds.comp_scale), _lib.ptr(eng.ds.func_off), eng.sb.nshell, n, e - s,
                  base + s * 8, _lib.ptr(pt), _lib.ptr(J), 1, _lib.ptr(pk), _lib.ptr(K),
                  _lib.ptr(dmax), 1e-13, mixed_cut)
        if noalloc:
            rc = L.gs_fock_jk_mixed_noalloc(*common, _lib.stream())
        else:
            need = L.gs_fock_jk_mixed_workspace(e - s)
            ws = torch.empty(int(need), dtype=torch.uint8, device="cuda")
            rc = L.gs_fock_jk_mixed(*common, _lib.ptr(ws), ws.numel(), _lib.stream())
        assert rc == 0, L.gs_status_string(rc)
    torch.cuda.synchronize()
    return (J + J.T).cpu().numpy(), (K[0] + K[0].T).cpu().numpy()


def test_noalloc_matches_workspace_entry_twice(gpu_lib):
    eng, p = _setup()
    assert gpu_lib.gs_fock_jk_mixed_noalloc_max_tasks() == 1 << 20
    assert max(e - s for _, s, e in eng.segments) <= gpu_lib.gs_fock_jk_mixed_noalloc_max_tasks()
    j_ref, k_ref = _run(eng, gpu_lib, p, noalloc=False)
    for _ in range(2):
        j, k = _run(eng, gpu_lib, p, noalloc=True)
        assert np.max(np.abs(j - j_ref)) < 1e-12
        assert np.max(np.abs(k - k_ref)) < 1e-12


def test_noalloc_rejects_oversized_task_counts(gpu_lib):
    from gaussium_gb300 import _lib
    eng, p = _setup()
    too_many = gpu_lib.gs_fock_jk_mixed_noalloc_max_tasks() + 1
    cls, s, e = eng.segments[0]
    rc = gpu_lib.gs_fock_jk_mixed_noalloc(*cls, _lib.ptr(eng.pairs.rec), _lib.ptr(eng.pairs.p64),
                                          _lib.ptr(eng.pairs.p32), _lib.ptr(eng.ds.comp_scale),
                                          _lib.ptr(eng.ds.func_off), eng.sb.nshell, eng.sb.nbf,
                                          too_many, eng.tasks.data_ptr(), None, None, 0, None,
                                          None, None, 1e-13, 1e-3, _lib.stream())
    assert rc == 6
    assert b"no-allocation" in gpu_lib.gs_status_string(rc)
