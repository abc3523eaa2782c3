"""Host-side failure injection: malformed shell data, out-of-range shell indices and a
singular overlap are rejected on the host, with ValueError, before anything reaches a
kernel (the kernels trust their inputs).  No GPU is needed: every check runs before the
first device allocation.  The reference's own failure handling on this path is Python
exceptions (e.g. the DIIS fallback on a singular B matrix, diismethod/diis.py:105-112)."""
import types

import numpy as np
import pytest
import torch

from gaussium_gb300 import engine, scf
from gaussium_gb300.basis import ShellBasis


def _shells():
    # an s shell (2 primitives) and a p shell (1 primitive)
    return dict(l=[0, 1], centre=[[0, 0, 0], [0, 0, 1.4]], prim_off=[0, 2, 3],
                expo=[3.4, 0.6, 0.8], coef=[0.4, 0.6, 1.0], comp_scale=np.ones((2, 6)))


def test_valid_shells_accepted():
    sb = ShellBasis(**_shells())
    assert sb.nshell == 2 and sb.nbf == 4


@pytest.mark.parametrize("field,value", [
    ("expo", [3.4, np.nan, 0.8]),
    ("expo", [3.4, -0.6, 0.8]),
    ("expo", [3.4, 0.0, 0.8]),
    ("coef", [0.4, np.inf, 1.0]),
    ("centre", [[0, 0, np.nan], [0, 0, 1.4]]),
    ("prim_off", [0, 2, 2]),          # a shell without primitives
    ("prim_off", [0, 3, 2]),          # not monotone
    ("prim_off", [1, 2, 3]),          # does not start at 0
    ("prim_off", [0, 2, 4]),          # past the last exponent
    ("l", [0, 3]),                    # above the built classes
    ("l", [-1, 1]),
])
def test_malformed_shells_rejected(field, value):
    kw = _shells()
    kw[field] = value
    with pytest.raises(ValueError):
        ShellBasis(**kw)


def _host_only(sb):
    # stands in for DeviceShells: the checks run before any device buffer is touched
    return types.SimpleNamespace(host=sb, device=torch.device("cpu"))


@pytest.mark.parametrize("q", [[[0, 1, 0, 2]], [[0, 1, -1, 0]], [[5, 0, 0, 0]]])
def test_out_of_range_shell_indices_rejected(q):
    sb = ShellBasis(**_shells())
    with pytest.raises(ValueError):
        engine.QuartetBatch(_host_only(sb), np.array(q))
    with pytest.raises(ValueError):
        engine.PairSet(_host_only(sb), np.array(q)[:, :2])


def test_singular_overlap_rejected():
    s = np.array([[1.0, 1.0], [1.0, 1.0]])           # two identical functions
    with pytest.raises(ValueError):
        scf.LinearAlgebra(s)
    with pytest.raises(ValueError):
        scf.LinearAlgebra(np.array([[1.0, np.nan], [np.nan, 1.0]]))


def test_diis_falls_back_on_singular_b_matrix():
    """The reference's only recovery on this path: a singular DIIS B matrix drops the
    oldest vector and retries (diismethod/diis.py:105-112)."""
    la = scf.LinearAlgebra(np.eye(2))
    d = scf.DIIS(np.eye(2), la)
    e = np.array([[0.0, 1e-3], [-1e-3, 0.0]])
    d.error_array = [e, e, e]                          # identical: B is singular
    d.fock_array = [np.eye(2), 2 * np.eye(2), 3 * np.eye(2)]
    c = d._coefficients()
    assert np.isfinite(c).all()
    assert len(d.fock_array) < 3


def test_device_comparison_is_exact(monkeypatch):
    """An engine on 'cuda' means the current device: a tensor on another GPU is refused
    (its pointer would be read as this device's memory)."""
    from gaussium_gb300 import _lib
    monkeypatch.setattr(torch.cuda, "current_device", lambda: 0)
    assert engine.indexed_device("cuda") == torch.device("cuda", 0)
    assert engine.indexed_device("cuda:1") == torch.device("cuda", 1)

    class FakeCuda:                 # stands in for a float64 tensor on cuda:1
        is_cuda = True
        dtype = torch.float64
        device = torch.device("cuda", 1)
        shape = (2, 2)

        def is_contiguous(self):
            return True
    monkeypatch.setattr(engine.torch, "Tensor", FakeCuda)
    with pytest.raises(_lib.GsError):
        engine._check_device_tensor(FakeCuda(), "cuda", "density matrix")
    engine._check_device_tensor(FakeCuda(), "cuda:1", "density matrix")


def test_quartet_batch_host_planning(monkeypatch):
    """QuartetBatch's host planning without a device (the pair records stubbed): class
    segments in canonical order, tasks sorted by descending primitive work inside each,
    and the heavy prefix counted with every class's threshold."""
    from gaussium_gb300.workloads import random_shell_quartets
    sb, q, _ = random_shell_quartets(3000, seed=2)

    class StubPairs:
        def __init__(self, ds, pairs, want32=True, max_exp=0.0):
            self.nprim = (sb.nprim[pairs[:, 0]].astype(np.int64) * sb.nprim[pairs[:, 1]])

    monkeypatch.setattr(engine, "PairSet", StubPairs)
    monkeypatch.setattr(engine.torch.Tensor, "to", lambda self, dev: self)
    b = engine.QuartetBatch(_host_only(sb), q)
    assert [s for _, s, _ in b.segments] == sorted(s for _, s, _ in b.segments)
    work = b.sorted_bra_nprim * b.sorted_ket_nprim
    for (cls, s, e), (split, coop) in zip(b.segments, b.heavy):
        assert np.all(np.diff(work[s:e]) <= 0)
        assert split == np.count_nonzero(work[s:e] >= engine.heavy_threshold(cls))
        assert np.all(work[s:s + split] >= engine.heavy_threshold(cls))
        assert coop == np.count_nonzero(work[s:e] >= engine.COOP_PRIM_QUARTETS)
        assert np.all(work[s:s + coop] >= engine.COOP_PRIM_QUARTETS)
    assert sum(c for _, c in b.heavy) > 0


def test_mixed_prefix_bands(monkeypatch):
    """The heavy prefix of a mixed-precision build: banded launches whose bands tile the
    density-weighted bound at the cut exactly as the partition does (FP64 at or above it,
    FP32 below), over the same prefix in both precisions -- each precision's heavy tasks
    in its heavy form (split for a thread-form class, cooperative for a warp-form one) and
    the rest of the prefix in its configured form; nothing when neither precision has a
    heavy form."""
    forms = {64: engine.THREAD_FORM, 32: engine.THREAD_FORM}

    class StubLib:
        def gs_class_form(self, la, lb, lc, ld, precision):
            return forms[precision]

    monkeypatch.setattr(engine._lib, "lib", lambda: StubLib())
    cls, inf = (1, 0, 0, 0), float("inf")
    S, C = engine.SPLIT_FORM, engine.COOP_FORM
    assert engine.mixed_prefix(cls, (0, 0), 1e-2) == (0, [])
    assert engine.mixed_prefix(cls, (7, 2), 1e-2) == (7, [
        (64, S, 0, 7, 1e-2, inf), (32, S, 0, 7, 0.0, 1e-2)])
    monkeypatch.setattr(engine, "SPLIT_OFF", {(cls, 64)})
    assert engine.mixed_prefix(cls, (7, 2), 1e-2) == (7, [
        (64, 0, 0, 7, 1e-2, inf), (32, S, 0, 7, 0.0, 1e-2)])
    monkeypatch.setattr(engine, "SPLIT_OFF", set())
    forms[32] = engine.WARP_FORM             # FP64 splits 7, FP32 runs 2 cooperatively
    assert engine.mixed_prefix(cls, (7, 2), 1e-2) == (7, [
        (64, S, 0, 7, 1e-2, inf), (32, C, 0, 2, 0.0, 1e-2), (32, 0, 2, 5, 0.0, 1e-2)])
    forms[64] = engine.GROUPED_FORM
    assert engine.mixed_prefix(cls, (7, 2), 1e-2) == (2, [
        (64, C, 0, 2, 1e-2, inf), (32, C, 0, 2, 0.0, 1e-2)])
    assert engine.mixed_prefix(cls, (7, 0), 1e-2) == (0, [])


def test_split_forms_by_class_form(monkeypatch):
    """split_forms picks the heavy count and form that match the class's form."""
    form = [engine.THREAD_FORM]

    class StubLib:
        def gs_class_form(self, la, lb, lc, ld, precision):
            return form[0]

    monkeypatch.setattr(engine._lib, "lib", lambda: StubLib())
    cls = (2, 2, 2, 2)
    assert engine.split_forms(cls, 64, (5, 3)) == [(engine.SPLIT_FORM, 0, 5), (engine.THREAD_FORM, 5, None)]
    form[0] = engine.WARP_FORM
    assert engine.split_forms(cls, 64, (5, 3)) == [(engine.COOP_FORM, 0, 3), (engine.WARP_FORM, 3, None)]
    assert engine.split_forms(cls, 64, (5, 0)) == [(0, 0, None)]
    w = np.array([600, 300, 200, 128, 127, 40, 1])
    assert engine.heavy_counts(cls, w) == (int(np.count_nonzero(w >= engine.heavy_threshold(cls))), 4)


@pytest.mark.parametrize("case", ["random", "empty", "one", "repeated", "int32"])
def test_device_planning_matches_host_planning(monkeypatch, case):
    """QuartetBatch(plan="device") restated with torch on the CPU (the pair records
    stubbed: every primitive pair kept): the same task list byte for byte, the same class
    segments, heavy counts, block offsets and primitive-quartet totals as the host
    planning, for 5,000 seeded quartets, none, one, one repeated 7 times, and int32
    input."""
    import torch
    from gaussium_gb300.workloads import random_shell_quartets
    sb, q, _ = random_shell_quartets(5000, seed=3)
    q = {"random": q, "empty": np.zeros((0, 4), dtype=np.int64), "one": q[:1],
         "repeated": np.repeat(q[:1], 7, 0), "int32": q.astype(np.int32)}[case]

    class StubPairs:
        def __init__(self, ds, pairs, want32=True, max_exp=0.0):
            pairs = np.asarray(pairs).reshape(-1, 2)
            self.nprim = (sb.nprim[pairs[:, 0]].astype(np.int64) * sb.nprim[pairs[:, 1]])

    def stub_build(self, stream=None, want32=True):
        self.kept[:self.n] = (self.ds.nprim[self.shells[:, 0].long()] *
                              self.ds.nprim[self.shells[:, 1].long()]).to(torch.int32)

    ds = _host_only(sb)
    ds.device = torch.device("cpu")
    ds.l = torch.as_tensor(sb.l.astype(np.int32))
    ds.nprim = torch.as_tensor(sb.nprim.astype(np.int64))
    monkeypatch.setattr(engine, "PairSet", StubPairs)
    monkeypatch.setattr(engine.DevicePairSet, "build", stub_build)
    monkeypatch.setattr(engine.torch.Tensor, "to", lambda self, *a, **k: self)
    host = engine.QuartetBatch(ds, q)
    dev = engine.QuartetBatch(ds, q, plan="device")
    assert np.array_equal(dev.tasks.numpy(), host.tasks.numpy())
    assert dev.segments == host.segments
    assert dev.heavy == host.heavy
    assert np.array_equal(dev.offsets, host.offsets) and dev.total == host.total
    assert np.array_equal(dev.sorted_bra_nprim, host.sorted_bra_nprim)
    assert (dev.prim_quartets, dev.full_prim_quartets) == (host.prim_quartets,
                                                           host.full_prim_quartets)
    with pytest.raises(ValueError):
        engine.QuartetBatch(ds, np.array([[0, 1, 2, sb.nshell]]), plan="device")
