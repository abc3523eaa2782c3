"""ERI class kernels on the GPU (through the C ABI) against the oracle."""
import numpy as np
import pytest
import torch

import oracle
from conftest import golden, synthetic_shells
from molecules import load
import hostcheck

pytestmark = pytest.mark.gpu


def test_boys_device_matches_exact(gpu_lib):
    from gaussium_gb300 import _lib
    g = golden("boys")
    xs = torch.tensor(g["x"], dtype=torch.float64, device="cuda")
    for M in (0, 4, 8, 10):
        ex = np.array([[oracle.boys_exact(m, x) for m in range(M + 1)] for x in g["x"]])
        for prec, rtol, atol in ((64, 5e-15, 0.0), (32, 2e-6, 1e-30)):
            F = torch.zeros(len(xs) * (M + 1), dtype=torch.float64, device="cuda")
            _lib.check(gpu_lib.gs_boys_eval(M, prec, len(xs), _lib.ptr(xs), _lib.ptr(F),
                                            _lib.stream()), "boys")
            F = F.view(-1, M + 1).cpu().numpy()
            assert np.all(np.abs(F - ex) <= atol + rtol * np.abs(ex)), (M, prec)


@pytest.mark.parametrize("precision,rtol,atol", [(64, 1e-11, 1e-13), (32, 1e-4, 1e-8)])
def test_synthetic_every_class(gpu_lib, precision, rtol, atol):
    from gaussium_gb300 import engine
    from gaussium_gb300.basis import ShellBasis
    shells = synthetic_shells()
    sb = ShellBasis.from_shell_dicts(shells)
    table = oracle.FunctionTable.from_shells(shells)
    g = golden("synthetic")
    quartets = np.array([q for q in g["quartets"]
                         if gpu_lib.gs_class_available(*sorted(sb.l[q][:2], reverse=True),
                                                       *sorted(sb.l[q][2:], reverse=True))
                         or gpu_lib.gs_class_available(*sorted(sb.l[q][2:], reverse=True),
                                                       *sorted(sb.l[q][:2], reverse=True))])
    out, off = engine.eri_blocks(sb, quartets, precision=precision)
    for i, q in enumerate(quartets):
        ref = oracle.eri_functions(table, hostcheck.function_quartets(sb, q), boys_mode=1)
        got = out[off[i]:off[i + 1]]
        assert np.max(np.abs(got - ref)) <= atol + rtol * np.max(np.abs(ref)), q


def test_h2o_631gs_all_quartets_match_reference(gpu_lib):
    """Every canonical function quartet of water/6-31G* against the as-is reference
    (its Boys error bounds the difference) and the exact-Boys oracle (1e-13)."""
    from gaussium_gb300.dropin import TwoElectronRepulsionGPU
    g, funcs, table = load("h2o_631gs")
    dense = TwoElectronRepulsionGPU(funcs, None, None, 1).create_repulsion_matrix()
    keys = g["keys"].astype(np.int64)
    got = dense[keys[:, 0], keys[:, 1], keys[:, 2], keys[:, 3]]
    assert np.max(np.abs(got - g["eri"])) < 1e-10
    exact = oracle.eri_functions(table, keys, boys_mode=1)
    assert np.max(np.abs(got - exact)) < 1e-13
    # 8-fold symmetry of the dense tensor
    assert np.array_equal(dense, dense.transpose(1, 0, 2, 3))
    assert np.array_equal(dense, dense.transpose(2, 3, 0, 1))


def test_dense_tensor_h2o_sto3g(gpu_lib):
    from gaussium_gb300.dropin import TwoElectronRepulsionMatrixOSGPU
    g, funcs, _ = load("h2o_sto3g")
    dense = TwoElectronRepulsionMatrixOSGPU(funcs, None, 4).create_repulsion_matrix()
    assert np.max(np.abs(dense - g["dense"])) < 1e-10


def test_integral_objects_reference_unit_quartets(gpu_lib):
    """The reference's own ERI unit test (test_electron_repulsion_matrix.py) through the
    drop-in integral objects, for all three scheme names."""
    from types import SimpleNamespace as NS
    from gaussium_gb300.dropin import GpuObaraSaika, GpuHeadGordonPople, GpuElectronRepulsion
    g = golden("eri_heh")
    he_r, h_r = (0, 0, 0.7316), (0, 0, -0.7316)

    def fn(r, prims):
        return NS(primitive_gaussian_array=[NS(contraction=c, exponent=a, coordinates=r,
                                                integral_exponents=(0, 0, 0), normalisation=n)
                                             for c, a, n in prims],
                  coordinates=r, integral_exponents=(0, 0, 0), normalisation=1)
    he = fn(he_r, [(0.15432897, 9.75393461, 3.9336432656254527),
                   (0.53532814, 1.77669115, 1.0967787981767012),
                   (0.44463454, 0.48084429, 0.41154131374122654)])
    h = fn(h_r, [(0.15432897, 3.42525091, 1.794441832218435),
                 (0.53532814, 0.62391373, 0.5003264923314032),
                 (0.44463454, 0.16885540, 0.18773545851092535)])
    basis = [he, h]
    for cls, ref in ((GpuObaraSaika, g["os"]), (GpuHeadGordonPople, g["hgp"]),
                     (GpuElectronRepulsion, g["cook"])):
        obj = cls()
        got = np.array([obj.integrate(*[basis[i] for i in k]) for k in g["keys"]])
        assert np.max(np.abs(got - ref)) < 1e-10
        for v, want in zip(got, g["test_values"]):
            np.testing.assert_approx_equal(v, want, 4)


def test_integral_object_p_and_d_functions(gpu_lib):
    """Single-function calls with p and d components and arbitrary given normalisations."""
    from gaussium_gb300.dropin import GpuObaraSaika
    g, funcs, table = load("h2o_631gs")
    rng = np.random.default_rng(3)
    keys = rng.integers(0, len(funcs), size=(40, 4))
    obj = GpuObaraSaika()
    got = np.array([obj.integrate(*[funcs[i] for i in k]) for k in keys])
    ref = oracle.eri_functions(table, keys, boys_mode=1)
    assert np.max(np.abs(got - ref)) < 1e-13


def test_empty_batch(gpu_lib):
    from gaussium_gb300 import engine
    from gaussium_gb300.basis import ShellBasis
    sb = ShellBasis.from_shell_dicts(synthetic_shells()[:4])
    out, off = engine.eri_blocks(sb, np.zeros((0, 4), dtype=np.int64))
    assert len(off) == 1 and off[0] == 0


def test_permuted_quartets_agree(gpu_lib):
    from gaussium_gb300 import engine
    from gaussium_gb300.basis import ShellBasis
    shells = synthetic_shells()
    sb = ShellBasis.from_shell_dicts(shells)
    g = golden("synthetic")
    q = [x for x in g["quartets"] if sum(sb.l[x]) <= 5][:12]
    perms = [(0, 1, 2, 3), (1, 0, 2, 3), (0, 1, 3, 2), (2, 3, 0, 1), (3, 2, 1, 0)]
    allq = np.array([[x[p] for p in perm] for x in q for perm in perms])
    out, off = engine.eri_blocks(sb, allq)
    n = [[len(engine.COMPONENTS[int(sb.l[s])]) for s in x] for x in allq]
    for i in range(len(q)):
        base = out[off[5 * i]:off[5 * i + 1]].reshape(n[5 * i])
        for j, perm in enumerate(perms):
            blk = out[off[5 * i + j]:off[5 * i + j + 1]].reshape(n[5 * i + j])
            np.testing.assert_allclose(blk, base.transpose(perm), rtol=0, atol=1e-15)


def test_primitive_screening_changes_nothing_measurable(gpu_lib):
    """Dropping primitive pairs with a Gaussian-product factor below 1e-24 changes no
    block element by more than 1e-13 on the microbench's distribution."""
    import torch
    from gaussium_gb300 import engine
    from gaussium_gb300.workloads import random_shell_quartets
    sb, q, _ = random_shell_quartets(20000, seed=5)
    ds = engine.DeviceShells(sb)
    outs = []
    for max_exp in (0.0, engine.PRIM_SCREEN):
        b = engine.QuartetBatch(ds, q, want32=False, max_exp=max_exp)
        o = torch.zeros(b.total, dtype=torch.float64, device="cuda")
        b.run(o, 64)
        outs.append(o)
        kept = b.prim_quartets / b.full_prim_quartets
    assert float((outs[0] - outs[1]).abs().max()) < 1e-13
    assert kept < 0.8      # the screen does drop work on this distribution


@pytest.mark.parametrize("precision", [64, 32])
def test_heavy_quartet_forms_match_plain_forms(gpu_lib, precision):
    """Quartets with many primitive quartets run in the split form (thread-form classes)
    or the cooperative form (warp-form classes); with the default forms and with every
    class on the warp form, the blocks agree with the same forms run without the heavy
    forms (the sums differ in order only): within 1e-12 of the largest element in FP64;
    in FP32 both within 1e-4 of it from the FP64 blocks (the tolerance of every FP32
    class test: the FP32 recursions' own error, which a different summation order moves
    by the same amount)."""
    import torch
    from gaussium_gb300 import autotune, engine
    from gaussium_gb300.workloads import random_shell_quartets
    sb, q, _ = random_shell_quartets(6000, seed=21)
    ds = engine.DeviceShells(sb)
    b = engine.QuartetBatch(ds, q, want32=precision == 32, max_exp=engine.PRIM_SCREEN)
    assert sum(h[0] for h in b.heavy) > 0 and sum(h[1] for h in b.heavy) > 0
    classes = [c for c, _, _ in b.segments]
    ref = torch.zeros(b.total, dtype=torch.float64, device="cuda")
    b.run(ref, 64)
    scale = float(ref.abs().max())
    try:
        for warp_all in (False, True):
            if warp_all:
                for c in classes:
                    autotune.set_form(c, precision, autotune.WARP)
            heavy = torch.zeros(b.total, dtype=torch.float64, device="cuda")
            b.run(heavy, precision)
            engine.SPLIT_OFF.update((c, precision) for c in classes)
            plain = torch.zeros_like(heavy)
            b.run(plain, precision)
            engine.SPLIT_OFF.clear()
            if precision == 64:
                assert float((heavy - plain).abs().max()) <= 1e-12 * scale, warp_all
            else:
                for x in (heavy, plain):
                    assert float((x - ref).abs().max()) <= 1e-4 * scale, warp_all
    finally:
        engine.SPLIT_OFF.clear()
        autotune.reset([(c, 0, 0) for c in classes], (precision,))


def test_cooperative_jk_matches_plain_forms(gpu_lib):
    """J/K of six seeded centres with one s, p and d shell of six primitives each, every
    class on the warp form: the heavy quartets in the cooperative form agree with the
    plain warp form, in FP64 and in a mixed build (banded heavy prefix ahead of the
    partitioned launch)."""
    import torch
    from gaussium_gb300 import autotune, engine
    from gaussium_gb300.basis import ShellBasis
    rng = np.random.default_rng(7)
    shells = []
    for _ in range(6):
        centre = rng.uniform(-1.5, 1.5, 3)
        for l in (0, 1, 2):
            shells.append({"l": l, "centre": centre.tolist(),
                           "expo": np.sort(10 ** rng.uniform(-1, 1.5, 6))[::-1].tolist(),
                           "coef": rng.uniform(0.2, 1.0, 6).tolist()})
    sb = ShellBasis.from_shell_dicts(shells)
    eng = engine.JKEngine(sb, schwarz_thr=1e-12)
    assert sum(h[1] for h in eng.heavy) > 0
    rng = np.random.default_rng(4)
    a = rng.standard_normal((sb.nbf, sb.nbf))
    P = torch.tensor(a + a.T, device="cuda")
    try:
        for c, _, _ in eng.segments:
            for prec in (64, 32):
                autotune.set_form(c, prec, autotune.WARP)
        for kw in (dict(), dict(mixed_cut=1e-2, screen_thr=1e-14)):
            J1, K1 = eng.jk(P, [P], **kw)
            engine.SPLIT_OFF.update((c, p) for c, _, _ in eng.segments for p in (64, 32))
            J0, K0 = eng.jk(P, [P], **kw)
            engine.SPLIT_OFF.clear()
            tol = 1e-11 if not kw else 1e-7      # FP32 quartets: sums in another order
            for x, y in ((J1, J0), (K1[0], K0[0])):
                assert float((x - y).abs().max()) <= tol * float(y.abs().max()), kw
    finally:
        engine.SPLIT_OFF.clear()
        autotune.reset(eng.segments)


def test_device_planning_matches_host_planning_gpu(gpu_lib):
    """QuartetBatch planned on the device against the host planning, with the real pair
    build and screen: the same task bytes, segments, heavy counts and offsets, and
    bit-identical blocks."""
    import torch
    from gaussium_gb300 import engine
    from gaussium_gb300.workloads import random_shell_quartets
    sb, q, _ = random_shell_quartets(20000, seed=8)
    ds = engine.DeviceShells(sb)
    bh = engine.QuartetBatch(ds, q, want32=True, max_exp=engine.PRIM_SCREEN)
    bd = engine.QuartetBatch(ds, q, want32=True, max_exp=engine.PRIM_SCREEN, plan="device")
    assert torch.equal(bd.tasks, bh.tasks)
    assert bd.segments == bh.segments and bd.heavy == bh.heavy
    assert np.array_equal(bd.offsets, bh.offsets)
    for prec in (64, 32):
        oh = torch.zeros(bh.total, dtype=torch.float64, device="cuda")
        od = torch.zeros_like(oh)
        bh.run(oh, prec)
        bd.run(od, prec)
        assert torch.equal(od, oh), prec
