"""Every kernel form of every class built with several (thread per quartet, warp per
quartet, grouped warp, stacked warp) gives the same integrals and J/K, and the autotuner
picks one of them per class."""
import numpy as np
import pytest
import torch

from conftest import golden, synthetic_shells
from molecules import load, random_density

pytestmark = pytest.mark.gpu


def _multi_form_classes(precision):
    from gaussium_gb300 import autotune, build
    return [c for c in build.classes() if len(autotune.forms(c, precision)) >= 2]


@pytest.mark.parametrize("precision,rtol", [(64, 1e-12), (32, 1e-5)])
def test_forms_agree_on_synthetic_blocks(gpu_lib, precision, rtol):
    """Every class built with more than one form gives the same blocks in each."""
    from gaussium_gb300 import autotune
    from gaussium_gb300.basis import ShellBasis
    from gaussium_gb300.engine import DeviceShells, QuartetBatch
    multi = _multi_form_classes(precision)
    assert multi, "no class is built with more than one form"
    sb = ShellBasis.from_shell_dicts(synthetic_shells())
    q = golden("synthetic")["quartets"]
    ds = DeviceShells(sb)
    batch = QuartetBatch(ds, q, want32=precision == 32)

    def run():
        buf = torch.zeros(max(1, batch.total), dtype=torch.float64, device="cuda")
        batch.run(buf, precision)
        return buf.cpu().numpy()

    ref = run()
    tried = set()
    try:
        for v in (autotune.THREAD, autotune.WARP, autotune.GROUPED, autotune.STACKED):
            for cls in multi:
                autotune.set_form(cls, precision, v if v in autotune.forms(cls, precision) else 0)
                if v in autotune.forms(cls, precision):
                    tried.add((cls, v))
            got = run()
            assert np.max(np.abs(got - ref)) <= rtol * np.max(np.abs(ref)), v
    finally:
        autotune.reset([(c, 0, 0) for c in multi], (precision,))
    if precision == 64:
        assert any(v == autotune.GROUPED for _, v in tried)
    assert any(v == autotune.STACKED for _, v in tried)


def test_tuner_chooses_and_jk_unchanged(gpu_lib):
    from gaussium_gb300 import autotune
    from gaussium_gb300.basis import ShellBasis
    from gaussium_gb300.engine import JKEngine
    g, funcs, table = load("h2o_631gs")
    eng = JKEngine(ShellBasis.from_functions(funcs), schwarz_thr=0.0)
    p = torch.tensor(random_density(eng.sb.nbf, 3), device="cuda")
    J0, (K0,) = eng.jk(p, [p])
    try:
        chosen = autotune.tune_jk(eng, p, precisions=(64,), reps=2)
        assert chosen
        for (cls, prec), r in chosen.items():
            assert r["form"] in autotune.forms(cls, prec)
            if len(autotune.forms(cls, prec)) >= 2:
                assert set(r["ms"]) == set(autotune.forms(cls, prec))
        J1, (K1,) = eng.jk(p, [p])
    finally:
        autotune.reset(eng.segments)
    assert torch.max(torch.abs(J1 - J0)).item() < 1e-12
    assert torch.max(torch.abs(K1 - K0)).item() < 1e-12


def test_stacked_jk_matches_warp_form(gpu_lib):
    """J/K of water / 6-31G* with every class on the stacked warp form (where built) against
    the plain warp form: FP64, FP32, and a mixed build whose partitioned launches read the
    task counts from the device."""
    from gaussium_gb300 import autotune
    from gaussium_gb300.basis import ShellBasis
    from gaussium_gb300.engine import JKEngine
    g, funcs, table = load("h2o_631gs")
    eng = JKEngine(ShellBasis.from_functions(funcs), schwarz_thr=0.0)
    p = torch.tensor(random_density(eng.sb.nbf, 5), device="cuda")
    runs = (dict(precision=64), dict(precision=32), dict(mixed_cut=1e-2, screen_thr=1e-14))
    out = {}
    stacked = 0
    try:
        for form in (autotune.WARP, autotune.STACKED):
            for cls, _, _ in eng.segments:
                for prec in (64, 32):
                    fs = autotune.forms(cls, prec)
                    v = form if form in fs else (autotune.WARP if autotune.WARP in fs else 0)
                    stacked += v == autotune.STACKED
                    autotune.set_form(cls, prec, v)
            out[form] = [eng.jk(p, [p], **kw) for kw in runs]
    finally:
        autotune.reset(eng.segments)
    assert stacked > 0
    for kw, (Jw, (Kw,)), (Js, (Ks,)) in zip(runs, out[autotune.WARP], out[autotune.STACKED]):
        tol = 1e-12 if kw.get("precision") == 64 else 1e-5
        for a, b in ((Js, Jw), (Ks, Kw)):
            assert torch.max(torch.abs(a - b)).item() <= tol * torch.max(torch.abs(b)).item(), kw
