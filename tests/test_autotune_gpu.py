"""Both kernel forms of every class built with two (thread per quartet, warp per quartet)
give the same integrals and J/K, and the autotuner picks one of them per class."""
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
        for v in (autotune.THREAD, autotune.WARP, autotune.GROUPED):
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
            assert r["form"] in (autotune.THREAD, autotune.WARP, autotune.GROUPED)
            assert set(r["ms"]) == set(autotune.forms(cls, prec))
        J1, (K1,) = eng.jk(p, [p])
    finally:
        autotune.reset(eng.segments)
    assert torch.max(torch.abs(J1 - J0)).item() < 1e-12
    assert torch.max(torch.abs(K1 - K0)).item() < 1e-12
