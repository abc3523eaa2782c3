"""The pipelined host-to-host block API: consecutive batches with different shell data
come back equal to one-at-a-time evaluation of each (slots and copy streams keep them
apart)."""
import numpy as np
import pytest
import torch

from conftest import golden, synthetic_shells

pytestmark = pytest.mark.gpu


def test_pipeline_batches_match_direct_evaluation(gpu_lib):
    from gaussium_gb300.basis import ShellBasis
    from gaussium_gb300.engine import PRIM_SCREEN, DeviceShells, QuartetBatch
    from gaussium_gb300.pipeline import BlockPipeline
    sb = ShellBasis.from_shell_dicts(synthetic_shells())
    q = golden("synthetic")["quartets"]
    variants = []
    for shift in (0.0, 0.3, -0.2, 0.5):
        v = ShellBasis(sb.l, sb.centre + shift * np.arange(sb.nshell)[:, None] / sb.nshell,
                       sb.prim_off, sb.expo, sb.coef, sb.comp_scale)
        ds = DeviceShells(v)
        b = QuartetBatch(ds, q, want32=False, max_exp=PRIM_SCREEN)
        ref = torch.zeros(b.total, dtype=torch.float64, device="cuda")
        b.run(ref, 64)
        variants.append((BlockPipeline.pinned_shells(v), ref.cpu().numpy()))
    pipe = BlockPipeline(sb, q, precision=64)
    outs = [torch.full((pipe.total,), np.nan, dtype=torch.float64).pin_memory() for _ in variants]
    events = [pipe.submit(host_in, o) for (host_in, _), o in zip(variants, outs)]
    assert len({id(e) for e in events}) == len(events)     # one event per batch
    for (_, ref), o, e in zip(variants, outs, events):
        e.synchronize()
        assert np.array_equal(o.numpy(), ref)
    pipe.synchronize()
