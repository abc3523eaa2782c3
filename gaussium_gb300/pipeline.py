"""Host-to-host ERI block evaluation, pipelined across batches.

A caller that holds its shells in host memory and wants the integral blocks back in host
memory pays two copies per batch: the shell arrays in, the blocks out.  ``BlockPipeline``
keeps two device slots (shells, primitive-pair records, task list, output blocks) and two
copy streams, so that while batch i is evaluated on the compute stream, the shells of
batch i+1 are already moving in and the blocks of batch i-1 moving out.  Each batch still
makes both copies; only their overlap with compute changes.

Stream order per slot k = i mod 2:
    h2d stream:     wait(computed[k])  -> copy shells and tasks of batch i -> record h2d[k]
    compute stream: wait(h2d[k]), wait(d2h[k]) -> pair records, class kernels -> record computed[k]
    d2h stream:     wait(computed[k])  -> copy blocks of batch i -> record d2h[k]
so a slot's inputs are never overwritten while its kernels read them, and its output
buffer never while its previous copy-out is in flight.
"""
import numpy as np
import torch

from .engine import PRIM_SCREEN, DeviceShells, QuartetBatch

SHELL_FIELDS = ("centre", "l", "prim_off", "expo", "coef", "comp_scale")


class BlockPipeline:
    def __init__(self, sb, quartets, precision=64, max_exp=PRIM_SCREEN, device="cuda"):
        self.precision = precision
        self.slots = []
        for _ in range(2):
            ds = DeviceShells(sb, device)
            batch = QuartetBatch(ds, quartets, want32=precision == 32, max_exp=max_exp)
            out = torch.empty(max(1, batch.total), dtype=torch.float64, device=ds.device)
            self.slots.append({"ds": ds, "batch": batch, "out": out,
                               "h2d": torch.cuda.Event(), "computed": torch.cuda.Event(),
                               "d2h": torch.cuda.Event(), "used": False})
        self.total = self.slots[0]["batch"].total
        self.offsets = self.slots[0]["batch"].offsets
        self.h2d_stream = torch.cuda.Stream(device=device)
        self.d2h_stream = torch.cuda.Stream(device=device)
        self.n = 0
        # the task list travels with every batch (it is part of the batch's input)
        self.host_tasks = self.slots[0]["batch"].tasks.cpu().pin_memory()

    @staticmethod
    def pinned_shells(sb):
        """The shell arrays of a ShellBasis in pinned host memory (the per-batch input)."""
        return {k: torch.from_numpy(np.ascontiguousarray(getattr(sb, k))).pin_memory()
                for k in SHELL_FIELDS}

    def h2d_bytes(self, host_shells):
        return sum(t.numel() * t.element_size() for t in host_shells.values()) + \
            self.host_tasks.numel() * self.host_tasks.element_size()

    def submit(self, host_shells, host_out):
        """Queue one batch: ``host_shells`` (pinned, as from ``pinned_shells``) in, blocks
        out into the pinned float64 tensor ``host_out`` (``total`` elements).  Returns a
        new event, recorded for this batch only, that completes when ``host_out`` holds
        the blocks."""
        slot = self.slots[self.n % 2]
        compute = torch.cuda.current_stream()
        if slot["used"]:
            self.h2d_stream.wait_event(slot["computed"])
        with torch.cuda.stream(self.h2d_stream):
            for k in SHELL_FIELDS:
                getattr(slot["ds"], k).copy_(host_shells[k], non_blocking=True)
            slot["batch"].tasks.copy_(self.host_tasks, non_blocking=True)
            slot["h2d"].record(self.h2d_stream)
        compute.wait_event(slot["h2d"])
        if slot["used"]:
            compute.wait_event(slot["d2h"])
        slot["batch"].pairs.build(stream=compute, want32=self.precision == 32)
        slot["batch"].run(slot["out"], self.precision, stream=compute)
        slot["computed"].record(compute)
        self.d2h_stream.wait_event(slot["computed"])
        done = torch.cuda.Event()
        with torch.cuda.stream(self.d2h_stream):
            host_out.copy_(slot["out"][:self.total], non_blocking=True)
            slot["d2h"].record(self.d2h_stream)
            done.record(self.d2h_stream)
        slot["used"] = True
        self.n += 1
        return done

    def synchronize(self):
        for s in self.slots:
            if s["used"]:
                s["d2h"].synchronize()
