#!/usr/bin/env python3
"""ERI microbench: 2,000,000 seeded shell quartets (four independent s/p/d shells each,
contraction degree 1-6, exponents log-uniform in [0.05, 1e4], centres in a 10 A cube),
evaluated to full contracted Cartesian blocks (~2 GB of FP64 output) on one GB300.

One step = the hot path over the whole batch with the shell data resident in HBM:
  K0 shell-pair build (primitive-pair records, FP64 and FP32) and the 21 angular-momentum
  class kernels writing every block.
``value`` is shell quartets/s of the FP64 path (each integral within 1e-10 of the oracle);
``fp32`` and ``mixed`` report the same batch evaluated in FP32 and with the precision
chosen per quartet from its Schwarz bound; ``e2e`` times the public host-buffer call
(host shells -> device, pair build, kernels, blocks -> host) per step.

Reference arm (--impl reference): the oracle's C restatement of the reference's
Obara-Saika recursion on the host cores, on a seeded sample of the same quartets.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gaussium_gb300|reference]
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "ERI quartets/s & Fock-build time, mixed vs FP64 GPU at |ΔE|≤1e-6 Eh"
UNIT = "shell quartets/s"
WORKLOAD = "synthetic ERI microbench: 2,000,000 seeded shell quartets, l uniform {s,p,d}, " \
           "K uniform 1-6, exponents log-uniform [0.05,1e4], centres in a 10 A cube"


# dram__bytes_read.sum + dram__bytes_write.sum per quartet of the dominant kernel, from one
# ncu capture of the 1,000,000-quartet case of this workload (its output blocks, 256 MB for
# (dd|dp), exceed the 129 MB L2, as at full size); empty until such a capture exists, and
# the line then reports traffic null
NCU_DRAM_BYTES_PER_QUARTET = {(2, 2, 2, 1): (56363520 + 195581952) / 48606}
NCU_TRAFFIC_SOURCE = ("ncu dram__bytes_read.sum + dram__bytes_write.sum of k_wide_write<2,2,2,1,"
                      "double> on the 1,000,000-quartet case (the one-warp launch over 48,606 "
                      "of the class's 49,552 quartets, 252.0 MB of output blocks > L2)")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gaussium_gb300", choices=["gaussium_gb300", "reference"])
    ap.add_argument("--quartets", type=int, default=2_000_000)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-fock", action="store_true",
                    help="leave out the (H2O)n / 6-31G* Fock-build arms of the default line")
    ap.add_argument("--forms", default=None,
                    help="path prefix for the tuned kernel forms: loaded from <prefix>.<workload>"
                         ".json when present, else tuned and saved there (a profiled run then "
                         "uses the forms its plain run chose)")
    ap.add_argument("--no-tune", action="store_true",
                    help="keep the built-in kernel form of every class (no autotuning)")
    ap.add_argument("--cpu-sample", type=int, default=1024)
    ap.add_argument("--workload", default="microbench", choices=["microbench", "water", "batch", "gradient", "optimize", "mo", "xc"])
    ap.add_argument("--nm-evals", type=int, default=4000,
                    help="energy evaluations the Nelder-Mead comparison may spend")
    ap.add_argument("--fd-coords", type=int, default=72)
    ap.add_argument("--molecules", type=int, default=256)
    ap.add_argument("--waters", type=int, default=16)
    ap.add_argument("--xc-waters", type=int, default=8,
                    help="water molecules of the XC workload (19 6-31G* functions each)")
    ap.add_argument("--mo-waters", type=int, default=6,
                    help="water molecules of the AO->MO workload (13 6-31G functions each)")
    ap.add_argument("--grad-mixed-cut", type=float, default=1e-3,
                    help="gradient workload: density-weighted bound below which the adjoint's "
                         "recursion runs in FP32")
    ap.add_argument("--grad-basis", default="6-31G",
                    help="basis of the gradient workload (6-31G, or 6-31G* with d shells)")
    ap.add_argument("--opt-basis", default="6-31G",
                    help="basis of the optimize workload (6-31G, or 6-31G* with d shells)")
    ap.add_argument("--opt-waters", type=int, default=4, help="waters of the optimize workload")
    ap.add_argument("--optimizer", default="L-BFGS-B", choices=["L-BFGS-B", "BFGS"],
                    help="quasi-Newton method of the geometry-optimisation workload")
    ap.add_argument("--guess", default="sad", choices=["core", "sad"],
                    help="starting density of the batch workload's SCF")
    ap.add_argument("--batch-check", type=int, default=16,
                    help="molecules of the batch workload checked against single FP64 RHF")
    ap.add_argument("--mixed-cut", type=float, default=1e-2,
                    help="density-weighted bound below which a quartet runs in FP32 (water, batch)")
    ap.add_argument("--prim-screen", type=float, default=55.262,
                    help="drop primitive pairs with alpha*beta/p |AB|^2 above this (0: keep all)")
    return ap.parse_args()


# ---------------------------------------------------------------------- distributed plumbing
def dist_init(args=None):
    """Replicas: one process per GPU (torchrun env), NCCL on GPUs; the same plumbing runs
    over gloo on CPU for the tests.  No collective is on the data path: ranks only meet at
    barriers and for the max-over-ranks time."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        backend = os.environ.get("GS_DIST_BACKEND") or ("nccl" if torch.cuda.is_available() else "gloo")
        if backend == "nccl":
            torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group(backend)
    return rank, world


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ---------------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms while running."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.samples = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", os.environ.get("LOCAL_RANK", "0")],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 7:
                self.samples.append(parts)

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4)
                          if s[3 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.samples)}


# ---------------------------------------------------------------------- CPU baseline (oracle)
def oracle_table(sb):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    from gaussium_gb300.basis import COMPONENTS
    centre, lmn, cnorm, prims = [], [], [], []
    for s in range(sb.nshell):
        k0, k1 = sb.prim_off[s], sb.prim_off[s + 1]
        for ci, c in enumerate(COMPONENTS[int(sb.l[s])]):
            centre.append(sb.centre[s]); lmn.append(c); cnorm.append(sb.comp_scale[s, ci])
            prims.append(list(zip(sb.coef[k0:k1], sb.expo[k0:k1], np.ones(k1 - k0))))
    return oracle, oracle.FunctionTable(np.array(centre), np.array(lmn), np.array(cnorm), prims)


def cpu_oracle_rate(sample, seed, threads):
    """Shell quartets/s of the oracle port (the reference's Obara-Saika recursion with
    memoised nodes, bit-identical results) on `sample` quartets drawn from the workload."""
    from gaussium_gb300.workloads import random_shell_quartets
    sb, q, _ = random_shell_quartets(sample, seed=seed + 1000)
    oracle, table = oracle_table(sb)
    fo = np.concatenate([[0], np.cumsum(sb.nfunc)])
    fq = []
    for a, b, c, d in q:
        ia, ib, ic, id_ = (np.arange(fo[x], fo[x + 1]) for x in (a, b, c, d))
        g = np.stack(np.meshgrid(ia, ib, ic, id_, indexing="ij"), -1).reshape(-1, 4)
        fq.append(g)
    fq = np.concatenate(fq)
    t0 = time.perf_counter()
    oracle.eri_functions(table, fq, boys_mode=0, memo=True, threads=threads)
    dt = time.perf_counter() - t0
    return sample / dt, dt, len(fq)


# ---------------------------------------------------------------------- GPU arm
def flops_model(batch, opcount):
    """Algorithmic FLOPs per class launch: K_bra*K_ket primitive quartets times the
    per-primitive-quartet count (VRR + its set-up and Boys) plus the per-quartet HRR and
    output scaling, FMA = 2."""
    out = {}
    nb = batch.sorted_bra_nprim.astype(np.float64)
    nk = batch.sorted_ket_nprim.astype(np.float64)
    for cls, s, e in batch.segments:
        tag = "".join(map(str, cls))
        oc = opcount[tag]
        L = oc["L"]
        prim = oc["vrr_flops"] + 64 + 3 * L       # set-up (~50) + Boys (~14 + 3 per order)
        contr = oc["hrr_flops"] + 2 * oc["nblk"]  # HRR + per-element scaling
        out[cls] = float(np.sum(nb[s:e] * nk[s:e])) * prim + (e - s) * contr
    return out


def fma_peak(precision, lanes=32):
    """FMA rate of the gs_fma_probe kernel (TFLOP/s counted over the active lanes)."""
    import torch
    from gaussium_gb300 import _lib
    L = _lib.lib()
    sm = torch.cuda.get_device_properties(0).multi_processor_count
    blocks, threads = sm * 8, 256
    sink = torch.zeros(blocks * threads, dtype=torch.float64, device="cuda")
    iters = 400 if precision == 64 else 8000
    L.gs_fma_probe_lanes(precision, blocks, threads, 10, lanes, _lib.ptr(sink), _lib.stream())
    best = 0.0
    for _ in range(3):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        _lib.check(L.gs_fma_probe_lanes(precision, blocks, threads, iters, lanes, _lib.ptr(sink),
                                        _lib.stream()), "fma")
        e1.record()
        torch.cuda.synchronize()
        best = max(best, blocks * threads * lanes / 32 * iters * 16 * 8 * 2 /
                   (e0.elapsed_time(e1) * 1e-3))
    return best / 1e12


def run_gpu(args, rank, world):
    import torch
    from gaussium_gb300 import build, engine, _lib
    from gaussium_gb300.workloads import random_shell_quartets
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    build.build()
    opcount = build.opcount()
    sb, quartets, _ = random_shell_quartets(args.quartets, seed=args.seed + rank)
    ds = engine.DeviceShells(sb)
    batch = engine.QuartetBatch(ds, quartets, want32=True, max_exp=args.prim_screen)
    out = torch.empty(batch.total, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream()
    classes = [c for c, _, _ in batch.segments]
    forms = {}
    if not args.no_tune:
        # kernel form (thread / warp per quartet) of every class built with both, chosen
        # on this batch by the autotuner before the timed region
        from gaussium_gb300 import autotune
        batch.pairs.build()
        chosen = autotune.tune_or_load(forms_file(args, "microbench"),
                                       lambda: autotune.tune_blocks(batch, out, reps=2))
        forms = {"%d%d%d%d/fp%d" % (*c, p): autotune.describe(r)
                 for (c, p), r in chosen.items()}

    def step(precision, timing=None):
        # the FP64 pass needs only the FP64 primitive-pair records
        batch.pairs.build(want32=precision == 32)
        if timing is None:
            batch.run(out, precision)
            return
        for cls, s, e in batch.segments:
            ev0 = torch.cuda.Event(enable_timing=True)
            ev1 = torch.cuda.Event(enable_timing=True)
            ev0.record(stream)
            batch.run(out, precision, classes=[cls])
            ev1.record(stream)
            timing.setdefault(cls, []).append((ev0, ev1))

    res = {}
    for precision in (64, 32):
        for _ in range(args.warmup):
            step(precision)
        torch.cuda.synchronize()
        timing = {}
        barrier(world)
        torch.cuda.synchronize()
        with ClockSampler() as clk:
            t0 = torch.cuda.Event(enable_timing=True)
            t1 = torch.cuda.Event(enable_timing=True)
            t0.record(stream)
            for _ in range(args.steps):
                step(precision, timing)
            t1.record(stream)
            torch.cuda.synchronize()
        barrier(world)
        ms = max_over_ranks(t0.elapsed_time(t1) / args.steps, world)
        per_cls = {c: float(np.mean([a.elapsed_time(b) for a, b in v])) for c, v in timing.items()}
        res[precision] = dict(ms=ms, per_cls=per_cls, clocks=clk.summary())
        if precision == 64:
            ref64 = out.clone()
    err32 = float((out - ref64).abs().max())
    del ref64

    # roofline of the dominant FP64 kernel
    peak64 = fma_peak(64)
    peak32 = fma_peak(32)
    # FP64 rate with 8 of 32 lanes active: equal time per warp instruction means a quarter
    # of the rate, the reason narrow recursion levels are filled with several quartets
    peak64_8lanes = fma_peak(64, lanes=8)
    fl = flops_model(batch, opcount)
    dom = max(res[64]["per_cls"], key=res[64]["per_cls"].get)
    achieved = fl[dom] / (res[64]["per_cls"][dom] * 1e-3) / 1e12
    total_flops = sum(fl.values())

    # e2e: host shells and tasks -> device, pair build, kernels, blocks -> host, every
    # step, through the pipelined host-to-host API (copies of batch i+1 in and of batch
    # i-1 out overlap the kernels of batch i)
    e2e = None
    if not args.no_e2e:
        from gaussium_gb300.pipeline import BlockPipeline
        del out
        torch.cuda.empty_cache()
        pipe = BlockPipeline(sb, quartets, precision=64, max_exp=args.prim_screen)
        host_in = BlockPipeline.pinned_shells(sb)
        host_out = [torch.empty(pipe.total, dtype=torch.float64).pin_memory() for _ in range(2)]
        for i in range(args.warmup):
            pipe.submit(host_in, host_out[i % 2])
        pipe.synchronize()
        torch.cuda.synchronize()
        barrier(world)
        t0 = time.perf_counter()
        for i in range(args.steps):
            pipe.submit(host_in, host_out[i % 2])
        pipe.synchronize()
        torch.cuda.synchronize()
        barrier(world)
        e2e_ms = max_over_ranks((time.perf_counter() - t0) * 1e3 / args.steps, world)
        e2e = {"value": args.quartets * world / (e2e_ms * 1e-3), "unit": UNIT,
               "h2d_bytes_per_step": int(pipe.h2d_bytes(host_in)),
               "d2h_bytes_per_step": int(pipe.total * 8), "ms_per_step": e2e_ms,
               "api": "gaussium_gb300.pipeline.BlockPipeline.submit (two device slots, "
                      "copy-in and copy-out streams overlapping the kernels)",
               "planning": "the class-sorted task list of this quartet set is built once, "
                           "before the timed steps (e2e_with_planning builds it per step)"}
        del pipe, host_out
        torch.cuda.empty_cache()
        # the same batch as a caller with new quartets every step sees it: shells and
        # quartets in, QuartetBatch planning on the device (canonical order, class sort,
        # primitive-pair records), the kernels and the blocks out, one step after another,
        # nothing overlapped
        host_blk = torch.empty(batch.total, dtype=torch.float64).pin_memory()
        nplan = max(1, min(args.steps, 5))

        def planned_step():
            dsn = engine.DeviceShells(sb)
            bn = engine.QuartetBatch(dsn, quartets, want32=False, max_exp=args.prim_screen,
                                     plan="device")
            on = torch.empty(bn.total, dtype=torch.float64, device="cuda")
            bn.run(on, 64)
            host_blk.copy_(on)
            return bn
        # warm-up as in the other arms: the first two steps are slower (block download
        # 55 ms and shell upload up to 240 ms, against 10 ms and 8 ms after)
        for _ in range(max(3, args.warmup)):
            planned_step()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(nplan):
            bn = planned_step()
        torch.cuda.synchronize()
        plan_ms = max_over_ranks((time.perf_counter() - t0) * 1e3 / nplan, world)
        e2e["e2e_with_planning"] = {
            "value": args.quartets * world / (plan_ms * 1e-3), "unit": UNIT,
            "ms_per_step": plan_ms, "steps": nplan, "warmup": max(3, args.warmup),
            "h2d_bytes_per_step": int(sum(getattr(sb, k).nbytes for k in
                                          ("centre", "l", "prim_off", "expo", "coef",
                                           "comp_scale", "func_off", "nprim")) + quartets.nbytes),
            "d2h_bytes_per_step": int(batch.total * 8),
            "api": "gaussium_gb300.engine.DeviceShells + QuartetBatch(quartets, "
                   "plan='device') + run, blocks copied to pinned host memory"}
        del host_blk, bn
        torch.cuda.empty_cache()

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        rate, dt, nf = cpu_oracle_rate(args.cpu_sample, args.seed, threads)
        cpu = {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{args.cpu_sample} seeded shell quartets of the same distribution "
                         f"({nf} function quartets), oracle C restatement of the reference's "
                         f"Obara-Saika recursion (memoised nodes), {dt:.1f} s on {threads} threads",
               "memoised": True}

    fock = None
    if not args.no_fock:
        # the metric's Fock-build half: (H2O)16 / 6-31G*, plain FP64 vs screened incremental
        # FP64 vs mixed, on the same engine
        fock = fock_arms(args.waters, args.waters + rank, args.mixed_cut, tune=not args.no_tune,
                         forms_path=forms_file(args, "fock"))

    n_all = args.quartets * world
    ms64, ms32 = res[64]["ms"], res[32]["ms"]
    # DRAM bytes per quartet of the dominant kernel from one ncu capture of a 200,000-quartet
    # case of this workload (dram__bytes_read.sum + dram__bytes_write.sum), scaled by the
    # class's quartet count here
    traffic, traffic_src = None, None
    nq_dom = sum(e - s for c, s, e in batch.segments if c == dom)
    if dom in NCU_DRAM_BYTES_PER_QUARTET:
        traffic = NCU_DRAM_BYTES_PER_QUARTET[dom] * nq_dom
        traffic_src = NCU_TRAFFIC_SOURCE + f", scaled by quartets ({nq_dom} of this class)"
    # algorithmic bytes of the dominant launch: its output blocks (written once) and the
    # primitive-pair records of its quartets (read at least once)
    out_bytes = 8 * nq_dom * int(np.prod([engine.NCART[x] for x in dom]))
    line = {
        "metric": METRIC,
        "value": n_all / (ms64 * 1e-3),
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms64,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded), shells resident in HBM; inputs (4.9 GB of pair records) "
                "larger than L2",
        "config": {"workload": WORKLOAD, "quartets_per_gpu": args.quartets,
                   "function_quartets_per_gpu": int(batch.total),
                   "primitive_quartets_per_gpu": int(batch.full_prim_quartets),
                   "primitive_quartets_evaluated_per_gpu": int(batch.prim_quartets),
                   "primitive_pair_screen": (f"alpha*beta/p|AB|^2 > {args.prim_screen} dropped "
                                             "(Gaussian-product factor < 1e-24)")
                   if args.prim_screen > 0 else "none",
                   "parallelism": f"replicas x{world}", "l2": "inputs larger than L2",
                   "kernel_forms_autotuned": forms},
        "roofline": {"bound": "fp64", "kernel": "eri class " + "".join(map(str, dom)) + " FP64",
                     "achieved": achieved, "peak": peak64, "unit": "TFLOP/s",
                     "frac": achieved / peak64, "traffic": traffic,
                     "traffic_unit": "bytes per launch (dram read + write)",
                     "traffic_source": traffic_src,
                     "algorithmic_output_bytes": out_bytes,
                     "peak_source": "gs_fma_probe FP64 FMA rate measured in this run "
                                    "(no FP64 figure among the pool's measured peaks)"},
        "fp64": {"value": n_all / (ms64 * 1e-3), "ms_per_step": ms64,
                 # the same step counted in the reference's unit (function quartets) and
                 # in primitive quartets (all, and those left after the pair screen)
                 "function_quartets_per_s": batch.total * world / (ms64 * 1e-3),
                 "primitive_quartets_per_s": batch.full_prim_quartets * world / (ms64 * 1e-3),
                 "primitive_quartets_evaluated_per_s": batch.prim_quartets * world / (ms64 * 1e-3),
                 "tflops": total_flops / (ms64 * 1e-3) / 1e12,
                 "frac_of_fp64_peak": total_flops / (ms64 * 1e-3) / 1e12 / peak64},
        "fp64_rate_with_8_of_32_lanes_active_tflops": peak64_8lanes,
        "fp32": {"value": n_all / (ms32 * 1e-3), "ms_per_step": ms32,
                 "max_abs_err_vs_fp64": err32, "fp32_peak_tflops": peak32},
        "per_class_ms_fp64": {"".join(map(str, c)): round(v, 3) for c, v in res[64]["per_cls"].items()},
        "per_class_ms_fp32": {"".join(map(str, c)): round(v, 3) for c, v in res[32]["per_cls"].items()},
        "per_class_gflop": {"".join(map(str, c)): round(v / 1e9, 3) for c, v in fl.items()},
        "clocks": res[64]["clocks"],
        "e2e": e2e,
        # the FP64 timed steps: the pair build and each class's launches (a class whose heavy
        # prefix runs in its own form launches twice)
        "gpu_launches": (1 + batch.launch_count(64)) * args.steps,
        "cpu_baseline": cpu,
        "fock": fock,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------- Fock-build workload
def forms_file(args, label):
    """Where ``--forms`` keeps the tuned kernel forms of one workload (None without it)."""
    return f"{args.forms}.{label}.json" if getattr(args, "forms", None) else None


def fock_arms(n_waters, seed, mixed_cut, tune=True, forms_path=None):
    """RHF of a seeded (H2O)n / 6-31G* cluster three times on one engine (Schwarz 1e-12):
      fp64                       plain FP64 integral-direct builds;
      fp64_screened_incremental  FP64 with density screening at 1e-12 and incremental
                                 (Delta P) builds, full build every 8;
      mixed                      the same screening and incremental builds, quartets with
                                 density-weighted bound below ``mixed_cut`` in FP32.
    Per arm: mean and total Fock-build time (host density in, Fock matrix out, as the
    SCF sees it), builds, energy, |dE| against the fp64 arm.  The mixed arm's energy is
    its own SCF energy (the FP32 error in full); a final FP64 build at its converged
    density is reported beside it, timed separately."""
    import torch
    from gaussium_gb300 import driver, molecules
    from gaussium_gb300.engine import JKEngine
    mol = molecules.water_cluster(n_waters, seed=seed)
    eng = JKEngine(molecules.shell_basis(mol, "6-31G*"), schwarz_thr=1e-12)
    forms = {}
    if tune:
        from gaussium_gb300 import autotune
        rng = np.random.default_rng(0)
        a = rng.standard_normal((eng.sb.nbf, eng.sb.nbf)) * 0.1
        chosen = autotune.tune_or_load(
            forms_path, lambda: autotune.tune_jk(eng, torch.tensor(a + a.T, device="cuda"), reps=2))
        forms = {"%d%d%d%d/fp%d" % (*c, p): autotune.describe(r)
                 for (c, p), r in chosen.items()}
    # warm-up: one build of each kind
    driver.rhf(mol, engine=eng, threshold=1e-10, max_iter=2)
    driver.rhf(mol, engine=eng, threshold=1e-10, max_iter=2, mixed_cut=mixed_cut,
               screen_thr=1e-12, incremental=True)
    runs = {
        "fp64": dict(),
        "fp64_screened_incremental": dict(screen_thr=1e-12, incremental=True),
        "mixed": dict(mixed_cut=mixed_cut, screen_thr=1e-12, incremental=True, final_fp64=True),
    }
    out = {}
    with ClockSampler() as clk:
        for name, kw in runs.items():
            r = driver.rhf(mol, engine=eng, threshold=1e-10, **kw)
            secs = list(r["fock_seconds"])
            fin = None
            if kw.get("final_fp64"):
                fin = secs.pop()            # the final FP64 build, reported on its own
            out[name] = {"ms_per_build": float(np.mean(secs)) * 1e3,
                         "fock_ms_total": float(np.sum(secs)) * 1e3, "builds": len(secs),
                         "iterations": r["iterations"], "converged": bool(r["converged"]),
                         "energy": r["scf_energy"]}
            if fin is not None:
                out[name]["final_fp64_build_ms"] = fin * 1e3
                out[name]["energy_after_final_fp64_build"] = r["energy"]
    e64 = out["fp64"]["energy"]
    for name in out:
        out[name]["abs_dE_vs_fp64"] = abs(out[name]["energy"] - e64)
    if "energy_after_final_fp64_build" in out["mixed"]:
        out["mixed"]["abs_dE_after_final_fp64_build"] = abs(
            out["mixed"]["energy_after_final_fp64_build"] - e64)
    t = {k: v["ms_per_build"] for k, v in out.items()}
    return {
        "workload": f"RHF (H2O){n_waters}/6-31G* (seed {seed}), {eng.sb.nbf} functions, "
                    f"Schwarz 1e-12, {eng.ntasks} unique shell quartets",
        "mixed_cut": mixed_cut, "screen_thr": 1e-12, "incremental_reset_every": 8,
        "arms": out,
        "speedup_mixed_vs_fp64": t["fp64"] / t["mixed"],
        "speedup_screened_incremental_vs_fp64": t["fp64"] / t["fp64_screened_incremental"],
        "speedup_mixed_vs_screened_incremental": t["fp64_screened_incremental"] / t["mixed"],
        "kernel_forms_autotuned": forms,
        "clocks": clk.summary(),
    }


def run_water(args, rank, world):
    """RHF on a seeded (H2O)n / 6-31G* cluster: plain FP64 integral-direct Fock builds vs
    the mixed FP32/FP64 incremental builds; times per build, |dE|."""
    import torch
    from gaussium_gb300 import build
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    build.build()
    f = fock_arms(args.waters, args.waters + rank, args.mixed_cut, tune=not args.no_tune,
                  forms_path=forms_file(args, "fock"))
    mx = f["arms"]["mixed"]
    line = {
        "metric": METRIC, "value": mx["ms_per_build"], "unit": "ms per Fock build (mixed)",
        "n_gpus": world, "steps": mx["builds"], "warmup": 1, "ms_per_step": mx["ms_per_build"],
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64+f32",
        "data": "synthetic (seeded water cluster)", "config": {"workload": f["workload"]},
        "fock": f, "clocks": f["clocks"],
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------- batched serving workload
def run_batch(args, rank, world):
    """256 seeded C/H/N/O chain molecules (3-30 atoms, 6-31G*): full batched SCF with
    graph-captured mixed-precision incremental Fock builds, molecules/s; per-molecule
    |dE| of a sample against one-at-a-time all-FP64 RHF."""
    import torch
    from gaussium_gb300 import batch, build, driver, molecules
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    build.build()
    mols = [molecules.random_chain(1000 * rank + s) for s in range(args.molecules)]
    opts = dict(mixed_cut=args.mixed_cut, screen_thr=1e-12, incremental=True, guess=args.guess)
    # outside the timed region: kernel loading, the per-element atomic densities of the
    # guess, and the kernel forms, tuned on 32 other molecules of the same kind
    other = batch.BatchedRHF([molecules.random_chain(100000 + s) for s in range(32)])
    if args.guess == "sad":
        from gaussium_gb300 import guess
        for sym in sorted(set(s for m in mols for s in m.symbols)):
            guess.element_density(sym, "6-31G*")
    forms = {}
    if not args.no_tune:
        from gaussium_gb300 import autotune
        chosen = autotune.tune_or_load(forms_file(args, "batch"), lambda: other.tune(reps=2))
        forms = {"%d%d%d%d/fp%d" % (*c, p): autotune.describe(r)
                 for (c, p), r in chosen.items()}
    other.run(max_iter=2, **opts)
    del other
    torch.cuda.synchronize()
    # timed: everything per batch -- one-electron integrals, pair records, Schwarz bounds,
    # task lists, graph capture and the SCF of all molecules -- with the Fock builds as one
    # launch per class, then the SCF again with one persistent launch per precision over
    # all classes (both captured in a CUDA graph); the faster Fock-build form is reported
    with ClockSampler() as clk:
        t0 = time.perf_counter()
        eng = batch.BatchedRHF(mols)
        torch.cuda.synchronize()
        t_setup = time.perf_counter() - t0
        e_cls, it_cls = eng.run(threshold=1e-10, **opts)
        torch.cuda.synchronize()
        t_cls = time.perf_counter() - t0 - t_setup
        conv_cls = eng.converged.copy()
        t1 = time.perf_counter()
        e_per, it_per = eng.run(threshold=1e-10, persistent=True, **opts)
        torch.cuda.synchronize()
        t_per = time.perf_counter() - t1
        conv_per = eng.converged.copy()
    persistent_faster = t_per < t_cls
    e, iters = (e_per, it_per) if persistent_faster else (e_cls, it_cls)
    dt = t_setup + min(t_per, t_cls)
    forms_compared = {
        "per_class_graph": {"scf_s": t_cls, "iterations": it_cls, "converged": int(conv_cls.sum())},
        "persistent_graph": {"scf_s": t_per, "iterations": it_per, "converged": int(conv_per.sum()),
                             "max_abs_dE_vs_per_class": float(np.max(np.abs(
                                 (e_per - e_cls)[conv_cls & conv_per]))) if (conv_cls & conv_per).any() else None},
        "reported": "persistent_graph" if persistent_faster else "per_class_graph"}
    # the same run again with per-iteration timing (one device sync per iteration), for
    # the record of where the time goes; not the timed number
    eng.run(threshold=1e-10, log_iterations=True, persistent=persistent_faster, **opts)
    it_log = [(i, round(sec, 3), n) for i, sec, n in eng.iteration_log]
    conv_mixed = eng.converged.copy()
    # one full FP64 build of every molecule, for scale
    P = eng.to_packed(torch.zeros_like(eng.Hb))
    eng.fock_packed(P)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    eng.fock_packed(P)
    torch.cuda.synchronize()
    t_fp64_build = time.perf_counter() - t1
    # the all-FP64 batched SCF (no density screening, no incremental builds): per-molecule
    # |dE| of the mixed run against it
    t1 = time.perf_counter()
    e64, it64 = eng.run(threshold=1e-10, guess=args.guess)
    torch.cuda.synchronize()
    t_fp64_scf = time.perf_counter() - t1
    conv64 = eng.converged.copy()
    both = conv64 & conv_mixed
    de = np.abs(e - e64)
    # and a sample against one-molecule-at-a-time FP64 RHF (the restated reference loop)
    sample = list(range(0, len(mols), max(1, len(mols) // args.batch_check)))
    single = [driver.rhf(mols[i], threshold=1e-10, max_iter=200) for i in sample]
    ok = [k for k, r in enumerate(single) if r["converged"] and both[sample[k]]]
    de1 = np.array([abs(e[sample[k]] - single[k]["energy"]) for k in ok])
    line = {
        "metric": METRIC, "value": len(mols) * world / dt, "unit": "molecules/s (full SCF)",
        "n_gpus": world, "steps": 1, "warmup": 1, "ms_per_step": dt * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64+f32",
        "data": "synthetic (seeded C/H/N/O chains)",
        "config": {"workload": f"batched RHF of {len(mols)} molecules, 6-31G*, "
                               f"{int(eng.nbf.sum())} functions in total",
                   "scf_iterations": iters, "converged": int(conv_mixed.sum()),
                   "unique_quartets": int(eng.ntasks),
                   "timed": "engine set-up (one-electron integrals, pairs, Schwarz, tasks) + "
                            "graph capture + SCF",
                   "setup_s": t_setup, "scf_s": dt - t_setup,
                   "kernel_forms_tuned_on": "32 other molecules of the same kind",
                   "mixed_cut": args.mixed_cut, "screen_thr": 1e-12, "incremental_reset_every": 8,
                   "guess": args.guess,
                   "final_energy": "one full FP64 build at the converged densities",
                   "kernel_forms_autotuned": forms},
        "fock_build_forms": forms_compared,
        "fp64_full_build_ms_all_molecules": t_fp64_build * 1e3,
        "iterations_seconds_converged": it_log,
        "fp64_batched_scf": {"seconds": t_fp64_scf, "iterations": it64,
                             "converged": int(conv64.sum())},
        "abs_dE_vs_fp64": {"molecules": int(both.sum()), "max": float(de[both].max()),
                           "median": float(np.median(de[both])),
                           "over_1e-6": int((de[both] > 1e-6).sum())},
        "abs_dE_vs_single_molecule_fp64": {"molecules_checked": len(ok),
                                           "single_not_converged": len(sample) - len(ok),
                                           "max": float(de1.max()) if len(ok) else None},
        "clocks": clk.summary(),
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------- gradient workload
def run_gradient(args, rank, world):
    """Analytic RHF gradient of a seeded (H2O)8 / 6-31G (or --grad-basis): time against one
    Fock build, and central finite differences (h = 1e-4 bohr) on --fd-coords coordinates."""
    import torch
    from gaussium_gb300 import build, gradient, molecules
    from gaussium_gb300.driver import TimedFock
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    build.build()
    basis = args.grad_basis
    mol = molecules.water_cluster(8, seed=8)
    gradient.rhf_energy_gradient(molecules.water_cluster(1, seed=1), basis)      # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e, g, res = gradient.rhf_energy_gradient(mol, basis, screen_thr=0.0, mixed_cut=None)
    torch.cuda.synchronize()
    t_total = time.perf_counter() - t0
    # gradient part alone, and one full Fock build, on the converged state
    sb = molecules.shell_basis(mol, basis)
    from gaussium_gb300.engine import JKEngine
    eng = JKEngine(sb, schwarz_thr=1e-14)
    fock_forms = {}
    if not args.no_tune:
        # the Fock build it is compared with gets its own tuned kernel forms
        from gaussium_gb300 import autotune
        chosen = autotune.tune_jk(eng, torch.tensor(res.density, device="cuda"), precisions=(64,),
                                  reps=2)
        fock_forms = {"%d%d%d%d" % c: autotune.describe(r) for (c, p), r in chosen.items()}
    fb = TimedFock(np.zeros((sb.nbf, sb.nbf)), eng)
    for _ in range(5):
        fb.create(res.density)
    t_fock = float(np.median(fb.builds))
    nocc = mol.electrons // 2
    P = res.density
    import gaussium_gb300.scf as scf
    from gaussium_gb300.hamiltonian import one_electron
    S, T, V = one_electron(sb, mol.coords, mol.charges)
    eps, C = scf.LinearAlgebra(S).diagonalize(res.fock)
    W = 2.0 * (C[:, :nocc] * eps[:nocc]) @ C[:, :nocc].T
    sa = gradient.shell_atoms(mol, sb)
    natom = len(mol.symbols)
    forms = {}
    if not args.no_tune:
        from gaussium_gb300 import autotune
        chosen = gradient.tune_eri_gradient(sb, eng, sa, P, natom, reps=2)
        forms = {"%d%d%d%d" % c: autotune.NAMES[r["form"]] for c, r in chosen.items()}
    gradient.eri_gradient(sb, eng, sa, P, natom)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ge = gradient.eri_gradient(sb, eng, sa, P, natom)
    torch.cuda.synchronize()
    t_eri_grad = time.perf_counter() - t0
    # the default: density screening (1e-12) and FP32 recursions below the mixed cut
    mx = dict(screen_thr=1e-12, mixed_cut=args.grad_mixed_cut)
    gradient.eri_gradient(sb, eng, sa, P, natom, **mx)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ge_mx = gradient.eri_gradient(sb, eng, sa, P, natom, **mx)
    torch.cuda.synchronize()
    t_eri_grad_mx = time.perf_counter() - t0
    g_mx = g - ge + ge_mx
    # per-class device time of the ERI gradient launches
    per_cls = {}
    st = torch.cuda.current_stream()
    for cls, s0, s1 in eng.segments:
        a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a0.record(st)
        gradient.eri_gradient(sb, eng, sa, P, natom, classes=[cls], host=False)
        a1.record(st)
        a1.synchronize()
        per_cls["%d%d%d%d" % cls] = round(a0.elapsed_time(a1), 3)
    gradient.one_electron_gradient_kernel(sb, mol, sa, P, W)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    g1 = gradient.one_electron_gradient_kernel(sb, mol, sa, P, W)
    torch.cuda.synchronize()
    t_one_grad = time.perf_counter() - t0
    # finite differences
    rng = np.random.default_rng(0)
    ncoord = min(args.fd_coords, 3 * len(mol.symbols))
    pick = rng.choice(3 * len(mol.symbols), size=ncoord, replace=False)
    h = 1e-4
    err = err_mx = 0.0
    for k in pick:
        a, x = divmod(int(k), 3)
        cp, cm = mol.coords.copy(), mol.coords.copy()
        cp[a, x] += h
        cm[a, x] -= h
        ep = gradient.rhf_energy_gradient(molecules.Molecule(mol.symbols, cp), basis, want_gradient=False)[0]
        em = gradient.rhf_energy_gradient(molecules.Molecule(mol.symbols, cm), basis, want_gradient=False)[0]
        fd = (ep - em) / (2 * h)
        err = max(err, abs(fd - g[a, x]))
        err_mx = max(err_mx, abs(fd - g_mx[a, x]))
    line = {
        "metric": METRIC, "value": (t_eri_grad_mx + t_one_grad) / t_fock,
        "unit": "gradient time / one Fock build", "n_gpus": world, "steps": 1, "warmup": 1,
        "ms_per_step": (t_eri_grad_mx + t_one_grad) * 1e3, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
        "config": {"workload": f"RHF gradient (H2O)8/{basis}, {sb.nbf} functions",
                   "fd_coordinates_checked": int(ncoord), "fd_step_bohr": h},
        "energy": e, "max_abs_grad_minus_fd": err_mx,
        "eri_gradient_ms": t_eri_grad_mx * 1e3, "one_electron_gradient_ms": t_one_grad * 1e3,
        "eri_gradient": {"screen_thr": 1e-12, "mixed_cut": args.grad_mixed_cut,
                         "max_abs_minus_fp64_gradient": float(np.max(np.abs(g_mx - g)))},
        "fp64_adjoint": {"eri_gradient_ms": t_eri_grad * 1e3,
                         "gradient_over_fock_build": (t_eri_grad + t_one_grad) / t_fock,
                         "max_abs_grad_minus_fd": err},
        "eri_gradient_ms_per_class": per_cls, "gradient_kernel_forms_autotuned": forms,
        "fock_kernel_forms_autotuned": fock_forms,
        "fock_build_ms": t_fock * 1e3, "scf_plus_gradient_s": t_total,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------- geometry optimisation
def run_optimize(args, rank, world):
    """Seeded (H2O)n (default 4) / 6-31G (or --opt-basis), each nucleus moved 0.1 A: BFGS
    on the analytic gradient against the reference's Nelder-Mead restated over the same GPU
    energy."""
    import torch
    from gaussium_gb300 import build, molecules, optimize
    from gaussium_gb300.gradient import rhf_energy_gradient
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    build.build()
    basis, nw = args.opt_basis, args.opt_waters
    mol = molecules.perturbed(molecules.water_cluster(nw, seed=nw), 0.1, seed=nw)
    rhf_energy_gradient(molecules.water_cluster(1, seed=1), basis)      # warm-up
    e0 = rhf_energy_gradient(mol, basis, want_gradient=False)[0]
    t0 = time.perf_counter()
    e_b, x_b, n_b, gmax_b = optimize.optimize_bfgs(mol, basis, gtol=1e-5, method=args.optimizer)
    t_b = time.perf_counter() - t0
    nm = optimize.NelderMead(mol.symbols, mol.coords,
                             lambda m: rhf_energy_gradient(m, basis, want_gradient=False)[0],
                             threshold=1e-6, max_evals=args.nm_evals)
    t0 = time.perf_counter()
    e_n, x_n = nm.optimize()
    t_n = time.perf_counter() - t0
    line = {
        "metric": METRIC, "value": t_b, "unit": "s (gradient-driven geometry optimisation)",
        "n_gpus": world, "steps": 1, "warmup": 1, "ms_per_step": t_b * 1e3,
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": f"synthetic (seeded (H2O){nw}, 0.1 A perturbation)",
        "config": {"workload": f"geometry optimisation (H2O){nw}/{basis}", "gtol": 1e-5,
                   "optimizer": args.optimizer + " on the analytic gradient, internal frame",
                   "nelder_mead_threshold": 1e-6, "nelder_mead_max_evals": args.nm_evals},
        "start_energy": e0,
        "gradient_driven": {"energy": e_b, "evaluations": n_b, "seconds": t_b,
                 "max_abs_gradient_internal": gmax_b},
        "nelder_mead": {"energy": e_n, "evaluations": nm.evals, "seconds": t_n,
                        "stopped_at_cap": nm.evals >= args.nm_evals},
        "energy_bfgs_minus_nelder_mead": e_b - e_n,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------- AO -> MO transform
def hbm_peak():
    """Measured HBM copy bandwidth of this GPU type (GB/s) and where it came from."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def run_mo(args, rank, world):
    """AO -> MO four-index transform and spin-orbital expansion of (H2O)n / 6-31G with a
    seeded orthogonal coefficient matrix (the operation count does not depend on its
    values).  One step = molecular_orbitals (four FP64 GEMM quarter transforms) followed by
    spin_basis_anti_physicist (the gs_spin_expand kernel), on device-resident tensors.
    The tensor has the pair symmetries of real integrals, so the transform takes its
    pair-packed form (about 4 n^5 GEMM flops).  ``roofline`` is the spin-orbital kernel's:
    17 n^4 doubles per launch (16 n^4 written, n^4 read) over its CUDA-event time."""
    import torch
    from gaussium_gb300 import _lib, build, molecules, transform
    from gaussium_gb300.dropin import dense_eri
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    build.build()
    L = _lib.lib()
    mol = molecules.water_cluster(args.mo_waters, seed=args.mo_waters)
    sb = molecules.shell_basis(mol, "6-31G")
    n = sb.nbf
    ao = dense_eri(sb)
    rng = np.random.default_rng(args.seed)
    c_host, _ = np.linalg.qr(rng.standard_normal((n, n)))
    c = torch.tensor(c_host, device="cuda")
    spin = torch.empty((2 * n,) * 4, dtype=torch.float64, device="cuda")
    st = torch.cuda.current_stream()

    def expand(mo, mode):
        _lib.check(L.gs_spin_expand(_lib.ptr(mo), n, mode, _lib.ptr(spin), _lib.stream()),
                   "gs_spin_expand")

    def ev():
        return torch.cuda.Event(enable_timing=True)

    for _ in range(max(3, args.warmup)):
        expand(transform.transform_device(ao, c), transform.SPIN_ANTI_PHYSICIST)
    torch.cuda.synchronize()
    t_tr, t_sp = [], []
    with ClockSampler() as clk:
        e_start = ev()
        e_start.record(st)
        for _ in range(args.steps):
            a, b, d = ev(), ev(), ev()
            a.record(st)
            mo = transform.transform_device(ao, c)
            b.record(st)
            expand(mo, transform.SPIN_ANTI_PHYSICIST)
            d.record(st)
            t_tr.append((a, b))
            t_sp.append((b, d))
            del mo
        e_end = ev()
        e_end.record(st)
        torch.cuda.synchronize()
    ms_total = e_start.elapsed_time(e_end)
    ms_tr = float(np.mean([x.elapsed_time(y) for x, y in t_tr]))
    ms_sp = float(np.mean([x.elapsed_time(y) for x, y in t_sp]))
    # each spin mode alone (inputs 16x smaller than the output, which is > L2)
    mo = transform.transform_device(ao, c)
    per_mode = {}
    for mode, name in ((0, "spin_basis_set"), (1, "blocked_spin_basis_set"),
                       (2, "spin_basis_anti_physicist")):
        expand(mo, mode)
        a, b = ev(), ev()
        a.record(st)
        for _ in range(args.steps):
            expand(mo, mode)
        b.record(st)
        b.synchronize()
        per_mode[name] = a.elapsed_time(b) / args.steps
    spin_bytes = 17 * n ** 4 * 8           # (2n)^4 written + n^4 read
    peak, peak_kind = hbm_peak()
    achieved = spin_bytes / (ms_sp * 1e-3) / 1e9
    # GEMM flops of the pair-packed transform the symmetric tensor takes: C^T X C over
    # P = n(n+1)/2 pairs in each half, 2 GEMMs of 2 n^3 flops per pair and half
    npair = n * (n + 1) // 2
    flops = 8.0 * npair * n ** 3
    fp64 = fma_peak(64)
    # end to end through the host-array API: AO tensor in, MO tensor back (molecular_orbitals),
    # then the MO tensor in and the spin-orbital tensor back (spin_basis_anti_physicist)
    ao_host = ao.cpu().numpy()
    e2e = []
    for k in range(args.warmup + args.steps):
        inp = ao_host.copy()            # molecular_orbitals overwrites its argument
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        mo_h = transform.molecular_orbitals(inp, c_host)
        sp_h = transform.spin_basis_anti_physicist(mo_h)
        t1 = time.perf_counter()
        if k >= args.warmup:
            e2e.append(t1 - t0)
        del sp_h
    h2d = (n ** 4 + n * n) * 8 + n ** 4 * 8
    d2h = n ** 4 * 8 + 16 * n ** 4 * 8
    # CPU baseline: the oracle's restatement of transformations.py:5-26 on the same
    # tensor (numpy matrix products over index pairs), and its spin-orbital expansion
    # (pure Python element loops) on a 6-orbital sample, scaled per output element
    cpu = None
    if not args.no_cpu_baseline and rank == 0:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle
        t0 = time.perf_counter()
        oracle.molecular_orbitals(ao_host, c_host)
        t_cpu_tr = time.perf_counter() - t0
        small = np.asarray(mo.cpu().numpy()[:6, :6, :6, :6])
        t0 = time.perf_counter()
        oracle.spin_basis_anti_physicist(small)
        t_cpu_sp = (time.perf_counter() - t0) * (n / 6) ** 4
        cpu = {"value": (t_cpu_tr + t_cpu_sp) * 1e3, "unit": "ms per step", "cores": 1,
               "kind": "port",
               "sample": f"transform: the full {n}-function tensor; spin expansion: 6 orbitals "
                         f"(1296 spin-orbital elements per orbital^4), scaled by (n/6)^4",
               "transform_ms": t_cpu_tr * 1e3, "spin_ms_scaled": t_cpu_sp * 1e3}
    line = {
        "metric": "AO->MO transform + spin-orbital expansion time", "value": ms_tr + ms_sp,
        "unit": "ms per step", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_total / args.steps, "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded water cluster, seeded C)",
        "config": {"workload": f"AO->MO (H2O){args.mo_waters}/6-31G, {n} functions, "
                               f"spin-orbital tensor (2*{n})^4",
                   "l2": "output (2n)^4 doubles far larger than L2"},
        "transform_ms": ms_tr, "transform_form": "pair-packed (tensor symmetric in a<->b, c<->d)",
        "transform_gemm_gflop": flops / 1e9, "transform_tflops": flops / (ms_tr * 1e-3) / 1e12,
        "transform_frac_of_fp64_fma_peak": flops / (ms_tr * 1e-3) / 1e12 / fp64,
        "fp64_fma_peak_tflops": fp64,
        "spin_expand_ms": ms_sp, "spin_expand_ms_per_mode": per_mode,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": None,
                     "kernel": "k_spin_expand (spin_basis_anti_physicist)",
                     "peak_source": peak_kind},
        "cpu_baseline": cpu,
        "e2e": {"value": float(np.mean(e2e)) * 1e3, "unit": "ms per step",
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "clocks": clk.summary(),
        "gpu_launches": args.steps,
        "library_launches_per_step": "4 cuBLAS DGEMM calls (the quarter transforms)",
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------- LDA XC quadrature
def run_xc(args, rank, world):
    """LDA exchange-correlation matrix and energy (Slater + VWN3) of (H2O)n / 6-31G* on the
    reference's grid placement (one spherical grid about the origin; 200 radial x 648
    angular points).  One step = one XC build for a new density matrix with the basis
    values on the grid kept from the first build, as an SCF iteration does: rho (GEMM),
    the functionals (k_lda), V = Phi^T diag(w v) Phi (GEMM), E = sum w rho eps."""
    import torch
    from gaussium_gb300 import build, guess, kohnsham, molecules
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    build.build()
    mol = molecules.water_cluster(args.xc_waters, seed=args.xc_waters)
    sb = molecules.shell_basis(mol, "6-31G*")
    n = sb.nbf
    P = guess.sad_density(mol, "6-31G*")
    xc = kohnsham.ExchangeCorrelationGPU(sb, params=(2 / 3, kohnsham.VWN3))
    st = torch.cuda.current_stream()
    g = xc.points.shape[0]
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    xc.phi()
    e1.record(st)
    e1.synchronize()
    ms_phi = e0.elapsed_time(e1)
    Pd = torch.as_tensor(P).to(xc.device)
    for _ in range(max(3, args.warmup)):
        xc.evaluate_device(Pd)
    torch.cuda.synchronize()
    with ClockSampler() as clk:
        e0.record(st)
        for k in range(args.steps):
            v, e = xc.evaluate_device(Pd * (1.0 + 1e-9 * k))
        e1.record(st)
        e1.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    flops = 2.0 * 2.0 * g * n * n          # Phi P and Phi^T (w v Phi)
    fp64 = fma_peak(64)
    # end to end through the reference surface: host P in, XC matrix and energy back
    e2e = []
    for k in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        V = xc.potential_matrix(P * (1.0 + 1e-9 * (k + 100)))
        E = xc.integrate_energy(P * (1.0 + 1e-9 * (k + 100)))
        if k >= args.warmup:
            e2e.append(time.perf_counter() - t0)
    cpu = None
    if not args.no_cpu_baseline and rank == 0:
        # the oracle's restatement of integrate_potential (kohnsham/integration.py:26-40) on
        # a sample of matrix elements, scaled to the n(n+1)/2 the reference evaluates
        oracle, table = oracle_table(sb)
        sample = 2
        t0 = time.perf_counter()
        for i in range(sample):
            def f(pts, i=i):
                phi = oracle.basis_values(table, pts)
                rho = np.einsum("ga,ab,gb->g", phi, P, phi)
                m = rho > 1e-300
                vv = np.zeros_like(rho)
                vv[m] = oracle._xc_parts(rho[m], 2 / 3, oracle.VWN3)[1]
                return phi[:, i] * vv * phi[:, i]
            oracle.xc_integrate(f)
        per = (time.perf_counter() - t0) / sample
        cpu = {"value": per * n * (n + 1) / 2 * 1e3, "unit": "ms per XC build", "cores": 1,
               "kind": "port",
               "sample": f"{sample} of the {n * (n + 1) // 2} matrix elements (adaptive radial "
                         "quad x degree-35 angular rule, numpy), scaled by the element count"}
    line = {
        "metric": "LDA XC matrix build time", "value": ms, "unit": "ms per XC build",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded water cluster, SAD density)",
        "config": {"workload": f"LDA (Slater + VWN3) XC, (H2O){args.xc_waters}/6-31G*, {n} "
                               f"functions, {g} grid points about the origin",
                   "l2": f"basis values on the grid {g * n * 8 / 1e6:.0f} MB"},
        "basis_on_grid_ms": ms_phi,
        "basis_on_grid_gbs_written": g * n * 8 / (ms_phi * 1e-3) / 1e9,
        "roofline": {"bound": "tensor", "achieved": flops / (ms * 1e-3) / 1e12, "peak": fp64,
                     "unit": "TFLOP/s", "frac": flops / (ms * 1e-3) / 1e12 / fp64,
                     "traffic": None, "kernel": "cuBLAS DGEMM (rho and V contractions)",
                     "peak_source": "FP64 FMA probe (gs_fma_probe) in this process"},
        "cpu_baseline": cpu,
        "e2e": {"value": float(np.mean(e2e)) * 1e3, "unit": "ms per XC build",
                "h2d_bytes_per_step": n * n * 8, "d2h_bytes_per_step": n * n * 8 + 8},
        "clocks": clk.summary(),
        "gpu_launches": args.steps,
        "energy": float(e.item()),
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------- reference arm
def run_reference(args, rank, world):
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_oracle_rate(32, args.seed, threads)
    vals = []
    t_all = time.perf_counter()
    for k in range(args.steps):
        rate, dt, nf = cpu_oracle_rate(args.cpu_sample // 4, args.seed + k, threads)
        vals.append(rate)
    wall = time.perf_counter() - t_all
    v = float(np.mean(vals))
    line = {
        "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": wall * 1e3 / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
        "config": {"workload": WORKLOAD, "quartets_per_gpu": args.quartets},
        "impl": "reference",
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{args.cpu_sample // 4} seeded shell quartets per step, "
                                   "oracle C restatement of the reference's Obara-Saika "
                                   "recursion with memoised recursion nodes (bit-identical "
                                   "results; faster than the reference's unmemoised Python "
                                   "recursion, so the GPU ratio against it understates the "
                                   "speed-up over the reference itself)",
                         "memoised": True},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    rank, world = dist_init(args)
    if args.impl == "reference":
        run_reference(args, rank, world)
    elif args.workload == "water":
        run_water(args, rank, world)
    elif args.workload == "batch":
        run_batch(args, rank, world)
    elif args.workload == "gradient":
        run_gradient(args, rank, world)
    elif args.workload == "optimize":
        run_optimize(args, rank, world)
    elif args.workload == "mo":
        run_mo(args, rank, world)
    elif args.workload == "xc":
        run_xc(args, rank, world)
    else:
        run_gpu(args, rank, world)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
