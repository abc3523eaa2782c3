"""Per-class kernel-form autotuner.

A class (la lb|lc ld) whose total angular momentum lies in the overlap of the kernel
families is built as the one-thread-per-quartet kernel, as the warp-per-quartet kernel,
where its narrow recursion levels leave lanes idle as the warp kernel that pushes several
primitive quartets through each pass, and as the stacked warp kernel whose lanes each run
their node record on several primitive quartets (``gs_class_variants``).  Which is faster
depends on the workload, chiefly on the primitive counts of the quartets and on how much
shared memory the grouped buffers take from occupancy.  The
tuner times both forms of every such class on the caller's own task lists (CUDA events on
the launching stream, after a warm-up launch, median of ``reps``) and selects the faster
with ``gs_set_class_variant``; then, for every class, it times the class with and without
its heavy form (split or cooperative, for the quartets with many primitive quartets) and
keeps the faster.  The choices are process-wide and stay until changed.
"""
import json

import torch

from . import _lib

THREAD, WARP, GROUPED, SPLIT, COOP, STACKED = 1, 2, 3, 4, 5, 6
NAMES = {THREAD: "thread", WARP: "warp", GROUPED: "warp-grouped", SPLIT: "thread-split",
         COOP: "warp-cooperative", STACKED: "warp-stacked"}


def forms(cls, precision):
    """Kernel forms built for a class: a subset of {THREAD, WARP, GROUPED, STACKED}."""
    m = _lib.lib().gs_class_variants(*cls, precision)
    if m < 0:
        _lib.check(-m, f"gs_class_variants{cls}")
    # the split and cooperative forms serve the heavy quartets of a thread-form or warp-form
    # class (engine.split_forms); as whole-class forms they would leave most lanes idle on
    # light quartets
    return [v for v in (THREAD, WARP, GROUPED, STACKED) if m & (1 << (v - 1))]


def describe(row):
    """Name of a tuned class's forms: its form, with the heavy form where the tuner kept
    its heavy quartets in the split or cooperative form."""
    name = NAMES[row["form"]]
    if row.get("heavy_form"):
        name += "+split" if row["form"] == THREAD else "+cooperative"
    return name


def set_form(cls, precision, variant):
    _lib.check(_lib.lib().gs_set_class_variant(*cls, precision, variant),
               f"gs_set_class_variant{cls}")


def _time(fn, reps):
    st = torch.cuda.current_stream()
    fn()                                         # warm-up
    out = []
    for _ in range(reps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(st)
        fn()
        b.record(st)
        b.synchronize()
        out.append(a.elapsed_time(b))
    out.sort()
    return out[len(out) // 2]


def tune(segments, run_class, precisions=(64, 32), reps=3, min_tasks=1):
    """Choose the faster form for every class of ``segments`` ([(cls, start, end)]) that
    has two; ``run_class(cls, precision)`` launches that class's work once on the current
    stream.  Returns {(cls, precision): {"form": v, "ms": {v: t}}}."""
    chosen = {}
    from . import engine
    for prec in precisions:
        for cls, s, e in segments:
            if e - s < min_tasks:
                continue
            fs = forms(cls, prec)
            times = {}
            if len(fs) >= 2:
                for v in fs:
                    set_form(cls, prec, v)
                    times[v] = _time(lambda: run_class(cls, prec), reps)
                best = min(times, key=times.get)
                set_form(cls, prec, best)
                t_best = times[best]
            else:
                best = fs[0]
                t_best = _time(lambda: run_class(cls, prec), reps)
            row = {"form": best, "ms": times}
            # the class's heavy quartets run in the split form (thread form) or the
            # cooperative form (warp forms); keep that only where it measures faster than
            # leaving them on the class's own form
            engine.SPLIT_OFF.add((cls, prec))
            off = _time(lambda: run_class(cls, prec), reps)
            engine.SPLIT_OFF.discard((cls, prec))
            row["heavy_form"] = off >= t_best
            row["ms_without_heavy_form"] = off
            if not row["heavy_form"]:
                engine.SPLIT_OFF.add((cls, prec))
            chosen[(cls, prec)] = row
    return chosen


def tune_jk(engine, density, precisions=(64, 32), reps=3):
    """Tune the J/K class launches of a JKEngine on its task list with one density."""
    P = density if torch.is_tensor(density) else torch.as_tensor(density).to(engine.dev)
    return tune(engine.segments, lambda cls, prec: engine.jk(P, [P], precision=prec, classes=[cls]),
                precisions, reps)


def tune_blocks(batch, out, precisions=(64, 32), reps=3):
    """Tune the integral-block class launches of a QuartetBatch writing into ``out``."""
    return tune(batch.segments, lambda cls, prec: batch.run(out, prec, classes=[cls]),
                precisions, reps)


def grad_forms(cls):
    """Kernel forms built for a gradient class: a subset of {THREAD, WARP}."""
    m = _lib.lib().gs_eri_grad_variants(*cls)
    if m < 0:
        _lib.check(-m, f"gs_eri_grad_variants{cls}")
    return [v for v in (THREAD, WARP) if m & (1 << (v - 1))]


def set_grad_form(cls, variant):
    _lib.check(_lib.lib().gs_set_eri_grad_variant(*cls, variant), f"gs_set_eri_grad_variant{cls}")


def tune_gradient(segments, run_class, reps=3):
    """Choose the faster form of every gradient class of ``segments`` that has two;
    ``run_class(cls)`` launches that class's gradient work once.  Returns {cls: {...}}."""
    chosen = {}
    for cls, s, e in segments:
        fs = grad_forms(cls)
        if e <= s or len(fs) < 2:
            continue
        times = {}
        for v in fs:
            set_grad_form(cls, v)
            times[v] = _time(lambda: run_class(cls), reps)
        best = min(times, key=times.get)
        set_grad_form(cls, best)
        chosen[cls] = {"form": best, "ms": times}
    return chosen


def reset(segments, precisions=(64, 32)):
    """Back to the built-in default form for every class of ``segments`` (heavy quartets
    in the split or cooperative form again)."""
    from . import engine
    for prec in precisions:
        for cls, _, _ in segments:
            set_form(cls, prec, 0)
            engine.SPLIT_OFF.discard((cls, prec))


def save(chosen, path):
    rows = [{"class": list(cls), "precision": prec, "form": r["form"],
             "heavy_form": r.get("heavy_form", True),
             "ms": {str(k): v for k, v in r["ms"].items()}} for (cls, prec), r in chosen.items()]
    with open(path, "w") as f:
        json.dump(rows, f, indent=1)


def load(path):
    """Apply a saved choice (form and heavy form of every class); returns it in the form
    ``tune`` returns."""
    from . import engine
    with open(path) as f:
        rows = json.load(f)
    chosen = {}
    for r in rows:
        cls, prec = tuple(r["class"]), r["precision"]
        set_form(cls, prec, r["form"])
        heavy = r.get("heavy_form", True)
        if heavy:
            engine.SPLIT_OFF.discard((cls, prec))
        else:
            engine.SPLIT_OFF.add((cls, prec))
        chosen[(cls, prec)] = {"form": r["form"], "heavy_form": heavy,
                               "ms": {int(k): v for k, v in r["ms"].items()}}
    return chosen


def tune_or_load(path, tune_fn):
    """The saved choice at ``path`` if the file exists, else ``tune_fn()`` saved there
    (None: always tune).  A run under a profiler, whose per-launch overheads would change
    the choices, loads what a plain run of the same command chose."""
    import os
    if path and os.path.exists(path):
        return load(path)
    chosen = tune_fn()
    if path:
        save(chosen, path)
    return chosen
