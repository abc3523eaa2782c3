"""The autotuner's choice logic with the library calls replaced by fakes (no GPU): every
class with several forms is timed in each and left on its fastest; every class is then
timed with and without its heavy form (split or cooperative) and keeps the faster; empty
segments are skipped."""

from gaussium_gb300 import autotune


def test_tune_picks_fastest_form(monkeypatch):
    from gaussium_gb300 import engine
    built = {(2, 1, 0, 0): [1, 2, 3], (1, 0, 0, 0): [1], (2, 2, 2, 2): [2, 3]}
    cost = {((2, 1, 0, 0), 1): 3.0, ((2, 1, 0, 0), 2): 2.0, ((2, 1, 0, 0), 3): 1.0,
            ((1, 0, 0, 0), 1): 1.0, ((2, 2, 2, 2), 2): 1.0, ((2, 2, 2, 2), 3): 5.0}
    # time without the heavy form: slower for (2,1,0,0), faster for (1,0,0,0)
    off_cost = {(2, 1, 0, 0): 1.5, (1, 0, 0, 0): 0.5}
    state = {}
    monkeypatch.setattr(autotune, "forms", lambda cls, prec: built[cls])
    monkeypatch.setattr(autotune, "set_form", lambda cls, prec, v: state.__setitem__((cls, prec), v))
    monkeypatch.setattr(engine, "SPLIT_OFF", set())
    current = {}

    def run_class(cls, prec):
        if (cls, prec) in engine.SPLIT_OFF:
            current["t"] = off_cost[cls]
        else:
            current["t"] = cost[(cls, state.get((cls, prec), built[cls][0]))]

    monkeypatch.setattr(autotune, "_time", lambda fn, reps: (fn(), current["t"])[1])
    segs = [((2, 1, 0, 0), 0, 10), ((1, 0, 0, 0), 10, 20), ((2, 2, 2, 2), 20, 20)]
    chosen = autotune.tune(segs, run_class, precisions=(64,), reps=1)
    assert chosen[((2, 1, 0, 0), 64)]["form"] == 3
    assert state[((2, 1, 0, 0), 64)] == 3
    assert chosen[((2, 1, 0, 0), 64)]["heavy_form"] is True
    assert ((2, 1, 0, 0), 64) not in engine.SPLIT_OFF
    assert chosen[((1, 0, 0, 0), 64)]["form"] == 1           # one form: heavy choice only
    assert chosen[((1, 0, 0, 0), 64)]["heavy_form"] is False
    assert ((1, 0, 0, 0), 64) in engine.SPLIT_OFF
    assert autotune.describe(chosen[((2, 1, 0, 0), 64)]) == "warp-grouped+cooperative"
    assert autotune.describe(chosen[((1, 0, 0, 0), 64)]) == "thread"
    assert ((2, 2, 2, 2), 64) not in chosen          # empty segment (min_tasks)


def test_vrr_group_choice():
    """Classes whose node program fills a warp's waves poorly get a grouped form, whose
    waves of 32/VG nodes times VG primitive quartets fill the lanes; the grouped buffers
    stay within the budget; (dd|dd)'s ungrouped waves are already 94 % full."""
    import os
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                                    "gaussium_gb300", "csrc"))
    import gen_eri
    vg, prog = gen_eri.vrr_group((2, 1, 0, 0))
    base = gen_eri.wide_program((2, 1, 0, 0))
    assert vg > 1
    assert (gen_eri.wave_efficiency(prog["vrec"], prog["vseg"], vg) >
            gen_eri.wave_efficiency(base["vrec"], base["vseg"]) + 0.3)
    # waves of 32 // vg records share a term count (the kernel reads it per record)
    rec = prog["vrec"]
    for noff, _, cnt, _, _, _ in prog["vseg"]:
        for w0 in range(0, cnt, 32 // vg):
            nts = {rec[8 * (noff + n)] >> 16 for n in range(w0, min(cnt, w0 + 32 // vg))}
            assert len(nts) == 1
    for cls in ((2, 2, 2, 1), (2, 2, 2, 2)):
        vg, prog = gen_eri.vrr_group(cls)
        assert vg * prog["nvslot"] <= gen_eri.VGROUP_SLOT_BUDGET
    base = gen_eri.wide_program((2, 2, 2, 2))
    assert gen_eri.wave_efficiency(base["vrec"], base["vseg"]) > 0.94


def test_tune_or_load_round_trip(monkeypatch, tmp_path):
    """A saved choice (form and heavy form per class) is re-applied by tune_or_load without
    tuning again; without a path it always tunes."""
    from gaussium_gb300 import engine
    state = {}
    monkeypatch.setattr(autotune, "set_form", lambda cls, prec, v: state.__setitem__((cls, prec), v))
    monkeypatch.setattr(engine, "SPLIT_OFF", set())
    chosen = {((2, 1, 0, 0), 64): {"form": 3, "heavy_form": True, "ms": {3: 1.0}},
              ((1, 0, 0, 0), 32): {"form": 1, "heavy_form": False, "ms": {}}}
    calls = []

    def tune():
        calls.append(1)
        return chosen

    path = str(tmp_path / "forms.json")
    assert autotune.tune_or_load(path, tune) == chosen and len(calls) == 1
    state.clear()
    engine.SPLIT_OFF.clear()
    again = autotune.tune_or_load(path, tune)
    assert len(calls) == 1                                   # loaded, not tuned
    assert state == {((2, 1, 0, 0), 64): 3, ((1, 0, 0, 0), 32): 1}
    assert engine.SPLIT_OFF == {((1, 0, 0, 0), 32)}
    assert again[((2, 1, 0, 0), 64)]["heavy_form"] is True
    autotune.tune_or_load(None, tune)
    assert len(calls) == 2
