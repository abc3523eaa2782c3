"""Host side of the point-group screen (no GPU): the tables the drop-in reads from the
reference's Symmetry object, checked against the oracle's restatement on the reference's
own outputs (tests/golden/symmetry.npz)."""
import types

import numpy as np

import oracle
from conftest import golden
from gaussium_gb300 import dropin

PARITIES = [(p & 1, (p >> 1) & 1, (p >> 2) & 1) for p in range(8)]


def fake_reference_symmetry(g, name):
    """An object shaped like the reference's Symmetry (common/symmetry.py:10-16): an object
    symmetry_matrix with a label row and identity column, and int_operate_dict, rebuilt
    from the golden tables; plus duck-typed basis functions with coordinates/exponents."""
    table, flip = g[f"{name}_table"], g[f"{name}_flip"]
    n, nops = table.shape
    sm = np.empty((n + 1, nops + 1), dtype=object)
    sm[0, 0] = "E"
    for m in range(nops):
        sm[0, m + 1] = f"op{m + 1}"
    for f in range(n):
        sm[f + 1, 0] = f + 1
        for m in range(nops):
            sm[f + 1, m + 1] = int(table[f, m])
    ops = {}
    for m in range(nops):
        for p in range(8):
            # any tuple that differs from p exactly when the operation flips it
            ops[(m + 1, PARITIES[p])] = tuple(-x for x in PARITIES[p]) if flip[m, p] \
                else PARITIES[p]
            if flip[m, p] and PARITIES[p] == (0, 0, 0):
                ops[(m + 1, PARITIES[p])] = (9, 9, 9)
    funcs = [types.SimpleNamespace(coordinates=tuple(c), integral_exponents=tuple(int(x) for x in l))
             for c, l in zip(g[f"{name}_centre"], g[f"{name}_lmn"])]
    sym = types.SimpleNamespace(symmetry_matrix=sm, int_operate_dict=ops,
                                point_group=types.SimpleNamespace(label=str(g[f"{name}_label"])))
    return sym, funcs


def test_tables_from_reference_object_give_reference_screen():
    g = golden("symmetry")
    for name in ("ethene", "water", "o2"):
        sym, funcs = fake_reference_symmetry(g, name)
        table, flip, cid, par = dropin.symmetry_tables(sym, funcs)
        assert np.array_equal(table, g[f"{name}_table"])
        assert np.array_equal(flip.astype(bool), g[f"{name}_flip"])
        keys, ref = oracle.canonical_keys(g[f"{name}_table"].shape[0]), g[f"{name}_nonzero"]
        pick = np.random.default_rng(1).choice(len(keys), min(2000, len(keys)), replace=False)
        got = [oracle.symmetry_nonzero(table, flip.astype(bool), cid, par, keys[t]) for t in pick]
        assert np.array_equal(got, ref[pick]), name


def test_objects_without_tables_use_the_per_key_path():
    class Mock:                       # like the reference's MagicMock symmetry double
        def __getattr__(self, name):
            return Mock()
    assert dropin.symmetry_tables(Mock(), [object()] * 3) is None
    assert dropin.symmetry_tables(types.SimpleNamespace(), [object()]) is None
