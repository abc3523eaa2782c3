"""Host packing: reference functions -> shells, normalisation folding, canonical orders."""
from types import SimpleNamespace as NS

import numpy as np
import pytest

import oracle
from conftest import golden, synthetic_shells
from molecules import functions
from gaussium_gb300.basis import ShellBasis, Basis, PrimitiveBasis
from gaussium_gb300.engine import canonicalize


def test_grouping_of_water_631gs():
    g = golden("h2o_631gs")
    sb = ShellBasis.from_functions(functions(g))
    assert sb.nbf == 19
    assert list(sb.l) == [0, 0, 1, 0, 1, 2, 0, 0, 0, 0]
    # the effective coefficients reproduce every function's c*N_prim*N_contr
    for s in range(sb.nshell):
        for ci in range(len(sb.comp_scale[s]) if sb.l[s] == 2 else 1):
            f = sb.func_off[s] + ci
            k0, k1 = sb.prim_off[s], sb.prim_off[s + 1]
            want = g["coef"][f, :k1 - k0] * g["pnorm"][f, :k1 - k0] * g["norm"][f]
            np.testing.assert_allclose(sb.coef[k0:k1] * sb.comp_scale[s, ci], want, rtol=1e-14)


def test_normalisation_matches_reference_objects():
    g = golden("synthetic")
    sb = ShellBasis.from_shell_dicts(synthetic_shells())
    # d shells: component scale is sqrt(3) for xy, xz, yz relative to xx
    d = np.flatnonzero(sb.l == 2)
    np.testing.assert_allclose(sb.comp_scale[d][:, 3:], np.sqrt(3.0), rtol=1e-13)
    np.testing.assert_allclose(sb.comp_scale[d][:, :3], 1.0, rtol=1e-13)
    b = Basis([PrimitiveBasis(c, e, (0, 0, 0), (1, 1, 0)) for c, e in ((0.3, 1.2), (0.7, 0.4))],
              (0, 0, 0), (1, 1, 0))
    t = oracle.FunctionTable.from_shells([dict(l=2, centre=np.zeros(3), expo=[1.2, 0.4], coef=[0.3, 0.7])])
    assert abs(b.normalisation - t.cnorm[3]) < 1e-14 * t.cnorm[3]


def test_rejects_non_reference_component_order():
    c = (0.0, 0.0, 0.0)
    f = [NS(primitive_gaussian_array=[NS(contraction=1.0, exponent=1.0, normalisation=1.0)],
            coordinates=c, integral_exponents=lmn, normalisation=1.0)
         for lmn in ((0, 1, 0), (1, 0, 0), (0, 0, 1))]
    with pytest.raises(ValueError):
        ShellBasis.from_functions(f)


def test_canonicalize_codes():
    l4 = np.array([[0, 1, 2, 2], [2, 2, 0, 1], [1, 0, 0, 0], [0, 0, 2, 1]])
    pos, code, pcb, pck = canonicalize(l4)
    for row, p, c in zip(l4, pos, code):
        canon = row[p]
        assert canon[0] >= canon[1] and canon[2] >= canon[3]
    assert list(code) == [6, 2, 0, 4]
