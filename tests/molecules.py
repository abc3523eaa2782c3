"""Test helper: reference-ordered functions of the golden molecules as duck-typed objects
(the attributes the reference's integral code reads), and oracle tables for them."""
from types import SimpleNamespace

import numpy as np

import oracle
from conftest import golden


def functions(g):
    out = []
    for i in range(len(g["norm"])):
        k = int(g["nprim"][i])
        c = tuple(float(x) for x in g["centre"][i])
        prims = [SimpleNamespace(contraction=float(g["coef"][i, j]), exponent=float(g["expo"][i, j]),
                                 normalisation=float(g["pnorm"][i, j]), coordinates=c,
                                 integral_exponents=tuple(int(x) for x in g["lmn"][i]))
                 for j in range(k)]
        out.append(SimpleNamespace(primitive_gaussian_array=prims, coordinates=c,
                                   integral_exponents=tuple(int(x) for x in g["lmn"][i]),
                                   normalisation=float(g["norm"][i])))
    return out


def load(name):
    g = golden(name)
    return g, functions(g), oracle.FunctionTable.from_arrays(g)


def random_density(n, seed):
    rng = np.random.default_rng(seed)
    a = rng.standard_normal((n, n))
    return (a + a.T) / 4
