"""Import the reference Gaussium package in this container, with import-time shims only.

Test infrastructure, used solely by ``make_golden.py`` to produce the committed golden
vectors under ``tests/golden/``.  The reference source tree is read in place and never
written to (``sys.dont_write_bytecode``).  Nothing on the product path imports this file,
and the GPU tests run without the reference tree.

Shims (none of them changes the reference's arithmetic on the ERI path):

1. ``quadpy`` is absent; ``gaussium/kohnsham/integration.py:4`` imports it at package
   import time although only DFT exchange-correlation uses it.  An empty module stands in.
2. numpy 2 removed ``ndarray.itemset``.  The call sites (``create_matrix.py:34``,
   ``electron_repulsion_matrix.py:45``, ``symmetry.py:101-110``, ``diis.py:95-103``) get a
   module-level ``np`` proxy whose ``zeros``/``empty`` return an ndarray subclass with
   ``itemset``.
3. scipy >= 1.11 returns ``factorial2(-1) == 0``; the reference relies on the old value 1
   (``primitive_basis_function.py:26-42``, ``basis_function.py:22-53``,
   ``orbital_overlap_integral.py:9-13``).  Those modules get ``factorial2(n<=0) = 1``.
4. ``numpy.linalg.linalg.LinAlgError`` is looked up by ``diis.py:108``; numpy 2 keeps it
   only in ``numpy.linalg``.
"""
import os
import sys
import types


def reference_root():
    """Root of the reference source tree, from the GAUSSIUM_REFERENCE environment variable
    (the directory holding ``src/gaussium`` and ``examples/``).  There is no default."""
    root = os.environ.get("GAUSSIUM_REFERENCE")
    if not root or not os.path.isdir(os.path.join(root, "src", "gaussium")):
        raise RuntimeError("set GAUSSIUM_REFERENCE to the reference Gaussium source tree "
                           "(the directory with src/gaussium and examples/)")
    return root


_loaded = None


import numpy as _np


class ItemsetArray(_np.ndarray):
    """ndarray with the ``itemset`` method numpy 2 removed (module level so it pickles
    into the reference's multiprocessing workers)."""

    def itemset(self, *args):
        if len(args) != 2:
            raise TypeError("itemset expects (index, value)")
        index, value = args
        self[index] = value


def _make_np_proxy(np):
    class NpProxy(types.ModuleType):
        def __getattr__(self, name):
            return getattr(np, name)

    proxy = NpProxy("numpy_itemset_proxy")
    proxy.zeros = lambda *a, **k: np.zeros(*a, **k).view(ItemsetArray)
    proxy.empty = lambda *a, **k: np.empty(*a, **k).view(ItemsetArray)
    return proxy


def load():
    """Return the imported ``gaussium`` package with the shims applied."""
    global _loaded
    if _loaded is not None:
        return _loaded
    sys.dont_write_bytecode = True
    import numpy as np
    import scipy.special

    if "quadpy" not in sys.modules:
        sys.modules["quadpy"] = types.ModuleType("quadpy")
    if not hasattr(np.linalg, "linalg"):
        np.linalg.linalg = types.SimpleNamespace(LinAlgError=np.linalg.LinAlgError)
    elif not hasattr(np.linalg.linalg, "LinAlgError"):
        np.linalg.linalg.LinAlgError = np.linalg.LinAlgError
    src = os.path.join(reference_root(), "src")
    if src not in sys.path:
        sys.path.insert(0, src)
    import gaussium  # noqa: F401

    proxy = _make_np_proxy(np)
    import gaussium.matrixelements.create_matrix as m1
    import gaussium.matrixelements.electron_repulsion_matrix as m2
    import gaussium.common.symmetry as m3
    import gaussium.diismethod.diis as m4
    for mod in (m1, m2, m3, m4):
        mod.np = proxy

    def factorial2(n):
        if n <= 0:
            return 1.0
        return float(scipy.special.factorial2(n))

    import gaussium.objects.primitive_basis_function as o1
    import gaussium.objects.basis_function as o2
    import gaussium.integrals.orbital_overlap_integral as o3
    for mod in (o1, o2, o3):
        mod.factorial2 = factorial2

    _loaded = gaussium
    return gaussium


def c1_symmetry(basis_set):
    """A C1 ``Symmetry`` object as ``Energy.__init__`` builds it (``energy/energy.py:21``)."""
    g = load()
    from gaussium.objects import PointGroup
    from gaussium.common import Symmetry
    return Symmetry(PointGroup([], [], [], [], 'C_{1}'), basis_set)
