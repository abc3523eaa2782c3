"""Generate ``mo_transform.npz`` by running the reference's transformations here.

Run from this directory:  ``python make_mo_golden.py``.  It needs the reference source tree
(the GAUSSIUM_REFERENCE environment variable) and ``h2o_sto3g.npz`` (the water/STO-3G dense tensor written
by make_golden.py); it writes only ``mo_transform.npz`` beside itself.  Contents: a seeded
orthogonal coefficient matrix C and the reference outputs of
``matrixelements/transformations.py``: ``molecular_orbitals`` (lines 5-26),
``blocked_spin_basis_set`` (29-70), ``spin_basis_set`` (73-92) and
``spin_basis_anti_physicist`` (114-136), the last three applied to the MO tensor.  The
module's ``np`` gets the harness's numpy-2 ``itemset`` shim (ref_harness.py), nothing else.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import ref_harness  # noqa: E402


def main():
    ref_harness.load()
    from gaussium.matrixelements import transformations as tr
    # the same numpy-2 shim the harness applies elsewhere: zeros() arrays with itemset
    tr.np = ref_harness._make_np_proxy(np)
    dense = np.load(os.path.join(HERE, "h2o_sto3g.npz"))["dense"]
    n = dense.shape[0]
    rng = np.random.default_rng(21)
    c, _ = np.linalg.qr(rng.standard_normal((n, n)))
    ao = dense.copy().view(ref_harness.ItemsetArray)
    mo = np.asarray(tr.molecular_orbitals(ao, c)).copy()
    mo_it = mo.copy().view(ref_harness.ItemsetArray)
    spin = np.asarray(tr.spin_basis_set(mo_it))
    blocked = np.asarray(tr.blocked_spin_basis_set(mo_it))
    anti = np.asarray(tr.spin_basis_anti_physicist(mo_it))
    np.savez_compressed(os.path.join(HERE, "mo_transform.npz"), coefficients=c, ao=dense, mo=mo,
                        spin=spin, blocked=blocked, anti=anti)


if __name__ == "__main__":
    main()
