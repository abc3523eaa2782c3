"""Generate ``scf_parts.npz``: the reference's own SCF host functions run on the HeH+
STO-3G inputs of its unit tests, as fixtures for the restated ``gaussium_gb300.scf``.

Run from this directory:  ``python make_scf_parts.py``.  It needs the reference source
tree (the GAUSSIUM_REFERENCE environment variable, read by ``ref_harness``) and writes
only ``scf_parts.npz`` beside itself.  The CPU tests read that file, never the reference.

Inputs, as the reference's tests give them (file:line within the reference project):

* ``P``, ``H``, ``F``  tests/testsfast/hartreefock/test_total_energy.py:10-23
* ``S``               tests/testsfast/hartreefock/test_linear_algebra.py:12
* ``C``               tests/testsfast/matrixelements/test_density_matrix.py:10-13
  (``H`` is also the matrix test_linear_algebra.py:23 diagonalises)

Outputs, from running the reference:

* ``energy``      ``TotalEnergy(H).restricted(P, F)``       hartreefock/total_energy.py:16-35
* ``X``           ``LinearAlgebra(S).transformation_matrix``  hartreefock/linear_algebra.py:6-25
* ``eps``, ``Cd`` ``LinearAlgebra(S).diagonalize(H)``          linear_algebra.py:9-16, with the
                  transformation matrix made from ``S`` (the reference's test substitutes a
                  rounded copy of it)
* ``D``           ``density_matrix_restricted(C, 2)``         matrixelements/density_matrix.py:4-9
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import ref_harness  # noqa: E402


def main():
    ref_harness.load()
    from gaussium.hartreefock import LinearAlgebra, TotalEnergy
    from gaussium.matrixelements import density_matrix_restricted
    P = np.array([[1.7266, 0.2599], [0.2599, 0.0391]])
    H = np.array([[-2.6527, -1.3472], [-1.3472, -1.7318]])
    F = np.array([[-1.3904, -0.9732], [-0.9732, -0.7429]])
    S = np.array([[1.0, 0.4508], [0.4508, 1.0]])
    C = np.array([[0.9291, -0.6259], [0.1398, 1.1115]])
    energy = float(TotalEnergy(H).restricted(P, F))
    la = LinearAlgebra(S)
    X = np.asarray(la.transformation_matrix, dtype=np.float64)
    eps, Cd = la.diagonalize(H)
    D = np.asarray(density_matrix_restricted(C, 2), dtype=np.float64)
    out = os.path.join(HERE, "scf_parts.npz")
    np.savez(out, P=P, H=H, F=F, S=S, C=C, energy=energy, X=X,
             eps=np.asarray(eps, dtype=np.float64), Cd=np.asarray(Cd, dtype=np.float64), D=D)
    print("wrote", out, "energy", energy)


if __name__ == "__main__":
    main()
