"""Generate ``xc.npz`` by running the reference's exchange-correlation code here.

Run from this directory:  ``python make_xc_golden.py``.  It needs the reference source tree
(the GAUSSIUM_REFERENCE environment variable); it writes only ``xc.npz`` beside itself.  Contents:

* ``density``: densities from 1e-14 to 1e3 and exactly 0, and at each of them the
  reference's ``SlaterExchange(alpha).energy/potential`` for alpha = 2/3 and 0.7
  (``kohnsham/exchange/slater_exchange.py``) and ``VoskoWilkNusair.energy/potential``
  with the VWN3 and VWN5 parameters that ``kohnsham/kohn_sham.py:21-28`` passes
  (``kohnsham/correlation/local_density.py``).
* ``points``, ``pmat``, ``rho``: ``ExchangeCorrelation.electron_density``
  (``kohnsham/integration.py:14-24``) of the water/STO-3G functions of ``h2o_sto3g.npz``
  (rebuilt from the same reference readers as make_golden.py) for a seeded symmetric
  density matrix at seeded points.
* ``he_energy_s``, ``he_energy_svwn3``: the reference's own expected DFT energies of He
  in STO-3G, copied from its test file ``tests/testslow/start/test_start.py:50-61``
  (checked there to 6 significant figures).  The reference cannot produce them here: its
  angular rule comes from ``quadpy``, which is not installed.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import ref_harness  # noqa: E402
import make_golden  # noqa: E402


def main():
    ref_harness.load()
    from gaussium.kohnsham.exchange import SlaterExchange
    from gaussium.kohnsham.correlation import VoskoWilkNusair
    from gaussium.kohnsham.integration import ExchangeCorrelation
    density = np.concatenate([[0.0], np.logspace(-14, 3, 69)])
    out = {"density": density}
    for tag, alpha in (("s", 2 / 3), ("xa", 0.7)):
        x = SlaterExchange(alpha)
        out[f"slater_{tag}_energy"] = np.array([x.energy(d) for d in density])
        out[f"slater_{tag}_potential"] = np.array([x.potential(d) for d in density])
    for tag, prm in (("vwn3", (0.0621814, -0.409286, 13.0720, 42.7198)),
                     ("vwn5", (0.0621814, -0.10498, 3.72744, 12.9352))):
        c = VoskoWilkNusair(*prm)
        out[f"{tag}_energy"] = np.array([float(c.energy(d)) for d in density])
        out[f"{tag}_potential"] = np.array([float(c.potential(d)) for d in density])

    mol = make_golden.write_tmp("water.mol", make_golden.water_mol_text())
    gbs = os.path.join(make_golden.ref_harness.reference_root(), "tests", "testslow", "start", "STO-3G.gbs")
    _, _, _, basis = make_golden.load_molecule(mol, gbs)
    n = len(basis)
    rng = np.random.default_rng(31)
    a = rng.standard_normal((n, n)) * 0.3
    pmat = a @ a.T
    points = rng.uniform(-3.0, 3.0, size=(24, 3))
    xc = ExchangeCorrelation(basis, None, None)
    rho = np.array([xc.electron_density(np.asarray(pmat), *p) for p in points])
    out.update(points=points, pmat=pmat, rho=rho,
               he_energy_s=np.float64(-2.657311972), he_energy_svwn3=np.float64(-2.809598595))
    np.savez_compressed(os.path.join(HERE, "xc.npz"), **out)


if __name__ == "__main__":
    main()
