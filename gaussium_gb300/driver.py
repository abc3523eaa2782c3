"""End-to-end RHF on the device engine: the call path of the reference's
``Energy.calculate_energy`` -> ``RestrictedHF`` (energy/energy.py:24-81,
hartreefock/hartree_fock.py:20-84) with the ERI tensor replaced by the integral-direct
Fock builder.  Records the wall time of every Fock build (CUDA-synchronised)."""
import time

import torch

from . import scf
from .engine import JKEngine
from .fock import FockMatrixRestrictedGPU
from .hamiltonian import one_electron
from .molecules import shell_basis


class TimedFock(FockMatrixRestrictedGPU):
    def create(self, density_matrix):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        f = super().create(density_matrix)
        torch.cuda.synchronize()
        self.builds.append(time.perf_counter() - t0)
        return f


def rhf(mol, basis="6-31G*", schwarz_thr=1e-12, mixed_cut=None, screen_thr=0.0,
        incremental=False, reset_every=8, threshold=1e-10, max_iter=100, engine=None,
        final_fp64=False):
    """RHF total energy of ``mol``.  Returns a dict with the energy, iteration count,
    per-build Fock times and the engine (reusable across calls on the same geometry).
    ``final_fp64`` re-evaluates the converged density's Fock matrix with a full FP64 build
    for the reported energy (the mixed/incremental builds only steer the iterations)."""
    sb = engine.sb if engine is not None else shell_basis(mol, basis)
    t0 = time.perf_counter()
    S, T, V = one_electron(sb, mol.coords, mol.charges)
    hcore = T + V
    t1 = time.perf_counter()
    if engine is None:
        engine = JKEngine(sb, schwarz_thr=schwarz_thr)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    fb = TimedFock(hcore, engine, screen_thr=screen_thr, mixed_cut=mixed_cut,
                   incremental=incremental, reset_every=reset_every)
    res = scf.restricted_scf(S, hcore, mol.electrons, fb, threshold=threshold, max_iter=max_iter)
    e_el = res.energy
    if final_fp64:
        fin = TimedFock(hcore, engine)
        f = fin.create(res.density)
        e_el = scf.total_energy_restricted(hcore, res.density, f)
        fb.builds.extend(fin.builds)
    e_nuc = mol.nuclear_repulsion()
    return dict(energy=e_el + e_nuc, electronic=e_el, iterations=res.iterations,
                converged=res.converged, fock_seconds=list(fb.builds), one_electron_s=t1 - t0,
                setup_s=t2 - t1, nbf=sb.nbf, ntasks=engine.ntasks, engine=engine,
                density=res.density, scf_energy=res.energy + e_nuc)
