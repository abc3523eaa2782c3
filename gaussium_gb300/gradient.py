"""Analytic RHF nuclear gradients (new: the reference optimises geometries with
Nelder-Mead on energies, geometryoptimization/nelder_mead.py:28-144).

dE/dR = sum P dH/dR - sum W dS/dR + sum Gamma d(ab|cd)/dR + dE_nuc/dR, with
W = 2 sum_occ e_k C_k C_k^T and Gamma_abcd = 1/2 P_ab P_cd - 1/8 (P_ac P_bd + P_ad P_bc).

Derivative integrals come from "raised" shells (l+1, primitive coefficients times
2 alpha, unit component scales) and "lowered" shells (l-1):
    d phi_a / dA_x = 2 alpha phi_{a+1x} - a_x phi_{a-1x},
evaluated by the same one-electron and ERI class kernels as the energy; the ERI part is
contracted with Gamma by the adjoint kernel gs_eri_grad_contract.  The nuclear-attraction
operator derivative uses translational invariance per nucleus.

``EnergyGradient`` wraps energy and gradient as a torch.autograd.Function of the
nuclear coordinates.
"""
import numpy as np
import torch

from . import _lib, scf
from .basis import ShellBasis
from .engine import DeviceShells, HeavyLane, JKEngine, QuartetBatch
from .fock import FockMatrixRestrictedGPU
from .hamiltonian import one_electron
from .molecules import Molecule, shell_basis

# quartets of a thread-form gradient class with many primitive quartets (the engine's heavy
# prefix) run in the split form: one warp per quartet over its primitive quartets
GRAD_SPLIT = True

_COMP = {0: [(0, 0, 0)], 1: [(1, 0, 0), (0, 1, 0), (0, 0, 1)],
         2: [(2, 0, 0), (0, 2, 0), (0, 0, 2), (1, 1, 0), (1, 0, 1), (0, 1, 1)]}


def _idx(lmn):
    return _COMP[sum(lmn)].index(tuple(lmn))


def combined_basis(sb: ShellBasis):
    """Original shells, then a raised copy of every shell, then a lowered copy of every
    shell with l >= 1.  Returns the ShellBasis and the raised/lowered shell indices."""
    if np.any(sb.l >= 2):
        # the raised copies of d shells are f shells, which the ERI class kernels of this
        # host cross-check do not cover; the fused adjoint kernels (eri_gradient) and the
        # one-electron derivative kernel handle d shells themselves
        raise NotImplementedError("the block-path cross-check covers s/p shells; use "
                                  "eri_gradient / one_electron_gradient_kernel for d shells")
    ns = sb.nshell
    l, cen, expo, coef, scale, off = [], [], [], [], [], [0]

    def add(ll, s, cf, sc):
        k0, k1 = sb.prim_off[s], sb.prim_off[s + 1]
        l.append(ll)
        cen.append(sb.centre[s])
        expo.extend(sb.expo[k0:k1])
        coef.extend(cf)
        off.append(len(expo))
        scale.append(sc)

    for s in range(ns):
        add(int(sb.l[s]), s, sb.coef[sb.prim_off[s]:sb.prim_off[s + 1]], sb.comp_scale[s])
    raised = np.arange(ns, 2 * ns)
    for s in range(ns):
        k0, k1 = sb.prim_off[s], sb.prim_off[s + 1]
        add(int(sb.l[s]) + 1, s, sb.coef[k0:k1] * 2.0 * sb.expo[k0:k1], np.ones(6))
    lowered = np.full(ns, -1)
    for s in range(ns):
        if sb.l[s] >= 1:
            lowered[s] = len(l)
            add(int(sb.l[s]) - 1, s, sb.coef[sb.prim_off[s]:sb.prim_off[s + 1]], np.ones(6))
    comb = ShellBasis(l, np.array(cen), off, np.array(expo), np.array(coef), np.array(scale))
    return comb, raised, lowered


def _derivative_maps(sb, comb, raised, lowered):
    """Row indices into the combined matrices: d M_ij / d(centre of i)_x =
    scale_i (M[up[x, i], j] - fac[x, i] M[dn[x, i], j])."""
    n = sb.nbf
    up = np.zeros((3, n), dtype=np.int64)
    dn = np.zeros((3, n), dtype=np.int64)
    fac = np.zeros((3, n))
    scale = np.zeros(n)
    for s in range(sb.nshell):
        for ci, lmn in enumerate(_COMP[int(sb.l[s])]):
            i = sb.func_off[s] + ci
            scale[i] = sb.comp_scale[s, ci]
            for x in range(3):
                u = list(lmn)
                u[x] += 1
                up[x, i] = comb.func_off[raised[s]] + _idx(u)
                if lmn[x] > 0:
                    d = list(lmn)
                    d[x] -= 1
                    dn[x, i] = comb.func_off[lowered[s]] + _idx(d)
                    fac[x, i] = lmn[x]
    return up, dn, fac, scale


def _derivative_rows(sb, comb, raised, lowered, M, maps=None):
    """For matrix M over (combined x original) functions, D[x][i, j] = d M_ij / d(centre of i)_x."""
    up, dn, fac, scale = maps if maps is not None else _derivative_maps(sb, comb, raised, lowered)
    n = sb.nbf
    return scale[None, :, None] * (M[up, :n] - fac[:, :, None] * M[dn, :n])


def one_electron_gradient(sb, mol, shell_atom, P, W):
    comb, raised, lowered = combined_basis(sb)
    func_atom = np.repeat(shell_atom, sb.nfunc)
    g = np.zeros((len(mol.symbols), 3))
    maps = _derivative_maps(sb, comb, raised, lowered)
    S, T, _ = one_electron(comb, mol.coords[:1], np.zeros(1))
    dS = _derivative_rows(sb, comb, raised, lowered, S, maps)
    dT = _derivative_rows(sb, comb, raised, lowered, T, maps)
    for x in range(3):
        contrib = 2.0 * np.sum(P * dT[x] - W * dS[x], axis=1)
        np.add.at(g[:, x], func_atom, contrib)
    for c in range(len(mol.symbols)):
        _, _, Vc = one_electron(comb, mol.coords[c:c + 1], mol.charges[c:c + 1])
        dV = _derivative_rows(sb, comb, raised, lowered, Vc, maps)
        for x in range(3):
            h = 2.0 * np.sum(P * dV[x], axis=1)
            np.add.at(g[:, x], func_atom, h)
            g[c, x] -= h.sum()
    return g


def tune_eri_gradient(sb, engine: JKEngine, shell_atom, P, natom, reps=3):
    """Choose the kernel form (thread or warp per quartet) of every gradient class on this
    engine's task lists (gaussium_gb300.autotune)."""
    from . import autotune
    return autotune.tune_gradient(
        engine.segments,
        lambda cls: eri_gradient(sb, engine, shell_atom, P, natom, classes=[cls], host=False),
        reps)


def one_electron_gradient_kernel(sb, mol, shell_atom, P, W, device="cuda"):
    """The one-electron gradient terms in one launch (gs_one_electron_grad)."""
    ds = DeviceShells(sb, device)
    dev = ds.device
    i, j = np.tril_indices(sb.nshell)
    t = lambda a, dt: torch.as_tensor(np.ascontiguousarray(a, dtype=dt)).to(dev)
    pairs = t(np.stack([i, j], 1), np.int32)
    grad = torch.zeros(len(mol.symbols) * 3, dtype=torch.float64, device=dev)
    # every buffer the launch reads stays referenced until after it: a temporary freed to
    # the caching allocator inside the argument list would be handed to the next one
    sa_d, xyz_d, z_d = t(shell_atom, np.int32), t(mol.coords, np.float64), t(mol.charges, np.float64)
    p_d, w_d = t(P, np.float64), t(W, np.float64)
    L = _lib.lib()
    _lib.check(L.gs_one_electron_grad(_lib.ptr(ds.centre), _lib.ptr(ds.l), _lib.ptr(ds.prim_off),
                                      _lib.ptr(ds.expo), _lib.ptr(ds.coef), _lib.ptr(ds.comp_scale),
                                      _lib.ptr(ds.func_off), _lib.ptr(sa_d), len(i), _lib.ptr(pairs),
                                      sb.nbf, len(mol.symbols), _lib.ptr(xyz_d), _lib.ptr(z_d),
                                      _lib.ptr(p_d), _lib.ptr(w_d), _lib.ptr(grad), _lib.stream()),
               "gs_one_electron_grad")
    return grad.view(-1, 3).cpu().numpy()


def nuclear_repulsion_gradient(mol):
    R, Z = mol.coords, mol.charges
    g = np.zeros_like(R)
    for a in range(len(Z)):
        d = R[a] - R
        r = np.linalg.norm(d, axis=1)
        r[a] = np.inf
        g[a] = -np.sum((Z[a] * Z / r ** 3)[:, None] * d, axis=0)
    return g


def _check_atoms(shell_atom, natom):
    sa = np.asarray(shell_atom)
    if sa.size and (sa.min() < 0 or sa.max() >= natom):
        raise ValueError("shell_atom holds an atom index outside [0, natom)")


def eri_gradient(sb, engine: JKEngine, shell_atom, P, natom, classes=None, host=True,
                 screen_thr=0.0, mixed_cut=None):
    """Two-electron gradient through the fused adjoint kernels, launched per class over the
    engine's Schwarz-screened unique quartets (``classes``: only those).  ``screen_thr``
    skips quartets whose Schwarz bound times the largest |P| of their six shell blocks is
    below it; with ``mixed_cut``, the quartets of the thread-form classes whose such bound
    is below the cut run their recursion in FP32 (FP64 HRR, contraction and sums).
    Returns natom x 3 (host numpy, or the device tensor with ``host=False``)."""
    _check_atoms(shell_atom, natom)
    dev = engine.dev
    grad = torch.zeros(natom * 3, dtype=torch.float64, device=dev)
    pt = torch.as_tensor(np.ascontiguousarray(P)).to(dev)
    sa = torch.as_tensor(np.ascontiguousarray(shell_atom, dtype=np.int32)).to(dev)
    dmax, thr = None, 0.0
    if screen_thr > 0 or mixed_cut is not None:
        dmax = engine.shell_dmax([pt])
        thr = screen_thr if screen_thr > 0 else 1e-300
    L = _lib.lib()
    base = engine.tasks.data_ptr()
    lane = HeavyLane(dev)
    inf = float("inf")
    for (cls, s, e), heavy in zip(engine.segments, engine.heavy):
        if classes is not None and cls not in classes:
            continue
        thread = L.gs_eri_grad_class_form(*cls) == 1
        # a thread-form class's quartets with many primitive quartets (the task list's
        # prefix) in the split form, on the side stream beside the other launches
        h = heavy[0] if GRAD_SPLIT and thread else 0
        bands = [(64, mixed_cut, inf), (32, 0.0, mixed_cut)] \
            if (mixed_cut is not None and thread) else [(64, 0.0, inf)]
        for prec, lo, hi in bands:
            prims = engine.pairs.p64 if prec == 64 else engine.pairs.p32
            for form, first, count, side in ((3, 0, h, True), (0, h, e - s - h, False)):
                if count <= 0:
                    continue
                _lib.check(L.gs_eri_grad_band(
                    *cls, form, prec, _lib.ptr(engine.pairs.rec), _lib.ptr(prims),
                    _lib.ptr(engine.ds.comp_scale), _lib.ptr(engine.ds.func_off), _lib.ptr(sa),
                    count, base + (s + first) * 8, sb.nbf, natom, _lib.ptr(pt), sb.nshell,
                    _lib.ptr(dmax), thr, lo, hi, _lib.ptr(grad),
                    lane.stream() if side else _lib.stream()), f"gs_eri_grad_band{cls}")
    lane.join()
    return grad.view(natom, 3).cpu().numpy() if host else grad.view(natom, 3)


def eri_gradient_blocks(sb, engine: JKEngine, shell_atom, P, natom):
    """The same two-electron gradient from explicit raised/lowered blocks (gs_eri_blocks)
    contracted by gs_eri_grad_contract; slower, kept as an independent cross-check."""
    _check_atoms(shell_atom, natom)
    comb, raised, lowered = combined_basis(sb)
    tasks = engine.tasks[:engine.ntasks].cpu().numpy()
    ps = engine.pairs.host_shells
    quart = np.concatenate([ps[tasks[:, 0]], ps[tasks[:, 1]]], axis=1).astype(np.int64)
    nq = len(quart)
    mods = []
    owner = []
    slot = []
    for cen in range(3):
        s = quart[:, cen]
        up = quart.copy()
        up[:, cen] = raised[s]
        mods.append(up); owner.append(np.arange(nq)); slot.append(np.full(nq, 2 * cen))
        has = lowered[s] >= 0
        dn = quart[has].copy()
        dn[:, cen] = lowered[s[has]]
        mods.append(dn); owner.append(np.flatnonzero(has)); slot.append(np.full(has.sum(), 2 * cen + 1))
    mods = np.concatenate(mods)
    owner = np.concatenate(owner)
    slot = np.concatenate(slot)
    ds = DeviceShells(comb, engine.dev)
    batch = QuartetBatch(ds, mods, want32=False)
    blocks = torch.zeros(max(1, batch.total), dtype=torch.float64, device=engine.dev)
    batch.run(blocks, 64)
    boff = np.full((nq, 6), -1, dtype=np.int64)
    boff[owner, slot] = batch.offsets[:-1]
    dev = engine.dev
    t = lambda a, dt: torch.as_tensor(np.ascontiguousarray(a, dtype=dt)).to(dev)
    grad = torch.zeros(natom * 3, dtype=torch.float64, device=dev)
    pt = torch.as_tensor(np.ascontiguousarray(P)).to(dev)
    qd, bd, sa_d = t(quart, np.int32), t(boff, np.int64), t(shell_atom, np.int32)
    L = _lib.lib()
    _lib.check(L.gs_eri_grad_contract(nq, _lib.ptr(qd), _lib.ptr(bd), _lib.ptr(blocks),
                                      _lib.ptr(engine.ds.l), _lib.ptr(engine.ds.func_off),
                                      _lib.ptr(engine.ds.comp_scale), _lib.ptr(sa_d), sb.nbf, _lib.ptr(pt),
                                      _lib.ptr(grad), _lib.stream()), "gs_eri_grad_contract")
    return grad.view(natom, 3).cpu().numpy()


def shell_atoms(mol, sb):
    """Atom index of every shell (shells are generated atom by atom)."""
    out = np.empty(sb.nshell, dtype=np.int64)
    for s in range(sb.nshell):
        d = np.linalg.norm(mol.coords - sb.centre[s], axis=1)
        out[s] = int(np.argmin(d))
    return out


class RHFState:
    """A converged RHF solution with what its gradient needs: the molecule, basis, engine
    (pair records, Schwarz-screened quartet tasks), the density P and the energy-weighted
    density W."""

    def __init__(self, mol, sb, engine, energy, scf_result, P, W):
        self.mol, self.sb, self.engine = mol, sb, engine
        self.energy, self.scf = energy, scf_result
        self.P, self.W = P, W


def rhf_state(mol, basis="6-31G", threshold=1e-12, schwarz_thr=1e-14):
    """Converged RHF energy (Eh) and the densities its analytic gradient contracts."""
    sb = shell_basis(mol, basis)
    S, T, V = one_electron(sb, mol.coords, mol.charges)
    hcore = T + V
    eng = JKEngine(sb, schwarz_thr=schwarz_thr)
    fb = FockMatrixRestrictedGPU(hcore, eng)
    res = scf.restricted_scf(S, hcore, mol.electrons, fb, threshold=threshold, max_iter=200)
    if not res.converged:
        raise RuntimeError("SCF did not converge")
    nocc = mol.electrons // 2
    la = scf.LinearAlgebra(S)
    eps, C = la.diagonalize(res.fock)
    P = 2.0 * C[:, :nocc] @ C[:, :nocc].T
    W = 2.0 * (C[:, :nocc] * eps[:nocc]) @ C[:, :nocc].T
    return RHFState(mol, sb, eng, res.energy + mol.nuclear_repulsion(), res, P, W)


# the adjoint's defaults: quartets whose Schwarz bound times max |P| is below 1e-12 are
# skipped, and those below 1e-3 run their recursion in FP32 (FP64 Boys function at small T,
# HRR, contraction and sums); on (H2O)8 this moves the gradient by < 4e-9 Eh/bohr
GRAD_SCREEN_THR = 1e-12
GRAD_MIXED_CUT = 1e-3


def gradient_from_state(st: RHFState, screen_thr=GRAD_SCREEN_THR, mixed_cut=GRAD_MIXED_CUT):
    """dE/dR (natom x 3, Eh/bohr) from a converged state: the one-electron derivative
    kernel (P dH/dR - W dS/dR), the fused ERI adjoint kernels contracting d(ab|cd)/dR with
    the density-weighted quartet weights Gamma(P), and the nuclear repulsion.
    ``screen_thr`` / ``mixed_cut``: density screening and FP32 recursions for the quartets
    with small density-weighted bounds (eri_gradient; 0.0 / None: every quartet in FP64)."""
    sa = shell_atoms(st.mol, st.sb)
    g = one_electron_gradient_kernel(st.sb, st.mol, sa, st.P, st.W)
    g += eri_gradient(st.sb, st.engine, sa, st.P, len(st.mol.symbols), screen_thr=screen_thr,
                      mixed_cut=mixed_cut)
    g += nuclear_repulsion_gradient(st.mol)
    return g


def rhf_energy_gradient(mol, basis="6-31G", threshold=1e-12, schwarz_thr=1e-14,
                        want_gradient=True, screen_thr=GRAD_SCREEN_THR, mixed_cut=GRAD_MIXED_CUT):
    """Converged RHF energy and analytic gradient (Eh, Eh/bohr)."""
    st = rhf_state(mol, basis, threshold, schwarz_thr)
    if not want_gradient:
        return st.energy, None, st.scf
    return st.energy, gradient_from_state(st, screen_thr, mixed_cut), st.scf


class EnergyGradient(torch.autograd.Function):
    """E(R) for nuclear coordinates R (natom x 3, bohr).  The forward pass runs the SCF
    only and keeps the converged state (densities, engine); the backward pass launches the
    adjoint kernels on it -- the ERI adjoint takes the density-weighted quartet weights
    dE/d(ab|cd) = Gamma_abcd(P) and returns the nuclear-coordinate gradient -- and scales
    it by the incoming gradient.  A forward without backward computes no gradient."""

    @staticmethod
    def forward(ctx, coords, symbols, basis):
        mol = Molecule(symbols, coords.detach().cpu().numpy())
        ctx.state = rhf_state(mol, basis)
        ctx.dtype = coords.dtype
        return torch.tensor(ctx.state.energy, dtype=coords.dtype)

    @staticmethod
    def backward(ctx, grad_out):
        g = torch.as_tensor(gradient_from_state(ctx.state), dtype=ctx.dtype)
        ctx.state = None
        return grad_out * g, None, None
