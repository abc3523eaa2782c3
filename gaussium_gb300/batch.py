"""Batched RHF over many molecules of uneven size on one GPU.

All molecules' shells, shell pairs and Schwarz-screened unique quartets are packed into
one engine; a Fock build for every molecule at once is one set of class-kernel launches
(``gs_fock_jk_batched``: each quartet digests into its own molecule's block of the packed
J/K), captured once in a CUDA graph and replayed every SCF iteration.  Orthogonalisation,
DIIS and diagonalisation run batched in FP64 on the device (torch) over zero-padded
matrices.  The per-molecule algorithm is the reference's restricted SCF
(hartreefock/scf_procedure.py:24-42: core-Hamiltonian guess, canonical orthogonalisation
hartreefock/linear_algebra.py:18-25, Pulay DIIS diismethod/diis.py:39-112) with a
plain always-on DIIS after the first iteration.
"""
import numpy as np
import torch

from . import _lib
from .basis import ShellBasis
from .engine import (COOP_PRIM_QUARTETS, PAIR_ORDER, PRIM_SCREEN, DeviceShells, HeavyLane, PairSet,
                     _pc_lut, heavy_threshold, mixed_prefix, split_forms)
from .hamiltonian import one_electron
from .molecules import shell_basis


class BatchedRHF:
    def __init__(self, molecules, basis="6-31G*", schwarz_thr=1e-12, device="cuda",
                 max_exp=PRIM_SCREEN):
        self.mols = molecules
        self.basis = basis
        self.dev = torch.device(device)
        sbs = [shell_basis(m, basis) for m in molecules]
        self.sbs = sbs
        nm = len(sbs)
        self.nbf = np.array([s.nbf for s in sbs])
        self.nmax = int(self.nbf.max())
        self.base = np.concatenate([[0], np.cumsum(self.nbf ** 2)])
        self.mat_stride = int(self.base[-1])
        # packed shells (global shell indices, molecule-local function offsets)
        ls, cen, expo, coef, scale, off = [], [], [], [], [], [0]
        shell_mol, local_fo, shell0 = [], [], [0]
        for m, sb in enumerate(sbs):
            for s in range(sb.nshell):
                k0, k1 = sb.prim_off[s], sb.prim_off[s + 1]
                ls.append(sb.l[s]); cen.append(sb.centre[s]); scale.append(sb.comp_scale[s])
                expo.extend(sb.expo[k0:k1]); coef.extend(sb.coef[k0:k1]); off.append(len(expo))
                shell_mol.append(m); local_fo.append(sb.func_off[s])
            shell0.append(shell0[-1] + sb.nshell)
        big = ShellBasis(ls, np.array(cen), off, np.array(expo), np.array(coef), np.array(scale))
        self.ds = DeviceShells(big, device)
        t = lambda a, dt: torch.as_tensor(np.ascontiguousarray(a, dtype=dt)).to(self.dev)
        self.local_fo = t(local_fo, np.int32)
        self.shell_mol = t(shell_mol, np.int32)
        self.mol_base = t(self.base[:-1], np.int64)
        self.mol_n = t(self.nbf, np.int32)
        # shell pairs inside each molecule
        pairs, pair_mol = [], []
        for m in range(nm):
            i, j = np.tril_indices(sbs[m].nshell)
            i, j = i + shell0[m], j + shell0[m]
            sw = big.l[i] < big.l[j]
            pairs.append(np.stack([np.where(sw, j, i), np.where(sw, i, j)], 1))
            pair_mol.append(np.full(len(i), m))
        pairs = np.concatenate(pairs)
        pair_mol = np.concatenate(pair_mol)
        self.pairs = PairSet(self.ds, pairs, want32=True, max_exp=max_exp)
        pc = _pc_lut[big.l[pairs[:, 0]], big.l[pairs[:, 1]]]
        q = torch.zeros(len(pairs), dtype=torch.float64, device=self.dev)
        L = _lib.lib()
        for c, (la, lb) in enumerate(PAIR_ORDER):
            idx = np.flatnonzero(pc == c).astype(np.int32)
            if len(idx):
                it = t(idx, np.int32)
                _lib.check(L.gs_schwarz(la, lb, _lib.ptr(self.pairs.rec), _lib.ptr(self.pairs.p64),
                                        _lib.ptr(self.ds.comp_scale), len(idx), _lib.ptr(it),
                                        _lib.ptr(q), len(pairs), _lib.stream()), "gs_schwarz")
        self._tasks(q, pc, pair_mol, schwarz_thr)
        # per-molecule shell-block tables of max |P| (density-weighted bounds): molecule m's
        # ns_m x ns_m table starts at sbase[m]; every packed density element maps to its block
        ns = np.array([sb.nshell for sb in sbs], dtype=np.int64)
        sbase = np.concatenate([[0], np.cumsum(ns * ns)])
        self.nblocks = int(sbase[-1])
        self.mol_shell0 = t(np.array(shell0[:-1]), np.int32)
        self.mol_nshell = t(ns, np.int32)
        self.mol_sbase = t(sbase[:-1], np.int64)
        blk = np.empty(self.mat_stride, dtype=np.int64)
        for m, sb in enumerate(sbs):
            fs = np.repeat(np.arange(sb.nshell), sb.nfunc)
            blk[self.base[m]:self.base[m + 1]] = sbase[m] + (fs[:, None] * ns[m] + fs[None, :]).ravel()
        self.block_of = torch.as_tensor(blk).to(self.dev)
        self.block_mol = torch.as_tensor(np.repeat(np.arange(len(sbs)), ns * ns)).to(self.dev)
        # one-electron matrices, orthogonalisers, padded index maps
        self.S, self.H = [], []
        for m, (mol, sb) in enumerate(zip(molecules, sbs)):
            S, T, V = one_electron(sb, mol.coords, mol.charges)
            self.S.append(S)
            self.H.append(T + V)
        self._padded_setup()
        self._graphs = {}           # (mixed_cut, screen_thr) -> (P_static, graph, G_static)

    def _tasks(self, q, pc, pair_mol, thr):
        nprim = torch.as_tensor(np.asarray(self.pairs.nprim, dtype=np.int64)).to(self.dev)
        pc_d = torch.as_tensor(np.asarray(pc, dtype=np.int64)).to(self.dev)
        pm_d = torch.as_tensor(np.asarray(pair_mol, dtype=np.int64)).to(self.dev)
        self.segments, self.tasks = batched_task_list(q, pc_d, pm_d, nprim, thr, len(PAIR_ORDER),
                                                      len(self.sbs))
        self.ntasks = int(self.tasks.shape[0])
        # tasks of each segment with many primitive quartets (prefixes: the segments are
        # sorted by descending primitive work); they run in the split or cooperative form
        # (engine.split_forms)
        work = nprim[self.tasks[:, 0].long()] * nprim[self.tasks[:, 1].long()] \
            if self.ntasks else torch.zeros(0, dtype=torch.int64, device=self.dev)
        self.heavy = [(int((work[s:e] >= heavy_threshold(cls)).sum()),
                       int((work[s:e] >= COOP_PRIM_QUARTETS).sum())) for cls, s, e in self.segments]

    def _padded_setup(self):
        B, N = len(self.sbs), self.nmax
        dev = self.dev
        # gather map packed <-> padded [B, N, N]
        idx = np.full((B, N, N), -1, dtype=np.int64)
        for m, n in enumerate(self.nbf):
            idx[m, :n, :n] = self.base[m] + np.arange(n * n).reshape(n, n)
        flat = idx.reshape(-1)
        pos = np.flatnonzero(flat >= 0)
        self.pos_padded = torch.as_tensor(pos).to(dev)          # into [B*N*N]
        self.pos_packed = torch.as_tensor(flat[pos]).to(dev)    # into packed storage
        self.Sb, self.Hb, self.X, self.occ_mask, self.pad_orb = padded_system(
            self.S, self.H, [mol.electrons // 2 for mol in self.mols], dev)

    def to_packed(self, Pb):
        out = torch.zeros(self.mat_stride, dtype=torch.float64, device=self.dev)
        out.index_copy_(0, self.pos_packed, Pb.reshape(-1).index_select(0, self.pos_padded))
        return out

    def to_padded(self, v):
        Pb = torch.zeros(len(self.sbs) * self.nmax * self.nmax, dtype=torch.float64, device=self.dev)
        Pb.index_copy_(0, self.pos_padded, v.index_select(0, self.pos_packed))
        return Pb.view(len(self.sbs), self.nmax, self.nmax)

    def _class_starts(self):
        """Start of every canonical class's segment in the task array (22 entries, the
        last = number of tasks), for the persistent launch."""
        import sys
        import os
        sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "csrc"))
        try:
            import gen_eri
        finally:
            sys.path.pop(0)
        seg = {cls: (s, e) for cls, s, e in self.segments}
        out, pos = [], 0
        for cls in gen_eri.canonical_classes(2):
            if cls in seg:
                assert seg[cls][0] == pos, "task segments must follow the canonical class order"
                out.append(pos)
                pos = seg[cls][1]
            else:
                out.append(pos)
        out.append(pos)
        assert pos == self.ntasks
        return np.array(out, dtype=np.int32)

    def _jk_persistent(self, P, J, K, dmax, mixed_cut, screen_thr):
        """All classes of all molecules in one persistent launch per precision
        (gs_fock_jk_batched_persistent), after one partition pass over every task."""
        L = _lib.lib()
        if getattr(self, "_starts", None) is None:
            self._starts = self._class_starts()
        need = L.gs_fock_jk_persistent_workspace(self.ntasks)
        if getattr(self, "_pws", None) is None or self._pws.numel() < need:
            self._pws = torch.empty(int(need), dtype=torch.uint8, device=self.dev)
        cut = mixed_cut if mixed_cut is not None else 0.0
        rc = L.gs_fock_jk_batched_persistent(
            _lib.ptr(self.pairs.rec), _lib.ptr(self.pairs.p64), _lib.ptr(self.pairs.p32),
            _lib.ptr(self.ds.comp_scale), _lib.ptr(self.local_fo), _lib.ptr(self.shell_mol),
            _lib.ptr(self.mol_base), _lib.ptr(self.mol_n), _lib.ptr(dmax), _lib.ptr(self.mol_shell0),
            _lib.ptr(self.mol_nshell), _lib.ptr(self.mol_sbase), self.mat_stride,
            self._starts.ctypes.data, self.ntasks, _lib.ptr(self.tasks), _lib.ptr(P), _lib.ptr(J),
            1, _lib.ptr(P), _lib.ptr(K), screen_thr, cut, _lib.ptr(self._pws), self._pws.numel(),
            _lib.stream())
        _lib.check(rc, "gs_fock_jk_batched_persistent")

    def _jk_launch(self, P, J, K, precision=64, mixed_cut=None, dmax=None, screen_thr=0.0,
                   classes=None):
        L = _lib.lib()
        st = _lib.stream()
        lane = HeavyLane(self.dev)
        base = self.tasks.data_ptr()
        if mixed_cut is not None or screen_thr > 0:
            # partitioned path: screened tasks are dropped on the device before any class
            # kernel runs, FP64/FP32 by the density-weighted bound
            cut = mixed_cut if mixed_cut is not None else 0.0
            thr = screen_thr if screen_thr > 0 else 1e-300
            need = max(L.gs_fock_jk_mixed_workspace(e - s) for _, s, e in self.segments)
            if getattr(self, "_ws", None) is None or self._ws.numel() < need:
                self._ws = torch.empty(int(need), dtype=torch.uint8, device=self.dev)
            mol_dmax = None
            for (cls, s, e), heavy in zip(self.segments, self.heavy):
                if classes is not None and cls not in classes:
                    continue
                # the heavy prefix in the split form, one banded launch per precision; the
                # bound there takes each molecule's largest |P| (at least the block value the
                # partition uses, so no quartet is screened or demoted that the partition
                # would keep)
                h, launches = mixed_prefix(cls, heavy, cut)
                for prec, form, first, count, lo, hi in launches:
                    if mol_dmax is None:
                        mol_dmax = torch.zeros(len(self.mol_n), dtype=torch.float64,
                                               device=self.dev)
                        mol_dmax.scatter_reduce_(0, self.block_mol, dmax, "amax",
                                                 include_self=True)
                    rc = L.gs_fock_jk_batched(
                        *cls, prec | (form << 8), _lib.ptr(self.pairs.rec),
                        _lib.ptr(self.pairs.prims(prec)), _lib.ptr(self.ds.comp_scale),
                        _lib.ptr(self.local_fo), _lib.ptr(self.shell_mol), _lib.ptr(self.mol_base),
                        _lib.ptr(self.mol_n), _lib.ptr(mol_dmax), self.mat_stride, count,
                        base + (s + first) * 8, _lib.ptr(P), _lib.ptr(J), 1, _lib.ptr(P),
                        _lib.ptr(K), thr, lo, hi, lane.stream())
                    _lib.check(rc, f"gs_fock_jk_batched{cls}")
                rc = L.gs_fock_jk_batched_mixed(
                    *cls, _lib.ptr(self.pairs.rec), _lib.ptr(self.pairs.p64),
                    _lib.ptr(self.pairs.p32), _lib.ptr(self.ds.comp_scale), _lib.ptr(self.local_fo),
                    _lib.ptr(self.shell_mol), _lib.ptr(self.mol_base), _lib.ptr(self.mol_n),
                    _lib.ptr(dmax), _lib.ptr(self.mol_shell0), _lib.ptr(self.mol_nshell),
                    _lib.ptr(self.mol_sbase), self.mat_stride, e - s - h, base + (s + h) * 8,
                    _lib.ptr(P), _lib.ptr(J), 1,
                    _lib.ptr(P), _lib.ptr(K), thr, cut, _lib.ptr(self._ws), self._ws.numel(), st)
                _lib.check(rc, f"gs_fock_jk_batched_mixed{cls}")
            lane.join()
            return
        thr = 0.0
        runs = [(precision, 0.0, float("inf"))]
        if mixed_cut is not None:
            runs = [(64, mixed_cut, float("inf")), (32, 0.0, mixed_cut)]
        for prec, lo, hi in runs:
            prims = self.pairs.prims(prec)
            plan = [(cls, s, e, split_forms(cls, prec, heavy))
                    for (cls, s, e), heavy in zip(self.segments, self.heavy)
                    if classes is None or cls in classes]
            # heavy prefixes first, on side 0; then every class's rest, alternating streams
            for heavy_pass in (True, False):
                for i, (cls, s, e, parts) in enumerate(plan):
                    for k, (form, first, count) in enumerate(parts):
                        if (k == 0 and len(parts) > 1) != heavy_pass:
                            continue
                        m = (e - s - first) if count is None else count
                        rc = L.gs_fock_jk_batched(
                            *cls, prec | (form << 8), _lib.ptr(self.pairs.rec), _lib.ptr(prims),
                            _lib.ptr(self.ds.comp_scale), _lib.ptr(self.local_fo),
                            _lib.ptr(self.shell_mol), _lib.ptr(self.mol_base), _lib.ptr(self.mol_n),
                            _lib.ptr(dmax), self.mat_stride, m, base + (s + first) * 8,
                            _lib.ptr(P), _lib.ptr(J), 1, _lib.ptr(P), _lib.ptr(K), thr, lo, hi,
                            lane.stream() if heavy_pass else lane.alternate(i))
                        _lib.check(rc, f"gs_fock_jk_batched{cls}")
        lane.join()

    def tune(self, precisions=(64, 32), reps=3):
        """Choose the kernel form of every class with two on this batch's task lists."""
        from . import autotune
        P = torch.zeros(self.mat_stride, dtype=torch.float64, device=self.dev)
        J, K = torch.zeros_like(P), torch.zeros_like(P)
        return autotune.tune(self.segments,
                             lambda cls, prec: self._jk_launch(P, J, K, prec, classes=[cls]),
                             precisions, reps)

    def density(self, m):
        """Converged density of molecule m (host nbf_m x nbf_m) after ``run``."""
        n = int(self.nbf[m])
        return self.densities[m, :n, :n].cpu().numpy()

    def fock_packed(self, P, precision=64, mixed_cut=None, screen_thr=0.0, persistent=False):
        """G = J - K/2 (padded [B, N, N], symmetric) for packed densities P, all molecules.
        With ``screen_thr`` a quartet is skipped when its Schwarz bound times the largest
        |P| element of the six shell blocks it touches is below it; with ``mixed_cut`` the
        quartets whose such bound is below the cut run in FP32 (FP64 accumulation).
        ``persistent``: every class in one persistent launch per precision instead of one
        launch per class (quartets whose bound is exactly zero are skipped there)."""
        J = torch.zeros_like(P)
        K = torch.zeros_like(P)
        dmax = None
        if mixed_cut is not None or screen_thr > 0 or persistent:
            dmax = torch.zeros(self.nblocks, dtype=torch.float64, device=self.dev)
            dmax.scatter_reduce_(0, self.block_of, P.abs(), "amax", include_self=True)
        if persistent:
            if precision != 64 and mixed_cut is None:
                raise ValueError("the persistent launch evaluates FP64 unless mixed_cut is given")
            self._jk_persistent(P, J, K, dmax, mixed_cut, screen_thr)
        else:
            self._jk_launch(P, J, K, precision, mixed_cut, dmax, screen_thr)
        Jb, Kb = self.to_padded(J), self.to_padded(K)
        G = (Jb + Jb.transpose(1, 2)) - 0.5 * (Kb + Kb.transpose(1, 2))
        return G

    def run(self, threshold=1e-10, max_iter=60, mixed_cut=None, screen_thr=0.0,
            incremental=False, reset_every=8, final_fp64=None, use_graph=True,
            log_iterations=False, guess="core", persistent=False):
        """Batched SCF; returns total energies (numpy) and the iteration count.

        With ``incremental`` the Fock build of iteration i evaluates G(P_i - P_ref) and adds
        it to G(P_ref) (a full build every ``reset_every`` iterations); with screening this
        skips most quartets once the densities settle, and a converged molecule (dP = 0)
        costs nothing.  ``final_fp64`` (default: on whenever a build is approximate)
        evaluates the reported energies from one full, unscreened FP64 build at the final
        densities.  ``persistent`` builds every Fock matrix with the persistent launch
        (one kernel per precision over all classes and molecules) instead of one launch per
        class; either way the build is captured in one CUDA graph.  ``log_iterations`` records (iteration, seconds, converged molecules) in
        ``iteration_log`` (it synchronises the device once per iteration).  ``guess`` is
        "core" (the reference's core-Hamiltonian start) or "sad" (superposed atomic
        densities, gaussium_gb300.guess)."""
        key = (mixed_cut, screen_thr, persistent)
        if key in self._graphs:
            P_static, g, G_static = self._graphs[key]
        else:
            P_static = torch.zeros(self.mat_stride, dtype=torch.float64, device=self.dev)
            g = G_static = None

        def build():
            return self.fock_packed(P_static, mixed_cut=mixed_cut, screen_thr=screen_thr,
                                    persistent=persistent)

        if use_graph and g is None:
            build()                                  # warm-up outside capture
            torch.cuda.synchronize()
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g):
                G_static = build()
            self._graphs[key] = (P_static, g, G_static)
        state = {"n": 0, "P": None, "G": None}

        def two_electron(Pb, active):
            # incremental: G(P_ref) + G(P - P_ref); a full build (first, and every
            # reset_every-th) evaluates only the molecules still iterating
            inc = incremental and state["P"] is not None and state["n"] % reset_every != 0
            if inc:
                Pin = Pb - state["P"]
            elif state["G"] is not None:
                Pin = torch.where(active[:, None, None], Pb, torch.zeros_like(Pb))
            else:
                Pin = Pb
            P_static.copy_(self.to_packed(Pin))
            if use_graph:
                g.replay()
                G = G_static.clone()
            else:
                G = build()
            if inc:
                G = G + state["G"]
            elif state["G"] is not None:
                G = torch.where(active[:, None, None], G, state["G"])
            state.update(n=state["n"] + 1, P=Pb.clone(), G=G)
            return G

        import time
        self.iteration_log = []
        t_start = [time.perf_counter()]

        def log(it, done):
            torch.cuda.synchronize()
            now = time.perf_counter()
            self.iteration_log.append((it, now - t_start[0], int(done.sum())))
            t_start[0] = now

        P_init = None
        if guess == "sad":
            from .guess import sad_density
            P_init = torch.zeros_like(self.Hb)
            for m, mol in enumerate(self.mols):
                n = int(self.nbf[m])
                P_init[m, :n, :n] = torch.as_tensor(sad_density(mol, self.basis)).to(self.dev)
        elif guess != "core":
            raise ValueError(f"unknown guess {guess!r}")
        energies, it, self.converged, Pb = batched_rhf_iterations(
            self.Sb, self.Hb, self.X, self.occ_mask, self.pad_orb, two_electron,
            threshold=threshold, max_iter=max_iter, on_iteration=log if log_iterations else None,
            P_init=P_init)
        self.iterations = it
        self.densities = Pb
        if final_fp64 is None:
            final_fp64 = incremental or mixed_cut is not None or screen_thr > 0
        if final_fp64:
            G = self.fock_packed(self.to_packed(Pb))
            energies = 0.5 * torch.sum(Pb * (2.0 * self.Hb + G), dim=(1, 2))
        e_nuc = torch.tensor([m.nuclear_repulsion() for m in self.mols], dtype=torch.float64,
                             device=self.dev)
        return (energies + e_nuc).cpu().numpy(), it


def batched_task_list(q, pair_class, pair_mol, nprim, thr, nclass, nmol):
    """Unique shell-quartet tasks (bra pair, ket pair) of many molecules, on the device of
    the inputs: for every class pair (cb >= ck) and every molecule, the pairs of that
    molecule with q_bra q_ket >= thr (bra >= ket within one class), quartets never
    crossing molecules.  Each class segment is ordered by primitive-quartet count, largest
    first, then (primitive pairs of the bra, of the ket), molecule by molecule otherwise.  Returns [((la, lb, lc, ld), start, end)]
    and the [ntask, 2] int32 task array."""
    dev = q.device
    key = pair_mol * nclass + pair_class
    order = torch.argsort(key, stable=True)
    cnt = torch.bincount(key, minlength=nmol * nclass).view(nmol, nclass)
    start = (torch.cumsum(cnt.reshape(-1), 0) - cnt.reshape(-1)).view(nmol, nclass)
    cnt_h = cnt.cpu().numpy()
    mols = torch.arange(nmol, device=dev)
    segs, chunks, n = [], [], 0
    for cb in range(nclass):
        for ck in range(cb + 1):
            nb, nk = cnt[:, cb], cnt[:, ck]
            total = int((cnt_h[:, cb] * cnt_h[:, ck]).sum())
            if total == 0:
                continue
            tot = nb * nk
            mol = torch.repeat_interleave(mols, tot)
            local = torch.arange(total, device=dev) - (torch.cumsum(tot, 0) - tot)[mol]
            nk_m = nk[mol]
            bra = order[start[mol, cb] + local // nk_m]
            ket = order[start[mol, ck] + local % nk_m]
            del mol, local, nk_m
            keep = q[bra] * q[ket] >= thr
            if cb == ck:
                keep &= bra >= ket
            bra, ket = bra[keep], ket[keep]
            if bra.numel() == 0:
                continue
            # most primitive quartets first, equal (K_bra, K_ket) together
            perm = torch.argsort((nprim[bra] * nprim[ket]) * 4096 + nprim[bra] * 64 + nprim[ket],
                                 descending=True, stable=True)
            tk = torch.stack([bra[perm], ket[perm]], 1).to(torch.int32)
            (la, lb), (lc, ld) = PAIR_ORDER[cb], PAIR_ORDER[ck]
            segs.append(((la, lb, lc, ld), n, n + tk.shape[0]))
            chunks.append(tk)
            n += tk.shape[0]
    tasks = torch.cat(chunks) if chunks else torch.zeros((0, 2), dtype=torch.int32, device=dev)
    return segs, tasks.contiguous()


_POOL = None


def _host_eigh(Fo):
    """Eigenvectors of a batch of symmetric matrices on the host: torch's LAPACK path over
    chunks of the batch on a pool of threads (the calls release the interpreter lock)."""
    global _POOL
    import os
    from concurrent.futures import ThreadPoolExecutor
    nthr = max(1, os.cpu_count() or 1)
    if _POOL is None:
        _POOL = ThreadPoolExecutor(nthr)
    host = Fo.cpu()
    chunks = host.split(max(1, -(-host.shape[0] // nthr)))
    vecs = list(_POOL.map(lambda c: torch.linalg.eigh(c)[1], chunks))
    return torch.cat(vecs).to(Fo.device)


def padded_system(S_list, H_list, nocc, device):
    """Zero-padded [B, N, N] overlap and core Hamiltonian (identity overlap on the padding),
    the canonical orthogonaliser of each molecule (eigenvalues ascending, as the reference
    sorts them, hartreefock/linear_algebra.py:18-25; padded orbitals are zero columns at
    positions n..N-1), the occupied-orbital mask and the padded-orbital indicator."""
    dev = torch.device(device)
    B, N = len(S_list), max(s.shape[0] for s in S_list)
    S = torch.zeros((B, N, N), dtype=torch.float64, device=dev)
    H = torch.zeros_like(S)
    X = torch.zeros_like(S)
    pad = torch.zeros((B, N), dtype=torch.float64, device=dev)
    for m, (Sm, Hm) in enumerate(zip(S_list, H_list)):
        n = Sm.shape[0]
        S[m, :n, :n] = torch.as_tensor(np.asarray(Sm, dtype=np.float64)).to(dev)
        H[m, :n, :n] = torch.as_tensor(np.asarray(Hm, dtype=np.float64)).to(dev)
        S[m, n:, n:] = torch.eye(N - n, dtype=torch.float64, device=dev)
        s, u = torch.linalg.eigh(S[m, :n, :n])
        X[m, :n, :n] = u * s.rsqrt().unsqueeze(0)
        pad[m, n:] = 1.0
    nocc = torch.as_tensor(np.asarray(nocc), device=dev)
    occ = (torch.arange(N, device=dev)[None, :] < nocc[:, None]).double()
    return S, H, X, occ, pad


def batched_rhf_iterations(Sb, Hb, X, occ_mask, pad_orb, two_electron, threshold=1e-10,
                           max_iter=60, diis_subspace=8, level_shift=0.3, shift_after=30,
                           shifted_error=1e-5, on_iteration=None, P_init=None, eigh_on="host"):
    """Restricted SCF of B molecules at once over zero-padded [B, N, N] FP64 matrices.

    ``two_electron(P, active)`` returns G = J - K/2 for the padded densities; ``active``
    flags the molecules still iterating (the others' densities no longer change).  Per
    molecule: the core-Hamiltonian guess, canonical orthogonaliser ``X`` (zero columns for
    padded orbitals, which ``pad_orb`` lifts to the top of the spectrum), Pulay DIIS on the
    orthogonalised commutator SPF - FPS, and the reference's stopping rule |dE| <
    threshold (hartreefock/scf_procedure.py:24-42).  A molecule that has converged keeps
    its density (its energy is final) while the others iterate; the DIIS matrix of each
    molecule is scaled by its largest diagonal element so that a nearly converged molecule
    does not make the batched solve singular.  A molecule still iterating after
    ``shift_after`` iterations gets a level shift of its virtual orbitals,
    F + level_shift (S - S P S / 2) (the converged density is unchanged by it), and must then
    also bring its largest commutator element below ``shifted_error`` to stop, since the
    shift slows the energy change.  ``on_iteration(it, done)`` is called after each
    iteration's convergence test.  ``P_init`` ([B, N, N], optional) replaces the
    core-Hamiltonian guess as the first iteration's densities.  Returns the electronic
    energies, the iteration count, the per-molecule converged flags and the last
    densities."""
    dev = Hb.device
    B = Hb.shape[0]
    big = 1e6 * pad_orb

    def eigh(Fo):
        if eigh_on == "device":
            return torch.linalg.eigh(Fo)[1]
        return _host_eigh(Fo)

    def diag(F):
        Fo = X.transpose(1, 2) @ F @ X + torch.diag_embed(big)
        return None, X @ eigh(Fo)

    _, C = diag(Hb)
    prev = torch.zeros(B, dtype=torch.float64, device=dev)
    done = torch.zeros(B, dtype=torch.bool, device=dev)
    shifted = torch.zeros(B, dtype=torch.bool, device=dev)
    hist_f, hist_e = [], []
    energies = None
    it = 0
    for it in range(1, max_iter + 1):
        if it == 1 and P_init is not None:
            Pb = P_init
        else:
            Cocc = C * occ_mask[:, None, :]
            Pb = 2.0 * Cocc @ Cocc.transpose(1, 2)
        F = Hb + two_electron(Pb, ~done)
        e_now = 0.5 * torch.sum(Pb * (Hb + F), dim=(1, 2))
        energies = e_now if energies is None else torch.where(done, energies, e_now)
        err = Sb @ Pb @ F - F @ Pb @ Sb
        err = X.transpose(1, 2) @ err @ X
        if it > 1:
            small = (e_now - prev).abs() < threshold
            small &= ~shifted | (err.abs().amax(dim=(1, 2)) < shifted_error)
            done = done | small
        prev = e_now
        if on_iteration is not None:
            on_iteration(it, done)
        if bool(done.all()):
            break
        hist_f.append(F)
        hist_e.append(err)
        if len(hist_f) > diis_subspace:
            hist_f.pop(0)
            hist_e.pop(0)
        if len(hist_f) > 1:
            k = len(hist_f)
            E = torch.stack(hist_e, 1)                       # [B, k, N, N]
            Bk = torch.einsum("bkij,blij->bkl", E, E)
            scale = Bk.diagonal(dim1=1, dim2=2).amax(-1).clamp_min(1e-300)
            eye = torch.eye(k, dtype=torch.float64, device=dev)
            Bm = torch.zeros((B, k + 1, k + 1), dtype=torch.float64, device=dev)
            Bm[:, :k, :k] = Bk / scale[:, None, None] + 1e-12 * eye
            Bm[:, :k, k] = 1
            Bm[:, k, :k] = 1
            rhs = torch.zeros((B, k + 1), dtype=torch.float64, device=dev)
            rhs[:, k] = 1
            c = torch.linalg.solve(Bm, rhs)[:, :k]
            F = torch.einsum("bk,bkij->bij", c, torch.stack(hist_f, 1))
        if level_shift > 0 and it >= shift_after:
            shifted = ~done
            sigma = level_shift * shifted.double()
            F = F + sigma[:, None, None] * (Sb - 0.5 * Sb @ Pb @ Sb)
        # diagonalise only the molecules still iterating (a batched eigh of every molecule
        # would dominate the late iterations, when few are left)
        act = torch.nonzero(~done).flatten()
        if act.numel() == B:
            _, C = diag(F)
        else:
            Xa = X.index_select(0, act)
            Fo = Xa.transpose(1, 2) @ F.index_select(0, act) @ Xa + \
                torch.diag_embed(big.index_select(0, act))
            ca = eigh(Fo)
            C = C.clone()
            C.index_copy_(0, act, Xa @ ca)
    return energies, it, done.cpu().numpy(), Pb
