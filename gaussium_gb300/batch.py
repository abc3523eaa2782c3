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
from .engine import PAIR_ORDER, PRIM_SCREEN, DeviceShells, PairSet, _pc_lut
from .hamiltonian import one_electron
from .molecules import shell_basis


class BatchedRHF:
    def __init__(self, molecules, basis="6-31G*", schwarz_thr=1e-12, device="cuda",
                 max_exp=PRIM_SCREEN):
        self.mols = molecules
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
        self._tasks(q.cpu().numpy(), pc, pair_mol, schwarz_thr)
        # one-electron matrices, orthogonalisers, padded index maps
        self.S, self.H = [], []
        for m, (mol, sb) in enumerate(zip(molecules, sbs)):
            S, T, V = one_electron(sb, mol.coords, mol.charges)
            self.S.append(S)
            self.H.append(T + V)
        self._padded_setup()
        self.graph = None

    def _tasks(self, q, pc, pair_mol, thr):
        nprim = self.pairs.nprim
        out = {}
        for m in range(len(self.sbs)):
            pm = np.flatnonzero(pair_mol == m)
            for cb in range(len(PAIR_ORDER)):
                bra = pm[pc[pm] == cb]
                if len(bra) == 0:
                    continue
                for ck in range(cb + 1):
                    ket = pm[pc[pm] == ck]
                    if len(ket) == 0:
                        continue
                    bi, ki = np.meshgrid(bra, ket, indexing="ij")
                    bi, ki = bi.ravel(), ki.ravel()
                    keep = q[bi] * q[ki] >= thr
                    if cb == ck:
                        keep &= bi >= ki
                    out.setdefault((cb, ck), []).append(np.stack([bi[keep], ki[keep]], 1))
        segs, chunks, n = [], [], 0
        for (cb, ck), lst in sorted(out.items()):
            tk = np.concatenate(lst)
            if len(tk) == 0:
                continue
            order = np.lexsort((nprim[tk[:, 1]], nprim[tk[:, 0]]))
            tk = tk[order]
            (la, lb), (lc, ld) = PAIR_ORDER[cb], PAIR_ORDER[ck]
            segs.append(((la, lb, lc, ld), n, n + len(tk)))
            chunks.append(tk)
            n += len(tk)
        self.segments = segs
        self.ntasks = n
        self.tasks = torch.as_tensor(np.concatenate(chunks).astype(np.int32)).to(self.dev)

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
        S = torch.zeros((B, N, N), dtype=torch.float64, device=dev)
        H = torch.zeros_like(S)
        for m, n in enumerate(self.nbf):
            S[m, :n, :n] = torch.as_tensor(self.S[m]).to(dev)
            H[m, :n, :n] = torch.as_tensor(self.H[m]).to(dev)
            S[m, n:, n:] = torch.eye(N - n, dtype=torch.float64, device=dev)
        self.Sb, self.Hb = S, H
        # canonical orthogonaliser per molecule (eigenvalues ascending, as the reference
        # sorts them); padded orbitals are zero columns at positions n..N-1
        X = torch.zeros_like(S)
        for m, n in enumerate(self.nbf):
            s, u = torch.linalg.eigh(S[m, :n, :n])
            X[m, :n, :n] = u * s.rsqrt().unsqueeze(0)
        self.X = X
        self.nocc = torch.as_tensor([mol.electrons // 2 for mol in self.mols], device=dev)
        self.occ_mask = (torch.arange(N, device=dev)[None, :] < self.nocc[:, None]).double()
        self.pad_orb = torch.zeros((B, N), dtype=torch.float64, device=dev)
        for m, n in enumerate(self.nbf):
            self.pad_orb[m, n:] = 1.0

    def to_packed(self, Pb):
        out = torch.zeros(self.mat_stride, dtype=torch.float64, device=self.dev)
        out.index_copy_(0, self.pos_packed, Pb.reshape(-1).index_select(0, self.pos_padded))
        return out

    def to_padded(self, v):
        Pb = torch.zeros(len(self.sbs) * self.nmax * self.nmax, dtype=torch.float64, device=self.dev)
        Pb.index_copy_(0, self.pos_padded, v.index_select(0, self.pos_packed))
        return Pb.view(len(self.sbs), self.nmax, self.nmax)

    def _jk_launch(self, P, J, K, precision=64, mixed_cut=None, dmax=None):
        L = _lib.lib()
        st = _lib.stream()
        base = self.tasks.data_ptr()
        runs = [(precision, 0.0, float("inf"), 0.0)]
        if mixed_cut is not None:
            runs = [(64, mixed_cut, float("inf"), 1e-300), (32, 0.0, mixed_cut, 1e-300)]
        for prec, lo, hi, thr in runs:
            prims = self.pairs.prims(prec)
            for cls, s, e in self.segments:
                rc = L.gs_fock_jk_batched(*cls, prec, _lib.ptr(self.pairs.rec), _lib.ptr(prims),
                                          _lib.ptr(self.ds.comp_scale), _lib.ptr(self.local_fo),
                                          _lib.ptr(self.shell_mol), _lib.ptr(self.mol_base),
                                          _lib.ptr(self.mol_n), _lib.ptr(dmax), self.mat_stride,
                                          e - s, base + s * 8, _lib.ptr(P), _lib.ptr(J), 1,
                                          _lib.ptr(P), _lib.ptr(K), thr, lo, hi, st)
                _lib.check(rc, f"gs_fock_jk_batched{cls}")

    def fock_packed(self, P, precision=64, mixed_cut=None):
        """G = J - K/2 (packed, symmetric) for packed densities P, all molecules."""
        J = torch.zeros_like(P)
        K = torch.zeros_like(P)
        dmax = None
        if mixed_cut is not None:
            Pb = self.to_padded(P).abs().amax(dim=(1, 2))
            dmax = Pb.contiguous()
        self._jk_launch(P, J, K, precision, mixed_cut, dmax)
        Jb, Kb = self.to_padded(J), self.to_padded(K)
        G = (Jb + Jb.transpose(1, 2)) - 0.5 * (Kb + Kb.transpose(1, 2))
        return G

    def run(self, threshold=1e-10, max_iter=60, mixed_cut=None, use_graph=True):
        """Batched SCF; returns total energies (numpy) and the iteration count."""
        dev = self.dev
        B, N = len(self.sbs), self.nmax
        P_static = torch.zeros(self.mat_stride, dtype=torch.float64, device=dev)
        G_static = None

        def build():
            return self.fock_packed(P_static, mixed_cut=mixed_cut)

        if use_graph:
            build()                                  # warm-up outside capture
            torch.cuda.synchronize()
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g):
                G_static = build()
            self.graph = g
        Xb, Hb, Sb = self.X, self.Hb, self.Sb
        big = 1e6 * self.pad_orb

        def diag(F):
            Fo = Xb.transpose(1, 2) @ F @ Xb + torch.diag_embed(big)
            e, c = torch.linalg.eigh(Fo)
            return e, Xb @ c

        e_orb, C = diag(Hb)
        prev = torch.zeros(B, dtype=torch.float64, device=dev)
        hist_f, hist_e = [], []
        energies = None
        for it in range(1, max_iter + 1):
            Cocc = C * self.occ_mask[:, None, :]
            Pb = 2.0 * Cocc @ Cocc.transpose(1, 2)
            P_static.copy_(self.to_packed(Pb))
            if use_graph:
                self.graph.replay()
                G = G_static
            else:
                G = build()
            F = Hb + G
            energies = 0.5 * torch.sum(Pb * (Hb + F), dim=(1, 2))
            de = (energies - prev).abs()
            prev = energies
            if it > 1 and bool((de < threshold).all()):
                break
            err = Sb @ Pb @ F - F @ Pb @ Sb
            err = Xb.transpose(1, 2) @ err @ Xb
            hist_f.append(F)
            hist_e.append(err)
            if len(hist_f) > 8:
                hist_f.pop(0)
                hist_e.pop(0)
            if len(hist_f) > 1:
                k = len(hist_f)
                Bm = torch.zeros((B, k + 1, k + 1), dtype=torch.float64, device=dev)
                E = torch.stack(hist_e, 1)                       # [B, k, N, N]
                Bm[:, :k, :k] = torch.einsum("bkij,blij->bkl", E, E)
                Bm[:, :k, k] = 1
                Bm[:, k, :k] = 1
                rhs = torch.zeros((B, k + 1), dtype=torch.float64, device=dev)
                rhs[:, k] = 1
                c = torch.linalg.solve(Bm, rhs)[:, :k]
                F = torch.einsum("bk,bkij->bij", c, torch.stack(hist_f, 1))
            e_orb, C = diag(F)
        e_nuc = torch.as_tensor([m.nuclear_repulsion() for m in self.mols], device=dev)
        return (energies + e_nuc).cpu().numpy(), it
