"""Generate the golden vectors in ``tests/golden/`` by running the reference Gaussium here.

Run from this directory:  ``python make_golden.py [--quick]``.  It needs the reference
source tree (the GAUSSIUM_REFERENCE environment variable, read by ``ref_harness``) and
writes only ``*.npz`` files beside itself.
The fixtures it writes are committed; the GPU tests read them and never the reference.

Each file records what produced it:

* ``boys.npz``       reference ``boys_function`` (``integrals/boys_function.py:4-54``) on a
                     (v, x) grid, plus 40-digit mpmath values of the same F_v(x).
* ``eri_heh.npz``    the six HeH+ STO-3G quartets of ``test_electron_repulsion_matrix.py``
                     through ObaraSaika, HeadGordonPople and Cook.
* ``h2o_sto3g.npz``  water (O at origin, H at (+-0.757, 0.587, 0) A, converted to bohr),
                     STO-3G: all 406 canonical ERIs (OS), the dense tensor from
                     ``create_repulsion_matrix``, the RHF total energy and iteration count,
                     and reference Fock builds (RHF, UHF, GUHF, KS-J) from a fixed density.
* ``h2o_631gs.npz``  ``examples/molfiles/H2O.mol`` in 6-31G*: all canonical ERIs (OS) and
                     the RHF total energy.
* ``synthetic.npz``  random s/p/d shells (seeded): for every (la,lb,lc,ld) class a few
                     shell quartets, sampled function quartets through ObaraSaika, and a
                     subset through HeadGordonPople and Cook; also the reference's contracted
                     and primitive normalisations of every shell.
* ``synthetic_k6.npz`` the microbench's own contraction range: for every canonical
                     (la lb|lc ld) class two shell quartets, one with K drawn uniform 1-6 per
                     shell in the 10 A cube, one with K = 6 on all four shells in a 1.5 A
                     cube; sampled function quartets through ObaraSaika.
* ``gradient_fd.npz`` reference RHF total energies of water (``examples/molfiles/H2O.mol``
                     with its first hydrogen moved by (0.05, -0.03, 0.02) bohr) in 6-31G and
                     6-31G*, at that geometry and with every coordinate moved by +-1e-4
                     bohr: the reference energy differentiated numerically.  6-31G is the
                     6-31G* file without its D shells.
* ``energies.npz``   reference total energies of test_start.py systems run without
                     point-group symmetry (HeH+ STO-3G RHF, O2 UHF/GUHF STO-3G).
* ``heh_sto3g.npz``, ``o2_sto3g.npz``  their basis functions and S, T, V matrices.
* ``heh_6311pgss.npz``, ``ethene_321g.npz``  the other RHF systems of test_start.py:15-25
                     (HeH+ in 6-311+G**, ethene in 3-21G): reference RHF total energy and
                     SCF iteration count, basis functions, and S, T, V.
* ``co_sto3g.npz``   carbon monoxide in STO-3G (test_start.py:45-49): reference RHF and MP2
                     total energies (their difference is the MP2 correlation energy of
                     moellerplesset/moeller_plesset.py), basis functions, and S, T, V.
"""
import argparse
import contextlib
import io
import itertools
import multiprocessing as mp
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import ref_harness  # noqa: E402

BOHR_PER_ANGSTROM = 1.0 / 0.529177210903
COMPONENTS = {0: [(0, 0, 0)],
              1: [(1, 0, 0), (0, 1, 0), (0, 0, 1)],
              2: [(2, 0, 0), (0, 2, 0), (0, 0, 2), (1, 1, 0), (1, 0, 1), (0, 1, 1)]}


def quiet(fn, *a, **k):
    with contextlib.redirect_stdout(io.StringIO()):
        return fn(*a, **k)


def water_mol_text():
    b = BOHR_PER_ANGSTROM
    return ("0 1\n"
            f"OXYGEN 8 16 0.0 0.0 0.0\n"
            f"HYDROGEN 1 1 {0.757 * b!r} {0.587 * b!r} 0.0\n"
            f"HYDROGEN 1 1 {-0.757 * b!r} {0.587 * b!r} 0.0\n")


def write_tmp(name, text):
    path = os.path.join("/tmp", "gaussium_golden_" + name)
    with open(path, "w") as f:
        f.write(text)
    return path


# ---------------------------------------------------------------- Boys
def make_boys():
    g = ref_harness.load()
    from gaussium.integrals import boys_function
    import mpmath
    mpmath.mp.dps = 40
    xs = np.concatenate([[0.0, 4.802164876034457e-31, 1e-12, 1e-6],
                         np.linspace(0.0, 40.0, 161)[1:],
                         [4.4757221852728435, 12.0769452374367, 24.999, 25.0, 25.001,
                          45.0, 60.0, 100.0, 130.80051761256559, 500.0, 1e3, 1e5, 1e8]])
    vs = np.arange(0, 13)
    ref = np.zeros((len(vs), len(xs)))
    exact = np.zeros((len(vs), len(xs)))
    for i, v in enumerate(vs.tolist()):
        for j, x in enumerate(xs.tolist()):
            ref[i, j] = boys_function(v, x)
            xm = mpmath.mpf(float(x))
            if xm == 0:
                exact[i, j] = 1.0 / (2 * int(v) + 1)
            else:
                # F_v(x) = gamma(v+1/2) * gammainc_lower(v+1/2, x) / (2 x^(v+1/2))
                a = mpmath.mpf(v) + mpmath.mpf(1) / 2
                exact[i, j] = float(mpmath.gammainc(a, 0, xm) / (2 * xm ** a))
    np.savez_compressed(os.path.join(HERE, "boys.npz"), v=vs, x=xs, reference=ref, exact=exact)


# ---------------------------------------------------------------- HeH+ unit-test quartets
def make_heh():
    g = ref_harness.load()
    from gaussium.objects import Basis, PrimitiveBasis
    from gaussium.integrals import ObaraSaika, HeadGordonPople, ElectronRepulsion

    def prim(c, a, r, n):
        p = PrimitiveBasis(c, a, r, (0, 0, 0))
        p.normalisation_memo = n
        return p

    he_r, h_r = (0, 0, 0.7316), (0, 0, -0.7316)
    he = Basis([prim(0.15432897, 9.75393461, he_r, 3.9336432656254527),
                prim(0.53532814, 1.77669115, he_r, 1.0967787981767012),
                prim(0.44463454, 0.48084429, he_r, 0.41154131374122654)], he_r, (0, 0, 0))
    he.normalisation_memo = 1
    h = Basis([prim(0.15432897, 3.42525091, h_r, 1.794441832218435),
               prim(0.53532814, 0.62391373, h_r, 0.5003264923314032),
               prim(0.44463454, 0.16885540, h_r, 0.18773545851092535)], h_r, (0, 0, 0))
    h.normalisation_memo = 1
    basis = [he, h]
    keys = [(0, 0, 0, 0), (1, 0, 0, 0), (1, 0, 1, 0), (1, 1, 0, 0), (1, 1, 1, 0), (1, 1, 1, 1)]
    out = {}
    for name, obj in (("os", ObaraSaika()), ("hgp", HeadGordonPople()), ("cook", ElectronRepulsion())):
        out[name] = np.array([obj.integrate(*[basis[i] for i in k]) for k in keys])
    np.savez_compressed(os.path.join(HERE, "eri_heh.npz"), keys=np.array(keys), **out,
             test_values=np.array([1.3072, 0.4373, 0.1773, 0.6057, 0.3118, 0.7746]))


# ---------------------------------------------------------------- molecules
def load_molecule(mol_path, basis_path):
    g = ref_harness.load()
    from gaussium.common import read_mol_file, read_basis_set_file
    nuclei, electrons, mult = read_mol_file(mol_path)
    basis = read_basis_set_file(basis_path, nuclei)
    return nuclei, electrons, mult, basis


def basis_arrays(basis):
    """Flatten reference Basis objects: per function centre, lmn, contracted norm and
    primitives (coef, exponent, primitive norm), padded to the largest K."""
    n = len(basis)
    kmax = max(len(b.primitive_gaussian_array) for b in basis)
    centre = np.array([b.coordinates for b in basis], dtype=np.float64)
    lmn = np.array([b.integral_exponents for b in basis], dtype=np.int64)
    norm = np.array([b.normalisation for b in basis], dtype=np.float64)
    nprim = np.array([len(b.primitive_gaussian_array) for b in basis], dtype=np.int64)
    coef = np.zeros((n, kmax)); expo = np.zeros((n, kmax)); pnorm = np.zeros((n, kmax))
    for i, b in enumerate(basis):
        for k, p in enumerate(b.primitive_gaussian_array):
            coef[i, k] = p.contraction
            expo[i, k] = p.exponent
            pnorm[i, k] = p.normalisation
    return dict(centre=centre, lmn=lmn, norm=norm, nprim=nprim, coef=coef, expo=expo, pnorm=pnorm)


_WORK = {}


def _eri_worker(key):
    basis = _WORK["basis"]
    obj = _WORK["integral"]
    return obj.integrate(*[basis[i] for i in key])


def canonical_keys(n):
    return [(a, b, c, d) for a, b, c, d in itertools.product(range(n), repeat=4)
            if not (a > b or c > d or a > c or (a == c and b > d))]


def eri_all(basis, procs):
    g = ref_harness.load()
    from gaussium.integrals import ObaraSaika
    keys = canonical_keys(len(basis))
    _WORK["basis"] = basis
    _WORK["integral"] = ObaraSaika()
    with mp.get_context("fork").Pool(procs) as pool:
        vals = pool.map(_eri_worker, keys, chunksize=64)
    return np.array(keys, dtype=np.int16), np.array(vals)


def run_rhf(nuclei, electrons, basis, procs):
    """Reference RHF total energy through ``Energy.calculate_energy`` (energy/energy.py:24-81)
    with the SCF iteration count taken from the printed SCF lines."""
    g = ref_harness.load()
    from gaussium.energy import Energy
    energy = Energy(electrons, 1, procs, 'RHF')
    energy.symmetry_object = ref_harness.c1_symmetry(basis)
    buf = io.StringIO()
    with contextlib.redirect_stdout(buf):
        e = energy.calculate_energy(nuclei, basis)
    iters = sum(1 for line in buf.getvalue().splitlines() if line.startswith('SCF ENERGY: '))
    return float(e), iters


def make_h2o_sto3g(procs):
    g = ref_harness.load()
    from gaussium.matrixelements import TwoElectronRepulsionMatrixOS
    from gaussium.hartreefock import (FockMatrixRestricted, FockMatrixUnrestricted,
                                      BlockedFockMatrixUnrestricted)
    from gaussium.kohnsham.kohn_sham_hamiltonian import RestrictedKohnShamHamiltonian
    from gaussium.matrixelements import blocked_spin_basis_set
    mol = write_tmp("h2o.mol", water_mol_text())
    nuclei, electrons, mult, basis = load_molecule(mol, f"{ref_harness.reference_root()}/examples/basissets/STO-3G.gbs")
    keys, vals = eri_all(basis, procs)
    dense = quiet(TwoElectronRepulsionMatrixOS(basis, ref_harness.c1_symmetry(basis), 1).create_repulsion_matrix)
    dense = np.asarray(dense)
    energy, iters = run_rhf(nuclei, electrons, basis, procs)
    n = len(basis)
    rng = np.random.default_rng(7)
    a = rng.standard_normal((n, n)); pa = (a + a.T) / 4
    b = rng.standard_normal((n, n)); pb = (b + b.T) / 4
    hcore = np.zeros((n, n))
    f_rhf = FockMatrixRestricted(hcore, dense).create(pa)
    f_ua, f_ub = FockMatrixUnrestricted(hcore, dense).create(pa, pb)
    big = np.block([[pa, np.zeros((n, n))], [np.zeros((n, n)), pb]])
    f_guhf = BlockedFockMatrixUnrestricted(np.zeros((2 * n, 2 * n)),
                                           np.asarray(blocked_spin_basis_set(dense))).create(big)
    ks = RestrictedKohnShamHamiltonian(hcore, dense, None)
    j_ks = ks.create_matrix(lambda i, j: sum(pa.item(x, y) * dense.item(i, j, x, y)
                                             for x in range(n) for y in range(n)))
    np.savez_compressed(os.path.join(HERE, "h2o_sto3g.npz"), keys=keys, eri=vals, dense=dense,
             energy=energy, iterations=iters, electrons=electrons,
             coords=np.array([x.coordinates for x in nuclei]),
             charges=np.array([x.charge for x in nuclei]),
             density_a=pa, density_b=pb, fock_rhf=f_rhf, fock_uhf_a=f_ua, fock_uhf_b=f_ub,
             fock_guhf=f_guhf, coulomb_ks=j_ks, **one_electron(nuclei, basis),
             **basis_arrays(basis))


def one_electron(nuclei, basis):
    """Reference S, T and V matrices (matrixelements/*_matrix.py)."""
    g = ref_harness.load()
    from gaussium.matrixelements import (OrbitalOverlapMatrix, KineticEnergyMatrix,
                                         NuclearAttractionMatrix)
    return dict(overlap=OrbitalOverlapMatrix(basis).create(),
                kinetic=KineticEnergyMatrix(basis).create(),
                nuclear=NuclearAttractionMatrix(basis, nuclei).create())


def make_h2o_631gs(procs):
    nuclei, electrons, mult, basis = load_molecule(f"{ref_harness.reference_root()}/examples/molfiles/H2O.mol",
                                                   f"{ref_harness.reference_root()}/examples/basissets/6-31GP.gbs")
    keys, vals = eri_all(basis, procs)
    energy, iters = run_rhf(nuclei, electrons, basis, procs)
    np.savez_compressed(os.path.join(HERE, "h2o_631gs.npz"), keys=keys, eri=vals, energy=energy,
             **one_electron(nuclei, basis),
             iterations=iters, electrons=electrons,
             coords=np.array([x.coordinates for x in nuclei]),
             charges=np.array([x.charge for x in nuclei]), **basis_arrays(basis))


# ---------------------------------------------------------------- synthetic shells
def synthetic_shell(rng, l, kmax, box=10.0):
    k = int(rng.integers(1, kmax + 1))
    expo = np.exp(rng.uniform(np.log(0.05), np.log(1e4), size=k))
    coef = rng.standard_normal(k)
    centre = rng.uniform(0.0, box, size=3) * BOHR_PER_ANGSTROM
    # Two of every four shells share a centre with another one, so that the
    # one-centre and two-centre special cases of the recursions are exercised.
    return dict(l=l, expo=expo, coef=coef, centre=centre)


def reference_functions(shell):
    g = ref_harness.load()
    from gaussium.objects import Basis, PrimitiveBasis
    c = tuple(float(x) for x in shell["centre"])
    out = []
    for lmn in COMPONENTS[shell["l"]]:
        prims = [PrimitiveBasis(float(cf), float(ex), c, lmn)
                 for cf, ex in zip(shell["coef"], shell["expo"])]
        out.append(Basis(prims, c, lmn))
    return out


def _synthetic_worker(task):
    qi, shells, comp, which = task
    g = ref_harness.load()
    from gaussium.integrals import ObaraSaika, HeadGordonPople, ElectronRepulsion
    funcs = [reference_functions(s) for s in shells]
    fq = [funcs[x][comp[x]] for x in range(4)]
    obj = {"os": ObaraSaika, "hgp": HeadGordonPople, "cook": ElectronRepulsion}[which]()
    t = time.perf_counter()
    v = obj.integrate(*fq)
    return qi, which, v, time.perf_counter() - t


def make_synthetic(procs, quick):
    rng = np.random.default_rng(20261203)
    shells = []
    quartets = []
    classes = list(itertools.product(range(3), repeat=4))
    for cls in classes:
        ltot = sum(cls)
        nq = 3 if ltot <= 6 else 2
        for rep in range(nq):
            kmax = 4 if ltot <= 4 else (3 if ltot <= 6 else 2)
            # rep 0: the microbench's 10 A cube; rep 1: 1.5 A cube with shared centres;
            # rep 2: 1.5 A cube, four distinct centres.
            box = 10.0 if rep == 0 else 1.5
            sh = [synthetic_shell(rng, l, kmax, box) for l in cls]
            if rep == 1:
                sh[1]["centre"] = sh[0]["centre"].copy()      # (aa|cd)-type centres
                sh[3]["centre"] = sh[2]["centre"].copy()
            if cls == (2, 2, 2, 2):
                sh[2]["centre"] = sh[0]["centre"].copy()      # one-centre bra/ket overlap
            base = len(shells)
            shells.extend(sh)
            quartets.append([base, base + 1, base + 2, base + 3])
    # sampled function quartets
    samples = []
    for qi, q in enumerate(quartets):
        ls = [shells[s]["l"] for s in q]
        ncomp = [len(COMPONENTS[l]) for l in ls]
        nsamp = min(int(np.prod(ncomp)), 6 if sum(ls) <= 6 else 3)
        all_comp = list(itertools.product(*[range(n) for n in ncomp]))
        pick = rng.choice(len(all_comp), size=nsamp, replace=False)
        for p in pick:
            samples.append((qi, all_comp[p]))
    tasks = []
    for si, (qi, comp) in enumerate(samples):
        sh = [shells[s] for s in quartets[qi]]
        tasks.append((si, sh, comp, "os"))
        if si % 3 == 0 and not quick:
            tasks.append((si, sh, comp, "hgp"))
        if si % 5 == 0 and sum(s["l"] for s in sh) <= 4 and not quick:
            tasks.append((si, sh, comp, "cook"))
    with mp.get_context("fork").Pool(procs) as pool:
        res = pool.map(_synthetic_worker, tasks, chunksize=1)
    val = {w: np.full(len(samples), np.nan) for w in ("os", "hgp", "cook")}
    sec = np.zeros(len(samples))
    for si, which, v, dt in res:
        val[which][si] = v
        if which == "os":
            sec[si] = dt
    # reference normalisations of every synthetic shell component
    kmax = max(len(s["expo"]) for s in shells)
    nsh = len(shells)
    sh_l = np.array([s["l"] for s in shells]); sh_k = np.array([len(s["expo"]) for s in shells])
    sh_c = np.array([s["centre"] for s in shells])
    sh_e = np.zeros((nsh, kmax)); sh_cf = np.zeros((nsh, kmax))
    cnorm = np.zeros((nsh, 6)); pnorm = np.zeros((nsh, 6, kmax))
    for i, s in enumerate(shells):
        sh_e[i, :len(s["expo"])] = s["expo"]; sh_cf[i, :len(s["coef"])] = s["coef"]
        for ci, f in enumerate(reference_functions(s)):
            cnorm[i, ci] = f.normalisation
            for k, p in enumerate(f.primitive_gaussian_array):
                pnorm[i, ci, k] = p.normalisation
    np.savez_compressed(os.path.join(HERE, "synthetic.npz"), shell_l=sh_l, shell_k=sh_k, shell_centre=sh_c,
             shell_expo=sh_e, shell_coef=sh_cf, contracted_norm=cnorm, primitive_norm=pnorm,
             quartets=np.array(quartets), sample_quartet=np.array([s[0] for s in samples]),
             sample_comp=np.array([s[1] for s in samples]), os=val["os"], hgp=val["hgp"],
             cook=val["cook"], os_seconds=sec)


def make_synthetic_k6(procs):
    """Sampled function quartets of shells with the microbench's contraction degrees
    (K = 1-6, and K = 6 on every shell), one pair of shell quartets per canonical class."""
    rng = np.random.default_rng(20261204)
    shells, quartets = [], []
    pairs = [(0, 0), (1, 0), (1, 1), (2, 0), (2, 1), (2, 2)]
    classes = [p + q for i, p in enumerate(pairs) for q in pairs[:i + 1]]
    for cls in classes:
        for rep in range(2):
            if rep == 0:
                sh = [synthetic_shell(rng, l, 6, 10.0) for l in cls]
            else:
                sh = []
                for l in cls:
                    s = synthetic_shell(rng, l, 1, 1.5)
                    s["expo"] = np.exp(rng.uniform(np.log(0.05), np.log(1e4), size=6))
                    s["coef"] = rng.standard_normal(6)
                    sh.append(s)
            base = len(shells)
            shells.extend(sh)
            quartets.append([base, base + 1, base + 2, base + 3])
    samples = []
    for qi, q in enumerate(quartets):
        ls = [shells[s]["l"] for s in q]
        ncomp = [len(COMPONENTS[l]) for l in ls]
        nsamp = min(int(np.prod(ncomp)), 4 if sum(ls) <= 5 else 2)
        all_comp = list(itertools.product(*[range(n) for n in ncomp]))
        for p in rng.choice(len(all_comp), size=nsamp, replace=False):
            samples.append((qi, all_comp[p]))
    tasks = [(si, [shells[s] for s in quartets[qi]], comp, "os")
             for si, (qi, comp) in enumerate(samples)]
    # longest first, so the pool does not end on one (dd|dd) K=6 quartet
    tasks.sort(key=lambda t: -sum(s["l"] for s in t[1]) * np.prod([len(s["expo"]) for s in t[1]]))
    with mp.get_context("fork").Pool(procs) as pool:
        res = pool.map(_synthetic_worker, tasks, chunksize=1)
    val = np.full(len(samples), np.nan)
    sec = np.zeros(len(samples))
    for si, which, v, dt in res:
        val[si], sec[si] = v, dt
    nsh = len(shells)
    sh_l = np.array([s["l"] for s in shells]); sh_k = np.array([len(s["expo"]) for s in shells])
    sh_c = np.array([s["centre"] for s in shells])
    sh_e = np.zeros((nsh, 6)); sh_cf = np.zeros((nsh, 6))
    for i, s in enumerate(shells):
        sh_e[i, :len(s["expo"])] = s["expo"]; sh_cf[i, :len(s["coef"])] = s["coef"]
    np.savez_compressed(os.path.join(HERE, "synthetic_k6.npz"), shell_l=sh_l, shell_k=sh_k,
                        shell_centre=sh_c, shell_expo=sh_e, shell_coef=sh_cf,
                        quartets=np.array(quartets),
                        sample_quartet=np.array([s[0] for s in samples]),
                        sample_comp=np.array([s[1] for s in samples]), os=val, os_seconds=sec)


FD_STEP = 1e-4
FD_SHIFT = (0.05, -0.03, 0.02)


def _without_d_shells(path):
    out, skip = [], False
    for line in open(path).read().splitlines():
        w = line.split()
        if w and w[0] in ("S", "L", "P", "D", "F") and len(w) == 2:
            skip = w[0] == "D"
        elif not line.strip() or line.startswith("#"):
            skip = False
        if not skip:
            out.append(line)
    return write_tmp("631g.gbs", "\n".join(out) + "\n")


def _mol_text(symbols, z, coords):
    lines = ["0 1"]
    for sym, zz, c in zip(symbols, z, coords):
        mass = {1: 1, 8: 16}[zz]
        lines.append(f"{sym} {zz} {mass} {float(c[0])!r} {float(c[1])!r} {float(c[2])!r}")
    return "\n".join(lines) + "\n"


def make_gradient_fd(procs):
    root = ref_harness.reference_root()
    basis_files = {"6-31G*": f"{root}/examples/basissets/6-31GP.gbs"}
    basis_files["6-31G"] = _without_d_shells(basis_files["6-31G*"])
    symbols, z = ["OXYGEN", "HYDROGEN", "HYDROGEN"], [8, 1, 1]
    x0 = np.array([[0.0, -0.143225816552, 0.0], [1.638036840407, 1.136548822547, 0.0],
                   [-1.638036840407, 1.136548822547, 0.0]])
    x0[1] += np.array(FD_SHIFT)
    out = dict(coords=x0, charges=np.array(z, dtype=np.float64), step=FD_STEP)
    for name, gbs in basis_files.items():
        tag = name.replace("*", "s").replace("-", "")
        e = np.zeros((3, 3, 2))
        for a in range(3):
            for k in range(3):
                for si, sign in enumerate((1.0, -1.0)):
                    x = x0.copy()
                    x[a, k] += sign * FD_STEP
                    mol = write_tmp("fd.mol", _mol_text(symbols, z, x))
                    nuclei, electrons, _, basis = load_molecule(mol, gbs)
                    e[a, k, si] = run_rhf(nuclei, electrons, basis, procs)[0]
        nuclei, electrons, _, basis = load_molecule(write_tmp("fd.mol", _mol_text(symbols, z, x0)), gbs)
        out[f"energy_{tag}"] = run_rhf(nuclei, electrons, basis, procs)[0]
        out[f"displaced_{tag}"] = e
        out[f"fd_gradient_{tag}"] = (e[..., 0] - e[..., 1]) / (2 * FD_STEP)
    np.savez_compressed(os.path.join(HERE, "gradient_fd.npz"), **out)


# ---------------------------------------------------------------- energies of test_start systems
def make_energies(procs):
    g = ref_harness.load()
    from gaussium.energy import Energy
    from gaussium.hartreefock import RestrictedHF
    out = {}
    d = f"{ref_harness.reference_root()}/tests/testslow/start"
    nuclei, electrons, mult, basis = load_molecule(f"{d}/HeH+.mol", f"{d}/STO-3G.gbs")
    out["heh_sto3g_rhf"], out["heh_sto3g_rhf_iterations"] = run_rhf(nuclei, electrons, basis, procs)
    np.savez_compressed(os.path.join(HERE, "heh_sto3g.npz"), electrons=electrons, multiplicity=mult,
                        coords=np.array([x.coordinates for x in nuclei]),
                        charges=np.array([x.charge for x in nuclei]),
                        **one_electron(nuclei, basis), **basis_arrays(basis))
    for method in ("UHF", "GUHF"):
        nuclei, electrons, mult, basis = load_molecule(f"{d}/O2.mol", f"{d}/STO-3G.gbs")
        energy = Energy(electrons, mult, procs, method)
        energy.symmetry_object = ref_harness.c1_symmetry(basis)
        out[f"o2_sto3g_{method.lower()}"] = float(quiet(energy.calculate_energy, nuclei, basis))
    np.savez_compressed(os.path.join(HERE, "o2_sto3g.npz"), electrons=electrons, multiplicity=mult,
                        coords=np.array([x.coordinates for x in nuclei]),
                        charges=np.array([x.charge for x in nuclei]),
                        **one_electron(nuclei, basis), **basis_arrays(basis))
    np.savez_compressed(os.path.join(HERE, "energies.npz"), **out)


def make_start_rhf(procs):
    ref_harness.load()
    d = f"{ref_harness.reference_root()}/tests/testslow/start"
    for tag, mol, gbs in (("heh_6311pgss", "HeH+.mol", "6-311+GPP.gbs"),
                          ("ethene_321g", "C2H4.mol", "3-21G.gbs")):
        nuclei, electrons, mult, basis = load_molecule(f"{d}/{mol}", f"{d}/{gbs}")
        energy, iterations = run_rhf(nuclei, electrons, basis, procs)
        np.savez_compressed(os.path.join(HERE, f"{tag}.npz"), energy=energy,
                            iterations=iterations, electrons=electrons, multiplicity=mult,
                            coords=np.array([x.coordinates for x in nuclei]),
                            charges=np.array([x.charge for x in nuclei]),
                            **one_electron(nuclei, basis), **basis_arrays(basis))
        print(f"{tag}: {len(basis)} functions, E = {energy:.10f} in {iterations} iterations",
              flush=True)


def make_start_mp2(procs):
    g = ref_harness.load()
    from gaussium.energy import Energy
    d = f"{ref_harness.reference_root()}/tests/testslow/start"
    nuclei, electrons, mult, basis = load_molecule(f"{d}/CO.mol", f"{d}/STO-3G.gbs")
    energy_rhf, iterations = run_rhf(nuclei, electrons, basis, procs)
    energy = Energy(electrons, mult, procs, "MP2")
    energy.symmetry_object = ref_harness.c1_symmetry(basis)
    energy_mp2 = float(quiet(energy.calculate_energy, nuclei, basis))
    np.savez_compressed(os.path.join(HERE, "co_sto3g.npz"), energy_rhf=energy_rhf,
                        energy_mp2=energy_mp2, iterations=iterations, electrons=electrons,
                        multiplicity=mult, coords=np.array([x.coordinates for x in nuclei]),
                        charges=np.array([x.charge for x in nuclei]),
                        **one_electron(nuclei, basis), **basis_arrays(basis))
    print(f"co_sto3g: {len(basis)} functions, RHF {energy_rhf:.10f}, MP2 {energy_mp2:.10f}",
          flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--quick", action="store_true")
    ap.add_argument("--only", default="")
    ap.add_argument("--procs", type=int, default=os.cpu_count())
    args = ap.parse_args()
    ref_harness.load()
    steps = {"boys": make_boys, "heh": make_heh,
             "h2o_sto3g": lambda: make_h2o_sto3g(args.procs),
             "h2o_631gs": lambda: make_h2o_631gs(args.procs),
             "synthetic": lambda: make_synthetic(args.procs, args.quick),
             "synthetic_k6": lambda: make_synthetic_k6(args.procs),
             "gradient_fd": lambda: make_gradient_fd(args.procs),
             "energies": lambda: make_energies(args.procs),
             "start_rhf": lambda: make_start_rhf(args.procs),
             "start_mp2": lambda: make_start_mp2(args.procs)}
    for name, fn in steps.items():
        if args.only and name not in args.only.split(","):
            continue
        t = time.time()
        fn()
        print(f"{name}: {time.time() - t:.1f}s", flush=True)


if __name__ == "__main__":
    main()
