"""Analytic RHF gradients (one-electron derivative terms, ERI adjoint kernel, nuclear
repulsion) against central finite differences of the GPU energy."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _fd(mol_fn, coords, basis, h=1e-4):
    from gaussium_gb300.gradient import rhf_energy_gradient
    g = np.zeros_like(coords)
    for a in range(coords.shape[0]):
        for x in range(3):
            cp, cm = coords.copy(), coords.copy()
            cp[a, x] += h
            cm[a, x] -= h
            ep = rhf_energy_gradient(mol_fn(cp), basis)[0]
            em = rhf_energy_gradient(mol_fn(cm), basis)[0]
            g[a, x] = (ep - em) / (2 * h)
    return g


def test_water_631g_gradient_matches_finite_differences(gpu_lib):
    from gaussium_gb300.molecules import Molecule, water_cluster
    from gaussium_gb300.gradient import rhf_energy_gradient
    base = water_cluster(1, seed=3)
    coords = base.coords.copy()
    coords[1] += np.array([0.05, -0.03, 0.02])        # off equilibrium
    mol_fn = lambda c: Molecule(["O", "H", "H"], c)
    e, g, _ = rhf_energy_gradient(mol_fn(coords), "6-31G")
    gfd = _fd(mol_fn, coords, "6-31G")
    assert np.max(np.abs(g - gfd)) < 1e-6
    assert np.max(np.abs(g.sum(0))) < 1e-8          # translational invariance


@pytest.mark.parametrize("basis", ["6-31G", "6-31G*"])
def test_autograd_function(gpu_lib, monkeypatch, basis):
    """Forward runs the SCF only; backward launches the adjoint kernels on the saved
    density and scales the gradient by the incoming one."""
    import torch
    from gaussium_gb300 import gradient
    from gaussium_gb300.molecules import water_cluster
    calls = []
    real = gradient.gradient_from_state
    monkeypatch.setattr(gradient, "gradient_from_state",
                        lambda st, *args, **kw: calls.append(1) or real(st, *args, **kw))
    m = water_cluster(1, seed=4)
    c = torch.tensor(m.coords, requires_grad=True)
    e = gradient.EnergyGradient.apply(c, m.symbols, basis)
    assert not calls                                   # no gradient work in forward
    (3.0 * e).backward()
    assert len(calls) == 1
    e_ref, g, _ = gradient.rhf_energy_gradient(m, basis)
    assert abs(float(e) - e_ref) < 1e-10
    assert np.allclose(c.grad.numpy(), 3.0 * g, atol=1e-12)


@pytest.mark.parametrize("form", [0, 1, 2])
def test_fused_adjoint_matches_block_path(gpu_lib, form):
    """Default forms, every class with a thread form on threads, every class on warps."""
    from gaussium_gb300 import autotune, build, gradient, molecules
    from gaussium_gb300.engine import JKEngine
    mol = molecules.water_cluster(2, seed=9)
    sb = molecules.shell_basis(mol, "6-31G")
    eng = JKEngine(sb, schwarz_thr=1e-14)
    rng = np.random.default_rng(1)
    a = rng.standard_normal((sb.nbf, sb.nbf))
    P = (a + a.T) / 8
    sa = gradient.shell_atoms(mol, sb)
    classes = [c for c in build.classes() if max(c) <= 1]
    try:
        for c in classes:
            autotune.set_grad_form(c, form if form in autotune.grad_forms(c) else 0)
        g1 = gradient.eri_gradient(sb, eng, sa, P, len(mol.symbols))
    finally:
        for c in classes:
            autotune.set_grad_form(c, 0)
    g2 = gradient.eri_gradient_blocks(sb, eng, sa, P, len(mol.symbols))
    assert np.max(np.abs(g1 - g2)) < 1e-10


def test_one_electron_gradient_kernel_matches_host_assembly(gpu_lib):
    from gaussium_gb300 import gradient, molecules
    mol = molecules.water_cluster(2, seed=12)
    sb = molecules.shell_basis(mol, "6-31G")
    rng = np.random.default_rng(4)
    a = rng.standard_normal((sb.nbf, sb.nbf)); P = (a + a.T) / 8
    b = rng.standard_normal((sb.nbf, sb.nbf)); W = (b + b.T) / 8
    sa = gradient.shell_atoms(mol, sb)
    g1 = gradient.one_electron_gradient_kernel(sb, mol, sa, P, W)
    g2 = gradient.one_electron_gradient(sb, mol, sa, P, W)
    assert np.max(np.abs(g1 - g2)) < 1e-9


@pytest.mark.parametrize("basis", ["6-31G", "6-31G*"])
def test_gradient_parts_against_fixed_density_differences(gpu_lib, basis):
    """Each part of the analytic gradient against central differences of its own energy
    expression with the densities held fixed: the one-electron part
    sum P (T + V) - sum W S (operator and basis-function derivatives), and the
    two-electron part 1/2 sum P (J[P] - K[P]/2) (the ERI adjoint kernels)."""
    from gaussium_gb300 import gradient, molecules
    from gaussium_gb300.engine import JKEngine
    from gaussium_gb300.hamiltonian import one_electron
    from gaussium_gb300.molecules import Molecule
    import torch
    base = molecules.water_cluster(1, seed=3)
    coords = base.coords.copy()
    coords[1] += np.array([0.05, -0.03, 0.02])
    mol = Molecule(["O", "H", "H"], coords)
    st = gradient.rhf_state(mol, basis)
    P, W = st.P, st.W
    sa = gradient.shell_atoms(mol, st.sb)
    g1 = gradient.one_electron_gradient_kernel(st.sb, mol, sa, P, W)
    g2 = gradient.eri_gradient(st.sb, st.engine, sa, P, 3)

    def parts(xyz):
        m = Molecule(["O", "H", "H"], xyz)
        sb = molecules.shell_basis(m, basis)
        S, T, V = one_electron(sb, m.coords, m.charges)
        e1 = float(np.sum(P * (T + V)) - np.sum(W * S))
        eng = JKEngine(sb, schwarz_thr=0.0)
        pt = torch.tensor(P, device="cuda")
        J, (K,) = eng.jk(pt, [pt])
        e2 = 0.5 * float(torch.sum(pt * (J - 0.5 * K)))
        return e1, e2

    h = 1e-4
    for a, x in ((0, 0), (1, 1), (2, 2), (1, 0)):
        xp, xm = coords.copy(), coords.copy()
        xp[a, x] += h
        xm[a, x] -= h
        (p1, p2), (m1, m2) = parts(xp), parts(xm)
        fd1, fd2 = (p1 - m1) / (2 * h), (p2 - m2) / (2 * h)
        assert abs(g1[a, x] - fd1) < 1e-6, ("one-electron", a, x, g1[a, x], fd1)
        assert abs(g2[a, x] - fd2) < 1e-6, ("two-electron", a, x, g2[a, x], fd2)


def test_eri_gradient_per_class_against_differences(gpu_lib):
    """Water / 6-31G*: the fused ERI adjoint of every angular-momentum class on its own
    against central differences of that class's two-electron energy
    1/2 sum P (J[P] - K[P]/2) at fixed density (the same quartet list at every geometry)."""
    import torch
    from gaussium_gb300 import gradient, molecules
    from gaussium_gb300.engine import JKEngine
    from gaussium_gb300.molecules import Molecule
    base = molecules.water_cluster(1, seed=3)
    coords = base.coords.copy()
    coords[1] += np.array([0.05, -0.03, 0.02])
    mol = Molecule(["O", "H", "H"], coords)
    st = gradient.rhf_state(mol, "6-31G*")
    P = st.P
    sb = st.sb
    eng = JKEngine(sb, schwarz_thr=0.0)
    sa = gradient.shell_atoms(mol, sb)
    pt = torch.tensor(P, device="cuda")

    def e2(xyz, cls):
        m = Molecule(["O", "H", "H"], xyz)
        e = JKEngine(molecules.shell_basis(m, "6-31G*"), schwarz_thr=0.0)
        J, (K,) = e.jk(pt, [pt], classes=[cls])
        return 0.5 * float(torch.sum(pt * (J - 0.5 * K)))

    h, bad = 1e-4, []
    for cls, _, _ in eng.segments:
        g = gradient.eri_gradient(sb, eng, sa, P, 3, classes=[cls])
        for a, x in ((0, 0), (1, 1), (2, 2)):
            xp, xm = coords.copy(), coords.copy()
            xp[a, x] += h
            xm[a, x] -= h
            fd = (e2(xp, cls) - e2(xm, cls)) / (2 * h)
            if abs(g[a, x] - fd) > 1e-7:
                bad.append((cls, a, x, float(g[a, x]), fd))
    assert not bad, bad


def test_gradient_split_form_matches_thread_form(gpu_lib):
    """(H2O)2 / 6-31G: the ERI gradient with the heavy quartets of thread-form classes in
    the split form (one warp per quartet) equals the all-thread-form gradient."""
    from gaussium_gb300 import gradient, molecules
    from gaussium_gb300.engine import JKEngine
    mol = molecules.water_cluster(2, seed=2)
    _, _, res = gradient.rhf_energy_gradient(mol, "6-31G")
    sb = molecules.shell_basis(mol, "6-31G")
    eng = JKEngine(sb, schwarz_thr=1e-14)
    assert sum(h[0] for h in eng.heavy) > 0
    sa = gradient.shell_atoms(mol, sb)
    n = len(mol.symbols)
    try:
        gradient.GRAD_SPLIT = True
        g1 = gradient.eri_gradient(sb, eng, sa, res.density, n)
        gradient.GRAD_SPLIT = False
        g0 = gradient.eri_gradient(sb, eng, sa, res.density, n)
    finally:
        gradient.GRAD_SPLIT = True
    assert np.max(np.abs(g1 - g0)) <= 1e-11 * max(1.0, np.max(np.abs(g0)))


@pytest.mark.parametrize("basis", ["6-31G", "6-31G*"])
def test_screened_mixed_gradient_against_fp64(gpu_lib, basis):
    """(H2O)4: the ERI gradient with density screening at 1e-12 and FP32 recursions below
    a density-weighted bound of 1e-3 (thread-form classes; HRR, contraction and sums in
    FP64) against the all-FP64 gradient: within 1e-7 Eh/bohr, well inside the 1e-6 bar
    against finite differences."""
    from gaussium_gb300 import gradient, molecules
    from gaussium_gb300.engine import JKEngine
    mol = molecules.water_cluster(4, seed=4)
    _, _, res = gradient.rhf_energy_gradient(mol, basis)
    sb = molecules.shell_basis(mol, basis)
    eng = JKEngine(sb, schwarz_thr=1e-14)
    sa = gradient.shell_atoms(mol, sb)
    n = len(mol.symbols)
    g64 = gradient.eri_gradient(sb, eng, sa, res.density, n)
    gmx = gradient.eri_gradient(sb, eng, sa, res.density, n, screen_thr=1e-12, mixed_cut=1e-3)
    err = float(np.max(np.abs(gmx - g64)))
    print(f"\n(H2O)4/{basis} screened + mixed ERI gradient vs FP64: max {err:.2e} Eh/bohr")
    assert err <= 1e-7
