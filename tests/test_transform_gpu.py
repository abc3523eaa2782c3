"""AO -> MO transform and spin-orbital expansions on the GPU against the reference's own
outputs (tests/golden/mo_transform.npz, made by tests/golden/make_mo_golden.py) and the
oracle's restatements of matrixelements/transformations.py, plus size-independent
properties at sizes the oracle cannot reach."""
import numpy as np
import pytest
import torch

import oracle
from conftest import golden
from molecules import load

pytestmark = pytest.mark.gpu


def random_symmetric_eri(n, seed):
    """A tensor with the 8-fold permutational symmetry of real (ab|cd)."""
    rng = np.random.default_rng(seed)
    x = rng.standard_normal((n, n, n, n))
    x = x + x.transpose(1, 0, 2, 3)
    x = x + x.transpose(0, 1, 3, 2)
    return x + x.transpose(2, 3, 0, 1)


def test_golden_molecular_orbitals_mutates_and_returns_its_argument(gpu_lib):
    from gaussium_gb300 import transform
    g = golden("mo_transform")
    ao = g["ao"].copy()
    out = transform.molecular_orbitals(ao, g["coefficients"])
    assert out is ao
    assert np.max(np.abs(out - g["mo"])) < 1e-13


def test_molecular_orbitals_other_input_layouts(gpu_lib):
    """Fortran-ordered input is still overwritten and returned; a read-only input is left
    alone and a new array returned; a nested list gives an array."""
    from gaussium_gb300 import transform
    g = golden("mo_transform")
    f = np.asfortranarray(g["ao"])
    assert transform.molecular_orbitals(f, g["coefficients"]) is f
    assert np.max(np.abs(f - g["mo"])) < 1e-13
    ro = g["ao"].copy()
    ro.flags.writeable = False
    out = transform.molecular_orbitals(ro, g["coefficients"])
    assert out is not ro and np.array_equal(ro, g["ao"])
    assert np.max(np.abs(out - g["mo"])) < 1e-13
    out = transform.molecular_orbitals(g["ao"].tolist(), g["coefficients"])
    assert isinstance(out, np.ndarray) and np.max(np.abs(out - g["mo"])) < 1e-13


def test_golden_spin_expansions_exact(gpu_lib):
    from gaussium_gb300 import transform
    g = golden("mo_transform")
    assert np.array_equal(transform.spin_basis_set(g["mo"]), g["spin"])
    assert np.array_equal(transform.blocked_spin_basis_set(g["mo"]), g["blocked"])
    assert np.array_equal(transform.spin_basis_anti_physicist(g["mo"]), g["anti"])


@pytest.mark.parametrize("symmetric", [True, False])
@pytest.mark.parametrize("n,m", [(1, 1), (13, 13), (24, 24), (20, 11)])
def test_transform_matches_oracle(gpu_lib, n, m, symmetric):
    """Square and rectangular (fewer orbitals than functions) coefficient matrices; a
    tensor with the integrals' symmetry (pair-packed form) and one without (general)."""
    from gaussium_gb300 import transform
    ao = random_symmetric_eri(n, seed=n)
    if not symmetric:
        ao = ao + np.random.default_rng(50 + n).standard_normal(ao.shape) * 1e-3
    c = np.random.default_rng(100 + n).standard_normal((n, m)) / np.sqrt(n)
    got = transform.transform_device(torch.tensor(ao, device="cuda"),
                                     torch.tensor(c, device="cuda")).cpu().numpy()
    if m == n:
        ref = oracle.molecular_orbitals(ao, c)
    else:
        ref = np.einsum("abcd,ap,bq,cr,ds->pqrs", ao, c, c, c, c, optimize=True)
    assert np.max(np.abs(got - ref)) <= 1e-12 * max(1.0, np.max(np.abs(ref)))


@pytest.mark.parametrize("h", [1, 2, 5, 8, 9])
def test_spin_expansions_match_oracle(gpu_lib, h):
    from gaussium_gb300 import transform
    mo = random_symmetric_eri(h, seed=7 * h)
    for fn, ref_fn in ((transform.spin_basis_set, oracle.spin_basis_set),
                       (transform.blocked_spin_basis_set, oracle.blocked_spin_basis_set),
                       (transform.spin_basis_anti_physicist, oracle.spin_basis_anti_physicist)):
        assert np.array_equal(fn(mo), ref_fn(mo)), (fn.__name__, h)


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_spin_expand_unaligned_output_matches_aligned(gpu_lib, mode):
    """An output 8 bytes off a 16-byte boundary takes the scalar kernel; it must agree
    with the 16-byte-pair kernel element for element."""
    from gaussium_gb300 import _lib, transform
    h = 11
    mo = torch.tensor(random_symmetric_eri(h, seed=99), device="cuda")
    want = transform.spin_expand_device(mo, mode)
    buf = torch.full(((2 * h) ** 4 + 2,), 7.0, dtype=torch.float64, device="cuda")
    out = buf[1:1 + (2 * h) ** 4]
    assert out.data_ptr() % 16 == 8
    _lib.check(gpu_lib.gs_spin_expand(_lib.ptr(mo), h, mode, _lib.ptr(out), _lib.stream()), "spin")
    assert torch.equal(out.view(want.shape), want)
    assert buf[0].item() == 7.0 and buf[-1].item() == 7.0


def test_water_mo_integrals_from_shells(gpu_lib):
    """Shells -> dense AO tensor -> MO tensor without leaving the device, against the
    reference's MO tensor of the same coefficients."""
    from gaussium_gb300 import transform
    from gaussium_gb300.basis import ShellBasis
    g = golden("mo_transform")
    _, funcs, _ = load("h2o_sto3g")
    mo = transform.mo_integrals(ShellBasis.from_functions(funcs), g["coefficients"])
    assert np.max(np.abs(mo.cpu().numpy() - g["mo"])) < 1e-10


def test_spin_expand_properties_at_size(gpu_lib):
    """h = 64 (128 spin orbitals, 2 GiB per tensor): every element against its source by
    index arithmetic on the device, and the antisymmetry of <rs||tu>."""
    from gaussium_gb300 import transform
    h = 64
    torch.manual_seed(3)
    mo = torch.randn((h,) * 4, dtype=torch.float64, device="cuda")
    # the 8-fold symmetry of real integrals; <rs||tu> = -<sr||tu> needs (rt|su) = (su|rt)
    mo = mo + mo.permute(1, 0, 2, 3)
    mo = mo + mo.permute(0, 1, 3, 2)
    mo = mo + mo.permute(2, 3, 0, 1)
    n = 2 * h
    r = torch.arange(n, device="cuda")
    half, spin = r // 2, r % 2
    same = spin[:, None] == spin[None, :]

    sp = transform.spin_expand_device(mo, transform.SPIN_INTERLEAVED)
    zero = torch.zeros((), dtype=mo.dtype, device="cuda")
    for a in range(0, n, 37):   # slabs of the first index, compared in full
        m = mo[half[a]][half][:, half][:, :, half]      # [x, y, z] = (a/2 x/2 | y/2 z/2)
        assert torch.equal(sp[a], torch.where(same[a][:, None, None] & same[None, :, :], m, zero))

    bl = transform.spin_expand_device(mo, transform.SPIN_BLOCKED)
    perm = torch.cat([torch.arange(0, n, 2, device="cuda"), torch.arange(1, n, 2, device="cuda")])
    for a in range(0, n, 37):   # blocked = interleaved with the alpha orbitals first
        assert torch.equal(bl[a], sp[perm[a]][perm][:, perm][:, :, perm])
    del sp, bl

    an = transform.spin_expand_device(mo, transform.SPIN_ANTI_PHYSICIST)
    assert torch.equal(an, -an.transpose(2, 3))
    assert torch.equal(an, -an.transpose(0, 1))
    for a in range(0, n, 37):   # <a s||t u> = [a t][s u] (a t|s u) - [a u][s t] (a u|s t)
        m = mo[half[a]][half][:, half][:, :, half]
        first = torch.where((spin[a] == spin)[None, :, None] & same[:, None, :], m.permute(1, 0, 2), zero)
        second = torch.where((spin[a] == spin)[None, None, :] & same[:, :, None], m.permute(1, 2, 0), zero)
        assert torch.equal(an[a], first - second)


def test_spin_expand_limits(gpu_lib):
    from gaussium_gb300 import _lib, transform
    hmax = transform.max_spatial_orbitals()
    assert 100 <= hmax <= 400
    dummy = torch.zeros(2, dtype=torch.float64, device="cuda")
    # over the limit: refused before any launch (the dummy buffers are never touched)
    assert gpu_lib.gs_spin_expand(_lib.ptr(dummy), hmax + 1, 0, _lib.ptr(dummy), _lib.stream()) == 6
    assert gpu_lib.gs_spin_expand(_lib.ptr(dummy), 1, 3, _lib.ptr(dummy), _lib.stream()) == 1
    assert gpu_lib.gs_spin_expand(None, 0, 0, None, _lib.stream()) == 0
    with pytest.raises(ValueError):
        transform.spin_expand_device(torch.zeros((2, 3, 2, 2), dtype=torch.float64, device="cuda"), 0)


def test_co_mp2_energy_matches_reference(gpu_lib):
    """Carbon monoxide / STO-3G (the reference's test_start.py:45-49) end to end: RHF on the
    GPU Fock builder, the AO tensor from the GPU ERI-matrix drop-in, the AO->MO transform on
    the GPU, and the MP2 sum of moellerplesset/moeller_plesset.py:14-22 (restated in the
    oracle) give the reference's RHF and MP2 total energies to 1e-8 Eh."""
    from gaussium_gb300 import scf, transform
    from gaussium_gb300.dropin import TwoElectronRepulsionGPU
    from gaussium_gb300.fock import FockMatrixRestrictedGPU
    g, funcs, _ = load("co_sto3g")
    hcore = g["kinetic"] + g["nuclear"]
    res = scf.restricted_scf(g["overlap"], hcore, int(g["electrons"]),
                             FockMatrixRestrictedGPU(hcore, funcs), threshold=1e-12)
    e_nuc = scf.nuclear_repulsion(g["charges"], g["coords"])
    assert res.converged
    assert abs(res.energy + e_nuc - float(g["energy_rhf"])) < 1e-8
    ao = TwoElectronRepulsionGPU(funcs, None, None, 1).create_repulsion_matrix()
    mo = transform.molecular_orbitals(ao, res.coefficients)
    corr = oracle.mp2_correlation(mo, res.orbital_energies, int(g["electrons"]) // 2)
    assert abs(res.energy + e_nuc + corr - float(g["energy_mp2"])) < 1e-8
