"""The internal-frame BFGS driver on a rotation- and translation-invariant model energy
(harmonic springs between all nuclei): it must find the springs' rest geometry, and the
frame's variables must reproduce the coordinates they came from."""
import numpy as np

from gaussium_gb300.molecules import Molecule
from gaussium_gb300.optimize import NelderMead, optimize_bfgs


def _springs(rest):
    def eg(m):
        c = m.coords
        e, g = 0.0, np.zeros_like(c)
        for i in range(len(c)):
            for j in range(i + 1, len(c)):
                d = c[i] - c[j]
                r = np.linalg.norm(d)
                e += 0.5 * (r - rest[i, j]) ** 2
                f = (r - rest[i, j]) * d / r
                g[i] += f
                g[j] -= f
        return e, g
    return eg


def test_internal_frame_round_trip():
    rng = np.random.default_rng(3)
    c = rng.standard_normal((5, 3))
    nm = NelderMead(["H"] * 5, c, None)
    v = nm._vector(nm.frame)
    assert len(v) == 3 * 5 - 6
    assert np.allclose(nm.coordinates(v), nm.frame)
    # the frame is a rigid motion of the input: all distances kept
    d0 = np.linalg.norm(c[:, None] - c[None], axis=-1)
    d1 = np.linalg.norm(nm.frame[:, None] - nm.frame[None], axis=-1)
    assert np.allclose(d0, d1)


def test_bfgs_in_internal_frame_reaches_rest_geometry():
    rng = np.random.default_rng(5)
    target = rng.standard_normal((4, 3)) * 1.5
    rest = np.linalg.norm(target[:, None] - target[None], axis=-1)
    start = target + 0.2 * rng.standard_normal(target.shape)
    e, x, n, gmax = optimize_bfgs(Molecule(["H"] * 4, start), gtol=1e-8,
                                  energy_gradient=_springs(rest))
    d = np.linalg.norm(x[:, None] - x[None], axis=-1)
    assert e < 1e-12 and gmax < 1e-8
    assert np.allclose(d, rest, atol=1e-6)
