"""Host-side behaviour of the Python layer that needs no GPU: argument
checks that run before any device work, and host formulas."""
import numpy as np
import pytest

from streamsculptor_gb300 import potential as P
from streamsculptor_gb300.streamhelpers import gen_stream_batches

G = 4.498502151469554e-12


def _batches(**kw):
    args = dict(pot_base=P.NFWPotential(m=1e12, r_s=20.0), ts=np.arange(11.0) - 10.0,
                prog_w0s=np.array([10.0, 0, 0, 0, 0.2, 0]), Msat=1e4, normals=None, n_batches=2, seed_num=3,
                dt=1.0)
    args.update(kw)
    return list(gen_stream_batches(**args))


@pytest.mark.parametrize("kw, msg", [
    (dict(precision="mlp"), "precision"),
    (dict(prog_w0_at="middle"), "prog_w0_at"),
    (dict(ts=np.array([-10.0, -7.0, -6.5, -2.0, 0.0])), "uniform"),
    (dict(n_batches=None), "n_batches"),
    (dict(prog_w0s=[np.zeros(6)] * 3, normals=[None] * 2), "equal length"),
    (dict(release="spray"), "release"),
    (dict(seed_num=None), "seed_num"),
])
def test_gen_stream_batches_rejects_bad_arguments(kw, msg):
    """Every check runs before the first device call (a generator: the
    checks run at the first next())."""
    with pytest.raises((ValueError, NotImplementedError), match=msg):
        _batches(**kw)


def test_zhao_density_is_the_reference_formula():
    """ZhaoPotential.density (potential.py:308-319): alpha = 1, beta = 4,
    gamma = 1 is the Hernquist sphere, rho = m r_s / (2 pi r (r + r_s)^3),
    and a cored case (alpha = 0.5, beta = 5, gamma = 0) against the formula
    written out."""
    from math import gamma as Gf
    z = P.ZhaoPotential(1e11, 10.0, 1.0, 4.0, 1.0)
    x = np.array([[1.0, 2.0, 3.0], [20.0, -5.0, 1.0]])
    r = np.linalg.norm(x, axis=1)
    assert np.allclose(z.density(x, 0.0), 1e11 * 10.0 / (2 * np.pi * r * (r + 10.0) ** 3), rtol=1e-13, atol=0)
    m, rs, al, be, ga = 3e10, 5.0, 0.5, 5.0, 0.0
    z2 = P.ZhaoPotential(m, rs, al, be, ga)
    a1, b1 = al * (3 - ga), al * (be - 3)
    rho0 = m / (4 * np.pi * al * Gf(a1) * Gf(b1) / Gf(a1 + b1))
    u = r / rs
    want = rho0 / rs ** 3 / u ** ga / (1 + u ** (1 / al)) ** ((be - ga) * al)
    assert np.allclose(z2.density(x, 0.0), want, rtol=1e-13, atol=0)
