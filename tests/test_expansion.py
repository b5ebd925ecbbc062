"""Spherical-harmonic expansion potential (SS_SH_EXPANSION): the oracle's
restatement pinned against an independent scipy evaluation of the same
definition (CPU), then the kernels against the oracle (GPU): Phi, gradient
and Hessian, the progenitor orbit, the release and FP64 / FP32-compensated
streams through the expansion."""
from math import factorial

import numpy as np
import pytest

from streamsculptor_gb300 import _abi

from .conftest import PROG_WF, rel_err


def _expansion(units=None, **kw):
    from streamsculptor_gb300 import potential as P
    return P.seeded_triaxial_expansion(units=units, **kw)


def _model(oracle, pot):
    return oracle.HostModel([(_abi.SS_SH_EXPANSION, 0, (1.0,))], G=4.498502151469553e-12,
                            expansion=(pot.l_max, pot.log_r0, pot.dlog_r, pot.coef.numpy()))


def _phi_scipy(pot, x):
    """The definition, term by term, with scipy's associated Legendre
    functions (Condon-Shortley phase removed)."""
    from scipy.special import lpmv
    coef, L = pot.coef.numpy(), pot.l_max
    r = np.linalg.norm(x)
    th, ph = np.arccos(x[2] / r), np.arctan2(x[1], x[0])
    us = (np.log(r) - pot.log_r0) / pot.dlog_r
    k = int(np.clip(np.floor(us), 0, coef.shape[0] - 2))
    s = us - k
    sc = min(max(s, 0.0), 1.0)
    e = s - sc
    h = [(1 + 2 * sc) * (1 - sc) ** 2, sc * (1 - sc) ** 2, sc * sc * (3 - 2 * sc), sc * sc * (sc - 1)]
    d = [6 * sc * (sc - 1), (1 - sc) * (1 - 3 * sc), 6 * sc * (1 - sc), sc * (3 * sc - 2)]
    tot = 0.0
    for l in range(L + 1):
        for m in range(-l, l + 1):
            j = l * l + l + m
            c = [coef[k, j, 0], coef[k, j, 1] * pot.dlog_r, coef[k + 1, j, 0], coef[k + 1, j, 1] * pot.dlog_r]
            f = np.dot(h, c) + e * np.dot(d, c)
            am = abs(m)
            norm = 1.0 if am == 0 else np.sqrt(2 * factorial(l - am) / factorial(l + am))
            Y = norm * lpmv(am, l, np.cos(th)) * (-1) ** am * (np.cos(am * ph) if m >= 0 else np.sin(am * ph))
            tot += f * Y
    return tot


def _points(n=200, seed=3):
    x = np.random.default_rng(seed).normal(0, 12, size=(n, 3))
    x[0] = [0.05, 0.02, 0.01]       # inside the first knot (linear continuation)
    x[1] = [300.0, 20.0, -50.0]     # beyond the last knot
    x[2] = [3.0, 0.0, 0.0]          # on the x axis
    return x


def test_oracle_expansion_matches_scipy_definition(oracle):
    pot = _expansion(l_max=8)
    # make every term nonzero (odd l and sin parts too) for the pin
    rng = np.random.default_rng(0)
    pot.coef[:, 1:, :] += 1e-3 * pot.coef[:, :1, :] * rng.standard_normal((1, pot.coef.shape[1] - 1, 1))
    x = _points(40)
    phi, g, _ = oracle.potential_eval(_model(oracle, pot), x)
    ref = np.array([_phi_scipy(pot, xi) for xi in x])
    assert rel_err(phi, ref) < 1e-13
    h = 1e-5
    gfd = np.stack([(oracle.potential_eval(_model(oracle, pot), x + h * np.eye(3)[i])[0] -
                     oracle.potential_eval(_model(oracle, pot), x - h * np.eye(3)[i])[0]) / (2 * h)
                    for i in range(3)], axis=1)
    assert rel_err(g, gfd) < 1e-6


@pytest.mark.gpu
@pytest.mark.parametrize("general", [False, True])
def test_expansion_eval_matches_oracle(ss, oracle, general):
    pot = _expansion(units=ss.usys)
    if general:  # every (l, m) term nonzero
        rng = np.random.default_rng(1)
        pot.coef[:, 1:, :] += 1e-2 * pot.coef[:, :1, :] * rng.standard_normal((1, pot.coef.shape[1] - 1, 1))
    x = _points()
    phi_o, g_o, H_o = oracle.potential_eval(_model(oracle, pot), x)
    assert rel_err(np.asarray(pot.potential(x, 0.0).cpu()), phi_o) < 1e-12
    assert rel_err(np.asarray(pot.gradient(x, 0.0).cpu()), g_o) < 1e-12
    assert rel_err(np.asarray(pot.jacobian_force(x, 0.0).cpu()), H_o) < 1e-11


def _phase_err(a, b):
    a, b = np.asarray(a).reshape(-1, 6), np.asarray(b).reshape(-1, 6)
    ex = np.linalg.norm(a[:, :3] - b[:, :3], axis=1) / np.linalg.norm(b[:, :3], axis=1)
    ev = np.linalg.norm(a[:, 3:] - b[:, 3:], axis=1) / np.linalg.norm(b[:, 3:], axis=1)
    return float(np.max(np.maximum(ex, ev)))


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol", [("f64", 1e-10), ("f32k", 1e-5)])
def test_expansion_stream_matches_oracle(ss, oracle, precision, tol):
    """Back orbit, release and stream through the expansion: 300 releases x
    4 particles, 600 steps of 1 Myr."""
    pot = _expansion(units=ss.usys)
    orc = _model(oracle, pot)
    n_rel, ppr, dt = 300, 4, 1.0
    back_o = oracle.orbit(orc, PROG_WF, 0.0, -dt, 2 * n_rel, 2 * n_rel)[0, -1]
    back = pot.integrate_orbit(w0=PROG_WF, ts=np.array([0.0, -2 * n_rel * dt]), t0=0.0, t1=-2 * n_rel * dt,
                               dt=dt).ys[-1]
    assert _phase_err(np.asarray(back.cpu()), back_o) < 1e-11
    ts = -2 * n_rel * dt + np.arange(n_rel + 1) * 2 * dt
    normals = np.random.default_rng(5).standard_normal((n_rel + 1, ppr // 2, 4))
    from streamsculptor_gb300.streamhelpers import gen_stream
    out = gen_stream(pot, ts, back_o, 2e4, normals=normals, dt=dt, n_particles_per_release=ppr,
                     precision=precision)
    ws = oracle.orbit(orc, back_o, ts[0], dt, 2 * n_rel, 2)[0]
    ics, _ = oracle.release(orc, ws, ts, 2e4, normals)
    final, _, st = oracle.stream(orc, ts[0], dt, 2 * n_rel, ics[:n_rel].reshape(-1, 6), ppr, 2)
    assert (st == 0).all()
    got = np.stack([np.asarray(out[0].cpu()), np.asarray(out[1].cpu())], axis=2).reshape(-1, 6)
    err = _phase_err(got, final)
    print(f"expansion stream {precision}: {err:.3e}")
    assert err <= tol
