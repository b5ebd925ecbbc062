"""Gradient of a binned stream-track loss through the hand-written adjoint,
against central finite differences of the CPU FP64 oracle pipeline
(progenitor back/forward orbit, release, stream, loss) with h = 1e-4
relative.  Bin membership is frozen at the evaluation point on both sides
(it is piecewise constant and carries no gradient).  The reference's own
gradient (jax.jacfwd / jax.grad through diffrax) cannot run here: JAX is not
installed."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

THETA0 = np.array([5.4e11, 15.62, 0.9, 6.8e10, 3.0, 0.28, 5e9, 1.0, 12.0, 0.0, 4.0, 0.0, 0.18, 0.04])
# finite-difference steps: 1e-4 relative, absolute where the value is 0
STEP = np.array([1e-4 * abs(v) if v != 0 else s for v, s in
                 zip(THETA0, [0, 0, 0, 0, 0, 0, 0, 0, 1e-3, 1e-3, 1e-3, 1e-5, 1e-5, 1e-5])])


def _setup(A, n_rel=150, ppr=10):
    rng = np.random.default_rng(5)
    return A.StreamSetup(n_rel=n_rel, spr=2, dt=1.0, ppr=ppr, msat=2e4,
                         normals=rng.standard_normal((n_rel + 1, ppr // 2, 4)))


def _oracle_final(oracle, model, theta, setup):
    m = oracle.HostModel([tuple(c) for c in model.components(theta)])
    n = setup.n_steps
    back = oracle.orbit(m, theta[-6:], 0.0, -setup.dt, n, n)[0, -1]
    ws = oracle.orbit(m, back, setup.t0, setup.dt, n, setup.spr)[0]
    ts = setup.t0 + np.arange(setup.n_rel + 1) * setup.spr * setup.dt
    ics, _ = oracle.release(m, ws, ts, setup.msat, setup.normals)
    final, _, _ = oracle.stream(m, setup.t0, setup.dt, n, ics[:setup.n_rel].reshape(-1, 6), setup.ppr, setup.spr)
    return final


def _loss_np(loss, final, b, ok):
    """TrackLoss with frozen membership b, in numpy FP64."""
    R, sx, sv = loss.R.cpu().numpy(), loss.sx.cpu().numpy(), loss.sv.cpu().numpy()
    xs = final[:, :3] - sx
    vs = final[:, 3:] - sv
    u = xs @ R.T
    d = np.linalg.norm(xs, axis=1)
    obs = np.stack([np.arcsin(u[:, 2] / d), d, (xs * vs).sum(1) / d], axis=1)
    nb = loss.n_bins
    cnt = np.bincount(b, minlength=nb).astype(np.float64)
    s = np.stack([np.bincount(b, weights=obs[:, q], minlength=nb) for q in range(3)], axis=1)
    mean = s / np.maximum(cnt, 1.0)[:, None]
    r = (mean - loss.target.cpu().numpy()) / loss.scales.cpu().numpy()
    return float((r[ok] ** 2).sum())


def test_adjoint_gradient_matches_oracle_finite_differences(ss, oracle):
    from streamsculptor_gb300 import adjoint as A
    model = A.TriaxialHaloModel
    setup = _setup(A)
    rng = np.random.default_rng(9)
    theta_t = THETA0 + STEP * 300 * rng.standard_normal(14)
    target = A.forward_stream(model, theta_t, setup)
    loss = A.TrackLoss(THETA0[-6:], target, n_bins=16)
    th = torch.tensor(THETA0, dtype=torch.float64, device="cuda", requires_grad=True)
    final = A.StreamFn.apply(th, model, setup)
    L = loss(final)
    L.backward()
    g_gpu = th.grad.cpu().numpy()
    # membership frozen at theta0 (from the same forward stream)
    with torch.no_grad():
        phi1, _ = loss.observables(final)
        b = torch.bucketize(phi1, loss.edges[1:-1]).cpu().numpy()
        cnt = np.bincount(b, minlength=loss.n_bins)
        ok = (cnt > 0) & (loss.target_count.cpu().numpy() > 0)
    L0 = _loss_np(loss, _oracle_final(oracle, model, THETA0, setup), b, ok)
    assert abs(L0 - float(L)) <= 1e-4 * abs(L0) + 1e-9
    g_fd = np.zeros(14)
    for k in range(14):
        tp, tm = THETA0.copy(), THETA0.copy()
        tp[k] += STEP[k]
        tm[k] -= STEP[k]
        g_fd[k] = (_loss_np(loss, _oracle_final(oracle, model, tp, setup), b, ok) -
                   _loss_np(loss, _oracle_final(oracle, model, tm, setup), b, ok)) / (2 * STEP[k])
    # compare in units of the finite-difference step (the loss change per step)
    scaled_gpu, scaled_fd = g_gpu * STEP, g_fd * STEP
    err = np.abs(scaled_gpu - scaled_fd) / np.max(np.abs(scaled_fd))
    print("adjoint vs FD (scaled):", np.array2string(err, precision=2))
    assert np.max(err) < 2e-3
