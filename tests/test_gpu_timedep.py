"""GPU parity of the time-dependent potentials: the rotating bars
(BarPotential, DehnenBarPotential), the uniform frame acceleration,
MW_LMC_Potential (linear LMC and Milky Way velocity tracks) and
GrowingPotential (cubic and linear growth tracks) — the potential,
gradient and Hessian at points and times, the release at each release
time, and whole streams in FP64 (<= 1e-10) and FP32 compensated (<= 1e-5),
all against the oracle."""
import numpy as np
import pytest

from streamsculptor_gb300 import _abi

from .conftest import PROG_WF, mw3_gpu, rel_err

pytestmark = pytest.mark.gpu

BAR = (_abi.SS_BAR, 0, (2e10, 4.0, 1.0, 0.5, 0.045))
DEHNEN = (_abi.SS_DEHNEN_BAR, 0, (0.01, 0.22, 8.0, 3.5, 0.4, 0.045))


def np64(t):
    return t.detach().cpu().double().numpy()


def phase_err(a, b):
    a, b = np.asarray(a).reshape(-1, 6), np.asarray(b).reshape(-1, 6)
    ex = np.linalg.norm(a[:, :3] - b[:, :3], axis=1) / np.linalg.norm(b[:, :3], axis=1)
    ev = np.linalg.norm(a[:, 3:] - b[:, 3:], axis=1) / np.linalg.norm(b[:, 3:], axis=1)
    return float(np.max(np.maximum(ex, ev)))


def _bars(ss):
    from streamsculptor_gb300 import potential as P
    u = ss.usys
    return (P.BarPotential(m=2e10, a=4.0, b=1.0, c=0.5, Omega=0.045, units=u),
            P.DehnenBarPotential(alpha=0.01, v0=0.22, R0=8.0, Rb=3.5, phib=0.4, Omega=0.045, units=u))


def _lmc_tracks():
    tk = np.arange(121) * 25.0 - 3000.0
    s = tk / 1000.0
    lmc = np.stack([-1.0 + 40 * s - 20 * s ** 2, -41.0 - 90 * s, -28.0 + 60 * s + 15 * s ** 3], 1)
    vel = np.stack([0.01 * np.sin(tk / 300), 0.02 * np.cos(tk / 200), -0.005 * tk / 800], 1)
    return tk, lmc, vel


def _mw_lmc(ss, oracle):
    from streamsculptor_gb300 import potential as P
    tk, lmc, vel = _lmc_tracks()
    gpu = P.MW_LMC_Potential(units=ss.usys, lmc_track=(tk, lmc), mw_velocity=(tk, vel))
    m_lmc = 0.85e11
    orc = oracle.HostModel([(_abi.SS_HERNQUIST, 0, (5e9, 1.0, 0.0)), (_abi.SS_MIYAMOTO_NAGAI, 0, (5e10, 3.0, 0.3)),
                            (_abi.SS_NFW, 0, (5.4e11, 15.62, 0.0)),
                            (_abi.SS_NFW, 1, (m_lmc, (m_lmc / 1e11) ** 0.6 * 8.5, 0.0)),
                            (_abi.SS_UNIFORM_ACCEL, 0, ())],
                           track=(tk[0], 25.0, lmc, "linear"), frame_velocity=(tk[0], 25.0, vel, "linear"))
    return gpu, orc


def test_bar_potentials_eval(ss, oracle):
    from streamsculptor_gb300 import potential as P
    bar, dehnen = _bars(ss)
    rng = np.random.default_rng(5)
    x = rng.normal(0, 5, (400, 3))
    x[:100] *= 0.4  # inside the Dehnen bar's Rb as well
    t = rng.uniform(-3000, 0, 400)
    for gpu, spec in ((bar, BAR), (dehnen, DEHNEN)):
        phi_o, g_o, H_o = oracle.potential_eval(oracle.HostModel([spec]), x, t)
        assert rel_err(np64(gpu.potential(x, t)), phi_o) < 1e-12
        assert rel_err(np64(gpu.gradient(x, t)), g_o) < 1e-12
        assert rel_err(np64(gpu.jacobian_force(x, t)), H_o) < 1e-10
    comb = P.Potential_Combine([mw3_gpu(ss), bar], units=ss.usys)
    phi_o, g_o, _ = oracle.potential_eval(oracle.HostModel(oracle.mw3() + [BAR]), x, t)
    assert rel_err(np64(comb.gradient(x, t)), g_o) < 1e-12


def test_mw_lmc_force(ss, oracle):
    gpu, orc = _mw_lmc(ss, oracle)
    rng = np.random.default_rng(6)
    x = rng.normal(0, 30, (300, 3))
    t = rng.uniform(-3100, 50, 300)  # beyond both ends too: linear continuation
    _, g_o, H_o = oracle.potential_eval(orc, x, t)
    assert rel_err(np64(gpu.gradient(x, t)), g_o) < 1e-12
    assert rel_err(np64(gpu.jacobian_force(x, t)), H_o) < 1e-10
    with pytest.raises(NotImplementedError):
        gpu.potential(x, 0.0)


@pytest.mark.parametrize("which", ["bar", "dehnen", "mw_lmc"])
def test_time_dependent_streams(ss, oracle, which):
    """Fardal stream (400 releases, 1 Myr steps) through each potential:
    progenitor orbit, release at each release time and particles, FP64 and
    FP32 compensated, against the oracle."""
    from streamsculptor_gb300 import potential as P
    n = 400
    if which == "mw_lmc":
        gpu, orc = _mw_lmc(ss, oracle)
    else:
        bar, dehnen = _bars(ss)
        g = bar if which == "bar" else dehnen
        gpu = P.Potential_Combine([mw3_gpu(ss), g], units=ss.usys)
        orc = oracle.HostModel(oracle.mw3() + [BAR if which == "bar" else DEHNEN])
    back = oracle.orbit(orc, PROG_WF, 0.0, -1.0, n, n)[0, -1]
    ts = -n + np.arange(n + 1) * 1.0
    normals = np.random.default_rng(17).standard_normal((n + 1, 1, 4))
    ws = oracle.orbit(orc, back, ts[0], 1.0, n, 1)[0]
    ics, _ = oracle.release(orc, ws, ts, 2e4, normals)
    final, _, st = oracle.stream(orc, ts[0], 1.0, n, ics[:-1].reshape(-1, 6), 2, 1)
    assert (st == 0).all()
    final = final.reshape(n, 2, 6)
    for precision, tol in (("f64", 1e-10), ("f32k", 1e-5)):
        lead, trail = gpu.gen_stream_vmapped(ts=ts, prog_w0=back, Msat=2e4, normals=normals, precision=precision)
        assert phase_err(np64(lead), final[:, 0]) <= tol, precision
        assert phase_err(np64(trail), final[:, 1]) <= tol, precision


def _tnfw(ss, rng, n=4, t0=None, x0=None):
    """TNFW subhalos (potential.py:1022-1108) and the oracle's table of them."""
    from streamsculptor_gb300 import potential as P
    from streamsculptor_gb300.potential import _cubic_knot_slopes
    m = 10 ** rng.uniform(7.5, 9.0, n)
    c = rng.uniform(10, 20, n)
    z = rng.uniform(1.0, 3.0, n)
    f = rng.uniform(0.05, 0.8, n)
    x0 = rng.normal(0, 8, (n, 3)) if x0 is None else x0
    v = rng.normal(0, 0.15, (n, 3))
    t0 = rng.uniform(-300, -50, n) if t0 is None else t0
    pot = P.TNFWSubhaloLinePotential(m, c, z, f, x0, v, t0, 120.0, units=ss.usys)
    du = pot.log_r_grids[:, 1] - pot.log_r_grids[:, 0]
    grid = np.stack([pot.phi_grids, _cubic_knot_slopes(pot.phi_grids, du[:, None])], axis=2)
    sh = dict(kind=_abi.SS_SH_GRID, m=np.zeros(n), a=pot.a, x0=x0, v=v, t0=t0, t_window=120.0, grid=grid,
              grid_u0=pot.log_r_grids[:, 0], grid_du=du)
    return pot, sh


def test_tnfw_subhalos_eval_and_streams(ss, oracle):
    """Per-subhalo potential and gradient, then a stream in base + TNFW
    subhalos (FP64 and FP32 compensated) and the mass response (6 columns),
    all against the oracle's spline of the same tables."""
    from streamsculptor_gb300 import _core, perturbative
    from streamsculptor_gb300.streamhelpers import gen_stream_vmapped_with_pert_fixed_prog
    rng = np.random.default_rng(44)
    n_rel = 300
    orc = oracle.HostModel(oracle.mw3())
    back = oracle.orbit(orc, PROG_WF, 0.0, -1.0, n_rel, n_rel)[0, -1]
    ts = -n_rel + np.arange(n_rel + 1) * 1.0
    ws = oracle.orbit(orc, back, ts[0], 1.0, n_rel, 1)[0]
    pot, sh = _tnfw(ss, rng, x0=ws[[60, 140, 200, 250], :3] + rng.normal(0, 0.8, (4, 3)),
                    t0=ts[[60, 140, 200, 250]])
    x = ws[::7, :3] + rng.normal(0, 1.0, (len(ws[::7]), 3))
    for t in (ts[60], ts[200]):
        phi_g = np64(pot.potential_per_SH(x, t))
        g_g = np64(pot.gradient_per_SH(x, t))
        phi_o, g_o, _, _ = oracle.subhalo_eval(oracle.HostModel(oracle.mw3(), subhalos=sh), x, t)
        assert rel_err(phi_g, phi_o) < 1e-12 and rel_err(g_g, g_o) < 1e-12
    normals = rng.standard_normal((n_rel + 1, 1, 4))
    ics, _ = oracle.release(orc, ws, ts, 2e4, normals)
    tot = oracle.HostModel(oracle.mw3(), subhalos=sh)
    final, _, st = oracle.stream(tot, ts[0], 1.0, n_rel, ics[:-1].reshape(-1, 6), 2, 1)
    assert (st == 0).all()
    final = final.reshape(n_rel, 2, 6)
    for precision, tol in (("f64", 1e-10), ("f32k", 1e-5)):
        lead, trail = gen_stream_vmapped_with_pert_fixed_prog(mw3_gpu(ss), pot, ts=ts, prog_w0=back, Msat=2e4,
                                                              normals=normals, precision=precision)
        assert phase_err(np64(lead), final[:, 0]) <= tol, precision
        assert phase_err(np64(trail), final[:, 1]) <= tol, precision
    # first-order mass response of every particle (GenerateMassPerturbation)
    bsm = perturbative.BaseStreamModel(mw3_gpu(ss), back, ts, 2e4, 0, normals=normals)
    gen = perturbative.GenerateMassPerturbation(mw3_gpu(ss), pot, bsm)
    (lb, ld), (tb, td) = gen.compute_perturbation_OTF()
    base = np.stack([np64(gen.base_realspace_ICs_lead[:n_rel]), np64(gen.base_realspace_ICs_trail[:n_rel])], 1)
    pert = np.stack([np64(gen.perturbation_ICs_lead[:n_rel]), np64(gen.perturbation_ICs_trail[:n_rel])], 1)
    bo, po = oracle.pert_response(tot, ts[0], 1.0, n_rel, base.reshape(-1, 6), pert.reshape(2 * n_rel, 4, 6), 2, 1,
                                  ncol=6)
    d = np.stack([np64(ld), np64(td)], 1).reshape(2 * n_rel, 4, 6)
    assert rel_err(d, po[0]) <= 1e-9
    with pytest.raises(_abi.SSError):
        perturbative.GenerateMassRadiusPerturbation(mw3_gpu(ss), pot, pot, bsm)  # no scale-radius response


def test_potential_from_density_gpu(ss, oracle):
    """The tabulated spherical potential on the GPU: its force against the
    analytic Plummer force (to the spline's accuracy) and a stream through it against
    the oracle's evaluation of the same spline (FP64 <= 1e-10)."""
    from streamsculptor_gb300 import _core, potential as P
    M, a = 8e11, 20.0
    rho = lambda r: 3 * M / (4 * np.pi * a ** 3) * (1 + r * r / (a * a)) ** -2.5  # noqa: E731
    pot = P.get_potential_from_density(rho, units=ss.usys)
    G = _core.G_for(ss.usys)
    x = np.random.default_rng(2).normal(0, 10, (200, 3))
    r = np.linalg.norm(x, axis=1, keepdims=True)
    g_exact = G * M * x / (r * r + a * a) ** 1.5
    # the spline's own accuracy: 128 knots over six decades (d ln r = 0.109)
    # with interpax-'cubic' knot slopes put the force within ~2e-3
    assert rel_err(np64(pot.gradient(x, 0.0)), g_exact) < 5e-3
    sp = pot._spline
    orc = oracle.HostModel([(_abi.SS_SH_EXPANSION, 0, (1.0,))],
                           expansion=(0, sp.log_r0, sp.dlog_r, sp.coef.cpu().numpy()))
    n = 200
    back = oracle.orbit(orc, PROG_WF, 0.0, -1.0, n, n)[0, -1]
    ts = -n + np.arange(n + 1) * 1.0
    normals = np.random.default_rng(3).standard_normal((n + 1, 1, 4))
    ws = oracle.orbit(orc, back, ts[0], 1.0, n, 1)[0]
    ics, _ = oracle.release(orc, ws, ts, 2e4, normals)
    final, _, _ = oracle.stream(orc, ts[0], 1.0, n, ics[:-1].reshape(-1, 6), 2, 1)
    lead, trail = pot.gen_stream_vmapped(ts=ts, prog_w0=back, Msat=2e4, normals=normals)
    final = final.reshape(n, 2, 6)
    assert phase_err(np64(lead), final[:, 0]) <= 1e-10 and phase_err(np64(trail), final[:, 1]) <= 1e-10


def _growing(ss, oracle, linear):
    """GrowingPotential (potential.py:464-477) of the stream workloads'
    potential with a growth factor from 0.6 to 1 over 3 Gyr (knots every
    50 Myr), and the oracle's model of it."""
    import torch

    from streamsculptor_gb300 import potential as P
    from streamsculptor_gb300._core import CenterTrack
    tk = np.arange(61) * 50.0 - 3000.0
    g = 0.6 + 0.4 * (1.0 + tk / 3000.0) ** 1.5 + 0.02 * np.sin(tk / 170.0)
    tr = CenterTrack.growth_from_samples(tk, torch.as_tensor(g, device="cuda"), linear=linear)
    gpu = P.GrowingPotential(mw3_gpu(ss), tr, units=ss.usys)
    orc = oracle.HostModel([(k, c | _abi.SS_GROWS, p) for (k, c, p) in oracle.mw3()],
                           growth=(tk[0], 50.0, g) + (("linear",) if linear else ()))
    return gpu, orc


@pytest.mark.parametrize("linear", [False, True])
def test_growing_potential_eval(ss, oracle, linear):
    """Potential, gradient and Hessian of a growing potential at points and
    times spread over the growth track, against the oracle."""
    gpu, orc = _growing(ss, oracle, linear)
    rng = np.random.default_rng(23)
    x = rng.normal(0, 10, (400, 3))
    t = rng.uniform(-3100.0, 50.0, 400)  # past both ends too (the end segments continue)
    phi_o, g_o, H_o = oracle.potential_eval(orc, x, t)
    import torch
    tt = torch.as_tensor(t, device="cuda")
    assert rel_err(np64(gpu.potential(x, tt)), phi_o) < 1e-12
    assert rel_err(np64(gpu.gradient(x, tt)), g_o) < 1e-12
    assert rel_err(np64(gpu.jacobian_force(x, tt)), H_o) < 1e-11


def test_growing_potential_stream(ss, oracle):
    """A Fardal stream (400 releases, 1 Myr steps) in a growing potential:
    progenitor orbit, release and particles, FP64 and FP32 compensated,
    against the oracle."""
    gpu, orc = _growing(ss, oracle, False)
    n = 400
    back = oracle.orbit(orc, PROG_WF, 0.0, -1.0, n, n)[0, -1]
    ts = -n + np.arange(n + 1) * 1.0
    normals = np.random.default_rng(29).standard_normal((n + 1, 1, 4))
    ws = oracle.orbit(orc, back, ts[0], 1.0, n, 1)[0]
    ics, _ = oracle.release(orc, ws, ts, 2e4, normals)
    final, _, st = oracle.stream(orc, ts[0], 1.0, n, ics[:-1].reshape(-1, 6), 2, 1)
    assert (st == 0).all()
    final = final.reshape(n, 2, 6)
    for precision, tol in (("f64", 1e-10), ("f32k", 1e-5)):
        lead, trail = gpu.gen_stream_vmapped(ts=ts, prog_w0=back, Msat=2e4, normals=normals, precision=precision)
        assert phase_err(np64(lead), final[:, 0]) <= tol, precision
        assert phase_err(np64(trail), final[:, 1]) <= tol, precision
