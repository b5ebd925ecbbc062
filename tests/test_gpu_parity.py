"""GPU parity: every kernel against the CPU FP64 oracle on the same seeded
inputs, through the C ABI (via the package facade).

Tolerances: FP64 paths <= 1e-10 relative in final phase-space coordinates
(1e-12 for single evaluations); FP32-compensated streams <= 1e-5 relative;
FP32 responses as stated per test."""
import numpy as np
import pytest
import torch

from streamsculptor_gb300 import _abi

from .conftest import PROG_WF, mw3_gpu, rel_err

pytestmark = pytest.mark.gpu


def np64(t):
    return t.detach().cpu().double().numpy()


def phase_err(a, b):
    """max over particles of max(|dx|/|x|, |dv|/|v|)."""
    a, b = np.asarray(a).reshape(-1, 6), np.asarray(b).reshape(-1, 6)
    ex = np.linalg.norm(a[:, :3] - b[:, :3], axis=1) / np.linalg.norm(b[:, :3], axis=1)
    ev = np.linalg.norm(a[:, 3:] - b[:, 3:], axis=1) / np.linalg.norm(b[:, 3:], axis=1)
    return float(np.max(np.maximum(ex, ev)))


KINDS = [
    ("NFWPotential", dict(m=5.4e11, r_s=15.62), (_abi.SS_NFW, 0, (5.4e11, 15.62, 0.0))),
    ("TriaxialNFWPotential", dict(m=3e11, r_s=12.0, q1=1.0, q2=0.9, q3=0.8),
     (_abi.SS_TRIAXIAL_NFW, 0, (3e11, 12.0, 1.0, 0.9, 0.8))),
    ("MiyamotoNagaiDisk", dict(m=6.8e10, a=3.0, b=0.28), (_abi.SS_MIYAMOTO_NAGAI, 0, (6.8e10, 3.0, 0.28))),
    ("HernquistPotential", dict(m=5e9, r_s=1.0, soft=0.01), (_abi.SS_HERNQUIST, 0, (5e9, 1.0, 0.01))),
    ("PlummerPotential", dict(m=2e9, r_s=0.5), (_abi.SS_PLUMMER, 0, (2e9, 0.5))),
    ("Isochrone", dict(m=4e9, a=1.5), (_abi.SS_ISOCHRONE, 0, (4e9, 1.5))),
]


@pytest.mark.parametrize("name,kw,spec", KINDS)
def test_potential_eval_every_kind(ss, oracle, name, kw, spec):
    from streamsculptor_gb300 import potential as P
    pot = getattr(P, name)(**kw, units=ss.usys)
    x = np.random.default_rng(7).normal(0, 8, size=(300, 3))
    x = x[np.linalg.norm(x, axis=1) > 0.3]
    phi_o, g_o, H_o = oracle.potential_eval(oracle.HostModel([spec]), x)
    assert rel_err(np64(pot.potential(x, 0.0)), phi_o) < 1e-12
    assert rel_err(np64(pot.gradient(x, 0.0)), g_o) < 1e-12
    assert rel_err(np64(pot.jacobian_force(x, 0.0)), H_o) < 1e-11


def test_nfw_golden_through_gpu(ss):
    # examples/tests.ipynb:1671: hamiltonian_field(NFW(1e12, 20)).term(0, [1,2,3,.2,.3,.4])
    from streamsculptor_gb300 import fields, potential as P
    f = fields.hamiltonian_field(P.NFWPotential(m=1e12, r_s=20.0, units=ss.usys))
    out = np64(f.term(0.0, np.array([1.0, 2.0, 3.0, 0.2, 0.3, 0.4])))
    printed = np.array([0.2, 0.3, 0.4, -0.0011937, -0.00238739, -0.00358109])
    assert np.all(np.abs(out - printed) <= 5e-9)


def test_notebook_pins_through_gpu(ss):
    """The reference notebooks' printed values through the public API on the
    GPU (the same pins as the oracle's, tests/test_oracle.py): the two NFW
    orbits of examples/tests.ipynb (cells 17 and 61, integrate_orbit and
    integrate_field), the Gala Milky Way orbit of
    examples/StreamSubhaloExample.ipynb cell 1 (fixed dt = 0.5 Myr; the
    notebook's ts spacing of 3.5 Myr would be a coarse fixed step), its
    Plummer and Hernquist subhalo lines (cell 9) and the Zhao density-derived
    potential of examples/potential_from_1D_Density.ipynb (cells 7-8)."""
    from streamsculptor_gb300 import fields, potential as P

    from .test_oracle import (GALA_IC_PRINTED, GALA_W_TODAY, NFW_T30_PRINTED, NFW_W0_A, NFW_W0_B, SH_PHI_PRINTED,
                              check_nfw_field_rows, sh_example_table, zhao_density)
    u = ss.usys
    nfw = P.NFWPotential(m=1e12, r_s=20.0, units=u)
    w = np64(nfw.integrate_orbit(w0=NFW_W0_A, ts=np.array([0.0, 30.0]), dt=0.5).ys[-1])
    assert np.all(np.abs(w - NFW_T30_PRINTED) <= 1e-8)
    sol = fields.integrate_field(w0=NFW_W0_B, ts=np.linspace(0, 3000, 1000), field=fields.hamiltonian_field(nfw),
                                 dt=3000.0 / 999 / 6)
    check_nfw_field_rows(np64(sol.ys))
    sol = P.GalaMilkyWayPotential(units=u).integrate_orbit(w0=GALA_W_TODAY, ts=np.array([0.0, -3500.0]), t0=0.0,
                                                           t1=-3500.0, dt=0.5)
    w, ref = np64(sol.ys[-1]), GALA_IC_PRINTED
    assert np.linalg.norm(w[:3] - ref[:3]) / np.linalg.norm(ref[:3]) <= 2e-5
    assert np.linalg.norm(w[3:] - ref[3:]) / np.linalg.norm(ref[3:]) <= 2e-5
    x = np.array([1.0, 2.0, 3.0])
    t = sh_example_table(1)
    plummer = P.SubhaloLinePotential(t["m"], t["a"], t["x0"], t["v"], t["t0"], t["t_window"], units=u)
    hern = P.SubhaloLinePotential_Custom(P.HernquistPotential(m=1e7, r_s=0.2, units=u), t["x0"], t["v"], t["t0"],
                                         t["t_window"], units=u)
    for pot, kind in ((plummer, 1), (hern, 2)):
        phi = float(np64(pot.potential(x, -850.0)).reshape(-1)[0])
        assert abs(phi / SH_PHI_PRINTED[kind] - 1.0) <= 1e-7
    zhao = P.get_potential_from_density(zhao_density, units=u)
    assert abs(float(np64(zhao.potential(x, 0.0)).reshape(-1)[0]) / -0.08283585 - 1.0) <= 1e-6
    g = np64(zhao.gradient(x, 0.0)).reshape(-1)
    assert np.all(np.abs(g - np.array([0.0004346, 0.0008692, 0.0013038])) <= 5e-9)


def _track_and_subhalos(ss, oracle):
    from streamsculptor_gb300 import potential as P
    rng = np.random.default_rng(11)
    tk = np.arange(40) * 2.0 - 20.0
    knots = np.stack([8 + np.cos(tk / 30), np.sin(tk / 25) * 3, 0.1 * tk], axis=1)
    track = ss.CenterTrack.from_samples(tk, knots)
    nsh = 5
    sh = dict(m=10 ** rng.uniform(6, 8, nsh), a=rng.uniform(0.1, 1.0, nsh), x0=rng.normal(0, 5, (nsh, 3)),
              v=rng.normal(0, 0.1, (nsh, 3)), t0=rng.uniform(-10, 10, nsh), t_window=15.0)
    gpu = P.Potential_Combine([mw3_gpu(ss),
                               P.TimeDepTranslatingPotential(P.PlummerPotential(m=3e8, r_s=0.3, units=ss.usys), track,
                                                             units=ss.usys),
                               P.SubhaloLinePotential(sh["m"], sh["a"], sh["x0"], sh["v"], sh["t0"], sh["t_window"],
                                                      units=ss.usys)], units=ss.usys)
    orc = oracle.HostModel(oracle.mw3() + [(_abi.SS_PLUMMER, 1, (3e8, 0.3))], track=(tk[0], 2.0, knots),
                           subhalos=dict(sh, kind=1))
    return gpu, orc


def test_time_dependent_potential_eval(ss, oracle):
    gpu, orc = _track_and_subhalos(ss, oracle)
    x = np.random.default_rng(3).normal(0, 6, size=(200, 3))
    for t in (-30.0, -5.5, 0.0, 13.3, 90.0):
        phi_o, g_o, H_o = oracle.potential_eval(orc, x, t)
        assert rel_err(np64(gpu.potential(x, t)), phi_o) < 1e-12
        assert rel_err(np64(gpu.gradient(x, t)), g_o) < 1e-12


def test_orbit_backwards_f64(ss, oracle):
    pot = mw3_gpu(ss)
    ts = np.array([0.0, -1000.0, -3000.0])
    sol = pot.integrate_orbit(w0=PROG_WF, ts=ts, t0=0.0, t1=-3000.0, dt=1.0)
    ref = oracle.orbit(oracle.HostModel(oracle.mw3()), PROG_WF, 0.0, -1.0, 3000, 1000)[0]
    assert sol.ys.shape == (3, 6)
    assert phase_err(np64(sol.ys), ref[[0, 1, 3]]) < 1e-11


def test_orbit_batch(ss, oracle):
    pot = mw3_gpu(ss)
    w0 = PROG_WF + np.random.default_rng(0).normal(0, 0.5, size=(64, 6)) * np.array([1, 1, 1, .01, .01, .01])
    ts = np.arange(0, 501.0, 50.0)
    ys = np64(pot.integrate_orbit_batch_vmapped(w0=w0, ts=ts, dt=0.5).ys)
    ref = oracle.orbit(oracle.HostModel(oracle.mw3()), w0, 0.0, 0.5, 1000, 100)
    assert ys.shape == (64, 11, 6)
    assert phase_err(ys, ref) < 1e-11


@pytest.mark.parametrize("model", ["fardal", "chen25"])
def test_release_and_jacobian(ss, oracle, model):
    from streamsculptor_gb300.streamhelpers import CHEN25_MEAN, chen25_factor
    pot = mw3_gpu(ss)
    orc = oracle.HostModel(oracle.mw3())
    w = oracle.orbit(orc, PROG_WF, 0.0, 1.0, 300, 10)[0]
    n = w.shape[0]
    kind = 1 if model == "chen25" else 0
    nz = 6 if kind else 4
    z = np.random.default_rng(5).standard_normal((n, 3, nz))
    chen = (CHEN25_MEAN, chen25_factor()) if kind else None
    ics, J = pot._release(w, np.arange(n) * 10.0, 2e4, z, model=kind, chen=chen, jac=True)
    ics_o, J_o = oracle.release(orc, w, np.arange(n) * 10.0, 2e4, z, model_kind=kind, chen=chen, jac=True)
    assert phase_err(np64(ics), ics_o) < 1e-12
    assert rel_err(np64(J), J_o) < 1e-9


def _c1_setup(oracle, n_rel=3000, dt=1.0):
    orc = oracle.HostModel(oracle.mw3())
    T = n_rel * dt
    back = oracle.orbit(orc, PROG_WF, 0.0, -dt, n_rel, n_rel)[0, -1]
    ts = -T + np.arange(n_rel + 1) * dt
    normals = np.random.default_rng(2024).standard_normal((n_rel + 1, 1, 4))
    return orc, back, ts, normals


def test_stream_f64_c1_full_parity(ss, oracle):
    """3000 releases x 2 = 6000 particles, 3000 steps of 1 Myr, final snapshot."""
    orc, back, ts, normals = _c1_setup(oracle)
    pot = mw3_gpu(ss)
    lead, trail = pot.gen_stream_vmapped(ts=ts, prog_w0=back, Msat=2e4, normals=normals)
    ws = oracle.orbit(orc, back, ts[0], 1.0, 3000, 1)[0]
    ics, _ = oracle.release(orc, ws, ts, 2e4, normals)
    final, _, st = oracle.stream(orc, ts[0], 1.0, 3000, ics[:-1].reshape(-1, 6), 2, 1)
    final = final.reshape(3000, 2, 6)
    assert (st == 0).all()
    assert phase_err(np64(lead), final[:, 0]) <= 1e-10
    assert phase_err(np64(trail), final[:, 1]) <= 1e-10


def test_stream_f32k_c1_error_bound(ss, oracle):
    """FP32 stages + compensated accumulation vs the FP64 oracle: <= 1e-5."""
    orc, back, ts, normals = _c1_setup(oracle)
    pot = mw3_gpu(ss)
    lead, trail = pot.gen_stream_vmapped(ts=ts, prog_w0=back, Msat=2e4, normals=normals, precision="f32k")
    ws = oracle.orbit(orc, back, ts[0], 1.0, 3000, 1)[0]
    ics, _ = oracle.release(orc, ws, ts, 2e4, normals)
    final, _, _ = oracle.stream(orc, ts[0], 1.0, 3000, ics[:-1].reshape(-1, 6), 2, 1)
    final = final.reshape(3000, 2, 6)
    err = max(phase_err(np64(lead), final[:, 0]), phase_err(np64(trail), final[:, 1]))
    print(f"f32k C1 max relative phase-space error: {err:.3e}")
    assert err <= 1e-5


def _moving_prog_case(ss, oracle, n_rel=150, ppr=8, dt=0.5, spr=2):
    from streamsculptor_gb300 import potential as P
    orc = oracle.HostModel(oracle.mw3())
    T = n_rel * spr * dt
    back = oracle.orbit(orc, PROG_WF, 0.0, -dt, n_rel * spr, n_rel * spr)[0, -1]
    ts = -T + np.arange(n_rel + 1) * spr * dt
    normals = np.random.default_rng(99).standard_normal((n_rel + 1, ppr // 2, 4))
    ws = oracle.orbit(orc, back, ts[0], dt, n_rel * spr, spr)[0]
    ics, _ = oracle.release(orc, ws, ts, 2e4, normals)
    orc_mov = oracle.HostModel(oracle.mw3() + [(_abi.SS_PLUMMER, 1, (2e4, 0.01))], track=(ts[0], spr * dt, ws[:, :3]))
    prog = P.PlummerPotential(m=2e4, r_s=0.01, units=ss.usys)
    return orc_mov, back, ts, normals, ics, prog, dict(n_rel=n_rel, ppr=ppr, dt=dt, spr=spr)


@pytest.mark.parametrize("precision,tol", [("f64", 1e-10), ("f32k", 1e-5)])
def test_moving_progenitor_stream_with_snapshots(ss, oracle, precision, tol):
    from streamsculptor_gb300.streamhelpers import gen_stream
    orc_mov, back, ts, normals, ics, prog, c = _moving_prog_case(ss, oracle)
    n_rel, ppr, dt, spr = c["n_rel"], c["ppr"], c["dt"], c["spr"]
    lead, trail, snaps = gen_stream(mw3_gpu(ss), ts, back, 2e4, normals=normals, dt=dt, prog_pot=prog,
                                    n_particles_per_release=ppr, precision=precision, snapshot_every=25)
    final, snaps_o, st = oracle.stream(orc_mov, ts[0], dt, n_rel * spr, ics[:-1].reshape(-1, 6), ppr, spr,
                                       snap_stride=25)
    final = final.reshape(n_rel, ppr // 2, 2, 6)
    assert phase_err(np64(lead), final[:, :, 0]) <= tol
    assert phase_err(np64(trail), final[:, :, 1]) <= tol
    s = snaps.detach().cpu().numpy().reshape(snaps_o.shape)
    assert np.array_equal(np.isnan(s), np.isnan(snaps_o))
    ok = ~np.isnan(snaps_o[..., 0])
    # float32 snapshots: one float32 rounding on top of the path's own error
    assert phase_err(s[ok], snaps_o[ok].astype(np.float64)) <= tol + 3e-7


def test_nonlinear_subhalo_stream_parity(ss, oracle):
    from streamsculptor_gb300 import potential as P
    from streamsculptor_gb300.streamhelpers import gen_stream_vmapped_with_pert_fixed_prog
    orc, back, ts, normals = _c1_setup(oracle, n_rel=400)
    rng = np.random.default_rng(8)
    sh = dict(m=np.array([3e7, 1e6, 5e7]), a=np.array([0.5, 0.2, 0.8]), x0=rng.normal(0, 8, (3, 3)),
              v=rng.normal(0, 0.15, (3, 3)), t0=np.array([-300.0, -150.0, -50.0]), t_window=120.0)
    pert = P.SubhaloLinePotential(sh["m"], sh["a"], sh["x0"], sh["v"], sh["t0"], sh["t_window"], units=ss.usys)
    lead, trail = gen_stream_vmapped_with_pert_fixed_prog(mw3_gpu(ss), pert, ts=ts, prog_w0=back, Msat=2e4,
                                                          normals=normals)
    ws = oracle.orbit(orc, back, ts[0], 1.0, 400, 1)[0]
    ics, _ = oracle.release(orc, ws, ts, 2e4, normals)
    tot = oracle.HostModel(oracle.mw3(), subhalos=dict(sh, kind=1))
    final, _, _ = oracle.stream(tot, ts[0], 1.0, 400, ics[:-1].reshape(-1, 6), 2, 1)
    final = final.reshape(400, 2, 6)
    assert phase_err(np64(lead), final[:, 0]) <= 1e-10
    assert phase_err(np64(trail), final[:, 1]) <= 1e-10


def _ensemble_oracle(oracle, sh, b, back, ts_grid, t_end, normals, prog_in_pert, dt=1.0):
    """Stream b of an ensemble on the oracle: its progenitor orbit (in base +
    its own subhalo when prog_in_pert), the release in the base potential,
    the particles in base + subhalo to the last release and then to t_end."""
    row = {k: (v[b:b + 1] if isinstance(v, np.ndarray) else v) for k, v in sh.items()}
    tot = oracle.HostModel(oracle.mw3(), subhalos=dict(row, kind=1))
    base = oracle.HostModel(oracle.mw3())
    n_grid = len(ts_grid)
    ws = oracle.orbit(tot if prog_in_pert else base, back, ts_grid[0], dt, n_grid - 1, 1)[0]
    ics, _ = oracle.release(base, ws, ts_grid, 2e4, normals[:n_grid])
    if t_end is None:
        final, _, _ = oracle.stream(tot, ts_grid[0], dt, n_grid - 1, ics[:-1].reshape(-1, 6), 2, 1)
        return final.reshape(n_grid - 1, 2, 6)
    f1, _, _ = oracle.stream(tot, ts_grid[0], dt, n_grid - 1, ics.reshape(-1, 6), 2, 1)
    span = t_end - ts_grid[-1]
    m = int(np.ceil(span / dt - 1e-9))
    f2, _, _ = oracle.stream(tot, ts_grid[-1], span / m, m, f1, f1.shape[0], 0)
    return f2.reshape(n_grid, 2, 6)


@pytest.mark.parametrize("tail,prog_in_pert", [(False, True), (True, True), (True, False)])
def test_stream_ensemble_parity(ss, oracle, tail, prog_in_pert):
    """gen_stream_ensemble: B streams, each with its own subhalo, in one
    orbit launch, one release launch and one stream launch (FP64 and FP32
    compensated) against the oracle stream by stream; with `tail` the release
    times are followed by an end time off their grid (the reference notebooks'
    ts = [linspace(-t_age, t_dissolve, n), 0])."""
    from streamsculptor_gb300 import potential as P
    from streamsculptor_gb300.streamhelpers import gen_stream_ensemble, gen_stream_vmapped_with_pert
    n = 120
    orc, back, ts, normals = _c1_setup(oracle, n_rel=n)
    if tail:
        ts = np.concatenate([ts[:-1], [ts[-1] + 17.4]])
    rng = np.random.default_rng(12)
    B = 4
    ws = oracle.orbit(orc, back, ts[0], 1.0, n - 1, 1)[0]
    sh = dict(m=10 ** rng.uniform(6.5, 7.7, B), a=rng.uniform(0.2, 0.8, B),
              x0=ws[rng.integers(30, 100, B), :3] + rng.normal(0, 0.6, (B, 3)), v=rng.normal(0, 0.15, (B, 3)),
              t0=ts[0] + rng.uniform(30, 100, B), t_window=60.0)
    pert = P.SubhaloLinePotential(sh["m"], sh["a"], sh["x0"], sh["v"], sh["t0"], sh["t_window"], units=ss.usys)
    ts_grid = ts[:-1] if tail else ts
    t_end = float(ts[-1]) if tail else None
    for precision, tol in (("f64", 1e-10), ("f32k", 1e-5)):
        lead, trail = gen_stream_ensemble(mw3_gpu(ss), pert, 1, ts=ts, prog_w0=back, Msat=2e4, normals=normals,
                                          prog_in_pert=prog_in_pert, precision=precision)
        assert lead.shape == (B, n, 6)
        for b in range(B):
            o = _ensemble_oracle(oracle, sh, b, back, ts_grid, t_end, normals, prog_in_pert)
            assert phase_err(np64(lead[b]), o[:, 0]) <= tol, (precision, b)
            assert phase_err(np64(trail[b]), o[:, 1]) <= tol, (precision, b)
    if prog_in_pert:
        # the single-stream generator on one row gives the ensemble's stream
        b = 2
        one = P.SubhaloLinePotential(sh["m"][b:b + 1], sh["a"][b:b + 1], sh["x0"][b:b + 1], sh["v"][b:b + 1],
                                     sh["t0"][b:b + 1], sh["t_window"], units=ss.usys)
        l1, t1 = gen_stream_vmapped_with_pert(mw3_gpu(ss), one, ts=ts, prog_w0=back, Msat=2e4, normals=normals,
                                              prog_method="serial")
        lead, trail = gen_stream_ensemble(mw3_gpu(ss), pert, 1, ts=ts, prog_w0=back, Msat=2e4, normals=normals)
        assert phase_err(np64(l1), np64(lead[b])) <= 1e-13 and phase_err(np64(t1), np64(trail[b])) <= 1e-13


def test_ensemble_batches_pipelined(ss, oracle):
    """gen_stream_ensemble_batches (two CUDA streams, batch i + 1's orbits
    under batch i's streams) gives every batch exactly what
    gen_stream_ensemble gives it alone; with prog_w0_at="end" each
    progenitor is first integrated back in base + its own subhalo (checked
    against the oracle for one stream)."""
    from streamsculptor_gb300 import potential as P
    from streamsculptor_gb300.streamhelpers import gen_stream_ensemble, gen_stream_ensemble_batches
    n = 80
    orc, back, ts, normals = _c1_setup(oracle, n_rel=n)
    ts = np.concatenate([ts[:-1], [ts[-1] + 6.5]])
    rng = np.random.default_rng(2)
    perts, shs = [], []
    for _ in range(3):
        sh = dict(m=10 ** rng.uniform(6.5, 7.5, 3), a=rng.uniform(0.2, 0.6, 3), x0=rng.normal(0, 9, (3, 3)),
                  v=rng.normal(0, 0.15, (3, 3)), t0=ts[0] + rng.uniform(10, 70, 3), t_window=50.0)
        shs.append(sh)
        perts.append(P.SubhaloLinePotential(sh["m"], sh["a"], sh["x0"], sh["v"], sh["t0"], sh["t_window"],
                                            units=ss.usys))
    kw = dict(ts=ts, prog_w0=PROG_WF, Msat=2e4, normals=normals, prog_w0_at="end")
    for precision in ("f64", "f32k"):
        outs = gen_stream_ensemble_batches(mw3_gpu(ss), perts, 1, precision=precision, **kw)
        for i, pert in enumerate(perts):
            lead, trail = gen_stream_ensemble(mw3_gpu(ss), pert, 1, precision=precision, **kw)
            assert torch.equal(outs[i][0], lead) and torch.equal(outs[i][1], trail)
    # stream 1 of batch 2 on the oracle: back from t_end in base + its subhalo, then as usual
    sh, b = shs[2], 1
    row = {k: (v[b:b + 1] if isinstance(v, np.ndarray) else v) for k, v in sh.items()}
    tot = oracle.HostModel(oracle.mw3(), subhalos=dict(row, kind=1))
    span = ts[-1] - ts[0]
    n_back = int(np.ceil(span / 1.0 - 1e-9))
    start = oracle.orbit(tot, PROG_WF, ts[-1], -span / n_back, n_back, n_back)[0, -1]
    o = _ensemble_oracle(oracle, sh, b, start, ts[:-1], float(ts[-1]), normals, True)
    assert phase_err(np64(outs[2][0][b]), o[:, 0]) <= 1e-5  # outs holds the f32k run
    lead64, _ = gen_stream_ensemble(mw3_gpu(ss), perts[2], 1, precision="f64", **kw)
    assert phase_err(np64(lead64[b]), o[:, 0]) <= 1e-10


def test_orbit_ensemble_own_steps(ss, oracle):
    """ss_orbit_ensemble_f64: every orbit with its own step and end time,
    against the oracle orbit of each."""
    from streamsculptor_gb300 import _core
    orc = oracle.HostModel(oracle.mw3())
    rng = np.random.default_rng(3)
    w0 = PROG_WF + rng.normal(0, 0.5, (7, 6)) * np.array([1, 1, 1, 0.01, 0.01, 0.01])
    t1 = -rng.uniform(100, 900, 7)
    n = 600
    out = np64(_core.orbit_ensemble(mw3_gpu(ss)._desc(), _core.f64(w0), 0.0, _core.f64(t1 / n), n))
    for i in range(7):
        ref = oracle.orbit(orc, w0[i], 0.0, t1[i] / n, n, n)[0, -1]
        assert phase_err(out[i, -1], ref) <= 1e-11


@pytest.mark.parametrize("fixed", [True, False])
def test_chen25_perturbed_stream_parity(ss, oracle, fixed):
    """gen_stream_vmapped_with_pert_Chen25[_fixed_prog] (streamhelpers.py:546-653):
    Chen25 release, Hernquist subhalos on lines, moving Plummer progenitor;
    the progenitor orbit in base + perturbation unless fixed."""
    from streamsculptor_gb300 import potential as P
    from streamsculptor_gb300 import streamhelpers as H
    n_rel, dt = 300, 1.0
    orc_base = oracle.HostModel(oracle.mw3())
    back = oracle.orbit(orc_base, PROG_WF, 0.0, -dt, n_rel, n_rel)[0, -1]
    ts = -n_rel * dt + np.arange(n_rel + 1) * dt
    rng = np.random.default_rng(12)
    sh = dict(m=np.array([4e7, 2e6]), a=np.array([0.6, 0.3]), x0=rng.normal(0, 8, (2, 3)),
              v=rng.normal(0, 0.15, (2, 3)), t0=np.array([-200.0, -80.0]), t_window=150.0)
    pert = P.SubhaloLinePotential_Custom(P.HernquistPotential(m=sh["m"], r_s=sh["a"], units=ss.usys), sh["x0"],
                                         sh["v"], sh["t0"], sh["t_window"], units=ss.usys)
    normals = rng.standard_normal((n_rel + 1, 1, 6))
    prog = P.PlummerPotential(m=2e4, r_s=0.01, units=ss.usys)
    fn = H.gen_stream_vmapped_with_pert_Chen25_fixed_prog if fixed else H.gen_stream_vmapped_with_pert_Chen25
    lead, trail = fn(pot_base=mw3_gpu(ss), pot_pert=pert, prog_pot=prog, ts=ts, prog_w0=back, Msat=2e4,
                     normals=normals)
    orc_total = oracle.HostModel(oracle.mw3(), subhalos=dict(sh, kind=2))
    ws = oracle.orbit(orc_base if fixed else orc_total, back, ts[0], dt, n_rel, 1)[0]
    from streamsculptor_gb300.streamhelpers import CHEN25_MEAN, chen25_factor
    ics, _ = oracle.release(orc_base, ws, ts, 2e4, normals, model_kind=1, chen=(CHEN25_MEAN, chen25_factor()))
    integ = oracle.HostModel(oracle.mw3() + [(_abi.SS_PLUMMER, 1, (2e4, 0.01))], track=(ts[0], dt, ws[:, :3]),
                             subhalos=dict(sh, kind=2))
    final, _, st = oracle.stream(integ, ts[0], dt, n_rel, ics[:-1].reshape(-1, 6), 2, 1)
    final = final.reshape(n_rel, 2, 6)
    assert (st == 0).all()
    assert phase_err(np64(lead), final[:, 0]) <= 1e-10
    assert phase_err(np64(trail), final[:, 1]) <= 1e-10


def _pert_case(oracle, N=24, nsh=7, n_steps=120, seed=4):
    rng = np.random.default_rng(seed)
    sh = dict(kind=1, m=10 ** rng.uniform(5, 8, nsh), a=rng.uniform(0.1, 1.0, nsh), x0=rng.normal(0, 10, (nsh, 3)),
              v=rng.normal(0, 0.12, (nsh, 3)), t0=rng.uniform(0, 100, nsh), t_window=60.0)
    orc = oracle.HostModel(oracle.mw3(), subhalos=sh)
    base = PROG_WF + rng.normal(0, 0.3, (N, 6)) * np.array([1, 1, 1, 0.01, 0.01, 0.01])
    pert = rng.normal(0, 1e-3, (N, nsh, 18))
    return sh, orc, base, pert


@pytest.mark.parametrize("ncol", [12, 6, 18])
def test_pert_response_f64_and_f32(ss, oracle, ncol):
    """First-order response (6 mass or 12 mass + radius columns) and the
    second-order mass response (18 columns: + x2, v2 of
    MassRadiusPerturbation_OTF_SecondOrder, fields.py:260-320)."""
    from streamsculptor_gb300 import _core
    sh, orc, base, pert = _pert_case(oracle)
    pert = np.ascontiguousarray(pert[:, :, :ncol])
    N, nsh = pert.shape[0], pert.shape[1]
    ppr, spr, n_steps, dt = 4, 10, 120, 1.0
    bo, po = oracle.pert_response(orc, 0.0, dt, n_steps, base, pert, ppr, spr, ncol=ncol, save_stride=30)
    table = _core.SubhaloTable(1, *(_core.f64(sh[k]) for k in ("m", "a")), _core.f64(sh["x0"]), _core.f64(sh["v"]),
                               _core.f64(sh["t0"]), sh["t_window"])
    cfg = _abi.ss_pert_cfg()
    cfg.t0, cfg.dt, cfg.n_steps, cfg.n_particles = 0.0, dt, n_steps, N
    cfg.particles_per_release, cfg.steps_per_release, cfg.ncol, cfg.save_stride = ppr, spr, ncol, 30
    P = mw3_gpu(ss)._desc()
    for prec, tol in ((64, 1e-10), (32, 2e-4)):
        # a small chunk forces several particle chunks through the workspace
        b, p = _core.pert_response(P, table, cfg, prec, _core.f64(base), _core.f64(pert), chunk_particles=5)
        assert phase_err(np64(b), bo) < 1e-12
        assert rel_err(np64(p), po) < tol, prec


def test_pert_field_term_matches_oracle(ss, oracle):
    from streamsculptor_gb300 import fields, perturbative, potential as P
    sh, orc, base, pert = _pert_case(oracle, N=1)
    pot_sh = P.SubhaloLinePotential(sh["m"], sh["a"], sh["x0"], sh["v"], sh["t0"], sh["t_window"], units=ss.usys)
    pot_st = P.SubhaloLinePotential_dRadius(sh["m"], sh["a"], sh["x0"], sh["v"], sh["t0"], sh["t_window"],
                                            units=ss.usys)
    gen = perturbative.GenerateMassRadiusPerturbation(mw3_gpu(ss), pot_sh, pot_st)
    f = fields.MassRadiusPerturbation_OTF(gen)
    for t in (10.0, 55.0):
        d0, d1 = f.term(t, [base[0], pert[0][:, :12]])
        o0, o1 = oracle.pert_term(orc, t, base[0], pert[0][:, :12])
        assert rel_err(np64(d0), o0) < 1e-12
        assert rel_err(np64(d1), o1) < 1e-11


@pytest.mark.parametrize("ncol", [6, 12, 18])
def test_pert_term_kernel_matches_oracle(ss, oracle, ncol):
    """ss_pert_term (the field at one point) for the first- and second-order
    layouts, and the second-order field class built on it."""
    from types import SimpleNamespace

    from streamsculptor_gb300 import _core, fields
    sh, orc, base, pert = _pert_case(oracle, N=1)
    table = _core.SubhaloTable(1, *(_core.f64(sh[k]) for k in ("m", "a")), _core.f64(sh["x0"]), _core.f64(sh["v"]),
                               _core.f64(sh["t0"]), sh["t_window"])
    pot = mw3_gpu(ss)
    u = pert[0][:, :ncol]
    for t in (10.0, 55.0):
        dy = np64(_core.pert_term(pot._desc(), table, ncol, t, _core.f64(np.concatenate([base[0], u.ravel()]))))
        o0, o1 = oracle.pert_term(orc, t, base[0], u, ncol=ncol)
        assert rel_err(dy[:6], o0) < 1e-12
        d1 = dy[6:].reshape(-1, ncol)
        assert rel_err(d1[:, :6], o1[:, :6]) < 1e-11
        if ncol >= 12:
            assert rel_err(d1[:, 6:12], o1[:, 6:12]) < 1e-11
        if ncol == 18:
            assert rel_err(d1[:, 12:], o1[:, 12:]) < 1e-11
            f = fields.MassRadiusPerturbation_OTF_SecondOrder(SimpleNamespace(potential_base=pot, sh_table=table))
            c0, c1, c2 = f.term(t, [base[0], u[:, :12], u[:, 12:]])
            assert rel_err(np64(c1), o1[:, :12]) < 1e-11 and rel_err(np64(c2), o1[:, 12:]) < 1e-11


def test_custom_base_second_order_matches_oracle(ss, oracle):
    """GenerateMassRadiusPerturbation_CustomBase(_SecondOrder) on a
    CustomBaseStreamModel (perturbative.py:299-585): the progenitor's 18-column
    response integrated backwards from zero at t_obs, the identity release
    Jacobian, every particle's response forward to t_obs; the first-order
    generator gives the same 12 columns."""
    from streamsculptor_gb300 import perturbative, potential as P
    n_rel = 60
    orc, back, ts, _ = _c1_setup(oracle, n_rel=n_rel)
    rng = np.random.default_rng(31)
    pos_rel = rng.normal(0, 0.05, (n_rel + 1, 3))
    vel_rel = rng.normal(0, 0.002, (n_rel + 1, 3))
    ws = oracle.orbit(orc, back, ts[0], 1.0, n_rel, 1)[0]
    sh = dict(kind=1, m=np.array([3e6, 2e7, 8e6]), a=np.array([0.3, 0.6, 0.4]),
              x0=ws[[20, 40, 50], :3] + rng.normal(0, 0.5, (3, 3)), v=rng.normal(0, 0.1, (3, 3)),
              t0=np.array([ts[20], ts[40], ts[50]]), t_window=30.0)
    args = (sh["m"], sh["a"], sh["x0"], sh["v"], sh["t0"], sh["t_window"])
    pot_sh = P.SubhaloLinePotential(*args, units=ss.usys)
    pot_st = P.SubhaloLinePotential_dRadius(*args, units=ss.usys)
    bsm = perturbative.CustomBaseStreamModel(mw3_gpu(ss), back, ts, pos_rel, vel_rel)
    gen2 = perturbative.GenerateMassRadiusPerturbation_CustomBase_SecondOrder(mw3_gpu(ss), pot_sh, pot_st, bsm)
    base, d1, d2 = gen2.compute_perturbation_OTF()
    gen1 = perturbative.GenerateMassRadiusPerturbation_CustomBase(mw3_gpu(ss), pot_sh, pot_st, bsm)
    b1, e1 = gen1.compute_perturbation_OTF()
    ics = ws + np.concatenate([pos_rel, vel_rel], axis=1)
    orc_sh = oracle.HostModel(oracle.mw3(), subhalos=sh)
    _, prog = oracle.pert_response(orc_sh, ts[-1], -1.0, n_rel, ws[-1:], None, 1, 0, ncol=18, save_stride=1)
    pf = np.ascontiguousarray(prog[::-1, 0])  # [n_rel + 1, n_sh, 18], time increasing
    assert rel_err(np64(gen2.prog_fieldICs_all), pf) <= 1e-10
    bo, po = oracle.pert_response(orc_sh, ts[0], 1.0, n_rel, ics[:-1], pf[:-1], 1, 1, ncol=18)
    assert base.shape == (n_rel, 6) and d1.shape == (n_rel, 3, 12) and d2.shape == (n_rel, 3, 6)
    assert phase_err(np64(base), bo) <= 1e-10
    assert rel_err(np64(d1), po[0][..., :12]) <= 1e-9
    assert rel_err(np64(d2), po[0][..., 12:]) <= 1e-9
    assert np.abs(np64(d2)).max() > 0
    assert phase_err(np64(b1), np64(base)) <= 1e-14
    assert rel_err(np64(e1), np64(d1)) <= 1e-12
    s0 = bsm.gen_stream()
    assert phase_err(np64(s0), bo) <= 1e-10


def test_linear_response_matches_nonlinear_difference(ss, oracle):
    """d(stream)/d(eps) from the perturbation generator vs the nonlinear
    stream with a small subhalo (the check of examples/tests.ipynb cells
    120-130).  The linear theory holds the progenitor's present-day state
    fixed (its response is integrated backwards from t_obs), so the
    nonlinear stream starts from the progenitor integrated back from the
    same present-day state in base + subhalo."""
    from streamsculptor_gb300 import perturbative, potential as P
    from streamsculptor_gb300.streamhelpers import gen_stream_vmapped_with_pert
    n_rel = 300
    orc, back, ts, normals = _c1_setup(oracle, n_rel=n_rel)
    base_pot = mw3_gpu(ss)
    ws = oracle.orbit(orc, back, ts[0], 1.0, n_rel, 1)[0]
    t_imp = ts[200]
    x_imp = ws[200, :3] * 0.995
    m_sh, a_sh = 1e5, 0.3
    v_sh = np.array([0.05, -0.1, 0.08])
    args = (np.array([m_sh]), np.array([a_sh]), x_imp[None], v_sh[None], np.array([t_imp]), 1e9)
    pot_sh = P.SubhaloLinePotential(*args, units=ss.usys)
    pot_st = P.SubhaloLinePotential_dRadius(*args, units=ss.usys)
    bsm = perturbative.BaseStreamModel(base_pot, back, ts, 2e4, 0, normals=normals)
    gen = perturbative.GenerateMassRadiusPerturbation(base_pot, pot_sh, pot_st, bsm)
    (lb, ld), (tb, td) = gen.compute_perturbation_OTF()
    lead0, trail0 = base_pot.gen_stream_vmapped(ts=ts, prog_w0=back, Msat=2e4, normals=normals)
    assert phase_err(np64(lb), np64(lead0)) < 1e-12
    total = P.Potential_Combine([base_pot, pot_sh], units=ss.usys)
    w_obs = np64(bsm.prog_loc_fwd[-1])
    back_p = total.integrate_orbit(w0=w_obs, ts=[ts[-1], ts[0]], t0=ts[-1], t1=ts[0], dt=1.0).ys[-1]
    lead1, trail1 = gen_stream_vmapped_with_pert(base_pot, pot_sh, ts=ts, prog_w0=back_p, Msat=2e4, normals=normals)
    for nl, base, lin in ((lead1, lead0, ld), (trail1, trail0, td)):
        dn = np64(nl) - np64(base)
        dl = np64(lin)[:, 0, :6]
        # the remainder is second order in the subhalo mass
        assert np.max(np.abs(dn - dl)) <= 0.02 * np.max(np.abs(dn))


def test_binned_track_matches_oracle(ss, oracle):
    from streamsculptor_gb300 import computed_binned_track
    rng = np.random.default_rng(12)
    stream = rng.normal(size=(5000, 6))
    stream[::31, 2] = np.nan
    phi1 = rng.uniform(-1.0, 1.5, 5000)
    out = np64(computed_binned_track(stream, phi1, bins=33))
    edges = np.linspace(phi1.min(), phi1.max(), 33)
    sums, counts = oracle.binned_sums(stream, phi1, edges)
    with np.errstate(invalid="ignore", divide="ignore"):
        ref = sums / counts
    ref[ref == 0] = np.nan
    assert out.shape == (32, 6)
    assert np.array_equal(np.isnan(out), np.isnan(ref))
    ok = ~np.isnan(ref)
    assert rel_err(out[ok], ref[ok]) < 1e-12


def test_edge_cases(ss):
    from streamsculptor_gb300 import _core
    pot = mw3_gpu(ss)
    # empty batch
    assert pot.gradient(np.zeros((0, 3)), 0.0).shape == (0, 3)
    # non-finite initial condition -> status 1, others 0
    P = pot._desc()
    cfg = _abi.ss_stream_cfg()
    cfg.t0, cfg.dt, cfg.n_steps, cfg.n_particles = 0.0, 1.0, 10, 4
    cfg.particles_per_release, cfg.steps_per_release = 2, 1
    ics = torch.tensor(np.tile(PROG_WF, (4, 1)), dtype=torch.float64, device="cuda")
    ics[3, 0] = float("nan")
    for prec in ("f64", "f32k"):
        final, st = _core.stream(P, cfg, ics, prec)
        assert st.tolist() == [0, 0, 0, 1]
    # a particle released at the last step keeps its initial state
    cfg.n_particles, cfg.particles_per_release, cfg.steps_per_release = 2, 1, 10
    final, st = _core.stream(P, cfg, ics[:2].contiguous(), "f64")
    assert torch.equal(final[1], ics[1]) and st.tolist() == [0, 0]
    # invalid arguments raise with the library's message
    bad = _abi.ss_stream_cfg()
    bad.dt = 0.0
    bad.particles_per_release = 1
    with pytest.raises(_abi.SSError, match="dt"):
        _core.stream(P, bad, ics, "f64")
    with pytest.raises(NotImplementedError):
        pot.integrate_orbit(w0=PROG_WF, ts=[0.0, 10.0], solver="Dopri8")


def test_chen25_perturbation_matches_oracle(ss, oracle):
    """GenerateMassRadiusPerturbation_Chen25: base stream in base + moving
    progenitor, zero initial response (perturbative.py:661-773)."""
    from streamsculptor_gb300 import perturbative, potential as P
    from streamsculptor_gb300.streamhelpers import CHEN25_MEAN, chen25_factor
    n_rel = 60
    orc, back, ts, _ = _c1_setup(oracle, n_rel=n_rel)
    rng = np.random.default_rng(21)
    z = rng.standard_normal((n_rel + 1, 1, 6))
    sh = dict(kind=1, m=np.array([3e6, 2e7]), a=np.array([0.3, 0.6]), x0=rng.normal(0, 8, (2, 3)),
              v=rng.normal(0, 0.1, (2, 3)), t0=np.array([ts[20], ts[45]]), t_window=30.0)
    prog = P.PlummerPotential(m=2e4, r_s=0.01, units=ss.usys)
    bsm = perturbative.BaseStreamModelChen25(mw3_gpu(ss), ts, back, 2e4, 7, prog_pot=prog, normals=z)
    pot_sh = P.SubhaloLinePotential(sh["m"], sh["a"], sh["x0"], sh["v"], sh["t0"], sh["t_window"], units=ss.usys)
    gen = perturbative.GenerateMassRadiusPerturbation_Chen25(mw3_gpu(ss), pot_sh, bsm)
    base, derivs = gen.compute_perturbation_OTF()
    ws = oracle.orbit(orc, back, ts[0], 1.0, n_rel, 1)[0]
    ics, _ = oracle.release(orc, ws, ts, 2e4, z, model_kind=1, chen=(CHEN25_MEAN, chen25_factor()))
    model = oracle.HostModel(oracle.mw3() + [(_abi.SS_PLUMMER, 1, (2e4, 0.01))], track=(ts[0], 1.0, ws[:, :3]),
                             subhalos=sh)
    bo, po = oracle.pert_response(model, ts[0], 1.0, n_rel, ics.reshape(-1, 6), None, 2, 1, ncol=12)
    N = 2 * (n_rel + 1) - 1
    assert base.shape == (N, 6) and derivs.shape == (N, 2, 12)
    assert phase_err(np64(base), bo[:N]) <= 1e-10
    assert rel_err(np64(derivs), po[0][:N]) <= 1e-9


def test_orbit_parallel_in_time_vs_oracle(ss, oracle):
    """Multiple-shooting FP64 orbit (8000 steps back, 500 slices) against the
    serial FP64 oracle, and the serial GPU kernel."""
    pot = mw3_gpu(ss)
    ts = [0.0, -1000.0, -2000.0, -3000.0, -4000.0]
    shoot = pot.integrate_orbit(w0=PROG_WF, ts=ts, t0=0.0, t1=-4000.0, dt=0.5, method="shoot")
    serial = pot.integrate_orbit(w0=PROG_WF, ts=ts, t0=0.0, t1=-4000.0, dt=0.5, method="serial")
    ref = oracle.orbit(oracle.HostModel(oracle.mw3()), PROG_WF, 0.0, -0.5, 8000, 2000)[0]
    assert phase_err(np64(shoot.ys), ref) < 1e-11
    assert phase_err(np64(shoot.ys), np64(serial.ys)) < 1e-12
    # a length that is not a multiple of the slice, saved every step
    w = pot.integrate_orbit(w0=PROG_WF, ts=np.arange(0.0, 101.5, 0.5), dt=0.5, method="shoot").ys  # 202 steps
    ref2 = oracle.orbit(oracle.HostModel(oracle.mw3()), PROG_WF, 0.0, 0.5, 202, 1)[0]
    assert phase_err(np64(w), ref2) < 1e-12
    # time-dependent potentials fall back to the serial kernel
    gpu, orc = _track_and_subhalos(ss, oracle)
    w3, _, _ = gpu._prog_orbit(np.arange(0.0, 41.0, 2.0) - 20.0, PROG_WF, 0.5, method="shoot")
    ref3 = oracle.orbit(orc, PROG_WF, -20.0, 0.5, 80, 4)[0]
    assert phase_err(np64(w3), ref3) < 1e-11


@pytest.mark.parametrize("precision,host_mode", [("f64", "direct"), ("f32k", "direct"), ("f64", "chunked"),
                                                  ("f32k", "chunked")])
def test_host_output_matches_device(ss, oracle, precision, host_mode):
    """gen_stream(out='host'): 'direct' writes the snapshots from the stream
    kernel straight into pinned host memory, 'chunked' runs the stream in
    particle sub-ranges (first_particle / snap_pitch) with overlapped copies;
    every particle's arithmetic is unchanged, so both equal the device run.
    12 particles per release: the paired kernel's warps cover 64 particles,
    so rows are written both as whole-warp lines and per particle."""
    from streamsculptor_gb300.streamhelpers import gen_stream
    orc_mov, back, ts, normals, ics, prog, c = _moving_prog_case(ss, oracle, n_rel=150, ppr=12)
    kw = dict(normals=normals, dt=c["dt"], prog_pot=prog, n_particles_per_release=c["ppr"], precision=precision,
              snapshot_every=20)
    d = gen_stream(mw3_gpu(ss), ts, back, 2e4, **kw)
    h = gen_stream(mw3_gpu(ss), ts, back, 2e4, out="host", host_mode=host_mode, **kw)
    assert not h[0].is_cuda and h[0].is_pinned()
    for a, b in zip(d, h):
        a, b = a.cpu().numpy(), b.numpy()
        assert a.shape == b.shape
        assert np.array_equal(a, b, equal_nan=True)


@pytest.mark.parametrize("precision", [64, 32])
def test_interp_response_equals_otf_for_several_batches(ss, oracle, precision):
    """compute_perturbation_Interp (stored base track, perturbative.py:178-221)
    gives the OTF results for every subhalo batch built on one base stream,
    and the Interp field term equals the OTF term at the stored base state."""
    from streamsculptor_gb300 import fields, perturbative, potential as P
    n_rel = 120
    orc, back, ts, normals = _c1_setup(oracle, n_rel=n_rel)
    base_pot = mw3_gpu(ss)
    bsm = perturbative.BaseStreamModel(base_pot, back, ts, 2e4, 0, normals=normals)
    rng = np.random.default_rng(21)
    for batch in range(2):
        nsh = 5 + 3 * batch
        args = (10 ** rng.uniform(5, 7, nsh), rng.uniform(0.1, 0.5, nsh), rng.normal(0, 8, (nsh, 3)),
                rng.normal(0, 0.1, (nsh, 3)), rng.uniform(ts[0], ts[-1], nsh), 1e9)
        gen = perturbative.GenerateMassRadiusPerturbation(base_pot, P.SubhaloLinePotential(*args, units=ss.usys),
                                                          P.SubhaloLinePotential_dRadius(*args, units=ss.usys), bsm,
                                                          precision=precision)
        (lo, ldo), (to, tdo) = gen.compute_perturbation_OTF()
        (li, ldi), (ti, tdi) = gen.compute_perturbation_Interp()
        for a, b in ((lo, li), (ldo, ldi), (to, ti), (tdo, tdi)):
            assert torch.equal(a, b)
    # the Interp field at a stored state equals the OTF field there
    f_i = fields.MassRadiusPerturbation_Interp(gen)
    f_o = fields.MassRadiusPerturbation_OTF(gen)
    d = torch.as_tensor(rng.normal(0, 1e-3, (gen.num_pert, 12)), device="cuda")
    out_i = f_i.term(ts[-1], d, {"idx": 10, "tail_bool": True})
    out_o = f_o.term(ts[-1], [lo[10], d])[1]
    assert rel_err(np64(out_i), np64(out_o)) < 1e-12


@pytest.mark.parametrize("precision", ["f64", "f32k"])
def test_release_range_equals_whole_stream(ss, oracle, precision):
    """One rank's share of a stream split across GPUs (gen_stream(release_range=),
    the ranges of sharding.balanced_ranges) equals the same releases of the
    whole stream, bit for bit."""
    from streamsculptor_gb300.sharding import balanced_ranges
    from streamsculptor_gb300.streamhelpers import gen_stream
    n = 300
    _, back, ts, normals = _c1_setup(oracle, n_rel=n)
    pot = mw3_gpu(ss)
    lead, trail = gen_stream(pot, ts, back, 2e4, normals=normals, precision=precision)
    for p0, p1 in balanced_ranges(2 * n, 2, 1, n, 3):
        r0, r1 = p0 // 2, p1 // 2
        l, t = gen_stream(pot, ts, back, 2e4, normals=normals, precision=precision, release_range=(r0, r1))
        assert torch.equal(l, lead[r0:r1]) and torch.equal(t, trail[r0:r1])


@pytest.mark.parametrize("precision", ["f64", "f32k"])
def test_gen_stream_sharded_ranks_tile_the_whole_stream(ss, oracle, precision):
    """sharding.gen_stream_sharded called as each of 3 ranks would call it
    (in one process, without the gather): the ranks' release ranges tile the
    stream in order and each rank's result equals the same releases of the
    whole stream, bit for bit.  The gather itself is tested on CPU with two
    gloo ranks (tests/test_sharding.py)."""
    from streamsculptor_gb300.sharding import gen_stream_sharded
    from streamsculptor_gb300.streamhelpers import gen_stream
    n = 300
    _, back, ts, normals = _c1_setup(oracle, n_rel=n)
    pot = mw3_gpu(ss)
    lead, trail = gen_stream(pot, ts, back, 2e4, normals=normals, precision=precision)
    edge = 0
    for rank in range(3):
        l, t, (r0, r1) = gen_stream_sharded(pot, ts, back, 2e4, rank, 3, gather=False, normals=normals,
                                            precision=precision)
        assert r0 == edge and r1 > r0
        assert torch.equal(l, lead[r0:r1]) and torch.equal(t, trail[r0:r1])
        edge = r1
    assert edge == n


_PAIR_MODELS = {
    "mw3p": None,  # NFW + MN + Hernquist + the moving Plummer progenitor
    "tri3": [("TriaxialNFWPotential", dict(m=3e11, r_s=12.0, q1=1.0, q2=0.9, q3=0.8),
              (_abi.SS_TRIAXIAL_NFW, 0, (3e11, 12.0, 1.0, 0.9, 0.8))),
             ("MiyamotoNagaiDisk", dict(m=6.8e10, a=3.0, b=0.28), (_abi.SS_MIYAMOTO_NAGAI, 0, (6.8e10, 3.0, 0.28))),
             ("HernquistPotential", dict(m=5e9, r_s=1.0), (_abi.SS_HERNQUIST, 0, (5e9, 1.0, 0.0)))],
    "gala": [("MiyamotoNagaiDisk", dict(m=6.8e10, a=3.0, b=0.28), (_abi.SS_MIYAMOTO_NAGAI, 0, (6.8e10, 3.0, 0.28))),
             ("HernquistPotential", dict(m=5e9, r_s=1.0), (_abi.SS_HERNQUIST, 0, (5e9, 1.0, 0.0))),
             ("HernquistPotential", dict(m=1.7e9, r_s=0.07), (_abi.SS_HERNQUIST, 0, (1.7e9, 0.07, 0.0))),
             ("NFWPotential", dict(m=5.4e11, r_s=15.62), (_abi.SS_NFW, 0, (5.4e11, 15.62, 0.0)))],
}


@pytest.mark.parametrize("model,ppr,first", [("mw3p", 3, 5), ("mw3p", 8, 7), ("tri3", 5, 0), ("gala", 3, 2)])
def test_f32k_paired_lanes_odd_layouts(ss, oracle, model, ppr, first):
    """The FP32 stream kernel carries two particles per thread.  An odd
    particle count per release splits a pair across two release times, an
    odd first particle shifts every pair, and an odd particle count leaves
    the last thread one particle: each particle still matches the oracle
    (<= 1e-5), snapshots included (NaN rows before release)."""
    from streamsculptor_gb300 import _core, potential as P
    n_rel, dt, spr, stride = 60, 0.5, 3, 7
    n_steps = n_rel * spr
    if model == "mw3p":
        comps, gpu = oracle.mw3(), mw3_gpu(ss)
    else:
        comps = [spec for _, _, spec in _PAIR_MODELS[model]]
        gpu = P.Potential_Combine([getattr(P, name)(**kw, units=ss.usys) for name, kw, _ in _PAIR_MODELS[model]],
                                  units=ss.usys)
    base = oracle.HostModel(comps)
    back = oracle.orbit(base, PROG_WF, 0.0, -dt, n_steps, n_steps)[0, -1]
    ts = -n_steps * dt + np.arange(n_rel + 1) * spr * dt
    ws = oracle.orbit(base, back, ts[0], dt, n_steps, spr)[0]  # the progenitor at the release times
    orc = base
    if model == "mw3p":
        orc = oracle.HostModel(comps + [(_abi.SS_PLUMMER, 1, (2e4, 0.01))], track=(ts[0], spr * dt, ws[:, :3]))
        track = ss.CenterTrack.from_samples(ts, ws[:, :3])
        gpu = P.Potential_Combine([gpu, P.TimeDepTranslatingPotential(P.PlummerPotential(m=2e4, r_s=0.01,
                                                                                         units=ss.usys),
                                                                      track, units=ss.usys)], units=ss.usys)
    rng = np.random.default_rng(17)
    n_all = n_rel * ppr
    scale = np.array([0.05, 0.05, 0.05, 0.005, 0.005, 0.005])
    ics_all = np.repeat(ws[:n_rel], ppr, axis=0) + rng.normal(0, 1, (n_all, 6)) * scale
    n = n_all - first
    n -= 1 - n % 2  # an odd count
    ics = ics_all[first:first + n]
    cfg = _abi.ss_stream_cfg()
    cfg.t0, cfg.dt, cfg.n_steps, cfg.n_particles = float(ts[0]), dt, n_steps, n
    cfg.particles_per_release, cfg.steps_per_release, cfg.snap_stride = ppr, spr, stride
    cfg.first_particle = first
    snaps = torch.full((n_steps // stride, first + n, 6), 7.0, dtype=torch.float32, device="cuda")
    final, st = _core.stream(gpu._desc(), cfg, torch.as_tensor(ics, device="cuda"), "f32k", snaps=snaps)
    torch.cuda.synchronize()
    final_o, snaps_o, st_o = oracle.stream(orc, ts[0], dt, n_steps, ics, ppr, spr, snap_stride=stride,
                                           first_particle=first)
    assert (np64(st) == 0).all() and (st_o == 0).all()
    assert phase_err(np64(final), final_o) <= 1e-5
    s = snaps.cpu().numpy()
    assert (s[:, :first] == 7.0).all()  # rows of other particles untouched
    s = s[:, first:]
    assert np.array_equal(np.isnan(s), np.isnan(snaps_o))
    ok = ~np.isnan(snaps_o[..., 0])
    assert phase_err(s[ok], snaps_o[ok].astype(np.float64)) <= 1e-5 + 3e-7


@pytest.mark.parametrize("kind,grp,first", [("plummer", 0, 0), ("hernquist", 0, 3), ("plummer", 60, 0),
                                            ("hernquist", 60, 60), ("plummer", 60, 5), ("hernquist", 57, 0)])
def test_f32k_paired_lanes_with_subhalo_lines(ss, oracle, kind, grp, first):
    """FP32 streams through Plummer or Hernquist subhalo lines against the
    oracle (<= 1e-5 per particle).  grp = 0: every particle feels the whole
    table; grp > 0: an ensemble of streams of grp particles, stream b feeling
    subhalo rows [2b, 2b + 2).  The two-particle kernel runs when a pair
    never straddles two streams (whole table, or an even stream length and an
    even first particle); an odd stream length or an odd first particle takes
    the one-particle kernel, with the same answer."""
    from streamsculptor_gb300 import _core, potential as P
    n_rel, dt, spr, ppr = 20, 0.5, 3, 3
    n_steps = n_rel * spr + 40
    base = oracle.HostModel(oracle.mw3())
    back = oracle.orbit(base, PROG_WF, 0.0, -dt, n_steps, n_steps)[0, -1]
    t0 = -n_steps * dt
    ws = oracle.orbit(base, back, t0, dt, n_steps, 1)[0]  # the progenitor at every step
    rng = np.random.default_rng(23)
    B = 3
    n_sh = 2 * B
    when = rng.integers(10, n_steps - 10, n_sh)
    sh = dict(m=10 ** rng.uniform(7.0, 8.0, n_sh), a=rng.uniform(0.2, 0.6, n_sh),
              x0=ws[when, :3] + rng.normal(0, 0.3, (n_sh, 3)), v=rng.normal(0, 0.15, (n_sh, 3)),
              t0=t0 + when * dt, t_window=15.0)
    if kind == "plummer":
        pert = P.SubhaloLinePotential(sh["m"], sh["a"], sh["x0"], sh["v"], sh["t0"], sh["t_window"],
                                      units=ss.usys)
        okind = 1
    else:
        sh["m"][:] = 4e7
        sh["a"][:] = 0.4
        pert = P.SubhaloLinePotential_Custom(P.HernquistPotential(m=4e7, r_s=0.4, units=ss.usys), sh["x0"],
                                             sh["v"], sh["t0"], sh["t_window"], units=ss.usys)
        okind = 2
    gpu = P.Potential_Combine([mw3_gpu(ss), pert], units=ss.usys)
    orc = oracle.HostModel(oracle.mw3(), subhalos=dict(sh, kind=okind))
    n_all = B * grp if grp else n_rel * ppr
    rel = (np.arange(n_all) % (grp or n_all)) // ppr  # release index of each particle in its stream
    scale = np.array([0.05, 0.05, 0.05, 0.005, 0.005, 0.005])
    ics_all = ws[rel * spr] + rng.normal(0, 1, (n_all, 6)) * scale
    n = n_all - first
    ics = ics_all[first:]
    cfg = _abi.ss_stream_cfg()
    cfg.t0, cfg.dt, cfg.n_steps, cfg.n_particles = t0, dt, n_steps, n
    cfg.particles_per_release, cfg.steps_per_release = ppr, spr
    cfg.first_particle = first
    if grp:
        cfg.stream_particles, cfg.subhalos_per_stream = grp, 2
    final, st = _core.stream(gpu._desc(), cfg, torch.as_tensor(ics, device="cuda"), "f32k")
    torch.cuda.synchronize()
    final_o, _, st_o = oracle.stream(orc, t0, dt, n_steps, ics, ppr, spr, stream_particles=grp if grp else 0,
                                     subhalos_per_stream=2 if grp else 0, first_particle=first)
    assert (np64(st) == 0).all() and (st_o == 0).all()
    # the subhalos move the particles: the comparison is not of unperturbed tracks
    free, _, _ = oracle.stream(base, t0, dt, n_steps, ics, ppr, spr, stream_particles=grp if grp else 0,
                               first_particle=first)
    assert phase_err(free, final_o) > 1e-4
    assert phase_err(np64(final), final_o) <= 1e-5


def test_structural_subhalo_classes(ss, oracle):
    """The structural (dPhi_s/da_s) subhalo potentials: per subhalo and summed
    (SubhaloLinePotential_dRadius.potential, potential.py:867-884) for the
    Plummer lines, and SubhaloLinePotentialCustom_dRadius_fromFunc
    (potential.py:1215-1262) for Plummer and Hernquist profiles, against the
    oracle's derivatives with respect to the scale radius (forward-mode
    autodiff of the profiles); one point gives a scalar sum."""
    from streamsculptor_gb300 import potential as P
    sh, _, _, _ = _pert_case(oracle)
    x = np.random.default_rng(5).normal(0, 10, (50, 3))
    t = 40.0
    args = (sh["m"], sh["a"], sh["x0"], sh["v"], sh["t0"], sh["t_window"])
    for kind, func in ((1, P.PlummerPotential), (2, P.HernquistPotential)):
        _, _, d_o, gd_o = oracle.subhalo_eval(oracle.HostModel([], subhalos=dict(sh, kind=kind)), x, t)
        assert (np.abs(d_o) > 0).sum() > 100  # most subhalos are inside their window at t
        pots = [P.SubhaloLinePotentialCustom_dRadius_fromFunc(func, *args, units=ss.usys)]
        if kind == 1:
            pots.append(P.SubhaloLinePotential_dRadius(*args, units=ss.usys))
        for s in pots:
            assert rel_err(np64(s.potential_per_SH(x, t)), d_o) < 1e-12
            assert rel_err(np64(s.gradient_per_SH(x, t)), gd_o) < 1e-12
            assert rel_err(np64(s.potential(x, t)), d_o.sum(axis=1)) < 1e-12
            assert rel_err(np64(s.gradient(x, t)), gd_o.sum(axis=1)) < 1e-12
            assert float(np64(s.potential(x[0], t))) == pytest.approx(float(d_o[0].sum()), rel=1e-12)
    with pytest.raises(NotImplementedError):
        P.SubhaloLinePotential_dRadius_Custom(lambda xyz, t: 0.0, *args[2:], units=ss.usys)


@pytest.mark.parametrize("precision,tol", [("f64", 1e-10), ("f32k", 1e-5)])
def test_streakline_matches_oracle(ss, oracle, precision, tol):
    """gen_streakline (streamhelpers.py:708-732): the progenitor forward from
    t0, one particle per Lagrange point at each of Nstrip release times
    (get_Streakline_ICs, streamhelpers.py:657-705), every pair integrated to
    t1 (the last pair, released at t1, is its initial state), against the
    oracle's restatement; 2 Myr between releases in 1 Myr steps."""
    from streamsculptor_gb300.streamhelpers import gen_streakline, get_Streakline_ICs
    pot = mw3_gpu(ss)
    orc = oracle.HostModel(oracle.mw3())
    t0, t1, n = -1000.0, 0.0, 501
    w0 = oracle.orbit(orc, PROG_WF, 0.0, -1.0, 1000, 1000)[0, -1]
    lead, trail, ts = gen_streakline(pot, w0, 2e4, t0, t1, n, dt=1.0, precision=precision)
    ws = oracle.orbit(orc, w0, t0, 1.0, 1000, 2)[0]
    ics = oracle.streakline_ics(orc, ws, ts, 2e4)
    Lc, vl, Lf, vt, _ = get_Streakline_ICs(pot, w0, 2e4, t0, t1, n, dt=1.0)
    got_ics = np.stack([np.concatenate([np64(Lc), np64(vl)], 1), np.concatenate([np64(Lf), np64(vt)], 1)], 1)
    assert phase_err(got_ics.reshape(-1, 6), ics.reshape(-1, 6)) < 1e-11
    ref, _, _ = oracle.stream(orc, t0, 1.0, 1000, ics.reshape(-1, 6), 2, 2)
    got = np.stack([np64(lead), np64(trail)], 1).reshape(-1, 6)
    err = phase_err(got, ref)
    print(f"streakline ({precision}) vs oracle: {err:.2e}")
    assert err <= tol
    # released at t1: the pair's initial states (hi + lo in the FP32 form)
    np.testing.assert_allclose(got[-2:], got_ics[-1], rtol=1e-15 if precision == "f64" else 1e-13)


@pytest.mark.parametrize("snap", [0, 25])
def test_f64_split_kernel_matches_plain_kernel(ss, snap):
    """Runs with fewer warps than the GPU has schedulers take the
    component-split FP64 kernel (one warp per potential component, the
    gradients exchanged through shared memory); larger runs the
    one-thread-per-particle kernel.  The same particles through both (the
    first 6400 of a run just above the threshold, then alone): the same
    arithmetic but the order of the component sum, so the final states agree
    to 1e-13 and the status and snapshot NaN pattern exactly."""
    from streamsculptor_gb300 import _core
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    n_big, n_small, ppr, n_steps = 4 * sms * 32 + 96, 6400, 100, 300
    rng = np.random.default_rng(11)
    ics = PROG_WF + rng.normal(0, 0.4, (n_big, 6)) * np.array([1, 1, 1, 0.01, 0.01, 0.01])
    ics_d = torch.as_tensor(ics, device="cuda")
    P = mw3_gpu(ss)._desc()
    outs = []
    for n in (n_big, n_small):
        cfg = _abi.ss_stream_cfg()
        cfg.t0, cfg.dt, cfg.n_steps, cfg.n_particles = 0.0, 1.0, n_steps, n
        cfg.particles_per_release, cfg.steps_per_release, cfg.snap_stride = ppr, 1, snap
        snaps = torch.empty(n_steps // snap, n, 6, dtype=torch.float32, device="cuda") if snap else None
        final, st = _core.stream(P, cfg, ics_d[:n].contiguous(), "f64", snaps=snaps)
        outs.append((final, st, snaps))
    (fb, sb, snb), (fs, ss_, sns) = outs
    assert torch.equal(sb[:n_small], ss_)
    assert bool((ss_ == 0).all())
    assert phase_err(np64(fs), np64(fb[:n_small])) <= 1e-13
    if snap:
        a, b = np64(snb[:, :n_small]), np64(sns)
        assert np.array_equal(np.isnan(a), np.isnan(b))
        ok = ~np.isnan(a)
        assert np.max(np.abs(a[ok] - b[ok]) / np.maximum(np.abs(a[ok]), 1e-3)) <= 1e-6


@pytest.mark.parametrize("precision", ["f32k", "f64"])
def test_gen_stream_batches_equal_gen_stream(ss, precision):
    """gen_stream_batches (the progenitor orbits, release and track tables of
    the next stream on a side stream while the current stream integrates)
    gives, stream by stream, exactly what gen_stream gives after an
    integrate_orbit back from the present: the same kernels on the same
    inputs, only in another order."""
    from streamsculptor_gb300 import potential as P
    from streamsculptor_gb300.streamhelpers import gen_stream, gen_stream_batches
    pot = mw3_gpu(ss)
    prog = P.PlummerPotential(m=2e4, r_s=0.01, units=ss.usys)
    n_rel, ppr, dt = 60, 8, 1.0
    ts = -float(n_rel) * dt + np.arange(n_rel + 1) * dt
    rng = np.random.default_rng(21)
    normals = [rng.standard_normal((n_rel + 1, ppr // 2, 4)) for _ in range(3)]
    w_now = [PROG_WF, PROG_WF + np.array([0.3, -0.2, 0.1, 0.002, -0.001, 0.001]), PROG_WF]
    got = list(gen_stream_batches(pot, ts, w_now, 2e4, normals, dt=dt, prog_pot=prog, n_particles_per_release=ppr,
                                  precision=precision, snapshot_every=10, prog_w0_at="end"))
    assert len(got) == 3
    for i in range(3):
        back = pot.integrate_orbit(w0=w_now[i], ts=np.array([ts[-1], ts[0]]), t0=float(ts[-1]), t1=float(ts[0]),
                                   dt=dt).ys[-1]
        want = gen_stream(pot, ts, back, 2e4, normals=normals[i], dt=dt, prog_pot=prog, n_particles_per_release=ppr,
                          precision=precision, snapshot_every=10)
        for a, b in zip(got[i], want):
            assert a.shape == b.shape
            assert torch.equal(torch.nan_to_num(a, nan=7.0), torch.nan_to_num(b, nan=7.0)), i


def test_gen_stream_batches_seeded_draws(ss):
    """Streams without given normals draw them from seed_num + their index,
    as gen_stream does from its seed_num."""
    from streamsculptor_gb300.streamhelpers import gen_stream, gen_stream_batches
    pot = mw3_gpu(ss)
    n_rel, dt = 40, 1.0
    ts = -float(n_rel) * dt + np.arange(n_rel + 1) * dt
    w_start = [PROG_WF, PROG_WF + np.array([0.2, 0.1, -0.1, 0.001, 0.0, -0.001])]
    got = list(gen_stream_batches(pot, ts, w_start, 2e4, seed_num=5, dt=dt, n_particles_per_release=4))
    for i in range(2):
        want = gen_stream(pot, ts, w_start[i], 2e4, seed_num=5 + i, dt=dt, n_particles_per_release=4,
                          precision="f32k")
        for a, b in zip(got[i], want):
            assert torch.equal(a, b), i
