"""Potentials of the reference's catalogue beyond the core kinds:
MN3ExponentialDiskPotential (potential.py:224-280), three Miyamoto-Nagai
disks from the published coefficient table; PowerLawCutoffPotential
(potential.py:357-388), a kernel kind with its own incomplete gamma
function; BovyMWPotential2014 (potential.py:420-446) built from them.  The
GPU evaluation and streams are checked against the oracle."""
import numpy as np
import pytest

from .conftest import rel_err

MN3_CASES = [dict(m=5e10, h_R=3.0, h_z=0.3, positive_density=True, sech2_z=True),
             dict(m=5e10, h_R=2.5, h_z=0.5, positive_density=False, sech2_z=False),
             dict(m=3e10, h_R=4.0, h_z=0.2, positive_density=True, sech2_z=False)]


@pytest.mark.parametrize("kw", MN3_CASES)
def test_mn3_components_match_oracle(kw, oracle):
    """Host-side mapping (no GPU): the three (m, a, b) triples."""
    from streamsculptor_gb300 import potential as P
    m, h_R, h_z = kw["m"], kw["h_R"], kw["h_z"]
    got = P.MN3ExponentialDiskPotential(units=P.usys, **kw)._flatten().comps
    want = oracle.mn3_components(m, h_R, h_z, kw["positive_density"], kw["sech2_z"])
    assert len(got) == 3
    for (k1, c1, p1), (k2, c2, p2) in zip(got, want):
        assert (k1, c1) == (k2, c2)
        np.testing.assert_allclose(p1, p2, rtol=1e-14, atol=0)


@pytest.mark.gpu
@pytest.mark.parametrize("kw", MN3_CASES)
def test_mn3_eval_and_stream_match_oracle(ss, oracle, kw):
    from streamsculptor_gb300 import potential as P
    comps = oracle.mn3_components(kw["m"], kw["h_R"], kw["h_z"], kw["positive_density"], kw["sech2_z"])
    disk = P.MN3ExponentialDiskPotential(units=ss.usys, **kw)
    x = np.random.default_rng(3).normal(0, 6, size=(400, 3))
    phi_o, g_o, H_o = oracle.potential_eval(oracle.HostModel(comps), x)
    assert rel_err(disk.potential(x, 0.0).cpu().numpy(), phi_o) < 1e-12
    assert rel_err(disk.gradient(x, 0.0).cpu().numpy(), g_o) < 1e-12
    assert rel_err(disk.jacobian_force(x, 0.0).cpu().numpy(), H_o) < 1e-11
    # a short FP64 stream in MN3 + NFW against the oracle
    pot = P.Potential_Combine([disk, P.NFWPotential(m=5.4e11, r_s=15.62, units=ss.usys)], units=ss.usys)
    orc = oracle.HostModel(comps + [(1, 0, (5.4e11, 15.62, 0.0))])
    wf = np.array([10.0, 0.0, 1.0, 0.0, 0.2, 0.02])
    n_rel = 150
    back = oracle.orbit(orc, wf, 0.0, -1.0, n_rel, n_rel)[0, -1]
    ts = -float(n_rel) + np.arange(n_rel + 1)
    normals = np.random.default_rng(5).standard_normal((n_rel + 1, 1, 4))
    ws = oracle.orbit(orc, back, ts[0], 1.0, n_rel, 1)[0]
    ics, _ = oracle.release(orc, ws, ts, 2e4, normals)
    ref, _, _ = oracle.stream(orc, ts[0], 1.0, n_rel, ics[:-1].reshape(-1, 6), 2, 1)
    lead, trail = pot.gen_stream_vmapped(ts=ts, prog_w0=back, Msat=2e4, normals=normals, precision="f64")
    got = np.stack([lead.cpu().numpy(), trail.cpu().numpy()], axis=1).reshape(-1, 6)
    err = np.max(np.maximum(np.linalg.norm(got[:, :3] - ref[:, :3], axis=1) / np.linalg.norm(ref[:, :3], axis=1),
                            np.linalg.norm(got[:, 3:] - ref[:, 3:], axis=1) / np.linalg.norm(ref[:, 3:], axis=1)))
    assert err <= 1e-10


PLC_CASES = [(4.5e9, 1.8, 1.9), (1e10, 1.0, 0.5), (3e9, 0.5, 3.0)]


@pytest.mark.gpu
@pytest.mark.parametrize("m,alpha,r_c", PLC_CASES)
def test_powerlaw_cutoff_eval_matches_oracle(ss, oracle, m, alpha, r_c):
    """PowerLawCutoffPotential (potential.py:357-388; the kernels' own
    regularised incomplete gamma function) against the oracle, from 1e-3 to
    200 kpc, on both sides of the series / continued-fraction switch."""
    from streamsculptor_gb300 import _abi, potential as P
    rng = np.random.default_rng(1)
    d = rng.normal(size=(600, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    x = d * np.exp(rng.uniform(np.log(1e-3), np.log(200.0), 600))[:, None]
    pot = P.PowerLawCutoffPotential(m=m, alpha=alpha, r_c=r_c, units=ss.usys)
    phi_o, g_o, H_o = oracle.potential_eval(oracle.HostModel([(_abi.SS_POWERLAW_CUTOFF, 0, (m, alpha, r_c))]), x)
    assert rel_err(pot.potential(x, 0.0).cpu().numpy(), phi_o) < 1e-12
    assert rel_err(pot.gradient(x, 0.0).cpu().numpy(), g_o) < 1e-12
    assert rel_err(pot.jacobian_force(x, 0.0).cpu().numpy(), H_o) < 1e-11


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol", [("f64", 1e-10), ("f32k", 1e-5)])
def test_bovy_mw_stream_matches_oracle(ss, oracle, precision, tol):
    """A stream in BovyMWPotential2014 (potential.py:420-446: Miyamoto-Nagai
    disk, power-law bulge with cutoff, NFW halo) against the oracle: FP64 to
    1e-10, the FP32-compensated form to 1e-5."""
    from streamsculptor_gb300 import _abi, potential as P
    pot = P.BovyMWPotential2014(units=ss.usys)
    orc = oracle.HostModel([(_abi.SS_MIYAMOTO_NAGAI, 0, (6.82e10, 3.0, 0.28)),
                            (_abi.SS_POWERLAW_CUTOFF, 0, (4.50e9, 1.80, 1.90)),
                            (_abi.SS_NFW, 0, (4.37e11, 16.0, 0.0))])
    wf = np.array([10.0, 0.0, 1.0, 0.0, 0.2, 0.02])
    n_rel = 150
    back = oracle.orbit(orc, wf, 0.0, -1.0, n_rel, n_rel)[0, -1]
    ts = -float(n_rel) + np.arange(n_rel + 1)
    normals = np.random.default_rng(5).standard_normal((n_rel + 1, 1, 4))
    ws = oracle.orbit(orc, back, ts[0], 1.0, n_rel, 1)[0]
    ics, _ = oracle.release(orc, ws, ts, 2e4, normals)
    ref, _, _ = oracle.stream(orc, ts[0], 1.0, n_rel, ics[:-1].reshape(-1, 6), 2, 1)
    lead, trail = pot.gen_stream_vmapped(ts=ts, prog_w0=back, Msat=2e4, normals=normals, precision=precision)
    got = np.stack([lead.cpu().numpy(), trail.cpu().numpy()], axis=1).reshape(-1, 6)
    err = np.max(np.maximum(np.linalg.norm(got[:, :3] - ref[:, :3], axis=1) / np.linalg.norm(ref[:, :3], axis=1),
                            np.linalg.norm(got[:, 3:] - ref[:, 3:], axis=1) / np.linalg.norm(ref[:, 3:], axis=1)))
    print(f"Bovy MW stream ({precision}) vs oracle: {err:.2e}")
    assert err <= tol


ZHAO_CASES = [(1e11, 10.0, 1.0, 4.0, 1.0), (5e11, 15.0, 0.5, 3.5, 0.5), (2e10, 3.0, 2.0, 5.0, 1.5),
              (1e11, 20.0, 1.0, 3.2, 0.0)]


def _zhao_midpoint(p, x, Gv):
    """The exact form the kernels evaluate, with scipy.special.betainc:
    dPhi/dr = G m I_z(a1, b1) / r^2 at r_m = r + dr / 2 along x / r, and its
    Jacobian."""
    from scipy import special
    m, rs, al, be, ga = p
    a1, b1 = al * (3 - ga), al * (be - 3)
    r = np.linalg.norm(x, axis=1)
    dr = 1e-5 * r + 1e-8
    rm = r + dr / 2
    xa = (rm / rs) ** (1 / al)
    z, zc = xa / (1 + xa), 1 / (1 + xa)
    I = special.betainc(a1, b1, z)
    gr = Gv * m * I / rm ** 2
    dI = z ** (a1 - 1) * zc ** (b1 - 1) / special.beta(a1, b1) * z * zc / (al * rm)
    dgr = Gv * m * (dI - 2 * I / rm) / rm ** 2 * (1 + 5e-6)
    g = gr / r
    h = (dgr - g) / r ** 2
    H = g[:, None, None] * np.eye(3)[None] + h[:, None, None] * x[:, :, None] * x[:, None, :]
    depth = Gv * m * special.beta(al * (2 - ga), al * (be - 2)) / (special.beta(a1, b1) * rs)
    return g[:, None] * x, H, depth, dr, r


@pytest.mark.gpu
@pytest.mark.parametrize("p", ZHAO_CASES)
def test_zhao_eval_matches_oracle(ss, oracle, p):
    """ZhaoPotential (potential.py:282-355) from 1e-2 to 300 kpc.  The
    potential against the oracle to 1e-12.  The kernels' gradient and
    Hessian (the exact derivative at the forward difference's midpoint)
    against the same form written with scipy.special.betainc to 1e-12 / 1e-11,
    and against the oracle's forward difference (gradient_func as written) and
    its autodiff Jacobian to 1e-9 / 1e-8 plus the difference's rounding
    bound, 16 eps |Phi(0)| / dr (times 1 / r + 1e-5 / dr for the Jacobian):
    where dPhi/dr is small against Phi / dr the reference's own gradient
    carries that noise."""
    from streamsculptor_gb300 import _abi, potential as P
    rng = np.random.default_rng(2)
    d = rng.normal(size=(600, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    x = d * np.exp(rng.uniform(np.log(1e-2), np.log(300.0), 600))[:, None]
    pot = P.ZhaoPotential(*p, units=ss.usys)
    phi_o, g_o, H_o = oracle.potential_eval(oracle.HostModel([(_abi.SS_ZHAO, 0, p)]), x)
    phi = pot.potential(x, 0.0).cpu().numpy()
    g = pot.gradient(x, 0.0).cpu().numpy()
    H = pot.jacobian_force(x, 0.0).cpu().numpy()
    g_m, H_m, depth, dr, r = _zhao_midpoint(p, x, pot._G)
    assert rel_err(phi, phi_o) < 1e-12
    assert np.max(np.linalg.norm(g - g_m, axis=1) / np.linalg.norm(g_m, axis=1)) < 1e-12
    assert np.max(np.linalg.norm((H - H_m).reshape(-1, 9), axis=1) / np.linalg.norm(H_m.reshape(-1, 9), axis=1)) < 1e-11
    noise = 16 * np.finfo(float).eps * depth / dr
    assert np.all(np.linalg.norm(g - g_o, axis=1) <= 1e-9 * np.linalg.norm(g_o, axis=1) + noise)
    assert np.all(np.linalg.norm((H - H_o).reshape(-1, 9), axis=1)
                  <= 1e-8 * np.linalg.norm(H_o.reshape(-1, 9), axis=1) + noise * (1 / r + 1e-5 / dr))


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol", [("f64", 2e-9), ("f32k", 1e-5)])
def test_zhao_stream_matches_oracle(ss, oracle, precision, tol):
    """A stream in a Miyamoto-Nagai disk plus a Zhao halo against the oracle.
    FP64 to 2e-9: the oracle, like the reference, takes the halo's force as a
    forward difference of its potential, whose rounding noise (~1e-10 of the
    force at these radii) moves 300-step orbits by 1e-11 to 1.2e-10 from the
    exact-derivative form the kernels evaluate.  The FP32-compensated form to
    1e-5."""
    from streamsculptor_gb300 import _abi, potential as P
    zp = (5e11, 15.0, 1.0, 3.5, 1.0)
    pot = P.Potential_Combine([P.MiyamotoNagaiDisk(m=6.8e10, a=3.0, b=0.28, units=ss.usys),
                               P.ZhaoPotential(*zp, units=ss.usys)], units=ss.usys)
    orc = oracle.HostModel([(_abi.SS_MIYAMOTO_NAGAI, 0, (6.8e10, 3.0, 0.28)), (_abi.SS_ZHAO, 0, zp)])
    wf = np.array([10.0, 0.0, 1.0, 0.0, 0.2, 0.02])
    n_rel = 150
    back = oracle.orbit(orc, wf, 0.0, -1.0, n_rel, n_rel)[0, -1]
    ts = -float(n_rel) + np.arange(n_rel + 1)
    normals = np.random.default_rng(6).standard_normal((n_rel + 1, 1, 4))
    ws = oracle.orbit(orc, back, ts[0], 1.0, n_rel, 1)[0]
    ics, _ = oracle.release(orc, ws, ts, 2e4, normals)
    ref, _, _ = oracle.stream(orc, ts[0], 1.0, n_rel, ics[:-1].reshape(-1, 6), 2, 1)
    lead, trail = pot.gen_stream_vmapped(ts=ts, prog_w0=back, Msat=2e4, normals=normals, precision=precision)
    got = np.stack([lead.cpu().numpy(), trail.cpu().numpy()], axis=1).reshape(-1, 6)
    err = np.max(np.maximum(np.linalg.norm(got[:, :3] - ref[:, :3], axis=1) / np.linalg.norm(ref[:, :3], axis=1),
                            np.linalg.norm(got[:, 3:] - ref[:, 3:], axis=1) / np.linalg.norm(ref[:, 3:], axis=1)))
    print(f"Zhao stream ({precision}) vs oracle: {err:.2e}")
    assert err <= tol


@pytest.mark.gpu
def test_zhao_rejects_gamma_at_least_two(ss):
    """gamma >= 2 (where the reference replaces alpha (2 - gamma) by
    sqrt(eps), a different potential) and beta <= 3 are refused with an
    argument error, before any kernel runs."""
    from streamsculptor_gb300 import potential as P
    for bad in [(1e11, 10.0, 1.0, 4.0, 2.0), (1e11, 10.0, 1.0, 3.0, 1.0), (1e11, 10.0, 0.0, 4.0, 1.0)]:
        with pytest.raises(Exception, match="Zhao"):
            P.ZhaoPotential(*bad, units=ss.usys).gradient(np.array([[1.0, 2.0, 3.0]]), 0.0)


@pytest.mark.gpu
@pytest.mark.parametrize("ncol", [6, 12])
def test_zhao_pert_response_matches_oracle(ss, oracle, ncol):
    """The first-order subhalo response (perturbative.py:24-135) on base
    tracks in a Miyamoto-Nagai disk plus a Zhao halo: the base track needs
    the Zhao Hessian along the track (the generic component loop of
    pert_base_kernel).  Against the oracle, whose Hessian is the autodiff of
    the reference's forward-difference gradient (its rounding noise is
    ~1e-10 of the force at these radii): FP64 base track and response to
    1e-10, FP32 response to 2e-4."""
    from streamsculptor_gb300 import _abi, _core, potential as P
    from .conftest import PROG_WF
    zp = (5e11, 15.0, 1.0, 3.5, 1.0)
    rng = np.random.default_rng(8)
    N, nsh, ppr, spr, n_steps, dt = 16, 5, 4, 10, 100, 1.0
    sh = dict(kind=1, m=10 ** rng.uniform(5, 8, nsh), a=rng.uniform(0.1, 1.0, nsh), x0=rng.normal(0, 10, (nsh, 3)),
              v=rng.normal(0, 0.12, (nsh, 3)), t0=rng.uniform(0, 100, nsh), t_window=60.0)
    orc = oracle.HostModel([(_abi.SS_MIYAMOTO_NAGAI, 0, (6.8e10, 3.0, 0.28)), (_abi.SS_ZHAO, 0, zp)], subhalos=sh)
    base = PROG_WF + rng.normal(0, 0.3, (N, 6)) * np.array([1, 1, 1, 0.01, 0.01, 0.01])
    pert = np.ascontiguousarray(rng.normal(0, 1e-3, (N, nsh, ncol)))
    bo, po = oracle.pert_response(orc, 0.0, dt, n_steps, base, pert, ppr, spr, ncol=ncol, save_stride=25)
    pot = P.Potential_Combine([P.MiyamotoNagaiDisk(m=6.8e10, a=3.0, b=0.28, units=ss.usys),
                               P.ZhaoPotential(*zp, units=ss.usys)], units=ss.usys)
    table = _core.SubhaloTable(1, *(_core.f64(sh[k]) for k in ("m", "a")), _core.f64(sh["x0"]), _core.f64(sh["v"]),
                               _core.f64(sh["t0"]), sh["t_window"])
    cfg = _abi.ss_pert_cfg()
    cfg.t0, cfg.dt, cfg.n_steps, cfg.n_particles = 0.0, dt, n_steps, N
    cfg.particles_per_release, cfg.steps_per_release, cfg.ncol, cfg.save_stride = ppr, spr, ncol, 25
    for prec, tol in ((64, 1e-10), (32, 2e-4)):
        b, p = _core.pert_response(pot._desc(), table, cfg, prec, _core.f64(base), _core.f64(pert))
        b = b.double().cpu().numpy()
        eb = np.max(np.linalg.norm(b - bo, axis=1) / np.linalg.norm(bo, axis=1))
        ep = rel_err(p.double().cpu().numpy(), po)
        print(f"Zhao response ({prec}, ncol {ncol}): base {eb:.2e}, response {ep:.2e}")
        assert eb < 1e-10
        assert ep < tol, prec
