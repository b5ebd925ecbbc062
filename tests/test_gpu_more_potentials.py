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
