"""GPU tests of the impact sampler (GenerateImpactParams.py) and of
gen_perturbed_stream (perturbedstream.py): the back-integrated stream patches
and stream-length history against the oracle's orbits, the impact geometry
restated on the host from the oracle's states, and the perturbed stream
against the oracle's stream in the sampled subhalos."""
import numpy as np
import pytest

from streamsculptor_gb300 import _abi

from .conftest import PROG_WF, mw3_gpu

pytestmark = pytest.mark.gpu


def np64(t):
    return np.asarray(t.detach().cpu().double().numpy() if hasattr(t, "detach") else t, dtype=np.float64)


def _phase_err(a, b):
    a, b = np.asarray(a).reshape(-1, 6), np.asarray(b).reshape(-1, 6)
    ex = np.linalg.norm(a[:, :3] - b[:, :3], axis=1) / np.linalg.norm(b[:, :3], axis=1)
    ev = np.linalg.norm(a[:, 3:] - b[:, 3:], axis=1) / np.linalg.norm(b[:, 3:], axis=1)
    return float(np.max(np.maximum(ex, ev)))


@pytest.fixture(scope="module")
def base_stream(ss, oracle):
    """A 400-release Fardal stream observed at t = 0, its phi1 and stripping times."""
    pot = mw3_gpu(ss)
    n = 400
    orc = oracle.HostModel(oracle.mw3())
    back = oracle.orbit(orc, PROG_WF, 0.0, -1.0, n, n)[0, -1]
    ts = -n + np.arange(n + 1) * 1.0
    lead, trail = pot.gen_stream_vmapped(ts=ts, prog_w0=back, Msat=2e4, seed_num=4)
    stream = np.concatenate([np64(lead), np64(trail)])
    phi1 = np.degrees(np.arctan2(stream[:, 1], stream[:, 0]))
    tstrip = np.concatenate([ts[:-1], ts[:-1]])
    return pot, orc, back, ts, stream, phi1, tstrip


def test_impact_generator_against_oracle(ss, oracle, base_stream):
    from streamsculptor_gb300.GenerateImpactParams import ImpactGenerator
    pot, orc, back, ts, stream, phi1, tstrip = base_stream
    gen = ImpactGenerator(pot=pot, tobs=0.0, stream=stream, stream_phi1=phi1, stripping_times=tstrip,
                          prog_today=PROG_WF, phi1window=2.0, NumImpacts=6, tImpactBounds=[-350.0, 0.0],
                          bImpact_bounds=[0.0, 0.5], phi1_bounds=[phi1.min() + 3, phi1.max() - 3],
                          phi1_exclude=[-1.0, 1.0], seednum=9)
    # stream length history: three orbits back 350 Myr saved at 2000 times
    lo = gen.length_osc
    t_age = 350.0
    h = t_age / 1999
    o = oracle.orbit(orc, np.stack([stream[0], stream[len(tstrip) // 2], PROG_WF]), 0.0, -h, 1999, 1)
    d = np.sqrt(((o[0, :, :3] - o[2, :, :3]) ** 2 + (o[1, :, :3] - o[2, :, :3]) ** 2).sum(1))[::-1]
    from streamsculptor_gb300.streamhelpers import compute_stream_length
    L = float(compute_stream_length(stream, phi1))
    assert np.max(np.abs(np64(lo["length_func"]) - L * d / d[-1])) <= 1e-9 * L
    assert np.allclose(np64(lo["ts"]), np.linspace(0, -t_age, 2000)[::-1])
    # sampled impact frame parameters
    p = gen.sample_impact_params()
    assert ((p["bImpact"] >= 0) & (p["bImpact"] <= 0.5)).all()
    assert ((p["tImpact"] >= -t_age) & (p["tImpact"] <= 0)).all()
    assert ((p["phi1_samples"] <= -1.0) | (p["phi1_samples"] >= 1.0)).all()
    # windowed means
    means, tm = gen.get_particle_mean(p["phi1_samples"])
    for i, c in enumerate(p["phi1_samples"]):
        sel = (phi1 > c - 2.0) & (phi1 < c + 2.0)
        assert np.allclose(np64(means[i]), stream[sel].mean(0), rtol=1e-12, atol=1e-14)
        assert np64(tm[i]) == pytest.approx(tstrip[sel].mean(), rel=1e-12)
    # Cartesian impacts: patch back to tImpact (oracle orbit with the same steps), then the frame
    xv, bhat = gen._get_subhalo_ImpactParamsCartesian(0.0, means, tm, p["tImpact"], p["bImpact"], p["perp_angle"],
                                                      np.arange(6))
    xv, bhat = np64(xv), np64(bhat)
    m = np64(means)
    n_steps = int(np.ceil(np.abs(p["tImpact"]).max() / 1.0 - 1e-9))
    zpar = np.random.default_rng(gen.keys[0]).normal(size=6) * gen.sigma
    zperp = gen.w_perpendicular_sample()
    for i in range(6):
        W0 = oracle.orbit(orc, m[i], 0.0, p["tImpact"][i] / n_steps, n_steps, n_steps)[0, -1]
        T = W0[3:] / np.linalg.norm(W0[3:])
        B = np.cross(W0[:3], W0[3:])
        B /= np.linalg.norm(B)
        N = np.cross(B, T)
        a = p["perp_angle"][i]
        bh = N * np.cos(a) + B * np.sin(a)
        X = W0[:3] + p["bImpact"][i] * bh
        V = zpar[i] * T + zperp[i] * (-N * np.sin(a) + B * np.cos(a))
        assert np.allclose(bhat[i], bh, rtol=0, atol=1e-10)
        assert np.allclose(xv[i, :3], X, rtol=1e-10, atol=1e-10)
        assert np.allclose(xv[i, 3:], V, rtol=1e-9, atol=1e-12)
        assert abs(np.dot(bh, T)) < 1e-12 and abs(np.linalg.norm(bh) - 1) < 1e-12
    full = gen.get_subhalo_ImpactParams()
    assert full["CartesianImpactParams"].shape == (6, 6)


def test_gen_perturbed_stream_against_oracle(ss, oracle, base_stream):
    """The stream in the sampled Hernquist subhalos equals the oracle's Chen+25
    stream in the same subhalos (the progenitor unperturbed, its Plummer
    potential moving on its orbit)."""
    from streamsculptor_gb300 import perturbative, potential as P
    from streamsculptor_gb300.main import release_normals
    from streamsculptor_gb300.perturbedstream import gen_perturbed_stream
    from streamsculptor_gb300.streamhelpers import CHEN25_MEAN, chen25_factor
    from streamsculptor_gb300.subhalostatistics import RateCalculator, split_key
    pot, orc, back, ts, stream, phi1, tstrip = base_stream
    prog = P.PlummerPotential(m=2e4, r_s=0.01, units=ss.usys)
    bsm = perturbative.BaseStreamModelChen25(pot, ts, back, 2e4, 7, prog_pot=prog)
    orbit = pot.integrate_orbit(w0=PROG_WF, ts=np.linspace(0, -400.0, 401), t0=0.0, t1=-400.0)
    rate = RateCalculator(orbit, t_age=400.0, b_max_fac=5.0, l_obs=10.0)
    key = 21
    out = gen_perturbed_stream(bsm, rate, stream, phi1, 6.0, 8.0, key, [phi1.min() + 3, phi1.max() - 3],
                               [-350.0, 0.0], normalization=5.0, Max_Num_Impacts=8, phi1window=2.0)
    imp = out["impactors"]
    mass = np64(imp["mass"])
    assert mass.shape == (8,) and (mass > 0).any()
    n_rel = len(ts) - 1
    assert out["leading"].shape == (n_rel, 6) and out["trailing"].shape == (n_rel, 6)
    sh = dict(kind=2, m=mass, a=np64(imp["r_s"]), x0=np64(imp["cartImpact"])[:, :3], v=np64(imp["cartImpact"])[:, 3:],
              t0=np64(imp["tImpact"]), t_window=150.0)
    _, k2 = split_key(key, 2)
    normals = release_normals(k2, len(ts), 1, 6)
    ws = oracle.orbit(orc, back, ts[0], 1.0, n_rel, 1)[0]
    ics, _ = oracle.release(orc, ws, ts, 2e4, normals, model_kind=1, chen=(CHEN25_MEAN, chen25_factor()))
    integ = oracle.HostModel(oracle.mw3() + [(_abi.SS_PLUMMER, 1, (2e4, 0.01))], track=(ts[0], 1.0, ws[:, :3]),
                             subhalos=sh)
    final, _, st = oracle.stream(integ, ts[0], 1.0, n_rel, ics[:-1].reshape(-1, 6), 2, 1)
    final = final.reshape(n_rel, 2, 6)
    assert (st == 0).all()
    assert _phase_err(np64(out["leading"]), final[:, 0]) <= 1e-10
    assert _phase_err(np64(out["trailing"]), final[:, 1]) <= 1e-10
