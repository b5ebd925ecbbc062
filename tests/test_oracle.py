"""CPU tests of the oracle: pins against the reference notebook's printed
values, autodiff vs finite differences, integrator order and invariants.
No GPU needed."""
import numpy as np
import pytest

from streamsculptor_gb300 import _abi

from .conftest import G, PROG_WF, rel_err


def test_nfw_acceleration_golden(oracle):
    # hamiltonian_field(NFWPotential(m=1e12, r_s=20, units=usys)).term(0, [1,2,3,.2,.3,.4])
    # printed as [0.2, 0.3, 0.4, -0.0011937, -0.00238739, -0.00358109]
    # (examples/tests.ipynb:1671, cell 58)
    m = oracle.HostModel([(_abi.SS_NFW, 0, (1e12, 20.0, 0.0))])
    _, g, _ = oracle.potential_eval(m, [1.0, 2.0, 3.0])
    printed = np.array([-0.0011937, -0.00238739, -0.00358109])
    assert np.all(np.abs(-g[0] - printed) <= 5e-9)


def test_softened_nfw_perturbation_term_golden(oracle):
    # MassRadiusPerturbation_OTF(pert_Gen).term(0, [ones(6), ones((10,12))]) with the
    # NFW(1e12, 20) base (examples/tests.ipynb:3672-3702, cell 151) printed
    # a0 = -0.00290453 and d(pdot)/d(eps) = 3.09774548e-04 per component.  That
    # output predates the removal of the NFW softening (r^2 + 0.001,
    # potential.py:83 comment); the oracle reproduces it with soft = 0.001.
    # The printed rows differ from each other by <= 3e-12 (subhalo terms of
    # that run, not reproducible); the tidal part alone is checked.
    m = oracle.HostModel([(_abi.SS_NFW, 0, (1e12, 20.0, 0.001))],
                         subhalos=dict(m=[0.0] * 10, a=[0.2] * 10, x0=np.zeros((10, 3)), v=np.zeros((10, 3)),
                                       t0=np.zeros(10), t_window=250.0))
    d0, d1 = oracle.pert_term(m, 0.0, np.ones(6), np.ones((10, 12)))
    assert np.all(np.abs(d0[3:] - (-0.00290453)) <= 5e-9)
    assert np.all(np.abs(d1[:, 3:6] - 3.09774548e-04) <= 5e-12)
    assert np.all(np.abs(d1[:, 9:12] - 3.09774549e-04) <= 5e-12)
    assert np.all(d1[:, 0:3] == 1.0) and np.all(d1[:, 6:9] == 1.0)


# GalaMilkyWayPotential (potential.py:390-418): disk, bulge, nucleus, halo
GALA_MW = [(_abi.SS_MIYAMOTO_NAGAI, 0, (6.8e10, 3.0, 0.28)), (_abi.SS_HERNQUIST, 0, (5e9, 1.0, 0.0)),
           (_abi.SS_HERNQUIST, 0, (1.71e9, 0.07, 0.0)), (_abi.SS_NFW, 0, (5.4e11, 15.62, 0.0))]
# examples/StreamSubhaloExample.ipynb cell 1: integrate_orbit of w_today back
# 3500 Myr in GalaMilkyWayPotential (adaptive Dopri8, rtol = atol = 1e-7,
# main.py:126) printed "Initial condition = [...]" to 8 digits
GALA_W_TODAY = np.array([20.0, 0.0, 20.0, 0.0, 0.15, 0.0])
GALA_IC_PRINTED = np.array([-7.23164146, -7.96692572, -10.81840286, 0.19182623, -0.20351324, -0.01770436])
# cell 7 printed the impact location; cell 9 evaluated a Plummer and a
# Hernquist subhalo (m = 1e7, r_s = 0.2) on the line through it, with the
# velocity offset by (0.02, 0, 0.02), at x = (1, 2, 3), t = -850 Myr
SH_W_IMPACT = np.array([-18.84511332, 4.23873108, -17.32878089, -0.04416233, -0.15074649, -0.07956093])
SH_PHI_PRINTED = {1: -1.053815931966235e-06, 2: -1.048913077256255e-06}  # Plummer, Hernquist


def sh_example_table(kind):
    """The subhalo line of StreamSubhaloExample.ipynb cells 7-9."""
    w = SH_W_IMPACT + np.array([0.0, 0.0, 0.0, 0.02, 0.0, 0.02])
    return dict(kind=kind, m=np.array([1e7]), a=np.array([0.2]), x0=w[None, :3], v=w[None, 3:],
                t0=np.array([-1000.0]), t_window=250.0)


def test_gala_orbit_golden(oracle):
    """The oracle's converged fixed-step orbit (dt = 0.5 Myr, 7000 steps)
    against the notebook's printed state.  The residual (8e-6) is the
    reference's own adaptive tolerance over 3.5 Gyr; a 1e-4 change in the
    halo mass or scale radius moves the result by ~4e-3 and a 1e-5 change in
    G by ~5e-4, so the pin fixes the potential's parameters, summation and
    units."""
    m = oracle.HostModel(GALA_MW)
    w = oracle.orbit(m, GALA_W_TODAY, 0.0, -0.5, 7000, 7000)[0, -1]
    ref = GALA_IC_PRINTED
    assert np.linalg.norm(w[:3] - ref[:3]) / np.linalg.norm(ref[:3]) <= 2e-5
    assert np.linalg.norm(w[3:] - ref[3:]) / np.linalg.norm(ref[3:]) <= 2e-5


@pytest.mark.parametrize("kind", [1, 2])
def test_subhalo_line_potential_golden(oracle, kind):
    """Plummer and Hernquist subhalo lines (potential.py:802-850, 908-956)
    against the notebook's printed values; the printed 8-digit impact
    location limits the agreement to ~1e-7.  Outside the window the
    potential is zero."""
    m = oracle.HostModel([], subhalos=sh_example_table(kind))
    phi = oracle.potential_eval(m, np.array([[1.0, 2.0, 3.0]]), -850.0)[0][0]
    assert abs(phi / SH_PHI_PRINTED[kind] - 1.0) <= 1e-7
    assert oracle.potential_eval(m, np.array([[1.0, 2.0, 3.0]]), -1300.0)[0][0] == 0.0


# examples/tests.ipynb cell 17: NFW(1e12, 20) orbit from NFW_W0_A, dense
# output at t = 30 Myr, printed to 8 decimals
NFW_W0_A = np.array([20.0, 15.0, 20.0, 0.08, 0.1, -0.05])
NFW_T30_PRINTED = np.array([21.9793661, 17.67654451, 18.10530132, 0.051923, 0.07815599, -0.07552167])
# cell 61: integrate_field(hamiltonian_field(NFW(1e12, 20))) from NFW_W0_B
# saved at linspace(0, 3000, 1000); rows 1, 2 and the last three printed
NFW_W0_B = np.array([20.0, 0.0, 20.0, 0.0, 0.2, 0.0])
NFW_FIELD_ROWS_PRINTED = {
    1: [1.99947007e+01, 6.00547553e-01, 1.99947007e+01, -3.52920125e-03, 1.99947006e-01, -3.52920125e-03],
    2: [1.99788050e+01, 1.20077683e+00, 1.99788050e+01, -7.05704492e-03, 1.99788029e-01, -7.05704492e-03],
    997: [1.54653741e+01, -1.50646962e+01, 1.54653741e+01, 9.87262702e-02, 1.62473824e-01, 9.87262702e-02],
    998: [1.57572297e+01, -1.45723635e+01, 1.57572297e+01, 9.56423786e-02, 1.65401168e-01, 9.56423786e-02],
    999: [1.60397604e+01, -1.40714069e+01, 1.60397604e+01, 9.25163046e-02, 1.68217294e-01, 9.25163046e-02],
}


def check_nfw_field_rows(ys):
    """ys [1000, 6] at the notebook's save times against its printed rows:
    the first rows to their 9 printed digits, the rows after 3 Gyr to 5e-6
    (the reference's adaptive tolerance; measured 1.6e-6)."""
    for k, row in NFW_FIELD_ROWS_PRINTED.items():
        r = np.array(row)
        tol = 1e-8 if k < 10 else 5e-6
        assert np.max(np.abs(ys[k] - r) / np.abs(r)) <= tol, k


def test_nfw_orbit_and_field_golden(oracle):
    """The two NFW orbits of examples/tests.ipynb (cells 17 and 61) on the
    oracle's fixed-step Dopri5."""
    m = oracle.HostModel([(_abi.SS_NFW, 0, (1e12, 20.0, 0.0))])
    w = oracle.orbit(m, NFW_W0_A, 0.0, 0.5, 60, 60)[0, -1]
    assert np.all(np.abs(w - NFW_T30_PRINTED) <= 1e-8)
    h = 3000.0 / 999 / 6
    check_nfw_field_rows(oracle.orbit(m, NFW_W0_B, 0.0, h, 999 * 6, 6)[0])


def zhao_density(r, m=1e11, r_s=10.0, alpha=1.0, beta=2.5, gamma=1.0):
    """examples/potential_from_1D_Density.ipynb cells 2-4."""
    uu = r / r_s
    rho0 = m / (4 * np.pi * r_s ** 3)
    return rho0 / uu ** gamma / (1.0 + uu ** (1.0 / alpha)) ** ((beta - gamma) * alpha)


def test_potential_from_density_golden(oracle):
    """get_potential_from_density of the Zhao density (potential.py:504-552),
    evaluated by the oracle from the spline the host builds, against the
    notebook's printed potential (-0.08283585) and gradient at (1, 2, 3).
    The spline's own error is ~2e-8 absolute and the reference's knots come
    from quadgk at its default tolerance, so the potential is pinned to
    1e-6 and the gradient to its printed precision (~1e-5)."""
    from streamsculptor_gb300 import _core, potential as P
    pot = P.get_potential_from_density(zhao_density, units=_core.usys)
    sp = pot._spline
    m = oracle.HostModel([(_abi.SS_SH_EXPANSION, 0, (1.0,))],
                         expansion=(0, sp.log_r0, sp.dlog_r, sp.coef.cpu().numpy()))
    phi, g, _ = oracle.potential_eval(m, np.array([[1.0, 2.0, 3.0]]), 0.0)
    assert abs(phi[0] / -0.08283585 - 1.0) <= 1e-6
    assert np.all(np.abs(g[0] - np.array([0.0004346, 0.0008692, 0.0013038])) <= 5e-9)


def _all_kinds():
    return [
        (_abi.SS_NFW, 0, (5.4e11, 15.62, 0.0)),
        (_abi.SS_TRIAXIAL_NFW, 0, (3e11, 12.0, 1.0, 0.9, 0.8)),
        (_abi.SS_MIYAMOTO_NAGAI, 0, (6.8e10, 3.0, 0.28)),
        (_abi.SS_HERNQUIST, 0, (5e9, 1.0, 0.01)),
        (_abi.SS_PLUMMER, 0, (2e9, 0.5)),
        (_abi.SS_ISOCHRONE, 0, (4e9, 1.5)),
        (_abi.SS_POWERLAW_CUTOFF, 0, (4.5e9, 1.8, 1.9)),
    ]


@pytest.mark.parametrize("k", range(7))
def test_autodiff_matches_finite_differences(oracle, k):
    m = oracle.HostModel([_all_kinds()[k]])
    rng = np.random.default_rng(k)
    for x in rng.normal(0, 6, size=(5, 3)):
        phi, g, H = oracle.potential_eval(m, x)
        eps = 1e-5 * max(1.0, np.linalg.norm(x))
        gfd = np.array([(oracle.potential_eval(m, x + eps * e)[0][0] - oracle.potential_eval(m, x - eps * e)[0][0])
                        / (2 * eps) for e in np.eye(3)])
        Hfd = np.stack([(oracle.potential_eval(m, x + eps * e)[1][0] - oracle.potential_eval(m, x - eps * e)[1][0])
                        / (2 * eps) for e in np.eye(3)], axis=1)
        assert rel_err(g[0], gfd) < 1e-7
        assert rel_err(H[0], Hfd) < 1e-6
        assert np.allclose(H[0], H[0].T, rtol=1e-13, atol=0)


def test_spherical_potential_closed_forms(oracle):
    # closed-form radial forces at r = 10 kpc
    r = 10.0
    x = np.array([r, 0, 0])
    for kind, p, dphidr in [
        (_abi.SS_PLUMMER, (1e10, 2.0), lambda: G * 1e10 * r / (r * r + 4.0) ** 1.5),
        (_abi.SS_HERNQUIST, (1e10, 2.0, 0.0), lambda: G * 1e10 / (r + 2.0) ** 2),
        (_abi.SS_NFW, (1e12, 20.0, 0.0), lambda: G * 1e12 * (np.log1p(r / 20) / r ** 2 - 1 / (r * (r + 20)))),
        (_abi.SS_ISOCHRONE, (1e10, 2.0), lambda: G * 1e10 * r / (np.sqrt(r * r + 4) * (2 + np.sqrt(r * r + 4)) ** 2)),
    ]:
        _, g, _ = oracle.potential_eval(oracle.HostModel([(kind, 0, p)]), x)
        assert abs(g[0, 0] - dphidr()) <= 1e-13 * abs(dphidr())


@pytest.mark.parametrize("m,alpha,r_c", [(4.5e9, 1.8, 1.9), (1e10, 1.0, 0.5), (3e9, 0.5, 3.0)])
def test_powerlaw_cutoff_matches_scipy(oracle, m, alpha, r_c):
    """The oracle's PowerLawCutoffPotential (its own regularised incomplete
    gamma function, forces by autodiff of the potential) against the
    reference's potential formula and gradient_func (potential.py:365-388)
    evaluated with scipy.special.gammainc and gamma, from 1e-3 to 200 kpc."""
    from scipy import special
    rng = np.random.default_rng(0)
    d = rng.normal(size=(300, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    r = np.exp(rng.uniform(np.log(1e-3), np.log(200.0), 300))
    x = d * r[:, None]
    phi, g, _ = oracle.potential_eval(oracle.HostModel([(_abi.SS_POWERLAW_CUTOFF, 0, (m, alpha, r_c))]), x)
    t0 = alpha / 2
    t1, t2, xx = -t0, 1.5 - t0, r ** 2 / r_c ** 2
    t6 = G * m * special.gammainc(t2, xx) * special.gamma(t2) / (r * special.gamma(t1 + 2.5))
    phi_ref = t0 * t6 - 1.5 * t6 + G * m * special.gammainc(t1 + 1, xx) * special.gamma(t1 + 1) / (r_c * special.gamma(t2))
    g_ref = (G * m / r ** 2 * special.gammainc(t2, xx))[:, None] * x / r[:, None]
    assert np.max(np.abs(phi - phi_ref) / np.abs(phi_ref)) < 1e-13
    assert np.max(np.linalg.norm(g - g_ref, axis=1) / np.linalg.norm(g_ref, axis=1)) < 1e-13


ZHAO_CASES = [(1e11, 10.0, 1.0, 4.0, 1.0), (5e11, 15.0, 0.5, 3.5, 0.5), (2e10, 3.0, 2.0, 5.0, 1.5),
              (1e11, 20.0, 1.0, 3.2, 0.0)]


def zhao_reference(p, r, Gv):
    """ZhaoPotential (potential.py:282-355) as the reference writes it, with
    scipy.special's beta, betaln and betainc: the potential at r and
    gradient_func's forward difference dPhi/dr; also the potential's depth
    |Phi(0)| = G m B(p0, c0 - p0) / (B(a1, b1) r_s), which bounds the
    rounding noise of that difference."""
    from scipy import special
    m, rs, al, be, ga = p

    def phi(r):
        rho0 = m / (4 * np.pi * al * special.beta(al * (3 - ga), al * (be - 3)))
        xa = (r / rs) ** (1 / al)
        z = xa / (1 + xa)
        p0, q0, c0 = al * (2 - ga), al * (be - 3), al * (be - ga)
        term_l = special.beta(c0 - q0, q0) * special.betainc(c0 - q0, q0, z)
        p0s = p0 if p0 > 0 else np.sqrt(np.finfo(float).eps)
        term_r = np.exp(special.betaln(p0s, c0 - p0) + np.log1p(-special.betainc(p0s, c0 - p0, z)))
        return -4 * np.pi * Gv * rho0 * al * (term_l / r + term_r / rs)

    dr = 1e-5 * r + 1e-8
    depth = Gv * m * special.beta(al * (2 - ga), al * (be - 2)) / (special.beta(al * (3 - ga), al * (be - 3)) * rs)
    return phi(r), (phi(r + dr) - phi(r)) / dr, depth, dr


@pytest.mark.parametrize("p", ZHAO_CASES)
def test_zhao_matches_scipy(oracle, p):
    """The oracle's ZhaoPotential (its own incomplete beta function from the
    hypergeometric series; the gradient as gradient_func's forward difference,
    potential.py:347-354) against the reference's formulas evaluated with
    scipy.special, from 1e-2 to 300 kpc.  The difference cancels most of the
    potential's digits where dPhi/dr is small against Phi / dr, so the
    gradients are compared to 1e-9 plus that rounding bound,
    16 eps |Phi(0)| / dr."""
    rng = np.random.default_rng(0)
    d = rng.normal(size=(300, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    r = np.exp(rng.uniform(np.log(1e-2), np.log(300.0), 300))
    x = d * r[:, None]
    phi, g, _ = oracle.potential_eval(oracle.HostModel([(_abi.SS_ZHAO, 0, p)]), x)
    phi_ref, dphi, depth, dr = zhao_reference(p, r, G)
    assert np.max(np.abs(phi - phi_ref) / np.abs(phi_ref)) < 1e-13
    g_ref = dphi[:, None] * x / r[:, None]
    bound = 1e-9 * np.linalg.norm(g_ref, axis=1) + 16 * np.finfo(float).eps * depth / dr
    assert np.all(np.linalg.norm(g - g_ref, axis=1) <= bound)


@pytest.mark.parametrize("p", ZHAO_CASES[:3])
def test_zhao_oracle_hessian_is_the_jacobian_of_its_gradient(oracle, p):
    """The oracle's Zhao Hessian (forward-mode autodiff through the forward
    difference of gradient_func) against central differences of its own
    gradient, at 1-100 kpc where the difference's rounding noise is small:
    within 1e-5 of the differences, and symmetric to 1e-9 (differentiating
    the forward difference cancels about five digits, so the two orders of
    a mixed derivative round apart by ~1e-11)."""
    m = oracle.HostModel([(_abi.SS_ZHAO, 0, p)])
    rng = np.random.default_rng(3)
    for x in rng.normal(0, 1, size=(6, 3)):
        x = x / np.linalg.norm(x) * np.exp(rng.uniform(0.0, np.log(100.0)))
        _, g, H = oracle.potential_eval(m, x)
        eps = 1e-3 * np.linalg.norm(x)  # the gradient's own rounding noise / eps stays below 1e-6
        Hfd = np.stack([(oracle.potential_eval(m, x + eps * e)[1][0] - oracle.potential_eval(m, x - eps * e)[1][0])
                        / (2 * eps) for e in np.eye(3)], axis=1)
        assert rel_err(H[0], Hfd) < 1e-5
        assert np.abs(H[0] - H[0].T).max() <= 1e-9 * np.abs(H[0]).max()


def test_zhao_closed_form_hernquist(oracle):
    """alpha = 1, beta = 4, gamma = 1 is the Hernquist sphere: the oracle's
    Zhao potential equals -G m / (r + r_s) to round-off, and its forward
    difference the Hernquist force to the difference's truncation (5e-6)."""
    r = np.array([0.5, 3.0, 10.0, 40.0])
    x = np.stack([r, 0 * r, 0 * r], axis=1)
    phi, g, _ = oracle.potential_eval(oracle.HostModel([(_abi.SS_ZHAO, 0, (1e11, 10.0, 1.0, 4.0, 1.0))]), x)
    assert np.max(np.abs(phi / (-G * 1e11 / (r + 10.0)) - 1)) < 1e-13
    assert np.max(np.abs(g[:, 0] / (G * 1e11 / (r + 10.0) ** 2) - 1)) < 1e-5


def test_dopri5_fifth_order(oracle):
    # smooth (Plummer) potential so the asymptotic regime is reached
    m = oracle.HostModel([(_abi.SS_PLUMMER, 0, (1e11, 5.0))])
    w0 = np.array([10.0, 0, 0, 0, 0.2, 0.05])
    T = 1600.0
    ref = oracle.orbit(m, w0, 0.0, T / 25600, 25600, 25600)[0, -1]
    errs = []
    for dt in (2.0, 1.0, 0.5):
        n = int(T / dt)
        errs.append(np.max(np.abs(oracle.orbit(m, w0, 0.0, dt, n, n)[0, -1] - ref)))
    ratios = [errs[0] / errs[1], errs[1] / errs[2]]
    # global error ~ dt^5: halving dt divides it by ~32
    assert all(20 < q < 40 for q in ratios), ratios


def test_orbit_invariants_and_reversibility(oracle):
    m = oracle.HostModel(oracle.mw3())
    out = oracle.orbit(m, PROG_WF, 0.0, 1.0, 3000, 1)[0]
    E = 0.5 * (out[:, 3:] ** 2).sum(1) + oracle.potential_eval(m, out[:, :3])[0]
    Lz = out[:, 0] * out[:, 4] - out[:, 1] * out[:, 3]
    assert np.max(np.abs(E - E[0])) / abs(E[0]) < 5e-9
    assert np.max(np.abs(Lz - Lz[0])) / abs(Lz[0]) < 1e-10
    back = oracle.orbit(m, out[-1], 3000.0, -1.0, 3000, 3000)[0, -1]
    assert rel_err(back, PROG_WF) < 1e-6  # Dopri5 is not time-symmetric: truncation error only


def test_release_symmetry_and_offsets(oracle):
    m = oracle.HostModel(oracle.mw3())
    w = oracle.orbit(m, PROG_WF, 0.0, 1.0, 50, 10)[0]
    z = np.zeros((w.shape[0], 1, 4))
    ics, _ = oracle.release(m, w, np.arange(w.shape[0]) * 10.0, 2e4, z)
    # zero draws: kr = 2, kvphi = 0.6, kz = kvz = 0 -> lead/trail mirror about the progenitor
    assert np.allclose(ics[:, 0, 0] + ics[:, 0, 1], 2 * w, rtol=1e-14, atol=1e-14)
    r = np.linalg.norm(w[:, :3], axis=1)
    dr = np.linalg.norm(ics[:, 0, 1, :3] - w[:, :3], axis=1)
    # trailing offset is kr * r_t radially outwards
    assert np.all(np.linalg.norm(ics[:, 0, 1, :3], axis=1) > r)
    assert np.all((dr > 0.005) & (dr < 1.0))


def test_release_jacobian_matches_fd(oracle):
    m = oracle.HostModel(oracle.mw3())
    w = oracle.orbit(m, PROG_WF, 0.0, 1.0, 20, 20)[0, -1:]
    z = np.random.default_rng(3).standard_normal((1, 2, 4))
    ics, J = oracle.release(m, w, [20.0], 2e4, z, jac=True)
    for j in range(6):
        h = 1e-6 * max(1.0, abs(w[0, j]))
        wp, wm = w.copy(), w.copy()
        wp[0, j] += h
        wm[0, j] -= h
        fd = (oracle.release(m, wp, [20.0], 2e4, z)[0] - oracle.release(m, wm, [20.0], 2e4, z)[0]) / (2 * h)
        assert rel_err(J[..., j], fd) < 1e-6


def test_stream_snapshots_and_nan_flags(oracle):
    m = oracle.HostModel(oracle.mw3())
    ts = np.arange(11) * 2.0
    w = oracle.orbit(m, PROG_WF, 0.0, 1.0, 20, 2)[0]
    ics, _ = oracle.release(m, w, ts, 2e4, np.random.default_rng(0).standard_normal((11, 1, 4)))
    final, snaps, st = oracle.stream(m, 0.0, 1.0, 20, ics[:10].reshape(-1, 6), 2, 2, snap_stride=5)
    assert snaps.shape == (4, 20, 6)
    # particle of release r starts at step 2r: snapshot k (step 5(k+1)) is NaN iff 5(k+1) < 2r
    for k in range(4):
        for p in range(20):
            assert np.isnan(snaps[k, p]).all() == (5 * (k + 1) < 2 * (p // 2))
    assert np.allclose(snaps[-1], final.astype(np.float32))
    assert (st == 0).all()
    # release exactly at a snapshot step keeps its initial state there (step 10, release 5)
    assert np.allclose(snaps[1, 10], ics[5, 0, 0].astype(np.float32))


def test_binned_sums_reference_semantics(oracle):
    rng = np.random.default_rng(1)
    vals = rng.normal(size=(500, 3))
    vals[::17, 1] = np.nan
    key = rng.uniform(-1, 2, 500)
    edges = np.linspace(key.min(), key.max(), 12)
    sums, counts = oracle.binned_sums(vals, key, edges)
    d = np.digitize(key, edges)
    for b in range(11):
        sel = vals[d == b]
        assert np.allclose(counts[b], np.sum(~np.isnan(sel), axis=0))
        assert np.allclose(sums[b], np.nansum(sel, axis=0))
    assert counts[0].sum() == 0  # bin 0 is always empty (reference quirk)


def test_track_slopes_restatement(oracle):
    t = np.arange(6) * 0.5
    knots = np.stack([t ** 2, np.sin(t), 3 * t], axis=1)
    s = oracle.track_slopes(knots, 0.5)
    assert np.allclose(s[1:-1], (knots[2:] - knots[:-2]) / 1.0)
    assert np.allclose(s[0], (knots[1] - knots[0]) / 0.5) and np.allclose(s[-1], (knots[-1] - knots[-2]) / 0.5)


def test_second_order_term_matches_finite_differences(oracle):
    """The 18-column term (MassRadiusPerturbation_OTF_SecondOrder.term,
    fields.py:284-320): columns 0-11 equal the first-order term, dx2/dt = v2
    and dv2/dt = T x2 + (d2a/dx2 : x1 x1) - Hess(Phi_s) x1, the third
    derivatives and the subhalo Hessian checked against central differences
    of the oracle's analytic Hessian and subhalo gradient."""
    rng = np.random.default_rng(8)
    nsh = 5
    sh = dict(kind=1, m=10 ** rng.uniform(6, 8, nsh), a=rng.uniform(0.3, 1.0, nsh),
              x0=PROG_WF[:3] + rng.normal(0, 2.0, (nsh, 3)), v=rng.normal(0, 0.12, (nsh, 3)),
              t0=rng.uniform(0, 20, nsh), t_window=60.0)
    m = oracle.HostModel(oracle.mw3(), subhalos=sh)
    base = PROG_WF.copy()
    u = rng.normal(0, 1.0, (nsh, 18))
    t = 12.0
    d0, d1 = oracle.pert_term(m, t, base, u, ncol=18)
    e0, e1 = oracle.pert_term(m, t, base, u[:, :12], ncol=12)
    assert np.array_equal(d0, e0) and np.array_equal(d1[:, :12], e1)
    assert np.array_equal(d1[:, 12:15], u[:, 15:18])
    mb = oracle.HostModel(oracle.mw3())  # the base potential alone
    _, _, T0 = oracle.potential_eval(mb, base[None, :3], t)
    T0 = -T0[0]
    h = 1e-3
    for s in range(nsh):
        x1 = u[s, 0:3]
        _, _, Hp = oracle.potential_eval(mb, (base[:3] + h * x1)[None], t)
        _, _, Hm = oracle.potential_eval(mb, (base[:3] - h * x1)[None], t)
        third = -(Hp[0] - Hm[0]) / (2 * h) @ x1
        _, gp, _, _ = oracle.subhalo_eval(m, (base[:3] + h * x1)[None], t)
        _, gm, _, _ = oracle.subhalo_eval(m, (base[:3] - h * x1)[None], t)
        hs = (gp[0, s] - gm[0, s]) / (2 * h)
        want = T0 @ u[s, 12:15] + third - hs
        assert np.max(np.abs(d1[s, 15:18] - want)) <= 1e-6 * np.max(np.abs(want)), s


def test_stream_ensemble_mode_equals_separate_streams(oracle):
    """ss_stream_cfg.stream_particles / subhalos_per_stream on the oracle:
    an ensemble run equals the streams run one by one with their own
    subhalo row (release layout restarting in every stream)."""
    rng = np.random.default_rng(5)
    B, n_rel, ppr = 3, 20, 2
    sh = dict(kind=1, m=10 ** rng.uniform(6, 8, B), a=rng.uniform(0.2, 0.8, B),
              x0=PROG_WF[:3] + rng.normal(0, 1.0, (B, 3)), v=rng.normal(0, 0.1, (B, 3)),
              t0=rng.uniform(0, 30, B), t_window=40.0)
    ics = PROG_WF + rng.normal(0, 0.2, (B, n_rel * ppr, 6)) * np.array([1, 1, 1, 0.01, 0.01, 0.01])
    full, _, st = oracle.stream(oracle.HostModel(oracle.mw3(), subhalos=sh), 0.0, 1.0, n_rel, ics.reshape(-1, 6),
                                ppr, 1, stream_particles=n_rel * ppr, subhalos_per_stream=1)
    assert (st == 0).all()
    for b in range(B):
        row = {k: (v[b:b + 1] if isinstance(v, np.ndarray) else v) for k, v in sh.items()}
        one, _, _ = oracle.stream(oracle.HostModel(oracle.mw3(), subhalos=row), 0.0, 1.0, n_rel, ics[b], ppr, 1)
        assert np.array_equal(full.reshape(B, -1, 6)[b], one)


def test_rotating_bars_and_frame_acceleration(oracle):
    """The oracle's time-dependent components: a bar at time t is the bar at
    t = 0 seen at the point rotated by -Omega t (potential.py:185-198,
    205-222); autodiff gradients against central differences; the uniform
    acceleration's gradient is the frame velocity's derivative (the slope of
    the linear track, potential.py:497-499)."""
    rng = np.random.default_rng(3)
    kinds = [(_abi.SS_BAR, 0, (2e10, 4.0, 1.0, 0.5, 0.045)),
             (_abi.SS_DEHNEN_BAR, 0, (0.01, 0.22, 8.0, 3.5, 0.4, 0.045))]
    for comp in kinds:
        m = oracle.HostModel([comp])
        x = rng.normal(0, 5, (20, 3))
        x[:5] *= 0.3  # points inside the Dehnen bar's Rb too
        t = 37.0
        om = comp[2][4] if comp[0] == _abi.SS_BAR else comp[2][5]
        a = -om * t
        xr = np.stack([np.cos(a) * x[:, 0] - np.sin(a) * x[:, 1], np.sin(a) * x[:, 0] + np.cos(a) * x[:, 1], x[:, 2]], 1)
        phi_t, g, _ = oracle.potential_eval(m, x, t)
        phi_0, _, _ = oracle.potential_eval(m, xr, 0.0)
        assert np.allclose(phi_t, phi_0, rtol=1e-12, atol=1e-16)
        h = 1e-5
        for k in range(3):
            e = np.zeros(3)
            e[k] = h
            fd = (oracle.potential_eval(m, x + e, t)[0] - oracle.potential_eval(m, x - e, t)[0]) / (2 * h)
            assert np.max(np.abs(fd - g[:, k])) <= 1e-6 * np.max(np.abs(g))
    tv = np.arange(40) * 25.0 - 800.0
    vel = np.stack([0.01 * np.sin(tv / 300), 0.02 * np.cos(tv / 200), -0.005 * tv / 800], 1)
    m = oracle.HostModel([(_abi.SS_UNIFORM_ACCEL, 0, ())], frame_velocity=(tv[0], 25.0, vel, "linear"))
    for t in (-790.0, -312.5, -13.0):
        k = int((t - tv[0]) // 25.0)
        _, g, H = oracle.potential_eval(m, rng.normal(0, 5, (4, 3)), t)
        assert np.allclose(g, (vel[k + 1] - vel[k]) / 25.0, rtol=1e-13, atol=1e-18)
        assert np.all(H == 0)


def test_growing_potential_oracle(oracle):
    """GrowingPotential on the oracle (potential.py:474-477): the wrapped
    potential times the growth track's value at t (linear here, so the
    factor is known in closed form), in the potential and its derivatives."""
    comps = [(_abi.SS_NFW, 0, (5.4e11, 15.62, 0.0)), (_abi.SS_MIYAMOTO_NAGAI, 0, (6.8e10, 3.0, 0.28))]
    tk = np.arange(11) * 100.0 - 1000.0
    g = 0.5 + 0.05 * np.arange(11) ** 1.3
    grow = oracle.HostModel([(k, c | _abi.SS_GROWS, p) for (k, c, p) in comps], growth=(tk[0], 100.0, g, "linear"))
    plain = oracle.HostModel(comps)
    rng = np.random.default_rng(3)
    x = rng.normal(0, 8, (50, 3))
    t = rng.uniform(-1000.0, 0.0, 50)
    gt = np.interp(t, tk, g)
    p1, g1, H1 = oracle.potential_eval(grow, x, t)
    p0, g0, H0 = oracle.potential_eval(plain, x, t)
    assert np.allclose(p1, gt * p0, rtol=1e-14, atol=0)
    assert np.allclose(g1, gt[:, None] * g0, rtol=1e-14, atol=0)
    assert np.allclose(H1, gt[:, None, None] * H0, rtol=1e-13, atol=1e-30)
