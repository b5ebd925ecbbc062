"""Tidally stripped NFW subhalos (TNFWSubhaloLinePotential,
potential.py:958-1108): the host-side tables against numerical quadrature
of their defining integrals, and the oracle's spline of them.  No GPU."""
import numpy as np
import pytest
from scipy import integrate

from streamsculptor_gb300 import _abi


def _params():
    from streamsculptor_gb300 import potential as P
    return P.tidally_evolved_nfw_params_from_infall(np.array([3e7, 2e8, 1e9]), np.array([18.0, 14.0, 11.0]),
                                                    np.array([1.5, 2.0, 3.0]), np.array([0.3, 0.05, 0.8]))


def test_tnfw_grid_matches_quadrature():
    from streamsculptor_gb300 import potential as P
    from streamsculptor_gb300._core import G_for, usys
    G = G_for(usys)
    rhos, rs, ft, rt = _params()
    for i in range(3):
        rho = lambda r: rhos[i] * ft[i] / ((r / rs[i]) * (1 + r / rs[i]) ** 2 * (1 + (r / rt[i]) ** 2))  # noqa: E731
        grid = P.make_tnfw_potential_from_density_profile(rhos[i], rs[i], ft[i], rt[i])
        assert grid.r_grid.shape == (256,)
        for k in range(0, 256, 23):
            r = grid.r_grid[k]
            inner = integrate.quad(lambda x: rho(x) * x * x, 0, r, epsabs=0, epsrel=1e-12, limit=200)[0]
            outer = integrate.quad(lambda x: rho(x) * x, r, np.inf, epsabs=0, epsrel=1e-12, limit=200)[0]
            want = -4 * np.pi * G * (inner / r + outer)
            assert grid.phi_grid[k] == pytest.approx(want, rel=1e-11)
            # the reference's closed form loses digits to cancellation at small r / r_s only
            tol = 1e-12 if r / rs[i] > 0.1 else 1e-8
            assert P.tnfw_enclosed_mass(r, rhos[i], rs[i], ft[i], rt[i]) == pytest.approx(4 * np.pi * inner,
                                                                                          rel=tol)


def test_oracle_grid_spline(oracle):
    """The oracle's SS_SH_GRID spline goes through the knots and its
    gradient approaches the profile's force G M(<r) / r^2 between them."""
    from streamsculptor_gb300 import potential as P
    from streamsculptor_gb300._core import G_for, usys
    G = G_for(usys)
    pot = P.TNFWSubhaloLinePotential([2e8], [14.0], [2.0], [0.05], np.zeros((1, 3)), np.zeros((1, 3)), [0.0],
                                     np.inf, units=usys)
    du = pot.log_r_grids[0, 1] - pot.log_r_grids[0, 0]
    from streamsculptor_gb300.potential import _cubic_knot_slopes
    grid = np.stack([pot.phi_grids, _cubic_knot_slopes(pot.phi_grids, du)], axis=2)
    sh = dict(kind=_abi.SS_SH_GRID, m=[0.0], a=pot.a, x0=np.zeros((1, 3)), v=np.zeros((1, 3)), t0=[0.0],
              t_window=np.inf, grid=grid, grid_u0=pot.log_r_grids[:, 0], grid_du=[du])
    m = oracle.HostModel(oracle.mw3(), subhalos=sh)
    r = np.exp(pot.log_r_grids[0, 10:250:20])
    x = np.stack([r, np.zeros_like(r), np.zeros_like(r)], 1)
    phi, g, _, _ = oracle.subhalo_eval(m, x, 0.0)
    assert np.allclose(phi[:, 0], pot.phi_grids[0, 10:250:20], rtol=1e-13)
    rm = np.exp(pot.log_r_grids[0, 10:250:20] + 0.5 * du)  # mid-interval
    _, gm, _, _ = oracle.subhalo_eval(m, np.stack([rm, 0 * rm, 0 * rm], 1), 0.0)
    M = P.tnfw_enclosed_mass(rm, pot.rhos[0], pot.rs[0], pot.ft[0], pot.rt[0])
    assert np.allclose(gm[:, 0, 0], G * M / rm ** 2, rtol=2e-3)


def test_potential_from_density_grid():
    """get_potential_from_density (potential.py:504-552) for a Plummer
    density reproduces the Plummer potential at its knots."""
    from streamsculptor_gb300 import _core, potential as P
    M, a = 1e10, 2.0
    rho = lambda r: 3 * M / (4 * np.pi * a ** 3) * (1 + r * r / (a * a)) ** -2.5  # noqa: E731
    pot = P.get_potential_from_density(rho, units=_core.usys)
    G = _core.G_for(_core.usys)
    r = pot.r_grid
    assert np.allclose(pot.phi_grid, -G * M / np.sqrt(r * r + a * a), rtol=1e-12, atol=0)
    assert pot.density(np.array([[1.0, 0, 0]]), 0.0)[0] == pytest.approx(rho(1.0))
