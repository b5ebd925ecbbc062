"""CPU tests of the encounter-rate and sampling helpers
(subhalostatistics.py, streamhelpers.sample_from_1D_pdf): the trapezoid
integrals against scipy's adaptive quadrature, scalar/array agreement, the
Poisson/mass sampler against its own density (Kolmogorov-Smirnov), and the
inverse-CDF sampler against a closed-form CDF.  No GPU needed."""
from types import SimpleNamespace

import numpy as np
import pytest
from scipy import integrate, stats

from .conftest import PROG_WF


@pytest.fixture(scope="module")
def rate(oracle):
    from streamsculptor_gb300.subhalostatistics import RateCalculator
    orc = oracle.HostModel(oracle.mw3())
    t_age = 3000.0
    ys = oracle.orbit(orc, PROG_WF, 0.0, -t_age / 600, 600, 1)[0]
    orbit = SimpleNamespace(ys=ys, ts=np.linspace(0.0, -t_age, 601))
    return RateCalculator(orbit, t_age=t_age, b_max_fac=5.0, l_obs=10.0)


def test_encounter_rate_integrals(rate):
    lm = np.array([5.3, 6.1, 7.7])
    arr = rate.dN_encounter_dlog10M(lm)
    for i, v in enumerate(lm):
        assert arr[i] == pytest.approx(rate.dN_encounter_dlog10M(float(v)), rel=1e-14)
    # N_encounter (1000-point trapezoid over log10 M) vs adaptive quadrature
    ref, _ = integrate.quad(lambda x: rate.dN_encounter_dlog10M(x), 5.0, 8.0, epsabs=0, epsrel=1e-10)
    assert rate.N_encounter(5.0, 8.0) == pytest.approx(ref, rel=1e-5)
    # dN_encounter is the time integral of the rate along the orbit (trapezoid in the reference)
    t = rate.orbit_ts
    r = rate.orbital_r
    lmv = 6.4
    f = (rate.b_max_func(lmv) * rate.dn_dlog10M(r, lmv) + rate.db_max_dlog10M(lmv) * rate.nsub(r)) * t
    pref = np.sqrt(2 * np.pi) * rate.sigma * rate.disk_factor * rate.l_obs / rate.t_age
    assert rate.dN_encounter_dlog10M(lmv) == pytest.approx(integrate.trapezoid(f, t) * pref, rel=1e-13)
    # the derivative of b_max is the derivative of the function
    h = 1e-6
    fd = (rate.b_max_func(6.0 + h) - rate.b_max_func(6.0 - h)) / (2 * h)
    assert rate.db_max_dlog10M(6.0) == pytest.approx(fd, rel=1e-7)


def test_enclosed_number_matches_quadrature(rate):
    ref, _ = integrate.dblquad(lambda r, lm: rate.dn_dlog10M(r, lm) * 4 * np.pi * r ** 2, 6.0, 8.0, 1.0, 50.0,
                               epsrel=1e-9)
    assert rate.compute_N_enclosed(6.0, 8.0, 1.0, 50.0) == pytest.approx(ref, rel=2e-3)


def test_sample_masses(rate):
    d = rate.sample_masses(5.0, 8.0, key=11, normalization=20.0, array_length=4000)
    d2 = rate.sample_masses(5.0, 8.0, key=11, normalization=20.0, array_length=4000)
    assert np.array_equal(d["log10_mass"], d2["log10_mass"])  # a fixed key gives fixed draws
    n = d["N_encounter"]
    assert n == int((d["log10_mass"] > 0).sum()) and (d["log10_mass"][n:] == 0).all()
    assert abs(n - d["N_encounter_rate"]) < 6 * np.sqrt(d["N_encounter_rate"]) + 1
    # the masses follow dN_encounter/dlog10M (KS against its normalised CDF)
    big = rate.sample_masses(5.0, 8.0, key=3, normalization=1e4, array_length=20000)["log10_mass"]
    big = big[big > 0]
    lm = np.linspace(5.0, 8.0, 5000)
    cdf = np.cumsum(rate.dN_encounter_dlog10M(lm))
    cdf /= cdf[-1]
    ks = stats.kstest(big, lambda x: np.interp(x, lm, cdf))
    assert ks.pvalue > 1e-3


def test_sample_from_1d_pdf_inverse_cdf():
    from streamsculptor_gb300.streamhelpers import sample_from_1D_pdf
    x = np.linspace(0.0, 1.0, 4001)
    s = sample_from_1D_pdf(x, 3 * x ** 2, key=5, num_samples=50000)
    assert s.min() >= 0.0 and s.max() <= 1.0
    assert stats.kstest(s, lambda v: np.clip(v, 0, 1) ** 3).pvalue > 1e-3
    assert np.array_equal(s, sample_from_1D_pdf(x, 3 * x ** 2, key=5, num_samples=50000))
