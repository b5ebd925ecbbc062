"""Subhalo encounter statistics — the reference's subhalostatistics.py API.

RateCalculator (subhalostatistics.py:14-219) turns a stream's orbit into an
expected number of subhalo encounters per mass (Yoon+2011, Erkal+2016) and
samples encounter masses from it.  It is host-side arithmetic over a few
thousand orbit samples and mass points (numpy, float64); the orbit comes
from the GPU orbit kernels through `Potential.integrate_orbit`.

Random draws: the reference uses JAX PRNG keys; here `key` is an integer
seed (or an array whose last entry is one, as a JAX key's) feeding numpy's
PCG64, split into independent child streams the way the reference splits
its key.  The distributions are the reference's; the draws themselves
differ.
"""
from __future__ import annotations

import numpy as np

# 180 km/s in kpc/Myr (astropy: (180*u.km/u.s).to(u.kpc/u.Myr))
KPC_PER_MYR_PER_KMS = 1.0227121650537077e-3
sigma = 180.0 * KPC_PER_MYR_PER_KMS


def seed_of(key) -> int:
    """Integer seed from an int, a numpy Generator draw, or a JAX-style key array."""
    if isinstance(key, np.random.Generator):
        return int(key.integers(0, 2 ** 63 - 1))
    return int(np.asarray(key).ravel()[-1])


def split_key(key, n: int):
    """n independent child seeds of `key` (jax.random.split's role)."""
    return [int(c.generate_state(1, np.uint64)[0]) for c in np.random.SeedSequence(seed_of(key)).spawn(n)]


def _trapezoid(y, x, axis=-1):
    return np.trapezoid(y, x=x, axis=axis)


class RateCalculator:
    """Encounter rate of a stream with subhalos (subhalostatistics.py:14-219).

    orbit: an orbit solution with .ys [n, 6] and .ts [n] (e.g. the
    progenitor's integrate_orbit(...) saved over the stream's age)."""

    def __init__(self, orbit, t_age, b_max_fac, l_obs, sigma=sigma, a0=1.77e-5, c0=2.02e-13, m0=2.52e7,
                 alpha=0.678, r_minus2=162.4, disk_factor=1.0):
        ys = np.asarray(_host(orbit.ys), dtype=np.float64)
        ts = np.asarray(_host(orbit.ts), dtype=np.float64)
        self.orbital_r = np.sqrt(np.sum(ys[:, 0:3] ** 2, axis=1))
        self.orbit_ts = np.linspace(0.0, np.max(np.abs(ts)), len(ts))
        self.t_age = float(t_age)
        self.b_max_fac = float(b_max_fac)
        self.sigma = float(sigma)
        self.l_obs = float(l_obs)
        self.a0 = float(a0)
        self.c0 = float(c0)
        self.m0 = float(m0)
        self.alpha = float(alpha)
        self.r_minus2 = float(r_minus2)
        self.disk_factor = float(disk_factor)

    def r_s_func(self, log10M, concentration_fac=1.0):
        return 1.05 * np.sqrt(10.0 ** np.asarray(log10M) / 1e8) * concentration_fac

    def b_max_func(self, log10M, concentration_fac=1.0):
        return self.b_max_fac * self.r_s_func(log10M, concentration_fac)

    def db_max_dlog10M(self, log10M, concentration_fac=1.0):
        M = 10.0 ** np.asarray(log10M)
        d_r_s = 1.05 * 0.5 * (M / 1e8) ** (-0.5) * 1e-8 * (M * np.log(10.0))
        return self.b_max_fac * d_r_s * concentration_fac

    def dN_dlog10M(self, log10M, slope=-1.9, gamma=2.7, M_hm=0.0, beta=0.99):
        """Subhalo mass function per dex, with the WDM suppression of arXiv:1911.02663."""
        M = 10.0 ** np.asarray(log10M)
        wdm = (1.0 + gamma * (M_hm / M)) ** (-beta)
        return (self.a0 * (M / self.m0) ** slope) * M * np.log(10.0) * wdm

    def spatial_density(self, r):
        """Einasto profile (unnormalised number per volume)."""
        return np.exp(-(2.0 / self.alpha) * ((np.asarray(r) / self.r_minus2) ** self.alpha - 1.0))

    def dn_dlog10M(self, r, log10M, slope=-1.9, gamma=2.7, M_hm=0.0, beta=0.99):
        return (self.c0 / self.a0) * self.dN_dlog10M(log10M, slope, gamma, M_hm, beta) * self.spatial_density(r)

    def nsub(self, r):
        return (self.c0 / self.a0) * self.spatial_density(r)

    def dN_encounter_dlog10M(self, log10M, normalization=1.0, slope=-1.9, concentration_fac=1.0, gamma=2.7,
                             M_hm=0.0, beta=0.99):
        """Encounters per dex at log10M, integrated over the orbit (scalar or
        array of masses)."""
        lm = np.asarray(log10M, dtype=np.float64)
        scalar = lm.ndim == 0
        lm = lm.reshape(-1, 1)
        r = self.orbital_r[None, :]
        dn = self.dn_dlog10M(r, lm, slope, gamma, M_hm, beta)
        integrand = (self.b_max_func(lm, concentration_fac) * dn +
                     self.db_max_dlog10M(lm, concentration_fac) * self.nsub(r)) * self.orbit_ts[None, :]
        prefac = np.sqrt(2.0 * np.pi) * self.sigma * self.disk_factor * (self.l_obs / self.t_age)
        out = _trapezoid(integrand, self.orbit_ts, axis=1) * prefac * normalization
        return float(out[0]) if scalar else out

    def N_encounter(self, log10M_min, log10M_max, normalization=1.0, slope=-1.9, concentration_fac=1.0, gamma=2.7,
                    M_hm=0.0, beta=0.99):
        """Poisson mean of the number of encounters in [M_min, M_max]."""
        lm = np.linspace(log10M_min, log10M_max, 1000)
        f = self.dN_encounter_dlog10M(lm, normalization, slope, concentration_fac, gamma, M_hm, beta)
        return float(_trapezoid(f, lm))

    def sample_masses(self, log10M_min, log10M_max, key, normalization=1.0, slope=-1.9, concentration_fac=1.0,
                      gamma=2.7, M_hm=0.0, beta=0.99, array_length=1_000):
        """Poisson number of encounters and their log10 masses
        (subhalostatistics.py:144-171): entries past the drawn number are 0."""
        k1, k2, _ = split_key(key, 3)
        rate = self.N_encounter(log10M_min, log10M_max, normalization, slope, concentration_fac, gamma, M_hm, beta)
        n_enc = int(np.random.default_rng(k1).poisson(rate))
        lm = np.linspace(log10M_min, log10M_max, 5_000)
        f = self.dN_encounter_dlog10M(lm, normalization, slope, concentration_fac, gamma, M_hm, beta)
        p = f * (lm[1] - lm[0])
        p = p / p.sum()
        samps = np.random.default_rng(k2).choice(lm, size=int(array_length), p=p, replace=True)
        idx = np.arange(int(array_length))
        return dict(log10_mass=np.where(idx >= n_enc, 0.0, samps), N_encounter=n_enc, N_encounter_rate=rate)

    def compute_N_enclosed(self, log10M_min, log10M_max, r_min, r_max, slope=-1.9, gamma=2.7, M_hm=0.0, beta=0.99):
        """Number of subhalos with masses and radii in the given ranges."""
        lm = np.linspace(log10M_min, log10M_max, 101)
        r = np.linspace(r_min, r_max, 100)
        LM, R = np.meshgrid(lm, r, indexing="ij")
        inp = self.dn_dlog10M(R, LM, slope, gamma, M_hm, beta) * 4.0 * np.pi * R ** 2
        return float(_trapezoid(_trapezoid(inp, lm, axis=0), r))


def _host(x):
    if hasattr(x, "detach"):
        return x.detach().cpu().numpy()
    return x


__all__ = ["RateCalculator", "sigma", "seed_of", "split_key"]
