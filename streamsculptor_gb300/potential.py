"""Potential classes — the reference's potential.py names and keyword arguments.

Each class flattens into components of the device descriptor
(ss_potential).  Supported on the GPU path (jnibauer/streamsculptor
potential.py): MiyamotoNagaiDisk (66-72), NFWPotential (74-84),
TriaxialNFWPotential (86-97), Isochrone (114-122), PlummerPotential
(124-130), HernquistPotential (132-138), ProgenitorPotential (140-153),
GalaMilkyWayPotential (390-418), TimeDepTranslatingPotential (448-462),
SubhaloLinePotential (802-850), SubhaloLinePotential_dRadius (852-904),
SubhaloLinePotential_Custom (908-956) with a Plummer or Hernquist profile,
Potential_Combine (1279-1296), and the time-dependent BarPotential (178-198),
DehnenBarPotential (200-222), UniformAcceleration (480-502) and
MW_LMC_Potential (555-662, its tracks passed in).  CustomPotential (787-797) holds an arbitrary
Python callable and cannot run in a CUDA kernel: using it raises.
"""
from __future__ import annotations

import math

import numpy as np
import torch

from . import _abi, _core
from ._core import CenterTrack, Flat, SubhaloTable, f64, host64, usys  # noqa: F401
from .main import Potential


def _f(x) -> float:
    return float(host64(x))


class MiyamotoNagaiDisk(Potential):
    def __init__(self, m, a, b, units=None):
        super().__init__(units, {"m": m, "a": a, "b": b})

    def _flatten(self):
        return Flat([(_abi.SS_MIYAMOTO_NAGAI, _abi.SS_CENTER_ORIGIN, (_f(self.m), _f(self.a), _f(self.b)))])


class MN3ExponentialDiskPotential(Potential):
    """An exponential disk (scale length h_R, scale height h_z) as the sum of
    three Miyamoto-Nagai disks (MN3ExponentialDiskPotential, potential.py:224-280;
    Smith et al. 2015, MNRAS 448, 2934).  The three masses and scale
    lengths are K x (b^4, b^3, b^2, b, 1) with b = b_MN / h_R a cubic fit in
    h_z / h_R; K is the published 6 x 5 coefficient table for a positive
    (or, positive_density=False, the unconstrained) density, the cubic for
    a sech^2 (or exponential, sech2_z=False) vertical profile.  The three
    disks share b_MN and are summed in order, as Potential_Combine sums."""

    # Smith et al. (2015), Table 1: rows m1, m2, m3 (in m), a1, a2, a3 (in
    # h_R); columns the coefficients of (b/h_R)^4 .. (b/h_R)^0.
    K_POSITIVE = np.array([[0.0036, -0.0330, 0.1117, -0.1335, 0.1749],
                           [-0.0131, 0.1090, -0.3035, 0.2921, -5.7976],
                           [-0.0048, 0.0454, -0.1425, 0.1012, 6.7120],
                           [-0.0158, 0.0993, -0.2070, -0.7089, 0.6445],
                           [-0.0319, 0.1514, -0.1279, -0.9325, 2.6836],
                           [-0.0326, 0.1816, -0.2943, -0.6329, 2.3193]])
    K_NEGATIVE = np.array([[-0.0090, 0.0640, -0.1653, 0.1164, 1.9487],
                           [0.0173, -0.0903, 0.0877, 0.2029, -1.3077],
                           [-0.0051, 0.0287, -0.0361, -0.0544, 0.2242],
                           [-0.0358, 0.2610, -0.6987, -0.1193, 2.0074],
                           [-0.0830, 0.4992, -0.7967, -1.2966, 4.4441],
                           [-0.0247, 0.1718, -0.4124, -0.5944, 0.7333]])

    def __init__(self, m, h_R, h_z, units=None, positive_density=True, sech2_z=True):
        super().__init__(units, {"m": m, "h_R": h_R, "h_z": h_z})
        self.positive_density = bool(positive_density)
        self.sech2_z = bool(sech2_z)
        K = self.K_POSITIVE if self.positive_density else self.K_NEGATIVE
        q = _f(h_z) / _f(h_R)
        if self.sech2_z:
            b = -0.033 * q ** 3 + 0.262 * q ** 2 + 0.659 * q
        else:
            b = -0.269 * q ** 3 + 1.08 * q ** 2 + 1.092 * q
        pv = K @ np.array([b ** 4, b ** 3, b ** 2, b, 1.0])
        self._ms = pv[:3] * _f(m)
        self._as = pv[3:] * _f(h_R)
        self._b = b * _f(h_R)

    def _flatten(self):
        return Flat([(_abi.SS_MIYAMOTO_NAGAI, _abi.SS_CENTER_ORIGIN, (float(mi), float(ai), float(self._b)))
                     for mi, ai in zip(self._ms, self._as)])


class NFWPotential(Potential):
    """Phi = -G m log(1 + r/r_s) / r (unsoftened, potential.py:80-84)."""

    def __init__(self, m, r_s, units=None, _soft=0.0):
        super().__init__(units, {"m": m, "r_s": r_s})
        self._soft = float(_soft)

    def _flatten(self):
        return Flat([(_abi.SS_NFW, _abi.SS_CENTER_ORIGIN, (_f(self.m), _f(self.r_s), self._soft))])


class TriaxialNFWPotential(Potential):
    """Flattening in the potential: NFW of (x/q1, y/q2, z/q3)."""

    def __init__(self, m, r_s, q1=1.0, q2=1.0, q3=1.0, units=None):
        super().__init__(units, {"m": m, "r_s": r_s, "q1": q1, "q2": q2, "q3": q3})

    def _flatten(self):
        return Flat([(_abi.SS_TRIAXIAL_NFW, _abi.SS_CENTER_ORIGIN,
                      (_f(self.m), _f(self.r_s), _f(self.q1), _f(self.q2), _f(self.q3)))])


class Isochrone(Potential):
    def __init__(self, m, a, units=None):
        super().__init__(units, {"m": m, "a": a})

    def _flatten(self):
        return Flat([(_abi.SS_ISOCHRONE, _abi.SS_CENTER_ORIGIN, (_f(self.m), _f(self.a)))])


class PlummerPotential(Potential):
    def __init__(self, m, r_s, units=None):
        super().__init__(units, {"m": m, "r_s": r_s})

    def _flatten(self):
        return Flat([(_abi.SS_PLUMMER, _abi.SS_CENTER_ORIGIN, (_f(self.m), _f(self.r_s)))])


class HernquistPotential(Potential):
    def __init__(self, m, r_s, soft=0.0, units=None):
        super().__init__(units, {"m": m, "r_s": r_s, "soft": soft})

    def _flatten(self):
        return Flat([(_abi.SS_HERNQUIST, _abi.SS_CENTER_ORIGIN, (_f(self.m), _f(self.r_s), _f(self.soft)))])


class SphericalHarmonicExpansionPotential(Potential):
    """Multipole expansion Phi = scale * sum_lm f_lm(r) Y_lm(theta, phi) with
    real Schmidt semi-normalised harmonics up to l_max <= 8 and cubic Hermite
    radial splines in ln r (the layout of ss_expansion in the C header).
    The reference names an optional multipole package (bfeax) for such
    potentials; this class is the table-driven form the kernels evaluate.

    coef: [n_knots, (l_max+1)^2, 2] value and d f / d ln r of every f_lm at
    the knots ln r_k = log_r0 + k dlog_r; term index l*l + l + m (m < 0 are
    the sin(|m| phi) parts)."""

    def __init__(self, coef, log_r0, dlog_r, scale=1.0, units=None):
        c = torch.as_tensor(np.asarray(coef) if not torch.is_tensor(coef) else coef, dtype=torch.float64)
        if c.ndim != 3 or c.shape[2] != 2 or c.shape[0] < 2:
            raise ValueError("coef must be [n_knots >= 2, (l_max+1)^2, 2]")
        l_max = int(round(np.sqrt(c.shape[1]))) - 1
        if (l_max + 1) ** 2 != c.shape[1] or l_max > _abi.SS_SHEXP_LMAX:
            raise ValueError(f"coef has {c.shape[1]} terms: need (l_max+1)^2 with l_max <= {_abi.SS_SHEXP_LMAX}")
        super().__init__(units, {"coef": c, "log_r0": float(log_r0), "dlog_r": float(dlog_r), "scale": scale,
                                 "l_max": l_max})
        self._table = None

    def _flatten(self):
        if self._table is None:
            self._table = _core.ExpansionTable(self.l_max, self.log_r0, self.dlog_r,
                                               self.coef.to(_core.device()).contiguous())
        return Flat([(_abi.SS_SH_EXPANSION, _abi.SS_CENTER_ORIGIN, (_f(self.scale),))], expansion=self._table)


class get_potential_from_density(Potential):
    """Spherical potential tabulated from a density profile
    (potential.py:504-552): Phi(r_k) = -4 pi G (int_0^r rho r'^2 dr' / r +
    int_r^inf rho r' dr') on r_grid (default logspace(-3, 3, 128)), by
    adaptive quadrature on the host (the reference uses quadgk), then a cubic
    spline in ln r with the knot derivatives of interpax's 'cubic' rule.  The
    kernels evaluate it as a single-term (l_max = 0) spherical-harmonic
    expansion.  density_func is a Python callable of r (numpy scalars);
    r_grid must be log-spaced.  Outside r_grid the spline continues linearly
    in ln r (the reference's interpolant returns NaN there)."""

    def __init__(self, density_func, r_grid=None, units=None):
        from scipy import integrate
        super().__init__(units, {"density_func": density_func, "r_grid": r_grid})
        r = np.logspace(-3, 3, 128) if r_grid is None else np.asarray(host64(r_grid), dtype=np.float64)
        u = np.log(r)
        du = np.diff(u)
        if len(r) < 2 or not np.allclose(du, du[0], rtol=1e-9, atol=0) or du[0] <= 0:
            raise NotImplementedError("r_grid must be log-spaced and increasing")
        self.r_grid = r
        G = self._G
        f = lambda x, k: float(density_func(x)) * x ** k  # noqa: E731
        phi = np.empty_like(r)
        for i, ri in enumerate(r):
            inner = integrate.quad(f, 0.0, ri, args=(2,), epsabs=0, epsrel=1e-12, limit=200)[0]
            outer = integrate.quad(f, ri, np.inf, args=(1,), epsabs=0, epsrel=1e-12, limit=200)[0]
            phi[i] = -4 * np.pi * G * (inner / ri + outer)
        self.phi_grid = phi
        coef = np.stack([phi, _cubic_knot_slopes(phi, du[0])], axis=1)[:, None, :]
        self._spline = SphericalHarmonicExpansionPotential(coef, u[0], du[0], units=self.units)

    def _flatten(self):
        return self._spline._flatten()

    def density(self, xyz, t):
        x = np.asarray(host64(xyz), dtype=np.float64).reshape(-1, 3)
        return np.array([float(self.density_func(v)) for v in np.linalg.norm(x, axis=1)])


def _nfw_phi_and_rderiv(r, GM, rs):
    """NFW potential and r dPhi/dr (= dPhi/d ln r)."""
    L = np.log1p(r / rs)
    phi = -GM * L / r
    dphidr = GM * (L / r ** 2 - 1.0 / (r * (r + rs)))
    return phi, r * dphidr


def seeded_triaxial_expansion(m=5.4e11, r_s=15.62, eps=0.1, l_max=8, n_knots=64, r_min=0.1, r_max=200.0,
                              seed=4, units=None) -> SphericalHarmonicExpansionPotential:
    """A triaxial halo as a spherical-harmonic expansion: the monopole is the
    NFW(m, r_s) potential and every even-l, even-m cosine term (triaxial
    symmetry) with l >= 2 is
        f_lm(r) = eps 2^-l z_lm Phi_NFW(r) r^2 / (r^2 + r_s^2),   z_lm ~ N(0, 1)
    from numpy's PCG64(seed), on n_knots log-spaced knots over [r_min, r_max]
    with exact knot derivatives."""
    G = _core.G_for(units)
    rng = np.random.Generator(np.random.PCG64(seed))
    log_r0 = np.log(r_min)
    dlog_r = (np.log(r_max) - np.log(r_min)) / (n_knots - 1)
    r = np.exp(log_r0 + dlog_r * np.arange(n_knots))
    phi0, dphi0 = _nfw_phi_and_rderiv(r, G * m, r_s)
    g = r ** 2 / (r ** 2 + r_s ** 2)
    dg = 2.0 * r ** 2 * r_s ** 2 / (r ** 2 + r_s ** 2) ** 2  # r dg/dr
    nt = (l_max + 1) ** 2
    coef = np.zeros((n_knots, nt, 2))
    coef[:, 0, 0], coef[:, 0, 1] = phi0, dphi0
    for l in range(2, l_max + 1, 2):
        for mm in range(0, l + 1, 2):
            z = rng.standard_normal()
            a = eps * 2.0 ** -l * z
            j = l * l + l + mm
            coef[:, j, 0] = a * phi0 * g
            coef[:, j, 1] = a * (dphi0 * g + phi0 * dg)
    return SphericalHarmonicExpansionPotential(coef, log_r0, dlog_r, units=units)


class Potential_Combine(Potential):
    """Sum of potentials in list order (potential.py:1279-1296)."""

    def __init__(self, potential_list, units=None):
        super().__init__(units, {"potential_list": list(potential_list)})

    def _flatten(self):
        flat = Flat()
        for p in self.potential_list:
            flat.extend(p._flatten())
        return flat


class TimeDepTranslatingPotential(Potential):
    """pot evaluated at x - center(t) (potential.py:448-462).

    center_spl must be a CenterTrack (uniform knots; Hermite cubic with
    interpax-'cubic' slopes), e.g. CenterTrack.from_samples(ts, orbit[:, :3])."""

    def __init__(self, pot, center_spl, units=None):
        super().__init__(units, {"pot": pot, "center_spl": center_spl})

    def _flatten(self):
        if not isinstance(self.center_spl, CenterTrack):
            raise NotImplementedError("center_spl must be a CenterTrack (arbitrary callables cannot run on the GPU)")
        inner = self.pot._flatten()
        if inner.track is not None or inner.subhalos is not None:
            raise NotImplementedError("nested translating potentials / subhalos inside a translating potential")
        comps = [(k, _abi.SS_CENTER_TRACK, p) for (k, _, p) in inner.comps]
        return Flat(comps, track=self.center_spl)


class GrowingPotential(Potential):
    """pot times a growth factor g(t) (GrowingPotential, potential.py:464-477).

    growth_func must be a scalar track on uniform knots, e.g.
    CenterTrack.growth_from_samples(ts, g) (cubic Hermite with the
    interpax-'cubic' slopes of the center tracks, or linear=True); a Python
    callable cannot run in a kernel.  Every component of pot is multiplied
    by g(t) in the potential, its gradient and Hessian."""

    def __init__(self, pot, growth_func, units=None):
        super().__init__(units, {"pot": pot, "growth_func": growth_func})

    def _flatten(self):
        if not isinstance(self.growth_func, CenterTrack):
            raise NotImplementedError("growth_func must be a track (CenterTrack.growth_from_samples): arbitrary "
                                      "callables cannot run on the GPU")
        inner = self.pot._flatten()
        if inner.growth is not None or inner.subhalos is not None:
            raise NotImplementedError("nested growing potentials / subhalos inside a growing potential")
        comps = [(k, c | _abi.SS_GROWS, p) for (k, c, p) in inner.comps]
        return Flat(comps, track=inner.track, expansion=inner.expansion, frame_velocity=inner.frame_velocity,
                    growth=self.growth_func)


class ProgenitorPotential(Potential):
    """prog_pot(m, r_s) centred on the progenitor track (potential.py:140-153)."""

    def __init__(self, m, r_s, interp_func, prog_pot, units=None):
        super().__init__(units, {"m": m, "r_s": r_s, "interp_func": interp_func})
        self.prog_pot = prog_pot(m=m, r_s=r_s, units=units)

    def _flatten(self):
        return TimeDepTranslatingPotential(self.prog_pot, self.interp_func, units=self.units)._flatten()


class PowerLawCutoffPotential(Potential):
    """Spherical power law rho ~ r^-alpha with an exp(-(r / r_c)^2) cutoff
    (PowerLawCutoffPotential, potential.py:357-388): dPhi/dr = G m
    P((3 - alpha) / 2, r^2 / r_c^2) / r^2 with P the regularised lower
    incomplete gamma function, evaluated in the kernels (series or continued
    fraction); the potential value needs alpha < 2 (NaN otherwise, as the
    reference's formula gives)."""

    def __init__(self, m, alpha, r_c, units=None):
        super().__init__(units, {"m": m, "alpha": alpha, "r_c": r_c})

    def _flatten(self):
        return Flat([(_abi.SS_POWERLAW_CUTOFF, _abi.SS_CENTER_ORIGIN, (_f(self.m), _f(self.alpha), _f(self.r_c)))])


class ZhaoPotential(Potential):
    """Zhao (1996) double power-law sphere (ZhaoPotential, potential.py:282-355):
    rho = rho0 / (x^gamma (1 + x^(1/alpha))^((beta - gamma) alpha)), x = r / r_s,
    with rho0 normalising the total mass to m.  The kernels evaluate the
    potential with the regularised incomplete beta function (continued
    fraction) and the gradient as dPhi/dr = G m I_z(alpha (3 - gamma),
    alpha (beta - 3)) / r^2 at r + dr / 2, dr = 1e-5 r + 1e-8: the reference's
    forward difference of its potential over [r, r + dr] (gradient_func) to
    O(dr^2), without the difference's cancellation.  Needs alpha > 0,
    beta > 3 and 0 <= gamma < 2 (the reference replaces alpha (2 - gamma) <= 0
    by sqrt(eps), which changes the potential)."""

    def __init__(self, m, r_s, alpha, beta, gamma, units=None):
        super().__init__(units, {"m": m, "r_s": r_s, "alpha": alpha, "beta": beta, "gamma": gamma})

    def _flatten(self):
        return Flat([(_abi.SS_ZHAO, _abi.SS_CENTER_ORIGIN,
                      (_f(self.m), _f(self.r_s), _f(self.alpha), _f(self.beta), _f(self.gamma)))])

    def density(self, xyz, t):
        """ZhaoPotential._density (potential.py:308-319), on the host."""
        al, be, ga = _f(self.alpha), _f(self.beta), _f(self.gamma)
        a1, b1 = al * (3.0 - ga), al * (be - 3.0)
        rho0 = _f(self.m) / (4.0 * np.pi * al * np.exp(math.lgamma(a1) + math.lgamma(b1) - math.lgamma(a1 + b1)))
        r = np.linalg.norm(np.asarray(host64(xyz), dtype=np.float64).reshape(-1, 3), axis=1)
        x = r / _f(self.r_s)
        return rho0 / _f(self.r_s) ** 3 / x ** ga / (1.0 + x ** (1.0 / al)) ** ((be - ga) * al)


class BovyMWPotential2014(Potential):
    """Disk + bulge + halo of Bovy (2015) MWPotential2014 (potential.py:420-446):
    Miyamoto-Nagai disk, power-law bulge with cutoff, NFW halo, summed in
    that order."""

    def __init__(self, units=None):
        super().__init__(units, {"params": None})
        self.m_disk, self.a_disk, self.b_disk = 6.82e10, 3.0, 0.28
        self.m_bulge, self.alpha_bulge, self.r_c_bulge = 4.50e9, 1.80, 1.90
        self.m_halo, self.r_s_halo = 4.37e11, 16.0
        self.pot = Potential_Combine([
            MiyamotoNagaiDisk(m=self.m_disk, a=self.a_disk, b=self.b_disk, units=self.units),
            PowerLawCutoffPotential(m=self.m_bulge, alpha=self.alpha_bulge, r_c=self.r_c_bulge, units=self.units),
            NFWPotential(m=self.m_halo, r_s=self.r_s_halo, units=self.units),
        ], units=self.units)

    def _flatten(self):
        return self.pot._flatten()


class GalaMilkyWayPotential(Potential):
    """Disk + bulge + nucleus + halo (potential.py:390-418), summed in that order."""

    def __init__(self, units=None):
        super().__init__(units, {"params": None})
        self.m_disk, self.a_disk, self.b_disk = 6.80e10, 3.0, 0.28
        self.m_bulge, self.c_bulge = 5e9, 1.0
        self.m_nucleus, self.c_nucleus = 1.71e9, 0.07
        self.m_halo, self.r_s_halo = 5.4e11, 15.62
        self.pot = Potential_Combine([
            MiyamotoNagaiDisk(m=self.m_disk, a=self.a_disk, b=self.b_disk, units=self.units),
            HernquistPotential(m=self.m_bulge, r_s=self.c_bulge, units=self.units),
            HernquistPotential(m=self.m_nucleus, r_s=self.c_nucleus, units=self.units),
            NFWPotential(m=self.m_halo, r_s=self.r_s_halo, units=self.units),
        ], units=self.units)

    def _flatten(self):
        return self.pot._flatten()


class BarPotential(Potential):
    """Long & Murali (1992) bar rotating about z at pattern speed Omega
    (potential.py:178-198): the simulation-frame point is rotated by
    -Omega t into the bar frame.  The rotating components of one potential
    share one pattern speed."""

    def __init__(self, m, a, b, c, Omega, units=None):
        super().__init__(units, {"m": m, "a": a, "b": b, "c": c, "Omega": Omega})

    def _flatten(self):
        return Flat([(_abi.SS_BAR, _abi.SS_CENTER_ORIGIN,
                      (_f(self.m), _f(self.a), _f(self.b), _f(self.c), _f(self.Omega)))])


class DehnenBarPotential(Potential):
    """Dehnen (2000) bar: alpha v0^2/3 (R0/Rb)^3 (R/r)^2 U(r) cos 2(phi - phib -
    Omega t) with U = -(r/Rb)^-3 outside Rb and (r/Rb)^3 - 2 inside
    (potential.py:200-222)."""

    def __init__(self, alpha, v0, R0, Rb, phib, Omega, units=None):
        super().__init__(units, {"alpha": alpha, "v0": v0, "R0": R0, "Rb": Rb, "phib": phib, "Omega": Omega})

    def _flatten(self):
        return Flat([(_abi.SS_DEHNEN_BAR, _abi.SS_CENTER_ORIGIN,
                      (_f(self.alpha), _f(self.v0), _f(self.R0), _f(self.Rb), _f(self.phib), _f(self.Omega)))])


class UniformAcceleration(Potential):
    """Spatially uniform acceleration -dv/dt of the frame velocity
    (potential.py:480-502).  velocity_func must be a CenterTrack of the
    frame's velocity (uniform knots; CenterTrack.linear_from_samples for the
    reference's linear interpolant).  It has a force but no potential."""

    def __init__(self, velocity_func=None, units=None):
        super().__init__(units, {"velocity_func": velocity_func})

    def _flatten(self):
        if not isinstance(self.velocity_func, CenterTrack):
            raise NotImplementedError("velocity_func must be a CenterTrack (arbitrary callables cannot run on the GPU)")
        return Flat([(_abi.SS_UNIFORM_ACCEL, _abi.SS_CENTER_ORIGIN, ())], frame_velocity=self.velocity_func)

    def potential(self, xyz, t):
        raise NotImplementedError("UniformAcceleration has a force but no potential")


class MW_LMC_Potential(Potential):
    """Milky Way + LMC as rigid bodies in the Milky Way's non-inertial frame
    (potential.py:555-662): Hernquist bulge (5e9, 1.0), Miyamoto-Nagai disk
    (5e10, 3.0, 0.3), NFW halo (5.4e11, 15.62); the LMC an NFW of
    0.85e11 Msun and r_s = (m/1e11)^0.6 8.5 kpc moving on its track; the
    reflex acceleration -dv_MW/dt as a uniform field.  Both tracks are
    linear interpolants, as the reference's RegularGridInterpolator.

    The reference loads its tracks from data files shipped with its package;
    here they are arguments: lmc_track = (t [n], xyz [n, 3]) and
    mw_velocity = (t [n], v [n, 3]), uniformly spaced increasing times."""

    def __init__(self, units=None, lmc_track=None, mw_velocity=None):
        super().__init__(units, {"params": None})
        if lmc_track is None or mw_velocity is None:
            raise ValueError("MW_LMC_Potential needs lmc_track=(t, xyz) and mw_velocity=(t, v)")
        self.LMC_track = CenterTrack.linear_from_samples(*lmc_track)
        self.MW_velocity = CenterTrack.linear_from_samples(*mw_velocity)
        u = self.units
        self.pot_MW = Potential_Combine([HernquistPotential(m=5e9, r_s=1.0, units=u),
                                         MiyamotoNagaiDisk(m=5.0e10, a=3.0, b=0.3, units=u),
                                         NFWPotential(m=5.4e11, r_s=15.62, units=u)], units=u)
        massLMC = 0.85e11
        self.pot_LMC = NFWPotential(m=massLMC, r_s=(massLMC / 1e11) ** 0.6 * 8.5, units=u)
        self.translating_LMC_pot = TimeDepTranslatingPotential(pot=self.pot_LMC, center_spl=self.LMC_track, units=u)
        self.unif_acc = UniformAcceleration(velocity_func=self.MW_velocity, units=u)
        self.total_pot = Potential_Combine([self.pot_MW, self.translating_LMC_pot, self.unif_acc], units=u)

    def _flatten(self):
        return self.total_pot._flatten()

    def potential(self, xyz, t):
        raise NotImplementedError("Potential not implemented, force is non-conservative")


class _SubhaloLines(Potential):
    _kind = _abi.SS_SH_PLUMMER

    def _table(self) -> SubhaloTable:
        dev = _core.device()
        x0 = f64(self.subhalo_x0, dev).reshape(-1, 3)
        n = x0.shape[0]
        m = f64(np.broadcast_to(host64(self.m), (n,)).copy(), dev)
        a = f64(np.broadcast_to(host64(self.a), (n,)).copy(), dev)
        v = f64(self.subhalo_v, dev).reshape(n, 3)
        t0 = f64(np.broadcast_to(host64(self.subhalo_t0), (n,)).copy(), dev)
        return SubhaloTable(self._kind, m, a, x0, v, t0, _f(self.t_window))

    def table(self) -> SubhaloTable:
        key = ("table", _core.device().index)
        t = self._desc_cache.get(key)
        if t is None:
            t = self._table()
            self._desc_cache[key] = t
        return t

    def _flatten(self):
        return Flat([], subhalos=self.table())

    def _per_sh(self, xyz, t):
        pts = f64(xyz)
        single = pts.ndim == 1
        pts = pts.reshape(-1, 3).contiguous()
        o = _core.subhalo_eval(self.table(), self._G, pts, float(host64(t)))
        return o, single

    def potential_per_SH(self, xyz, t):
        """Phi_s(x, t) per subhalo, zero outside the window (potential.py:832-850)."""
        (phi, _, _, _), single = self._per_sh(xyz, t)
        return phi[0] if single else phi

    def gradient_per_SH(self, xyz, t):
        """jacfwd(potential_per_SH) (perturbative.py:40): [N_sh, 3]."""
        (_, g, _, _), single = self._per_sh(xyz, t)
        return g[0] if single else g


class SubhaloLinePotential(_SubhaloLines):
    """Plummer subhalos on lines x0 + v (t - t0), active while |t - t0| < t_window."""

    def __init__(self, m, a, subhalo_x0, subhalo_v, subhalo_t0, t_window, units=None):
        super().__init__(units, {"m": m, "a": a, "subhalo_x0": subhalo_x0, "subhalo_v": subhalo_v,
                                 "subhalo_t0": subhalo_t0, "t_window": t_window})


class SubhaloLinePotential_dRadius(_SubhaloLines):
    """dPhi_s/da_s of the Plummer subhalos (potential.py:852-904).

    It is the structural companion used by the perturbation generator; as a
    force potential of its own it is not part of any stream integration."""

    def __init__(self, m, a, subhalo_x0, subhalo_v, subhalo_t0, t_window, units=None):
        super().__init__(units, {"m": m, "a": a, "subhalo_x0": subhalo_x0, "subhalo_v": subhalo_v,
                                 "subhalo_t0": subhalo_t0, "t_window": t_window})

    def _flatten(self):
        raise NotImplementedError("SubhaloLinePotential_dRadius is a structural derivative, not a force potential")

    def potential_per_SH(self, xyz, t):
        (_, _, d, _), single = self._per_sh(xyz, t)
        return d[0] if single else d

    def gradient_per_SH(self, xyz, t):
        (_, _, _, gd), single = self._per_sh(xyz, t)
        return gd[0] if single else gd

    def potential(self, xyz, t):
        """Sum over the subhalos of dPhi_s/da_s (potential.py:867-884): [N]
        for [N, 3] points, a scalar for one point."""
        return self.potential_per_SH(xyz, t).sum(dim=-1)

    def gradient(self, xyz, t):
        """Sum over the subhalos of grad dPhi_s/da_s: [N, 3], or [3]."""
        return self.gradient_per_SH(xyz, t).sum(dim=-2)


class SubhaloLinePotential_Custom(_SubhaloLines):
    """One profile `pot` (PlummerPotential or HernquistPotential) for all
    subhalos on lines (potential.py:908-956)."""

    def __init__(self, pot, subhalo_x0, subhalo_v, subhalo_t0, t_window, units=None):
        if isinstance(pot, PlummerPotential):
            kind, m, a = _abi.SS_SH_PLUMMER, pot.m, pot.r_s
        elif isinstance(pot, HernquistPotential):
            if _f(pot.soft) != 0.0:
                raise NotImplementedError("softened Hernquist subhalos")
            kind, m, a = _abi.SS_SH_HERNQUIST, pot.m, pot.r_s
        else:
            raise NotImplementedError("SubhaloLinePotential_Custom supports Plummer and Hernquist profiles")
        super().__init__(units, {"pot": pot, "m": m, "a": a, "subhalo_x0": subhalo_x0, "subhalo_v": subhalo_v,
                                 "subhalo_t0": subhalo_t0, "t_window": t_window})
        self._kind = kind


class SubhaloLinePotential_dRadius_Custom(SubhaloLinePotential_dRadius):
    """dPhi_s/da_s from a Python callable dpot_dRadius(xyz, t)
    (potential.py:1110-1160).  A callable cannot run in a kernel: use
    SubhaloLinePotentialCustom_dRadius_fromFunc with PlummerPotential or
    HernquistPotential, whose derivative the kernels evaluate in closed form."""

    def __init__(self, dpot_dRadius, subhalo_x0, subhalo_v, subhalo_t0, t_window, units=None):
        raise NotImplementedError("SubhaloLinePotential_dRadius_Custom evaluates a Python callable; use "
                                  "SubhaloLinePotentialCustom_dRadius_fromFunc(PlummerPotential or "
                                  "HernquistPotential, m, r_s, ...)")


class SubhaloLinePotentialCustom_dRadius_fromFunc(SubhaloLinePotential_dRadius):
    """dPhi_s/dr_s of subhalos on lines with the profile class `func`
    (PlummerPotential or HernquistPotential) built from arrays m, r_s
    (potential.py:1215-1262, jax.grad of the profile's potential with respect
    to r_s): G m a / (r^2 + a^2)^(3/2) for Plummer, G m / (r + a)^2 for
    Hernquist, zero outside the window.  It is the structural companion of
    SubhaloLinePotentialCustom_fromFunc with the same arguments."""

    def __init__(self, func, m, r_s, subhalo_x0, subhalo_v, subhalo_t0, t_window, units=None):
        if func not in (PlummerPotential, HernquistPotential):
            raise NotImplementedError("SubhaloLinePotentialCustom_dRadius_fromFunc supports PlummerPotential and "
                                      "HernquistPotential")
        _SubhaloLines.__init__(self, units, {"func": func, "m": m, "r_s": r_s, "a": r_s, "subhalo_x0": subhalo_x0,
                                             "subhalo_v": subhalo_v, "subhalo_t0": subhalo_t0,
                                             "t_window": t_window})
        self._kind = _abi.SS_SH_PLUMMER if func is PlummerPotential else _abi.SS_SH_HERNQUIST


class SubhaloLinePotentialCustom_fromFunc(SubhaloLinePotential_Custom):
    """Subhalos on lines with the profile class `func` (PlummerPotential or
    HernquistPotential) built from arrays m, r_s (potential.py:1161-1213)."""

    def __init__(self, func, m, r_s, subhalo_x0, subhalo_v, subhalo_t0, t_window, units=None):
        if func not in (PlummerPotential, HernquistPotential):
            raise NotImplementedError("SubhaloLinePotentialCustom_fromFunc supports PlummerPotential and "
                                      "HernquistPotential")
        super().__init__(func(m=m, r_s=r_s, units=units), subhalo_x0, subhalo_v, subhalo_t0, t_window, units=units)
        self.func = func


# ------------------------------------------------- tidally stripped NFW subhalos
def tnfw_enclosed_mass(R, rhos, rs, ft, rt):
    """Mass inside R of the truncated NFW rho_s f_t / (x (1+x)^2 (1 + (r/r_t)^2))
    (potential.py:958-969)."""
    R, rhos, rs, ft, rt = (np.asarray(host64(v)) for v in (R, rhos, rs, ft, rt))
    tau = rt / rs
    u = R / rs
    t2 = tau ** 2
    term1 = (t2 - 1) / (t2 + 1) ** 2 * np.log1p(u)
    term2 = 1 / (t2 + 1) * (1 / (1 + u) - 1)
    term3 = -(t2 - 1) / (2 * (t2 + 1) ** 2) * np.log1p(u ** 2 / t2)
    term4 = 2 * tau / (t2 + 1) ** 2 * np.arctan(u / tau)
    return 4 * np.pi * rhos * ft * rs ** 3 * t2 * (term1 + term2 + term3 + term4)


def nfw_params_from_infall(m_infall, c_infall, z_infall, H0=67.4, Omega_m=0.315, Omega_L=0.685):
    """(rho_s, r_s, R200) of the NFW halo at infall, m200 with respect to
    rho_crit(z_infall) (potential.py:971-986; its own G = 4.498e-12 kpc^3
    Msun^-1 Myr^-2 and H0 conversion, Planck 2018 defaults)."""
    m, c, z = (np.asarray(host64(v)) for v in (m_infall, c_infall, z_infall))
    G = 4.498e-12
    H0_myr = H0 * 1e3 / 3.0856e22 * 3.15576e13
    Hz = H0_myr * np.sqrt(Omega_m * (1 + z) ** 3 + Omega_L)
    rho_crit = 3 * Hz ** 2 / (8 * np.pi * G)
    R200 = (3 * m / (4 * np.pi * 200 * rho_crit)) ** (1 / 3)
    rs = R200 / c
    rhos = m / (4 * np.pi * rs ** 3 * (np.log1p(c) - c / (1 + c)))
    return rhos, rs, R200


def tidally_evolved_nfw_params_from_infall(m_infall, c_infall, z_infall, f_bound):
    """(rho_s, r_s, f_t, r_t) on the Du et al. (2024) tidal track for the
    bound mass fraction f_bound (potential.py:987-1001)."""
    rhos, rs, r200 = nfw_params_from_infall(m_infall, c_infall, z_infall)
    f = np.asarray(host64(f_bound))
    A, B, C = 0.68492777, 0.66438857, 2.07766512
    D, E = 0.75826635, 0.23376409
    ft = np.minimum((1 + D) * f ** E / (1 + D * f ** (2 * E)), 1.0)
    rt = (1 + A) * f ** B / (1 + A * f ** (2 * B)) / np.exp(C * (1 - f)) * r200
    return rhos, rs, ft, rt


def _tnfw_inner(u, tau):
    """J(u) = int_0^u v dv / ((1+v)^2 (v^2 + tau^2)), M(<r) = 4 pi rho_s f_t
    r_s^3 tau^2 J(r/r_s).  The closed form (tnfw_enclosed_mass) cancels its
    O(u) terms at small u (3e-9 relative at u = 1e-4), so there the Taylor
    series of the integrand is integrated instead."""
    u = np.asarray(u, dtype=np.float64)
    t2 = tau ** 2
    A = (t2 - 1) / (t2 + 1) ** 2
    closed = (A * (np.log1p(u) - 0.5 * np.log1p(u ** 2 / t2)) - u / ((1 + u) * (1 + t2)) +
              2 * tau / (t2 + 1) ** 2 * np.arctan(u / tau))
    small = u < 0.05 * min(1.0, tau)
    if np.any(small):
        us = u[small]
        # v / ((1+v)^2 (tau^2 + v^2)) = sum_n c_n v^n; J = sum_n c_n u^(n+1) / (n+1)
        n_terms = 40
        a = np.array([(-1.0) ** k * (k + 1) for k in range(n_terms)])
        b = np.zeros(n_terms)
        b[0::2] = np.array([(-1.0 / t2) ** j for j in range((n_terms + 1) // 2)]) / t2
        c = np.convolve(a, b)[:n_terms - 1]  # coefficients of v^0.. of a*b; times v shifts by one
        series = np.zeros_like(us)
        for n in range(n_terms - 2, -1, -1):  # J = sum_n c_n u^(n+2) / (n+2)
            series = series * us + c[n] / (n + 2)
        closed = np.array(closed, dtype=np.float64, copy=True)
        closed[small] = series * us * us
    return closed


def _tnfw_outer(X, tau):
    """int_X^inf dx / ((1+x)^2 (x^2 + tau^2)), by partial fractions."""
    t2 = tau ** 2
    A = 2.0 / (1 + t2) ** 2
    B = 1.0 / (1 + t2)
    D = (1 - t2) / (1 + t2) ** 2
    return A * (0.5 * np.log(X ** 2 + t2) - np.log1p(X)) + B / (1 + X) + D / tau * (np.pi / 2 - np.arctan(X / tau))


class _TNFWGrid:
    """r_grid and phi_grid of one truncated NFW, as the reference's
    get_potential_from_density object exposes them (potential.py:504-552)."""

    def __init__(self, r_grid, phi_grid):
        self.r_grid = r_grid
        self.phi_grid = phi_grid


def make_tnfw_potential_from_density_profile(rhos, rs, ft, rt, n_grid=256, G=None):
    """Phi on r_grid = logspace(1e-4 r_s, 1e3 r_s, n_grid) (potential.py:1009-1020):
    Phi(r) = -4 pi G (M(<r) / (4 pi r) + int_r^inf rho r' dr'), here with
    the enclosed mass and the outer integral in closed form (the reference
    integrates both numerically with quadgk)."""
    G = _core.G_for(usys) if G is None else G
    rhos, rs, ft, rt = (float(host64(v)) for v in (rhos, rs, ft, rt))
    r = np.logspace(np.log10(1e-4 * rs), np.log10(1e3 * rs), int(n_grid))
    tau = rt / rs
    M = 4 * np.pi * rhos * ft * rs ** 3 * tau ** 2 * _tnfw_inner(r / rs, tau)
    outer = rhos * ft * tau ** 2 * rs ** 2 * _tnfw_outer(r / rs, tau)
    return _TNFWGrid(r, -G * M / r - 4 * np.pi * G * outer)


def make_tnfw_potential_from_infall(m_infall, c_infall, z_infall, f_bound):
    rhos, rs, ft, rt = tidally_evolved_nfw_params_from_infall(m_infall, c_infall, z_infall, f_bound)
    return make_tnfw_potential_from_density_profile(rhos, rs, ft, rt)


def _cubic_knot_slopes(f, du):
    """Knot derivatives of interpax's 'cubic' interpolant on a uniform grid:
    the mean of the adjacent secants, one-sided at the two ends."""
    d = np.empty_like(f)
    sec = np.diff(f, axis=-1) / du
    d[..., 1:-1] = 0.5 * (sec[..., 1:] + sec[..., :-1])
    d[..., 0] = sec[..., 0]
    d[..., -1] = sec[..., -1]
    return d


class TNFWSubhaloLinePotential(_SubhaloLines):
    """Tidally stripped NFW subhalos on lines (potential.py:1022-1108): each
    subhalo's potential is tabulated on 256 log-spaced radii from its infall
    mass, concentration, infall redshift and bound fraction, and the kernels
    evaluate the cubic spline in ln r (SS_SH_GRID).  Outside the tabulated
    radii (1e-4 to 1e3 r_s) the spline continues linearly in ln r where the
    reference's interpolant returns NaN."""

    _kind = _abi.SS_SH_GRID

    def __init__(self, m_infall, c_infall, z_infall, f_bound, subhalo_x0, subhalo_v, subhalo_t0, t_window,
                 units=None, n_grid=256):
        n = len(np.atleast_1d(host64(m_infall)))
        bc = [np.broadcast_to(np.asarray(host64(v), dtype=np.float64), (n,)) for v in
              (m_infall, c_infall, z_infall, f_bound)]
        rhos, rs, ft, rt = tidally_evolved_nfw_params_from_infall(*bc)
        super().__init__(units, {"subhalo_x0": subhalo_x0, "subhalo_v": subhalo_v, "subhalo_t0": subhalo_t0,
                                 "t_window": t_window})
        grids = [make_tnfw_potential_from_density_profile(rhos[i], rs[i], ft[i], rt[i], n_grid, G=self._G)
                 for i in range(n)]
        self.log_r_grids = np.stack([np.log(g.r_grid) for g in grids])
        self.phi_grids = np.stack([g.phi_grid for g in grids])
        self.rhos, self.rs, self.ft, self.rt = rhos, rs, ft, rt
        self.m = np.zeros(n)
        self.a = np.asarray(rs, dtype=np.float64)

    def _table(self) -> SubhaloTable:
        dev = _core.device()
        x0 = f64(self.subhalo_x0, dev).reshape(-1, 3)
        n = x0.shape[0]
        du = self.log_r_grids[:, 1] - self.log_r_grids[:, 0]
        slopes = _cubic_knot_slopes(self.phi_grids, du[:, None])
        grid = np.stack([self.phi_grids, slopes], axis=2)
        t0 = f64(np.broadcast_to(host64(self.subhalo_t0), (n,)).copy(), dev)
        return SubhaloTable(self._kind, f64(self.m, dev), f64(self.a, dev), x0, f64(self.subhalo_v, dev).reshape(n, 3),
                            t0, _f(self.t_window), grid=f64(grid, dev), grid_u0=f64(self.log_r_grids[:, 0], dev),
                            grid_du=f64(du, dev))


class CustomPotential(Potential):
    """Arbitrary Python potential_func(xyz, t): no GPU implementation."""

    def __init__(self, potential_func=None, units=None):
        super().__init__(units, {"potential_func": potential_func})


__all__ = ["GrowingPotential", "PowerLawCutoffPotential", "ZhaoPotential", "BovyMWPotential2014", "MiyamotoNagaiDisk", "NFWPotential",
           "TriaxialNFWPotential", "Isochrone", "PlummerPotential",
           "HernquistPotential", "Potential_Combine", "TimeDepTranslatingPotential", "ProgenitorPotential",
           "GalaMilkyWayPotential", "SubhaloLinePotential", "SubhaloLinePotential_dRadius", "BarPotential",
           "DehnenBarPotential", "UniformAcceleration", "MW_LMC_Potential", "TNFWSubhaloLinePotential",
           "tnfw_enclosed_mass", "nfw_params_from_infall", "tidally_evolved_nfw_params_from_infall",
           "make_tnfw_potential_from_density_profile", "make_tnfw_potential_from_infall",
           "get_potential_from_density",
           "SubhaloLinePotential_Custom", "SubhaloLinePotentialCustom_fromFunc", "SubhaloLinePotential_dRadius_Custom",
           "SubhaloLinePotentialCustom_dRadius_fromFunc", "CustomPotential", "CenterTrack", "usys"]
