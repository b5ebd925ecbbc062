"""Subhalo impact sampling — the reference's GenerateImpactParams.py API.

ImpactGenerator (GenerateImpactParams.py:9-213) draws impacts on a stream
(Yoon+2011, Erkal+2016): impact parameter, time (weighted by the stream's
length through time), location along the stream (phi1) and the
subhalo's velocity relative to the stream, then places each impactor in
Galactocentric Cartesian coordinates at its impact time.  The GPU part is
the back-integration of every stream patch from the observation time to its
own impact time: one ensemble orbit launch (ss_orbit_ensemble_f64, each
orbit with its own fixed step) instead of one adaptive solve per impact.

Random draws use numpy PCG64 children of `seednum` in the roles of the
reference's seven JAX keys (same distributions, different draws).  As with
a fixed JAX key, each sampling method returns the same draws every call.
"""
from __future__ import annotations

import math

import numpy as np
import torch

from . import _core
from ._core import f64, host64
from .streamhelpers import compute_length_oscillations, compute_stream_length, sample_from_1D_pdf
from .subhalostatistics import sigma as SIGMA, split_key


class ImpactGenerator:
    """Impact generator (GenerateImpactParams.py:9-213).

    pot               base potential (orbit integration)
    tobs              observation time
    stream            [N, 6] present-day stream, leading arm first, then trailing
    stream_phi1       [N] along-stream angle of each particle
    stripping_times   [N] release time of each particle
    prog_today        [6] progenitor today
    dt                fixed step (Myr) of the patch back-integrations (default 1)
    """

    def __init__(self, pot, tobs, stream, stream_phi1, stripping_times, prog_today, phi1window=0.1, NumImpacts=1,
                 tImpactBounds=None, bImpact_bounds=(0, 1.0), sigma=SIGMA, phi1_bounds=None, phi1_exclude=(1.0, 1.0),
                 stream_length=None, seednum=0, *, dt=1.0):
        self.pot = pot
        self.stream = f64(stream).reshape(-1, 6)
        self.stream_phi1 = f64(stream_phi1).reshape(-1)
        self.stripping_times = f64(stripping_times).reshape(-1)
        self.phi1window = float(phi1window)
        self.NumImpacts = int(NumImpacts)
        self.prog_today = f64(prog_today).reshape(6)
        self.tobs = float(host64(tobs))
        self.stream_length = stream_length
        self.sigma = float(sigma)
        self.seednum = int(seednum)
        self.phi1_exclude = [float(v) for v in host64(phi1_exclude).reshape(-1)]
        self.keys = split_key(self.seednum, 7)
        self.dt = float(dt)
        st = host64(self.stripping_times)
        self.tImpactBounds = [float(st.min()), 0.0] if tImpactBounds is None else \
            [float(v) for v in host64(tImpactBounds).reshape(-1)]
        p1 = host64(self.stream_phi1)
        self.phi1_bounds = [float(p1.min()), float(p1.max())] if phi1_bounds is None else \
            [float(v) for v in host64(phi1_bounds).reshape(-1)]
        b = np.asarray(host64(bImpact_bounds), dtype=np.float64)
        # [low, high] for every impact, or [NumImpacts, 2] (the reference tells
        # them apart by len == 2; the array rank is used here)
        if b.ndim == 1:
            self.b_low = np.full(self.NumImpacts, b[0])
            self.b_high = np.full(self.NumImpacts, b[1])
        else:
            self.b_low, self.b_high = b[:, 0].copy(), b[:, 1].copy()
        length = compute_stream_length(self.stream, self.stream_phi1) if stream_length is None else stream_length
        ind_break = len(st) // 2
        self.length_osc = compute_length_oscillations(self.pot, self.prog_today, self.stream[0], self.stream[ind_break],
                                                      t_age=abs(min(self.tImpactBounds)), length_today=length)

    def _rng(self, i):
        return np.random.default_rng(self.keys[i])

    def w_parallel_sample(self, vs):
        """Relative velocity along the stream: N(0, sigma) - vs, [NumImpacts]."""
        return self._rng(0).normal(size=self.NumImpacts) * self.sigma - np.asarray(host64(vs))

    def w_perpendicular_sample(self):
        """Relative speed across the stream, p(w) ~ w^2 exp(-w^2 / 2 sigma^2) on a
        10,000-point grid over [-7 sigma, 7 sigma], [NumImpacts]."""
        prefac = math.sqrt(2.0 / math.pi) / self.sigma ** 3
        w = np.linspace(-7 * self.sigma, 7 * self.sigma, 10_000)
        p = prefac * w ** 2 * np.exp(-w ** 2 / (2 * self.sigma ** 2))
        p = p / p.sum()
        return self._rng(1).choice(w, size=self.NumImpacts, p=p, replace=True)

    def sample_impact_params(self):
        """bImpact, tImpact, phi1 and the perpendicular angle of every impact
        (GenerateImpactParams.py:112-147)."""
        k = split_key(self.keys[-1], 4)
        n = self.NumImpacts
        bImpact = np.random.default_rng(k[0]).uniform(self.b_low, self.b_high, size=n)
        tImpact = sample_from_1D_pdf(self.length_osc["ts"], self.length_osc["length_func"], k[1], n)
        ex = self.phi1_exclude
        g = np.random.default_rng(k[2])
        if abs(ex[1] - ex[0]) > 0:
            seg1 = np.linspace(self.phi1_bounds[0], ex[0], 1000)
            seg2 = np.linspace(ex[1], self.phi1_bounds[1], 1000)
            l1 = ex[0] - self.phi1_bounds[0]
            l2 = self.phi1_bounds[1] - ex[1]
            p = np.concatenate([np.full(1000, l1 / (l1 + l2) / 1000), np.full(1000, l2 / (l1 + l2) / 1000)])
            phi1 = g.choice(np.concatenate([seg1, seg2]), size=n, replace=True, p=p / p.sum())
        else:
            phi1 = g.uniform(self.phi1_bounds[0], self.phi1_bounds[1], size=n)
        perp = np.random.default_rng(k[3]).uniform(0.0, 2.0 * np.pi, size=n)
        return {"bImpact": bImpact, "tImpact": tImpact, "phi1_samples": phi1, "perp_angle": perp}

    def get_particle_mean(self, phi1_0=None):
        """Mean phase-space state and mean stripping time of the particles with
        |phi1 - phi1_0| < phi1window (scalar or array of phi1_0)."""
        c = f64(phi1_0).reshape(-1, 1)
        inside = ((self.stream_phi1[None, :] > c - self.phi1window) &
                  (self.stream_phi1[None, :] < c + self.phi1window)).double()
        cnt = inside.sum(1)
        mean = inside @ self.stream / cnt[:, None]
        tmean = inside @ self.stripping_times / cnt
        if np.ndim(phi1_0) == 0:
            return mean[0], tmean[0]
        return mean, tmean

    def _get_subhalo_ImpactParamsCartesian(self, tobs=None, particle_mean=None, tstrip_mean=None, tImpact=None,
                                           bImpact=None, perp_angle=None, subidx=None):
        """Impactor phase-space state at its impact time
        (GenerateImpactParams.py:165-205), batched over impacts: each stream
        patch is integrated back from tobs to its tImpact, T is along its
        velocity, B along its angular momentum, N = B x T; the impact point is
        b (N cos a + B sin a) off the patch and the impactor's velocity is
        (w_par + v_s) T + w_perp (-N sin a + B cos a).  Returns (XV [n, 6],
        bImpact_hat [n, 3])."""
        tobs = self.tobs if tobs is None else float(host64(tobs))
        W = f64(particle_mean).reshape(-1, 6)
        n = W.shape[0]
        tI = f64(tImpact).reshape(n)
        subidx = np.arange(n) if subidx is None else np.asarray(subidx).reshape(n)
        span = float((tI - tobs).abs().max()) if n else 0.0
        n_steps = max(1, int(math.ceil(span / self.dt - 1e-9)))
        W0 = _core.orbit_ensemble(self.pot._desc(), W, tobs, (tI - tobs) / n_steps, n_steps)[:, -1]
        T = W0[:, 3:] / torch.linalg.norm(W0[:, 3:], dim=1, keepdim=True)
        Bv = torch.linalg.cross(W0[:, :3], W0[:, 3:], dim=1)
        Bv = Bv / torch.linalg.norm(Bv, dim=1, keepdim=True)
        N = torch.linalg.cross(Bv, T, dim=1)
        v_s = torch.linalg.norm(W0[:, 3:], dim=1)
        a = f64(perp_angle).reshape(n, 1)
        idx = torch.as_tensor(subidx, device=W0.device)
        # impact i: w_parallel_sample(v_s[i])[subidx[i]] + v_s[i], as the vmapped reference
        w_par = f64(self.w_parallel_sample(0.0))[idx] - v_s
        w_perp = f64(self.w_perpendicular_sample())
        V_par = (w_par + v_s)[:, None] * T
        V_perp = w_perp[idx][:, None] * (-N * torch.sin(a) + Bv * torch.cos(a))
        bhat = N * torch.cos(a) + Bv * torch.sin(a)
        X = W0[:, :3] + f64(bImpact).reshape(n, 1) * bhat
        return torch.cat([X, V_par + V_perp], dim=1), bhat

    def get_subhalo_ImpactParams(self):
        """{'CartesianImpactParams': [n, 6], 'ImpactFrameParams': the sampled
        bImpact, tImpact, phi1_samples, perp_angle} (GenerateImpactParams.py:207-213)."""
        d = self.sample_impact_params()
        means, tstrip = self.get_particle_mean(d["phi1_samples"])
        xv, _ = self._get_subhalo_ImpactParamsCartesian(self.tobs, means, tstrip, d["tImpact"], d["bImpact"],
                                                        d["perp_angle"], np.arange(self.NumImpacts))
        return {"CartesianImpactParams": xv, "ImpactFrameParams": d}


__all__ = ["ImpactGenerator"]
