"""Differentiable streams: gradients of a loss on the final stream with
respect to the potential's parameters and the progenitor's present-day
phase-space point, by a hand-written adjoint.

The reference differentiates streams with forward-mode jax.jacfwd through
diffrax (main.py:160, examples/tests.ipynb:2959).  Here `StreamFn` is a
torch.autograd.Function:

  forward   progenitor back from the present day and forward again
            (FP64, parallel in time), release (FP64), FP32-compensated stream that
            stores its state every 64 steps (ss_stream_f32k_ckpt);
  backward  ss_stream_adjoint_f32 (discrete adjoint of every particle's
            steps, recomputing each 64-step segment from its checkpoint),
            ss_release_vjp (release map, including the tidal radius's
            dependence on the potential), ss_prog_tangents_f64 (progenitor
            sensitivities by forward-mode tangents of the parallel-in-time
            orbit, one lane per direction).

Parameters are raw component parameters (Potential_Combine leaves in order,
p[j] of each) plus the present-day state.  `TriaxialHaloModel` packs the
14 parameters of the halo / disk / bulge model used for fitting.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import List, Sequence, Tuple

import numpy as np
import torch

from . import _abi, _core
from ._core import f64, ptr, stream_handle
from .main import release_normals

CKPT = 64


@dataclass
class StreamSetup:
    """Fixed part of a differentiable stream: release grid and draws."""

    n_rel: int            # releases (the last release time, the observation, releases nothing)
    spr: int              # steps per release interval
    dt: float             # step [Myr]
    ppr: int              # particles per release (2 per draw)
    msat: float
    normals: np.ndarray   # [n_rel + 1, ppr // 2, 4]

    @property
    def n_steps(self) -> int:
        return self.n_rel * self.spr

    @property
    def t0(self) -> float:
        return -self.n_steps * self.dt


class TriaxialHaloModel:
    """TriaxialNFW(M, r_s, q3) + Miyamoto-Nagai(M, a, b) + Hernquist(M, c), and
    the progenitor's present-day state: theta = [M_h, rs_h, q_h, M_d, a_d,
    b_d, M_b, c_b, x, y, z, vx, vy, vz] (kpc, Myr, Msun)."""

    names = ["M_halo", "rs_halo", "q_halo", "M_disk", "a_disk", "b_disk", "M_bulge", "c_bulge",
             "x", "y", "z", "vx", "vy", "vz"]
    # (component, raw parameter index) of each potential parameter
    slots = [(0, 0), (0, 1), (0, 4), (1, 0), (1, 1), (1, 2), (2, 0), (2, 1)]
    n_comp = 3

    @staticmethod
    def components(theta: Sequence[float]):
        t = [float(v) for v in theta]
        return [(_abi.SS_TRIAXIAL_NFW, _abi.SS_CENTER_ORIGIN, (t[0], t[1], 1.0, 1.0, t[2])),
                (_abi.SS_MIYAMOTO_NAGAI, _abi.SS_CENTER_ORIGIN, (t[3], t[4], t[5])),
                (_abi.SS_HERNQUIST, _abi.SS_CENTER_ORIGIN, (t[6], t[7], 0.0))]

    @classmethod
    def struct(cls, theta):
        flat = _core.Flat(cls.components(theta))
        return _core.make_struct(flat, _core.G_KPC_MYR_MSUN)

    @classmethod
    def raw(cls, theta) -> np.ndarray:
        raw = np.zeros((cls.n_comp, 6))
        for c, (_, _, p) in enumerate(cls.components(theta)):
            raw[c, :len(p)] = p
        return raw


def _release_cfg(setup: StreamSetup, n_release: int):
    cfg = _abi.ss_release_cfg()
    cfg.n_release = n_release
    cfg.n_draw = setup.ppr // 2
    cfg.model = _abi.SS_RELEASE_FARDAL
    for i, k in enumerate((2.0, 0.3, 0.0, 0.0, 0.4, 0.4, 0.5, 0.5)):
        cfg.kvals[i] = k
    return cfg


def _stream_cfg(setup: StreamSetup):
    cfg = _abi.ss_stream_cfg()
    cfg.t0, cfg.dt, cfg.n_steps = setup.t0, setup.dt, setup.n_steps
    cfg.n_particles = setup.n_rel * setup.ppr
    cfg.particles_per_release, cfg.steps_per_release = setup.ppr, setup.spr
    return cfg


def forward_stream(model, theta: np.ndarray, setup: StreamSetup, keep=False):
    """FP32-compensated stream at theta; returns final [N, 6] (and the
    tensors the backward pass needs when keep=True)."""
    dev = _core.device()
    P = model.struct(theta)
    w_obs = f64(np.asarray(theta[-6:], dtype=np.float64).reshape(1, 6), dev)
    ob, starts_back = _core.orbit(P, w_obs, 0.0, -setup.dt, setup.n_steps, setup.n_steps, keep_starts=True)
    back = ob[:, -1].contiguous()
    of, starts_fwd = _core.orbit(P, back, setup.t0, setup.dt, setup.n_steps, setup.spr, keep_starts=True)
    ws = of[0]
    ts = setup.t0 + np.arange(setup.n_rel + 1) * setup.spr * setup.dt
    normals = f64(setup.normals, dev)
    rcfg = _release_cfg(setup, setup.n_rel + 1)
    msat = f64(np.full(setup.n_rel + 1, setup.msat), dev)
    t_rel = f64(ts, dev)
    ics, _ = _core.release(P, rcfg, ws, t_rel, msat, normals)
    cfg = _stream_cfg(setup)
    N = cfg.n_particles
    stream_ics = ics[:setup.n_rel].reshape(N, 6).contiguous()
    n_seg = (setup.n_steps + CKPT - 1) // CKPT + 1
    ckpt = torch.empty(n_seg * N * 12, dtype=torch.float32, device=dev)
    final = torch.empty(N, 6, dtype=torch.float64, device=dev)
    status = torch.empty(N, dtype=torch.int32, device=dev)
    _abi.call("ss_stream_f32k_ckpt", C.byref(P), C.byref(cfg), ptr(stream_ics), ptr(final), ptr(status),
              ptr(ckpt), CKPT, stream_handle())
    if not keep:
        return final
    return final, dict(P=P, ws=ws, t_rel=t_rel, msat=msat, normals=normals, ckpt=ckpt, cfg=cfg,
                       starts=(starts_back, starts_fwd))


def backward_stream(model, theta: np.ndarray, setup: StreamSetup, saved: dict, lam_final: torch.Tensor):
    """dL/dtheta from dL/d(final states) [N, 6]."""
    dev = lam_final.device
    P, cfg = saved["P"], saved["cfg"]
    N = cfg.n_particles
    ns = 6 * model.n_comp
    lam_final = lam_final.to(torch.float64).contiguous()
    lam_ic = torch.empty(N, 6, dtype=torch.float64, device=dev)
    g_slot = torch.zeros(ns, dtype=torch.float64, device=dev)
    _abi.call("ss_stream_adjoint_f32", C.byref(P), C.byref(cfg), ptr(saved["ckpt"]), CKPT, ptr(lam_final),
              ptr(lam_ic), ptr(g_slot), stream_handle())
    # release: states and draws of the releases that made particles
    n_rel = setup.n_rel
    rcfg = _release_cfg(setup, n_rel)
    raw = f64(model.raw(theta), dev)
    g_prog = torch.zeros(setup.n_rel + 1, 6, dtype=torch.float64, device=dev)
    _abi.call("ss_release_vjp", C.byref(P), C.byref(rcfg), ptr(saved["ws"]), ptr(saved["t_rel"]), ptr(saved["msat"]),
              ptr(saved["normals"]), ptr(lam_ic), ptr(raw), ptr(g_prog), ptr(g_slot), stream_handle())
    # progenitor: d(state at every release time)/d(parameters, present-day state)
    n_dir = ns + 6
    n_save = setup.n_rel + 1
    w_obs = f64(np.asarray(theta[-6:], dtype=np.float64), dev)
    states = torch.empty(n_save, 6, dtype=torch.float64, device=dev)
    tang = torch.empty(n_save, n_dir, 6, dtype=torch.float64, device=dev)
    need = _abi.load().ss_prog_tangents_workspace_bytes(int(setup.n_steps), int(model.n_comp))
    ws, nb = _core.aligned_ptr(_core.Workspace.get(int(need), dev, slot="tangents"))
    sb, sf = saved.get("starts", (None, None))
    if sb is None or sf is None:
        sb = sf = None
    _abi.call("ss_prog_tangents_f64", C.byref(P), ptr(raw), ptr(w_obs), float(setup.dt), int(setup.n_steps),
              int(setup.spr), ptr(states), ptr(tang), ptr(sb), ptr(sf), ws, nb, stream_handle())
    g_dir = torch.einsum("ri,rki->k", g_prog, tang)
    g_slot = g_slot + g_dir[:ns]
    g = torch.empty(len(theta), dtype=torch.float64, device=dev)
    for k, (c, j) in enumerate(model.slots):
        g[k] = g_slot[6 * c + j]
    g[len(model.slots):] = g_dir[ns:]
    return g


class StreamFn(torch.autograd.Function):
    """final states [N, 6] = StreamFn.apply(theta, model, setup); theta a
    float64 tensor of the model's parameters."""

    @staticmethod
    def forward(ctx, theta, model, setup):
        th = theta.detach().cpu().numpy().astype(np.float64)
        final, saved = forward_stream(model, th, setup, keep=True)
        ctx.model, ctx.setup, ctx.saved, ctx.theta = model, setup, saved, th
        return final

    @staticmethod
    def backward(ctx, grad_final):
        g = backward_stream(ctx.model, ctx.theta, ctx.setup, ctx.saved, grad_final)
        return g.to(grad_final.device), None, None


# ------------------------------------------------------------------ loss
SUN_X = np.array([-8.122, 0.0, 0.0208])          # kpc
SUN_V = np.array([0.01319, 0.25135, 0.00797])     # kpc/Myr


class TrackLoss:
    """Squared error of a binned mean stream track.

    Frame: the great circle through the reference progenitor's heliocentric
    position with the pole of its heliocentric angular momentum.  Per particle:
    phi1 (along-stream angle), phi2 (cross-track angle), heliocentric distance
    d and line-of-sight velocity v_los.  Bins: `n_bins` equal phi1 bins over
    the target's range.  Loss = sum over bins (occupied in both) of
    ((mean phi2 - target)/s_phi2)^2 + ((mean d - target)/s_d)^2 +
    ((mean v_los - target)/s_v)^2.  Bin membership is piecewise constant and
    carries no gradient."""

    def __init__(self, prog_w: np.ndarray, target_final: torch.Tensor, n_bins: int = 64,
                 scales=(0.01, 0.1, 0.001)):
        x = np.asarray(prog_w[:3]) - SUN_X
        v = np.asarray(prog_w[3:]) - SUN_V
        e1 = x / np.linalg.norm(x)
        e3 = np.cross(x, v)
        e3 /= np.linalg.norm(e3)
        e2 = np.cross(e3, e1)
        dev = target_final.device
        self.R = torch.tensor(np.stack([e1, e2, e3]), dtype=torch.float64, device=dev)
        self.sx = torch.tensor(SUN_X, dtype=torch.float64, device=dev)
        self.sv = torch.tensor(SUN_V, dtype=torch.float64, device=dev)
        self.scales = torch.tensor(scales, dtype=torch.float64, device=dev)
        phi1, obs = self.observables(target_final.detach())
        lo, hi = float(phi1.min()), float(phi1.max())
        self.edges = torch.linspace(lo, hi, n_bins + 1, dtype=torch.float64, device=dev)
        self.n_bins = n_bins
        self.target, self.target_count = self.binned(phi1, obs)

    def observables(self, final):
        xs = final[:, :3] - self.sx
        vs = final[:, 3:] - self.sv
        u = xs @ self.R.T
        d = torch.linalg.norm(xs, dim=1)
        phi1 = torch.atan2(u[:, 1], u[:, 0])
        phi2 = torch.asin(u[:, 2] / d)
        vlos = (xs * vs).sum(1) / d
        return phi1, torch.stack([phi2, d, vlos], dim=1)

    def binned(self, phi1, obs):
        b = torch.bucketize(phi1.detach(), self.edges[1:-1])
        cnt = torch.zeros(self.n_bins, dtype=torch.float64, device=obs.device).index_add_(
            0, b, torch.ones_like(phi1))
        s = torch.zeros(self.n_bins, 3, dtype=torch.float64, device=obs.device).index_add(0, b, obs)
        return s / cnt.clamp(min=1.0)[:, None], cnt

    def __call__(self, final):
        phi1, obs = self.observables(final)
        mean, cnt = self.binned(phi1, obs)
        ok = (cnt > 0) & (self.target_count > 0)
        r = (mean - self.target) / self.scales
        return (r[ok] ** 2).sum()


__all__ = ["StreamSetup", "TriaxialHaloModel", "StreamFn", "TrackLoss", "forward_stream", "backward_stream"]
