"""ctypes wrapper of the CPU FP64 oracle (oracle/ss_oracle.cpp).

TEST INFRASTRUCTURE ONLY: used by tests/, the smoke check and the benchmark's
CPU-baseline leg as the checker; the product never imports it.  Arrays are
numpy float64; descriptors use host pointers.
"""
from __future__ import annotations

import ctypes as C
import os
import sys
from dataclasses import dataclass, field
from typing import List, Optional, Sequence, Tuple

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

from streamsculptor_gb300 import _abi  # noqa: E402  (ABI struct layout only)

from . import build_oracle  # noqa: E402

G_KPC = 4.498502151469553e-12

VP = C.c_void_p


def _p(a: Optional[np.ndarray]):
    return None if a is None else C.c_void_p(a.ctypes.data)


_SIG = {
    "or_abi_version": (C.c_int, []),
    "or_abi_sizeof": (C.c_int64, [C.c_int]),
    "or_track_slopes": (None, [VP, C.c_int64, C.c_double, VP]),
    "or_track_eval": (None, [C.POINTER(_abi.ss_potential), VP, C.c_int64, VP]),
    "or_potential_eval": (None, [C.POINTER(_abi.ss_potential), VP, C.c_int64, VP, C.c_double, VP, VP, VP]),
    "or_gradient": (None, [C.POINTER(_abi.ss_potential), VP, C.c_int64, C.c_double, VP]),
    "or_orbit": (None, [C.POINTER(_abi.ss_potential), VP, C.c_int64, C.c_double, C.c_double, C.c_int64,
                        C.c_int64, VP]),
    "or_release": (None, [C.POINTER(_abi.ss_potential), C.POINTER(_abi.ss_release_cfg), VP, VP, VP, VP, VP, VP]),
    "or_stream": (None, [C.POINTER(_abi.ss_potential), C.POINTER(_abi.ss_stream_cfg), VP, VP, VP, VP, C.c_int]),
    "or_subhalo_eval": (None, [C.POINTER(_abi.ss_subhalos), C.c_double, VP, C.c_int64, C.c_double, VP, VP, VP, VP]),
    "or_pert_term": (None, [C.POINTER(_abi.ss_potential), C.POINTER(_abi.ss_subhalos), C.c_int, C.c_double, VP, VP]),
    "or_pert_response": (None, [C.POINTER(_abi.ss_potential), C.POINTER(_abi.ss_subhalos),
                                C.POINTER(_abi.ss_pert_cfg), VP, VP, VP, VP]),
    "or_binned_sums": (None, [VP, VP, C.c_int64, C.c_int32, VP, C.c_int32, VP, VP]),
}

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = build_oracle.build()
        L = C.CDLL(path)
        for k, (r, a) in _SIG.items():
            f = getattr(L, k)
            f.restype = r
            f.argtypes = a
        _lib = L
    return _lib


def f8(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64))


# ------------------------------------------------------------- models
@dataclass
class HostModel:
    """A flattened potential on the host: components (kind, center, params),
    optional center track knots at t0 + k dt, optional subhalo table."""

    comps: List[Tuple[int, int, Sequence[float]]]
    G: float = G_KPC
    track: Optional[tuple] = None  # (t0, dt, knots [n,3]) or (t0, dt, knots, "linear")
    subhalos: Optional[dict] = None  # kind, m, a, x0, v, t0, t_window
    expansion: Optional[tuple] = None  # (l_max, log_r0, dlog_r, coef [n_knots, (l_max+1)^2, 2])
    frame_velocity: Optional[tuple] = None  # (t0, dt, velocities [n,3]) or (..., "linear")
    growth: Optional[tuple] = None  # (t0, dt, g [n]) or (..., "linear"): the SS_GROWS components' factor
    _keep: list = field(default_factory=list)

    def _track(self, spec) -> _abi.ss_track:
        t0, dt, knots = spec[:3]
        linear = len(spec) > 3 and spec[3] == "linear"
        knots = f8(knots)
        slopes = track_slopes(knots, dt)
        self._keep += [knots, slopes]
        tr = _abi.ss_track()
        tr.knots, tr.slopes = knots.ctypes.data, slopes.ctypes.data
        tr.t0, tr.dt, tr.n_knots, tr.linear = t0, dt, knots.shape[0], int(linear)
        return tr

    def struct(self) -> _abi.ss_potential:
        P = _abi.ss_potential()
        P.G = self.G
        P.n_components = len(self.comps)
        for i, (kind, center, params) in enumerate(self.comps):
            P.comp[i].kind = kind
            P.comp[i].center = center
            for j, v in enumerate(params):
                P.comp[i].p[j] = float(v)
        if self.track is not None:
            P.track = self._track(self.track)
        if self.frame_velocity is not None:
            P.frame_velocity = self._track(self.frame_velocity)
        if self.growth is not None:
            g = f8(self.growth[2]).reshape(-1)
            P.growth = self._track((self.growth[0], self.growth[1], np.stack([g, 0 * g, 0 * g], 1)) +
                                   tuple(self.growth[3:]))
        if self.subhalos is not None:
            P.subhalos = self.sh_struct()
        if self.expansion is not None:
            l_max, log_r0, dlog_r, coef = self.expansion
            coef = f8(coef)
            self._keep.append(coef)
            P.expansion.l_max = int(l_max)
            P.expansion.n_knots = coef.shape[0]
            P.expansion.log_r0 = float(log_r0)
            P.expansion.dlog_r = float(dlog_r)
            P.expansion.coef = coef.ctypes.data
        return P

    def sh_struct(self) -> _abi.ss_subhalos:
        s = self.subhalos
        arrs = {k: f8(s[k]) for k in ("m", "a", "x0", "v", "t0")}
        self._keep += list(arrs.values())
        S = _abi.ss_subhalos()
        S.kind = int(s.get("kind", _abi.SS_SH_PLUMMER))
        S.n = arrs["m"].shape[0]
        S.m, S.a, S.x0, S.v, S.t0 = (arrs[k].ctypes.data for k in ("m", "a", "x0", "v", "t0"))
        S.t_window = float(s.get("t_window", np.inf))
        if "grid" in s:  # SS_SH_GRID: [n, n_grid, 2] tables, u0 [n], du [n]
            g, u0, du = f8(s["grid"]), f8(s["grid_u0"]), f8(s["grid_du"])
            self._keep += [g, u0, du]
            S.grid, S.grid_u0, S.grid_du, S.n_grid = g.ctypes.data, u0.ctypes.data, du.ctypes.data, g.shape[1]
        return S


def mw3(G=G_KPC):
    """NFW + Miyamoto-Nagai + Hernquist: the stream workloads' potential."""
    return [(_abi.SS_NFW, 0, (5.4e11, 15.62, 0.0)),
            (_abi.SS_MIYAMOTO_NAGAI, 0, (6.8e10, 3.0, 0.28)),
            (_abi.SS_HERNQUIST, 0, (5e9, 1.0, 0.0))]


# ------------------------------------------------------------- calls
def track_slopes(knots, dt) -> np.ndarray:
    knots = f8(knots)
    out = np.empty_like(knots)
    lib().or_track_slopes(_p(knots), knots.shape[0], float(dt), _p(out))
    return out


def potential_eval(model: HostModel, xyz, t=0.0):
    P = model.struct()
    x = f8(xyz).reshape(-1, 3)
    n = x.shape[0]
    tt = None
    ts = 0.0
    if np.ndim(t) > 0:
        tt = f8(t).reshape(-1)
    else:
        ts = float(t)
    phi = np.empty(n)
    g = np.empty((n, 3))
    H = np.empty((n, 3, 3))
    lib().or_potential_eval(C.byref(P), _p(x), n, _p(tt), ts, _p(phi), _p(g), _p(H))
    return phi, g, H


def orbit(model: HostModel, w0, t0, dt, n_steps, save_every=1):
    P = model.struct()
    w = f8(w0).reshape(-1, 6)
    out = np.empty((w.shape[0], n_steps // save_every + 1, 6))
    lib().or_orbit(C.byref(P), _p(w), w.shape[0], float(t0), float(dt), int(n_steps), int(save_every), _p(out))
    return out


def release(model: HostModel, prog_w, t_rel, msat, normals, kvals=(2.0, 0.3, 0.0, 0.0, 0.4, 0.4, 0.5, 0.5),
            model_kind=0, chen=None, jac=False):
    P = model.struct()
    prog_w = f8(prog_w).reshape(-1, 6)
    n_rel = prog_w.shape[0]
    nz = 6 if model_kind == 1 else 4
    normals = f8(normals).reshape(n_rel, -1, nz)
    cfg = _abi.ss_release_cfg()
    cfg.n_release = n_rel
    cfg.n_draw = normals.shape[1]
    cfg.model = model_kind
    for i, k in enumerate(kvals):
        cfg.kvals[i] = k
    if chen is not None:
        mean, L = chen
        for i in range(6):
            cfg.chen_mean[i] = mean[i]
            for j in range(6):
                cfg.chen_L[6 * i + j] = L[i, j]
    t_rel = f8(t_rel).reshape(-1)
    msat = f8(np.broadcast_to(np.asarray(msat, dtype=np.float64), (n_rel,)))
    ics = np.empty((n_rel, cfg.n_draw, 2, 6))
    J = np.empty((n_rel, cfg.n_draw, 2, 6, 6)) if jac else None
    lib().or_release(C.byref(P), C.byref(cfg), _p(prog_w), _p(t_rel), _p(msat), _p(normals), _p(ics), _p(J))
    return ics, J


def streakline_ics(model: HostModel, prog_w, t_rel, msat):
    """Streakline release (get_Streakline_ICs, streamhelpers.py:657-705) on
    the oracle: Lagrange points x -/+ r_t x / |x| with the tidal radius
    r_t = (G M / (omega^2 - r^T H r / r^2))^(1/3) (main.py:88-112, H the
    oracle's autodiff Hessian), velocities along v / |v| with magnitude
    omega |x_L| / sin(theta).  Returns [n, 2, 6]: (close, far) per release."""
    w = f8(prog_w).reshape(-1, 6)
    x, v = w[:, :3], w[:, 3:]
    _, _, H = potential_eval(model, x, f8(t_rel).reshape(-1))
    r = np.linalg.norm(x, axis=1)
    rh = x / r[:, None]
    d2 = np.einsum("ni,nij,nj->n", rh, H, rh)
    om = np.linalg.norm(np.cross(x, v), axis=1) / r ** 2
    rt = (model.G * float(msat) / (om ** 2 - d2)) ** (1.0 / 3.0)
    ph = v / np.linalg.norm(v, axis=1)[:, None]
    sin_t = np.linalg.norm(np.cross(rh, ph), axis=1)
    out = np.empty((w.shape[0], 2, 6))
    for k, sgn in enumerate((-1.0, 1.0)):
        xl = x + sgn * rh * rt[:, None]
        out[:, k, :3] = xl
        out[:, k, 3:] = (om * np.linalg.norm(xl, axis=1) / sin_t)[:, None] * ph
    return out


def stream(model: HostModel, t0, dt, n_steps, ics, ppr, spr, snap_stride=0, n_threads=0, stream_particles=0,
           subhalos_per_stream=0, first_particle=0):
    P = model.struct()
    ics = f8(ics).reshape(-1, 6)
    cfg = _abi.ss_stream_cfg()
    cfg.t0, cfg.dt, cfg.n_steps, cfg.n_particles = float(t0), float(dt), int(n_steps), ics.shape[0]
    cfg.particles_per_release, cfg.steps_per_release, cfg.snap_stride = int(ppr), int(spr), int(snap_stride)
    cfg.stream_particles, cfg.subhalos_per_stream = int(stream_particles), int(subhalos_per_stream)
    cfg.first_particle = int(first_particle)  # ics are particles first_particle.. of the stream
    final = np.empty_like(ics)
    status = np.empty(ics.shape[0], dtype=np.int32)
    snaps = None
    if snap_stride:
        snaps = np.empty((n_steps // snap_stride, ics.shape[0], 6), dtype=np.float32)
    lib().or_stream(C.byref(P), C.byref(cfg), _p(ics), _p(final), _p(snaps), _p(status), int(n_threads))
    return final, snaps, status


def subhalo_eval(model: HostModel, xyz, t):
    S = model.sh_struct()
    x = f8(xyz).reshape(-1, 3)
    n, ns = x.shape[0], S.n
    phi = np.empty((n, ns))
    g = np.empty((n, ns, 3))
    d = np.empty((n, ns))
    gd = np.empty((n, ns, 3))
    lib().or_subhalo_eval(C.byref(S), model.G, _p(x), n, float(t), _p(phi), _p(g), _p(d), _p(gd))
    return phi, g, d, gd


def pert_term(model: HostModel, t, x0v0, derivs, ncol=12):
    P = model.struct()
    P.subhalos = _abi.ss_subhalos()
    S = model.sh_struct()
    y = f8(np.concatenate([np.asarray(x0v0, dtype=np.float64).ravel(), np.asarray(derivs).ravel()]))
    dy = np.empty_like(y)
    lib().or_pert_term(C.byref(P), C.byref(S), int(ncol), float(t), _p(y), _p(dy))
    return dy[:6], dy[6:].reshape(S.n, ncol)


def pert_response(model: HostModel, t0, dt, n_steps, base_ics, pert_ics, ppr, spr, ncol=12, save_stride=0):
    P = model.struct()
    P.subhalos = _abi.ss_subhalos()
    S = model.sh_struct()
    base = f8(base_ics).reshape(-1, 6)
    N = base.shape[0]
    pert = None if pert_ics is None else f8(pert_ics).reshape(N, S.n, ncol)
    cfg = _abi.ss_pert_cfg()
    cfg.t0, cfg.dt, cfg.n_steps, cfg.n_particles = float(t0), float(dt), int(n_steps), N
    cfg.particles_per_release, cfg.steps_per_release = int(ppr), int(spr)
    cfg.ncol, cfg.save_stride = int(ncol), int(save_stride)
    n_saves = n_steps // save_stride + 1 if save_stride else 1
    out = np.empty((n_saves, N, S.n, ncol))
    base_out = np.empty((N, 6))
    lib().or_pert_response(C.byref(P), C.byref(S), C.byref(cfg), _p(base), _p(pert), _p(base_out), _p(out))
    return base_out, out


def binned_sums(values, key, edges):
    v = f8(values)
    k = f8(key).reshape(-1)
    e = f8(edges).reshape(-1)
    n, nc = v.shape
    sums = np.empty((e.shape[0] - 1, nc))
    counts = np.empty_like(sums)
    lib().or_binned_sums(_p(v), _p(k), n, nc, _p(e), e.shape[0], _p(sums), _p(counts))
    return sums, counts


def mn3_components(m, h_R, h_z, positive_density=True, sech2_z=True):
    """The three Miyamoto-Nagai components of MN3ExponentialDiskPotential
    (reference potential.py:224-280): masses and scale lengths K x (b^4 ..
    1) from the published coefficient table (Smith et al. 2015, Table 1, as
    the reference holds it at potential.py:226-241), b = b_MN / h_R from the
    cubic fit in h_z / h_R; all three share b_MN."""
    Kp = [[0.0036, -0.0330, 0.1117, -0.1335, 0.1749], [-0.0131, 0.1090, -0.3035, 0.2921, -5.7976],
          [-0.0048, 0.0454, -0.1425, 0.1012, 6.7120], [-0.0158, 0.0993, -0.2070, -0.7089, 0.6445],
          [-0.0319, 0.1514, -0.1279, -0.9325, 2.6836], [-0.0326, 0.1816, -0.2943, -0.6329, 2.3193]]
    Kn = [[-0.0090, 0.0640, -0.1653, 0.1164, 1.9487], [0.0173, -0.0903, 0.0877, 0.2029, -1.3077],
          [-0.0051, 0.0287, -0.0361, -0.0544, 0.2242], [-0.0358, 0.2610, -0.6987, -0.1193, 2.0074],
          [-0.0830, 0.4992, -0.7967, -1.2966, 4.4441], [-0.0247, 0.1718, -0.4124, -0.5944, 0.7333]]
    K = np.array(Kp if positive_density else Kn)
    q = h_z / h_R
    b = (-0.033 * q ** 3 + 0.262 * q ** 2 + 0.659 * q) if sech2_z else (-0.269 * q ** 3 + 1.08 * q ** 2 + 1.092 * q)
    pv = K.dot(np.array([b ** 4, b ** 3, b ** 2, b, 1.0]))
    return [(_abi.SS_MIYAMOTO_NAGAI, 0, (pv[i] * m, pv[3 + i] * h_R, b * h_R)) for i in range(3)]
