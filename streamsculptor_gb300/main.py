"""Potential base class and stream generation — the reference's main.py API.

Mirrors streamsculptor/main.py (jnibauer/streamsculptor): same class and
method names, keyword arguments and return shapes.  Differences, all forced
by running on a GB300 instead of JAX:
  * inputs may be single points ([3], [6]) or batches ([N,3], [N,6]) — the
    batch dimension replaces jax.vmap; outputs are CUDA torch tensors;
  * integration is fixed-step Dopri5 (step `dt`; default: the spacing of ts)
    instead of diffrax's adaptive controller; rtol/atol/max_steps are
    accepted and ignored; other solvers raise NotImplementedError;
  * the Gaussian draws of the release model come from numpy's PCG64 seeded
    with seed_num (or are passed in as `normals=`), not from the JAX PRNG;
  * dense outputs are replaced by strided snapshots (`snapshot_every=`).
Every compute call goes through the C ABI of libssgb300.so (no CPU path).
"""
from __future__ import annotations

import ctypes as C
import math
from typing import Optional

import numpy as np
import torch

from . import _abi, _core
from ._core import G_for, dimensionless, f64, host64, usys, UnitSystem  # noqa: F401

DEFAULT_KVALS = (2.0, 0.3, 0.0, 0.0, 0.4, 0.4, 0.5, 0.5)  # main.py:214


class Solution:
    """diffrax-like result: .ts [T] and .ys [..., T, 6]."""

    def __init__(self, ts, ys):
        self.ts = ts
        self.ys = ys

    def __repr__(self):
        return f"Solution(ts={tuple(self.ts.shape)}, ys={tuple(self.ys.shape)})"


def release_normals(seed_num: int, n_release: int, n_draw: int = 1, nz: int = 4) -> np.ndarray:
    """Gaussian draws of the release model, [n_release, n_draw, nz].

    Release i always gets the same numbers for a given (seed_num, n_draw, nz)
    whatever n_release is (row-major fill of one PCG64 stream)."""
    rng = np.random.Generator(np.random.PCG64(int(seed_num)))
    return rng.standard_normal((int(n_release), int(n_draw), int(nz)))


def _kvals(kval_arr) -> tuple:
    """release_model's kval_arr: scalar -> defaults (main.py:212-217)."""
    if np.isscalar(kval_arr) or np.ndim(kval_arr) == 0:
        return DEFAULT_KVALS
    k = np.broadcast_to(np.asarray(host64(kval_arr), dtype=np.float64), (8,))
    return tuple(float(x) for x in k)


def _points(x, width=3):
    t = f64(x)
    single = t.ndim == 1
    t = t.reshape(-1, width) if single else t
    if t.shape[-1] != width:
        raise ValueError(f"expected [..., {width}] input")
    return t.contiguous(), single


def _grid_spacing(ts_h: np.ndarray) -> Optional[float]:
    if len(ts_h) < 3:
        return None
    d = np.diff(np.sort(ts_h))
    if d[0] <= 0 or not np.allclose(d, d[0], rtol=1e-9, atol=1e-12):
        return None
    return float(d[0])


class Potential:
    """Base class (main.py:21-120).  Subclasses provide `_flatten()`."""

    def __init__(self, units, params):
        if units is None:
            units = dimensionless
        self.units = UnitSystem(units)
        self._G = G_for(self.units)
        for name, param in params.items():
            setattr(self, name, param)
        self._desc_cache = {}

    # ---------------------------------------------------------- model
    def _flatten(self) -> _core.Flat:
        raise NotImplementedError(f"{type(self).__name__} has no GPU implementation")

    def _desc(self):
        dev = _core.device()
        key = dev.index
        d = self._desc_cache.get(key)
        if d is None:
            flat = self._flatten()
            d = (_core.make_struct(flat, self._G), flat)
            self._desc_cache[key] = d
        return d[0]

    # ---------------------------------------------- potential & derivatives
    def _eval(self, xyz, t, phi=False, grad=False, hess=False):
        pts, single = _points(xyz)
        o = _core.potential_eval(self._desc(), pts, t, phi=phi, grad=grad, hess=hess)
        return o, single

    def potential(self, xyz, t):
        (phi, _, _), single = self._eval(xyz, t, phi=True)
        return phi[0] if single else phi

    def gradient(self, xyz, t):
        """main.py:37-40 (analytic gradient instead of jax.grad)."""
        (_, g, _), single = self._eval(xyz, t, grad=True)
        return g[0] if single else g

    def acceleration(self, xyz, t):
        return -self.gradient(xyz, t)

    def jacobian_force(self, xyz, t):
        """Jacobian of the gradient = Hessian of Phi (main.py:59-65)."""
        (_, _, H), single = self._eval(xyz, t, hess=True)
        return H[0] if single else H

    def density(self, xyz, t):
        """Laplacian / (4 pi G) (main.py:42-45)."""
        H = self.jacobian_force(xyz, t)
        return torch.diagonal(H, dim1=-2, dim2=-1).sum(-1) / (4 * math.pi * self._G)

    def local_circular_velocity(self, xyz, t):
        x = f64(xyz)
        r = torch.linalg.norm(x, dim=-1)
        g = self.gradient(x, t)
        return torch.sqrt(r * (g * x).sum(-1) / r)

    def dphidr(self, x, t):
        """main.py:67-74"""
        x = f64(x)
        r = torch.linalg.norm(x, dim=-1, keepdim=True)
        return (self.gradient(x, t) * x / r).sum(-1)

    def d2phidr2(self, x, t):
        """r_hat^T Hessian r_hat (main.py:76-85)."""
        x = f64(x)
        rh = x / torch.linalg.norm(x, dim=-1, keepdim=True)
        H = self.jacobian_force(x, t)
        return torch.einsum("...i,...ij,...j->...", rh, H, rh)

    def omega(self, x, v):
        """|x cross v| / r^2 (main.py:88-96)."""
        x, v = f64(x), f64(v)
        r2 = (x * x).sum(-1)
        return torch.linalg.norm(torch.linalg.cross(x, v, dim=-1), dim=-1) / r2

    def tidalr(self, x, v, Msat, t):
        """main.py:98-104"""
        return (self._G * f64(Msat) / (self.omega(x, v) ** 2 - self.d2phidr2(x, t))) ** (1.0 / 3.0)

    def lagrange_pts(self, x, v, Msat, t):
        """main.py:106-112"""
        x = f64(x)
        rt = self.tidalr(x, v, Msat, t)
        rh = x / torch.linalg.norm(x, dim=-1, keepdim=True)
        return x - rh * rt[..., None], x + rh * rt[..., None]

    def velocity_acceleration(self, t, xv, args=None):
        """Hamiltonian field (v, -grad Phi) (main.py:116-120)."""
        w, single = _points(xv, 6)
        a = -_core.potential_eval(self._desc(), w[:, :3].contiguous(), t, phi=False, grad=True)[1]
        out = torch.cat([w[:, 3:], a], dim=1)
        return out[0] if single else out

    # ---------------------------------------------------------- orbits
    def integrate_orbit(self, w0=None, ts=None, dense=False, solver=None, rtol=1e-7, atol=1e-7, dtmin=0.3,
                        dtmax=None, max_steps=10_000, t0=None, t1=None, steps=False, jump_ts=None, throw=False,
                        dt=None, method="auto"):
        """Fixed-step Dopri5 orbit(s) saved at ts (main.py:125-163).

        w0 [6] or [N,6]; returns Solution with ys [len(ts),6] or [N,len(ts),6].
        Integrates from t0 (default ts.min()) to t1 (default ts.max());
        every ts must lie on the step grid.  method: 'serial', 'shoot' (one
        orbit integrated parallel in time by multiple shooting, the serial
        FP64 orbit up to round-off, many times lower latency on GB300) or
        'auto' (shoot for a single long orbit in a static potential)."""
        if dense:
            raise NotImplementedError("dense output: use gen_stream_* with snapshot_every, or save at ts")
        if steps:
            raise NotImplementedError("SaveAt(steps=True) is not supported")
        _core.check_solver(solver)
        ts_h = host64(ts).reshape(-1)
        t_start = float(ts_h.min()) if t0 is None else float(host64(t0))
        t_end = float(ts_h.max()) if t1 is None else float(host64(t1))
        h, n = _core.fixed_step(t_end - t_start, dt=dt, grid=_grid_spacing(ts_h), dtmin=dtmin, dtmax=dtmax)
        idx = np.rint((ts_h - t_start) / h).astype(np.int64)
        if np.any(np.abs(t_start + idx * h - ts_h) > 1e-9 * max(1.0, abs(t_end - t_start))) or \
                np.any(idx < 0) or np.any(idx > n):
            raise ValueError("every ts must be on the fixed-step grid between t0 and t1; pass dt=")
        w, single = _points(w0, 6)
        out = _core.orbit(self._desc(), w, t_start, h, n, 1, method)
        ys = out[:, torch.as_tensor(idx, device=out.device)]
        if throw and not bool(torch.isfinite(ys).all()):
            raise RuntimeError("integrate_orbit: non-finite state")
        ts_t = torch.as_tensor(ts_h, device=out.device)
        return Solution(ts_t, ys[0] if single else ys)

    def integrate_orbit_batch_vmapped(self, w0=None, ts=None, **kw):
        """Batch of orbits, one GPU thread each (main.py:186-202)."""
        ts_h = host64(ts)
        if ts_h.ndim == 2:
            if not np.all(ts_h == ts_h[:1]):
                raise NotImplementedError("per-orbit save times must be identical")
            ts_h = ts_h[0]
        w = f64(w0).reshape(-1, 6)
        return self.integrate_orbit(w0=w, ts=ts_h, **kw)

    def integrate_orbit_batch_scan(self, w0=None, ts=None, **kw):
        """CPU-scan twin in the reference (main.py:166-183); same GPU batch here."""
        return self.integrate_orbit_batch_vmapped(w0=w0, ts=ts, **kw)

    # ------------------------------------------------------- release
    def _release(self, prog_w, t_rel, Msat, normals, kval_arr=1.0, model=_abi.SS_RELEASE_FARDAL, chen=None,
                 jac=False):
        prog_w = f64(prog_w).reshape(-1, 6)
        n_rel = prog_w.shape[0]
        normals = f64(normals)
        nz = 6 if model == _abi.SS_RELEASE_CHEN25 else 4
        normals = normals.reshape(n_rel, -1, nz)
        cfg = _abi.ss_release_cfg()
        cfg.n_release = n_rel
        cfg.n_draw = normals.shape[1]
        cfg.model = model
        for i, k in enumerate(_kvals(kval_arr)):
            cfg.kvals[i] = k
        if chen is not None:
            mean, L = chen
            for i in range(6):
                cfg.chen_mean[i] = float(mean[i])
                for j in range(6):
                    cfg.chen_L[6 * i + j] = float(L[i, j])
        msat = f64(torch.as_tensor(host64(Msat)).expand(n_rel).clone() if np.ndim(host64(Msat)) == 0
                   else host64(Msat))
        return _core.release(self._desc(), cfg, prog_w, f64(t_rel).reshape(-1), msat, normals, jac=jac)

    def release_model(self, x=None, v=None, Msat=None, i=None, t=None, seed_num=None, kval_arr=1.0,
                      normals=None):
        """Fardal-style particle spray at one release (main.py:209-280).

        Returns (pos_lead, pos_trail, v_lead, v_trail).  The four draws are
        release_normals(seed_num, i+1)[i] unless `normals` is given."""
        if normals is None:
            normals = release_normals(seed_num, int(i) + 1, 1, 4)[int(i)]
        w = torch.cat([f64(x).reshape(1, 3), f64(v).reshape(1, 3)], dim=1)
        ics, _ = self._release(w, [float(host64(t))], Msat, np.asarray(host64(normals)).reshape(1, 1, 4), kval_arr)
        o = ics[0, 0]
        return o[0, :3], o[1, :3], o[0, 3:], o[1, 3:]

    def _prog_orbit(self, ts_h, prog_w0, dt, dtmin=None, dtmax=None, method="auto"):
        grid = _grid_spacing(ts_h)
        if grid is None:
            raise NotImplementedError("release times ts must be uniformly spaced")
        if ts_h[1] < ts_h[0]:
            raise NotImplementedError("release times ts must increase")
        h, spr = _core.fixed_step(grid, dt=dt if dt is not None else grid, dtmax=dtmax)
        w0 = f64(prog_w0).reshape(1, 6)
        ws = _core.orbit(self._desc(), w0, float(ts_h[0]), h, spr * (len(ts_h) - 1), spr, method)[0]
        return ws, h, spr

    def gen_stream_ics(self, ts=None, prog_w0=None, Msat=None, seed_num=None, solver=None, kval_arr=1.0,
                       rtol=1e-7, atol=1e-7, dtmin=0.3, dtmax=None, max_steps=10_000, *, dt=None,
                       n_particles_per_release=2, normals=None):
        """Progenitor orbit at ts + release model at every ts (main.py:287-306).

        Returns (pos_close, pos_far, vel_close, vel_far), each [len(ts), 3]
        ([len(ts), n_draw, 3] when n_particles_per_release > 2)."""
        _core.check_solver(solver)
        ts_h = host64(ts).reshape(-1)
        ws, _, _ = self._prog_orbit(ts_h, prog_w0, dt, dtmin, dtmax)
        n_draw = _n_draw(n_particles_per_release)
        if normals is None:
            normals = release_normals(seed_num, len(ts_h), n_draw, 4)
        ics, _ = self._release(ws, ts_h, Msat, normals, kval_arr)
        return _split_ics(ics, n_draw)

    def gen_stream_vmapped(self, ts=None, prog_w0=None, Msat=None, seed_num=None, solver=None, kval_arr=1.0,
                           rtol=1e-7, atol=1e-7, dtmin=0.3, dtmax=None, max_steps=10_000, throw=False, *, dt=None,
                           n_particles_per_release=2, normals=None, precision="f64", snapshot_every=None):
        """Stream: every particle from its release ts[i] to ts[-1] (main.py:343-368).

        Returns (lead, trail), each [len(ts)-1, 6]; with snapshot_every=k also
        the float32 snapshots [n_steps//k, len(ts)-1, n_draw, 2, 6]."""
        from .streamhelpers import gen_stream
        return gen_stream(self, ts=ts, prog_w0=prog_w0, Msat=Msat, seed_num=seed_num, solver=solver,
                          kval_arr=kval_arr, dt=dt, dtmax=dtmax, n_particles_per_release=n_particles_per_release,
                          normals=normals, precision=precision, snapshot_every=snapshot_every, throw=throw)

    def gen_stream_scan(self, *args, **kw):
        """CPU-scan twin in the reference (main.py:312-340); same GPU kernel."""
        return self.gen_stream_vmapped(*args, **kw)

    def gen_stream_vmapped_dense(self, *args, **kw):
        raise NotImplementedError("dense stream interpolants are replaced by snapshots: "
                                  "gen_stream_vmapped(..., snapshot_every=k)")

    gen_stream_scan_dense = gen_stream_vmapped_dense


def _n_draw(n_particles_per_release: int) -> int:
    n = int(n_particles_per_release)
    if n < 2 or n % 2:
        raise ValueError("n_particles_per_release must be even (each draw releases a lead and a trail star)")
    return n // 2


def _split_ics(ics: torch.Tensor, n_draw: int):
    """[n_rel, n_draw, 2, 6] -> (pos_close, pos_far, vel_close, vel_far)."""
    if n_draw == 1:
        ics = ics[:, 0]
        return ics[:, 0, :3], ics[:, 1, :3], ics[:, 0, 3:], ics[:, 1, 3:]
    return ics[:, :, 0, :3], ics[:, :, 1, :3], ics[:, :, 0, 3:], ics[:, :, 1, 3:]


__all__ = ["Potential", "Solution", "UnitSystem", "usys", "dimensionless", "release_normals", "DEFAULT_KVALS"]
