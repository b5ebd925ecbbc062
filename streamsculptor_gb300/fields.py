"""Vector fields and their integrator — the reference's fields.py API.

Supported fields (jnibauer/streamsculptor fields.py): hamiltonian_field
(101-113), MassRadiusPerturbation_OTF (159-206), MassRadiusPerturbation_Interp
(208-257) and MassRadiusPerturbation_OTF_SecondOrder (260-320).  `term` evaluates the
field on the GPU; `integrate_field` (35-99) dispatches to the fixed-step
Dopri5 kernels (ss_orbit_f64 / ss_pert_response).  Other fields (N-body,
MW-LMC, custom Python callables) have no GPU implementation and raise.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _abi, _core
from ._core import f64, host64
from .main import Solution, _grid_spacing


class hamiltonian_field:
    """(x, v) -> (v, -grad Phi)  (fields.py:101-113)."""

    def __init__(self, pot):
        self.pot = pot

    def term(self, t, xv, args=None):
        return self.pot.velocity_acceleration(t, xv, args)


class MassRadiusPerturbation_OTF:
    """First-order mass/radius response field (fields.py:159-206).

    coords = [x0v0 (6), derivs (N_sh, 12)]; term returns the same pytree."""

    def __init__(self, perturbation_generator):
        self.pertgen = perturbation_generator

    def term(self, t, coords, args=None):
        g = self.pertgen
        x0v0 = f64(coords[0]).reshape(6)
        d = f64(coords[1])
        x0 = x0v0[:3].reshape(1, 3).contiguous()
        _, grad, H = _core.potential_eval(g.potential_base._desc(), x0, float(host64(t)), phi=False, grad=True,
                                          hess=True)
        T = -H[0]
        _, gphi, _, gdphi = _core.subhalo_eval(g.sh_table, g.potential_base._G, x0, float(host64(t)))
        a1 = -gphi[0]
        a1r = -gdphi[0]
        out0 = torch.cat([x0v0[3:], -grad[0]])
        x1, v1, dx1, dv1 = d[:, 0:3], d[:, 3:6], d[:, 6:9], d[:, 9:12]
        dp = a1 + x1 @ T.T
        dpr = a1r + dx1 @ T.T
        return [out0, torch.cat([v1, dp, dv1, dpr], dim=1)]


class MassRadiusPerturbation_Interp(MassRadiusPerturbation_OTF):
    """The response field along the stored base stream (fields.py:208-257):
    coords = derivs [N_sh, 12]; args = {'idx': release index, 'tail_bool':
    True for the leading arm}.  The base state at t is the particle's fixed-
    step FP64 orbit from its release (the reference interpolates its dense
    base stream there)."""

    def term(self, t, coords, args):
        g = self.pertgen
        b = g.base_stream
        idx, lead = int(args["idx"]), bool(args["tail_bool"])
        ics = g.base_realspace_ICs_lead if lead else g.base_realspace_ICs_trail
        t_rel, t = float(b._ts_h[idx]), float(host64(t))
        h, nst = _core.fixed_step(t - t_rel, b._h)
        w = f64(ics[idx]).reshape(1, 6)
        if nst > 0:
            w = _core.orbit(g.potential_base._desc(), w, t_rel, h, nst, nst)[:, -1]
        return super().term(t, [w.reshape(6), coords], args)[1]


class MassRadiusPerturbation_OTF_SecondOrder:
    """Second order in subhalo mass with the first-order radius response
    (fields.py:260-320).  coords = [x0v0 (6), first (N_sh, 12), second
    (N_sh, 6)]; term returns the same pytree:
      d(x2)/dt = v2,  d(v2)/dt = T x2 + (d2a/dx2 : x1 x1) + dapert/dx x1,
    with dapert/dx = -Hessian of each subhalo's potential, as the reference
    writes it.  Evaluated on the GPU by ss_pert_term (FP64, third
    derivatives of the base potential by forward-mode differentiation of its
    analytic Hessian)."""

    def __init__(self, perturbation_generator):
        self.pertgen = perturbation_generator
        self.potential_base = perturbation_generator.potential_base

    def term(self, t, coords, args=None):
        g = self.pertgen
        x0v0 = f64(coords[0]).reshape(6)
        ns = int(g.sh_table.m.shape[0])
        d = torch.cat([f64(coords[1]).reshape(ns, 12), f64(coords[2]).reshape(ns, 6)], dim=1)
        y = torch.cat([x0v0, d.reshape(-1)])
        dy = _core.pert_term(g.potential_base._desc(), g.sh_table, 18, float(host64(t)), y)
        r = dy[6:].reshape(ns, 18)
        return [dy[:6], r[:, :12], r[:, 12:]]


def _t_span(ts_h, backwards_int, t0, t1):
    """t0/t1 selection of integrate_field (fields.py:58-80)."""
    if float(t0) != float(t1):
        return float(t0), float(t1)
    if backwards_int:
        return float(ts_h.max()), float(ts_h.min())
    return float(ts_h.min()), float(ts_h.max())


def integrate_field(w0=None, ts=None, dense=False, solver=None, field=None, args=None, rtol=1e-7, atol=1e-7,
                    dtmin=0.05, dtmax=None, max_steps=1_000, jump_ts=None, backwards_int=False, t0=0.0, t1=0.0,
                    step_ts=None, *, dt=None, precision=64):
    """Integrate `field` from w0, saving at ts (fields.py:35-99), fixed-step Dopri5."""
    if dense:
        raise NotImplementedError("dense output is not supported; save at ts")
    _core.check_solver(solver)
    ts_h = host64(ts).reshape(-1)
    ta, tb = _t_span(ts_h, backwards_int, t0, t1)
    h, n = _core.fixed_step(tb - ta, dt=dt, grid=_grid_spacing(ts_h), dtmin=dtmin, dtmax=dtmax)
    idx = np.rint((ts_h - ta) / h).astype(np.int64)
    if np.any(np.abs(ta + idx * h - ts_h) > 1e-9 * max(1.0, abs(tb - ta))) or np.any(idx < 0) or np.any(idx > n):
        raise ValueError("every ts must be on the fixed-step grid; pass dt=")
    if isinstance(field, hamiltonian_field):
        w = f64(w0)
        single = w.ndim == 1
        out = _core.orbit(field.pot._desc(), w.reshape(-1, 6).contiguous(), ta, h, n, 1)
        ys = out[:, torch.as_tensor(idx, device=out.device)]
        return Solution(torch.as_tensor(ts_h, device=ys.device), ys[0] if single else ys)
    if isinstance(field, (MassRadiusPerturbation_OTF, MassRadiusPerturbation_OTF_SecondOrder)):
        g = field.pertgen
        base = f64(w0[0]).reshape(-1, 6).contiguous()
        second = isinstance(field, MassRadiusPerturbation_OTF_SecondOrder)
        pert = f64(w0[1])
        single = pert.ndim == 2
        N = base.shape[0]
        ns = int(g.sh_table.m.shape[0])
        pert = pert.reshape(N, ns, -1)
        if second:
            pert = torch.cat([pert, f64(w0[2]).reshape(N, ns, 6)], dim=2).contiguous()
        cfg = _abi.ss_pert_cfg()
        cfg.t0, cfg.dt, cfg.n_steps, cfg.n_particles = ta, h, n, N
        cfg.particles_per_release, cfg.steps_per_release = 1, 0
        cfg.ncol = pert.shape[2]
        cfg.save_stride = 1
        _, out = _core.pert_response(g.potential_base._desc(), g.sh_table, cfg, int(precision), base, pert)
        pys = out[torch.as_tensor(idx, device=out.device)]  # [len(ts), N, ns, ncol]
        bys = _core.orbit(g.potential_base._desc(), base, ta, h, n, 1)[:, torch.as_tensor(idx, device=out.device)]
        pys = pys[:, 0] if single else pys.transpose(0, 1)
        parts = [pys[..., :12], pys[..., 12:]] if second else [pys]
        return Solution(torch.as_tensor(ts_h, device=out.device), [bys[0] if single else bys] + parts)
    raise NotImplementedError(f"field {type(field).__name__} has no GPU implementation")


class CustomField:
    """Arbitrary Python vector field (fields.py:362-378): no GPU implementation."""

    def __init__(self, term):
        self.term = term


__all__ = ["integrate_field", "hamiltonian_field", "MassRadiusPerturbation_OTF", "MassRadiusPerturbation_Interp",
           "MassRadiusPerturbation_OTF_SecondOrder", "CustomField"]
