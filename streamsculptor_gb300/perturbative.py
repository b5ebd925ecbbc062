"""Perturbation generators — the reference's perturbative.py API.

BaseStreamModel (perturbative.py:243-296) holds the zeroth-order stream:
release ICs, the forward progenitor orbit and the release Jacobians
d(release)/d(progenitor w) (computed by forward-mode dual numbers on the GPU,
including the third derivatives of Phi that r_t needs).
GenerateMassRadiusPerturbation (perturbative.py:24-135) integrates the
progenitor's response backwards from the observation time, maps it through
the release Jacobians to per-particle initial responses and integrates every
(particle, subhalo) response forward with ss_pert_response.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _abi, _core
from ._core import f64, host64
from .main import Potential, _grid_spacing, release_normals


class BaseStreamModel(Potential):
    def __init__(self, potential_base, prog_w0, ts, Msat, seednum, solver=None, units=None, dense=False, cpu=True,
                 *, dt=None, normals=None, **kwargs):
        super().__init__(units, {"potential_base": potential_base, "prog_w0": prog_w0, "ts": ts, "Msat": Msat,
                                 "seednum": seednum, "solver": solver, "dense": dense, "cpu": cpu})
        if dense:
            raise NotImplementedError("dense stream interpolants are replaced by snapshots")
        _core.check_solver(solver)
        self.potential_base = potential_base
        ts_h = host64(ts).reshape(-1)
        self._ts_h = ts_h
        self._dt = dt
        self.normals = normals if normals is not None else release_normals(seednum, len(ts_h), 1, 4)
        ws, self._h, self._spr = potential_base._prog_orbit(ts_h, prog_w0, dt)
        self.prog_loc_fwd = ws  # [len(ts), 6]
        ics, J = potential_base._release(ws, ts_h, Msat, self.normals, jac=True)
        ics = ics[:, 0]
        self.streamICs = (ics[:, 0, :3], ics[:, 1, :3], ics[:, 0, 3:], ics[:, 1, 3:])
        self.IDs = torch.arange(len(ts_h), device=ws.device)
        self.dRel_dIC = J[:, 0]  # [len(ts), 2, 6, 6]
        self.stream_interp = None

    def release_func_jacobian(self):
        """[len(ts), 2, 6, 6]: d(lead/trail ICs)/d(progenitor w) (perturbative.py:280-296)."""
        return self.dRel_dIC


class GenerateMassRadiusPerturbation(Potential):
    """First-order response in subhalo mass and scale radius (perturbative.py:24-135)."""

    _ncol = 12

    def __init__(self, potential_base, potential_perturbation, potential_structural=None, BaseStreamModel=None,
                 units=None, *, precision=64, **kwargs):
        super().__init__(units, {"potential_base": potential_base, "potential_perturbation": potential_perturbation,
                                 "potential_structural": potential_structural, "BaseStreamModel": BaseStreamModel})
        self.potential_base = potential_base
        self.gradientPotentialBase = potential_base.gradient
        self.gradientPotentialPerturbation_per_SH = potential_perturbation.gradient_per_SH
        self.sh_table = potential_perturbation.table()
        if potential_structural is not None:
            self.gradientPotentialStructural_per_SH = potential_structural.gradient_per_SH
            if not self.sh_table.same_lines(potential_structural.table()):
                raise NotImplementedError("perturbation and structural potentials must share one subhalo table")
        self.precision = int(precision)
        if BaseStreamModel is not None:
            bsm = BaseStreamModel
            self.base_stream = bsm
            self.num_pert = int(self.sh_table.m.shape[0])
            self.jump_ts = None
            ts_h = bsm._ts_h
            n = len(ts_h)
            # backward progenitor response from the observation time, zero at t_obs
            cfg = _abi.ss_pert_cfg()
            cfg.t0, cfg.dt = float(ts_h[-1]), -float(bsm._h)
            cfg.n_steps, cfg.n_particles = bsm._spr * (n - 1), 1
            cfg.particles_per_release, cfg.steps_per_release = 1, 0
            cfg.ncol, cfg.save_stride = self._ncol, bsm._spr
            w_obs = bsm.prog_loc_fwd[-1:].contiguous()
            _, out = _core.pert_response(potential_base._desc(), self.sh_table, cfg, 64, w_obs, None)
            self.prog_fieldICs = torch.flip(out[:, 0], dims=[0])  # [len(ts), N_sh, ncol], time increasing
            self.perturbation_ICs_lead, self.perturbation_ICs_trail = self.compute_perturbation_ICs()
            self.base_realspace_ICs_lead = torch.cat([bsm.streamICs[0], bsm.streamICs[2]], dim=1)
            self.base_realspace_ICs_trail = torch.cat([bsm.streamICs[1], bsm.streamICs[3]], dim=1)

    def potential(self, xyz, t):
        raise NotImplementedError

    def compute_perturbation_ICs(self):
        """einsum of release Jacobians with the progenitor response (perturbative.py:84-98)."""
        J = self.base_stream.dRel_dIC
        pf = self.prog_fieldICs
        out = []
        for arm in (0, 1):
            parts = [torch.einsum("ijk,ilk->ilj", J[:, arm], pf[:, :, 6 * b:6 * b + 6])
                     for b in range(self._ncol // 6)]
            out.append(torch.cat(parts, dim=2))
        return out[0], out[1]

    def compute_base_stream(self, cpu=True):
        """perturbative.py:67-81"""
        b = self.base_stream
        return self.potential_base.gen_stream_vmapped(ts=b._ts_h, prog_w0=b.prog_w0, Msat=b.Msat,
                                                      seed_num=b.seednum, dt=b._dt, normals=b.normals)

    def compute_perturbation_OTF(self, cpu=True, solver=None, rtol=1e-6, atol=1e-6, dtmin=0.05, dtmax=None,
                                 max_steps=10_000, *, precision=None):
        """Per-particle response from release to the observation time
        (perturbative.py:100-135).  Returns (lead, trail), each
        [x0v0 [len(ts)-1, 6], derivs [len(ts)-1, N_sh, ncol]]."""
        _core.check_solver(solver)
        prec = int(precision or self.precision)
        b = self.base_stream
        n = len(b._ts_h)
        nrel = n - 1
        base = torch.stack([self.base_realspace_ICs_lead[:nrel], self.base_realspace_ICs_trail[:nrel]], dim=1)
        pert = torch.stack([self.perturbation_ICs_lead[:nrel], self.perturbation_ICs_trail[:nrel]], dim=1)
        cfg = _abi.ss_pert_cfg()
        cfg.t0, cfg.dt = float(b._ts_h[0]), float(b._h)
        cfg.n_steps, cfg.n_particles = b._spr * nrel, 2 * nrel
        cfg.particles_per_release, cfg.steps_per_release = 2, b._spr
        cfg.ncol, cfg.save_stride = self._ncol, 0
        base_out, out = _core.pert_response(self.potential_base._desc(), self.sh_table, cfg, prec,
                                            base.reshape(2 * nrel, 6).contiguous(),
                                            pert.reshape(2 * nrel, self.num_pert, self._ncol).contiguous())
        base_out = base_out.reshape(nrel, 2, 6)
        d = out[0].reshape(nrel, 2, self.num_pert, self._ncol)
        return [base_out[:, 0], d[:, 0]], [base_out[:, 1], d[:, 1]]

    def _stream_pert_cfg(self):
        b = self.base_stream
        nrel = len(b._ts_h) - 1
        cfg = _abi.ss_pert_cfg()
        cfg.t0, cfg.dt = float(b._ts_h[0]), float(b._h)
        cfg.n_steps, cfg.n_particles = b._spr * nrel, 2 * nrel
        cfg.particles_per_release, cfg.steps_per_release = 2, b._spr
        cfg.ncol, cfg.save_stride = self._ncol, 0
        return cfg, nrel

    def compute_perturbation_Interp(self, cpu=True, solver=None, rtol=1e-6, atol=1e-6, dtmin=0.05, dtmax=None, *,
                                    precision=None):
        """The response along the stored base stream (perturbative.py:178-221):
        the base track (stage positions and tidal tensors of every particle)
        is computed once per BaseStreamModel and precision and reused by every
        perturbation generator built on it, so each subhalo batch only
        integrates its response.  Same results as compute_perturbation_OTF."""
        _core.check_solver(solver)
        prec = int(precision or self.precision)
        b = self.base_stream
        cfg, nrel = self._stream_pert_cfg()
        cache = b.__dict__.setdefault("_pert_tracks", {})
        if prec not in cache:
            base = torch.stack([self.base_realspace_ICs_lead[:nrel], self.base_realspace_ICs_trail[:nrel]], dim=1)
            cache[prec] = _core.pert_base_track(self.potential_base._desc(), cfg, prec,
                                                base.reshape(2 * nrel, 6).contiguous())
        track, base_out = cache[prec]
        pert = torch.stack([self.perturbation_ICs_lead[:nrel], self.perturbation_ICs_trail[:nrel]], dim=1)
        out = _core.pert_response_track(self.sh_table, self.potential_base._G, cfg, prec, track,
                                        pert.reshape(2 * nrel, self.num_pert, self._ncol))
        base_out = base_out.reshape(nrel, 2, 6)
        d = out[0].reshape(nrel, 2, self.num_pert, self._ncol)
        return [base_out[:, 0], d[:, 0]], [base_out[:, 1], d[:, 1]]


class BaseStreamModelChen25(Potential):
    """Chen+25 base stream with the progenitor's own potential moving on its
    orbit (perturbative.py:588-658).  Particles are ordered by release time,
    lead before trail (the reference's sorted [ts, ts + 1e-12] stack)."""

    def __init__(self, pot_base, ts, prog_w0, Msat, key, solver=None, rtol=1e-7, atol=1e-7, dtmin=0.3, dtmax=None,
                 max_steps=10_000, throw=False, prog_pot=None, units=None, *, dt=None, normals=None):
        from . import potential as P
        from .streamhelpers import CHEN25_MEAN, chen25_factor
        units = units if units is not None else pot_base.units
        super().__init__(units, {"pot_base": pot_base, "ts": ts, "prog_w0": prog_w0, "Msat": Msat, "key": key,
                                 "solver": solver, "prog_pot": prog_pot})
        _core.check_solver(solver)
        if prog_pot is None:
            prog_pot = P.PlummerPotential(m=0.0, r_s=1.0, units=units)
        self.prog_pot = prog_pot
        ts_h = host64(ts).reshape(-1)
        self._ts_h = ts_h
        seed = int(np.asarray(key).ravel()[-1])
        self.normals = normals if normals is not None else release_normals(seed, len(ts_h), 1, 6)
        ws, self._h, self._spr = pot_base._prog_orbit(ts_h, prog_w0, dt)
        self.prog_loc_fwd = ws
        ics, _ = pot_base._release(ws, ts_h, Msat, self.normals, model=_abi.SS_RELEASE_CHEN25,
                                   chen=(CHEN25_MEAN, chen25_factor()))
        self.streamICs = ics[:, 0].reshape(-1, 6)  # [2 len(ts), 6]: lead_0, trail_0, lead_1, ...
        track = _core.CenterTrack.from_samples(ts_h, ws[:, :3])
        self.pot_tot = P.Potential_Combine(
            [pot_base, P.TimeDepTranslatingPotential(prog_pot, track, units=units)], units=units)
        self.BaseModel = self


class GenerateMassRadiusPerturbation_Chen25(Potential):
    """First-order response for the Chen+25 base stream (perturbative.py:661-773).

    As in the reference, the perturbation initial conditions are zero
    (perturbative.py:712) and the base potential includes the moving
    progenitor.  compute_perturbation_OTF returns
    [x0v0 [2 len(ts) - 1, 6], derivs [2 len(ts) - 1, N_sh, 12]] in release
    order (lead, trail), the last trail star dropped as in the reference."""

    def __init__(self, potential_base, potential_perturbation, BaseStreamModel, units=None, **kwargs):
        super().__init__(units if units is not None else potential_base.units,
                         {"potential_base": potential_base, "potential_perturbation": potential_perturbation,
                          "BaseStreamModel": BaseStreamModel})
        self.base_model = BaseStreamModel
        self.potential_base = potential_base
        self.sh_table = potential_perturbation.table()
        self.num_pert = int(self.sh_table.m.shape[0])
        self.gradientPotentialBase = BaseStreamModel.pot_tot.gradient
        self.gradientPotentialPerturbation_per_SH = potential_perturbation.gradient_per_SH

    def compute_perturbation_OTF(self, cpu=True, solver=None, rtol=1e-6, atol=1e-6, dtmin=0.05, max_steps=10_000,
                                 dtmax=None, *, precision=64):
        _core.check_solver(solver)
        b = self.base_model
        n = len(b._ts_h)
        N = 2 * n
        cfg = _abi.ss_pert_cfg()
        cfg.t0, cfg.dt = float(b._ts_h[0]), float(b._h)
        cfg.n_steps, cfg.n_particles = b._spr * (n - 1), N
        cfg.particles_per_release, cfg.steps_per_release = 2, b._spr
        cfg.ncol, cfg.save_stride = 12, 0
        base_out, out = _core.pert_response(b.pot_tot._desc(), self.sh_table, cfg, int(precision),
                                            b.streamICs.contiguous(), None)
        return [base_out[:N - 1], out[0][:N - 1]]

    def run_nonlinear_sim(self, pot_pert=None, solver=None, rtol=1e-6, atol=1e-6, dtmin=0.05, max_steps=10_000):
        """Nonlinear Chen+25 stream in base + perturbation with the unperturbed
        progenitor (perturbative.py:775-813): [2 (len(ts) - 1), 6], lead then trail."""
        from .streamhelpers import gen_stream
        b = self.base_model
        pot_pert = pot_pert if pot_pert is not None else self.potential_perturbation
        lead, trail = gen_stream(b.pot_base, b._ts_h, b.prog_w0, b.Msat, solver=solver, dt=b._h, release="chen25",
                                 prog_pot=b.prog_pot, pot_pert=pot_pert, normals=b.normals)
        return torch.cat([lead, trail], dim=0)


class CustomBaseStreamModel(Potential):
    """Base stream with a caller-given release (perturbative.py:299-364):
    particle i starts at the progenitor's state at ts[i] plus (pos_rel[i],
    vel_rel[i]) (custom_release_model, streamhelpers.py:187-198), so the
    release Jacobian d(ICs)/d(progenitor w) is the identity."""

    def __init__(self, potential_base=None, prog_w0=None, ts=None, pos_rel=None, vel_rel=None, solver=None,
                 units=None, dense=False, cpu=True, *, dt=None, **kwargs):
        super().__init__(units, {"potential_base": potential_base, "prog_w0": prog_w0, "ts": ts, "pos_rel": pos_rel,
                                 "vel_rel": vel_rel, "solver": solver, "dense": dense, "cpu": cpu})
        if dense:
            raise NotImplementedError("dense stream interpolants are replaced by snapshots")
        _core.check_solver(solver)
        self.potential_base = potential_base
        ts_h = host64(ts).reshape(-1)
        self._ts_h = ts_h
        ws, self._h, self._spr = potential_base._prog_orbit(ts_h, prog_w0, dt)
        self.prog_at_ts = ws
        self.prog_loc_fwd = ws
        rel = torch.cat([f64(pos_rel).reshape(-1, 3), f64(vel_rel).reshape(-1, 3)], dim=1).to(ws.device)
        if rel.shape[0] != len(ts_h):
            raise ValueError("pos_rel / vel_rel need one row per release time")
        self.streamICs = (ws + rel).contiguous()  # [len(ts), 6]
        self.IDs = torch.arange(len(ts_h), device=ws.device)
        self.dRel_dIC = self.release_func_jacobian()
        self.stream_interp = None

    def release_func_jacobian(self):
        """[len(ts), 6, 6]: identity (perturbative.py:348-364)."""
        n = len(self._ts_h)
        return torch.eye(6, dtype=torch.float64, device=self.streamICs.device).expand(n, 6, 6).contiguous()

    def gen_stream(self, *, precision="f64"):
        """Particles 0..len(ts)-2 from their release to ts[-1] (perturbative.py:336-345): [len(ts)-1, 6]."""
        n_rel = len(self._ts_h) - 1
        cfg = _abi.ss_stream_cfg()
        cfg.t0, cfg.dt = float(self._ts_h[0]), float(self._h)
        cfg.n_steps, cfg.n_particles = self._spr * n_rel, n_rel
        cfg.particles_per_release, cfg.steps_per_release = 1, self._spr
        final, _ = _core.stream(self.potential_base._desc(), cfg, self.streamICs[:n_rel].contiguous(), precision)
        return final


class GenerateMassRadiusPerturbation_CustomBase(Potential):
    """First-order mass / radius response of a CustomBaseStreamModel stream
    (perturbative.py:367-487): one particle per release time, perturbation
    ICs = dRel_dIC @ the progenitor's backward response."""

    _ncol = 12

    def __init__(self, potential_base, potential_perturbation, potential_structural, BaseStreamModel=None, units=None,
                 *, precision=64, **kwargs):
        super().__init__(units, {"potential_base": potential_base, "potential_perturbation": potential_perturbation,
                                 "potential_structural": potential_structural, "BaseStreamModel": BaseStreamModel})
        self.potential_base = potential_base
        self.potential_perturbation = potential_perturbation
        self.gradientPotentialBase = potential_base.gradient
        self.gradientPotentialPerturbation_per_SH = potential_perturbation.gradient_per_SH
        self.gradientPotentialStructural_per_SH = potential_structural.gradient_per_SH
        self.sh_table = potential_perturbation.table()
        if not self.sh_table.same_lines(potential_structural.table()):
            raise NotImplementedError("perturbation and structural potentials must share one subhalo table")
        self.precision = int(precision)
        self.base_stream = BaseStreamModel
        self.num_pert = int(self.sh_table.m.shape[0])
        self.jump_ts = None
        self.prog_fieldICs_all = self._prog_response()
        self.prog_fieldICs = self.prog_fieldICs_all[:, :, :12]
        self.perturbation_ICs = self.compute_perturbation_ICs()
        self.base_realspace_ICs = BaseStreamModel.streamICs

    def _prog_response(self):
        """Progenitor response backwards from the observation time, zero there
        (perturbative.py:389-397): [len(ts), N_sh, ncol], time increasing."""
        b = self.base_stream
        n = len(b._ts_h)
        cfg = _abi.ss_pert_cfg()
        cfg.t0, cfg.dt = float(b._ts_h[-1]), -float(b._h)
        cfg.n_steps, cfg.n_particles = b._spr * (n - 1), 1
        cfg.particles_per_release, cfg.steps_per_release = 1, 0
        cfg.ncol, cfg.save_stride = self._ncol, b._spr
        _, out = _core.pert_response(self.potential_base._desc(), self.sh_table, cfg, 64,
                                     b.prog_loc_fwd[-1:].contiguous(), None)
        return torch.flip(out[:, 0], dims=[0])

    def compute_perturbation_ICs(self):
        """perturbative.py:410-420: [N_star, N_sh, 12]."""
        J = self.base_stream.dRel_dIC
        pf = self.prog_fieldICs_all
        return torch.cat([torch.einsum("ijk,ilk->ilj", J, pf[:, :, 0:6]),
                          torch.einsum("ijk,ilk->ilj", J, pf[:, :, 6:12])], dim=2)

    def compute_base_stream(self, cpu=True):
        return self.base_stream.gen_stream()

    def _response(self, pert, prec):
        b = self.base_stream
        nrel = len(b._ts_h) - 1
        cfg = _abi.ss_pert_cfg()
        cfg.t0, cfg.dt = float(b._ts_h[0]), float(b._h)
        cfg.n_steps, cfg.n_particles = b._spr * nrel, nrel
        cfg.particles_per_release, cfg.steps_per_release = 1, b._spr
        cfg.ncol, cfg.save_stride = self._ncol, 0
        base_out, out = _core.pert_response(self.potential_base._desc(), self.sh_table, cfg, prec,
                                            self.base_realspace_ICs[:nrel].contiguous(), pert[:nrel].contiguous())
        return base_out, out[0]

    def compute_perturbation_OTF(self, cpu=True, solver=None, rtol=1e-6, atol=1e-6, dtmin=0.05, max_steps=10_000,
                                 dtmax=None, *, precision=None):
        """perturbative.py:424-456: [x0v0 [len(ts)-1, 6], derivs [len(ts)-1, N_sh, 12]]."""
        _core.check_solver(solver)
        base_out, d = self._response(self.perturbation_ICs, int(precision or self.precision))
        return [base_out, d]


class GenerateMassRadiusPerturbation_CustomBase_SecondOrder(GenerateMassRadiusPerturbation_CustomBase):
    """Second order in the subhalo mass with the first-order radius response
    (perturbative.py:491-585, field fields.py:260-320).  The progenitor's
    response and every particle's carry 18 columns per subhalo: the 12
    first-order ones and (x2, v2).  compute_perturbation_OTF returns
    [x0v0 [len(ts)-1, 6], first [len(ts)-1, N_sh, 12], second [len(ts)-1, N_sh, 6]]."""

    _ncol = 18

    def __init__(self, potential_base, potential_perturbation, potential_structural, BaseStreamModel=None, units=None,
                 **kwargs):
        super().__init__(potential_base, potential_perturbation, potential_structural, BaseStreamModel, units,
                         **kwargs)
        self.prog_fieldICs_first_order_mass = self.prog_fieldICs_all[:, :, :12]
        self.prog_fieldICs_second_order_mass = self.prog_fieldICs_all[:, :, 12:]

    def compute_perturbation_ICs(self):
        """perturbative.py:537-550: [[N_star, N_sh, 12], [N_star, N_sh, 6]]."""
        J = self.base_stream.dRel_dIC
        pf = self.prog_fieldICs_all
        first = torch.cat([torch.einsum("ijk,ilk->ilj", J, pf[:, :, 0:6]),
                           torch.einsum("ijk,ilk->ilj", J, pf[:, :, 6:12])], dim=2)
        return [first, torch.einsum("ijk,ilk->ilj", J, pf[:, :, 12:18])]

    def compute_perturbation_OTF(self, cpu=False, solver=None, rtol=1e-8, atol=1e-8, dtmin=0.05, max_steps=10_000,
                                 dtmax=None, *, precision=None):
        _core.check_solver(solver)
        pert = torch.cat(self.perturbation_ICs, dim=2)
        base_out, d = self._response(pert, int(precision or self.precision))
        return [base_out, d[:, :, :12], d[:, :, 12:]]


class GenerateMassPerturbation(GenerateMassRadiusPerturbation):
    """Mass-only response (6 columns per subhalo) at fixed subhalo radius
    (perturbative.py:224-241; the reference's constructor references an
    undefined name and cannot be built, this one works)."""

    _ncol = 6

    def __init__(self, potential_base, potential_perturbation, BaseStreamModel=None, units=None, **kw):
        super().__init__(potential_base, potential_perturbation, None, BaseStreamModel, units, **kw)


__all__ = ["BaseStreamModel", "GenerateMassRadiusPerturbation", "GenerateMassPerturbation", "BaseStreamModelChen25",
           "GenerateMassRadiusPerturbation_Chen25", "CustomBaseStreamModel", "GenerateMassRadiusPerturbation_CustomBase",
           "GenerateMassRadiusPerturbation_CustomBase_SecondOrder"]
