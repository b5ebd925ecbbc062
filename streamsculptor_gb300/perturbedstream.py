"""One stream perturbed by a sampled subhalo population — the reference's
perturbedstream.py API.

gen_perturbed_stream (perturbedstream.py:23-121): sample the number and
masses of encounters from a RateCalculator, place them with an
ImpactGenerator on the unperturbed stream, and generate the Chen+25 stream
in the base potential plus those Hernquist subhalos (the progenitor's orbit
unperturbed, its own potential moving with it).  Every orbit and stream runs
on the GPU kernels; the sampling is host arithmetic.
"""
from __future__ import annotations

import numpy as np
import torch

from . import potential
from .GenerateImpactParams import ImpactGenerator
from .streamhelpers import gen_stream_vmapped_with_pert_Chen25_fixed_prog
from .subhalostatistics import split_key
from ._core import host64


def gen_perturbed_stream(BaseStreamModel, RateCalculator, unperturbed_stream, phi1_unperturbed, log10M_min,
                         log10M_max, key, phi1_bounds, tImpactBounds, phi1_exclude=(1.0, 1.0), phi1window=1.0,
                         M_hm=0.0, normalization=1.0, slope=-1.9, Max_Num_Impacts=10, rtol=1e-7, atol=1e-7,
                         mass_fac=1.0, r_s_fac=1.0, *, dt=None, precision="f64"):
    """Returns dict(leading, trailing, impactors=dict(cartImpact [n, 6],
    tImpact [n], mass [n], r_s [n])), n = Max_Num_Impacts (entries past the
    drawn number of encounters have zero mass).

    BaseStreamModel: a perturbative.BaseStreamModelChen25 (ts, prog_w0,
    prog_pot, pot_base, Msat); unperturbed_stream [N, 6] and
    phi1_unperturbed [N] are that model's stream, leading arm first."""
    bsm = BaseStreamModel
    ts = host64(bsm.ts).reshape(-1)
    pot_base = bsm.pot_base
    step = dt if dt is not None else float(ts[1] - ts[0])
    prog_wtoday = pot_base.integrate_orbit(w0=bsm.prog_w0, t0=ts.min(), t1=ts.max(), ts=np.array([ts.max()]),
                                           dt=step).ys[0]
    sample = RateCalculator.sample_masses(log10M_min=log10M_min, log10M_max=log10M_max, key=key, M_hm=M_hm,
                                          normalization=normalization, slope=slope, array_length=Max_Num_Impacts)
    lm = sample["log10_mass"]
    mass = np.where(lm > 0, (10.0 ** lm) * mass_fac, 0.0)
    r_s = 1.05 * np.sqrt(mass / 1e8) * r_s_fac
    r_s = np.where(r_s == 0.0, 1.0, r_s)
    b_high = RateCalculator.b_max_fac * r_s
    b_bounds = np.stack([np.zeros_like(b_high), b_high], axis=1)
    k1, k2 = split_key(key, 2)
    seednum = int(np.random.default_rng(k1).integers(0, 10_000))
    tstrip = np.concatenate([ts[:-1], ts[:-1]])
    gen = ImpactGenerator(pot=pot_base, tobs=ts.max(), stream=unperturbed_stream, prog_today=prog_wtoday,
                          stream_phi1=phi1_unperturbed, phi1_bounds=phi1_bounds, tImpactBounds=tImpactBounds,
                          phi1window=phi1window, NumImpacts=len(mass), bImpact_bounds=b_bounds,
                          stripping_times=tstrip, phi1_exclude=phi1_exclude, seednum=seednum)
    params = gen.get_subhalo_ImpactParams()
    cart = params["CartesianImpactParams"]
    out = dict(cartImpact=cart, tImpact=torch.as_tensor(params["ImpactFrameParams"]["tImpact"], device=cart.device),
               mass=torch.as_tensor(mass, device=cart.device), r_s=torch.as_tensor(r_s, device=cart.device))
    pot_subhalos = potential.SubhaloLinePotentialCustom_fromFunc(
        func=potential.HernquistPotential, m=mass, r_s=r_s, subhalo_x0=host64(cart[:, :3]),
        subhalo_v=host64(cart[:, 3:]), subhalo_t0=host64(out["tImpact"]), t_window=150.0, units=pot_base.units)
    lead, trail = gen_stream_vmapped_with_pert_Chen25_fixed_prog(pot_base=pot_base, pot_pert=pot_subhalos,
                                                                 prog_pot=bsm.prog_pot, prog_w0=bsm.prog_w0, ts=ts,
                                                                 Msat=bsm.Msat, key=k2, dt=dt, precision=precision)
    return dict(leading=lead, trailing=trail, impactors=out)


__all__ = ["gen_perturbed_stream"]
