"""Algorithmic work per particle-step, counted from the kernel source.

Convention: add / sub / mul = 1 flop, fma = 2 flops; sqrt, rsqrt,
reciprocal / division and log1p are counted separately as "special" ops
(they expand to several pipe instructions, so flop rates computed from the
algorithmic count understate pipe utilisation; ncu gives the latter).

Force evaluation (ss_device.cuh, comp_grad without Hessian), per component:
  NFW          r^2 (5) + soft (1) + r*q (1) + (r+rs) (1) + 1/r^2 (1)
               + g = q0/r^2 (L/r - 1/(r+rs)) (4) + grad += g x (6)  = 19; specials 4
  TriaxialNFW  x/q (3) + NFW radial part (13) + grad (6) + 3 scale (3) = 25; specials 4
  MiyamotoNagai zeta (2) + a+zeta (1) + S^2 (5) + 1/S^3 (3) + fz (1) + grad (7) = 19; specials 3
  Hernquist    r^2 (5) + soft (1) + r+rs (1) + g (3) + grad (6)      = 16; specials 3
  Plummer      r^2 (5) + b^2 (1) + g (3) + grad (6)                    = 15; specials 1
  Isochrone    r^2 (5) + a^2 (1) + a+s (1) + g (3) + grad (6)          = 16; specials 3
  SH expansion (l_max, nt = (l_max+1)^2 terms; gradient only):
               r^2, n = x/r, ln r, spline basis (~45) + solid-harmonic
               recurrences up to degree 8 (232) + per term: spline value and
               slope (17), radial factors a0, a1, G1 (6), S1 += G1 K (2),
               angular gradient (5), V += a0 grad K (6) = 36 / term;
               total 270 + 36 nt (3186 at l_max = 8); specials 2 (rsqrt, log)
  translating  + 3 (x - c(t))
  subhalo line + 9 (line position) + 15 (Plummer form) + 1 window test
Dopri5 combinations per step (6 force evaluations, FSAL reuse):
  FP64 plain          6 components x (stages 35 + update 11)            = 276
  FP32 compensated    3 x (stages 84 + position update 27 + velocity 28) = 417
  FP32 compensated, Nystrom form (stream_f32k2_kernel, two particles per
  thread): per coordinate, stage positions 6, stage offsets 5 + 8 + 12 + 15
  + 24, position update 20, velocity update 20 = 110; x 3 = 330.  Its forces
  also restore the FP32 masses (and NFW's 1 / r_s) from their rounding
  residuals: one FMA each, 4 flops for NFW and 2 for the other spherical and
  disk kinds per force evaluation.

First-order response (pert_response2_kernel, two subhalos per thread in
packed f32x2 lanes, and pert_response_kernel, ss_pert.cu), per (particle,
subhalo)-step, mass columns only (ncol = 6), Plummer subhalos:
  stage states   per column a-sums of 1..5 terms (1 + 3 + 5 + 7 + 9) and
                 U = u + h acc (5 x 2)                          = 35; x 6 = 210
  right-hand side per stage: line position (6) + rel (3) + r^2 (5)
                 + Plummer g (5; 1 rsqrt) + g rel (3) + T x1 - on g (21) = 43;
                 x 6 stages = 258, 6 specials
  stage times    6 FMAs                                          = 12
  update         per column b-sum (9) + u + h sum (2)            = 11; x 6 = 66
  total 546 flops, 6 specials.  The radius columns (ncol = 12) repeat the
  stage, update and T x1 work for six more columns and add the structural
  gradient (4 per stage): 546 + 210 + 66 + 6 x (21 + 4) = 972.

The same step in Nystrom form (pert_response2_kernel: only the stage
accelerations are kept), per response dimension (3 per column block):
  stage positions  abar-sums of 0..4 terms (0 + 1 + 3 + 5 + 7 = 16) and
                   x + h (c v + h acc) for stages 2..6 (5 x 5 = 25)  = 41; x 3 = 123
  right-hand side  as above, 43 per stage (the position rows of the
                   first-order form are the velocity itself)         = 258
  stage times                                                        = 12
  update           bbar- and b-sums (9 + 9), x + h (v + h .) (4),
                   v + h . (2)                                       = 24; x 3 = 72
  total 465 flops, 6 specials.  With the radius columns (ncol = 12) the
  positions and update double and each stage adds T X, the structural
  gradient's force factor and its rel terms (25): 465 + 123 + 72 + 6 x 25
  = 810.
"""
from __future__ import annotations

from . import _abi

FORCE_FLOPS = {
    _abi.SS_NFW: (19, 4),
    _abi.SS_TRIAXIAL_NFW: (25, 4),
    _abi.SS_MIYAMOTO_NAGAI: (19, 3),
    _abi.SS_HERNQUIST: (16, 3),
    _abi.SS_PLUMMER: (15, 1),
    _abi.SS_ISOCHRONE: (16, 3),
}
TRANSLATE_FLOPS = 3
SUBHALO_FLOPS = (25, 1)
RK_FLOPS = {"f64": 276, "f32k": 417, "f32k2": 330}
RESIDUAL_FLOPS = {
    _abi.SS_NFW: 4,
    _abi.SS_MIYAMOTO_NAGAI: 2,
    _abi.SS_HERNQUIST: 2,
    _abi.SS_PLUMMER: 2,
    _abi.SS_ISOCHRONE: 2,
}
STAGES = 6


def force_work(flat, residuals: bool = False) -> tuple:
    """(flops, specials) of one force evaluation of a flattened potential;
    residuals adds the mass-residual FMAs of the packed two-particle kernel."""
    fl, sp = 0, 0
    for kind, center, _ in flat.comps:
        if kind == _abi.SS_SH_EXPANSION:
            nt = (flat.expansion.l_max + 1) ** 2
            f, s = 270 + 36 * nt, 2
        else:
            f, s = FORCE_FLOPS[kind]
        fl += f + (TRANSLATE_FLOPS if center == _abi.SS_CENTER_TRACK else 0)
        if residuals:
            fl += RESIDUAL_FLOPS.get(kind, 0)
        sp += s
    if flat.subhalos is not None:
        n = int(flat.subhalos.m.shape[0])
        fl += n * SUBHALO_FLOPS[0]
        sp += n * SUBHALO_FLOPS[1]
    return fl, sp


def particle_step_work(flat, precision: str) -> dict:
    """Flops and special ops of one Dopri5 step of one particle: precision
    "f64", "f32k" (scalar compensated kernel) or "f32k2" (packed two-particle
    compensated kernel, Nystrom form)."""
    fl, sp = force_work(flat, residuals=precision == "f32k2")
    return {"flops": STAGES * fl + RK_FLOPS[precision], "specials": STAGES * sp,
            "force_flops": fl, "force_specials": sp, "rk_flops": RK_FLOPS[precision]}


RESPONSE_FLOPS = {6: 546, 12: 972}
RESPONSE_FLOPS_NYSTROM = {6: 465, 12: 810}


def response_step_work(ncol: int = 6, form: str = "nystrom") -> dict:
    """Flops and special ops of one Dopri5 step of one (particle, subhalo)
    linear-response system (Plummer subhalos): form 'nystrom' (the packed
    FP32 kernel) or 'first_order' (the scalar kernel)."""
    table = {"nystrom": RESPONSE_FLOPS_NYSTROM, "first_order": RESPONSE_FLOPS}.get(form)
    if table is None:
        raise ValueError("form must be 'nystrom' or 'first_order'")
    if ncol not in table:
        raise ValueError("ncol must be 6 or 12")
    return {"flops": table[ncol], "specials": STAGES}
