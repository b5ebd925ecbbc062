"""Plumbing between the reference-style Python API and the C ABI.

* tensors: every array handed to the library is a contiguous CUDA tensor;
  torch is used for device memory and streams only.
* potentials: a tree of Potential objects is flattened into one
  ``ss_potential`` descriptor (components in list order, at most one center
  track, at most one subhalo table), cached per device.
* thin wrappers around each C entry point, issued on torch's current stream.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field
from typing import List, Optional, Tuple

import numpy as np
import torch

from . import _abi

G_KPC_MYR_MSUN = 4.498502151469553e-12  # kpc^3 / (Msun Myr^2), CODATA-2018 G, IAU Msun, Julian yr


# ----------------------------------------------------------------- units
class UnitSystem:
    """Minimal stand-in for gala's UnitSystem: only the reference's usys
    (kpc, Myr, Msun, radian) and dimensionless are supported."""

    def __init__(self, *units):
        if len(units) == 1 and isinstance(units[0], UnitSystem):
            units = units[0].units
        self.units = tuple(str(u) for u in units)

    def __eq__(self, other):
        return isinstance(other, UnitSystem) and self.units == other.units

    def __hash__(self):
        return hash(self.units)

    def __repr__(self):
        return f"UnitSystem{self.units}"


usys = UnitSystem("kpc", "Myr", "Msun", "radian")
dimensionless = UnitSystem()


def G_for(units) -> float:
    """Potential.__init__ (main.py:22-30): G = 1 when dimensionless."""
    if units is None or units == dimensionless:
        return 1.0
    if UnitSystem(units) == usys:
        return G_KPC_MYR_MSUN
    raise NotImplementedError(f"unit system {units!r}: only usys (kpc, Myr, Msun, radian) or dimensionless")


# --------------------------------------------------------------- tensors
def device() -> torch.device:
    if not torch.cuda.is_available():
        raise RuntimeError("streamsculptor_gb300 needs a CUDA device (GB300, sm_103a); there is no CPU path")
    return torch.device("cuda", torch.cuda.current_device())


def f64(x, dev=None) -> torch.Tensor:
    """Contiguous float64 CUDA tensor view/copy of x."""
    dev = dev or device()
    if isinstance(x, torch.Tensor):
        return x.to(device=dev, dtype=torch.float64).contiguous()
    return torch.as_tensor(np.asarray(x, dtype=np.float64), device=dev).contiguous()


def host64(x) -> np.ndarray:
    if isinstance(x, torch.Tensor):
        return x.detach().to("cpu", torch.float64).numpy()
    return np.asarray(x, dtype=np.float64)


def ptr(t: Optional[torch.Tensor]):
    return None if t is None else C.c_void_p(t.data_ptr())


def stream_handle():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


# ------------------------------------------------------ flattened model
@dataclass
class CenterTrack:
    """Uniform-knot progenitor track for TimeDepTranslatingPotential.

    The reference uses interpax.Interpolator1D(x=ts, f=positions,
    method='cubic') (streamhelpers.py:520).  Knot slopes are filled on the
    device by ss_track_slopes (mean of adjacent secants, one-sided ends)."""

    t0: float
    dt: float
    knots: torch.Tensor  # [n, 3] float64 (device)
    slopes: Optional[torch.Tensor] = None
    # piecewise-linear through the knots instead (the reference's
    # RegularGridInterpolator(method='linear') tracks, potential.py:575-590)
    linear: bool = False

    @staticmethod
    def linear_from_samples(ts, values) -> "CenterTrack":
        t = CenterTrack.from_samples(ts, values)
        t.linear = True
        return t

    def struct(self) -> _abi.ss_track:
        tr = _abi.ss_track()
        tr.knots = self.knots.data_ptr()
        if not self.linear:
            tr.slopes = self.ensure_slopes().data_ptr()
        tr.t0, tr.dt, tr.n_knots, tr.linear = self.t0, self.dt, self.knots.shape[0], int(self.linear)
        return tr

    @staticmethod
    def from_samples(ts, positions) -> "CenterTrack":
        ts_h = host64(ts)
        if ts_h.ndim != 1 or len(ts_h) < 2:
            raise ValueError("track needs >= 2 knot times")
        d = np.diff(ts_h)
        if not np.allclose(d, d[0], rtol=1e-9, atol=1e-12) or d[0] <= 0:
            raise NotImplementedError("track knots must be uniformly spaced and increasing")
        knots = f64(positions)
        if knots.ndim != 2 or knots.shape[1] < 3 or knots.shape[0] != len(ts_h):
            raise ValueError("positions must be [len(ts), >=3]")
        knots = knots[:, :3].contiguous()
        return CenterTrack(float(ts_h[0]), float(d[0]), knots)

    def ensure_slopes(self):
        if self.slopes is None or self.slopes.device != self.knots.device:
            self.slopes = torch.empty_like(self.knots)
            _abi.call("ss_track_slopes", ptr(self.knots), self.knots.shape[0], self.dt, ptr(self.slopes),
                      stream_handle())
        return self.slopes

    @staticmethod
    def growth_from_samples(ts, values, linear=False) -> "CenterTrack":
        """A scalar track (GrowingPotential's growth factor) through values at
        uniform times ts: column 0 of a three-column track."""
        v = f64(values).reshape(-1)
        t = CenterTrack.from_samples(ts, torch.stack([v, torch.zeros_like(v), torch.zeros_like(v)], 1))
        t.linear = bool(linear)
        return t


@dataclass
class SubhaloTable:
    kind: int
    m: torch.Tensor
    a: torch.Tensor
    x0: torch.Tensor
    v: torch.Tensor
    t0: torch.Tensor
    t_window: float
    # SS_SH_GRID: [n, n_grid, 2] (value, d/du) spline tables in u = ln r
    grid: Optional[torch.Tensor] = None
    grid_u0: Optional[torch.Tensor] = None
    grid_du: Optional[torch.Tensor] = None

    def struct(self) -> _abi.ss_subhalos:
        s = _abi.ss_subhalos()
        s.kind = self.kind
        s.n = int(self.m.shape[0])
        s.m, s.a, s.x0, s.v, s.t0 = (self.m.data_ptr(), self.a.data_ptr(), self.x0.data_ptr(),
                                     self.v.data_ptr(), self.t0.data_ptr())
        s.t_window = float(self.t_window)
        if self.grid is not None:
            s.grid, s.grid_u0, s.grid_du = self.grid.data_ptr(), self.grid_u0.data_ptr(), self.grid_du.data_ptr()
            s.n_grid = int(self.grid.shape[1])
        return s

    def same_lines(self, other: "SubhaloTable") -> bool:
        return (self.kind == other.kind and self.t_window == other.t_window and
                all(torch.equal(getattr(self, k), getattr(other, k)) for k in ("m", "a", "x0", "v", "t0")) and
                (self.grid is None) == (other.grid is None) and
                (self.grid is None or torch.equal(self.grid, other.grid)))


@dataclass
class ExpansionTable:
    """Spline table of a spherical-harmonic expansion (ss_expansion):
    coef [n_knots, (l_max+1)^2, 2] float64 on the device holds the value and
    d/dln r of every radial function f_lm at knots ln r = log_r0 + k dlog_r."""
    l_max: int
    log_r0: float
    dlog_r: float
    coef: torch.Tensor

    def struct(self) -> _abi.ss_expansion:
        e = _abi.ss_expansion()
        e.l_max = int(self.l_max)
        e.n_knots = int(self.coef.shape[0])
        e.log_r0 = float(self.log_r0)
        e.dlog_r = float(self.dlog_r)
        e.coef = self.coef.data_ptr()
        return e


@dataclass
class Flat:
    comps: List[Tuple[int, int, Tuple[float, ...]]] = field(default_factory=list)
    track: Optional[CenterTrack] = None
    subhalos: Optional[SubhaloTable] = None
    expansion: Optional[ExpansionTable] = None
    frame_velocity: Optional[CenterTrack] = None
    growth: Optional[CenterTrack] = None

    def extend(self, other: "Flat"):
        self.comps.extend(other.comps)
        if other.track is not None:
            if self.track is not None and self.track is not other.track:
                raise NotImplementedError("at most one center track per potential")
            self.track = other.track
        if other.subhalos is not None:
            if self.subhalos is not None:
                raise NotImplementedError("at most one subhalo table per potential")
            self.subhalos = other.subhalos
        if other.expansion is not None:
            if self.expansion is not None and self.expansion is not other.expansion:
                raise NotImplementedError("at most one spherical-harmonic expansion per potential")
            self.expansion = other.expansion
        if other.frame_velocity is not None:
            if self.frame_velocity is not None and self.frame_velocity is not other.frame_velocity:
                raise NotImplementedError("at most one uniform frame acceleration per potential")
            self.frame_velocity = other.frame_velocity
        if other.growth is not None:
            if self.growth is not None and self.growth is not other.growth:
                raise NotImplementedError("at most one growth track per potential")
            self.growth = other.growth


def make_struct(flat: Flat, G: float) -> _abi.ss_potential:
    if len(flat.comps) > _abi.SS_MAX_COMPONENTS:
        raise NotImplementedError(f"more than {_abi.SS_MAX_COMPONENTS} potential components")
    P = _abi.ss_potential()
    P.G = float(G)
    P.n_components = len(flat.comps)
    for i, (kind, center, params) in enumerate(flat.comps):
        P.comp[i].kind = kind
        P.comp[i].center = center
        for j, v in enumerate(params):
            P.comp[i].p[j] = float(v)
    if flat.track is not None:
        P.track = flat.track.struct()
    if flat.frame_velocity is not None:
        P.frame_velocity = flat.frame_velocity.struct()
    if flat.growth is not None:
        P.growth = flat.growth.struct()
    if flat.subhalos is not None:
        P.subhalos = flat.subhalos.struct()
    if flat.expansion is not None:
        P.expansion = flat.expansion.struct()
    return P


# ------------------------------------------------------------ fixed step
def fixed_step(span: float, dt=None, grid=None, dtmin=None, dtmax=None) -> Tuple[float, int]:
    """Step h (signed like span) and step count for a fixed-step solve.

    The reference's adaptive PIDController (main.py:146) becomes a fixed step:
    `dt` when given; else the spacing of the save grid (reduced to a divisor
    no larger than dtmax); else dtmin.  The span must be a whole number of
    steps."""
    if span == 0:
        return (1.0 if dt is None else float(abs(dt))), 0
    sign = 1.0 if span > 0 else -1.0
    if dt is not None:
        h = abs(float(dt))
    elif grid is not None and grid > 0:
        h = float(grid)
        if dtmax is not None and dtmax < h:
            h = h / math.ceil(h / float(dtmax) - 1e-12)
    elif dtmin is not None:
        h = float(dtmin)
    else:
        raise ValueError("fixed-step integration needs dt")
    n = round(abs(span) / h)
    if n < 1 or abs(n * h - abs(span)) > 1e-9 * max(1.0, abs(span)):
        raise ValueError(f"span {span} is not a whole number of steps of {h}; pass dt=")
    return sign * h, int(n)


def check_solver(solver):
    """Only Dopri5 is implemented (fixed step); others raise."""
    if solver is None:
        return
    name = solver if isinstance(solver, str) else type(solver).__name__
    if "dopri5" not in str(name).lower():
        raise NotImplementedError(f"solver {name!r}: only fixed-step Dopri5 is implemented on the GPU path")


# ------------------------------------------------------- entry wrappers
def potential_eval(P, xyz: torch.Tensor, t, phi=True, grad=True, hess=False):
    n = xyz.shape[0]
    dev = xyz.device
    tt = None
    ts = 0.0
    if isinstance(t, torch.Tensor) and t.ndim > 0 or isinstance(t, np.ndarray) and np.ndim(t) > 0:
        tt = f64(t, dev).reshape(-1)
        if tt.shape[0] != n:
            raise ValueError("t must be scalar or have one entry per point")
    else:
        ts = float(t)
    o_phi = torch.empty(n, dtype=torch.float64, device=dev) if phi else None
    o_g = torch.empty(n, 3, dtype=torch.float64, device=dev) if grad else None
    o_h = torch.empty(n, 3, 3, dtype=torch.float64, device=dev) if hess else None
    _abi.call("ss_potential_eval", C.byref(P), ptr(xyz), n, ptr(tt), ts, ptr(o_phi), ptr(o_g), ptr(o_h),
              stream_handle())
    return o_phi, o_g, o_h


SHOOT_TOL = 1e-14


def orbit(P, w0: torch.Tensor, t0: float, dt: float, n_steps: int, save_every: int,
          method: str = "auto", keep_starts: bool = False):
    """Fixed-step FP64 Dopri5 orbits.  method: 'serial' (one thread per
    orbit), 'shoot' (one orbit, parallel in time by multiple shooting; the
    serial orbit up to round-off) or 'auto' (shoot for a single long orbit in
    a static potential)."""
    n = w0.shape[0]
    out = torch.empty(n, n_steps // save_every + 1, 6, dtype=torch.float64, device=w0.device)
    if method == "auto":
        method = "shoot" if (n == 1 and n_steps >= 64 and is_static(P)) else "serial"
    if method == "shoot":
        if n != 1:
            raise ValueError("the parallel-in-time orbit integrates one orbit")
        need = _abi.load().ss_orbit_shoot_workspace_bytes(int(n_steps))
        buf = Workspace.get(int(need), w0.device, slot="shoot")
        ws, nb = aligned_ptr(buf)
        _abi.call("ss_orbit_shoot_f64", C.byref(P), ptr(w0), float(t0), float(dt), int(n_steps), int(save_every),
                  ptr(out), ws, nb, SHOOT_TOL, stream_handle())
        if keep_starts:
            # converged slice starts: the first 6 (S + 1) doubles of the workspace
            S = int(_abi.load().ss_orbit_shoot_slices(int(n_steps)))
            off = ws.value - buf.data_ptr()
            starts = buf[off:off + 48 * (S + 1)].view(torch.float64).reshape(S + 1, 6).clone()
            return out, starts
    elif method == "serial":
        _abi.call("ss_orbit_f64", C.byref(P), ptr(w0), n, float(t0), float(dt), int(n_steps), int(save_every),
                  ptr(out), stream_handle())
    else:
        raise ValueError("method must be 'auto', 'serial' or 'shoot'")
    if keep_starts:
        return out, None
    return out


def orbit_ensemble(P, w0: torch.Tensor, t0: float, dt, n_steps: int, save_every: int = 0,
                   subhalos_per_orbit: int = 0) -> torch.Tensor:
    """Orbits with their own step (dt: a float, or [n] steps) and, for
    subhalos_per_orbit = k > 0, their own subhalo rows [i k, (i + 1) k):
    [n, n_steps // save_every + 1, 6] (save_every 0: start and end only)."""
    n = w0.shape[0]
    every = int(save_every) if save_every else max(int(n_steps), 1)
    out = torch.empty(n, int(n_steps) // every + 1, 6, dtype=torch.float64, device=w0.device)
    if torch.is_tensor(dt) or np.ndim(dt) > 0:
        dts = f64(dt).reshape(n).contiguous()
        dptr, dall = ptr(dts), 0.0
    else:
        dts, dptr, dall = None, None, float(dt)
    _abi.call("ss_orbit_ensemble_f64", C.byref(P), ptr(w0.contiguous()), n, float(t0), dptr, dall, int(n_steps),
              every, int(subhalos_per_orbit), ptr(out), stream_handle())
    return out


TIME_DEPENDENT_KINDS = (_abi.SS_BAR, _abi.SS_DEHNEN_BAR, _abi.SS_UNIFORM_ACCEL)


def is_static(P) -> bool:
    """True when the descriptor has no center-track, rotating or frame-
    acceleration component and no subhalos."""
    return P.subhalos.n == 0 and all(P.comp[i].center == _abi.SS_CENTER_ORIGIN and
                                     P.comp[i].kind not in TIME_DEPENDENT_KINDS for i in range(P.n_components))


def release(P, cfg, prog_w, t_rel, msat, normals, jac=False):
    n_rel, n_draw = cfg.n_release, cfg.n_draw
    ics = torch.empty(n_rel, n_draw, 2, 6, dtype=torch.float64, device=prog_w.device)
    J = torch.empty(n_rel, n_draw, 2, 6, 6, dtype=torch.float64, device=prog_w.device) if jac else None
    _abi.call("ss_release_f64", C.byref(P), C.byref(cfg), ptr(prog_w), ptr(t_rel), ptr(msat), ptr(normals),
              ptr(ics), ptr(J), stream_handle())
    return ics, J


class Workspace:
    """Grow-only device scratch shared by the calls of one process."""

    _bufs = {}

    @classmethod
    def get(cls, nbytes: int, dev: torch.device, slot: str = "main") -> Optional[torch.Tensor]:
        if nbytes <= 0:
            return None
        key = (dev.type, dev.index, slot)
        buf = cls._bufs.get(key)
        if buf is None or buf.numel() < nbytes:
            buf = torch.empty(int(nbytes) + 256, dtype=torch.uint8, device=dev)
            cls._bufs[key] = buf
        return buf


def aligned_ptr(buf: Optional[torch.Tensor], align: int = 256):
    if buf is None:
        return None, 0
    p = buf.data_ptr()
    off = (-p) % align
    return C.c_void_p(p + off), buf.numel() - off


# When set to a list, stream() appends a (start, end) CUDA event pair recorded
# around each stream-kernel call on the current stream (benchmark timing).
STREAM_EVENTS = None


def stream(P, cfg, ics: torch.Tensor, precision: str, want_final=True, snaps=None, status=True, mlp=None,
           judge=None):
    """One stream launch.  precision 'mlp' integrates in the surrogate's force
    (mlp); with judge = dict(tol=, every=) the potential P is kept as its error
    judge and fallback (ss_stream_mlp_judged_bf16): judge['fallbacks_device']
    receives the device count of tiles that fell back (int64 [1], complete
    when the current stream is) and judge['tiles'] the number of tiles."""
    N = cfg.n_particles
    dev = ics.device
    final = torch.empty(N, 6, dtype=torch.float64, device=dev) if want_final else None
    st = torch.empty(N, dtype=torch.int32, device=dev) if status else None
    evs = STREAM_EVENTS
    if evs is not None:
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
    if precision == "f64":
        _abi.call("ss_stream_f64", C.byref(P), C.byref(cfg), ptr(ics), ptr(final), ptr(snaps), ptr(st),
                  stream_handle())
    elif precision == "f32k":
        need = _abi.load().ss_stream_workspace_bytes(C.byref(P), C.byref(cfg))
        if need < 0:
            raise _abi.SSError("ss_stream_workspace_bytes", need, _abi.load().ss_last_error().decode())
        ws, nb = aligned_ptr(Workspace.get(need, dev))
        _abi.call("ss_stream_f32k", C.byref(P), C.byref(cfg), ptr(ics), ptr(final), ptr(snaps), ptr(st),
                  ws, nb, stream_handle())
    elif precision == "mlp":
        if mlp is None:
            raise ValueError("precision='mlp' needs a force surrogate")
        m = mlp.struct()
        if judge is None:
            _abi.call("ss_stream_mlp_bf16", C.byref(m), C.byref(cfg), ptr(ics), ptr(final), ptr(snaps), ptr(st), None,
                      0, stream_handle())
        else:
            need = _abi.load().ss_stream_mlp_judged_workspace_bytes(C.byref(P), C.byref(cfg))
            if need < 0:
                raise _abi.SSError("ss_stream_mlp_judged_workspace_bytes", need, _abi.load().ss_last_error().decode())
            ws, nb = aligned_ptr(Workspace.get(need, dev, slot="judge"))
            count = torch.zeros(1, dtype=torch.int64, device=dev)
            _abi.call("ss_stream_mlp_judged_bf16", C.byref(m), C.byref(P), C.byref(cfg), C.c_float(judge["tol"]),
                      int(judge.get("every", 64)), ptr(ics), ptr(final), ptr(snaps), ptr(st), ptr(count), ws, nb,
                      stream_handle())
            judge["fallbacks_device"] = count
            judge["tiles"] = (int(N) + 127) // 128
    else:
        raise ValueError("precision must be 'f64', 'f32k' or 'mlp'")
    if evs is not None:
        e1.record()
        evs.append((e0, e1))
    return final, st


_AUX_STREAMS = {}


def _aux_stream(dev: torch.device, name: str, priority: int = 0) -> torch.cuda.Stream:
    key = (dev.type, dev.index, name, priority)
    if key not in _AUX_STREAMS:
        _AUX_STREAMS[key] = torch.cuda.Stream(device=dev, priority=priority)
    return _AUX_STREAMS[key]


def _chunk_priorities(n: int):
    """Stream priorities for n sub-range kernels, the first (its particles
    released first: the longest tracks) highest: spread over the device's
    range (lower numbers are higher priorities)."""
    try:
        lo, hi = torch.cuda.Stream.priority_range()  # (least, greatest)
    except (RuntimeError, AttributeError):
        return [0] * max(1, n)
    span = lo - hi
    if n <= 1 or span <= 0:
        return [hi] * max(1, n)
    return [hi + (span * i) // (n - 1) for i in range(n)]


def host_buffers(n_particles: int, n_snap: int = 0):
    """Pinned host output buffers for stream_to_host / gen_stream(out='host'):
    (final [N, 6] float64, snapshots [n_snap, N, 6] float32 or None)."""
    final_h = torch.empty(int(n_particles), 6, dtype=torch.float64, pin_memory=True)
    snaps_h = torch.empty(int(n_snap), int(n_particles), 6, dtype=torch.float32, pin_memory=True) if n_snap else None
    return final_h, snaps_h


def _check_host_buffers(bufs, N: int, n_snap: int):
    final_h, snaps_h = bufs
    if (not isinstance(final_h, torch.Tensor) or final_h.is_cuda or final_h.dtype != torch.float64 or
            tuple(final_h.shape) != (N, 6) or not final_h.is_contiguous() or not final_h.is_pinned()):
        raise ValueError(f"out_buffers[0] must be a contiguous pinned host float64 tensor [{N}, 6]")
    if n_snap:
        if (not isinstance(snaps_h, torch.Tensor) or snaps_h.is_cuda or snaps_h.dtype != torch.float32 or
                tuple(snaps_h.shape) != (n_snap, N, 6) or not snaps_h.is_contiguous() or not snaps_h.is_pinned()):
            raise ValueError(f"out_buffers[1] must be a contiguous pinned host float32 tensor [{n_snap}, {N}, 6]")
    elif snaps_h is not None:
        raise ValueError("out_buffers[1] must be None for a run without snapshots")


def _launch_stream(P, c, precision: str, ics, final, snaps_ptr, status, mlp, stream, slot: str):
    """One ss_stream_* launch on `stream` with snapshots at the raw pointer
    snaps_ptr (device memory, or pinned host memory that the device
    addresses directly)."""
    h = C.c_void_p(stream.cuda_stream)
    if precision == "f64":
        _abi.call("ss_stream_f64", C.byref(P), C.byref(c), ptr(ics), ptr(final), snaps_ptr, ptr(status), h)
    elif precision == "f32k":
        lib = _abi.load()
        need = lib.ss_stream_workspace_bytes(C.byref(P), C.byref(c))
        if need < 0:
            raise _abi.SSError("ss_stream_workspace_bytes", need, lib.ss_last_error().decode())
        ws, nb = aligned_ptr(Workspace.get(need, ics.device, slot=slot))
        _abi.call("ss_stream_f32k", C.byref(P), C.byref(c), ptr(ics), ptr(final), snaps_ptr, ptr(status), ws, nb, h)
    elif precision == "mlp":
        m = mlp.struct()
        _abi.call("ss_stream_mlp_bf16", C.byref(m), C.byref(c), ptr(ics), ptr(final), snaps_ptr, ptr(status), None,
                  0, h)
    else:
        raise ValueError("precision must be 'f64', 'f32k' or 'mlp'")


def stream_to_host(P, cfg, ics: torch.Tensor, precision: str, snap_every: int = 0, mlp=None, n_chunks: int = 8,
                   n_streams: int = 0, out_buffers=None, mode: str = "direct"):
    """The stream with its results in pinned host memory.  mode 'direct'
    (default): one launch that writes its snapshot rows straight into the
    pinned host buffer (pinned memory is addressable from the device under
    unified addressing; on Grace-Blackwell the stores cross the coherent
    chip-to-chip link while the stream integrates), then the final states
    (48 bytes per particle) copied after it.  Measured on the spray
    workload: the kernel takes 142 ms instead of 125 ms with its snapshots
    in HBM, and the step time varies by a few percent; the copy engine's
    device -> host rate, which the chunked mode depends on, varied between
    runs from 193 GB/s down to 15-50 GB/s for stretches of 100 ms and more.
    mode 'chunked': the stream in particle sub-ranges whose results are
    copied to pinned host memory while later sub-ranges integrate (as fast
    as the device-resident step when the copy engine keeps its rate).
    Each sub-range kernel has
    a CUDA stream of its own (n_streams = 0: one per sub-range), so that none
    waits in stream order behind another; the streams carry decreasing
    priorities, so that the block scheduler places the first sub-range (the
    earliest releases: the longest tracks, which set the run's length) ahead
    of the others whatever the launch race between streams (without that,
    a later sub-range taking the SMs first made some runs take twice as
    long).  Each sub-range's copies follow on a copy stream of its own
    (snapshots move as strided row blocks with ss_copy_rows_async).  Returns pinned host (final
    [N,6] float64, snapshots [n_snap,N,6] float32 or None) and the device
    status [N]; the host buffers are complete once the current stream is
    synchronised.  out_buffers: caller-owned pinned buffers (host_buffers())
    written in place, so that repeated calls allocate no pinned memory (a
    fresh multi-GB pinned allocation costs more than the copies)."""
    import copy as _cp
    if mode not in ("direct", "chunked"):
        raise ValueError("mode must be 'direct' or 'chunked'")
    N = int(cfg.n_particles)
    dev = ics.device
    n_snap = int(cfg.n_steps) // snap_every if snap_every else 0
    final_d = torch.empty(N, 6, dtype=torch.float64, device=dev)
    status_d = torch.empty(N, dtype=torch.int32, device=dev)
    if out_buffers is not None:
        _check_host_buffers(out_buffers, N, n_snap)
        final_h, snaps_h = out_buffers
    else:
        final_h, snaps_h = host_buffers(N, n_snap)
    main = torch.cuda.current_stream(dev)
    if mode == "direct":
        c = _cp.copy(cfg)
        c.snap_stride = snap_every if n_snap else 0
        c.snap_pitch = 0
        _launch_stream(P, c, precision, ics, final_d, C.c_void_p(snaps_h.data_ptr()) if n_snap else None, status_d,
                       mlp, main, "compute0")
        final_h.copy_(final_d, non_blocking=True)
        return final_h, snaps_h, status_d
    snaps_d = torch.empty(n_snap, N, 6, dtype=torch.float32, device=dev) if n_snap else None
    n_sub = -(-N // max(128, -(-N // max(1, n_chunks) // 128) * 128)) if N > 0 else 1
    n_cs = int(n_streams) if n_streams else n_sub
    prios = _chunk_priorities(n_cs)
    comp = [_aux_stream(dev, f"compute{i}", prios[i]) for i in range(max(1, n_cs))]
    # one copy stream per compute stream: a sub-range's copy never queues
    # behind the copy of a sub-range that is still integrating on the other
    copies = [_aux_stream(dev, f"copy{i}") for i in range(len(comp))]
    for st in comp + copies:
        st.wait_stream(main)  # inputs and buffers are ready on the main stream
    per = max(128, -(-N // max(1, n_chunks) // 128) * 128)
    for c_idx, p0 in enumerate(range(0, N, per)):
        p1 = min(N, p0 + per)
        c = _cp.copy(cfg)
        c.first_particle, c.n_particles = p0, p1 - p0
        c.snap_pitch = N if n_snap else 0
        c.snap_stride = snap_every if n_snap else 0
        sub_ics, fin, stt = ics[p0:p1], final_d[p0:p1], status_d[p0:p1]
        cs = comp[c_idx % len(comp)]
        _launch_stream(P, c, precision, sub_ics, fin, ptr(snaps_d), stt, mlp, cs, f"compute{c_idx % len(comp)}")
        ev = torch.cuda.Event()
        ev.record(cs)
        side = copies[c_idx % len(comp)]
        side.wait_event(ev)
        hs = C.c_void_p(side.cuda_stream)
        _abi.call("ss_copy_rows_async", C.c_void_p(final_h.data_ptr()), ptr(final_d), 1, N * 48, p0 * 48,
                  (p1 - p0) * 48, 0, hs)
        if n_snap:
            _abi.call("ss_copy_rows_async", C.c_void_p(snaps_h.data_ptr()), ptr(snaps_d), n_snap, N * 24, p0 * 24,
                      (p1 - p0) * 24, 0, hs)
    for st in comp + copies:
        main.wait_stream(st)
    for t in (final_d, status_d, snaps_d, ics):
        if t is not None:
            for st in comp + copies:
                t.record_stream(st)
    return final_h, snaps_h, status_d


def subhalo_eval(table: SubhaloTable, G: float, xyz: torch.Tensor, t: float):
    n, ns = xyz.shape[0], int(table.m.shape[0])
    dev = xyz.device
    phi = torch.empty(n, ns, dtype=torch.float64, device=dev)
    grad = torch.empty(n, ns, 3, dtype=torch.float64, device=dev)
    dphi = torch.empty(n, ns, dtype=torch.float64, device=dev)
    gdphi = torch.empty(n, ns, 3, dtype=torch.float64, device=dev)
    S = table.struct()
    _abi.call("ss_subhalo_eval", C.byref(S), float(G), ptr(xyz), n, float(t), ptr(phi), ptr(grad), ptr(dphi),
              ptr(gdphi), stream_handle())
    return phi, grad, dphi, gdphi


def pert_term(P, table: SubhaloTable, ncol: int, t: float, y: torch.Tensor) -> torch.Tensor:
    """d/dt of y = [x0v0 (6), n_sh x ncol] (FP64, device) at time t."""
    y = y.contiguous()
    dy = torch.empty_like(y)
    S = table.struct()
    _abi.call("ss_pert_term", C.byref(P), C.byref(S), int(ncol), float(t), ptr(y), ptr(dy), stream_handle())
    return dy


def pert_response(P, table: SubhaloTable, cfg, precision: int, base_ics, pert_ics, chunk_particles=None):
    dev = base_ics.device
    dtype = torch.float64 if precision == 64 else torch.float32
    N, ns, ncol = cfg.n_particles, int(table.m.shape[0]), cfg.ncol
    n_saves = cfg.n_steps // cfg.save_stride + 1 if cfg.save_stride > 0 else 1
    out = torch.empty(n_saves, N, ns, ncol, dtype=dtype, device=dev)
    base_out = torch.empty(N, 6, dtype=torch.float64, device=dev)
    if chunk_particles is None:
        # base-track records of up to a quarter of the free device memory
        # (at least 2 GB, at most 32 GB) per chunk: each chunk's FP64 base
        # pass lasts as long as its longest track whatever the chunk's size,
        # so few large chunks keep it from dominating
        per = max(1, cfg.n_steps) * (120 if ncol == 18 else 56) * (8 if precision == 64 else 4)
        free, _ = torch.cuda.mem_get_info(dev)
        budget = min(32 << 30, max(2 << 30, free // 4))
        chunk_particles = max(1, min(N, budget // per))
    need = _abi.load().ss_pert_workspace_bytes(C.byref(cfg), precision, int(chunk_particles))
    if need < 0:
        raise _abi.SSError("ss_pert_workspace_bytes", need, _abi.load().ss_last_error().decode())
    ws, nb = aligned_ptr(Workspace.get(need, dev))
    S = table.struct()
    if pert_ics is not None:
        pert_ics = pert_ics.to(dtype).contiguous()
    _abi.call("ss_pert_response", C.byref(P), C.byref(S), C.byref(cfg), int(precision), ptr(base_ics),
              ptr(pert_ics), ptr(base_out), ptr(out), ws, nb, stream_handle())
    return base_out, out


def pert_base_track(P, cfg, precision: int, base_ics):
    """Stored base track of every particle (ss_pert_base_track): (track
    buffer, final base states [N, 6])."""
    dev = base_ics.device
    nb = _abi.load().ss_pert_track_bytes(C.byref(cfg), int(precision))
    if nb < 0:
        raise _abi.SSError("ss_pert_track_bytes", nb, _abi.load().ss_last_error().decode())
    track = torch.empty(max(int(nb), 16) // 16 * 16 + 16, dtype=torch.uint8, device=dev)
    base_out = torch.empty(cfg.n_particles, 6, dtype=torch.float64, device=dev)
    _abi.call("ss_pert_base_track", C.byref(P), C.byref(cfg), int(precision), ptr(base_ics), ptr(base_out),
              ptr(track), track.numel(), stream_handle())
    return track, base_out


def pert_response_track(table: SubhaloTable, G: float, cfg, precision: int, track, pert_ics):
    """Response of the subhalos `table` along a stored base track."""
    dev = track.device
    dtype = torch.float64 if precision == 64 else torch.float32
    N, ns, ncol = cfg.n_particles, int(table.m.shape[0]), cfg.ncol
    n_saves = cfg.n_steps // cfg.save_stride + 1 if cfg.save_stride > 0 else 1
    out = torch.empty(n_saves, N, ns, ncol, dtype=dtype, device=dev)
    S = table.struct()
    if pert_ics is not None:
        pert_ics = pert_ics.to(dtype).contiguous()
    _abi.call("ss_pert_response_track", C.byref(S), float(G), C.byref(cfg), int(precision), ptr(track),
              ptr(pert_ics), ptr(out), stream_handle())
    return out


def binned_sums(values: torch.Tensor, key: torch.Tensor, edges: torch.Tensor):
    n, ncomp = values.shape
    nb = edges.shape[0] - 1
    sums = torch.empty(nb, ncomp, dtype=torch.float64, device=values.device)
    counts = torch.empty(nb, ncomp, dtype=torch.float64, device=values.device)
    _abi.call("ss_binned_sums", ptr(values), ptr(key), n, ncomp, ptr(edges), edges.shape[0], ptr(sums),
              ptr(counts), stream_handle())
    return sums, counts
