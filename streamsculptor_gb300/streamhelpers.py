"""Stream generators and helpers — the reference's streamhelpers.py API.

`gen_stream` is the one engine behind every generator here and behind
Potential.gen_stream_vmapped: FP64 progenitor orbit (ss_orbit_shoot_f64,
parallel in time, or ss_orbit_f64), release (ss_release_f64),
optional moving-progenitor potential on a cubic track, then the stream kernel
(ss_stream_f64 or ss_stream_f32k).
"""
from __future__ import annotations

from typing import Optional

import numpy as np
import torch

from . import _abi, _core
from ._core import CenterTrack, f64, host64
from .main import Potential, _grid_spacing, _kvals, _n_draw, _split_ics, release_normals
from . import potential as _pot

# release_model_Chen25 mean and covariance (streamhelpers.py:360-369)
CHEN25_MEAN = np.array([1.6, -30.0, 0.0, 1.0, 20.0, 0.0])
CHEN25_COV = np.array([
    [0.1225, 0, 0, 0, -4.9, 0],
    [0, 529, 0, 0, 0, 0],
    [0, 0, 144, 0, 0, 0],
    [0, 0, 0, 0, 0, 0],
    [-4.9, 0, 0, 0, 400, 0],
    [0, 0, 0, 0, 0, 484],
], dtype=np.float64)


def chen25_factor(cov=CHEN25_COV) -> np.ndarray:
    """L with L L^T = cov, from the SVD (jax multivariate_normal method='svd')."""
    u, s, _ = np.linalg.svd(cov)
    return u * np.sqrt(s)[None, :]


def gen_stream(pot_base: Potential, ts=None, prog_w0=None, Msat=None, seed_num=None, *, solver=None,
               kval_arr=1.0, dt=None, dtmax=None, n_particles_per_release=2, normals=None, precision="f64",
               snapshot_every=None, throw=False, release="fardal", prog_pot: Optional[Potential] = None,
               pot_pert: Optional[Potential] = None, prog_in_pert=False, return_ics=False, prog_method="auto",
               force_surrogate=None, out="device", release_range=None, out_buffers=None, surrogate_judge=None,
               host_mode="direct"):
    """Generate a particle-spray stream on the GPU.

    pot_base    smooth potential (release model and integration)
    prog_pot    optional progenitor potential moving on the progenitor's
                orbit (TimeDepTranslatingPotential on its cubic track,
                streamhelpers.py:520-522)
    pot_pert    optional perturbation (subhalos) added for integration
                (streamhelpers.py:89-146); with prog_in_pert the progenitor
                orbit is integrated in base + pert too (gen_stream_ics_pert)
    release     'fardal' (main.py:209-280) or 'chen25' (streamhelpers.py:352-432)
    prog_method progenitor orbit solver (FP64 either way): 'serial', 'shoot'
                (parallel in time, multiple shooting) or 'auto' (shoot when the
                progenitor's potential is static)
    out         'device' (CUDA tensors) or 'host': pinned host tensors, ready
                when the call returns
    host_mode   (out='host') 'direct': the stream kernel writes its snapshots
                straight into the pinned host buffer; 'chunked': the stream runs
                in particle sub-ranges whose results the copy engine moves to
                the host while the next sub-range integrates (_core.stream_to_host)
    surrogate_judge (precision='mlp') dict(tol=, every=): keep pot_base as the
                surrogate's error judge and fallback (ss_stream_mlp_judged_bf16):
                every `every` steps each 128-particle tile compares its surrogate
                force with the exact one and falls back to the exact force for
                good where any particle differs by more than tol (relative);
                fills in surrogate_judge['fallbacks'] and ['tiles']
    out_buffers (out='host' only) caller-owned pinned host buffers to write
                into, from _core.host_buffers(N, n_snap): (final [N, 6] float64,
                snapshots [n_snap, N, 6] float32 or None); repeated calls then
                allocate no pinned memory, and each call overwrites them
    precision   'f64', 'f32k' (FP32 compensated) or 'mlp': the particles move
                in the force of `force_surrogate` (surrogate.MLPSurrogate, BF16
                tensor cores) while the progenitor orbit and the release use
                the exact pot_base
    release_range (r0, r1): integrate only the particles of releases r0..r1-1
                (one rank's share of a stream split across GPUs, sharding.py);
                the progenitor orbit and the release are computed in full
    Returns (lead, trail) [len(ts)-1, 6] (or [len(ts)-1, n_draw, 6]; with
    release_range [r1-r0, ...]); with snapshot_every also the float32
    snapshots [n_snap, len(ts)-1, n_draw, 2, 6].
    """
    _core.check_solver(solver)
    ts_h = host64(ts).reshape(-1)
    if len(ts_h) < 2:
        raise ValueError("need at least two release times")
    ts_grid, t_end = _split_tail(ts_h)
    if t_end is not None and (prog_pot is not None or snapshot_every or out != "device"):
        raise NotImplementedError("ts with a last interval off the release grid: no moving progenitor, snapshots or "
                                  "host output")
    total = pot_base if pot_pert is None else _pot.Potential_Combine([pot_base, pot_pert], units=pot_base.units)
    prog_src = total if (pot_pert is not None and prog_in_pert) else pot_base
    ws, h, spr = prog_src._prog_orbit(ts_grid, prog_w0, dt, None, dtmax, method=prog_method)
    n_draw = _n_draw(n_particles_per_release)
    model = _abi.SS_RELEASE_CHEN25 if release == "chen25" else _abi.SS_RELEASE_FARDAL
    if release not in ("fardal", "chen25"):
        raise ValueError("release must be 'fardal' or 'chen25'")
    nz = 6 if model == _abi.SS_RELEASE_CHEN25 else 4
    if normals is None:
        normals = release_normals(seed_num, len(ts_h), n_draw, nz)
    chen = (CHEN25_MEAN, chen25_factor()) if model == _abi.SS_RELEASE_CHEN25 else None
    if t_end is not None:
        normals = np.asarray(host64(normals)) if not torch.is_tensor(normals) else normals
        normals = normals[:len(ts_grid)]
    ics, _ = pot_base._release(ws, ts_grid, Msat, normals, kval_arr, model=model, chen=chen)
    integ = total
    if prog_pot is not None:
        track = CenterTrack.from_samples(ts_h, ws[:, :3])
        moving = _pot.TimeDepTranslatingPotential(prog_pot, track, units=pot_base.units)
        integ = _pot.Potential_Combine([total, moving], units=pot_base.units)
    n_rel = len(ts_h) - 1
    ppr = 2 * n_draw
    N = n_rel * ppr
    cfg = _abi.ss_stream_cfg()
    cfg.t0 = float(ts_h[0])
    cfg.dt = float(h)
    # with a last interval off the grid, the grid part ends at the last release
    cfg.n_steps = spr * (n_rel if t_end is None else n_rel - 1)
    cfg.n_particles = N
    cfg.particles_per_release = ppr
    cfg.steps_per_release = spr
    cfg.snap_stride = int(snapshot_every or 0)
    snaps = None
    stream_ics = ics[:n_rel].reshape(N, 6).contiguous()
    if release_range is not None:
        r0, r1 = (int(v) for v in release_range)
        if not 0 <= r0 <= r1 <= n_rel:
            raise ValueError("release_range must lie within [0, len(ts) - 1]")
        if snapshot_every or out != "device":
            raise NotImplementedError("release_range runs return final states on the device only")
        cfg.first_particle, cfg.n_particles = r0 * ppr, (r1 - r0) * ppr
        stream_ics = stream_ics[r0 * ppr:r1 * ppr].contiguous()
        n_rel = r1 - r0
        if n_rel == 0:
            empty = torch.empty((0, n_draw, 6) if n_draw > 1 else (0, 6), dtype=torch.float64, device=ws.device)
            return (empty, empty.clone()) + ((ics, ws) if return_ics else ())
    if precision == "mlp" and (integ is not pot_base or force_surrogate is None):
        raise NotImplementedError("precision='mlp' integrates in the surrogate alone: give force_surrogate and no "
                                  "prog_pot / pot_pert")
    if out == "host":
        final, snaps, status = _core.stream_to_host(integ._desc(), cfg, stream_ics, precision,
                                                    int(snapshot_every or 0), mlp=force_surrogate,
                                                    out_buffers=out_buffers, mode=host_mode)
        torch.cuda.current_stream().synchronize()
    elif out == "device":
        if out_buffers is not None:
            raise ValueError("out_buffers is for out='host'")
        if snapshot_every:
            n_snap = cfg.n_steps // int(snapshot_every)
            snaps = torch.empty(n_snap, N, 6, dtype=torch.float32, device=ws.device)
        if surrogate_judge is not None and precision != "mlp":
            raise ValueError("surrogate_judge is for precision='mlp'")
        final, status = _core.stream(integ._desc(), cfg, stream_ics, precision, snaps=snaps, mlp=force_surrogate,
                                     judge=surrogate_judge)
        if surrogate_judge is not None:
            surrogate_judge["fallbacks"] = int(surrogate_judge.pop("fallbacks_device").item())
        if t_end is not None:
            final, status = _tail_phase(integ, cfg, final, status, float(ts_grid[-1]), float(t_end), h, precision,
                                        force_surrogate)
    else:
        raise ValueError("out must be 'device' or 'host'")
    if throw and bool((status != 0).any()):
        raise RuntimeError("gen_stream: non-finite particle state")
    final = final.reshape(n_rel, n_draw, 2, 6)
    if n_draw == 1:
        lead, trail = final[:, 0, 0], final[:, 0, 1]
    else:
        lead, trail = final[:, :, 0], final[:, :, 1]
    out = (lead, trail)
    if snapshot_every:
        out = out + (snaps.reshape(-1, n_rel, n_draw, 2, 6),)
    if return_ics:
        out = out + (ics, ws)
    return out


def gen_stream_batches(pot_base: Potential, ts=None, prog_w0s=None, Msat=None, normals=None, *, n_batches=None,
                       seed_num=None, dt=None, prog_pot: Optional[Potential] = None, n_particles_per_release=2,
                       precision="f32k", snapshot_every=None, release="fardal", kval_arr=1.0, prog_w0_at="start",
                       prog_method="auto", lookahead=1):
    """gen_stream for a sequence of streams (other progenitors, or the same
    one with other draws), pipelined on two CUDA streams: the progenitor
    orbits (with prog_w0_at='end', first back from the present, as
    integrate_orbit over [ts[-1], ts[0]]), the release and the track tables
    of the next `lookahead` streams run on a high-priority side stream while
    the current stream's kernel fills the GPU (those steps are a few blocks,
    bound by the issue latency of their warps).  Every stream does all of
    its own work; only its order against the others changes.

    prog_w0s and normals: one value for every stream or a list with one per
    stream (n_batches gives the count when neither is a list); a stream
    whose normals are None draws them from seed_num + its index.  ts must be a
    uniform release grid; no perturbation, device outputs; precision 'f64'
    or 'f32k'.  Yields each stream's gen_stream result ((lead, trail[,
    snapshots])), enqueued on the current stream."""
    if precision not in ("f64", "f32k"):
        raise ValueError("precision must be 'f64' or 'f32k'")
    if prog_w0_at not in ("start", "end"):
        raise ValueError("prog_w0_at must be 'start' or 'end'")
    ts_h = host64(ts).reshape(-1)
    if len(ts_h) < 2 or _grid_spacing(ts_h) is None:
        raise NotImplementedError("gen_stream_batches needs a uniform release grid ts")
    lists = [len(v) for v in (prog_w0s, normals) if isinstance(v, (list, tuple))]
    B = lists[0] if lists else n_batches
    if B is None or any(n != B for n in lists):
        raise ValueError("give lists of equal length for prog_w0s / normals, or n_batches")
    w0s = prog_w0s if isinstance(prog_w0s, (list, tuple)) else [prog_w0s] * B
    nrm = normals if isinstance(normals, (list, tuple)) else [normals] * B
    if seed_num is None and any(n is None for n in nrm):
        raise ValueError("give normals, or seed_num, for every stream")
    n_draw = _n_draw(n_particles_per_release)
    model = _abi.SS_RELEASE_CHEN25 if release == "chen25" else _abi.SS_RELEASE_FARDAL
    if release not in ("fardal", "chen25"):
        raise ValueError("release must be 'fardal' or 'chen25'")
    chen = (CHEN25_MEAN, chen25_factor()) if model == _abi.SS_RELEASE_CHEN25 else None
    nz = 6 if model == _abi.SS_RELEASE_CHEN25 else 4
    main = torch.cuda.current_stream()
    pot_base._desc()
    side = torch.cuda.Stream(priority=-1)
    side.wait_stream(main)
    n_rel = len(ts_h) - 1
    ppr = 2 * n_draw

    def prepare(i):
        with torch.cuda.stream(side):
            w0 = w0s[i]
            if prog_w0_at == "end":
                w0 = pot_base.integrate_orbit(w0=w0, ts=np.array([ts_h[-1], ts_h[0]]), t0=float(ts_h[-1]),
                                              t1=float(ts_h[0]), dt=dt).ys[-1]
            ws, h, spr = pot_base._prog_orbit(ts_h, w0, dt, None, None, method=prog_method)
            nm = nrm[i] if nrm[i] is not None else release_normals(int(seed_num) + i, len(ts_h), n_draw, nz)
            ics, _ = pot_base._release(ws, ts_h, Msat, nm, kval_arr, model=model, chen=chen)
            integ = pot_base
            keep = [ws, ics]
            if prog_pot is not None:
                track = CenterTrack.from_samples(ts_h, ws[:, :3])
                integ = _pot.Potential_Combine([pot_base, _pot.TimeDepTranslatingPotential(prog_pot, track,
                                                                                          units=pot_base.units)],
                                               units=pot_base.units)
                integ._desc()  # the track's slopes, on the side stream
                keep += [track.knots, track.slopes]
            stream_ics = ics[:n_rel].reshape(n_rel * ppr, 6).contiguous()
            keep.append(stream_ics)
            ev = torch.cuda.Event()
            ev.record(side)
        # the main stream reads these after the side stream made them
        for t in keep:
            t.record_stream(main)
        return dict(integ=integ, h=h, spr=spr, stream_ics=stream_ics, ev=ev)

    ready = {}
    for i in range(B):
        for j in range(i, min(i + max(1, int(lookahead)) + 1, B)):
            if j not in ready:
                ready[j] = prepare(j)
        prep = ready.pop(i)
        main.wait_event(prep["ev"])
        N = n_rel * ppr
        cfg = _abi.ss_stream_cfg()
        cfg.t0, cfg.dt = float(ts_h[0]), float(prep["h"])
        cfg.n_steps, cfg.n_particles = prep["spr"] * n_rel, N
        cfg.particles_per_release, cfg.steps_per_release = ppr, prep["spr"]
        cfg.snap_stride = int(snapshot_every or 0)
        snaps = None
        if snapshot_every:
            snaps = torch.empty(cfg.n_steps // int(snapshot_every), N, 6, dtype=torch.float32,
                                device=prep["stream_ics"].device)
        final, _ = _core.stream(prep["integ"]._desc(), cfg, prep["stream_ics"], precision, snaps=snaps)
        final = final.reshape(n_rel, n_draw, 2, 6)
        out = (final[:, 0, 0], final[:, 0, 1]) if n_draw == 1 else (final[:, :, 0], final[:, :, 1])
        if snapshot_every:
            out = out + (snaps.reshape(-1, n_rel, n_draw, 2, 6),)
        yield out


def _split_tail(ts_h: np.ndarray):
    """(release grid, end time): the reference integrates every release
    ts[i], i < len(ts) - 1, to ts[-1], and its notebooks end on a time off
    the release grid (ts = [linspace(-t_age, t_dissolve, n), 0]).  When ts is
    uniform the grid is ts and the end None; when only ts[:-1] is, the grid
    is ts[:-1] (every point a release) and the end ts[-1]."""
    if len(ts_h) < 4 or _grid_spacing(ts_h) is not None:
        return ts_h, None
    head = ts_h[:-1]
    if _grid_spacing(head) is None or not ts_h[-1] > ts_h[-2] or not head[1] > head[0]:
        return ts_h, None
    return head, float(ts_h[-1])


def _tail_phase(integ, cfg, final, status, t_last, t_end, h, precision, force_surrogate=None):
    """Every particle from the last release time to t_end in equal steps no
    longer than h (one more stream-kernel launch, all particles starting at
    its first step)."""
    span = t_end - t_last
    m = int(np.ceil(span / h - 1e-9))
    cfg2 = _abi.ss_stream_cfg()
    cfg2.t0, cfg2.dt, cfg2.n_steps = t_last, span / m, m
    cfg2.n_particles = cfg.n_particles
    cfg2.particles_per_release, cfg2.steps_per_release = max(int(cfg.n_particles), 1), 0
    cfg2.stream_particles, cfg2.subhalos_per_stream = cfg.stream_particles, cfg.subhalos_per_stream
    cfg2.first_particle = cfg.first_particle  # the same global particles (subhalo rows of an ensemble)
    final2, status2 = _core.stream(integ._desc(), cfg2, final.contiguous(), precision, mlp=force_surrogate)
    return final2, torch.maximum(status, status2)


def gen_stream_ensemble(pot_base: Potential, pot_pert: Potential, subhalos_per_stream: int, ts=None, prog_w0=None,
                        Msat=None, seed_num=None, *, solver=None, kval_arr=1.0, dt=None, normals=None,
                        prog_in_pert=True, precision="f64", prog_w0_at="start", return_ics=False):
    """B independent perturbed streams in one pass: jax.vmap of
    gen_stream_vmapped_with_pert (streamhelpers.py:89-116; _fixed_prog,
    :119-146, with prog_in_pert=False) over subhalo parameters, as the
    reference's GD-1 fitting notebook runs hundreds of samples at once.

    pot_pert    SubhaloLinePotential(-like) with B * subhalos_per_stream rows;
                stream b feels rows [b k, (b + 1) k) only
    prog_w0     [6] (every stream) or [B, 6]: the progenitor at ts[0], or at
                ts[-1] with prog_w0_at="end" (then each stream's progenitor is
                first integrated back to ts[0], in base + its own subhalos
                when prog_in_pert, as the notebook does per sample)
    normals     release draws [len(ts), 1, 4] shared by every stream (the
                reference reuses seed_num for every sample) or [B, len(ts), 1, 4]
    ts          uniform, or uniform release times followed by a later end time
    Every stream's progenitor orbit runs in one ensemble orbit launch, the
    releases in one release launch, and all B streams in one stream launch.
    Returns (lead, trail), each [B, n_rel, 6]."""
    _core.check_solver(solver)
    prep = _ensemble_prepare(pot_base, pot_pert, subhalos_per_stream, ts, prog_w0, Msat, seed_num, kval_arr, dt,
                             normals, prog_in_pert, prog_w0_at)
    return _ensemble_run(prep, precision, return_ics)


def gen_stream_ensemble_batches(pot_base: Potential, pot_perts, subhalos_per_stream: int, ts=None, prog_w0=None,
                                Msat=None, seed_num=None, *, solver=None, kval_arr=1.0, dt=None, normals=None,
                                prog_in_pert=True, precision="f64", prog_w0_at="start", lookahead=2):
    """gen_stream_ensemble over a sequence of subhalo batches (the notebook's
    loop of vmapped batches), pipelined on several CUDA streams: the FP64
    progenitor orbits and releases of the next `lookahead` batches (a few
    hundred threads each, bound by the FP64 issue rate of their warps, not
    by the GPU's capacity) run concurrently while the streams of the current
    batch fill the GPU.  Every host-to-device copy is made before the first
    launch, so the host never waits on the GPU inside the loop.  prog_w0 is
    one state / [B, 6] for every batch or a list with one per batch.
    Returns a list of (lead, trail), ready on the current stream."""
    _core.check_solver(solver)
    perts = list(pot_perts)
    if not perts:
        return []
    w0s = prog_w0 if isinstance(prog_w0, (list, tuple)) else [prog_w0] * len(perts)
    main = torch.cuda.current_stream()
    # device tables and inputs of every batch, made on the main stream up front
    totals = []
    for pert in perts:
        total = _pot.Potential_Combine([pot_base, pert], units=pot_base.units)
        total._desc()
        totals.append(total)
    pot_base._desc()
    shared = isinstance(prog_w0, (list, tuple)) is False
    inputs = [None] * len(perts)
    for i, pert in enumerate(perts):
        if i == 0 or not shared or int(pert.table().m.shape[0]) != int(perts[0].table().m.shape[0]):
            inputs[i] = _ensemble_inputs(pert, subhalos_per_stream, ts, w0s[i], Msat, seed_num, kval_arr, dt,
                                         normals)
        else:
            inputs[i] = inputs[0]
    depth = max(1, int(lookahead))
    # high priority: their few orbit blocks go first when the streams free a slot
    sides = [torch.cuda.Stream(priority=-1) for _ in range(depth)]
    for sd in sides:
        sd.wait_stream(main)

    def prepare(i):
        side = sides[i % depth]
        with torch.cuda.stream(side):
            prep = _ensemble_prepare(pot_base, perts[i], subhalos_per_stream, ts, None, Msat, seed_num, kval_arr, dt,
                                     normals, prog_in_pert, prog_w0_at, totals[i], inputs[i])
            ev = torch.cuda.Event()
            ev.record(side)
        for t in (prep["ics"], prep["ws"]):
            t.record_stream(main)
        return prep, ev

    outs = []
    ready = {}
    for i in range(len(perts)):
        for j in range(i, min(i + depth + 1, len(perts))):
            if j not in ready:
                ready[j] = prepare(j)
        prep, ev = ready.pop(i)
        main.wait_event(ev)
        outs.append(_ensemble_run(prep, precision, False))
    return outs


def _ensemble_grid(ts, dt):
    ts_h = host64(ts).reshape(-1)
    ts_grid, t_end = _split_tail(ts_h)
    grid = _grid_spacing(ts_grid)
    if grid is None or ts_grid[1] < ts_grid[0]:
        raise NotImplementedError("release times must be uniformly spaced and increasing")
    h, spr = _core.fixed_step(grid, dt=dt if dt is not None else grid)
    return ts_h, ts_grid, t_end, h, spr


def _ensemble_inputs(pot_pert, subhalos_per_stream, ts, prog_w0, Msat, seed_num, kval_arr, dt, normals):
    """Device copies of an ensemble's inputs (progenitor states, release
    times, satellite masses, release draws) and its release config."""
    k = int(subhalos_per_stream)
    n_sh = int(pot_pert.table().m.shape[0])
    if k < 1 or n_sh % k:
        raise ValueError("the subhalo table must hold subhalos_per_stream rows per stream")
    B = n_sh // k
    ts_h, ts_grid, _, _, _ = _ensemble_grid(ts, dt)
    n_grid = len(ts_grid)
    w0 = f64(prog_w0).reshape(-1, 6)
    if w0.shape[0] == 1:
        w0 = w0.expand(B, 6).contiguous()
    if w0.shape[0] != B:
        raise ValueError("prog_w0 must be [6] or [B, 6]")
    if normals is None:
        normals = release_normals(seed_num, len(ts_h), 1, 4)
    nrm = f64(normals)
    if nrm.ndim == 3:
        nrm = nrm.unsqueeze(0).expand(B, *nrm.shape)
    nrm = nrm[:, :n_grid].reshape(B * n_grid, -1, 4).contiguous()
    m = host64(Msat)
    msat = np.full(n_grid, float(m)) if m.ndim == 0 else m.reshape(-1)[:n_grid]
    rcfg = _abi.ss_release_cfg()
    rcfg.n_release, rcfg.n_draw, rcfg.model = B * n_grid, nrm.shape[1], _abi.SS_RELEASE_FARDAL
    for i, kv in enumerate(_kvals(kval_arr)):
        rcfg.kvals[i] = kv
    return dict(w0=w0, nrm=nrm, t_rel=f64(np.tile(ts_grid, B)), msat=f64(np.tile(np.asarray(msat, np.float64), B)),
                rcfg=rcfg, B=B)


def _ensemble_prepare(pot_base, pot_pert, subhalos_per_stream, ts, prog_w0, Msat, seed_num, kval_arr, dt, normals,
                      prog_in_pert, prog_w0_at, total=None, inputs=None):
    """Progenitor orbits (one ensemble launch, two with prog_w0_at="end")
    and the releases (one launch) of an ensemble, on the current stream;
    with `inputs` (from _ensemble_inputs) nothing here copies between host
    and device."""
    k = int(subhalos_per_stream)
    if prog_w0_at not in ("start", "end"):
        raise ValueError("prog_w0_at must be 'start' or 'end'")
    if inputs is None:
        inputs = _ensemble_inputs(pot_pert, k, ts, prog_w0, Msat, seed_num, kval_arr, dt, normals)
    B = inputs["B"]
    ts_h, ts_grid, t_end, h, spr = _ensemble_grid(ts, dt)
    n_grid = len(ts_grid)
    w0 = inputs["w0"]
    if total is None:
        total = _pot.Potential_Combine([pot_base, pot_pert], units=pot_base.units)
    src = total if prog_in_pert else pot_base
    kk = k if prog_in_pert else 0
    if prog_w0_at == "end":
        span = float(ts_h[-1] - ts_h[0])
        n_back = max(1, int(np.ceil(span / h - 1e-9)))
        w0 = _core.orbit_ensemble(src._desc(), w0, float(ts_h[-1]), -span / n_back, n_back, 0, kk)[:, -1]
        w0 = w0.contiguous()
    ws = _core.orbit_ensemble(src._desc(), w0, float(ts_grid[0]), h, spr * (n_grid - 1), spr, kk)  # [B, n_grid, 6]
    ics, _ = _core.release(pot_base._desc(), inputs["rcfg"], ws.reshape(B * n_grid, 6), inputs["t_rel"],
                           inputs["msat"], inputs["nrm"])  # [B n_grid, 1, 2, 6]
    n_rel = len(ts_h) - 1
    ics = ics.reshape(B, n_grid, 2, 6)[:, :n_rel].reshape(B * 2 * n_rel, 6).contiguous()
    N = 2 * n_rel
    cfg = _abi.ss_stream_cfg()
    cfg.t0, cfg.dt = float(ts_grid[0]), float(h)
    cfg.n_steps = spr * (n_rel if t_end is None else n_rel - 1)
    cfg.n_particles = B * N
    cfg.particles_per_release, cfg.steps_per_release = 2, spr
    cfg.stream_particles, cfg.subhalos_per_stream = N, k
    return dict(total=total, cfg=cfg, ics=ics, ws=ws, B=B, n_rel=n_rel, t_last=float(ts_grid[-1]), t_end=t_end, h=h)


def _ensemble_run(prep, precision, return_ics):
    """The stream launches of a prepared ensemble, on the current stream."""
    total, cfg, B, n_rel = prep["total"], prep["cfg"], prep["B"], prep["n_rel"]
    final, status = _core.stream(total._desc(), cfg, prep["ics"], precision)
    if prep["t_end"] is not None:
        final, status = _tail_phase(total, cfg, final, status, prep["t_last"], prep["t_end"], prep["h"], precision)
    final = final.reshape(B, n_rel, 2, 6)
    out = (final[:, :, 0], final[:, :, 1])
    if return_ics:
        out = out + (prep["ics"].reshape(B, n_rel, 2, 6), prep["ws"])
    return out


# ----------------------------------------------------- reference names
def eval_dense_stream(t_eval=None, dense_stream=None):
    raise NotImplementedError("dense streams are replaced by snapshots (gen_stream_vmapped(..., snapshot_every=k))")


def eval_dense_stream_id(time=None, interp_func=None, idx=None, lead=True):
    raise NotImplementedError("dense streams are replaced by snapshots (gen_stream_vmapped(..., snapshot_every=k))")


def gen_stream_ics_pert(pot_base=None, pot_pert=None, ts=None, prog_w0=None, Msat=None, seed_num=None, solver=None,
                        kval_arr=1.0, max_steps=10_000, rtol=1e-7, atol=1e-7, dtmin=0.1, *, dt=None,
                        n_particles_per_release=2, normals=None):
    """Release in the smooth potential from a progenitor orbit integrated in
    base + perturbation (streamhelpers.py:56-84)."""
    ts_h = host64(ts).reshape(-1)
    total = _pot.Potential_Combine([pot_base, pot_pert], units=pot_base.units)
    ws, _, _ = total._prog_orbit(ts_h, prog_w0, dt)
    n_draw = _n_draw(n_particles_per_release)
    if normals is None:
        normals = release_normals(seed_num, len(ts_h), n_draw, 4)
    ics, _ = pot_base._release(ws, ts_h, Msat, normals, kval_arr)
    return _split_ics(ics, n_draw)


def gen_stream_vmapped_with_pert(pot_base=None, pot_pert=None, ts=None, prog_w0=None, Msat=None, seed_num=None,
                                 solver=None, kval_arr=1.0, max_steps=10_000, rtol=1e-7, atol=1e-7, dtmin=0.1, *,
                                 dt=None, precision="f64", **kw):
    """Perturbed stream, progenitor in base + pert (streamhelpers.py:89-116)."""
    return gen_stream(pot_base, ts, prog_w0, Msat, seed_num, solver=solver, kval_arr=kval_arr, dt=dt,
                      pot_pert=pot_pert, prog_in_pert=True, precision=precision, **kw)


def gen_stream_vmapped_with_pert_fixed_prog(pot_base=None, pot_pert=None, ts=None, prog_w0=None, Msat=None,
                                            seed_num=None, solver=None, kval_arr=1.0, max_steps=10_000, rtol=1e-7,
                                            atol=1e-7, dtmin=0.1, *, dt=None, precision="f64", **kw):
    """Perturbed stream with the unperturbed progenitor (streamhelpers.py:119-146)."""
    return gen_stream(pot_base, ts, prog_w0, Msat, seed_num, solver=solver, kval_arr=kval_arr, dt=dt,
                      pot_pert=pot_pert, prog_in_pert=False, precision=precision, **kw)


gen_stream_scan_with_pert = gen_stream_vmapped_with_pert


def custom_release_model(pos_prog=None, vel_prog=None, pos_rel=None, vel_rel=None):
    """streamhelpers.py:186-198"""
    return f64(pos_prog) + f64(pos_rel), f64(vel_prog) + f64(vel_rel)


# ---------------------------------------------------------------- streakline
def _streakline_grid(t0, t1, Nstrip, dt):
    """Release times linspace(t0, t1, Nstrip) and the fixed step: the release
    spacing, or that spacing split into the fewest steps no longer than dt."""
    ts = np.linspace(float(t0), float(t1), int(Nstrip))
    if int(Nstrip) < 2:
        raise ValueError("Nstrip must be >= 2")
    gap = (ts[-1] - ts[0]) / (len(ts) - 1)
    spr = 1 if dt is None else max(1, int(np.ceil(abs(gap) / float(dt) - 1e-12)))
    return ts, gap / spr, spr


def get_Streakline_ICs(pot, prog_w0, Msat, t0, t1, Nstrip, solver=None, rtol=1e-6, atol=1e-6, dt=None):
    """Streakline release (streamhelpers.py:657-705): at Nstrip times
    linspace(t0, t1) one particle leaves each of the progenitor's Lagrange
    points (Potential.lagrange_pts, main.py:106-112) moving along the
    progenitor's velocity direction at the progenitor's angular velocity,
    |v| = omega |x_L| / sin(theta), theta between the progenitor's position
    and velocity.  The progenitor runs forward from prog_w0 at t0 (fixed-step
    FP64, the release spacing or steps of at most dt; the reference's
    adaptive solver arguments are accepted and not used).  Returns
    (L_close, v_lead, L_far, v_trail, ts), CUDA tensors and ts on the host."""
    _core.check_solver(solver)
    ts, h, _ = _streakline_grid(t0, t1, Nstrip, dt)
    w = pot.integrate_orbit(w0=prog_w0, ts=ts, dt=h).ys
    x, v = w[:, :3], w[:, 3:]
    L_close, L_far = pot.lagrange_pts(x, v, Msat, torch.as_tensor(ts, device=x.device))
    om = pot.omega(x, v)
    rh = x / torch.linalg.norm(x, dim=1, keepdim=True)
    ph = v / torch.linalg.norm(v, dim=1, keepdim=True)
    sin_t = torch.linalg.norm(torch.linalg.cross(rh, ph, dim=1), dim=1)
    v_lead = (om * torch.linalg.norm(L_close, dim=1) / sin_t)[:, None] * ph
    v_trail = (om * torch.linalg.norm(L_far, dim=1) / sin_t)[:, None] * ph
    return L_close, v_lead, L_far, v_trail, ts


def gen_streakline(pot, prog_w0, Msat, t0, t1, Nstrip, solver=None, rtol=1e-6, atol=1e-6, dt=None,
                   precision="f64"):
    """Streakline stream (streamhelpers.py:708-732): the particles of
    get_Streakline_ICs, each integrated from its release time to t1 (the last
    pair, released at t1, is its initial state).  One stream launch: release
    r is particles 2r (from L_close, 'lead') and 2r + 1 (L_far, 'trail'),
    starting at step r * steps_per_release.  precision 'f64' or 'f32k'.
    Returns (lead [Nstrip, 6], trail [Nstrip, 6], ts)."""
    ts, h, spr = _streakline_grid(t0, t1, Nstrip, dt)
    L_close, v_lead, L_far, v_trail, _ = get_Streakline_ICs(pot, prog_w0, Msat, t0, t1, Nstrip, solver=solver,
                                                            dt=dt)
    n = len(ts)
    ics = torch.stack([torch.cat([L_close, v_lead], 1), torch.cat([L_far, v_trail], 1)], 1).reshape(2 * n, 6)
    cfg = _abi.ss_stream_cfg()
    cfg.t0, cfg.dt, cfg.n_steps, cfg.n_particles = float(ts[0]), float(h), (n - 1) * spr, 2 * n
    cfg.particles_per_release, cfg.steps_per_release, cfg.snap_stride = 2, spr, 0
    final, _ = _core.stream(pot._desc(), cfg, ics.contiguous(), precision)
    final = final.reshape(n, 2, 6)
    return final[:, 0], final[:, 1], ts


def computed_binned_track(stream, phi1, bins=20):
    """Mean 6-D state in phi1 bins (streamhelpers.py:201-228).

    Same conventions as the reference: edges = linspace(min, max, bins),
    bin = digitize(phi1, edges), output row b is the nan-mean of the items
    with bin == b for b = 0..bins-2 (so row 0 and the last interval stay
    empty, as in the reference), and empty or exactly-zero means are NaN."""
    s = f64(stream).reshape(-1, 6)
    key = f64(phi1).reshape(-1)
    lo, hi = float(key.min()), float(key.max())
    edges = f64(np.linspace(lo, hi, int(bins)))
    sums, counts = _core.binned_sums(s, key, edges)
    mean = sums / counts
    return torch.where(mean == 0, torch.full_like(mean, float("nan")), mean)


def compute_stream_length(stream, phi1, bins=20):
    """Length of the stream's binned mean track (streamhelpers.py:230-243):
    the summed distances between consecutive bin means (positions), NaN
    bins skipped."""
    m = computed_binned_track(stream, phi1, bins)[:, :3]
    seg = torch.linalg.norm(m[1:] - m[:-1], dim=1)
    return torch.nansum(seg)


def compute_length_oscillations(pot, prog_today, first_stripped_lead, first_stripped_trail, t_age, length_today, *,
                                dt=None, n_samples=2_000):
    """Stream length through time from orbital oscillations
    (streamhelpers.py:246-303): the progenitor and the first stripped leading
    and trailing stars are integrated back t_age from t = 0 (one ensemble of
    three FP64 orbits, saved at 2000 times); the length is length_today times
    the quadrature sum of the two arm separations relative to today's.
    Returns dict(ts [increasing], length_func)."""
    t_age = float(host64(t_age))
    ts = np.linspace(0.0, -t_age, int(n_samples))
    w = torch.stack([f64(first_stripped_lead).reshape(6), f64(first_stripped_trail).reshape(6),
                     f64(prog_today).reshape(6)])
    ys = pot.integrate_orbit(w0=w, ts=ts, t0=0.0, t1=-t_age, dt=dt).ys  # [3, n, 6]
    diff = torch.sqrt(torch.sum((ys[0, :, :3] - ys[2, :, :3]) ** 2 + (ys[1, :, :3] - ys[2, :, :3]) ** 2, dim=1))
    diff_flip = torch.flip(diff, dims=[0])
    amp = diff_flip / diff_flip[-1]
    return dict(ts=torch.as_tensor(ts[::-1].copy(), device=diff.device), length_func=float(host64(length_today)) * amp)


def sample_from_1D_pdf(x, y, key, num_samples):
    """Inverse-CDF samples of the density y(x) (streamhelpers.py:306-349):
    y normalised by its trapezoid integral, CDF = cumulative sum normalised
    to 1, samples = interp(u, CDF, x) for u ~ U(0, 1) (numpy PCG64 seeded
    from `key`)."""
    from .subhalostatistics import seed_of
    xh = np.asarray(host64(x), dtype=np.float64).reshape(-1)
    yh = np.asarray(host64(y), dtype=np.float64).reshape(-1)
    pdf = yh / np.trapezoid(yh, xh)
    cdf = np.cumsum(pdf)
    cdf = cdf / cdf[-1]
    u = np.random.default_rng(seed_of(key)).uniform(size=int(num_samples))
    return np.interp(u, cdf, xh)


def release_model_Chen25(pot_base, key, x, v, Msat, t, normals=None):
    """Chen+25 6-D Gaussian release at one time (streamhelpers.py:352-432).

    `key` seeds numpy's PCG64 (JAX keys are not available)."""
    if normals is None:
        normals = release_normals(int(np.asarray(key).ravel()[-1]), 1, 1, 6)[0]
    w = torch.cat([f64(x).reshape(1, 3), f64(v).reshape(1, 3)], dim=1)
    ics, _ = pot_base._release(w, [float(host64(t))], Msat, np.asarray(host64(normals)).reshape(1, 1, 6),
                               model=_abi.SS_RELEASE_CHEN25, chen=(CHEN25_MEAN, chen25_factor()))
    o = ics[0, 0]
    return o[0, :3], o[1, :3], o[0, 3:], o[1, 3:]


def gen_stream_ics_Chen25(pot_base=None, ts=None, prog_w0=None, Msat=None, key=None, solver=None, rtol=1e-7,
                          atol=1e-7, dtmin=0.3, dtmax=None, max_steps=10_000, *, dt=None, normals=None):
    """streamhelpers.py:434-459: returns ([pos_close, pos_far, vel_close, vel_far], progenitor Solution)."""
    from .main import Solution
    ts_h = host64(ts).reshape(-1)
    ws, _, _ = pot_base._prog_orbit(ts_h, prog_w0, dt, dtmin, dtmax)
    if normals is None:
        normals = release_normals(int(np.asarray(key).ravel()[-1]), len(ts_h), 1, 6)
    ics, _ = pot_base._release(ws, ts_h, Msat, normals, model=_abi.SS_RELEASE_CHEN25,
                               chen=(CHEN25_MEAN, chen25_factor()))
    return list(_split_ics(ics, 1)), Solution(torch.as_tensor(ts_h, device=ws.device), ws)


def gen_stream_vmapped_Chen25(pot_base, ts, prog_w0, Msat, key, solver=None, rtol=1e-7, atol=1e-7, dtmin=0.3,
                              dtmax=None, max_steps=10_000, throw=False, prog_pot=None, *, dt=None,
                              precision="f64", snapshot_every=None, normals=None, n_particles_per_release=2):
    """Chen+25 stream with the progenitor's own potential moving on its
    orbit (streamhelpers.py:491-543)."""
    if prog_pot is None:
        prog_pot = _pot.PlummerPotential(m=0.0, r_s=1.0, units=pot_base.units)
    seed = int(np.asarray(key).ravel()[-1])
    return gen_stream(pot_base, ts, prog_w0, Msat, seed, solver=solver, dt=dt, dtmax=dtmax, release="chen25",
                      prog_pot=prog_pot, precision=precision, snapshot_every=snapshot_every, normals=normals,
                      n_particles_per_release=n_particles_per_release, throw=throw)


def gen_stream_ics_pert_Chen25(pot_base=None, pot_pert=None, ts=None, prog_w0=None, Msat=None, key=None, solver=None,
                               rtol=1e-7, atol=1e-7, dtmin=0.3, dtmax=None, max_steps=10_000, *, dt=None,
                               normals=None):
    """Chen+25 release in the smooth potential from a progenitor orbit
    integrated in base + perturbation (streamhelpers.py:462-489)."""
    from .main import Solution
    ts_h = host64(ts).reshape(-1)
    total = _pot.Potential_Combine([pot_base, pot_pert], units=pot_base.units)
    ws, _, _ = total._prog_orbit(ts_h, prog_w0, dt, dtmin, dtmax)
    if normals is None:
        normals = release_normals(int(np.asarray(key).ravel()[-1]), len(ts_h), 1, 6)
    ics, _ = pot_base._release(ws, ts_h, Msat, normals, model=_abi.SS_RELEASE_CHEN25,
                               chen=(CHEN25_MEAN, chen25_factor()))
    return list(_split_ics(ics, 1)), Solution(torch.as_tensor(ts_h, device=ws.device), ws)


def gen_stream_vmapped_with_pert_Chen25(pot_base=None, pot_pert=None, prog_pot=None, ts=None, prog_w0=None, Msat=None,
                                        key=None, solver=None, max_steps=10_000, rtol=1e-7, atol=1e-7, dtmin=0.1, *,
                                        dt=None, precision="f64", normals=None, n_particles_per_release=2,
                                        snapshot_every=None):
    """Chen+25 perturbed stream: progenitor orbit in base + perturbation,
    particles in base + perturbation + the progenitor's potential moving on
    that orbit (streamhelpers.py:546-598)."""
    if prog_pot is None:
        prog_pot = _pot.PlummerPotential(m=0.0, r_s=1.0, units=pot_base.units)
    seed = None if key is None else int(np.asarray(key).ravel()[-1])
    return gen_stream(pot_base, ts, prog_w0, Msat, seed, solver=solver, dt=dt, release="chen25", prog_pot=prog_pot,
                      pot_pert=pot_pert, prog_in_pert=True, precision=precision, normals=normals,
                      n_particles_per_release=n_particles_per_release, snapshot_every=snapshot_every)


def gen_stream_vmapped_with_pert_Chen25_fixed_prog(pot_base=None, pot_pert=None, prog_pot=None, ts=None, prog_w0=None,
                                                   Msat=None, key=None, solver=None, max_steps=10_000, rtol=1e-7,
                                                   atol=1e-7, dtmin=0.1, *, dt=None, precision="f64", normals=None,
                                                   n_particles_per_release=2, snapshot_every=None):
    """Chen+25 perturbed stream with the unperturbed progenitor orbit (its
    potential still moves on that orbit) (streamhelpers.py:601-653)."""
    if prog_pot is None:
        prog_pot = _pot.PlummerPotential(m=0.0, r_s=1.0, units=pot_base.units)
    seed = None if key is None else int(np.asarray(key).ravel()[-1])
    return gen_stream(pot_base, ts, prog_w0, Msat, seed, solver=solver, dt=dt, release="chen25", prog_pot=prog_pot,
                      pot_pert=pot_pert, prog_in_pert=False, precision=precision, normals=normals,
                      n_particles_per_release=n_particles_per_release, snapshot_every=snapshot_every)


__all__ = ["gen_stream", "gen_stream_batches", "eval_dense_stream", "eval_dense_stream_id", "gen_stream_ics_pert",
           "gen_stream_vmapped_with_pert", "gen_stream_vmapped_with_pert_fixed_prog", "gen_stream_scan_with_pert",
           "custom_release_model", "computed_binned_track", "gen_stream_ensemble", "gen_stream_ensemble_batches",
           "compute_stream_length",
           "compute_length_oscillations", "sample_from_1D_pdf", "release_model_Chen25", "gen_stream_ics_Chen25",
           "gen_stream_vmapped_Chen25", "gen_stream_ics_pert_Chen25", "gen_stream_vmapped_with_pert_Chen25",
           "gen_stream_vmapped_with_pert_Chen25_fixed_prog", "chen25_factor", "CHEN25_MEAN", "CHEN25_COV",
           "get_Streakline_ICs", "gen_streakline"]
