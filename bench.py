#!/usr/bin/env python
"""Benchmark: particle-steps/s of particle-spray stream generation on GB300.

Workload (default, --workload c2): NFW (5.4e11, 15.62) + Miyamoto-Nagai
(6.8e10, 3.0, 0.28) + Hernquist (5e9, 1.0) in kpc/Myr/Msun; progenitor at
present day (12, 0, 4) kpc, (0, 0.18, 0.04) kpc/Myr, integrated back 4 Gyr
and forward with fixed-step Dopri5 at dt = 0.5 Myr (FP64); 4000 release
times (1 Myr apart) x 250 particles (125 Fardal draws x lead/trail) = 1e6
particles; the progenitor's Plummer (2e4 Msun, 0.01 kpc) moves on its cubic
track; float32 snapshots every 50 steps [160, 1e6, 6] (3.84 GB, larger than
L2).  One step = one whole stream run (progenitor back/forward orbit,
release, stream integration with snapshots).  Inputs are seeded synthetic
Gaussian draws (numpy PCG64).

`value` is the FP32-compensated path; the same line carries the FP64 plain
path beside it, the FP32-vs-FP64 error with each track's FP64 conditioning,
both paths against the CPU oracle on a 100-release sample (parity_vs_oracle),
the end-to-end figure through the public API with host buffers, and one block
per other configuration: c1 (config 1 in full, FP64 and FP32, every particle
against the oracle), c3 (the first-order response at full size), c4 (the
learned force surrogate) and c5 (the adjoint gradient).  `--impl reference`
times the CPU FP64 restatement of the reference algorithm (the oracle;
OpenMP on all host cores) on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-steps/s on 1 GB300: FP64 plain vs FP32/MLP-force at stated error"
UNIT = "particle-steps/s"
WF = np.array([12.0, 0.0, 4.0, 0.0, 0.18, 0.04])
MSAT = 2e4
WORKLOADS = {
    "c2": dict(n_rel=4000, ppr=250, dt=0.5, spr=2, snap=50, moving=True,
               name="spray stream, 4000 releases x 250 particles (1e6), 4 Gyr at dt=0.5 Myr, NFW+MN+Hernquist "
                    "+ moving Plummer progenitor, float32 snapshots every 50 steps"),
    "c2s": dict(n_rel=4000, ppr=50, dt=0.5, spr=2, snap=50, moving=True,
                name="profiling case shaped like c2: 4000 releases x 50 particles (2e5), 4 Gyr at dt=0.5 Myr, "
                     "NFW+MN+Hernquist + moving Plummer progenitor, float32 snapshots every 50 steps"),
    "c2f": dict(n_rel=1000, ppr=100, dt=0.5, spr=2, snap=50, moving=True,
                name="profiling case for the FP64 kernel, shaped like c2: 1000 releases x 100 particles (1e5), "
                     "1 Gyr at dt=0.5 Myr, NFW+MN+Hernquist + moving Plummer progenitor, snapshots every 50 steps"),
    "c4x": dict(n_rel=3000, ppr=334, dt=1.0, spr=1, snap=0, moving=False, potential="expansion",
                name="spray stream, 3000 releases x 334 particles (1.0e6), 3 Gyr at dt=1 Myr, triaxial halo as a "
                     "spherical-harmonic expansion (l_max=8, 64 log knots over 0.1-200 kpc, seeded 2^-l "
                     "coefficients), exact expansion force, final state only"),
    "c4xs": dict(n_rel=600, ppr=334, dt=1.0, spr=1, snap=0, moving=False, potential="expansion",
                 name="profiling case shaped like the expansion stream: 600 releases x 334 particles (2.0e5), "
                      "600 steps of 1 Myr, spherical-harmonic expansion (l_max=8), final state only"),
    "c1": dict(n_rel=3000, ppr=2, dt=1.0, spr=1, snap=0, moving=False,
               name="spray stream, 3000 releases x 2 particles (6000), 3 Gyr at dt=1 Myr, NFW+MN+Hernquist, "
                    "final state only"),
}


def particle_steps(n_rel, ppr, spr):
    n_steps = n_rel * spr
    return ppr * (n_rel * n_steps - spr * n_rel * (n_rel - 1) // 2)


def config_for(wl):
    """The `config` object of the JSON line, the same in both arms."""
    n_steps = wl["n_rel"] * wl["spr"]
    n_snap = n_steps // wl["snap"] if wl["snap"] else 0
    snap_bytes = n_snap * wl["n_rel"] * wl["ppr"] * 24
    return {"workload": wl["name"], "particles": wl["n_rel"] * wl["ppr"], "n_steps": n_steps,
            "particle_steps_per_step": particle_steps(wl["n_rel"], wl["ppr"], wl["spr"]), "dt_myr": wl["dt"],
            "snapshot_every": wl["snap"],
            "l2": f"512 MB buffer zeroed between timed steps; snapshots ({snap_bytes / 1e9:.2f} GB) exceed L2"
                  if snap_bytes > 129e6 else "512 MB buffer zeroed between timed steps"}


def normals_for(wl, seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    return rng.standard_normal((wl["n_rel"] + 1, wl["ppr"] // 2, 4))


def emit(obj):
    print(json.dumps(obj), flush=True)


# ------------------------------------------------------------ clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_id: str):
        self.gpu_id = gpu_id
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", self.gpu_id], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out, _ = self.proc.communicate()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "samples": len(sm),
                "reasons": sorted(reasons)}


def gpu_id_for(local_rank: int) -> str:
    vis = os.environ.get("CUDA_VISIBLE_DEVICES")
    if vis:
        ids = [x.strip() for x in vis.split(",") if x.strip()]
        if local_rank < len(ids):
            return ids[local_rank]
    return str(local_rank)


# ------------------------------------------------------------ CPU legs
CPU_NATURE = ("the CPU oracle: a C++ FP64 restatement of the reference's fixed-step path that takes every "
              "gradient by forward-mode dual numbers (as the reference takes them by jax.grad), built -O3 without "
              "-march, OpenMP over particles; not a tuned CPU port")


def oracle_sample(wl, normals, n_sample_rel, threads, gpu_inputs=None):
    """Time the CPU FP64 oracle on `n_sample_rel` evenly spaced releases of
    the workload (all their particles, full length).

    The oracle computes its own progenitor orbit and release (outside the
    timed region).  With gpu_inputs = (ics [N, 6], ws [n_rel + 1, 6]) it
    integrates the GPU run's initial conditions on the GPU run's progenitor
    track instead, so that its final states check that run.  Releases run
    one per host thread when a release has fewer particles than there are
    threads, else one at a time with OpenMP over its particles.  Returns a
    dict: work (particle-steps), secs, cores, rels, idx (particle indices
    of the sample, kernel order), finals [n, 6], own_ics [n, 6] (the
    oracle's own release)."""
    from concurrent.futures import ThreadPoolExecutor

    from oracle import oracle as O
    from streamsculptor_gb300 import _abi
    n_rel, ppr, dt, spr = wl["n_rel"], wl["ppr"], wl["dt"], wl["spr"]
    n_steps = n_rel * spr
    base = O.HostModel(O.mw3())
    back = O.orbit(base, WF, 0.0, -dt, n_steps, n_steps)[0, -1]
    t0 = -n_steps * dt
    ws_o = O.orbit(base, back, t0, dt, n_steps, spr)[0]
    ts = t0 + np.arange(n_rel + 1) * spr * dt
    rels = np.unique(np.linspace(0, n_rel - 1, n_sample_rel).astype(np.int64))
    own, _ = O.release(base, ws_o[rels], ts[rels], MSAT, normals[rels])
    own = own.reshape(len(rels) * ppr, 6)
    idx = (rels[:, None] * ppr + np.arange(ppr)[None, :]).reshape(-1)
    ws = ws_o if gpu_inputs is None else np.asarray(gpu_inputs[1])
    src = own if gpu_inputs is None else np.ascontiguousarray(np.asarray(gpu_inputs[0])[idx])
    comps = O.mw3() + ([(_abi.SS_PLUMMER, 1, (MSAT, 0.01))] if wl["moving"] else [])
    integ = O.HostModel(comps, track=(ts[0], spr * dt, ws[:, :3]) if wl["moving"] else None)
    finals = [None] * len(rels)

    def run(j, n_threads):
        r = int(rels[j])
        f, _, _ = O.stream(integ, ts[r], dt, n_steps - r * spr, src[j * ppr:(j + 1) * ppr], ppr, 0,
                           n_threads=n_threads)
        finals[j] = f

    t_start = time.perf_counter()
    if ppr < threads:
        with ThreadPoolExecutor(threads) as ex:
            list(ex.map(lambda j: run(j, 1), range(len(rels))))
    else:
        for j in range(len(rels)):
            run(j, threads)
    secs = time.perf_counter() - t_start
    work = int(sum(ppr * (n_steps - int(r) * spr) for r in rels))
    return {"work": work, "secs": secs, "cores": threads, "rels": rels, "idx": idx,
            "finals": np.concatenate(finals), "own_ics": own}


def reference_arm(args, wl):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    normals = normals_for(wl, 1234)
    n_sample = 24 if args.workload == "c2" else 300
    for _ in range(args.warmup):
        oracle_sample(wl, normals, n_sample, threads)
    work, secs = 0, 0.0
    for _ in range(args.steps):
        o = oracle_sample(wl, normals, n_sample, threads)
        work += o["work"]
        secs += o["secs"]
    v = work / secs
    sample = (f"{n_sample} evenly spaced releases x {wl['ppr']} particles, full length, per step "
              f"({work // args.steps} particle-steps)")
    emit({"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
          "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * secs / args.steps,
          "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
          "data": "synthetic (seeded PCG64 Gaussian draws)",
          "config": config_for(wl),
          "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample,
                           "nature": CPU_NATURE},
          "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
          "note": "reference = CPU FP64 restatement of streamsculptor's path (the JAX reference cannot run: "
                  "jax/diffrax/astropy/gala are not installed); OpenMP over particles on all host threads"})


# ------------------------------------------------------------ GPU side
def prel(a, b):
    """Per-particle relative phase-space error max(|dx|/|x|, |dv|/|v|), b the reference."""
    import torch
    return torch.maximum(torch.linalg.norm(a[:, :3] - b[:, :3], dim=1) / torch.linalg.norm(b[:, :3], dim=1),
                         torch.linalg.norm(a[:, 3:] - b[:, 3:], dim=1) / torch.linalg.norm(b[:, 3:], dim=1))


def quant(x, q):
    import torch
    return float(torch.quantile(x.float(), q))


def err_stats(e):
    return {"max": float(e.max()), "p99": quant(e, 0.99), "median": float(e.median()),
            "frac_above_1e-5": float((e > 1e-5).double().mean())}


def measure_peak(precision, dev):
    """Best of 3 FMA-chain launches (ss_peak_fma): 32 scalar FP32, 2 packed
    FP32 pairs (the paired stream kernel's form), 64 FP64; TFLOP/s."""
    import ctypes as C

    import torch

    from streamsculptor_gb300 import _abi, _core
    sink = torch.empty(1024, dtype=torch.float32, device=dev)
    fl = C.c_double()
    iters = {32: 100000, 2: 50000, 64: 3000}[precision]
    _abi.call("ss_peak_fma", precision, iters, C.byref(fl), _core.ptr(sink), _core.stream_handle())
    torch.cuda.synchronize()
    best = 0.0
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        _abi.call("ss_peak_fma", precision, iters, C.byref(fl), _core.ptr(sink), _core.stream_handle())
        e1.record()
        torch.cuda.synchronize()
        best = max(best, fl.value / (e0.elapsed_time(e1) * 1e-3) / 1e12)
    return best


PEAK_SOURCE = ("measured in this run by ss_peak_fma (eight FMA chains per thread, 8 blocks of 256 per SM; the "
               "FP32 figure in the packed f32x2 form the paired kernel issues, the scalar form beside it); "
               "MEASURED_PEAKS.json has no FP32/FP64 pipe figure")


class Spray:
    """One particle-spray workload on this GPU through the public API:
    progenitor orbit back (FP64), release, stream (gen_stream)."""

    def __init__(self, wl, dev, seed=1234):
        import torch

        import streamsculptor_gb300 as ss
        from streamsculptor_gb300 import potential as P
        self.wl, self.dev = wl, dev
        u = ss.usys
        if wl.get("potential") == "expansion":
            self.pot = P.seeded_triaxial_expansion(units=u)
        else:
            self.pot = P.Potential_Combine([P.NFWPotential(m=5.4e11, r_s=15.62, units=u),
                                            P.MiyamotoNagaiDisk(m=6.8e10, a=3.0, b=0.28, units=u),
                                            P.HernquistPotential(m=5e9, r_s=1.0, units=u)], units=u)
        self.prog = P.PlummerPotential(m=MSAT, r_s=0.01, units=u) if wl["moving"] else None
        self.n_rel, self.ppr, self.dt, self.spr, self.snap = wl["n_rel"], wl["ppr"], wl["dt"], wl["spr"], wl["snap"]
        self.n_steps = self.n_rel * self.spr
        self.T = self.n_steps * self.dt
        self.ts = -self.T + np.arange(self.n_rel + 1) * self.spr * self.dt
        self.N = self.n_rel * self.ppr
        self.work = particle_steps(self.n_rel, self.ppr, self.spr)
        self.normals_h = normals_for(wl, seed)
        self.normals_d = torch.as_tensor(self.normals_h, device=dev)
        self.wf_d = torch.as_tensor(WF, device=dev)

    def back(self, wf):
        return self.pot.integrate_orbit(w0=wf, ts=np.array([0.0, -self.T]), t0=0.0, t1=-self.T, dt=self.dt).ys[-1]

    def step(self, precision, snapshots=True, **kw):
        from streamsculptor_gb300.streamhelpers import gen_stream
        return gen_stream(self.pot, self.ts, self.back(self.wf_d), MSAT, normals=kw.pop("normals", self.normals_d),
                          dt=self.dt, prog_pot=self.prog, n_particles_per_release=self.ppr, precision=precision,
                          snapshot_every=(self.snap or None) if snapshots else None, **kw)

    def finals(self, precision):
        """(final states [N, 6] in kernel order, initial conditions [N, 6],
        progenitor states at the release times) of one run."""
        import torch
        lead, trail, ics, ws = self.step(precision, snapshots=False, return_ics=True)
        return torch.stack([lead, trail], dim=-2).reshape(-1, 6), ics[:self.n_rel].reshape(-1, 6).contiguous(), ws

    def direct(self, ws):
        """The stream potential and config gen_stream builds, for direct
        ss_stream_* calls on other initial conditions."""
        from streamsculptor_gb300 import _abi, potential as P
        from streamsculptor_gb300.streamhelpers import CenterTrack
        integ = self.pot
        if self.prog is not None:
            track = CenterTrack.from_samples(self.ts, ws[:, :3])
            integ = P.Potential_Combine([self.pot, P.TimeDepTranslatingPotential(self.prog, track,
                                                                                 units=self.pot.units)],
                                        units=self.pot.units)
        cfg = _abi.ss_stream_cfg()
        cfg.t0, cfg.dt, cfg.n_steps, cfg.n_particles = float(self.ts[0]), float(self.dt), self.n_steps, self.N
        cfg.particles_per_release, cfg.steps_per_release, cfg.snap_stride = self.ppr, self.spr, 0
        return integ, cfg

    def timed(self, precision, K, W, flush, barrier=lambda: None, world=1):
        import torch
        import torch.distributed as dist

        from streamsculptor_gb300 import _abi, _core
        lib = _abi.load()
        for _ in range(W):
            self.step(precision)
        torch.cuda.synchronize()
        barrier()
        evs, kev = [], []
        _core.STREAM_EVENTS = kev
        l0 = lib.ss_kernel_launches()
        clocks = ClockSampler(gpu_id_for(self.dev.index or 0))
        clocks.start()
        for _ in range(K):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            self.step(precision)
            e1.record()
            evs.append((e0, e1))
        torch.cuda.synchronize()
        barrier()
        ck = clocks.stop()
        launches = lib.ss_kernel_launches() - l0
        _core.STREAM_EVENTS = None
        ms = sum(a.elapsed_time(b) for a, b in evs)
        kms = [a.elapsed_time(b) for a, b in kev]
        if world > 1:
            t = torch.tensor([ms], device=self.dev, dtype=torch.float64)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            ms = float(t.item())
        return {"ms_total": ms, "ms_per_step": ms / K, "kernel_ms": statistics.mean(kms) if kms else None,
                "samples_ms": [a.elapsed_time(b) for a, b in evs], "launches": launches, "clocks": ck,
                "steps": K, "warmup": W}

    def timed_pipelined(self, K, W, flush, barrier=lambda: None, world=1):
        """The same K FP32-compensated steps as timed('f32k') (the
        progenitor's orbit back from the present, its forward orbit, the
        release, the track tables and the stream with snapshots) through the
        public gen_stream_batches: each step's orbits, release and tables run
        on a side stream while the previous step's stream kernel fills the
        GPU.  The L2 flush stays between consecutive stream kernels."""
        import torch
        import torch.distributed as dist

        from streamsculptor_gb300 import _abi, _core
        from streamsculptor_gb300.streamhelpers import gen_stream_batches
        lib = _abi.load()

        def run(n, evs=None):
            for out in gen_stream_batches(self.pot, self.ts, self.wf_d, MSAT, self.normals_d, n_batches=n,
                                          dt=self.dt, prog_pot=self.prog, n_particles_per_release=self.ppr,
                                          precision="f32k", snapshot_every=self.snap or None, prog_w0_at="end"):
                del out
                flush.zero_()
                if evs is not None:
                    ev = torch.cuda.Event(enable_timing=True)
                    ev.record()
                    evs.append(ev)

        run(W)
        torch.cuda.synchronize()
        barrier()
        kev = []
        _core.STREAM_EVENTS = kev
        l0 = lib.ss_kernel_launches()
        clocks = ClockSampler(gpu_id_for(self.dev.index or 0))
        clocks.start()
        e0 = torch.cuda.Event(enable_timing=True)
        e0.record()
        evs = []
        run(K, evs)
        torch.cuda.synchronize()
        barrier()
        ck = clocks.stop()
        launches = lib.ss_kernel_launches() - l0
        _core.STREAM_EVENTS = None
        ms = e0.elapsed_time(evs[-1])
        marks = [e0] + evs
        samples = [a.elapsed_time(b) for a, b in zip(marks[:-1], marks[1:])]
        if world > 1:
            t = torch.tensor([ms], device=self.dev, dtype=torch.float64)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            ms = float(t.item())
        return {"ms_total": ms, "ms_per_step": ms / K, "kernel_ms": statistics.mean(a.elapsed_time(b) for a, b in kev),
                "samples_ms": samples, "launches": launches, "clocks": ck, "steps": K, "warmup": W}

    def roofline(self, r, precision, kernel, peak):
        from streamsculptor_gb300 import _core, potential as P, roofline
        parts = [self.pot]
        if self.prog is not None:
            parts.append(P.TimeDepTranslatingPotential(self.prog, _core.CenterTrack(0.0, 1.0, self.wf_d.reshape(2, 3)),
                                                       units=self.pot.units))
        flat = P.Potential_Combine(parts, units=self.pot.units)._flatten()
        w = roofline.particle_step_work(flat, precision)
        ach = w["flops"] * self.work / (r["kernel_ms"] * 1e-3) / 1e12
        n_snap = self.n_steps // self.snap if self.snap else 0
        return {"kernel": kernel, "bound": "fp32" if "f32" in precision else "fp64", "achieved": ach,
                "peak": peak, "unit": "TFLOP/s", "frac": ach / peak, "traffic": traffic_for(kernel),
                "flops_per_particle_step": w["flops"], "specials_per_particle_step": w["specials"],
                "kernel_ms": r["kernel_ms"], "peak_source": PEAK_SOURCE,
                "snapshot_write_GBps": (n_snap * self.N * 24) / (r["kernel_ms"] * 1e-3) / 1e9 if n_snap else 0.0}


def conditioning(spray, X0, ws, F64, n_dir=4, eps=1e-10):
    """Growth of each FP64 track: for n_dir random directions, the initial
    state is moved by eps relative in position and in velocity and the
    relative change of the final state is divided by eps; the largest over
    the directions (one direction can miss the most sensitive one).  Tracks
    that pass close by the progenitor's core amplify any rounding, FP64's
    included."""
    import torch

    from streamsculptor_gb300 import _core
    integ, cfg = spray.direct(ws)
    desc = integ._desc()
    g = torch.Generator(device=spray.dev).manual_seed(5)
    G = None
    for _ in range(n_dir):
        d = torch.randn(X0.shape, generator=g, device=spray.dev, dtype=torch.float64)
        d[:, :3] *= (eps * torch.linalg.norm(X0[:, :3], dim=1) / torch.linalg.norm(d[:, :3], dim=1))[:, None]
        d[:, 3:] *= (eps * torch.linalg.norm(X0[:, 3:], dim=1) / torch.linalg.norm(d[:, 3:], dim=1))[:, None]
        Xk = (X0 + d).contiguous()
        Fk, _ = _core.stream(desc, cfg, Xk, "f64")
        gk = prel(Fk, F64) / prel(Xk, X0).clamp_min(1e-300)
        G = gk if G is None else torch.maximum(G, gk)
    return G


def oracle_parity(spray, orc, F64, F32, G=None):
    """Final states of the GPU FP64 and FP32 paths against the oracle's
    integration of the same initial conditions (oracle_sample with
    gpu_inputs); ics_max: the GPU's progenitor orbit and release against
    the oracle's own, on the sampled releases."""
    import torch
    idx = torch.as_tensor(orc["idx"], device=spray.dev)
    Fo = torch.as_tensor(orc["finals"], device=spray.dev)
    e64, e32 = prel(F64[idx], Fo), prel(F32[idx], Fo)
    out = {"particles": int(idx.numel()), "releases": int(len(orc["rels"])),
           "f64_max": float(e64.max()), "f64_p99": quant(e64, 0.99),
           "f32k_max": float(e32.max()), "f32k_p99": quant(e32, 0.99), "f32k_median": float(e32.median()),
           "frac_f32k_above_1e-5": float((e32 > 1e-5).double().mean())}
    if G is not None:
        Gs = G[idx]
        reg = Gs <= 1e4
        out["f64_max_growth_le_1e4"] = float(e64[reg].max()) if bool(reg.any()) else None
        out["frac_growth_above_1e4"] = float((~reg).double().mean())
        out["f64_over_growth_max"] = float((e64 / Gs).max())
    return out


def ics_vs_oracle(X0, orc, dev):
    import torch
    own = torch.as_tensor(orc["own_ics"], device=dev)
    return float(prel(X0[torch.as_tensor(orc["idx"], device=dev)], own).max())


def gpu_arm(args, wl):
    import torch
    import torch.distributed as dist

    from streamsculptor_gb300 import _core

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl", init_method="env://")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    s = Spray(wl, dev, seed=1234 + rank)  # weak scaling: every rank runs its own stream
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)  # > L2 (129 MB)

    def barrier():
        if world > 1:
            dist.barrier()

    precisions = args.precisions.split(",")
    if len(precisions) == 1:
        # one precision alone (profiling runs)
        r1 = s.timed(precisions[0], args.steps, args.warmup, flush, barrier, world)
        if rank == 0:
            emit({"metric": METRIC, "value": world * s.work / (r1["ms_per_step"] * 1e-3), "unit": UNIT,
                  "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": r1["ms_per_step"],
                  "kernel_ms": r1["kernel_ms"], "config": config_for(wl), "clocks": r1["clocks"],
                  "gpu_launches": r1["launches"], "note": f"{precisions[0]} only (profiling run)"})
        return
    # --- headline: FP32-compensated, inputs resident; K steps one after the
    # other, then the same K steps pipelined (gen_stream_batches: a step's
    # orbits and release overlap the previous step's stream kernel)
    r32s = s.timed("f32k", args.steps, args.warmup, flush, barrier, world)
    r32 = s.timed_pipelined(args.steps, args.warmup, flush, barrier, world)
    value = world * s.work / (r32["ms_per_step"] * 1e-3)
    # --- e2e through the public API with host buffers (right after the device timing)
    from streamsculptor_gb300.streamhelpers import gen_stream
    n_snap = s.n_steps // s.snap if s.snap else 0
    normals_pin = torch.as_tensor(s.normals_h).pin_memory()
    host_out = _core.host_buffers(s.N, n_snap)  # caller-owned pinned outputs, reused by every call

    def e2e_step(mode):
        # public API with host inputs and host outputs: gen_stream(out="host");
        # "direct": the stream kernel writes its snapshots into the pinned
        # host buffer; "chunked": particle sub-ranges copied by the copy
        # engine while the next sub-range integrates
        sol = s.pot.integrate_orbit(w0=WF, ts=np.array([0.0, -s.T]), t0=0.0, t1=-s.T, dt=s.dt)
        out = gen_stream(s.pot, s.ts, sol.ys[-1], MSAT, normals=normals_pin, dt=s.dt, prog_pot=s.prog,
                         n_particles_per_release=s.ppr, precision="f32k", snapshot_every=s.snap or None,
                         out="host", out_buffers=host_out, host_mode=mode)
        assert not out[0].is_cuda
        torch.cuda.synchronize()

    for mode in ("direct", "chunked"):
        for _ in range(2):
            e2e_step(mode)
    k_e2e = max(1, min(2 * args.steps, 10))
    e2e_samples, chunked_samples = [], []
    e2e_clk = ClockSampler(gpu_id_for(local))
    e2e_clk.start()
    for _ in range(k_e2e):
        # the two host paths alternate, so both see the same conditions
        for mode, dst in (("direct", e2e_samples), ("chunked", chunked_samples)):
            flush.zero_()
            torch.cuda.synchronize()
            barrier()
            t0 = time.perf_counter()
            e2e_step(mode)
            barrier()
            dst.append((time.perf_counter() - t0) * 1e3)
    e2e_clocks = e2e_clk.stop()
    e2e_s = statistics.mean(e2e_samples) * 1e-3
    if world > 1:
        t = torch.tensor([e2e_s], device=dev, dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
    h2d = s.normals_h.nbytes + s.ts.nbytes + WF.nbytes + 2 * 8
    d2h = s.N * 6 * 8 + n_snap * s.N * 6 * 4  # final states + snapshots
    del host_out

    # --- FP64 plain beside it
    k64 = max(1, min(args.steps, args.f64_steps))
    r64 = s.timed("f64", k64, max(1, min(args.warmup, args.f64_warmup)), flush, barrier, world)
    value64 = world * s.work / (r64["ms_per_step"] * 1e-3)
    p32, p2, p64 = measure_peak(32, dev), measure_peak(2, dev), measure_peak(64, dev)
    line = None
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": r32["ms_per_step"], "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None,
                "dtype": "f32 (compensated hi+lo state; FP64 progenitor orbit, time and release)",
                "data": "synthetic (seeded PCG64 Gaussian draws)", "config": config_for(wl),
                "f64": {"value": value64, "unit": UNIT, "ms_per_step": r64["ms_per_step"], "steps": k64,
                        "clocks": r64["clocks"], "roofline": s.roofline(r64, "f64", "stream_f64_kernel", p64)},
                "speedup_f32k_vs_f64": value / value64,
                "roofline": dict(s.roofline(r32, "f32k2", "stream_f32k2_kernel", p2), peak_scalar_fma=p32,
                                 alone=s.roofline(r32s, "f32k2", "stream_f32k2_kernel", p2),
                                 note="kernel_ms over the pipelined steps (the stream kernel shares the GPU with the "
                                      "next step's orbits); 'alone': over the sequential steps"),
                "e2e": {"value": world * s.work / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                        "d2h_bytes_per_step": int(d2h), "ms_per_step": e2e_s * 1e3,
                        "ms_median": statistics.median(e2e_samples), "samples_ms": e2e_samples,
                        "clocks": e2e_clocks,
                        "path": "integrate_orbit + streamhelpers.gen_stream(out='host', out_buffers=...) with "
                                "pinned host inputs: the stream kernel writes its snapshot rows straight into the "
                                "caller-owned pinned host buffer, the final states are copied after it",
                        "chunked": {"ms_mean": statistics.mean(chunked_samples),
                                    "ms_median": statistics.median(chunked_samples),
                                    "samples_ms": chunked_samples,
                                    "path": "gen_stream(out='host', host_mode='chunked'): 8 particle sub-ranges, "
                                            "each copied by the copy engine while the next integrates"}},
                "samples_ms": r32["samples_ms"], "clocks": r32["clocks"], "gpu_launches": r32["launches"],
                "timing": "the K steps through gen_stream_batches (each step's progenitor orbits, release and track "
                          "tables on a side stream while the previous step's stream kernel runs; every step does "
                          "all of its work); 'sequential': the same K steps one after the other",
                "sequential": {"value": world * s.work / (r32s["ms_per_step"] * 1e-3), "ms_per_step": r32s["ms_per_step"],
                               "kernel_ms": r32s["kernel_ms"], "samples_ms": r32s["samples_ms"],
                               "clocks": r32s["clocks"]},
                "gpu_launches_per_step": r32["launches"] / args.steps}
    if not args.no_analysis:
        # --- the stated error: FP32 vs FP64 on the same inputs, the FP64
        # tracks' conditioning, the same without the progenitor's gravity,
        # and both paths against the oracle
        F32, X0, ws = s.finals("f32k")
        F64, _, _ = s.finals("f64")
        e = prel(F32, F64)
        G = conditioning(s, X0, ws, F64)
        reg = G <= 1e3
        err = dict(err_stats(e), measure="per particle max(|dx|/|x|, |dv|/|v|) of final states, "
                                         "FP32-compensated vs FP64 GPU path, same initial conditions")
        err["conditioning"] = {
            "perturbation": "4 random directions, 1e-10 relative in x and in v; growth = max over directions "
                            "of the final state's relative change / 1e-10",
            "growth_median": float(G.median()), "growth_p99": quant(G, 0.99), "growth_max": float(G.max()),
            "frac_growth_above_1e3": float((~reg).double().mean()),
            "max_err_growth_le_1e3": float(e[reg].max()), "p99_err_growth_le_1e3": quant(e[reg], 0.99),
            "frac_err_above_1e-5_growth_le_1e3": float(((e > 1e-5) & reg).double().mean()),
            "max_err_over_growth_growth_le_1e3": float((e / G)[reg].max()),
            "median_err_over_growth": float((e / G).median())}
        if s.prog is not None:
            # the same initial conditions without the progenitor's self-gravity
            from streamsculptor_gb300 import _core as CC
            cfg = s.direct(ws)[1]
            f32n, _ = CC.stream(s.pot._desc(), cfg, X0, "f32k")
            f64n, _ = CC.stream(s.pot._desc(), cfg, X0, "f64")
            err["without_progenitor_gravity"] = err_stats(prel(f32n, f64n))
            del f32n, f64n
        if rank == 0:
            line["error_vs_f64"] = err
            if world == 1 and not args.no_cpu_baseline:
                orc = oracle_sample(wl, s.normals_h, 100, os.cpu_count() or 1,
                                    gpu_inputs=(X0.cpu().numpy(), ws.cpu().numpy()))
                line["cpu_baseline"] = {
                    "value": orc["work"] / orc["secs"], "unit": UNIT, "cores": orc["cores"], "kind": "port",
                    "sample": f"CPU FP64 oracle (OpenMP) on 100 evenly spaced releases x {s.ppr} particles, full "
                              f"length ({orc['work']} particle-steps, {orc['secs']:.1f} s)", "nature": CPU_NATURE}
                line["parity_vs_oracle"] = dict(oracle_parity(s, orc, F64, F32, G), ics_max=ics_vs_oracle(X0, orc, dev),
                                                sample="the cpu_baseline sample: the oracle integrates this run's "
                                                       "initial conditions on this run's progenitor track")
                line["speedup_f64_gpu_vs_cpu_oracle"] = value64 / line["cpu_baseline"]["value"]
        del F32, F64, X0, G, e
    if rank == 0 and world == 1 and not args.no_legs:
        torch.cuda.empty_cache()
        line["c1"] = c1_leg(dev, flush)
        line["c3"] = c3_run(dev, 2, 1)
        line["c5"] = c5_run(dev, 3, 2)
        line["c4"] = c4_run(dev, args, 2, 1)
    if rank == 0:
        emit(line)
    if world > 1:
        dist.destroy_process_group()


# ------------------------------------------------------------ config 1
def c1_leg(dev, flush):
    """Config 1 in full: the plain FP64 path and the FP32 form, timed
    through the public API; both against the oracle on every particle."""
    import torch
    wl = WORKLOADS["c1"]
    s = Spray(wl, dev)
    r64 = s.timed("f64", 5, 3, flush)
    r32 = s.timed("f32k", 10, 3, flush)
    F64, X0, ws = s.finals("f64")
    F32, _, _ = s.finals("f32k")
    orc = oracle_sample(wl, s.normals_h, wl["n_rel"], os.cpu_count() or 1,
                        gpu_inputs=(X0.cpu().numpy(), ws.cpu().numpy()))
    p2, p64 = measure_peak(2, dev), measure_peak(64, dev)
    out = {"workload": wl["name"], "particle_steps_per_step": s.work,
           "f64": {"value": s.work / (r64["ms_per_step"] * 1e-3), "unit": UNIT, "ms_per_step": r64["ms_per_step"],
                   "steps": r64["steps"], "warmup": r64["warmup"], "clocks": r64["clocks"],
                   "roofline": s.roofline(r64, "f64", "stream_f64_split_kernel", p64)},
           "f32k": {"value": s.work / (r32["ms_per_step"] * 1e-3), "unit": UNIT, "ms_per_step": r32["ms_per_step"],
                    "steps": r32["steps"], "warmup": r32["warmup"], "clocks": r32["clocks"],
                    "roofline": s.roofline(r32, "f32k2", "stream_f32k2_kernel", p2)},
           "error_f32k_vs_f64": err_stats(prel(F32, F64)),
           "parity_vs_oracle": dict(oracle_parity(s, orc, F64, F32), ics_max=ics_vs_oracle(X0, orc, dev),
                                    sample="every particle; the oracle integrates this run's initial conditions"),
           "note": "6000 particles on 152 SMs: the FP64 time is set by the longest tracks' serial step chain "
                   "(3000 steps), not by the FP64 pipe; the FP64 run takes the component-split kernel (one warp "
                   "per potential component, 188 blocks of 3 warps)"}
    del F64, F32, X0
    torch.cuda.synchronize()
    return out


# ------------------------------------------------------------ config 3
C3 = dict(n_rel=2000, ppr=50, dt=1.0, n_sh=1000, ncol=6,
          name="first-order response: 2000 releases x 50 particles (1e5) x 1000 Plummer subhalos "
               "(log10 M ~ U(5,8), r_s = 1.62 kpc (M/1e8)^0.5, x0 uniform in 30 kpc, v ~ N(0, 0.12 kpc/Myr), "
               "always active), 2 Gyr at dt = 1 Myr, FP32 response (6 mass columns), FP64 base track and time")
C3S = dict(C3, n_rel=200, name="profiling case shaped like config 3: 200 releases x 50 particles x 1000 subhalos, "
                                 "200 steps")


def c3_subhalos(n, seed=3):
    rng = np.random.Generator(np.random.PCG64(seed))
    m = 10 ** rng.uniform(5, 8, n)
    a = 1.62 * np.sqrt(m / 1e8)
    d = rng.normal(size=(n, 3))
    x0 = d / np.linalg.norm(d, axis=1, keepdims=True) * (30.0 * rng.uniform(size=(n, 1)) ** (1 / 3))
    v = rng.normal(0, 0.12, (n, 3))
    return m, a, x0, v


def c3_run(dev, K, W, c3=C3):
    """The first-order response at config 3's size: (particle x subhalo)-steps/s
    of ss_pert_response (FP32 response, FP64 base track), its roofline, and
    its error against the FP64 response on the last 200 releases."""
    import torch

    import streamsculptor_gb300 as ss
    from streamsculptor_gb300 import _abi, _core, potential as P, roofline
    u = ss.usys
    pot = P.Potential_Combine([P.NFWPotential(m=5.4e11, r_s=15.62, units=u),
                               P.MiyamotoNagaiDisk(m=6.8e10, a=3.0, b=0.28, units=u),
                               P.HernquistPotential(m=5e9, r_s=1.0, units=u)], units=u)
    n_rel, ppr, dt, nsh, ncol = c3["n_rel"], c3["ppr"], c3["dt"], c3["n_sh"], c3["ncol"]
    T = n_rel * dt
    ts = -T + np.arange(n_rel + 1) * dt
    back = pot.integrate_orbit(w0=WF, ts=np.array([0.0, -T]), t0=0.0, t1=-T, dt=dt).ys[-1]
    normals = np.random.Generator(np.random.PCG64(77)).standard_normal((n_rel + 1, ppr // 2, 4))
    ws, _, _ = pot._prog_orbit(ts, back, dt)
    ics, _ = pot._release(ws, ts, MSAT, normals)
    base = ics[:n_rel].reshape(-1, 6).contiguous()
    m, a, x0, v = c3_subhalos(nsh)
    table = _core.SubhaloTable(_abi.SS_SH_PLUMMER, _core.f64(m), _core.f64(a), _core.f64(x0), _core.f64(v),
                               _core.f64(np.full(nsh, ts[0])), float("inf"))

    def cfg_for(r0):
        cfg = _abi.ss_pert_cfg()
        cfg.t0, cfg.dt, cfg.n_steps, cfg.n_particles = float(ts[r0]), dt, n_rel - r0, (n_rel - r0) * ppr
        cfg.particles_per_release, cfg.steps_per_release, cfg.ncol, cfg.save_stride = ppr, 1, ncol, 0
        return cfg

    cfg = cfg_for(0)
    Pd = pot._desc()
    work = ppr * (n_rel * n_rel - n_rel * (n_rel - 1) // 2) * nsh
    for _ in range(W):
        _core.pert_response(Pd, table, cfg, 32, base, None)
    torch.cuda.synchronize()
    l0 = _abi.load().ss_kernel_launches()
    ms = 0.0
    clocks = ClockSampler(gpu_id_for(dev.index or 0))
    clocks.start()
    for _ in range(K):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        _core.pert_response(Pd, table, cfg, 32, base, None)
        e1.record()
        torch.cuda.synchronize()
        ms += e0.elapsed_time(e1)
    ck = clocks.stop()
    launches = _abi.load().ss_kernel_launches() - l0
    ms /= K
    # the two phases apart, through the stored-track entry points
    # (ss_pert_base_track, then ss_pert_response_track on its track): the
    # response kernel's own time for the roofline
    tb = tr = 0.0
    for it in range(W + K):
        e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        e0.record()
        track, _ = _core.pert_base_track(Pd, cfg, 32, base)
        e1.record()
        resp = _core.pert_response_track(table, pot._G, cfg, 32, track, None)
        e2.record()
        torch.cuda.synchronize()
        if it >= W:
            tb += e0.elapsed_time(e1)
            tr += e1.elapsed_time(e2)
        del track, resp
    tb, tr = tb / K, tr / K
    # error of the FP32 response against the FP64 one on the last 200 releases
    r0 = max(0, n_rel - 200)
    sub = base[r0 * ppr:].contiguous()
    _, o32 = _core.pert_response(Pd, table, cfg_for(r0), 32, sub, None)
    _, o64 = _core.pert_response(Pd, table, cfg_for(r0), 64, sub, None)
    d = (o32.double() - o64).abs()
    scale = o64.abs().amax(dim=(0, 1, 2))  # per column
    err = {"max_abs_over_column_max": float((d.amax(dim=(0, 1, 2)) / scale).max()),
           "sample": f"the last {n_rel - r0} releases x {ppr} particles x {nsh} subhalos, FP32 vs FP64 response"}
    w = roofline.response_step_work(ncol)
    peak = measure_peak(2, dev)  # the response kernel issues packed f32x2 FMAs (two subhalos per thread)
    ach = w["flops"] * work / (tr * 1e-3) / 1e12
    del o32, o64, d
    return {"metric": "(particle x subhalo)-steps/s, first-order response", "value": work / (ms * 1e-3),
            "unit": "(particle x subhalo)-steps/s", "ms_per_step": ms, "steps": K, "warmup": W,
            "dtype": "f32 response, f64 base track", "config": {"workload": c3["name"], "system_steps_per_step": work},
            "error_vs_f64_response": err, "clocks": ck, "gpu_launches": launches,
            "roofline": {"kernel": "pert_response2_kernel", "bound": "fp32", "achieved": ach, "peak": peak,
                         "unit": "TFLOP/s", "frac": ach / peak, "traffic": traffic_for("pert_response2_kernel"),
                         "flops_per_system_step": w["flops"], "specials_per_system_step": w["specials"],
                         "kernel_ms": tr, "base_track_ms": tb,
                         "kernel_ms_note": "kernel_ms: the response phase alone (ss_pert_response_track on a stored "
                                           "base track, CUDA events); base_track_ms: the FP64 base-track phase "
                                           "(ss_pert_base_track, pert_base_kernel)",
                         "peak_source": "measured in this run by ss_peak_fma (packed f32x2 FMA chains)"}}


def c3_arm(args):
    import torch
    torch.cuda.set_device(0)
    c3 = C3S if args.workload == "c3s" else C3
    r = c3_run(torch.device("cuda", 0), args.steps, args.warmup, c3)
    emit(dict(r, n_gpus=1, higher_is_better=True, data="synthetic (seeded)"))


# ------------------------------------------------------------ config 5
C5 = dict(n_rel=2000, spr=2, dt=1.0, ppr=50,
          name="gradient of a 64-bin stream-track loss w.r.t. 14 parameters (TriaxialNFW M, r_s, q; MN M, a, b; "
               "Hernquist M, c; progenitor w0): 2000 releases x 50 particles (1e5), 4000 steps of 1 Myr, FP32 "
               "forward with checkpoints every 64 steps, hand-written adjoint")


def c5_run(dev, K, W):
    import torch

    from streamsculptor_gb300 import adjoint as A
    model = A.TriaxialHaloModel
    theta = np.array([5.4e11, 15.62, 0.9, 6.8e10, 3.0, 0.28, 5e9, 1.0, 12.0, 0.0, 4.0, 0.0, 0.18, 0.04])
    rng = np.random.Generator(np.random.PCG64(5))
    setup = A.StreamSetup(n_rel=C5["n_rel"], spr=C5["spr"], dt=C5["dt"], ppr=C5["ppr"], msat=MSAT,
                          normals=rng.standard_normal((C5["n_rel"] + 1, C5["ppr"] // 2, 4)))
    theta_t = theta * (1 + 0.01 * rng.standard_normal(14)) + np.r_[np.zeros(8), 0.05 * rng.standard_normal(3),
                                                                    1e-3 * rng.standard_normal(3)]
    loss = A.TrackLoss(theta[-6:], A.forward_stream(model, theta_t, setup), n_bins=64)
    work = setup.ppr * (setup.n_rel * setup.n_steps - setup.spr * setup.n_rel * (setup.n_rel - 1) // 2)

    def fwd():
        return A.forward_stream(model, theta, setup, keep=True)

    def grad(final, saved):
        f = final.detach().requires_grad_(True)
        L = loss(f)
        L.backward()
        return A.backward_stream(model, theta, setup, saved, f.grad)

    for _ in range(W):
        final, saved = fwd()
        grad(final, saved)
    torch.cuda.synchronize()
    tf, tb = 0.0, 0.0
    clocks = ClockSampler(gpu_id_for(dev.index or 0))
    clocks.start()
    for _ in range(K):
        e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        e0.record()
        final, saved = fwd()
        e1.record()
        g = grad(final, saved)
        e2.record()
        torch.cuda.synchronize()
        tf += e0.elapsed_time(e1)
        tb += e1.elapsed_time(e2)
    ck = clocks.stop()
    return {"metric": "adjoint gradient cost / forward stream cost", "value": tb / tf, "unit": "ratio",
            "higher_is_better": False, "target": "<= 3", "steps": K, "warmup": W,
            "forward_ms": tf / K, "gradient_ms": tb / K,
            "forward_particle_steps_per_s": work / (tf / K * 1e-3), "dtype": "f32 forward and adjoint, f64 progenitor",
            "config": {"workload": C5["name"], "particle_steps": work}, "clocks": ck,
            "grad_norm": float(torch.linalg.norm(g)),
            "gradient_check": "tests/test_gpu_adjoint.py: central finite differences (h = 1e-4 relative) of the "
                              "FP64 oracle, 14 parameters"}


def c5_arm(args):
    import torch
    torch.cuda.set_device(0)
    r = c5_run(torch.device("cuda", 0), args.steps, args.warmup)
    emit(dict(r, n_gpus=1, data="synthetic (seeded)"))


C4 = dict(n_rel=3000, ppr=334, dt=1.0, spr=1,
          name="learned force surrogate: 3000 releases x 334 particles (1.0e6), 3 Gyr at dt=1 Myr in a triaxial halo "
               "given as a spherical-harmonic expansion (l_max=8, 64 log knots over 0.1-200 kpc, seeded 2^-l "
               "coefficients); MLP (x,y,z,ln r) -> Phi, 4 x 128 SiLU, trained on 2^22 orbit points, forces from its "
               "hand-written backward on the tensor cores (BF16, FP32 accumulation)")
# tensor-core work of one surrogate force: layers 2-4 forward + 3 backward
# GEMMs of 128 x 128 per particle (2 flops per multiply-add)
MLP_TENSOR_FLOPS = 6 * 2 * 128 * 128


def c4_run(dev, args, K, W):
    """The learned force surrogate (config 4): training on the GPU, the
    surrogate stream at full size, the exact FP32 expansion beside it, and
    both against the FP64 exact expansion on a 600-release sample."""
    import torch

    import streamsculptor_gb300 as ss
    from streamsculptor_gb300 import _abi, _core, potential as P
    from streamsculptor_gb300.streamhelpers import gen_stream
    from streamsculptor_gb300.surrogate import MLPSurrogate, orbit_samples, residual_targets

    lib = _abi.load()
    u = ss.usys
    pot = P.seeded_triaxial_expansion(units=u)
    n_rel, ppr, dt = args.c4_releases, C4["ppr"], C4["dt"]
    T = n_rel * dt
    ts = -T + np.arange(n_rel + 1) * dt
    work = particle_steps(n_rel, ppr, 1)
    normals_h = np.random.Generator(np.random.PCG64(1234)).standard_normal((n_rel + 1, ppr // 2, 4))
    normals_d = torch.as_tensor(normals_h, device=dev)
    # --- training set and training (timed separately)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    x = orbit_samples(pot, WF, n_orbits=args.c4_points // 1024, n_per_orbit=1024, seed=0)
    # the network learns Phi minus the expansion's exact l = 0 term, which
    # every evaluation adds back; the force loss is relative to the total force
    phi, g, base = residual_targets(pot, x)
    g_scale = torch.linalg.norm(pot.gradient(x, 0.0), dim=1)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    sur = MLPSurrogate.init(seed=0, **MLPSurrogate.normalisation(x.cpu(), phi.cpu())).with_base(*base)
    sur.fit(x, phi, g, steps=args.c4_train_steps, batch=8192, lr=3e-3, seed=0,
            log_every=max(1, args.c4_train_steps // 5), force_scale=g_scale)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    xv = orbit_samples(pot, WF, n_orbits=64, n_per_orbit=256, seed=7)
    gv = pot.gradient(xv, 0.0)
    _, g32 = sur.potential_and_gradient(xv)
    g16 = sur.gradient_bf16(xv)
    nrm = torch.linalg.norm(gv, dim=1)
    e32 = torch.linalg.norm(g32 - gv, dim=1) / nrm
    e16 = torch.linalg.norm(g16 - gv, dim=1) / nrm
    del x, phi, g, g_scale
    back = pot.integrate_orbit(w0=WF, ts=np.array([0.0, -T]), t0=0.0, t1=-T, dt=dt).ys[-1]

    def step(precision, normals):
        return gen_stream(pot, ts, back, MSAT, normals=normals, dt=dt, n_particles_per_release=ppr,
                          precision=precision, force_surrogate=sur if precision == "mlp" else None)

    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)

    def timed(precision, K, W):
        for _ in range(W):
            step(precision, normals_d)
        torch.cuda.synchronize()
        evs, kev = [], []
        _core.STREAM_EVENTS = kev
        l0 = lib.ss_kernel_launches()
        clk = ClockSampler(gpu_id_for(0))
        clk.start()
        for _ in range(K):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            step(precision, normals_d)
            e1.record()
            evs.append((e0, e1))
        torch.cuda.synchronize()
        ck = clk.stop()
        _core.STREAM_EVENTS = None
        return {"ms_per_step": sum(a.elapsed_time(b) for a, b in evs) / K,
                "kernel_ms": statistics.mean(a.elapsed_time(b) for a, b in kev), "clocks": ck,
                "launches": lib.ss_kernel_launches() - l0}

    rm = timed("mlp", K, W)
    rx = timed("f32k", 1, 1)
    lm = step("mlp", normals_d)
    lx = step("f32k", normals_d)
    a = torch.stack([lm[0], lm[1]]).reshape(-1, 6)
    b = torch.stack([lx[0], lx[1]]).reshape(-1, 6)
    ex = torch.linalg.norm(a[:, :3] - b[:, :3], dim=1) / torch.linalg.norm(b[:, :3], dim=1)
    ev = torch.linalg.norm(a[:, 3:] - b[:, 3:], dim=1) / torch.linalg.norm(b[:, 3:], dim=1)
    e = torch.maximum(ex, ev)
    # FP64 exact expansion on a 600-release sub-workload (600 steps): its rate,
    # and the surrogate's and the FP32 path's final-state errors against it
    n_s = min(600, n_rel)
    T_s = n_s * dt
    back_s = pot.integrate_orbit(w0=WF, ts=np.array([0.0, -T_s]), t0=0.0, t1=-T_s, dt=dt).ys[-1]
    ts_s = -T_s + np.arange(n_s + 1) * dt
    nrm_s = normals_d[:n_s + 1].contiguous()

    def sub(precision):
        return gen_stream(pot, ts_s, back_s, MSAT, normals=nrm_s, dt=dt, n_particles_per_release=ppr,
                          precision=precision, force_surrogate=sur if precision == "mlp" else None)

    sub("f64")
    kev64 = []
    _core.STREAM_EVENTS = kev64
    r64 = sub("f64")
    torch.cuda.synchronize()
    _core.STREAM_EVENTS = None
    k64_ms = kev64[0][0].elapsed_time(kev64[0][1])
    work_s = particle_steps(n_s, ppr, 1)
    b64 = torch.stack([r64[0], r64[1]]).reshape(-1, 6)

    def err_vs(o):
        q = torch.stack([o[0], o[1]]).reshape(-1, 6)
        ex_ = torch.linalg.norm(q[:, :3] - b64[:, :3], dim=1) / torch.linalg.norm(b64[:, :3], dim=1)
        ev_ = torch.linalg.norm(q[:, 3:] - b64[:, 3:], dim=1) / torch.linalg.norm(b64[:, 3:], dim=1)
        e_ = torch.maximum(ex_, ev_)
        return {"median": float(e_.median()), "p99": float(torch.quantile(e_.float(), 0.99)), "max": float(e_.max())}

    sub_errs = {"f32k": err_vs(sub("f32k")), "mlp": err_vs(sub("mlp"))}
    # the exact expansion as the surrogate's error judge and fallback: every
    # 64 steps each 128-particle tile compares its surrogate force with the
    # exact one and takes the exact force for good where any particle is off
    # by more than tol
    judged = {}
    for tol in (1e-2, 1e-3):
        j = dict(tol=tol, every=64)
        kwj = dict(dt=dt, n_particles_per_release=ppr, precision="mlp", force_surrogate=sur)
        gen_stream(pot, ts, back, MSAT, normals=normals_d, surrogate_judge=dict(j), **kwj)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        gen_stream(pot, ts, back, MSAT, normals=normals_d, surrogate_judge=j, **kwj)
        e1.record()
        torch.cuda.synchronize()
        ms_j = e0.elapsed_time(e1)
        js = dict(tol=tol, every=64)
        oj = gen_stream(pot, ts_s, back_s, MSAT, normals=nrm_s, surrogate_judge=js, **kwj)
        judged[f"tol_{tol:g}"] = {"value": work / (ms_j * 1e-3), "ms_per_step": ms_j, "fallback_tiles": j["fallbacks"],
                                  "tiles": j["tiles"], "error_vs_exact_f64_sample": err_vs(oj),
                                  "sample_fallback_tiles": js["fallbacks"], "sample_tiles": js["tiles"]}
    # e2e: host normals in, final states to pinned host memory
    pin = torch.empty((2, n_rel, ppr // 2, 6), dtype=torch.float64, pin_memory=True)
    torch.cuda.synchronize()
    t3 = time.perf_counter()
    for _ in range(K):
        out = step("mlp", normals_h)
        pin[0].copy_(out[0], non_blocking=True)
        pin[1].copy_(out[1], non_blocking=True)
    torch.cuda.synchronize()
    e2e_s = (time.perf_counter() - t3) / K
    peak = MEASURED_BF16_TFLOPS
    ach = MLP_TENSOR_FLOPS * 6 * work / (rm["kernel_ms"] * 1e-3) / 1e12
    return ({"metric": METRIC, "value": work / (rm["ms_per_step"] * 1e-3), "unit": UNIT, "n_gpus": 1,
          "steps": K, "warmup": W, "ms_per_step": rm["ms_per_step"], "higher_is_better": True,
          "scaling": "weak", "vs_baseline": None, "dtype": "bf16 tensor-core force (FP32 accumulation), f32 "
          "compensated state, f64 progenitor and release",
          "data": "synthetic (seeded expansion, PCG64 draws; training points along orbits of the exact expansion)",
          "config": {"workload": C4["name"] if n_rel == C4["n_rel"] else
                     f"profiling case shaped like the surrogate workload: {n_rel} releases x {ppr} particles",
                     "particles": n_rel * ppr, "n_steps": n_rel, "particle_steps_per_step":
                     work, "l2": "512 MB buffer zeroed between timed steps"},
          "exact_expansion_f32k": {"value": work / (rx["ms_per_step"] * 1e-3), "ms_per_step": rx["ms_per_step"],
                                   "kernel_ms": rx["kernel_ms"]},
          "speedup_vs_exact_expansion": rx["ms_per_step"] / rm["ms_per_step"],
          "exact_expansion_f64": {"value": work_s / (k64_ms * 1e-3), "kernel_ms": k64_ms,
                                  "sample": f"{n_s} releases x {ppr} particles, {n_s} steps ({work_s} particle-steps)",
                                  "note": "stream kernel time only"},
          "error_vs_exact_f64_sample": sub_errs,
          "judged": judged,
          "verdict": {"target": "MLP-force stream at <= 1e-5 relative phase-space error vs the FP64 oracle, >= 10x "
                                "faster than the plain FP64 path",
                      "median_error_vs_exact_f64": sub_errs["mlp"]["median"],
                      "meets_1e-5": bool(sub_errs["mlp"]["max"] <= 1e-5),
                      "speedup_vs_fp64_exact": (work / (rm["ms_per_step"] * 1e-3)) / (work_s / (k64_ms * 1e-3)),
                      "speedup_vs_fp32_exact": rx["ms_per_step"] / rm["ms_per_step"],
                      "note": "the exact l_max = 8 expansion costs ~3.2 kflop per force on the CUDA cores against "
                              "~1.2 Mflop of tensor-core work per particle-step for the network: on GB300 the "
                              "surrogate cannot beat the exact FP32 expansion it replaces"},
          "surrogate": {"train_points": int(args.c4_points), "train_steps": args.c4_train_steps, "batch": 8192,
                        "form": "network on Phi minus the expansion's l = 0 term, which is added exactly",
                        "sample_s": t1 - t0, "train_s": t2 - t1, "loss_history": sur.history,
                        "force_rel_err_fp32": {"median": float(e32.median()), "p99": float(torch.quantile(e32.float(), 0.99))},
                        "force_rel_err_bf16": {"median": float(e16.median()), "p99": float(torch.quantile(e16.float(), 0.99))}},
          "error_vs_exact_expansion": {"median": float(e.median()), "p99": float(torch.quantile(e.float(), 0.99)),
                                       "max": float(e.max()), "measure": "per particle max(|dx|/|x|, |dv|/|v|) of "
                                       "final states, surrogate stream vs exact-expansion FP32-compensated stream"},
          "roofline": {"kernel": "stream_mlp_kernel", "bound": "tensor", "achieved": ach, "peak": peak,
                       "unit": "TFLOP/s", "frac": ach / peak, "traffic": None,
                       "flops_per_particle_step": MLP_TENSOR_FLOPS * 6, "kernel_ms": rm["kernel_ms"],
                       "peak_source": "MEASURED_PEAKS.json bf16_tflops (cuBLAS burst)"},
          "e2e": {"value": work / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(normals_h.nbytes),
                  "d2h_bytes_per_step": int(pin.numel() * 8), "ms_per_step": e2e_s * 1e3},
          "clocks": rm["clocks"], "gpu_launches": rm["launches"]})


def c4_arm(args):
    import torch
    torch.cuda.set_device(0)
    emit(c4_run(torch.device("cuda", 0), args, args.steps, args.warmup))


# ------------------------------------------------------------ GD-1 batch
GD1 = dict(n_samples=700, n_rel=2000, t_age=2500.0, t_dissolve=-300.0, msat=1e4, seed=532, t_window=100.0,
           wtoday=np.array([-4.0, 1.0, 13.0, -0.20, -0.12, 0.04]),
           name="batch of 700 perturbed streams (the reference's GD-1 subhalo-fitting batch): Gala Milky Way "
                "(NFW + Miyamoto-Nagai + two Hernquist), ts = [linspace(-2500, -300, 2000), 0] Myr, 4000 "
                "particles per stream, one Plummer subhalo per stream (t_window 100 Myr) placed on the "
                "unperturbed stream by ImpactGenerator from the notebook's prior, each progenitor integrated "
                "back 2.5 Gyr and forward in base + its own subhalo; fixed dt = 1.1 Myr")


def gd1_setup(n_samples, n_batches):
    """Unperturbed stream, its phi1, and n_batches x n_samples subhalos drawn
    from the notebook's prior and placed on the stream by ImpactGenerator."""
    import torch

    import streamsculptor_gb300 as ss
    from streamsculptor_gb300 import potential as P
    from streamsculptor_gb300.GenerateImpactParams import ImpactGenerator
    from streamsculptor_gb300.streamhelpers import gen_stream

    u = ss.usys
    pot = P.GalaMilkyWayPotential(units=u)
    ts = np.concatenate([np.linspace(-GD1["t_age"], GD1["t_dissolve"], GD1["n_rel"]), [0.0]])
    h = float(ts[1] - ts[0])
    n_back = int(np.ceil(GD1["t_age"] / h))
    ic = pot.integrate_orbit(w0=GD1["wtoday"], ts=np.array([-GD1["t_age"]]), t0=0.0, t1=-GD1["t_age"],
                             dt=GD1["t_age"] / n_back).ys[0]
    normals = np.random.Generator(np.random.PCG64(GD1["seed"])).standard_normal((len(ts), 1, 4))
    lead, trail = gen_stream(pot, ts, ic, GD1["msat"], normals=normals)
    stream = torch.cat([lead, trail]).double()
    w = torch.as_tensor(GD1["wtoday"], device=stream.device)
    e1 = w[:3] / torch.linalg.norm(w[:3])
    L = torch.linalg.cross(w[:3], w[3:], dim=0)
    e2 = torch.linalg.cross(L / torch.linalg.norm(L), e1, dim=0)
    phi1 = torch.rad2deg(torch.atan2(stream[:, :3] @ e2, stream[:, :3] @ e1))
    tstrip = np.concatenate([ts[:-1], ts[:-1]])
    rng = np.random.Generator(np.random.PCG64(8942))
    p1 = phi1.cpu().numpy()
    lo, hi = np.percentile(p1, 10), np.percentile(p1, 90)
    gen = ImpactGenerator(pot=pot, tobs=0.0, stream=stream, stream_phi1=phi1, stripping_times=tstrip,
                          prog_today=GD1["wtoday"], phi1window=0.8, NumImpacts=n_samples,
                          tImpactBounds=[-GD1["t_age"], 0.0], seednum=4)
    perts = []
    for _ in range(n_batches):
        log10_m = rng.uniform(6.0, 7.0, n_samples)
        log10_a = rng.uniform(np.log10(0.01), np.log10(0.2), n_samples)
        phi1_0 = rng.uniform(lo, hi, n_samples)
        t_imp = -10 ** rng.uniform(1.0, np.log10(2000.0), n_samples)
        b_imp = 10 ** rng.uniform(-5.0, np.log10(0.5), n_samples)
        perp = rng.uniform(0.0, 2 * np.pi, n_samples)
        means, tm = gen.get_particle_mean(phi1_0)
        xv, _ = gen._get_subhalo_ImpactParamsCartesian(0.0, means, tm, t_imp, b_imp, perp, np.arange(n_samples))
        xv = xv.cpu().numpy()
        perts.append(P.SubhaloLinePotential(10 ** log10_m, 10 ** log10_a, xv[:, :3], xv[:, 3:], t_imp,
                                            GD1["t_window"], units=u))
    return pot, perts, ts, normals


def gd1_arm(args):
    """Batches of 700 perturbed streams: each sample's progenitor is
    integrated back 2.5 Gyr from today and forward in base + its own subhalo
    (FP64 ensemble orbits), released (FP64) and its 4000 particles
    integrated (FP32 compensated; FP64 beside it).  Timed: K batches through
    gen_stream_ensemble_batches, which overlaps batch i + 1's latency-bound
    orbits with batch i's streams; the latency of one batch alone is
    reported beside it."""
    import torch

    from streamsculptor_gb300 import _abi
    from streamsculptor_gb300 import streamhelpers as H
    from streamsculptor_gb300.streamhelpers import gen_stream_ensemble, gen_stream_ensemble_batches

    torch.cuda.set_device(0)
    B = GD1["n_samples"]
    K, W = args.steps, args.warmup
    pot, perts, ts, normals = gd1_setup(B, max(K, args.f64_steps) + 1)
    n_rel = GD1["n_rel"]
    tail = int(np.ceil((ts[-1] - ts[-2]) / (ts[1] - ts[0]) - 1e-9))
    per_stream = 2 * ((n_rel - 1) * n_rel // 2) + 2 * n_rel * tail
    work = B * per_stream
    kw = dict(Msat=GD1["msat"], normals=normals, prog_w0_at="end")

    def timed(fn):
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        out = fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1), out

    res, outs = {}, {}
    for prec, k in (("f32k", K), ("f64", args.f64_steps)):
        if prec not in args.precisions.split(","):
            continue
        for _ in range(W if prec == "f32k" else 1):
            gen_stream_ensemble_batches(pot, perts[:2], 1, ts, GD1["wtoday"], precision=prec, **kw)
        l0 = _abi.load().ss_kernel_launches()
        clocks = ClockSampler(gpu_id_for(0))
        clocks.start()
        ms, out = timed(lambda: gen_stream_ensemble_batches(pot, perts[1:k + 1], 1, ts, GD1["wtoday"],
                                                            precision=prec, **kw))
        ck = clocks.stop()
        launches = _abi.load().ss_kernel_launches() - l0
        one_ms, _ = timed(lambda: gen_stream_ensemble(pot, perts[0], 1, ts, GD1["wtoday"], precision=prec, **kw))
        # the two halves of one batch alone: FP64 orbits + release, then the streams
        prep_ms, prep = timed(lambda: H._ensemble_prepare(pot, perts[0], 1, ts, GD1["wtoday"], GD1["msat"], None,
                                                          1.0, None, normals, True, "end"))
        run_ms, _ = timed(lambda: H._ensemble_run(prep, prec, False))
        res[prec] = dict(ms=ms / k, one_ms=one_ms, prep_ms=prep_ms, run_ms=run_ms, clocks=ck, launches=launches, k=k)
        outs[prec] = torch.stack(out[0], dim=2).cpu().numpy()  # batch perts[1]: [B, n_rel, 2, 6]
    r = res["f32k"]
    line = {"metric": "particle-steps/s, batches of 700 perturbed streams", "value": work / (r["ms"] * 1e-3),
            "unit": UNIT, "n_gpus": 1, "steps": K, "warmup": W, "ms_per_step": r["ms"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 (compensated) streams; FP64 progenitor orbits and release",
            "data": "synthetic (seeded): a GD-1-like progenitor state and the notebook's subhalo prior",
            "config": {"workload": GD1["name"], "streams": B, "particles_per_stream": 2 * n_rel,
                       "particle_steps_per_step": work, "step": "one batch of 700 streams",
                       "l2": "1.3e8 B of particle state per batch, larger than L2"},
            "s_per_batch": r["ms"] * 1e-3, "s_one_batch_alone": r["one_ms"] * 1e-3,
            "one_batch_split_ms": {"orbits_and_release": r["prep_ms"], "streams": r["run_ms"]},
            "clocks": r["clocks"], "gpu_launches": r["launches"],
            "reference_published": {"value": 11.30, "unit": "s per batch of 700 perturbed GD-1 streams",
                                    "hardware": "NVIDIA A100",
                                    "source": "examples/GD1_and_SubhaloFitting_GPU.ipynb:754",
                                    "note": "adaptive Dopri5 (rtol = atol = 1e-6) in FP64 under jax.vmap, and it "
                                            "includes the KDE likelihood of each stream; not the same step "
                                            "sequence"}}
    if "f64" in res:
        f = res["f64"]
        line["f64"] = {"value": work / (f["ms"] * 1e-3), "unit": UNIT, "s_per_batch": f["ms"] * 1e-3,
                       "s_one_batch_alone": f["one_ms"] * 1e-3, "batches": f["k"], "clocks": f["clocks"],
                       "gpu_launches": f["launches"]}
        a, b = outs["f32k"].reshape(-1, 6), outs["f64"].reshape(-1, 6)
        ex = np.linalg.norm(a[:, :3] - b[:, :3], axis=1) / np.linalg.norm(b[:, :3], axis=1)
        ev = np.linalg.norm(a[:, 3:] - b[:, 3:], axis=1) / np.linalg.norm(b[:, 3:], axis=1)
        e = np.maximum(ex, ev)
        line["error_vs_f64"] = {"median": float(np.median(e)), "p99": float(np.percentile(e, 99)),
                                "max": float(e.max()), "frac_above_1e-5": float((e > 1e-5).mean())}
    emit(line)


def _measured_bf16():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["bf16_tflops"])
    except (OSError, ValueError, KeyError):
        return 1900.0  # fallback figure of the profiling recipe


MEASURED_BF16_TFLOPS = _measured_bf16()


def traffic_for(kernel):
    """DRAM bytes per launch from the committed ncu summary, if present."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(p) as f:
            return json.load(f).get(kernel)
    except (OSError, ValueError):
        return None


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS) + ["c3", "c3s", "c4", "c5", "gd1"], default="c2")
    ap.add_argument("--c4-points", type=int, default=1 << 22, help="surrogate training points (c4)")
    ap.add_argument("--c4-train-steps", type=int, default=6000, help="surrogate Adam steps (c4)")
    ap.add_argument("--c4-releases", type=int, default=C4["n_rel"], help="release times (c4; smaller for profiling)")
    ap.add_argument("--f64-steps", type=int, default=2)
    ap.add_argument("--f64-warmup", type=int, default=1)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-analysis", action="store_true",
                    help="skip the error, conditioning and oracle comparison of the spray workloads")
    ap.add_argument("--no-legs", action="store_true", help="skip the config 1, 3, 4 and 5 blocks of the default run")
    ap.add_argument("--precisions", default="f32k,f64", help="f32k,f64 (default) or f32k alone for profiling")
    args = ap.parse_args()
    if args.workload in ("c3", "c3s"):
        c3_arm(args)
        return
    if args.workload == "c5":
        c5_arm(args)
        return
    if args.workload == "c4":
        c4_arm(args)
        return
    if args.workload == "gd1":
        gd1_arm(args)
        return
    wl = WORKLOADS[args.workload]
    if args.impl == "reference":
        reference_arm(args, wl)
    else:
        gpu_arm(args, wl)


if __name__ == "__main__":
    main()
