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

`value` is the FP32-compensated path (state error vs FP64 reported in the
same line); the FP64 plain path is reported beside it.  `--impl reference`
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
def oracle_sample(wl, normals, n_sample_rel, threads):
    """Time the CPU FP64 oracle on `n_sample_rel` evenly spaced releases of
    the workload (all their particles, full length).  Returns
    (particle_steps, seconds, cores)."""
    from oracle import oracle as O
    from streamsculptor_gb300 import _abi
    n_rel, ppr, dt, spr = wl["n_rel"], wl["ppr"], wl["dt"], wl["spr"]
    n_steps = n_rel * spr
    base = O.HostModel(O.mw3())
    back = O.orbit(base, WF, 0.0, -dt, n_steps, n_steps)[0, -1]
    t0 = -n_steps * dt
    ws = O.orbit(base, back, t0, dt, n_steps, spr)[0]
    ts = t0 + np.arange(n_rel + 1) * spr * dt
    comps = O.mw3() + ([(_abi.SS_PLUMMER, 1, (MSAT, 0.01))] if wl["moving"] else [])
    integ = O.HostModel(comps, track=(ts[0], spr * dt, ws[:, :3]) if wl["moving"] else None)
    rels = np.unique(np.linspace(0, n_rel - 1, n_sample_rel).astype(np.int64))
    ics, _ = O.release(base, ws[rels], ts[rels], MSAT, normals[rels])
    work = 0
    t_start = time.perf_counter()
    for j, r in enumerate(rels):
        nst = n_steps - int(r) * spr
        O.stream(integ, ts[r], dt, nst, ics[j].reshape(-1, 6), ppr, 0, n_threads=threads)
        work += ppr * nst
    return work, time.perf_counter() - t_start, threads


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
        w, s, _ = oracle_sample(wl, normals, n_sample, threads)
        work += w
        secs += s
    v = work / secs
    sample = (f"{n_sample} evenly spaced releases x {wl['ppr']} particles, full length, per step "
              f"({work // args.steps} particle-steps)")
    emit({"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
          "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * secs / args.steps,
          "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
          "data": "synthetic (seeded PCG64 Gaussian draws)",
          "config": {"workload": wl["name"]},
          "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
          "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
          "note": "reference = CPU FP64 restatement of streamsculptor's path (the JAX reference cannot run: "
                  "jax/diffrax/astropy/gala are not installed); OpenMP over particles on all host threads"})


# ------------------------------------------------------------ GPU leg
def gpu_arm(args, wl):
    import torch
    import torch.distributed as dist

    import streamsculptor_gb300 as ss
    from streamsculptor_gb300 import _abi, _core, potential as P, roofline
    from streamsculptor_gb300.streamhelpers import gen_stream

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl", init_method="env://")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    lib = _abi.load()
    u = ss.usys
    if wl.get("potential") == "expansion":
        pot = P.seeded_triaxial_expansion(units=u)
    else:
        pot = P.Potential_Combine([P.NFWPotential(m=5.4e11, r_s=15.62, units=u),
                                   P.MiyamotoNagaiDisk(m=6.8e10, a=3.0, b=0.28, units=u),
                                   P.HernquistPotential(m=5e9, r_s=1.0, units=u)], units=u)
    prog = P.PlummerPotential(m=MSAT, r_s=0.01, units=u) if wl["moving"] else None
    n_rel, ppr, dt, spr, snap = wl["n_rel"], wl["ppr"], wl["dt"], wl["spr"], wl["snap"]
    n_steps = n_rel * spr
    T = n_steps * dt
    ts = -T + np.arange(n_rel + 1) * spr * dt
    work = particle_steps(n_rel, ppr, spr)
    normals_h = normals_for(wl, 1234 + rank)  # weak scaling: every rank runs its own stream
    normals_d = torch.as_tensor(normals_h, device=dev)
    wf_d = torch.as_tensor(WF, device=dev)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)  # > L2 (129 MB)

    def barrier():
        if world > 1:
            dist.barrier()

    def step(precision, wf, normals):
        back = pot.integrate_orbit(w0=wf, ts=np.array([0.0, -T]), t0=0.0, t1=-T, dt=dt).ys[-1]
        return gen_stream(pot, ts, back, MSAT, normals=normals, dt=dt, prog_pot=prog, n_particles_per_release=ppr,
                          precision=precision, snapshot_every=snap or None)

    def timed(precision, K, W):
        for _ in range(W):
            step(precision, wf_d, normals_d)
        torch.cuda.synchronize()
        barrier()
        evs, kev = [], []
        _core.STREAM_EVENTS = kev
        l0 = lib.ss_kernel_launches()
        clocks = ClockSampler(gpu_id_for(local))
        clocks.start()
        for _ in range(K):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            step(precision, wf_d, normals_d)
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
            t = torch.tensor([ms], device=dev, dtype=torch.float64)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            ms = float(t.item())
        return {"ms_total": ms, "ms_per_step": ms / K, "kernel_ms": statistics.mean(kms) if kms else None,
                "launches": launches, "clocks": ck}

    def peak(precision):
        sink = torch.empty(1024, dtype=torch.float32, device=dev)
        import ctypes as C
        fl = C.c_double()
        iters = 100000 if precision == 32 else 3000
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

    precisions = args.precisions.split(",")
    # --- headline: FP32-compensated, inputs resident
    r32 = timed("f32k", args.steps, args.warmup)
    value = world * work / (r32["ms_per_step"] * 1e-3)
    if precisions == ["f32k"]:
        if rank == 0:
            emit({"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                  "warmup": args.warmup, "ms_per_step": r32["ms_per_step"], "kernel_ms": r32["kernel_ms"],
                  "config": {"workload": wl["name"]}, "clocks": r32["clocks"], "gpu_launches": r32["launches"],
                  "note": "f32k only (profiling run)"})
        return
    # --- e2e through the public API with host buffers (right after the device timing)
    n_snap = n_steps // snap if snap else 0

    def e2e_step():
        # public API with host inputs and host outputs: gen_stream(out="host")
        # integrates in particle sub-ranges and copies each one to pinned host
        # memory while the next integrates
        sol = pot.integrate_orbit(w0=WF, ts=np.array([0.0, -T]), t0=0.0, t1=-T, dt=dt)
        out = gen_stream(pot, ts, sol.ys[-1], MSAT, normals=normals_h, dt=dt, prog_pot=prog,
                         n_particles_per_release=ppr, precision="f32k", snapshot_every=snap or None, out="host")
        assert not out[0].is_cuda
        torch.cuda.synchronize()

    for _ in range(2):
        e2e_step()
    # host-side copies on a shared host see occasional slow samples: take up
    # to 10 and report the mean (the value) with the median beside it
    k_e2e = max(1, min(2 * args.steps, 10))
    tsum = 0.0
    e2e_samples = []
    e2e_clk = ClockSampler(gpu_id_for(local))
    e2e_clk.start()
    for _ in range(k_e2e):
        flush.zero_()
        torch.cuda.synchronize()
        barrier()
        t0 = time.perf_counter()
        e2e_step()
        barrier()
        dt_s = time.perf_counter() - t0
        tsum += dt_s
        e2e_samples.append(dt_s * 1e3)
    e2e_clocks = e2e_clk.stop()
    e2e_s = tsum / k_e2e
    if world > 1:
        t = torch.tensor([e2e_s], device=dev, dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
    h2d = normals_h.nbytes + ts.nbytes + WF.nbytes + 2 * 8
    d2h = n_rel * ppr * 6 * 8 + (n_snap * n_rel * ppr * 6 * 4 if snap else 0)  # final states + snapshots

    # --- FP64 plain beside it
    k64 = max(1, min(args.steps, args.f64_steps))
    r64 = timed("f64", k64, max(1, min(args.warmup, args.f64_warmup)))
    value64 = world * work / (r64["ms_per_step"] * 1e-3)

    # --- error of FP32-compensated vs FP64 on this workload
    l32, t32 = step("f32k", wf_d, normals_d)[:2]
    l64, t64 = step("f64", wf_d, normals_d)[:2]
    a = torch.stack([l32, t32]).reshape(-1, 6)
    b = torch.stack([l64, t64]).reshape(-1, 6)
    ex = torch.linalg.norm(a[:, :3] - b[:, :3], dim=1) / torch.linalg.norm(b[:, :3], dim=1)
    ev = torch.linalg.norm(a[:, 3:] - b[:, 3:], dim=1) / torch.linalg.norm(b[:, 3:], dim=1)
    e = torch.maximum(ex, ev)
    err = {"max": float(e.max()), "p99": float(torch.quantile(e.float(), 0.99)), "median": float(e.median()),
           "frac_above_1e-5": float((e > 1e-5).double().mean()),
           "measure": "per particle max(|dx|/|x|, |dv|/|v|) of final states, FP32-compensated vs FP64 GPU path"}
    # Sensitivity of each FP64 track to a tiny independent change of its own
    # initial state (release draws moved by 1e-9): growth = relative change
    # of the final state / relative change of the initial state.  Tracks
    # with close passages by the progenitor amplify any rounding, FP64's
    # included, so the FP32 error is also quoted on the tracks whose growth
    # stays below 1e3.
    def with_ics(nrm):
        back = pot.integrate_orbit(w0=wf_d, ts=np.array([0.0, -T]), t0=0.0, t1=-T, dt=dt).ys[-1]
        o = gen_stream(pot, ts, back, MSAT, normals=nrm, dt=dt, prog_pot=prog, n_particles_per_release=ppr,
                       precision="f64", return_ics=True)
        # particle order (arm, release, draw) as in the error above
        return torch.stack([o[0], o[1]]).reshape(-1, 6), o[2][:n_rel].permute(2, 0, 1, 3).reshape(-1, 6)

    gen = torch.Generator(device=dev).manual_seed(77)
    nrm_p = normals_d + 1e-9 * torch.randn(normals_d.shape, generator=gen, device=dev, dtype=normals_d.dtype)
    b0, ic0 = with_ics(normals_d)
    bp, icp = with_ics(nrm_p)

    def prel(u, v):
        return torch.maximum(torch.linalg.norm(u[:, :3] - v[:, :3], dim=1) / torch.linalg.norm(v[:, :3], dim=1),
                             torch.linalg.norm(u[:, 3:] - v[:, 3:], dim=1) / torch.linalg.norm(v[:, 3:], dim=1))

    growth = prel(bp, b0) / prel(icp, ic0).clamp_min(1e-300)
    regular = growth <= 1e3
    err["fp64_sensitivity"] = {
        "perturbation": "release draws + 1e-9 N(0,1) (independent per particle)",
        "growth_median": float(growth.median()), "growth_p99": float(torch.quantile(growth.float(), 0.99)),
        "growth_max": float(growth.max()), "frac_growth_above_1e3": float((~regular).double().mean()),
        "max_err_growth_le_1e3": float(e[regular].max()) if bool(regular.any()) else None,
        "p99_err_growth_le_1e3": float(torch.quantile(e[regular].float(), 0.99)) if bool(regular.any()) else None,
        "frac_err_above_1e-5_growth_le_1e3": float(((e > 1e-5) & regular).double().mean())}
    del l32, t32, l64, t64, a, b, bp, b0, ic0, icp

    # --- roofline of the dominant kernel (stream_f32k2_kernel: two particles
    # per thread in packed f32x2 lanes)
    flat = P.Potential_Combine([pot] + ([P.TimeDepTranslatingPotential(prog, _core.CenterTrack(0.0, 1.0, wf_d.reshape(2, 3)))]
                                        if prog is not None else []), units=u)._flatten()
    w32 = roofline.particle_step_work(flat, "f32k2")
    w64 = roofline.particle_step_work(flat, "f64")
    p32, p64 = peak(32), peak(64)

    def roof(r, w, pk, kernel):
        ach = w["flops"] * work / (r["kernel_ms"] * 1e-3) / 1e12
        return {"kernel": kernel, "bound": "fp32" if "f32" in kernel else "fp64", "achieved": ach, "peak": pk,
                "unit": "TFLOP/s", "frac": ach / pk, "traffic": traffic_for(kernel),
                "flops_per_particle_step": w["flops"], "specials_per_particle_step": w["specials"],
                "kernel_ms": r["kernel_ms"],
                "peak_source": "measured in this run by ss_peak_fma (FMA chains on every SM); "
                               "MEASURED_PEAKS.json has no FP32/FP64 pipe figure",
                "snapshot_write_GBps": (n_snap * n_rel * ppr * 24) / (r["kernel_ms"] * 1e-3) / 1e9 if snap else 0.0}

    if rank == 0:
        cpu = None
        if world == 1 and not args.no_cpu_baseline:
            cw, cs, cores = oracle_sample(wl, normals_h, 100 if args.workload == "c2" else 3000, os.cpu_count() or 1)
            cpu = {"value": cw / cs, "unit": UNIT, "cores": cores, "kind": "port",
                   "sample": f"CPU FP64 oracle (OpenMP) on 100 evenly spaced releases x {ppr} particles, "
                             f"full length ({cw} particle-steps, {cs:.1f} s)"}
        clk = r32["clocks"]
        emit({"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
              "warmup": args.warmup, "ms_per_step": r32["ms_per_step"], "higher_is_better": True,
              "scaling": "weak", "vs_baseline": None,
              "dtype": "f32 (compensated hi+lo state; FP64 progenitor orbit, time and release)",
              "data": "synthetic (seeded PCG64 Gaussian draws)",
              "config": {"workload": wl["name"], "particles": n_rel * ppr, "n_steps": n_steps,
                         "particle_steps_per_step": work, "dt_myr": dt, "snapshot_every": snap,
                         "l2": "512 MB buffer zeroed between timed steps; snapshots (3.84 GB) exceed L2"},
              "f64": {"value": value64, "unit": UNIT, "ms_per_step": r64["ms_per_step"], "steps": k64,
                      "clocks": r64["clocks"], "roofline": roof(r64, w64, p64, "stream_f64_kernel")},
              "speedup_f32k_vs_f64": value / value64,
              "error_vs_f64": err,
              "roofline": roof(r32, w32, p32, "stream_f32k2_kernel"),
              "cpu_baseline": cpu,
              "e2e": {"value": world * work / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                      "d2h_bytes_per_step": int(d2h), "ms_per_step": e2e_s * 1e3,
                      "ms_median": statistics.median(e2e_samples), "samples_ms": e2e_samples,
                      "clocks": e2e_clocks,
                      "path": "integrate_orbit + streamhelpers.gen_stream(out='host') with host numpy inputs: "
                              "particle sub-ranges copied to pinned host memory while the next integrates"},
              "clocks": clk, "gpu_launches": r32["launches"],
              "gpu_launches_per_step": r32["launches"] / args.steps})
    if world > 1:
        dist.destroy_process_group()


# ------------------------------------------------------------ config 3
C3 = dict(n_rel=2000, ppr=50, dt=1.0, n_sh=1000, ncol=6,
          name="first-order response: 2000 releases x 50 particles (1e5) x 1000 Plummer subhalos "
               "(log10 M ~ U(5,8), r_s = 1.62 kpc (M/1e8)^0.5, x0 uniform in 30 kpc, v ~ N(0, 0.12 kpc/Myr), "
               "always active), 2 Gyr at dt = 1 Myr, FP32 response (6 mass columns), FP64 base track and time")


def c3_subhalos(n, seed=3):
    rng = np.random.Generator(np.random.PCG64(seed))
    m = 10 ** rng.uniform(5, 8, n)
    a = 1.62 * np.sqrt(m / 1e8)
    d = rng.normal(size=(n, 3))
    x0 = d / np.linalg.norm(d, axis=1, keepdims=True) * (30.0 * rng.uniform(size=(n, 1)) ** (1 / 3))
    v = rng.normal(0, 0.12, (n, 3))
    return m, a, x0, v


C3S = dict(C3, n_rel=200, name="profiling case shaped like config 3: 200 releases x 50 particles x 1000 subhalos, "
                                 "200 steps")


def c3_arm(args):
    import torch

    import streamsculptor_gb300 as ss
    from streamsculptor_gb300 import _abi, _core, potential as P

    torch.cuda.set_device(0)
    c3 = C3S if args.workload == "c3s" else C3
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
    cfg = _abi.ss_pert_cfg()
    cfg.t0, cfg.dt, cfg.n_steps, cfg.n_particles = float(ts[0]), dt, n_rel, base.shape[0]
    cfg.particles_per_release, cfg.steps_per_release, cfg.ncol, cfg.save_stride = ppr, 1, ncol, 0
    Pd = pot._desc()
    work = ppr * (n_rel * n_rel - n_rel * (n_rel - 1) // 2) * nsh
    for _ in range(args.warmup):
        _core.pert_response(Pd, table, cfg, 32, base, None)
    torch.cuda.synchronize()
    l0 = _abi.load().ss_kernel_launches()
    ms = 0.0
    clocks = ClockSampler(gpu_id_for(0))
    clocks.start()
    for _ in range(args.steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        _core.pert_response(Pd, table, cfg, 32, base, None)
        e1.record()
        torch.cuda.synchronize()
        ms += e0.elapsed_time(e1)
    ck = clocks.stop()
    launches = _abi.load().ss_kernel_launches() - l0
    emit({"metric": "(particle x subhalo)-steps/s, first-order response", "value": work / (ms / args.steps * 1e-3),
          "unit": "(particle x subhalo)-steps/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
          "ms_per_step": ms / args.steps, "higher_is_better": True, "dtype": "f32 response, f64 base track",
          "data": "synthetic (seeded)", "config": {"workload": c3["name"], "system_steps_per_step": work},
          "clocks": ck, "gpu_launches": launches})


# ------------------------------------------------------------ config 5
C5 = dict(n_rel=2000, spr=2, dt=1.0, ppr=50,
          name="gradient of a 64-bin stream-track loss w.r.t. 14 parameters (TriaxialNFW M, r_s, q; MN M, a, b; "
               "Hernquist M, c; progenitor w0): 2000 releases x 50 particles (1e5), 4000 steps of 1 Myr, FP32 "
               "forward with checkpoints every 64 steps, hand-written adjoint")


def c5_arm(args):
    import torch

    from streamsculptor_gb300 import adjoint as A

    torch.cuda.set_device(0)
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
        th = torch.tensor(theta, dtype=torch.float64, device="cuda", requires_grad=True)
        f = final.detach().requires_grad_(True)
        L = loss(f)
        L.backward()
        return A.backward_stream(model, theta, setup, saved, f.grad)

    for _ in range(args.warmup):
        final, saved = fwd()
        grad(final, saved)
    torch.cuda.synchronize()
    tf, tb = 0.0, 0.0
    for _ in range(args.steps):
        e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        e0.record()
        final, saved = fwd()
        e1.record()
        g = grad(final, saved)
        e2.record()
        torch.cuda.synchronize()
        tf += e0.elapsed_time(e1)
        tb += e1.elapsed_time(e2)
    K = args.steps
    emit({"metric": "adjoint gradient cost / forward stream cost", "value": tb / tf, "unit": "ratio",
          "higher_is_better": False, "n_gpus": 1, "steps": K, "warmup": args.warmup,
          "forward_ms": tf / K, "gradient_ms": tb / K,
          "forward_particle_steps_per_s": work / (tf / K * 1e-3), "dtype": "f32 forward and adjoint, f64 progenitor",
          "data": "synthetic (seeded)", "config": {"workload": C5["name"], "particle_steps": work},
          "grad_norm": float(torch.linalg.norm(g))})


C4 = dict(n_rel=3000, ppr=334, dt=1.0, spr=1,
          name="learned force surrogate: 3000 releases x 334 particles (1.0e6), 3 Gyr at dt=1 Myr in a triaxial halo "
               "given as a spherical-harmonic expansion (l_max=8, 64 log knots over 0.1-200 kpc, seeded 2^-l "
               "coefficients); MLP (x,y,z,ln r) -> Phi, 4 x 128 SiLU, trained on 2^22 orbit points, forces from its "
               "hand-written backward on the tensor cores (BF16, FP32 accumulation)")
# tensor-core work of one surrogate force: layers 2-4 forward + 3 backward
# GEMMs of 128 x 128 per particle (2 flops per multiply-add)
MLP_TENSOR_FLOPS = 6 * 2 * 128 * 128


def c4_arm(args):
    import torch

    import streamsculptor_gb300 as ss
    from streamsculptor_gb300 import _abi, _core, potential as P
    from streamsculptor_gb300.streamhelpers import gen_stream
    from streamsculptor_gb300.surrogate import MLPSurrogate, orbit_samples

    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
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
    phi, g = pot.potential(x, 0.0), pot.gradient(x, 0.0)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    sur = MLPSurrogate.init(seed=0, **MLPSurrogate.normalisation(x.cpu(), phi.cpu()))
    sur.fit(x, phi, g, steps=args.c4_train_steps, batch=8192, lr=3e-3, seed=0, log_every=max(1, args.c4_train_steps // 5))
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    xv = orbit_samples(pot, WF, n_orbits=64, n_per_orbit=256, seed=7)
    gv = pot.gradient(xv, 0.0)
    _, g32 = sur.potential_and_gradient(xv)
    g16 = sur.gradient_bf16(xv)
    nrm = torch.linalg.norm(gv, dim=1)
    e32 = torch.linalg.norm(g32 - gv, dim=1) / nrm
    e16 = torch.linalg.norm(g16 - gv, dim=1) / nrm
    del x, phi, g
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

    rm = timed("mlp", args.steps, args.warmup)
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
    # e2e: host normals in, final states to pinned host memory
    pin = torch.empty((2, n_rel, ppr // 2, 6), dtype=torch.float64, pin_memory=True)
    torch.cuda.synchronize()
    t3 = time.perf_counter()
    for _ in range(args.steps):
        out = step("mlp", normals_h)
        pin[0].copy_(out[0], non_blocking=True)
        pin[1].copy_(out[1], non_blocking=True)
    torch.cuda.synchronize()
    e2e_s = (time.perf_counter() - t3) / args.steps
    peak = MEASURED_BF16_TFLOPS
    ach = MLP_TENSOR_FLOPS * 6 * work / (rm["kernel_ms"] * 1e-3) / 1e12
    emit({"metric": METRIC, "value": work / (rm["ms_per_step"] * 1e-3), "unit": UNIT, "n_gpus": 1,
          "steps": args.steps, "warmup": args.warmup, "ms_per_step": rm["ms_per_step"], "higher_is_better": True,
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
          "surrogate": {"train_points": int(args.c4_points), "train_steps": args.c4_train_steps, "batch": 8192,
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
    ap.add_argument("--f64-warmup", type=int, default=3)
    ap.add_argument("--no-cpu-baseline", action="store_true")
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
