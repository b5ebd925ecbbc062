"""The no-allocation FP32 stream entry point (ss_stream_f32k_noalloc).

Callers that cannot allocate device memory (a bare C FFI binding with no
device allocator, code that must not make a call that may synchronize the
device, an application whose memory belongs to another allocator) use this
entry point: it keeps the stream's scratch in a fixed device array inside
the library instead of a caller workspace.  These tests call it through the
C ABI and check it against ss_stream_f32k with a caller workspace.  Both run
the same kernels on the same inputs, so the outputs must be identical bit for
bit.  Two calls run back to back with different scratch contents and layouts
(a progenitor track followed by subhalo lines, then another progenitor orbit
on another time grid), so a read of the first call's scratch by the second
would change its result.  An oversized run must be refused.

This file sorts last so that a run stopping at the first failure has run
every other test before it."""
import ctypes as C

import numpy as np
import pytest
import torch

from streamsculptor_gb300 import _abi

from .conftest import PROG_WF, mw3_gpu

pytestmark = pytest.mark.gpu


def _case(ss, w_today, dt, n_rel, spr, with_lines):
    """A moving-progenitor stream (optionally with subhalo lines): the
    potential with its track, the config and the initial conditions."""
    from streamsculptor_gb300 import potential as P
    from streamsculptor_gb300.streamhelpers import CenterTrack
    base = mw3_gpu(ss)
    ppr = 4
    n_steps = n_rel * spr
    T = n_steps * dt
    ts = -T + np.arange(n_rel + 1) * spr * dt
    back = base.integrate_orbit(w0=w_today, ts=[0.0, -T], t0=0.0, t1=-T, dt=dt).ys[-1]
    ws, _, _ = base._prog_orbit(ts, back, dt)
    normals = np.random.default_rng(17).standard_normal((n_rel + 1, ppr // 2, 4))
    ics, _ = base._release(ws, ts, 2e4, normals)
    track = CenterTrack.from_samples(ts, ws[:, :3])
    parts = [base, P.TimeDepTranslatingPotential(P.PlummerPotential(m=2e4, r_s=0.01, units=ss.usys), track,
                                                 units=ss.usys)]
    if with_lines:
        rng = np.random.default_rng(5)
        n_sh = 40
        parts.append(P.SubhaloLinePotential(10 ** rng.uniform(6, 8, n_sh), rng.uniform(0.05, 0.5, n_sh),
                                            rng.normal(0, 10, (n_sh, 3)), rng.normal(0, 0.1, (n_sh, 3)),
                                            rng.uniform(ts[0], ts[-1], n_sh), 40.0, units=ss.usys))
    pot = P.Potential_Combine(parts, units=ss.usys)
    cfg = _abi.ss_stream_cfg()
    cfg.t0, cfg.dt, cfg.n_steps, cfg.n_particles = float(ts[0]), dt, n_steps, n_rel * ppr
    cfg.particles_per_release, cfg.steps_per_release, cfg.snap_stride = ppr, spr, 20
    return pot, cfg, ics[:n_rel].reshape(-1, 6).contiguous()


def _run_noalloc(pot, cfg, ics):
    lib = _abi.load()
    N = cfg.n_particles
    final = torch.empty(N, 6, dtype=torch.float64, device="cuda")
    snaps = torch.empty(cfg.n_steps // cfg.snap_stride, N, 6, dtype=torch.float32, device="cuda")
    status = torch.empty(N, dtype=torch.int32, device="cuda")
    P = pot._desc()
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = lib.ss_stream_f32k_noalloc(C.byref(P), C.byref(cfg), C.c_void_p(ics.data_ptr()),
                                    C.c_void_p(final.data_ptr()), C.c_void_p(snaps.data_ptr()),
                                    C.c_void_p(status.data_ptr()), stream)
    assert rc == _abi.SS_OK, lib.ss_last_error()
    return final, snaps, status


def _run_workspace(pot, cfg, ics):
    from streamsculptor_gb300 import _core
    snaps = torch.empty(cfg.n_steps // cfg.snap_stride, cfg.n_particles, 6, dtype=torch.float32, device="cuda")
    final, status = _core.stream(pot._desc(), cfg, ics, "f32k", snaps=snaps)
    return final, snaps, status


def _bits_equal(a, b):
    # bit patterns, so that the NaN rows of unreleased particles compare too
    it = torch.int64 if a.dtype == torch.float64 else torch.int32
    return torch.equal(a.view(it), b.view(it))


def test_no_alloc_matches_workspace_entry_point_twice(ss):
    w2 = PROG_WF + np.array([0.5, -0.3, 0.2, 0.01, -0.005, 0.003])
    cases = [_case(ss, PROG_WF, 0.5, 60, 2, with_lines=True),   # track table + subhalo table
             _case(ss, w2, 0.4, 45, 3, with_lines=False)]       # another orbit, another time grid
    # the two no-allocation calls back to back on one stream: the second
    # overwrites the first one's track table with different values
    got = [_run_noalloc(*c) for c in cases]
    want = [_run_workspace(*c) for c in cases]
    torch.cuda.synchronize()
    for (f, s, st), (fr, sr, str_) in zip(got, want):
        assert torch.equal(st, str_)
        assert bool((st == 0).all())
        assert _bits_equal(f, fr)
        assert _bits_equal(s, sr)
    # the two runs differ, so a stale table would show
    assert not torch.equal(got[0][0][:10], got[1][0][:10])


def test_no_alloc_rejects_oversized_runs(ss):
    pot, cfg, ics = _case(ss, PROG_WF, 0.5, 60, 2, with_lines=False)
    big = _abi.ss_stream_cfg()
    C.memmove(C.addressof(big), C.addressof(cfg), C.sizeof(cfg))
    big.n_steps = 200000  # track table alone: (5 * 200000 + 1) * 32 bytes > 4 MiB
    big.snap_stride = 0
    lib = _abi.load()
    P = pot._desc()
    assert lib.ss_stream_workspace_bytes(C.byref(P), C.byref(big)) > 4 << 20
    rc = lib.ss_stream_f32k_noalloc(C.byref(P), C.byref(big), C.c_void_p(ics.data_ptr()), None, None, None,
                                    C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == _abi.SS_ERR_WORKSPACE
    assert b"scratch" in lib.ss_last_error()
