"""The no-allocation FP32 stream entry point (ss_stream_f32k_noalloc).

Callers that cannot allocate device memory (a bare C FFI binding with no
device allocator, code that must not make a call that may synchronize the
device, an application whose memory belongs to another allocator) use this
entry point: it keeps the stream's scratch in a fixed device array inside
the library instead of a caller workspace.  These tests call it through the
C ABI and check it against ss_stream_f32k with a caller workspace, on two
calls in a row with different potentials (the second call must not see the
first call's scratch), and check that an oversized run is refused.

This file sorts last so that a run stopping at the first failure has run
every other test before it."""
import ctypes as C

import numpy as np
import pytest
import torch

from streamsculptor_gb300 import _abi

from .conftest import PROG_WF, mw3_gpu

pytestmark = pytest.mark.gpu


def _phase_err(a, b):
    a, b = a.reshape(-1, 6), b.reshape(-1, 6)
    ex = np.linalg.norm(a[:, :3] - b[:, :3], axis=1) / np.linalg.norm(b[:, :3], axis=1)
    ev = np.linalg.norm(a[:, 3:] - b[:, 3:], axis=1) / np.linalg.norm(b[:, 3:], axis=1)
    return float(np.max(np.maximum(ex, ev)))


def _case(ss, prog_mass):
    """A moving-progenitor stream: ICs, the potential with its track, the config."""
    from streamsculptor_gb300 import potential as P
    from streamsculptor_gb300.streamhelpers import CenterTrack
    base = mw3_gpu(ss)
    n_rel, ppr, dt, spr = 60, 4, 0.5, 2
    n_steps = n_rel * spr
    T = n_steps * dt
    ts = -T + np.arange(n_rel + 1) * spr * dt
    back = base.integrate_orbit(w0=PROG_WF, ts=[0.0, -T], t0=0.0, t1=-T, dt=dt).ys[-1]
    ws, _, _ = base._prog_orbit(ts, back, dt)
    normals = np.random.default_rng(17).standard_normal((n_rel + 1, ppr // 2, 4))
    ics, _ = base._release(ws, ts, 2e4, normals)
    track = CenterTrack.from_samples(ts, ws[:, :3])
    pot = P.Potential_Combine([base, P.TimeDepTranslatingPotential(
        P.PlummerPotential(m=prog_mass, r_s=0.01, units=ss.usys), track, units=ss.usys)], units=ss.usys)
    cfg = _abi.ss_stream_cfg()
    cfg.t0, cfg.dt, cfg.n_steps, cfg.n_particles = float(ts[0]), dt, n_steps, n_rel * ppr
    cfg.particles_per_release, cfg.steps_per_release, cfg.snap_stride = ppr, spr, 40
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
    torch.cuda.synchronize()
    return final, snaps, status


def _run_workspace(pot, cfg, ics):
    from streamsculptor_gb300 import _core
    snaps = torch.empty(cfg.n_steps // cfg.snap_stride, cfg.n_particles, 6, dtype=torch.float32, device="cuda")
    final, status = _core.stream(pot._desc(), cfg, ics, "f32k", snaps=snaps)
    torch.cuda.synchronize()
    return final, snaps, status


def test_no_alloc_matches_workspace_entry_point_twice(ss):
    for prog_mass in (2e4, 3e6):  # two calls in a row, different progenitor tracks' potentials
        pot, cfg, ics = _case(ss, prog_mass)
        f_ref, s_ref, st_ref = _run_workspace(pot, cfg, ics)
        f, s, st = _run_noalloc(pot, cfg, ics)
        assert st.tolist() == st_ref.tolist()
        assert _phase_err(f.cpu().numpy(), f_ref.cpu().numpy()) <= 1e-5
        sn, sr = s.cpu().numpy().astype(np.float64), s_ref.cpu().numpy().astype(np.float64)
        assert np.array_equal(np.isnan(sn), np.isnan(sr))
        ok = ~np.isnan(sr[..., 0])
        assert _phase_err(sn[ok], sr[ok]) <= 1e-5


def test_no_alloc_rejects_oversized_runs(ss):
    pot, cfg, ics = _case(ss, 2e4)
    big = _abi.ss_stream_cfg()
    C.memmove(C.addressof(big), C.addressof(cfg), C.sizeof(cfg))
    big.n_steps = 200000  # track table alone: (5 * 200000 + 1) * 32 bytes > 4 MiB
    big.snap_stride = 0
    lib = _abi.load()
    P = pot._desc()
    rc = lib.ss_stream_f32k_noalloc(C.byref(P), C.byref(big), C.c_void_p(ics.data_ptr()), None, None, None,
                                    C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == _abi.SS_ERR_WORKSPACE
    assert b"scratch" in lib.ss_last_error()
