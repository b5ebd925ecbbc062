"""The FP64 special functions of the force evaluations (ss_device.cuh:
s_rcp, s_rsqrt, s_log1p) against the CUDA math library, through the C ABI
(ss_math_f64).  They replace 1.0 / x, rsqrt(x) and log1p(x) in every FP64
force because GB300 issues FP64 at 1/64 of the FP32 rate: each is a
hardware estimate (or a 128-entry breakpoint table) and a short polynomial
correction.  The bound is a few ulp relative to the library's results, far
inside the 1e-10 stream tolerance."""
import ctypes as C

import numpy as np
import pytest
import torch

from streamsculptor_gb300 import _abi

pytestmark = pytest.mark.gpu

ULP = 2.0 ** -52


def _run(fn, x):
    xd = torch.as_tensor(x, dtype=torch.float64, device="cuda")
    out, ref = torch.empty_like(xd), torch.empty_like(xd)
    s = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    _abi.call("ss_math_f64", fn, C.c_void_p(xd.data_ptr()), xd.numel(), C.c_void_p(out.data_ptr()),
              C.c_void_p(ref.data_ptr()), s)
    torch.cuda.synchronize()
    return out.cpu().numpy(), ref.cpu().numpy()


def _rel(a, b):
    return np.abs(a - b) / np.abs(b)


@pytest.mark.parametrize("fn,name", [(0, "reciprocal"), (1, "rsqrt")])
def test_reciprocal_and_rsqrt_within_two_ulp(ss, fn, name):
    rng = np.random.default_rng(fn)
    x = 10.0 ** rng.uniform(-12, 12, 1 << 20)
    if fn == 0:
        x = x * np.where(rng.uniform(size=x.size) < 0.5, -1.0, 1.0)  # both signs
    out, ref = _run(fn, x)
    err = _rel(out, ref)
    print(f"{name}: max {err.max() / ULP:.2f} ulp, mean {err.mean() / ULP:.3f} ulp")
    assert err.max() <= 2 * ULP


def test_log1p_within_four_ulp(ss):
    rng = np.random.default_rng(7)
    x = np.concatenate([10.0 ** rng.uniform(-14, 4, 1 << 20),   # NFW's r / r_s over all scales
                        rng.uniform(0.0, 3.0, 1 << 18),          # around the breakpoints of ln w
                        [0.0, 1.0, 2.0, 1e-300, 0.5, 127.0 / 128.0]])
    out, ref = _run(2, x)
    nz = ref != 0
    err = _rel(out[nz], ref[nz])
    print(f"log1p: max {err.max() / ULP:.2f} ulp, mean {err.mean() / ULP:.3f} ulp")
    assert err.max() <= 4 * ULP
    assert np.all(out[~nz] == 0.0)
