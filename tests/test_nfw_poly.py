"""The FP32 NFW enclosed-mass polynomial of the paired stream kernel
(nfw_F2, streamsculptor_gb300/csrc/ss_stream2.cuh): its coefficients are the
fit that csrc/gen_nfw_poly.py makes, and F(u) evaluated with FP32 rounding
in the kernel's order stays within 6e-7 of the FP64 value over u in (0, 2)
(the Taylor form it replaced: 3.8e-7)."""
import importlib.util
import os

import numpy as np

CSRC = os.path.join(os.path.dirname(__file__), "..", "streamsculptor_gb300", "csrc")


def _gen():
    spec = importlib.util.spec_from_file_location("gen_nfw_poly", os.path.join(CSRC, "gen_nfw_poly.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


def test_kernel_coefficients_are_the_fit():
    g = _gen()
    c, err = g.fit()
    src = open(os.path.join(CSRC, "ss_stream2.cuh")).read()
    body = src[src.index("__device__ __forceinline__ f2 nfw_F2"):src.index("if (!(sx && sy))")]
    for x in c:
        assert ("%.9gf" % x) in body
    assert err < 5e-8


def test_fp32_enclosed_mass_accuracy():
    g = _gen()
    c, _ = g.fit()
    u = np.concatenate([np.geomspace(1e-6, 1e-4, 500), np.linspace(1e-4, 2, 40001)]).astype(np.float32)
    U = u.astype(np.float64)
    ref = np.log1p(U) - U / (1 + U)
    rel = np.abs(g.f32_F(u, c) - ref) / ref
    assert rel.max() < 6e-7
    assert np.median(rel) < 1.5e-7
    # no bias beyond rounding: the mean signed error stays far below one ulp
    assert abs(np.mean((g.f32_F(u, c) - ref) / ref)) < 2e-8
