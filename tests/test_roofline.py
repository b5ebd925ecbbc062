"""CPU tests of the algorithmic work counts behind bench.py's roofline
(streamsculptor_gb300/roofline.py).  No GPU needed."""
import numpy as np
import pytest
import torch

from streamsculptor_gb300 import _core, potential as P, roofline


def _headline_flat():
    """NFW + Miyamoto-Nagai + Hernquist and the Plummer progenitor on a center
    track: the composition of the spray-stream workload."""
    u = P.usys
    base = P.Potential_Combine([P.NFWPotential(m=5.4e11, r_s=15.62, units=u),
                                P.MiyamotoNagaiDisk(m=6.8e10, a=3.0, b=0.28, units=u),
                                P.HernquistPotential(m=5e9, r_s=1.0, units=u)], units=u)
    prog = P.TimeDepTranslatingPotential(P.PlummerPotential(m=2e4, r_s=0.01, units=u),
                                         _core.CenterTrack(0.0, 1.0, np.zeros((2, 3))), units=u)
    return P.Potential_Combine([base, prog], units=u)._flatten()


def test_headline_work_per_particle_step():
    """Per force evaluation: NFW 19 + MN 19 + Hernquist 16 + Plummer 15 + the
    track offset 3 = 72 flops, 11 special ops; six evaluations per step plus
    the Dopri5 combinations of each form.  The packed two-particle kernel
    adds the mass-residual FMAs (NFW 4, the others 2 each: 82 per force) and
    does its stages in Nystrom form (330)."""
    flat = _headline_flat()
    w64 = roofline.particle_step_work(flat, "f64")
    w32 = roofline.particle_step_work(flat, "f32k")
    w2 = roofline.particle_step_work(flat, "f32k2")
    assert (w64["force_flops"], w64["force_specials"]) == (72, 11)
    assert w64["flops"] == 6 * 72 + 276 == 708
    assert w32["flops"] == 6 * 72 + 417 == 849
    assert w2["force_flops"] == 82 and w2["flops"] == 6 * 82 + 330 == 822
    assert w64["specials"] == w32["specials"] == w2["specials"] == 66


def test_response_work_per_system_step():
    """First-order form, mass columns: 210 (stage states) + 6 x 43
    (right-hand sides) + 12 (stage times) + 66 (update) = 546 flops and one
    rsqrt per stage; Nystrom form: 3 x 41 (stage positions) + 6 x 43 + 12 +
    3 x 24 (update) = 465."""
    w = roofline.response_step_work(6, "first_order")
    assert w["flops"] == 210 + 6 * 43 + 12 + 66 == 546
    assert w["specials"] == 6
    assert roofline.response_step_work(12, "first_order")["flops"] == 546 + 210 + 66 + 6 * (21 + 4)
    n = roofline.response_step_work(6)
    assert n["flops"] == 3 * 41 + 6 * 43 + 12 + 3 * 24 == 465
    assert roofline.response_step_work(12)["flops"] == 465 + 3 * 41 + 3 * 24 + 6 * 25
    with pytest.raises(ValueError):
        roofline.response_step_work(18)


@pytest.mark.skipif(torch.cuda.is_available(), reason="checks the behaviour without a CUDA device")
def test_no_cpu_fallback_for_device_tables():
    """Subhalo tables live on the device; without CUDA the package raises
    instead of falling back to a CPU path."""
    u = P.usys
    n = 3
    sh = P.SubhaloLinePotential(np.full(n, 1e7), np.full(n, 0.3), np.zeros((n, 3)), np.zeros((n, 3)), np.zeros(n),
                                100.0, units=u)
    with pytest.raises(RuntimeError, match="no CPU path"):
        sh._flatten()
