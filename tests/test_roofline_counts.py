"""The committed per-step work figures match the operation counter."""
from excalibur_tool_gb300 import roofline
from oracle.opcount import count_rk4_flrw_step


def test_flrw_rk4_step_counts():
    flops, sqrt, counts = count_rk4_flrw_step()
    assert flops == roofline.FLOPS_PER_RK4_STEP_FLRW, counts
    assert sqrt == roofline.SQRT_PER_RK4_STEP_FLRW
    assert roofline.bytes_per_rk4_step(8) == 416
