"""The committed per-step work figures match the operation counter."""
from excalibur_tool_gb300 import roofline
from oracle.opcount import count_rk4_flrw_step


def test_flrw_rk4_step_counts():
    flops, sqrt, counts = count_rk4_flrw_step()
    assert flops == roofline.FLOPS_PER_RK4_STEP_FLRW, counts
    assert sqrt == roofline.SQRT_PER_RK4_STEP_FLRW
    assert roofline.bytes_per_rk4_step(8) == 416
    by_kind = {k: counts.get(k, 0) for k in roofline.OPS_PER_RK4_STEP_FLRW}
    assert by_kind == roofline.OPS_PER_RK4_STEP_FLRW
    assert counts["div_const"] == roofline.DIV_CONST_PER_RK4_STEP_FLRW
    assert sum(v for k, v in by_kind.items() if k != "sqrt") == roofline.FLOPS_PER_RK4_STEP_FLRW


def test_fp64_pipe_slots():
    ops = {"add": 1, "sub": 2, "mul": 3, "div": 4, "fmod": 5, "sqrt": 6}
    rates = {"addmul": 8.0, "div": 1.0, "fmod": 2.0, "sqrt": 4.0}
    assert roofline.fp64_pipe_slots(ops, rates) == 6 + 4 * 8 + 5 * 4 + 6 * 2


def test_fp64_pipe_slots_executed():
    ops = {"add": 1, "sub": 2, "mul": 3, "div": 4, "fmod": 5, "sqrt": 6}
    rates = {"addmul": 8.0, "div": 1.0, "fmod": 2.0, "sqrt": 4.0}
    # three of the four divisions by constants: 3 x (8 - 3) slots fewer
    assert roofline.fp64_pipe_slots_executed(ops, rates, div_const=3) == 6 + 4 * 8 + 5 * 4 + 6 * 2 - 3 * 5
