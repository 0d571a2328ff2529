"""Algorithmic work per photon-step, for roofline reporting.

Counted by executing the reference's formulas on a counting float
(oracle/opcount.py; tests/test_roofline_counts.py keeps these in sync):
one RK4 step of the FLRW-fast tracer = 4 RHS evaluations (periodic trilinear
Phi + base-node gradient, LCDM a(eta) and adot, tensorial Christoffel
contraction) + the RK4 combination.
"""

# floating-point add/sub/mul/div (+ the periodic wrap's fmod) per RK4 photon-step
FLOPS_PER_RK4_STEP_FLRW = 1009
SQRT_PER_RK4_STEP_FLRW = 4
# the same, by kind (a division or fmod costs several multiply/add slots of the FP64
# pipe; exc_probe_fp64_rates measures how many)
OPS_PER_RK4_STEP_FLRW = {"add": 228, "sub": 128, "mul": 492, "div": 149, "fmod": 12, "sqrt": 4}
# of those divisions, the ones by a launch constant (c^2, c^4, grid spacings, the a(eta) table
# step): the parity build takes them as correctly rounded FMA quotients from host reciprocals
# (one multiply and two FMAs, bit-identical to the IEEE division)
DIV_CONST_PER_RK4_STEP_FLRW = 129
CONST_DIV_SLOTS = 3


def fp64_pipe_slots(ops: dict, rates: dict) -> float:
    """Multiply/add-equivalent FP64 pipe slots of an operation mix, each kind weighted by
    the measured multiply/add rate over its own measured rate."""
    base = rates["addmul"]
    return (ops["add"] + ops["sub"] + ops["mul"] + ops["div"] * base / rates["div"] +
            ops["fmod"] * base / rates["fmod"] + ops["sqrt"] * base / rates["sqrt"])


def fp64_pipe_slots_executed(ops: dict, rates: dict, div_const: int = DIV_CONST_PER_RK4_STEP_FLRW) -> float:
    """fp64_pipe_slots with the divisions by launch constants at CONST_DIV_SLOTS slots each
    (how the parity build executes them) instead of an IEEE division's measured cost."""
    return fp64_pipe_slots(ops, rates) - div_const * (rates["addmul"] / rates["div"] - CONST_DIV_SLOTS)


# bytes gathered per RK4 photon-step: 4 RHS x (11 distinct grid nodes + 2 a(eta) table entries)
NODES_PER_RHS = 11
TABLE_ENTRIES_PER_RHS = 2


def bytes_per_rk4_step(field_itemsize: int) -> int:
    return 4 * (NODES_PER_RHS * field_itemsize + TABLE_ENTRIES_PER_RHS * 8)
