"""The one arithmetic difference between the CUDA library and the reference: x**3 (and x**4).

The reference evaluates ȧ = a² H0 E(z), E = sqrt(Ωm (1+z)**3 + …) with numpy/Python `**`,
i.e. glibc's pow(), which misrounds a small fraction of near-halfway cubes by one ulp. The
library evaluates the cube as a double-double product rounded once (pow3_cr in
csrc/exc_device.cuh), which is correctly rounded. The oracle can run either way
(`oracle.power_mode`): "libm" reproduces the reference bit for bit, "dd" the library's
arithmetic. These tests bound what the switch changes; the GPU tests then require the
library to equal the oracle in "dd" mode bit for bit, so that the power is shown to be the
only source of difference.
"""
from fractions import Fraction

import numpy as np

from conftest import golden
from helpers import lcdm_spacetime, rel_err
from excalibur_tool_gb300.trace import TraceConfig
from oracle import oracle as O


def _one_plus_z(n, seed=0):
    a = golden("cosmology.npz")["a_grid"]
    rng = np.random.default_rng(seed)
    return np.concatenate([1.0 / a, 1.0 / rng.uniform(a.min(), a.max(), n)])


def test_double_double_cube_is_correctly_rounded():
    x = _one_plus_z(200_000)
    lm, dd = O.power(x, 3, "libm"), O.power(x, 3, "dd")
    differ = np.nonzero(lm != dd)[0]
    rng = np.random.default_rng(1)
    check = np.concatenate([differ[:200], rng.choice(x.size, 200, replace=False)])
    for i in check:
        exact = Fraction(float(x[i])) ** 3
        got = float(dd[i])
        for nb in (np.nextafter(got, np.inf), np.nextafter(got, -np.inf)):
            assert abs(Fraction(got) - exact) <= abs(Fraction(float(nb)) - exact)


def test_libm_pow_differs_from_the_rounded_cube_by_at_most_one_ulp():
    x = _one_plus_z(1_000_000)
    for p in (3, 4):
        lm, dd = O.power(x, p, "libm"), O.power(x, p, "dd")
        ulps = np.abs(lm.view(np.int64) - dd.view(np.int64))
        assert ulps.max() <= 1
        assert 0.0 < (ulps > 0).mean() < 0.01      # rare, but the workloads meet it (0.09 % of cubes)


def test_power_mode_moves_adot_by_at_most_two_ulps():
    """A one-ulp cube moves E(z) = sqrt(Ωm (1+z)^3 + ΩΛ) and then a² H0 E by up to two ulps."""
    cz = golden("cosmology.npz")
    st = lcdm_spacetime(np.zeros((4, 4, 4)), 1.0)
    with O.power_mode("dd"):
        a, adot = O.cosmology(st, cz["etas"])
    assert np.array_equal(a, cz["a"])
    ulps = np.abs(adot.view(np.int64) - cz["adot"].view(np.int64))
    assert ulps.max() <= 2


def test_power_mode_keeps_the_reference_rk45_trajectory():
    """The RK45 record golden (30 adaptive steps through integrate_single) in "dd" mode: the
    same accepted steps, states within 1e-12 of the reference's."""
    g = golden("integrate.npz")
    st = lcdm_spacetime(g["field"], float(g["box"]))
    rtol, atol, dmin, dmax = g["case4_tol"]
    dt = float(g["dt"])
    cfg = TraceConfig(stepper="rk45", dt=dt, dt_min=dmin, dt_max=dmax, rtol=rtol, atol=atol, max_steps=30,
                      record_every=1, observables=False)
    with O.power_mode("dd"):
        res = O.trace(st, g["case4_init"][None], cfg)
    want = g["case4_records"]
    got = res.records[0, :res.n_records[0]]
    assert res.status[0] == 0 and got.shape == want.shape
    assert rel_err(res.state[0], g["case4_final"]).max() <= 1e-12
