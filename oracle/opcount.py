"""Algorithmic operation counts of one RK4 photon-step -- TEST INFRASTRUCTURE.

Re-executes the reference's formulas for one FLRW-fast RHS (periodic
trilinear Phi + base-node gradient, LCDM a(eta) and adot, tensorial
Christoffel contraction; perturbed_flrw_metric_fast.py:7-76, :227-273,
interpolator_4d_fast.py:195-255, cosmology.py:8-25, :69-93) and of the RK4
combination (integrator.py:10-22) on a counting float, and reports how many
floating-point operations of each kind they perform:
  flops = add + sub + mul + div (+ fmod in the periodic wrap); sqrt separately.
Index arithmetic (floor, int, integer modulo) and comparisons are not counted.
a(eta) is counted once per RHS (the reference evaluates it a second time
inside adot_of_eta; that repeat is not algorithmic work).

The integers are committed in excalibur_tool_gb300/roofline.py;
tests/test_roofline_counts.py checks them against this counter.
"""
from __future__ import annotations

import math
from collections import Counter

COUNTS = Counter()


class F:
    __slots__ = ("v",)

    def __init__(self, v):
        self.v = float(v.v if isinstance(v, F) else v)

    @staticmethod
    def _v(o):
        return o.v if isinstance(o, F) else float(o)

    def _op(self, kind, val):
        COUNTS[kind] += 1
        return F(val)

    def __add__(self, o): return self._op("add", self.v + self._v(o))
    def __radd__(self, o): return self._op("add", self._v(o) + self.v)
    def __sub__(self, o): return self._op("sub", self.v - self._v(o))
    def __rsub__(self, o): return self._op("sub", self._v(o) - self.v)
    def __mul__(self, o): return self._op("mul", self.v * self._v(o))
    def __rmul__(self, o): return self._op("mul", self._v(o) * self.v)
    def __truediv__(self, o):
        if not isinstance(o, F) or isinstance(o, Const):
            COUNTS["div_const"] += 1      # divisor fixed for the launch (c^2, c^4, spacing, table step)
        return self._op("div", self.v / self._v(o))
    def __rtruediv__(self, o): return self._op("div", self._v(o) / self.v)
    def __mod__(self, o): return self._op("fmod", math.fmod(self.v, self._v(o)) % self._v(o))
    def __neg__(self): return F(-self.v)

    def __pow__(self, n):
        # x**n by repeated multiplication: n-1 multiplies
        COUNTS["mul"] += int(n) - 1
        return F(self.v ** n)

    def __lt__(self, o): return self.v < self._v(o)
    def __le__(self, o): return self.v <= self._v(o)
    def __gt__(self, o): return self.v > self._v(o)
    def __ge__(self, o): return self.v >= self._v(o)
    def __float__(self): return self.v


class Const(F):
    """A launch constant (grid spacing, table step): a division by it, or by a plain Python
    number such as c**2, is counted as a division by a constant as well. Products and sums of
    constants stay constants (2.0 * spacing)."""
    __slots__ = ()

    def _op(self, kind, val):
        COUNTS[kind] += 1
        return F(val)

    def __mul__(self, o):
        COUNTS["mul"] += 1
        v = self.v * self._v(o)
        return Const(v) if not isinstance(o, F) or isinstance(o, Const) else F(v)

    __rmul__ = __mul__


def fsqrt(x):
    COUNTS["sqrt"] += 1
    return F(math.sqrt(x.v))


def _interp_periodic(field_get, x, y, z, o, s, n):
    L = [n * s[i] for i in range(3)]
    p = [o[i] + ((q - o[i]) % L[i]) for i, q in enumerate((x, y, z))]
    rel = [(p[i] - o[i]) / s[i] for i in range(3)]
    i0 = [int(math.floor(r.v)) for r in rel]
    d = [rel[i] - i0[i] for i in range(3)]
    dx, dy, dz = d
    c = [F(field_get(i0[0] + a, i0[1] + b, i0[2] + cc)) for a, b, cc in
         [(0, 0, 0), (1, 0, 0), (0, 1, 0), (0, 0, 1), (1, 1, 0), (1, 0, 1), (0, 1, 1), (1, 1, 1)]]
    val = (c[0] * (1 - dx) * (1 - dy) * (1 - dz) + c[1] * dx * (1 - dy) * (1 - dz) +
           c[2] * (1 - dx) * dy * (1 - dz) + c[3] * (1 - dx) * (1 - dy) * dz + c[4] * dx * dy * (1 - dz) +
           c[5] * dx * (1 - dy) * dz + c[6] * (1 - dx) * dy * dz + c[7] * dx * dy * dz)
    g = [(c[1 + k] - F(field_get(*(i0[j] - (j == k) for j in range(3))))) / (2.0 * s[k]) for k in range(3)]
    return val, g, F(0.0)


def _a_interp(eta, eta_min, eta_step, tab):
    max_eta = eta_min + eta_step * (len(tab) - 1)
    i = int(((eta - eta_min) / eta_step).v)
    t = (eta - (eta_min + i * eta_step)) / eta_step
    return (1 - t) * tab[i] + t * tab[i + 1], max_eta


def rhs(state, field_get, o, s, n, tab, eta_min, eta_step, H0, Om, Or, Ok, OL, c):
    eta = state[0]
    a, _ = _a_interp(eta, eta_min, eta_step, tab)
    z = 1.0 / a - 1.0
    zp = 1 + z
    E = fsqrt(Om * zp ** 3 + Or * zp ** 4 + Ok * zp ** 2 + OL)
    adot = a * a * (H0 * E)
    phi_si, (gx, gy, gz), phid_si = _interp_periodic(field_get, state[1], state[2], state[3], o, s, n)
    c2, c4 = float(c) ** 2, float(c) ** 4
    phi = phi_si / c2
    phi_dot = phid_si / c2
    u0, u1, u2, u3 = state[4], state[5], state[6], state[7]
    a2 = a * a
    adot_a = adot / a
    usq = u1 * u1 + u2 * u2 + u3 * u3
    psi = phi
    G000 = (phi_dot / c2) * u0 * u0
    G0ij = (a * adot / c2 + 2 * a * adot / c4 * (phi + psi) - a2 / c4 * phi_dot) * usq
    G00i = 2 * ((gx / c2) * u0 * u1 + (gy / c2) * u0 * u2 + (gz / c2) * u0 * u3)
    du0 = -(G000 + G0ij + G00i)
    out = [u0, u1, u2, u3, du0]
    for gi, ui, (gj, uj), (gk, uk) in ((gx, u1, (gy, u2), (gz, u3)), (gy, u2, (gx, u1), (gz, u3)),
                                       (gz, u3, (gx, u1), (gy, u2))):
        G100 = gi / a2 * u0 * u0
        G10i = 2 * (adot_a - phi_dot / c2) * u0 * ui
        G1ii = (-(gi / c2) * ui * ui + (gi / c2) * (uj * uj + uk * uk) + (-(gj / c2)) * ui * uj +
                (-(gk / c2)) * ui * uk)
        out.append(-(G100 + G10i + G1ii))
    return out


def count_rk4_flrw_step():
    """Counter of one RK4 step of the FLRW-fast tracer (4 RHS + combination)."""
    import numpy as np

    COUNTS.clear()
    rng = np.random.default_rng(0)
    n = 16
    field = rng.standard_normal((n, n, n)) * 1e11

    def fg(i, j, k):
        return field[i % n, j % n, k % n]

    tab = [F(v) for v in np.linspace(0.1, 2.0, 5000)]
    s = [Const(2.5e22)] * 3
    o = [F(0.0)] * 3
    state = [F(1.4e18), F(1.0e23), F(2.0e23), F(3.0e23), F(-1.0), F(2e8), F(1e8), F(1.5e8)]
    dt = F(5e13)
    args = (fg, o, s, n, tab, F(0.0), Const(3.5e14), F(2.27e-18), 0.3, 0.0, 0.0, 0.7, 299792458)
    k1 = rhs(state, *args)
    k2 = rhs([state[i] + 0.5 * dt * k1[i] for i in range(8)], *args)
    k3 = rhs([state[i] + 0.5 * dt * k2[i] for i in range(8)], *args)
    k4 = rhs([state[i] + dt * k3[i] for i in range(8)], *args)
    d6 = dt / 6
    _ = [state[i] + d6 * (k1[i] + 2 * k2[i] + 2 * k3[i] + k4[i]) for i in range(8)]
    counts = dict(COUNTS)
    flops = sum(v for k, v in counts.items() if k not in ("sqrt", "div_const"))
    return flops, counts.get("sqrt", 0), counts


if __name__ == "__main__":
    print(count_rk4_flrw_step())
