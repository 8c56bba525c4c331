"""The mixed mode's row split (CPU, no GPU): the radius the library chooses
for the double-float core of a primitive pair bounds every row outside it.

For random pairs (l ranges up to 3, exponents over three decades, distances
up to 3 bohr, the call's derivative shifts) the contributions of all
Cartesian pairs (a, b) of the sets, |(r - A)^a (r - B)^b| exp(-zeta_a |r - A|^2
- zeta_b |r - B|^2) summed (the factor 2 of pairs of different atoms
included), are evaluated at points of the sphere outside the cylinder around
the Gaussian product's x axis, many of them just outside it; none may exceed
the threshold the radius was computed for."""
import ctypes as C
import itertools

import numpy as np
import pytest

from cp2k_gb300 import grid as G

CORE_ALL = 3.0e38


def _lib():
    L = G.lib()
    f = L.grid_gb300_row_split_radius2
    f.argtypes = [C.c_int] * 4 + [C.c_double] * 2 + [C.c_void_p, C.c_double, C.c_int, C.c_int,
                                                     C.c_int, C.c_double, C.c_void_p]
    f.restype = C.c_double
    return f


def _cart(lmin, lmax):
    return [(ax, ay, l - ax - ay) for l in range(lmin, lmax + 1) for ax in range(l + 1)
            for ay in range(l - ax + 1)]


def _contribution(pts, A, B, za, zb, la_min, la_max, lb_min, lb_max, same):
    ra, rb = pts - A, pts - B
    g = np.exp(-za * (ra ** 2).sum(1) - zb * (rb ** 2).sum(1))
    s = np.zeros(len(pts))
    for a, b in itertools.product(_cart(la_min, la_max), _cart(lb_min, lb_max)):
        s += np.abs(np.prod(ra ** np.array(a) * rb ** np.array(b), axis=1))
    return s * g * (1.0 if same else 2.0)


def test_row_split_radius_bounds_outside_rows():
    f = _lib()
    rng = np.random.default_rng(7)
    tau = 0.1
    split = 0
    for trial in range(120):
        la_max, lb_max = int(rng.integers(0, 4)), int(rng.integers(0, 4))
        la_min, lb_min = int(rng.integers(0, la_max + 1)), int(rng.integers(0, lb_max + 1))
        za, zb = np.exp(rng.uniform(np.log(0.05), np.log(30.0), 2))
        d = rng.normal(size=3)
        rab = d / np.linalg.norm(d) * rng.uniform(0.0, 3.0)
        same = int(rng.integers(0, 2)) if np.linalg.norm(rab) < 1e-12 else 0
        dla, dlb = (0, 0) if trial % 3 else (1, 0)
        zp = za + zb
        pref = np.exp(-za * zb / zp * float(rab @ rab))
        radius = np.sqrt(np.log(1e12 * max(1.0, 50.0 * pref)) / zp)
        out = C.c_double()
        r2 = f(la_min, la_max, lb_min, lb_max, za, zb, rab.ctypes.data, radius, same, dla, dlb,
               tau, C.byref(out))
        if r2 >= CORE_ALL:
            assert out.value == 0.0
            continue
        split += 1
        assert 0.0 < r2 < radius * radius and 0.5 <= out.value <= 1.0
        # points of the sphere outside the cylinder, half of them within 5 %
        # of its radius
        n = 4000
        rho = np.sqrt(r2) * np.where(rng.random(n) < 0.5, 1.0 + 0.05 * rng.random(n),
                                     1.0 + rng.random(n) * (radius / np.sqrt(r2) - 1.0))
        phi = rng.uniform(0.0, 2 * np.pi, n)
        x = rng.uniform(-radius, radius, n)
        P = zb / zp * rab
        pts = P + np.stack([x, rho * np.cos(phi), rho * np.sin(phi)], axis=1)
        v = _contribution(pts, np.zeros(3), rab, za, zb, max(0, la_min - dla), la_max + dla,
                          max(0, lb_min - dlb), lb_max + dlb, same)
        assert float(v.max()) <= tau * (1.0 + 1e-9), (trial, float(v.max()))
    assert split >= 20  # the check saw enough split pairs


def test_row_split_radius_limits():
    """A pair whose every value stays under the threshold has no core (all
    rows outside); with a threshold nothing reaches inside the sphere, the
    pair stays whole."""
    f = _lib()
    out = C.c_double()
    rab = np.zeros(3)
    r2 = f(0, 0, 0, 0, 0.1, 0.1, rab.ctypes.data, 10.0, 1, 0, 0, 10.0, C.byref(out))
    assert r2 < 1e-30 and out.value == 1.0
    assert f(2, 2, 2, 2, 1.0, 1.0, rab.ctypes.data, 3.0, 1, 0, 0, 1e-30, C.byref(out)) >= CORE_ALL
