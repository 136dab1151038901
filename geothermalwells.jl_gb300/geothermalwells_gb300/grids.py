"""Host-side grid construction, mirroring ``src/grids.jl`` of GeothermalWells.jl.

Grids are one-time setup (not on the time-step path); they are built on the
host in float64 exactly as the reference does, then handed to the device by
:func:`geothermalwells_gb300.create_cache`.

The reference builds points with Julia ranges (``zmin:dz:zmax`` at
``src/grids.jl:32`` and ``range(a, b, n)`` at ``src/grids.jl:93``).  Julia
computes these from exact rational forms of their float endpoints when one
exists (so ``0:1.1:2200`` yields ``fl(k * 11 / 10)``, not a running sum).
:func:`julia_range` and :func:`julia_colon` restate that documented rule: find
the shortest continued-fraction rational that rounds back to each float and
return each point correctly rounded from exact rational arithmetic.
"""
from fractions import Fraction
import math

import numpy as np

_MAXINT_NARROW = 16777216  # 2**24, the integer range of the narrower float type


def _rat(x):
    """Continued-fraction rational ``p/q`` with ``float(p/q) == x`` and
    ``|p|, |q| <= 2**24``, or ``None`` if no such rational exists."""
    x = float(x)
    if x == 0.0:
        return 0, 1
    y = x
    a, b, c, d = 1, 0, 0, 1          # convergents h_n/k_n: (a/b) current, (c/d) previous
    a, b, c, d = 1, 0, 0, 1
    h_prev, h_cur = 0, 1
    k_prev, k_cur = 1, 0
    for _ in range(64):
        if abs(y) > _MAXINT_NARROW:
            break
        f = math.trunc(y)
        y -= f
        h_prev, h_cur = h_cur, f * h_cur + h_prev
        k_prev, k_cur = k_cur, f * k_cur + k_prev
        if max(abs(h_cur), abs(k_cur)) > _MAXINT_NARROW:
            return None
        if k_cur != 0 and h_cur / k_cur == x:
            return (h_cur, k_cur) if k_cur > 0 else (-h_cur, -k_cur)
        if y == 0.0:
            break
        y = 1.0 / y
    return None


def _exact(x):
    r = _rat(x)
    if r is not None:
        return Fraction(r[0], r[1])
    return Fraction(float(x))


def julia_range(start, stop, length):
    """``collect(range(start, stop, length))`` for Float64 endpoints."""
    length = int(length)
    if length < 1:
        return np.zeros(0)
    if length == 1:
        return np.array([float(start)])
    a, b = _exact(start), _exact(stop)
    n1 = length - 1
    return np.array([float((a * (n1 - i) + b * i) / n1) for i in range(length)])


def julia_colon(start, step, stop):
    """``collect(start:step:stop)`` for Float64 arguments."""
    a, s, b = _exact(start), _exact(step), _exact(stop)
    if s == 0:
        raise ValueError("range step cannot be zero")
    n = math.floor((b - a) / s) + 1
    n = max(0, n)
    return np.array([float(a + i * s) for i in range(n)])


def compute_domain(boreholes, buffer_x=100, buffer_y=100, buffer_z=200):
    """``src/grids.jl:8-18``: domain box around all boreholes."""
    xs = [bh.xc for bh in boreholes]
    ys = [bh.yc for bh in boreholes]
    zmax = max(bh.h for bh in boreholes) + buffer_z
    return dict(xmin=min(xs) - buffer_x, xmax=max(xs) + buffer_x,
                ymin=min(ys) - buffer_y, ymax=max(ys) + buffer_y,
                zmin=0.0 * zmax, zmax=zmax)


def create_uniform_gridz_with_borehole_depths(*, zmin, zmax, dz, boreholes, backend=None):
    """``src/grids.jl:29-48``: uniform z grid with every borehole depth ``h``
    inserted, sorted and de-duplicated (float64)."""
    g = list(julia_colon(zmin, dz, zmax))
    g.extend(float(bh.h) for bh in boreholes)
    return np.array(sorted(set(g)), dtype=np.float64)


def create_adaptive_grid_1d(*, xmin, xmax, dx_fine, growth_factor, dx_max, boreholes,
                            backend=None, Float_used=np.float64, direction="x"):
    """``src/grids.jl:80-147``: fine uniform interval around each borehole,
    geometric growth towards the domain edges and between boreholes."""
    if direction not in ("x", "y", ":x", ":y"):
        raise ValueError("direction must be x or y")
    key = (lambda bh: bh.xc) if direction in ("x", ":x") else (lambda bh: bh.yc)
    perm = sorted(range(len(boreholes)), key=lambda i: key(boreholes[i]))  # stable, like sortperm
    centers = [float(key(boreholes[i])) for i in perm]
    radii = [1.0 * float(boreholes[i].r_backfill) for i in perm]
    iv = [list(julia_range(centers[i] - radii[i], centers[i] + radii[i],
                           int(math.ceil((2 * radii[i]) / dx_fine)) + 1))
          for i in range(len(boreholes))]
    dx = float(dx_fine)
    x = iv[0][0]
    while x > xmin:
        dx = min(dx * growth_factor, dx_max)
        x = x - dx
        iv[0].insert(0, x if x > xmin else float(xmin))
    dx = float(dx_fine)
    x = iv[-1][-1]
    while x < xmax:
        dx = min(dx * growth_factor, dx_max)
        x = x + dx
        iv[-1].append(x if x < xmax else float(xmax))
    for i in range(len(boreholes) - 1):
        xi = iv[i][-1]
        xi1 = iv[i + 1][0]
        dx = float(dx_fine)
        while xi1 - xi > growth_factor * dx:
            dx = min(dx * growth_factor, dx_max)
            xi = xi + dx
            xi1 = xi1 - dx
            if xi1 - xi > dx:
                iv[i].append(xi)
                iv[i + 1].insert(0, xi1)
            else:
                iv[i].append((xi + xi1) / 2)
    grid = sorted(set(v for seg in iv for v in seg))
    return np.array(grid, dtype=np.float64).astype(Float_used)
