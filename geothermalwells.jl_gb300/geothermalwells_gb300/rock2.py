"""ROCK2 stage coefficients and stage-count rule (host side).

The coefficients are tabulated in ``csrc/rock2_table.h`` (written by
``csrc/gen_rock2_table.py`` from the published construction of the method);
this module reads that table so host code, the device library and the tests
all use the same numbers.  The library applies the same stage rule in C++.
"""
import os
import re

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
TABLE_H = os.path.join(os.path.dirname(_HERE), "csrc", "rock2_table.h")

S_MIN_RULE = 3  # at least one recurrence stage: R_s = w * P_{s-2} with s - 2 >= 1
_cache = None


def _parse():
    global _cache
    if _cache is not None:
        return _cache
    with open(TABLE_H) as f:
        src = f.read()
    tab = {}
    for name in ("gw_rock2_l", "gw_rock2_sigma", "gw_rock2_tau", "gw_rock2_mu",
                 "gw_rock2_nu", "gw_rock2_kappa", "gw_rock2_off"):
        m = re.search(r"%s\[\d+\]\s*=\s*\{(.*?)\};" % name, src, re.S)
        vals = [v.strip() for v in m.group(1).split(",") if v.strip()]
        tab[name] = np.array([float(v) for v in vals])
    tab["s_max"] = int(re.search(r"#define GW_ROCK2_S_MAX (\d+)", src).group(1))
    _cache = tab
    return tab


def s_max():
    return _parse()["s_max"]


def stability_interval(s):
    """l_s: |R_s(z)| <= 1 on [-l_s, 0]."""
    return float(_parse()["gw_rock2_l"][s - 2])


def coefficients(s):
    """(mu, nu, kappa, sigma, tau) for an s-stage step; mu/nu/kappa have
    length s - 2 (the recurrence stages)."""
    t = _parse()
    if not (2 <= s <= t["s_max"]):
        raise ValueError("ROCK2 stage count %d outside 2..%d" % (s, t["s_max"]))
    o = int(t["gw_rock2_off"][s - 2])
    n = s - 2
    return (t["gw_rock2_mu"][o:o + n].copy(), t["gw_rock2_nu"][o:o + n].copy(),
            t["gw_rock2_kappa"][o:o + n].copy(), float(t["gw_rock2_sigma"][s - 2]),
            float(t["gw_rock2_tau"][s - 2]))


def choose_stages(dt, eigen_est, max_stages=100):
    """Smallest s >= 3 whose stability interval covers dt * eigen_est,
    capped at ``max_stages`` (returned with covered=False when capped)."""
    x = abs(dt) * eigen_est
    cap = min(int(max_stages), s_max())
    for s in range(S_MIN_RULE, cap + 1):
        if stability_interval(s) >= x:
            return s, True
    return cap, False
