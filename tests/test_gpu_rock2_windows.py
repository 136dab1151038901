"""The mixed step's ROCK2 by windows (k_rock2_win: one warp per window of
32 x LPT levels of a column, s halo levels recomputed at interior window
edges, neighbour values by warp shuffles, a column's windows in one block
meeting at a named barrier before they store) against the block kernel
(k_rock2_reg, one block per column; GW_ROCK2_BLOCK=1).  Both do the same
arithmetic level for level, so the fields and outlet series must agree
bitwise: on one-window columns, columns of several windows, a column deeper
than 2048 levels (more windows than a block has warps: the block kernel),
many ROCK2 stages (the generic instance) and s = 3 (the instance without the
g_{j-2} stage), in-line and overlapped steps in both launch orders, and on
the 2 mm and large benchmark wells."""
import ctypes

import numpy as np
import pytest

from geothermalwells_gb300 import (GB300, ODEProblem, ROCK2, create_cache, eigen_estimator,
                                   rhs_diffusion_z, solve)
from geothermalwells_gb300 import _lib
from geothermalwells_gb300 import workloads as W

pytestmark = pytest.mark.gpu

CASES = {
    "one_window": lambda: W.small_case(nz_cells=12),
    "layers_hx_two_windows": lambda: W.small_case(n_layers=3, inlet="hx", nbh=2, nz_cells=300),
    "deep_column": lambda: W.small_case(nz_cells=2500, h=600.0),
    "four_stages": lambda: W.small_case(backfill_quirk=True, n_layers=2, nz_cells=400, dt=0.05),
    "many_stages": lambda: W.small_case(backfill_quirk=True, n_layers=2, nz_cells=400, dt=1.0),
    "2mm": W.single_well_2mm,
    "large": W.single_well_large,
}


def stages(cache, dt):
    s, cov = ctypes.c_int(), ctypes.c_int()
    _lib.check(_lib.load().gw_rock2_stages(cache.ctx, dt, 100, ctypes.byref(s), ctypes.byref(cov)))
    return s.value


def run(w, monkeypatch, block, overlap=None, nsteps=3, order=None):
    if order is None:
        monkeypatch.delenv("GW_STEP_ORDER", raising=False)
    else:
        monkeypatch.setenv("GW_STEP_ORDER", str(order))
    if block:
        monkeypatch.setenv("GW_ROCK2_BLOCK", "1")
    else:
        monkeypatch.delenv("GW_ROCK2_BLOCK", raising=False)
    c = create_cache(backend=GB300(precision="mixed"), gridx=w["gridx"], gridy=w["gridy"],
                     gridz=w["gridz"], materials=w["materials"], boreholes=w["boreholes"],
                     inlet_model=w["inlet_model"])
    if overlap is not None:
        _lib.check(_lib.load().gw_set_overlap(c.ctx, overlap))
    s = stages(c, w["dt"])
    sol = solve(ODEProblem(rhs_diffusion_z, w["T0"], (0.0, nsteps * w["dt"]), c),
                ROCK2(max_stages=100, eigen_est=eigen_estimator), dt=w["dt"])
    c.close()
    return sol, s


@pytest.mark.parametrize("name", list(CASES))
def test_windows_equal_block_kernel(name, gwlib, monkeypatch):
    w = CASES[name]()
    nsteps = 2 if name in ("2mm", "large") else 3
    a, s = run(w, monkeypatch, block=True, nsteps=nsteps)
    b, s2 = run(w, monkeypatch, block=False, nsteps=nsteps)
    assert s == s2
    if name == "four_stages":
        assert s == 4, s         # the generic instance
    if name == "many_stages":
        assert 8 < s <= 32, s    # halo of s levels, still windows (8 s <= W)
    if name in ("2mm", "large", "one_window"):
        assert s == 3, s
    if name == "deep_column":
        assert len(w["gridz"]) > 2048
    assert np.array_equal(a.u[-1], b.u[-1])
    assert np.array_equal(a.T_outlet, b.T_outlet)


@pytest.mark.parametrize("overlap", [0, 1])
def test_windows_equal_block_kernel_overlap(overlap, gwlib, monkeypatch):
    """The overlapped step runs ROCK2 as two launches over parts of the
    column order (the pipe rows first); both kernels take the same parts."""
    w = W.small_case(n_layers=2, nbh=3, nz_cells=600)
    a, _ = run(w, monkeypatch, block=True, overlap=overlap)
    b, _ = run(w, monkeypatch, block=False, overlap=overlap)
    assert np.array_equal(a.u[-1], b.u[-1])
    assert np.array_equal(a.T_outlet, b.T_outlet)


def test_six_window_columns_with_two_rock2_launches_at_once(gwlib, monkeypatch):
    """Columns of 1401 levels take six windows (slots that do not divide a
    block of eight warps).  In the overlapped step's order 1, two ROCK2
    launches run at once on two streams, so their blocks start apart.  With
    a column's windows spread over two blocks, a late window read its
    neighbour's stored levels as halo, and repeated runs differed by about
    1e-10.  Three runs, each bitwise equal to the block kernel."""
    w = W.small_case(nz_cells=1400, h=400.0)
    a, _ = run(w, monkeypatch, block=True, order=1)
    for _ in range(3):
        b, _ = run(w, monkeypatch, block=False, order=1)
        assert np.array_equal(a.u[-1], b.u[-1])
        assert np.array_equal(a.T_outlet, b.T_outlet)
