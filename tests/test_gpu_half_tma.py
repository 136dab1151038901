"""The mixed half step's tiles by tensor map (one cp.async.bulk.tensor 3-D
tile per chunk into a ring of buffers, mbarrier completion; the default)
against per-thread cp.async copies (GW_HALF_CPASYNC=1).  Both put the same
values in shared memory -- out-of-range levels, lines and rows read as 0 in
both -- so the fields and outlet series must agree bitwise: every tiling,
in-line and overlapped steps, one well and a row of wells, the padded column
pitch for nz = 0, 1, 2 and 3 mod 4, and the two benchmark wells."""
import numpy as np
import pytest

from geothermalwells_gb300 import (GB300, ODEProblem, ROCK2, create_cache, eigen_estimator,
                                   rhs_diffusion_z, solve)
from geothermalwells_gb300 import _lib
from geothermalwells_gb300 import workloads as W

pytestmark = pytest.mark.gpu

CASES = {
    "single": lambda: W.small_case(),
    "three_wells_layers_hx": lambda: W.small_case(n_layers=3, inlet="hx", nbh=3, nz_cells=40),   # nz = 43
    "deep": lambda: W.small_case(nz_cells=300, n_layers=2),   # nz = 301
    "2mm": W.single_well_2mm,
    "large": W.single_well_large,
}


def run(w, monkeypatch, cpasync, tiling=None, overlap=None, nsteps=3):
    if cpasync:
        monkeypatch.setenv("GW_HALF_CPASYNC", "1")
    else:
        monkeypatch.delenv("GW_HALF_CPASYNC", raising=False)
    c = create_cache(backend=GB300(precision="mixed"), gridx=w["gridx"], gridy=w["gridy"],
                     gridz=w["gridz"], materials=w["materials"], boreholes=w["boreholes"],
                     inlet_model=w["inlet_model"])
    L = _lib.load()
    if tiling is not None:
        _lib.check(L.gw_set_tiling(c.ctx, tiling))
    if overlap is not None:
        _lib.check(L.gw_set_overlap(c.ctx, overlap))
    sol = solve(ODEProblem(rhs_diffusion_z, w["T0"], (0.0, nsteps * w["dt"]), c),
                ROCK2(max_stages=100, eigen_est=eigen_estimator), dt=w["dt"])
    c.close()
    return sol


@pytest.mark.parametrize("name", list(CASES))
def test_tensor_map_tiles_equal_cp_async(name, gwlib, monkeypatch):
    w = CASES[name]()
    n = 2 if name in ("2mm", "large") else 3
    a = run(w, monkeypatch, cpasync=True, nsteps=n)
    b = run(w, monkeypatch, cpasync=False, nsteps=n)
    assert np.array_equal(a.u[-1], b.u[-1])
    assert np.array_equal(a.T_outlet, b.T_outlet)


@pytest.mark.parametrize("tiling", range(6))
def test_every_tiling(tiling, gwlib, monkeypatch):
    w = W.small_case(n_layers=2, nbh=2, nz_cells=30)
    a = run(w, monkeypatch, cpasync=True, tiling=tiling)
    b = run(w, monkeypatch, cpasync=False, tiling=tiling)
    assert np.array_equal(a.u[-1], b.u[-1])


@pytest.mark.parametrize("overlap", [0, 1])
def test_overlapped_step(overlap, gwlib, monkeypatch):
    w = W.small_case(n_layers=2, nbh=3, nz_cells=45)
    a = run(w, monkeypatch, cpasync=True, overlap=overlap)
    b = run(w, monkeypatch, cpasync=False, overlap=overlap)
    assert np.array_equal(a.u[-1], b.u[-1])
    assert np.array_equal(a.T_outlet, b.T_outlet)
