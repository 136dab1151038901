"""The mixed half step with its forward-elimination values in tensor memory
(TMEM; the default of the tensor-map half step) against the same kernel with
the values stored to and reloaded from global memory (GW_HALF_GLOBAL=1).
Both evaluate the same recurrences in the same order, so the fields and
outlet series must agree bitwise (the on-chip runs set GW_HALF_TMEM_FORCE=1:
without it a half step of fewer than four rounds of blocks keeps its values
in global memory): every tiling, in-line and overlapped steps,
lines of 36..88 rows (partial chunks and partial backward batches), lines
longer than 256 rows (the 8-line tilings then keep their values in global
memory, the others split them between 128 TMEM columns and shared memory),
and the two benchmark wells (the large well's 205-row lines take the split
form in tiling 0, the 2 mm well's 225-row lines whole-line TMEM)."""
import numpy as np
import pytest

from geothermalwells_gb300 import (GB300, ODEProblem, ROCK2, create_cache, eigen_estimator,
                                   rhs_diffusion_z, solve)
from geothermalwells_gb300 import _lib
from geothermalwells_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def refined(w, times):
    """The case with every x interval split in two, `times` times (more rows
    per x-line; the pipes keep their grid columns)."""
    gx = np.asarray(w["gridx"], dtype=np.float64)
    for _ in range(times):
        mid = 0.5 * (gx[1:] + gx[:-1])
        gx = np.sort(np.concatenate([gx, mid]))
    w = dict(w)
    w["gridx"] = gx
    w["T0"] = W.initial_condition_thermal_gradient(None, np.float64, gx, w["gridy"], w["gridz"],
                                                   T_surface=5.0, gradient=0.5)
    return w


CASES = {
    "single": lambda: W.small_case(),                                                   # 36 x 36 x 14
    "three_wells_layers_hx": lambda: W.small_case(n_layers=3, inlet="hx", nbh=3, nz_cells=40),   # 88 x 40
    "deep": lambda: W.small_case(nz_cells=300, n_layers=2),                             # nz = 301
    "2mm": W.single_well_2mm,
    "large": W.single_well_large,
}


def run(w, monkeypatch, global_y, tiling=None, overlap=None, nsteps=3):
    monkeypatch.delenv("GW_HALF_CPASYNC", raising=False)
    if global_y:
        monkeypatch.setenv("GW_HALF_GLOBAL", "1")
        monkeypatch.delenv("GW_HALF_TMEM_FORCE", raising=False)
    else:
        monkeypatch.delenv("GW_HALF_GLOBAL", raising=False)
        # on chip even where a half step has fewer than four rounds of blocks
        # (every grid here but the large well's)
        monkeypatch.setenv("GW_HALF_TMEM_FORCE", "1")
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


def test_default_small_grid_equals_global(gwlib, monkeypatch):
    """Without the override (the library's own choice of form for a grid of a
    few thousand cells) the field is the global form's, bitwise."""
    w = CASES["single"]()
    monkeypatch.delenv("GW_HALF_CPASYNC", raising=False)
    monkeypatch.delenv("GW_HALF_GLOBAL", raising=False)
    monkeypatch.delenv("GW_HALF_TMEM_FORCE", raising=False)
    c = create_cache(backend=GB300(precision="mixed"), gridx=w["gridx"], gridy=w["gridy"],
                     gridz=w["gridz"], materials=w["materials"], boreholes=w["boreholes"],
                     inlet_model=w["inlet_model"])
    sol = solve(ODEProblem(rhs_diffusion_z, w["T0"], (0.0, 3 * w["dt"]), c),
                ROCK2(max_stages=100, eigen_est=eigen_estimator), dt=w["dt"])
    c.close()
    assert np.array_equal(sol.u[-1], run(w, monkeypatch, global_y=True).u[-1])


@pytest.mark.parametrize("name", list(CASES))
def test_tmem_equals_global(name, gwlib, monkeypatch):
    w = CASES[name]()
    n = 2 if name in ("2mm", "large") else 3
    a = run(w, monkeypatch, global_y=True, nsteps=n)
    b = run(w, monkeypatch, global_y=False, nsteps=n)
    assert np.all(np.isfinite(b.u[-1]))
    assert np.array_equal(a.u[-1], b.u[-1])
    assert np.array_equal(a.T_outlet, b.T_outlet)


@pytest.mark.parametrize("tiling", range(6))
def test_every_tiling(tiling, gwlib, monkeypatch):
    w = W.small_case(n_layers=2, nbh=2, nz_cells=30)
    a = run(w, monkeypatch, global_y=True, tiling=tiling)
    b = run(w, monkeypatch, global_y=False, tiling=tiling)
    assert np.array_equal(a.u[-1], b.u[-1])
    assert np.array_equal(a.T_outlet, b.T_outlet)


@pytest.mark.parametrize("overlap", [0, 1])
def test_overlapped_step(overlap, gwlib, monkeypatch):
    w = W.small_case(n_layers=2, nbh=3, nz_cells=45)
    a = run(w, monkeypatch, global_y=True, overlap=overlap)
    b = run(w, monkeypatch, global_y=False, overlap=overlap)
    assert np.array_equal(a.u[-1], b.u[-1])
    assert np.array_equal(a.T_outlet, b.T_outlet)


@pytest.mark.parametrize("tiling", [0, 1, 3, 4])
def test_long_lines(tiling, gwlib, monkeypatch):
    w = refined(W.small_case(nz_cells=20), 3)
    assert len(w["gridx"]) > 256
    a = run(w, monkeypatch, global_y=True, tiling=tiling)
    b = run(w, monkeypatch, global_y=False, tiling=tiling)
    assert np.array_equal(a.u[-1], b.u[-1])
    assert np.array_equal(a.T_outlet, b.T_outlet)


def with_nx(w, n):
    """The case with exactly n x-points: outer points dropped (alternating
    ends; the pipes sit in the refined middle) or added beyond the ends at
    0.2 m spacing."""
    gx = list(np.asarray(w["gridx"], dtype=np.float64))
    left = True
    while len(gx) > n:
        gx.pop(0 if left else -1)
        left = not left
    while len(gx) < n:
        if left:
            gx.insert(0, gx[0] - 0.2)
        else:
            gx.append(gx[-1] + 0.2)
        left = not left
    gx = np.asarray(gx)
    w = dict(w)
    w["gridx"] = gx
    w["T0"] = W.initial_condition_thermal_gradient(None, np.float64, gx, w["gridy"], w["gridz"],
                                                   T_surface=5.0, gradient=0.5)
    return w


@pytest.mark.parametrize("nz_cells", [12, 45])
@pytest.mark.parametrize("nx", [20, 31, 33, 128, 129, 144, 208, 209, 256, 257])
def test_line_lengths_at_the_edges(nx, nz_cells, gwlib, monkeypatch):
    """x-lines whose length sits at the kernel's edges: one or two chunks,
    partial backward batches, the split form's 128-row boundary (129: one row
    in shared memory), its largest shared-memory share (208 / 209 rows) and
    the step to 512 columns per block (256 / 257); nz = 13 and 46 levels
    (one partial level block, two level blocks).  Tilings 0 (16-row chunks)
    and 3 (32-row chunks); bitwise the global-memory form."""
    w = with_nx(W.small_case(nz_cells=nz_cells), nx)
    assert len(w["gridx"]) == nx
    for tiling in (0, 3):
        a = run(w, monkeypatch, global_y=True, tiling=tiling, nsteps=2)
        b = run(w, monkeypatch, global_y=False, tiling=tiling, nsteps=2)
        assert np.all(np.isfinite(b.u[-1]))
        assert np.array_equal(a.u[-1], b.u[-1]), tiling
        assert np.array_equal(a.T_outlet, b.T_outlet), tiling
