"""Ensemble (batched designs): one graph launch per step advances every
design exactly as its own gw_step does, for every half-step tiling."""
import numpy as np
import pytest

from geothermalwells_gb300 import GB300, ODEProblem, ROCK2, create_cache, eigen_estimator, rhs_diffusion_z, solve
from geothermalwells_gb300.ensemble import Ensemble, TILINGS
from geothermalwells_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def designs():
    return [W.small_case(), W.small_case(n_layers=3, inlet="hx", nbh=2),
            W.small_case(backfill_quirk=True, n_layers=2, nz_cells=16)]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batch_equals_single_contexts(precision, gwlib):
    ds = designs()
    dt, n = 40.0, 5
    ens = Ensemble(ds, precision=precision)
    ens.step(dt, n)
    for d, (design, c) in enumerate(zip(ds, ens.caches)):
        single = create_cache(backend=GB300(precision=precision), gridx=design["gridx"],
                              gridy=design["gridy"], gridz=design["gridz"],
                              materials=design["materials"], boreholes=design["boreholes"],
                              inlet_model=design["inlet_model"])
        sol = solve(ODEProblem(rhs_diffusion_z, design["T0"], (0.0, n * dt), single),
                    ROCK2(max_stages=100, eigen_est=eigen_estimator), dt=dt)
        assert np.array_equal(c.get_field(), sol.u[-1])
        assert np.array_equal(ens.outlet_series(d, n), sol.T_outlet)
    ens.close()


@pytest.mark.parametrize("tiling", range(len(TILINGS)))
def test_every_tiling_gives_the_same_field(tiling, gwlib):
    """The row-tile tilings run the same elimination order: bitwise equal.
    The segmented tiling re-associates the line recurrences (segment scans):
    equal to float rounding, 1e-5 of the field's magnitude (float epsilon
    1.2e-7 times the ~200-row recurrences)."""
    ds = designs()
    a = Ensemble(ds, precision="mixed")
    a.step(40.0, 3)
    b = Ensemble(ds, precision="mixed")
    b.set_tiling(tiling)
    b.step(40.0, 3)
    for ca, cb in zip(a.caches, b.caches):
        fa, fb = ca.get_field(), cb.get_field()
        if TILINGS[tiling][1] == "seg8x32":
            assert np.max(np.abs(fa - fb)) <= 1e-5 * np.max(np.abs(fa))
        else:
            assert np.array_equal(fa, fb)
    a.close(); b.close()


def test_autotune_returns_valid_choices(gwlib):
    ens = Ensemble(designs(), precision="mixed")
    choice = ens.autotune(40.0, reps=1)
    assert len(choice) == 3 and all(0 <= t < len(TILINGS) for t in choice)
    ens.step(40.0, 2)
    ens.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_device_initial_field_equals_host_field(precision, gwlib):
    """gw_init_thermal_gradient fills the field on the device: the same field
    as the host-built initial_condition_thermal_gradient, and the same run."""
    from geothermalwells_gb300 import initial_condition_thermal_gradient
    ds = designs()
    ic = [(4.0 + q, 0.03 + 0.01 * q) for q in range(len(ds))]
    host = [dict(d, T0=initial_condition_thermal_gradient(None, np.float64, d["gridx"], d["gridy"],
                                                          d["gridz"], T_surface=ts, gradient=g))
            for d, (ts, g) in zip(ds, ic)]
    a = Ensemble(host, precision=precision)
    by_id = {id(d): v for d, v in zip(ds, ic)}
    b = Ensemble(ds, precision=precision, initial_gradient=lambda d: by_id[id(d)])
    for ca, cb, h in zip(a.caches, b.caches, host):
        assert np.array_equal(cb.get_field(), ca.get_field())
        assert np.array_equal(cb.get_field(), h["T0"])
    a.step(40.0, 3)
    b.step(40.0, 3)
    for d, (ca, cb) in enumerate(zip(a.caches, b.caches)):
        assert np.array_equal(ca.get_field(), cb.get_field())
        assert np.array_equal(a.outlet_series(d, 3), b.outlet_series(d, 3))
    a.close(); b.close()


def _refined_x(w, times):
    """The design with every x interval split in two, `times` times."""
    from geothermalwells_gb300.physics import initial_condition_thermal_gradient
    gx = np.asarray(w["gridx"], dtype=np.float64)
    for _ in range(times):
        gx = np.sort(np.concatenate([gx, 0.5 * (gx[1:] + gx[:-1])]))
    return dict(w, gridx=gx, T0=initial_condition_thermal_gradient(None, np.float64, gx, w["gridy"], w["gridz"],
                                                                   T_surface=5.0, gradient=0.5))


@pytest.mark.parametrize("tiling", [0, 1])
def test_on_chip_half_steps_of_designs_running_at_once(tiling, gwlib, monkeypatch):
    """Eight designs whose half steps keep their forward values in tensor
    memory run at once on their own streams: their blocks share every SM's
    512 TMEM columns (x-lines of 141 rows take the split form's 128 columns
    per block, x-lines of 481 rows all 512 with the 4-line tiling, so blocks
    of different designs wait for each other's columns).  The
    fields and outlet series equal those of the same ensemble with the
    forward values in global memory, bitwise."""
    ds = [_refined_x(W.small_case(n_layers=1 + q % 3, nbh=1 + q % 2, nz_cells=12 + 4 * q), 3 if q % 2 else 2)
          for q in range(8)]
    monkeypatch.delenv("GW_HALF_CPASYNC", raising=False)
    monkeypatch.delenv("GW_HALF_TMEM_FORCE", raising=False)
    monkeypatch.setenv("GW_HALF_GLOBAL", "1")
    a = Ensemble(ds, precision="mixed")
    monkeypatch.delenv("GW_HALF_GLOBAL")
    monkeypatch.setenv("GW_HALF_TMEM_FORCE", "1")
    b = Ensemble(ds, precision="mixed")
    a.set_tiling(tiling)
    b.set_tiling(tiling)
    a.step(40.0, 3)
    b.step(40.0, 3)
    for d, (ca, cb) in enumerate(zip(a.caches, b.caches)):
        assert np.all(np.isfinite(cb.get_field()))
        assert np.array_equal(ca.get_field(), cb.get_field())
        assert np.array_equal(a.outlet_series(d, 3), b.outlet_series(d, 3))
    a.close(); b.close()
