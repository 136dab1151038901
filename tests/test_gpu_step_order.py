"""Launch order of the overlapped step.  Order 0 runs ROCK2 of the pipe rows'
columns first, then forks the pipe passes onto a second stream. Order 1
starts the second stream at once with ROCK2 of the pipe columns and their
y-neighbours. Without GW_STEP_ORDER, gw_step times both orders on trial steps
whenever it captures a new graph, restores the state, and keeps the faster one.
All three runs must give the same field, outlet series, and energy values, bitwise:
over two consecutive gw_step calls (the second continues the first's state),
with constant, heat-exchanger and schedule inlets, and in both precisions."""
import ctypes

import numpy as np
import pytest

from geothermalwells_gb300 import GB300, ScheduleInlet, create_cache
from geothermalwells_gb300 import _lib
from geothermalwells_gb300 import workloads as W

pytestmark = pytest.mark.gpu

SCHED = ScheduleInlet([0.0, 100.0, 150.0, 220.0], [10.0, 14.0, 6.0, 9.0])


def run(w, precision, order, monkeypatch, n1=5, n2=12):
    if order is None:
        monkeypatch.delenv("GW_STEP_ORDER", raising=False)
    else:
        monkeypatch.setenv("GW_STEP_ORDER", str(order))
    c = create_cache(backend=GB300(precision=precision), gridx=w["gridx"], gridy=w["gridy"], gridz=w["gridz"],
                     materials=w["materials"], boreholes=w["boreholes"], inlet_model=w["inlet_model"])
    L = _lib.load()
    info = _lib.Info()
    _lib.check(L.gw_get_info(c.ctx, ctypes.byref(info)))
    assert info.overlap == 1
    c.set_field(w["T0"])
    dt = w["dt"]
    series = []
    t = 0.0
    for n in (n1, n2):
        _lib.check(L.gw_step(c.ctx, t, dt, n, 100))
        s = np.zeros(n * c.N_bh)
        _lib.check(L.gw_get_outlet_series(c.ctx, _lib.dptr(s), n))
        series.append(s)
        t += n * dt
    energy = np.zeros(c.N_bh)
    _lib.check(L.gw_get_energy(c.ctx, _lib.dptr(energy)))
    u = c.get_field()
    c.close()
    return u, np.concatenate(series), energy


CASES = {
    "constant": lambda: W.small_case(n_layers=2, nbh=3, nz_cells=45),
    "hx": lambda: W.small_case(n_layers=3, inlet="hx", nbh=2, nz_cells=40),
    "schedule": lambda: dict(W.small_case(n_layers=3, nbh=2), inlet_model=SCHED),
}


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
@pytest.mark.parametrize("name", list(CASES))
def test_orders_and_timed_choice_are_bitwise_equal(name, precision, gwlib, monkeypatch):
    w = CASES[name]()
    ref = run(w, precision, 0, monkeypatch)
    for order in (1, None):
        got = run(w, precision, order, monkeypatch)
        assert np.all(np.isfinite(got[0]))
        for a, b in zip(ref, got):
            assert np.array_equal(a, b), (name, precision, order)


def test_timed_choice_on_the_2mm_well(gwlib, monkeypatch):
    """The 2 mm well (225 x 225 x 402), whose second stream is the longer
    chain: the timed choice gives the fixed orders' state, bitwise."""
    w = W.single_well_2mm()
    ref = run(w, "mixed", 0, monkeypatch, n1=3, n2=9)
    got = run(w, "mixed", None, monkeypatch, n1=3, n2=9)
    for a, b in zip(ref, got):
        assert np.array_equal(a, b)
