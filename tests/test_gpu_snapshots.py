"""Asynchronous float snapshots (gw_snapshot): the SavingCallback of
save_and_print_callback (src/cache.jl:132-184) keeps u as Float32 at every
saveat time.  Here the conversion runs on the device and the copy to pinned
host memory overlaps the following steps.  Each snapshot must equal the
blocking read-back of the field at that time, rounded to float, bitwise --
through solve()'s callback and through the C ABI with three snapshots in
flight (the two staging buffers reused)."""
import ctypes

import numpy as np
import pytest

from geothermalwells_gb300 import (GB300, ODEProblem, ROCK2, create_cache, eigen_estimator,
                                   get_simulation_callback, rhs_diffusion_z, solve)
from geothermalwells_gb300 import _lib
from geothermalwells_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def make(w, precision):
    return create_cache(backend=GB300(precision=precision), gridx=w["gridx"], gridy=w["gridy"],
                        gridz=w["gridz"], materials=w["materials"], boreholes=w["boreholes"],
                        inlet_model=w["inlet_model"])


def blocking_fields(w, precision, steps):
    """get_field at each of the given step counts, rounded to float."""
    c = make(w, precision)
    c.set_field(w["T0"])
    out, done = {}, 0
    for n in sorted(steps):
        if n > done:
            _lib.check(_lib.load().gw_step(c.ctx, done * w["dt"], w["dt"], n - done, 100))
            done = n
        out[n] = c.get_field().astype(np.float32)
    c.close()
    return out


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_solve_snapshots_equal_blocking_reads(precision, gwlib):
    w = W.small_case(n_layers=2, nbh=2)
    dt = w["dt"]
    steps = [0, 2, 5, 6]
    cb, saved = get_simulation_callback(saveat=[n * dt for n in steps], print_every_n=0)
    c = make(w, precision)
    solve(ODEProblem(rhs_diffusion_z, w["T0"], (0.0, 6 * dt), c), ROCK2(max_stages=100, eigen_est=eigen_estimator),
          dt=dt, callback=cb)
    want = blocking_fields(w, precision, steps)
    assert saved.t == [n * dt for n in steps]
    for n, got in zip(steps, saved.saveval):
        assert got.dtype == np.float32 and got.shape == w["T0"].shape
        assert np.array_equal(got, want[n])
    c.close()


@pytest.mark.parametrize("pinned", [True, False])
def test_three_snapshots_in_flight(pinned, gwlib):
    L = _lib.load()
    w = W.single_well_2mm()
    c = make(w, "mixed")
    c.set_field(w["T0"])
    n = c.N
    bufs, keep = [], []
    for _ in range(3):
        if pinned:
            p = ctypes.c_void_p()
            _lib.check(L.gw_snapshot_host_alloc(c.ctx, ctypes.byref(p)))
            bufs.append(p)
        else:
            a = np.full(n, np.nan, dtype=np.float32)
            keep.append(a)
            bufs.append(ctypes.c_void_p(a.ctypes.data))
    steps = [1, 3, 4]
    done = 0
    for b, s in zip(bufs, steps):
        _lib.check(L.gw_step(c.ctx, done * w["dt"], w["dt"], s - done, 100))
        done = s
        _lib.check(L.gw_snapshot(c.ctx, b))
    _lib.check(L.gw_step(c.ctx, done * w["dt"], w["dt"], 2, 100))   # steps while the copies land
    _lib.check(L.gw_snapshot_wait(c.ctx))
    want = blocking_fields(w, "mixed", steps)
    for b, s in zip(bufs, steps):
        got = np.ctypeslib.as_array(ctypes.cast(b, ctypes.POINTER(ctypes.c_float)), shape=(n,))
        assert np.array_equal(got.reshape(w["T0"].shape, order="F"), want[s])
    if pinned:
        for b in bufs:
            _lib.check(L.gw_snapshot_host_free(c.ctx, b))
    c.close()
