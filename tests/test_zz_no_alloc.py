"""gw_advection_noalloc: the advection entry point for callers that cannot
let the library allocate device memory (a host integrator whose device
buffers all come from its own pool, or a process that reserves its share of
a shared GPU once at start-up).  It must give what gw_advection gives,
through the C ABI, on two calls in a row (the second call runs over the
first call's leftovers in the shared scratch array), for constant,
heat-exchanger and schedule inlets.

Collected last on purpose (file name), so a run that stops at the first
failure has already run every other test."""
import ctypes

import numpy as np
import pytest

from geothermalwells_gb300 import GB300, ScheduleInlet, create_cache
from geothermalwells_gb300 import _lib
from geothermalwells_gb300 import workloads as W

pytestmark = pytest.mark.gpu

RTOL = 1e-12   # the single-kernel tolerance of the parity tests


def rel_err(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def to_dev(torch, a):
    return torch.from_numpy(np.asfortranarray(a).ravel(order="F").copy()).cuda()


# a schedule whose points bracket the call times below (t between two points)
SCHED = ScheduleInlet([0.0, 100.0, 150.0, 220.0], [10.0, 14.0, 6.0, 9.0])


@pytest.mark.parametrize("case,times", [(dict(), (0.0, 0.0)),
                                        (dict(n_layers=3, inlet="hx", nbh=2), (0.0, 0.0)),
                                        (dict(nbh=2, schedule=True), (125.0, 60.0))])
def test_noalloc_matches_gw_advection_twice(case, times, gwlib, torch_cuda):
    torch = torch_cuda
    case = dict(case)
    sched = case.pop("schedule", False)
    w = W.small_case(**case)
    if sched:
        w["inlet_model"] = SCHED
    cache = create_cache(backend=GB300(), gridx=w["gridx"], gridy=w["gridy"], gridz=w["gridz"],
                         materials=w["materials"], boreholes=w["boreholes"],
                         inlet_model=w["inlet_model"])
    rng = np.random.default_rng(7)
    T_out_dev = torch.full((cache.N_bh,), np.nan, dtype=torch.float64, device="cuda")
    for call, (dt, t) in enumerate(zip((w["dt"] / 2, w["dt"] * 1.5), times)):
        phi = np.asfortranarray(w["T0"] + rng.uniform(-4.0, 4.0, w["T0"].shape))
        d_ref = to_dev(torch, phi)
        d_new = to_dev(torch, phi)
        torch.cuda.synchronize()
        _lib.check(gwlib.gw_advection(cache.ctx, d_ref.data_ptr(), dt, t))
        ref_outlet = cache.T_outlet
        _lib.check(gwlib.gw_advection_noalloc(cache.ctx, d_new.data_ptr(), dt, t,
                                              T_out_dev.data_ptr()))
        torch.cuda.synchronize()
        got = d_new.cpu().numpy()
        want = d_ref.cpu().numpy()
        assert rel_err(got, want) < RTOL, "call %d" % call
        assert rel_err(T_out_dev.cpu().numpy(), ref_outlet) < RTOL, "call %d" % call
        assert not np.array_equal(got, phi.ravel(order="F"))   # the pipes did move


def test_noalloc_rejects_oversized_problems(gwlib, torch_cuda):
    torch = torch_cuda
    # nz = 70001 > 65536 - 1: beyond the scratch array (a 3 x 3 x 70001 grid)
    w = W.small_case()
    g = np.array([-1.0, 0.0, 1.0])
    cache = create_cache(backend=GB300(), gridx=g, gridy=g, gridz=np.linspace(0.0, 700.0, 70001),
                         materials=w["materials"], boreholes=w["boreholes"],
                         inlet_model=w["inlet_model"])
    d = torch.zeros(cache.N, dtype=torch.float64, device="cuda")
    out = torch.zeros(cache.N_bh, dtype=torch.float64, device="cuda")
    rc = gwlib.gw_advection_noalloc(cache.ctx, d.data_ptr(), 1.0, 0.0, out.data_ptr())
    assert rc == _lib.GW_ERR_ARG
    assert b"limit" in gwlib.gw_last_error() or b"levels" in gwlib.gw_last_error()
