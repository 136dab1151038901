"""Context-level behaviour of the C ABI on the GPU: kernel attributes shared
between contexts, the step path a context reports, the half-step tiling
setter, and the device fields for hosts without a CUDA binding."""
import ctypes

import numpy as np
import pytest

from geothermalwells_gb300 import (GB300, ODEProblem, ROCK2, create_cache, eigen_estimator,
                                   rhs_diffusion_z, rock2, solve)
from geothermalwells_gb300 import _lib
from geothermalwells_gb300 import workloads as W
import oracle as O

pytestmark = pytest.mark.gpu


def make(w, precision="fp64"):
    return create_cache(backend=GB300(precision=precision), gridx=w["gridx"], gridy=w["gridy"],
                        gridz=w["gridz"], materials=w["materials"], boreholes=w["boreholes"],
                        inlet_model=w["inlet_model"])


def info(cache):
    i = _lib.Info()
    _lib.check(_lib.load().gw_get_info(cache.ctx, ctypes.byref(i)))
    return i


def run(cache, w, nsteps):
    return solve(ODEProblem(rhs_diffusion_z, w["T0"], (0.0, nsteps * w["dt"]), cache),
                 ROCK2(max_stages=100, eigen_est=eigen_estimator), dt=w["dt"], adaptive=False)


def test_column_kernel_limit_survives_a_smaller_context(gwlib):
    """An FP64 context with nz > 4096 runs the shared-memory column kernel;
    creating a context with few levels afterwards must not lower that
    kernel's shared-memory limit under the first one."""
    big = W.small_case(nz_cells=4200)
    a = make(big)
    first = run(a, big, 2)
    b = make(W.small_case())
    run(b, W.small_case(), 1)
    again = run(a, big, 2)
    assert info(a).fused == 1
    assert np.array_equal(first.u[-1], again.u[-1])
    assert np.array_equal(first.T_outlet, again.T_outlet)
    a.close(); b.close()


def test_fused_context_reports_fused(gwlib):
    c = make(W.small_case(), "fp64")
    i = info(c)
    assert i.fused == 1 and i.modular_reason == 0 and i.tiling == 0 and i.mixed_options == 0
    c.close()


def test_default_tiling(gwlib, monkeypatch):
    """Mixed contexts start with tiling 0 (4 lines x 16 rows, forward values
    on chip) where its half steps have at least four rounds of blocks, else
    with tiling 9 (8 x 8, forward values in global memory); FP64 contexts
    always with 0."""
    monkeypatch.delenv("GW_HALF_TMEM_FORCE", raising=False)
    monkeypatch.delenv("GW_HALF_GLOBAL", raising=False)
    monkeypatch.delenv("GW_HALF_CPASYNC", raising=False)
    c = make(W.small_case(), "mixed")          # 36 x 36 x 14: nine blocks per half step
    assert info(c).fused == 1 and info(c).tiling == 9
    c.close()
    c = make(W.single_well_large(), "mixed")   # 63 level blocks x 52 line groups
    assert info(c).tiling == 0
    c.close()
    monkeypatch.setenv("GW_HALF_TMEM_FORCE", "1")
    c = make(W.small_case(), "mixed")
    assert info(c).tiling == 0
    c.close()
    monkeypatch.delenv("GW_HALF_TMEM_FORCE")
    monkeypatch.setenv("GW_HALF_GLOBAL", "1")  # the same tiling with its values in global memory
    c = make(W.small_case(), "mixed")
    assert info(c).tiling == 0
    c.close()


def test_shared_pipe_column_runs_modular_and_says_so(gwlib):
    """Two boreholes whose pipes share grid columns (the later borehole
    overrides, src/physics.jl:204-229): FP64 contexts run the modular step
    and report why; it still matches the oracle.  Mixed contexts refuse."""
    w = W.small_case(nbh=2, spacing=0.05)
    c = make(w)
    i = info(c)
    assert i.fused == 0 and i.modular_reason == _lib.GW_MODULAR_SHARED_COLUMN
    orc = O.Oracle(w["gridx"], w["gridy"], w["gridz"], w["boreholes"], w["materials"], w["inlet_model"])
    s, _ = rock2.choose_stages(w["dt"], orc.eigen_estimate())
    u = w["T0"].copy(order="F")
    out = orc.simulate(u, 0.0, w["dt"], 3, s, rock2.coefficients(s))
    orc.close()
    sol = run(c, w, 3)
    assert np.max(np.abs(sol.u[-1] - u)) / np.max(np.abs(u)) < 1e-10
    assert np.max(np.abs(sol.T_outlet - out)) / np.max(np.abs(out)) < 1e-10
    c.close()
    with pytest.raises(_lib.GWError) as e:
        make(w, "mixed")
    assert e.value.code == _lib.GW_ERR_UNSUPPORTED


def test_set_tiling(gwlib):
    L = _lib.load()
    c = make(W.small_case(), "mixed")
    assert L.gw_set_tiling(c.ctx, _lib_tilings()) == _lib.GW_ERR_ARG
    assert L.gw_set_tiling(c.ctx, -1) == _lib.GW_ERR_ARG
    _lib.check(L.gw_set_tiling(c.ctx, 3))
    assert info(c).tiling == 3
    c.close()


def _lib_tilings():
    from geothermalwells_gb300.ensemble import TILINGS
    return len(TILINGS)


def test_device_fields_round_trip(gwlib):
    """gw_field_alloc / gw_field_copy / gw_field_free with gw_lincomb: the
    device fields a host language without a CUDA binding uses."""
    L = _lib.load()
    w = W.small_case()
    c = make(w)
    n = c.N
    rng = np.random.default_rng(2)
    a_h = rng.uniform(-1, 1, n)
    b_h = rng.uniform(-1, 1, n)
    pa, pb = ctypes.c_void_p(), ctypes.c_void_p()
    _lib.check(L.gw_field_alloc(c.ctx, ctypes.byref(pa)))
    _lib.check(L.gw_field_alloc(c.ctx, ctypes.byref(pb)))
    zero = np.ones(n)
    _lib.check(L.gw_field_copy(c.ctx, _lib.dptr(zero), pa))
    assert np.all(zero == 0.0)                          # allocated as zeros
    _lib.check(L.gw_field_copy(c.ctx, pa, _lib.dptr(a_h)))
    _lib.check(L.gw_field_copy(c.ctx, pb, _lib.dptr(b_h)))
    coeffs = np.array([2.0, -0.5])
    srcs = (ctypes.c_void_p * 2)(pa, pb)
    _lib.check(L.gw_lincomb(c.ctx, pa, 2, _lib.dptr(coeffs), srcs))   # a = 2a - b/2
    back = np.zeros(n)
    _lib.check(L.gw_field_copy(c.ctx, _lib.dptr(back), pa))
    assert np.allclose(back, 2.0 * a_h - 0.5 * b_h, rtol=0, atol=1e-15)
    _lib.check(L.gw_field_copy(c.ctx, pb, pa))          # device to device
    _lib.check(L.gw_field_copy(c.ctx, _lib.dptr(back), pb))
    assert np.allclose(back, 2.0 * a_h - 0.5 * b_h, rtol=0, atol=1e-15)
    _lib.check(L.gw_field_free(c.ctx, pa))
    _lib.check(L.gw_field_free(c.ctx, pb))
    c.close()


SETUP_CASES = {
    "small_layers_3wells": lambda: W.small_case(nbh=3, n_layers=3, insulation_depth=40.0, inlet="hx"),
    "well_array_example": W.example_well_array,
    "2mm": W.single_well_2mm,
    "ensemble_design": lambda: (lambda d: dict(d, T0=W.initial_field(d), dt=600.0))(W.ensemble()[1]),
}


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("name", list(SETUP_CASES))
def test_device_setup_equals_host_setup(name, precision, gwlib, monkeypatch):
    """The material classification, column profiles, coefficient tables and
    Thomas factors built on the GPU (the default) give the host builders'
    tables bitwise: the steps of both contexts agree bit for bit."""
    w = SETUP_CASES[name]()
    monkeypatch.setenv("GW_HOST_SETUP", "1")
    host = make(w, precision)
    monkeypatch.delenv("GW_HOST_SETUP")
    dev = make(w, precision)
    ih, id_ = info(host), info(dev)
    assert (ih.n_zclass, ih.n_profiles, ih.countxy_inner, ih.countxy_outer) == \
        (id_.n_zclass, id_.n_profiles, id_.countxy_inner, id_.countxy_outer)
    a = run(host, w, 3)
    b = run(dev, w, 3)
    assert np.array_equal(a.u[-1], b.u[-1])
    assert np.array_equal(a.T_outlet, b.T_outlet)
    host.close(); dev.close()
