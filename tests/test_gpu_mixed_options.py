"""The mixed step's two optional FP64 parts (gw_set_mixed_options):

* GW_MIXED_ROCK2_F64: the ROCK2 stages accumulated in double over the float
  field, rounded into it once per step;
* GW_MIXED_REFINE: after each float line solve, the residual of the half
  step's equation in double and one correction solve.

Each against the FP64 oracle on the small cases at the mixed path's bars
(outlet within 1e-4 K and field within 1e-3 K over these short runs; the
task's bar for the outlet is 1e-3 K), each visibly active (the field differs
from the default mixed step's), and the adjoint's refusal of a step it does
not transpose."""
import ctypes

import numpy as np
import pytest

from geothermalwells_gb300 import (GB300, ODEProblem, ROCK2, create_cache, eigen_estimator,
                                   rhs_diffusion_z, rock2, solve)
from geothermalwells_gb300 import _lib
from geothermalwells_gb300 import workloads as W
import oracle as O

pytestmark = pytest.mark.gpu

CASES = {
    "single_const": dict(),
    "two_wells_layers_hx": dict(n_layers=3, inlet="hx", nbh=2),
    "many_stages": dict(backfill_quirk=True, n_layers=2),
}
OPTIONS = {"rock2_f64": _lib.GW_MIXED_ROCK2_F64, "refine": _lib.GW_MIXED_REFINE,
           "both": _lib.GW_MIXED_ROCK2_F64 | _lib.GW_MIXED_REFINE}


def oracle_run(w, nsteps):
    orc = O.Oracle(w["gridx"], w["gridy"], w["gridz"], w["boreholes"], w["materials"], w["inlet_model"])
    s, _ = rock2.choose_stages(w["dt"], orc.eigen_estimate())
    u = w["T0"].copy(order="F")
    out = orc.simulate(u, 0.0, w["dt"], nsteps, s, rock2.coefficients(s))
    orc.close()
    return u, out


def mixed_run(w, nsteps, flags=0):
    cache = create_cache(backend=GB300(precision="mixed"), gridx=w["gridx"], gridy=w["gridy"],
                         gridz=w["gridz"], materials=w["materials"], boreholes=w["boreholes"],
                         inlet_model=w["inlet_model"])
    _lib.check(_lib.load().gw_set_mixed_options(cache.ctx, flags))
    i = _lib.Info()
    _lib.check(_lib.load().gw_get_info(cache.ctx, ctypes.byref(i)))
    assert i.mixed_options == flags
    sol = solve(ODEProblem(rhs_diffusion_z, w["T0"], (0.0, nsteps * w["dt"]), cache),
                ROCK2(max_stages=100, eigen_est=eigen_estimator), dt=w["dt"], adaptive=False)
    return cache, sol


@pytest.mark.parametrize("option", list(OPTIONS))
@pytest.mark.parametrize("name", list(CASES))
def test_option_against_oracle(name, option, gwlib):
    w = W.small_case(**CASES[name])
    n = w["nsteps"]
    u, out = oracle_run(w, n)
    c0, base = mixed_run(w, n)
    c1, sol = mixed_run(w, n, OPTIONS[option])
    assert np.max(np.abs(sol.T_outlet - out)) < 1e-4
    assert np.max(np.abs(sol.u[-1] - u)) < 1e-3
    assert not np.array_equal(sol.u[-1], base.u[-1])     # the option is active
    c0.close(); c1.close()


def test_options_in_the_example_pin(gwlib):
    """The reference example (test/test_integration.jl:17) with both options."""
    w = W.example_single_borehole()
    _, out = oracle_run(w, 10)
    c, sol = mixed_run(w, 10, OPTIONS["both"])
    assert abs(c.T_outlet[0] - 37.13620046384524) < 1e-3
    assert np.max(np.abs(sol.T_outlet - out)) < 1e-3
    c.close()


def test_option_validation(gwlib):
    L = _lib.load()
    w = W.small_case()
    c64 = create_cache(backend=GB300(precision="fp64"), gridx=w["gridx"], gridy=w["gridy"],
                       gridz=w["gridz"], materials=w["materials"], boreholes=w["boreholes"],
                       inlet_model=w["inlet_model"])
    assert L.gw_set_mixed_options(c64.ctx, _lib.GW_MIXED_REFINE) == _lib.GW_ERR_ARG
    assert L.gw_set_mixed_options(c64.ctx, 0) == _lib.GW_OK
    c, _ = mixed_run(w, 0)
    assert L.gw_set_mixed_options(c.ctx, 4) == _lib.GW_ERR_ARG
    c64.close(); c.close()


def test_adjoint_refuses_options(gwlib):
    from geothermalwells_gb300 import adjoint as A
    w = W.adjoint_small(n_layers=2, nsteps=2)
    c, _ = mixed_run(w, 0, OPTIONS["refine"])
    with pytest.raises(_lib.GWError) as e:
        A.adjoint(c, w["T0"], w["dt"], 2)
    assert e.value.code == _lib.GW_ERR_UNSUPPORTED
    c.close()


def fp64_run(w, nsteps):
    cache = create_cache(backend=GB300(precision="fp64"), gridx=w["gridx"], gridy=w["gridy"],
                         gridz=w["gridz"], materials=w["materials"], boreholes=w["boreholes"],
                         inlet_model=w["inlet_model"])
    sol = solve(ODEProblem(rhs_diffusion_z, w["T0"], (0.0, nsteps * w["dt"]), cache),
                ROCK2(max_stages=100, eigen_est=eigen_estimator), dt=w["dt"], adaptive=False)
    cache.close()
    return sol


@pytest.mark.parametrize("name", list(CASES) + ["2mm"])
def test_refine_double_float_matches_double(name, gwlib, monkeypatch):
    """GW_MIXED_REFINE forms its residual in double-float on the FP32 pipe
    (k_half_refine_df, the default) or in double (k_half_refine,
    GW_REFINE_F64=1).  Both residuals are exact far below the float rounding
    of the corrected field, so the two refined fields differ only where x + d
    rounds to neighbouring floats (carried on by the later steps), and the
    double-float one is as close to the FP64 solution as the double one."""
    w = W.single_well_2mm() if name == "2mm" else W.small_case(**CASES[name])
    n = 4
    ref = fp64_run(w, n)
    monkeypatch.setenv("GW_REFINE_F64", "1")
    c0, d64 = mixed_run(w, n, _lib.GW_MIXED_REFINE)
    monkeypatch.delenv("GW_REFINE_F64")
    c1, dff = mixed_run(w, n, _lib.GW_MIXED_REFINE)
    e64 = np.max(np.abs(d64.u[-1] - ref.u[-1]))
    eff = np.max(np.abs(dff.u[-1] - ref.u[-1]))
    o64 = np.max(np.abs(d64.T_outlet - ref.T_outlet))
    off = np.max(np.abs(dff.T_outlet - ref.T_outlet))
    assert eff <= 1.25 * e64 + 2e-5, (eff, e64)
    assert off <= 1.25 * o64 + 2e-6, (off, o64)
    assert np.max(np.abs(dff.u[-1] - d64.u[-1])) < 2e-4
    c0.close(); c1.close()
