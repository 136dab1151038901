"""GPU tests of the mixed-precision fused step (float storage of
theta = T - T_ref(z), float line solves, double outlet/energy balance)
against the FP64 oracle.  Bar (stated by the task for the mixed form): outlet
temperature within 1e-3 K; these short runs are held tighter."""
import numpy as np
import pytest

from geothermalwells_gb300 import (GB300, ODEProblem, ROCK2, create_cache, eigen_estimator,
                                   rhs_diffusion_z, rock2, solve)
from geothermalwells_gb300 import workloads as W
import oracle as O

pytestmark = pytest.mark.gpu

OUTLET_TOL_K = 1e-3
REF_T_OUTLET = 37.13620046384524   # test/test_integration.jl:17

CASES = {
    "single_const": dict(),
    "two_wells_layers_hx": dict(n_layers=3, inlet="hx", nbh=2),
    "many_stages": dict(backfill_quirk=True, n_layers=2),
}


def run_both(w, nsteps):
    cache = create_cache(backend=GB300(precision="mixed"), gridx=w["gridx"], gridy=w["gridy"],
                         gridz=w["gridz"], materials=w["materials"], boreholes=w["boreholes"],
                         inlet_model=w["inlet_model"])
    prob = ODEProblem(rhs_diffusion_z, w["T0"], (0.0, nsteps * w["dt"]), cache)
    sol = solve(prob, ROCK2(max_stages=100, eigen_est=eigen_estimator), dt=w["dt"], adaptive=False)
    orc = O.Oracle(w["gridx"], w["gridy"], w["gridz"], w["boreholes"], w["materials"],
                   w["inlet_model"])
    s, _ = rock2.choose_stages(w["dt"], orc.eigen_estimate())
    u = w["T0"].copy(order="F")
    out = orc.simulate(u, 0.0, w["dt"], nsteps, s, rock2.coefficients(s))
    return cache, sol, u, out


@pytest.mark.parametrize("name", list(CASES))
def test_mixed_small_cases(name, gwlib):
    w = W.small_case(**CASES[name])
    cache, sol, u, out = run_both(w, w["nsteps"])
    assert np.max(np.abs(sol.T_outlet - out)) < 1e-4
    assert np.max(np.abs(sol.u[-1] - u)) < 1e-3


def test_mixed_example_pin(gwlib):
    w = W.example_single_borehole()
    cache, sol, u, out = run_both(w, 10)
    assert abs(cache.T_outlet[0] - REF_T_OUTLET) < OUTLET_TOL_K
    assert np.max(np.abs(sol.T_outlet - out)) < OUTLET_TOL_K


def test_mixed_field_roundtrip(gwlib):
    """set_field / get_field through the theta representation."""
    w = W.small_case(n_layers=2)
    cache = create_cache(backend=GB300(precision="mixed"), gridx=w["gridx"], gridy=w["gridy"],
                         gridz=w["gridz"], materials=w["materials"], boreholes=w["boreholes"],
                         inlet_model=w["inlet_model"])
    rng = np.random.default_rng(3)
    T = np.asfortranarray(w["T0"] + rng.uniform(-1, 1, w["T0"].shape))
    cache.set_field(T)
    back = cache.get_field()
    assert np.max(np.abs(back - T)) < 1e-5


# The float ROCK2 column kernel takes 4..8 levels per thread, whichever pads
# the column least (gw_fused.cu, rock2_lpt); these z resolutions of the small
# well select each of them: nz = 14, 129, 161, 193, 225.
LPT_NZ_CELLS = {4: 12, 5: 127, 6: 159, 7: 191, 8: 223}


def float_levels_per_thread(nz):
    best, pad = 8, ((nz + 7) // 8 + 31) // 32 * 32 * 8
    for L in range(7, 3, -1):
        nt = ((nz + L - 1) // L + 31) // 32 * 32
        if nt <= 256 and nt * L < pad:
            best, pad = L, nt * L
    return best


@pytest.mark.parametrize("lpt", sorted(LPT_NZ_CELLS))
def test_mixed_rock2_levels_per_thread(lpt, gwlib):
    w = W.small_case(nz_cells=LPT_NZ_CELLS[lpt], n_layers=2)
    assert float_levels_per_thread(len(w["gridz"])) == lpt
    cache, sol, u, out = run_both(w, 4)
    assert np.max(np.abs(sol.T_outlet - out)) < 1e-4
    assert np.max(np.abs(sol.u[-1] - u)) < 1e-3
