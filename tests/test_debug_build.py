"""The bounds-checking debug build (gw_build.py --debug, -DGW_DEBUG): the
fused step's kernels check every global address against the registry of the
contexts' allocations and every dynamic shared-memory access against the
block's size, and a failed check comes back as GW_ERR_ARG (no trap).  This
target runs the small-case parity cases (both precisions, in-line and
overlapped steps), the reference's example and the 2 mm well, every
half-step tiling of the ensemble, and the mixed half steps with their forward
values in tensor memory and shared memory through that build in a child
process.

Opt-in (it compiles a second library, about 2.5 minutes):
    GW_DEBUG_BUILD_TESTS=1 python -m pytest tests/test_debug_build.py -m gpu"""
import os
import subprocess
import sys

import pytest

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not os.environ.get("GW_DEBUG_BUILD_TESTS"),
                                 reason="opt-in: set GW_DEBUG_BUILD_TESTS=1")]

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r'''
import sys, numpy as np
sys.path.insert(0, "geothermalwells.jl_gb300"); sys.path.insert(0, "oracle")
from geothermalwells_gb300 import (GB300, ODEProblem, ROCK2, create_cache, eigen_estimator,
                                   rhs_diffusion_z, rock2, solve, _lib)
from geothermalwells_gb300 import workloads as W
from geothermalwells_gb300.ensemble import Ensemble, TILINGS
import oracle as O
assert _lib.LIB_PATH.endswith("libgw_gb300_debug.so"), _lib.LIB_PATH
L = _lib.load()

def run(w, precision, n, overlap=None):
    c = create_cache(backend=GB300(precision=precision), gridx=w["gridx"], gridy=w["gridy"],
                     gridz=w["gridz"], materials=w["materials"], boreholes=w["boreholes"],
                     inlet_model=w["inlet_model"])
    if overlap is not None:
        _lib.check(L.gw_set_overlap(c.ctx, overlap))
    sol = solve(ODEProblem(rhs_diffusion_z, w["T0"], (0.0, n * w["dt"]), c),
                ROCK2(max_stages=100, eigen_est=eigen_estimator), dt=w["dt"])
    c.close()
    return sol

cases = [dict(), dict(n_layers=3, inlet="hx", nbh=2), dict(backfill_quirk=True, n_layers=2),
         dict(nbh=3, insulation_depth=40.0, inlet="hx", nz_cells=16)]
for kw in cases:
    w = W.small_case(**kw)
    orc = O.Oracle(w["gridx"], w["gridy"], w["gridz"], w["boreholes"], w["materials"], w["inlet_model"])
    s, _ = rock2.choose_stages(w["dt"], orc.eigen_estimate())
    u = w["T0"].copy(order="F"); out = orc.simulate(u, 0.0, w["dt"], 4, s, rock2.coefficients(s)); orc.close()
    for prec in ("fp64", "mixed"):
        for ov in (0, 1):
            sol = run(w, prec, 4, overlap=ov)
            tol = 1e-10 if prec == "fp64" else 1e-3
            err = np.max(np.abs(sol.u[-1] - u)) / (np.max(np.abs(u)) if prec == "fp64" else 1.0)
            assert err < tol, (kw, prec, ov, err)
for w in (W.example_single_borehole(), W.single_well_2mm()):
    for prec in ("fp64", "mixed"):
        run(w, prec, 2)
designs = [W.small_case(), W.small_case(n_layers=3, inlet="hx", nbh=2),
           W.small_case(backfill_quirk=True, n_layers=2, nz_cells=16)]
for prec in ("fp64", "mixed"):
    for t in range(len(TILINGS)):
        e = Ensemble(designs, precision=prec)
        e.set_tiling(t)
        e.step(40.0, 3)
        e.close()
# the mixed half steps with their forward values on chip (forced on these
# small grids): whole lines in TMEM, the split form (141-row lines), 512-column
# blocks (281-row lines), and the 2 mm well
import os
os.environ["GW_HALF_TMEM_FORCE"] = "1"
def refined(w, times):
    from geothermalwells_gb300.physics import initial_condition_thermal_gradient
    gx = np.asarray(w["gridx"], dtype=np.float64)
    for _ in range(times):
        gx = np.sort(np.concatenate([gx, 0.5 * (gx[1:] + gx[:-1])]))
    return dict(w, gridx=gx, T0=initial_condition_thermal_gradient(None, np.float64, gx, w["gridy"], w["gridz"],
                                                                   T_surface=5.0, gradient=0.5))
for w in (W.small_case(n_layers=2, nbh=2), refined(W.small_case(nz_cells=20), 2),
          refined(W.small_case(nz_cells=20), 3), W.single_well_2mm()):
    for t in (0, 1, 3):
        c = create_cache(backend=GB300(precision="mixed"), gridx=w["gridx"], gridy=w["gridy"],
                         gridz=w["gridz"], materials=w["materials"], boreholes=w["boreholes"],
                         inlet_model=w["inlet_model"])
        _lib.check(L.gw_set_tiling(c.ctx, t))
        solve(ODEProblem(rhs_diffusion_z, w["T0"], (0.0, 2 * w["dt"]), c),
              ROCK2(max_stages=100, eigen_est=eigen_estimator), dt=w["dt"])
        c.close()
print("debug build: no bounds check failed")
'''


def test_debug_build_runs_clean(gwlib):
    import gw_build
    lib = gw_build.build(debug=True)
    env = dict(os.environ, GW_LIB=lib)
    r = subprocess.run([sys.executable, "-c", CHILD], cwd=ROOT, env=env, capture_output=True, text=True,
                       timeout=1200)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "no bounds check failed" in r.stdout
