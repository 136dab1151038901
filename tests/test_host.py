"""CPU tests: the oracle against the reference's own known answers, the
host-side set-up (grids, materials, inlets, ROCK2 table), mirroring
``test/test_basic.jl`` and ``test/test_integration.jl`` of the reference."""
import math

import numpy as np
import pytest

from geothermalwells_gb300 import (Borehole, ConstantInlet, CustomInlet, HeatExchangerInlet,
                                   HomogenousMaterialProperties, StratifiedMaterialProperties,
                                   compute_domain, create_adaptive_grid_1d,
                                   create_uniform_gridz_with_borehole_depths,
                                   get_thermal_conductivity, get_volumetric_heat_capacity,
                                   initial_condition_thermal_gradient, julia_colon, julia_range,
                                   rock2)
from geothermalwells_gb300 import workloads as W
import oracle as O

# test/test_integration.jl:17 -- the reference's only known answer on the path
REF_T_OUTLET = 37.13620046384524


def run_oracle(w, nsteps=None):
    orc = O.Oracle(w["gridx"], w["gridy"], w["gridz"], w["boreholes"], w["materials"],
                   w["inlet_model"])
    s, _ = rock2.choose_stages(w["dt"], orc.eigen_estimate())
    u = w["T0"].copy(order="F")
    out = orc.simulate(u, w["t0"], w["dt"], nsteps or w["nsteps"], s, rock2.coefficients(s))
    return orc, u, out, s


@pytest.fixture(scope="module")
def example_run():
    w = W.example_single_borehole()
    orc, u, out, s = run_oracle(w)
    return w, orc, u, out, s


def test_example_grid_sizes(example_run):
    w = example_run[0]
    assert (len(w["gridx"]), len(w["gridy"]), len(w["gridz"])) == (157, 157, 38)


def test_oracle_pins_reference_outlet(example_run):
    """The oracle reproduces the reference's integration-test value to 1e-12
    (the reference test itself only asks rtol 0.05)."""
    w, orc, u, out, s = example_run
    assert s == 4
    assert math.isclose(out[-1, 0], REF_T_OUTLET, rel_tol=1e-12)


def test_oracle_integration_asserts(example_run):
    """test/test_integration.jl:20-34."""
    w, orc, u, out, s = example_run
    T0 = w["T0"]
    T_out = out[-1, 0]
    assert T_out < T0[-1, 0, 0] and T_out > 20.0
    assert np.all(np.isfinite(u)) and u.min() > -50 and u.max() < 200
    # Julia's isapprox on arrays: norm(x - y) <= rtol * max(norm(x), norm(y))
    for j, i in [(0, 0), (0, -1), (-1, 0), (-1, -1)]:
        a, b = u[:, j, i], T0[:, j, i]
        assert np.linalg.norm(a - b) <= 1e-5 * max(np.linalg.norm(a), np.linalg.norm(b))


def test_borehole_construction():
    """test/test_basic.jl:8-29."""
    bh = Borehole(0, 0, 3500, 0.0381, 0.01, 0.0889, 0.01, 0.0989, 10, 1000)
    assert bh.h == 3500.0 and bh.mdot == 10.0 and bh.insulation_depth == 1000.0
    assert bh.v_inner > 0 and bh.v_outer > 0
    assert bh.v_inner == 10.0 / (math.pi * 0.0381 ** 2 * 998.2)


def test_stratified_layers():
    """test/test_basic.jl:53-94: z <= depth selects the layer, deepest below."""
    m = StratifiedMaterialProperties((1.8, 2.6, 3.5, 5.3),
                                     (1780 * 1379.0, 2030 * 1450.0, 1510 * 1300.0, 2600 * 878.0),
                                     (500.0, 1000.0, 1500.0, 2000.0), 0.618, 4.166e6, 41.0,
                                     7850 * 475.0, 0.4, 1.955e6, 1.5, 1.76e6)
    assert [m.rock_k(z) for z in (100, 500, 750, 1250, 1750, 3000)] == [1.8, 1.8, 2.6, 3.5, 5.3, 5.3]
    assert m.rock_rho_c(100) == 1780 * 1379.0 and m.rock_rho_c(3000) == 2600 * 878.0
    d = max(max(k / r for k, r in zip(m.k_rock_layers, m.rho_c_rock_layers)), 0.618 / 4.166e6,
            41.0 / (7850 * 475.0), 0.4 / 1.955e6, 1.5 / 1.76e6)
    assert math.isclose(m.d_max(), d)


def test_material_lookup_matches_oracle():
    """Host lookups, oracle lookups: identical on every material class."""
    w = W.small_case(n_layers=3, nbh=2)
    orc = O.Oracle(w["gridx"], w["gridy"], w["gridz"], w["boreholes"], w["materials"],
                   w["inlet_model"])
    rng = np.random.default_rng(1)
    for _ in range(400):
        x = rng.choice(w["gridx"]); y = rng.choice(w["gridy"]); z = rng.choice(w["gridz"])
        k, r = orc.material(x, y, z)
        assert k == get_thermal_conductivity(x, y, z, w["boreholes"], w["materials"])
        assert r == get_volumetric_heat_capacity(x, y, z, w["boreholes"], w["materials"])


def test_grid_creation():
    """test/test_basic.jl:96-130."""
    bh = Borehole(0.0, 0.0, 2000 - 1, 0.0511, 0.0114, 0.0885, 0.00833, 0.115, 11.65, 0.0)
    dom = compute_domain([bh], buffer_x=100, buffer_y=100, buffer_z=200 + 1)
    assert dom["xmin"] == -100 and dom["xmax"] == 100 and dom["zmax"] == 2200
    gz = create_uniform_gridz_with_borehole_depths(zmin=0, zmax=2200, dz=100, boreholes=(bh,))
    assert bh.h in gz and gz[0] == 0
    gx = create_adaptive_grid_1d(xmin=-100, xmax=100, dx_fine=0.0025, growth_factor=1.3,
                                 dx_max=10.0, boreholes=(bh,), direction="x")
    assert gx[0] == -100 and gx[-1] == 100 and np.diff(gx).min() <= 0.0025


def test_grid_multiple_boreholes():
    """test/test_basic.jl:132-194."""
    b1 = Borehole(-15.0, 0.0, 1500.0, 0.0511, 0.0114, 0.0885, 0.00833, 0.115, 11.65, 0.0)
    b2 = Borehole(15.0, 0.0, 2000.0, 0.0511, 0.0114, 0.0885, 0.00833, 0.115, 11.65, 0.0)
    gx = create_adaptive_grid_1d(xmin=-100, xmax=100, dx_fine=0.0025, growth_factor=1.3,
                                 dx_max=10.0, boreholes=(b1, b2), direction="x")
    assert gx[0] == -100.0 and gx[-1] == 100.0
    assert np.all(np.diff(gx) > 0)
    assert np.any(np.abs(gx - b1.xc) < b1.r_backfill) and np.any(np.abs(gx - b2.xc) < b2.r_backfill)
    between = gx[(gx > b1.xc + b1.r_backfill) & (gx < b2.xc - b2.r_backfill)]
    assert len(between) > 0
    gz = create_uniform_gridz_with_borehole_depths(zmin=0, zmax=2500, dz=100, boreholes=(b1, b2))
    assert 1500.0 in gz and 2000.0 in gz and np.all(np.diff(gz) > 0)


def test_julia_range_rounding():
    """Points are correctly rounded from the decimal-rational endpoints, not
    accumulated: 0:1.1:2200 gives fl(k*11/10)."""
    g = julia_colon(0.0, 1.1, 2200.0)
    assert len(g) == 2001 and g[3] == 3.3 and g[-1] == 2200.0
    r = julia_range(-0.0989, 0.0989, 81)
    assert r[0] == -0.0989 and r[-1] == 0.0989 and r[40] == 0.0
    assert julia_range(0.0, 0.3, 4)[3] == 0.3


def test_initial_condition():
    """test/test_basic.jl:196-213."""
    gx = julia_colon(0.0, 10.0, 100.0)
    gz = julia_colon(0.0, 100.0, 3700.0)
    T0 = initial_condition_thermal_gradient(None, np.float64, gx, gx, gz, T_surface=2.29,
                                            gradient=0.035)
    assert T0.shape == (len(gz), len(gx), len(gx)) and T0.flags.f_contiguous
    assert math.isclose(T0[0, 0, 0], 2.29) and math.isclose(T0[-1, 0, 0], 2.29 + 0.035 * 3700.0)


def test_inlet_models():
    """test/test_basic.jl:215-236."""
    assert ConstantInlet(20.0)(0, [0.0], 0.0) == 20.0
    mdot = 42 * 998.2 / 3600
    dT = 200e3 / (mdot * 4174.0)
    assert math.isclose(HeatExchangerInlet(dT)(0, [50.0], 0.0), 50.0 - dT)
    assert math.isclose(CustomInlet(lambda b, T, t: 20.0 + 0.01 * t)(0, [0.0], 100.0), 21.0)


def test_array_domain():
    """test/test_basic.jl:238-257."""
    bhs = [Borehole(x, y, 2000.0, 0.0511, 0.0114, 0.0885, 0.00833, 0.115, 11.65, 0.0)
           for y in (-30.0, 0.0, 30.0) for x in (-30.0, 0.0, 30.0)]
    d = compute_domain(bhs, buffer_x=100, buffer_y=100, buffer_z=200)
    assert (d["xmin"], d["xmax"], d["ymin"], d["ymax"]) == (-130, 130, -130, 130)


def test_index_lists_counts():
    """Advection index lists (src/cache.jl:9-44) on the benchmark geometries."""
    w = W.single_well_2mm()
    orc = O.Oracle(w["gridx"], w["gridy"], w["gridz"], w["boreholes"], w["materials"],
                   w["inlet_model"])
    c = orc.counts()
    assert (c["countxy_inner"], c["countxy_outer"], c["countz"]) == (3069, 1924, 365)


# ---- ROCK2 table -----------------------------------------------------------

def _R(s, z):
    mu, nu, kappa, sigma, tau = rock2.coefficients(s)
    g0 = np.ones_like(z)
    gm, g = g0, g0
    for j in range(s - 2):
        gn = g + mu[0] * z * g if j == 0 else mu[j] * z * g - nu[j] * g - kappa[j] * gm
        gm, g = g, gn
    gq = g + sigma * z * g
    gs = gq + sigma * z * gq
    return gs - sigma * (1 - tau / sigma ** 2) * (z * gq - z * g)


@pytest.mark.parametrize("s", [2, 3, 4, 5, 8, 13, 21, 34, 55, 89, 100])
def test_rock2_order_and_stability(s):
    """Published properties of ROCK2: order two and a stability interval
    growing like ~0.8 s^2."""
    P = np.polynomial.Polynomial
    coef = _R(s, P([0.0, 1.0])).coef
    assert abs(coef[0] - 1) < 1e-12 and abs(coef[1] - 1) < 1e-9 and abs(coef[2] - 0.5) < 1e-8
    l = rock2.stability_interval(s)
    z = -l * (1 - np.cos(np.linspace(0, np.pi, 60 * s))) / 2
    assert np.abs(_R(s, z)).max() <= 1.0 + 1e-9
    if s >= 10:
        assert 0.79 < l / s ** 2 < 0.81
    mu, nu, kappa, _, _ = rock2.coefficients(s)
    assert np.allclose(-nu - kappa, 1.0, atol=1e-12)


def test_rock2_stage_rule():
    assert rock2.choose_stages(60.0, 2.4e-5) == (3, True)
    assert rock2.choose_stages(80.0, 0.08) == (4, True)
    s, ok = rock2.choose_stages(1.0, 1e9, max_stages=100)
    assert s == 100 and not ok
