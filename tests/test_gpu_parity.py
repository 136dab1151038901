"""GPU parity: every hot-path entry point of the C ABI against the FP64 CPU
oracle on the same inputs.  FP64 bar (stated by the benchmark spec): 1e-10 relative on
the temperature field and the outlet temperature; single kernels are held to
1e-12."""
import numpy as np
import pytest

from geothermalwells_gb300 import (GB300, ODEProblem, ROCK2, create_cache, eigen_estimator,
                                   get_simulation_callback, rhs_diffusion_z, diffusion_1d,
                                   thomas_I_minus_A, advection, ADI_and_ADV_callback, rock2, solve)
from geothermalwells_gb300 import workloads as W
import oracle as O

pytestmark = pytest.mark.gpu

FIELD_RTOL = 1e-10       # full steps, FP64
KERNEL_RTOL = 1e-12      # one kernel, FP64
REF_T_OUTLET = 37.13620046384524   # test/test_integration.jl:17

CASES = {
    "single_const": dict(),
    "two_wells_layers_hx": dict(n_layers=3, inlet="hx", nbh=2),
    "many_stages": dict(backfill_quirk=True, n_layers=2),
    "three_wells_insulated": dict(nbh=3, insulation_depth=40.0, inlet="hx", nz_cells=16),
}


def rel_err(a, b):
    a = np.asarray(a, dtype=np.float64); b = np.asarray(b, dtype=np.float64)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def make(w, precision="fp64"):
    cache = create_cache(backend=GB300(precision=precision), gridx=w["gridx"], gridy=w["gridy"],
                         gridz=w["gridz"], materials=w["materials"], boreholes=w["boreholes"],
                         inlet_model=w["inlet_model"])
    orc = O.Oracle(w["gridx"], w["gridy"], w["gridz"], w["boreholes"], w["materials"],
                   w["inlet_model"])
    return cache, orc


def to_dev(torch, a):
    return torch.from_numpy(np.asfortranarray(a).ravel(order="F").copy()).cuda()


def to_host(t, shape):
    return t.cpu().numpy().reshape(shape, order="F")


def perturbed(w, seed=0):
    rng = np.random.default_rng(seed)
    T = w["T0"] + rng.uniform(-3.0, 3.0, w["T0"].shape)
    return np.asfortranarray(T)


@pytest.mark.parametrize("name", list(CASES))
def test_cache_counts_match_oracle(name, gwlib):
    w = W.small_case(**CASES[name])
    cache, orc = make(w)
    c = orc.counts()
    assert (cache.countxy_inner, cache.countxy_outer, cache.countz) == \
        (c["countxy_inner"], c["countxy_outer"], c["countz"])
    assert cache.eigen_estimate == orc.eigen_estimate()


@pytest.mark.parametrize("name", list(CASES))
def test_rhs_diffusion_z(name, gwlib, torch_cuda):
    w = W.small_case(**CASES[name])
    cache, orc = make(w)
    phi = perturbed(w, 1)
    ref = np.zeros_like(phi, order="F")
    orc.rhs_diffusion_z(ref, phi)
    d_phi, d_out = to_dev(torch_cuda, phi), torch_cuda.zeros(phi.size, dtype=torch_cuda.float64, device="cuda")
    rhs_diffusion_z(d_out, d_phi, cache, 0.0)
    assert rel_err(to_host(d_out, phi.shape), ref) < KERNEL_RTOL


@pytest.mark.parametrize("name", list(CASES))
@pytest.mark.parametrize("direction", ["x", "y", "z"])
def test_explicit_sweep(name, direction, gwlib, torch_cuda):
    w = W.small_case(**CASES[name])
    cache, orc = make(w)
    phi = perturbed(w, 2)
    ref = np.zeros_like(phi, order="F")
    orc.diffusion_1d(ref, phi, w["dt"] / 2, direction, True)
    d_phi = to_dev(torch_cuda, phi)
    d_out = torch_cuda.zeros_like(d_phi)
    diffusion_1d(d_out, d_phi, cache, w["dt"] / 2, direction, True)
    assert rel_err(to_host(d_out, phi.shape), ref) < KERNEL_RTOL


@pytest.mark.parametrize("name", list(CASES))
@pytest.mark.parametrize("direction", ["x", "y"])
def test_thomas(name, direction, gwlib, torch_cuda):
    w = W.small_case(**CASES[name])
    cache, orc = make(w)
    rhs = perturbed(w, 3)
    ref = np.zeros_like(rhs, order="F")
    orc.thomas(ref, rhs, w["dt"] / 2, direction)
    d_rhs = to_dev(torch_cuda, rhs)
    d_U = torch_cuda.zeros_like(d_rhs)
    thomas_I_minus_A(d_U, d_rhs, cache, w["dt"] / 2, direction)
    assert rel_err(to_host(d_U, rhs.shape), ref) < KERNEL_RTOL


@pytest.mark.parametrize("name", list(CASES))
def test_advection(name, gwlib, torch_cuda):
    w = W.small_case(**CASES[name])
    cache, orc = make(w)
    phi = perturbed(w, 4)
    ref = phi.copy(order="F")
    orc.advection(ref, w["dt"] / 2, 0.0)
    d_phi = to_dev(torch_cuda, phi)
    advection(d_phi, w["dt"] / 2, 0.0, cache)
    assert rel_err(to_host(d_phi, phi.shape), ref) < KERNEL_RTOL
    assert rel_err(cache.T_outlet, orc.outlet()) < KERNEL_RTOL


@pytest.mark.parametrize("name", list(CASES))
def test_adi_adv_callback(name, gwlib, torch_cuda):
    w = W.small_case(**CASES[name])
    cache, orc = make(w)
    u = perturbed(w, 5)
    ref = u.copy(order="F")
    orc.adi_adv(ref, w["dt"], w["dt"])
    d_u = to_dev(torch_cuda, u)
    d_tmp = torch_cuda.zeros_like(d_u)
    ADI_and_ADV_callback(d_u, d_tmp, w["dt"], w["dt"], cache)
    assert rel_err(to_host(d_u, u.shape), ref) < KERNEL_RTOL
    assert rel_err(cache.T_outlet, orc.outlet()) < KERNEL_RTOL


def oracle_run(w, orc, nsteps):
    s, _ = rock2.choose_stages(w["dt"], orc.eigen_estimate())
    u = w["T0"].copy(order="F")
    out = orc.simulate(u, w["t0"], w["dt"], nsteps, s, rock2.coefficients(s))
    return u, out, s


def gpu_run(w, cache, nsteps, callback=None):
    prob = ODEProblem(rhs_diffusion_z, w["T0"], (w["t0"], w["t0"] + nsteps * w["dt"]), cache)
    return solve(prob, ROCK2(max_stages=100, eigen_est=eigen_estimator), dt=w["dt"],
                 adaptive=False, save_everystep=False, callback=callback)


@pytest.mark.parametrize("name", list(CASES))
def test_fused_steps_match_oracle(name, gwlib):
    w = W.small_case(**CASES[name])
    cache, orc = make(w)
    u_ref, out_ref, s = oracle_run(w, orc, w["nsteps"])
    sol = gpu_run(w, cache, w["nsteps"])
    assert sol.stages == s
    assert rel_err(sol.u[-1], u_ref) < FIELD_RTOL
    assert rel_err(sol.T_outlet, out_ref) < FIELD_RTOL
    assert rel_err(cache.T_outlet, orc.outlet()) < FIELD_RTOL


def test_many_stages_case_uses_many_stages(gwlib):
    w = W.small_case(**CASES["many_stages"])
    cache, orc = make(w)
    s, covered = rock2.choose_stages(w["dt"], orc.eigen_estimate())
    assert s > 8 and covered


def test_example_pin_on_gpu(gwlib):
    """The reference example through the GB300 path: saved snapshots, outlet
    pin and the integration test's checks (test/test_integration.jl)."""
    w = W.example_single_borehole()
    cache, orc = make(w)
    cb, saved = get_simulation_callback(saveat=np.linspace(0.0, 800.0, 11), print_every_n=1)
    sol = gpu_run(w, cache, 10, callback=cb)
    assert len(saved.t) == 11 and saved.t[-1] == 800.0
    T_out = cache.T_outlet[0]
    assert abs(T_out - REF_T_OUTLET) / REF_T_OUTLET < 1e-10
    assert 20.0 < T_out < w["T0"][-1, 0, 0]
    T_final = saved.saveval[-1]
    assert saved.saveval[0].dtype == np.float32
    assert np.all(np.isfinite(T_final)) and T_final.min() > -50 and T_final.max() < 200
    u_ref, out_ref, _ = oracle_run(w, orc, 10)
    assert rel_err(sol.u[-1], u_ref) < FIELD_RTOL
    assert rel_err(sol.T_outlet, out_ref) < FIELD_RTOL


def test_well_array_example(gwlib):
    """examples/well_array_basic.jl (2 x 2 wells, HeatExchangerInlet)."""
    w = W.example_well_array()
    cache, orc = make(w)
    u_ref, out_ref, _ = oracle_run(w, orc, 4)
    sol = gpu_run(w, cache, 4)
    assert rel_err(sol.u[-1], u_ref) < FIELD_RTOL
    assert rel_err(sol.T_outlet, out_ref) < FIELD_RTOL


def test_single_well_2mm_first_steps(gwlib):
    """The 225 x 225 x 402 benchmark well, first steps element-wise."""
    w = W.single_well_2mm()
    cache, orc = make(w)
    u_ref, out_ref, _ = oracle_run(w, orc, 3)
    sol = gpu_run(w, cache, 3)
    assert rel_err(sol.u[-1], u_ref) < FIELD_RTOL
    assert rel_err(sol.T_outlet, out_ref) < FIELD_RTOL


def test_energy_balance(gwlib):
    """Extracted heat = sum over steps of mdot c_w (T_out - T_in) dt."""
    w = W.small_case(**CASES["two_wells_layers_hx"])
    cache, orc = make(w)
    sol = gpu_run(w, cache, w["nsteps"])
    c_w = w["materials"].rho_c_water / 998.2
    for b, bh in enumerate(w["boreholes"]):
        to = sol.T_outlet[:, b]
        ti = to - w["inlet_model"].dT
        want = np.sum(bh.mdot * c_w * (to - ti) * w["dt"])
        assert abs(sol.energy[b] - want) <= 1e-12 * abs(want)


def test_nonfinite_detection(gwlib):
    from geothermalwells_gb300 import _lib
    w = W.small_case()
    cache, orc = make(w)
    T = w["T0"].copy(order="F")
    cache.set_field(T)
    assert _lib.load().gw_check_finite(cache.ctx) == _lib.GW_OK
    T[3, 2, 1] = np.nan
    cache.set_field(T)
    assert _lib.load().gw_check_finite(cache.ctx) == _lib.GW_ERR_NONFINITE


def test_aliasing_rejected(gwlib, torch_cuda):
    from geothermalwells_gb300 import _lib
    w = W.small_case()
    cache, orc = make(w)
    d = to_dev(torch_cuda, w["T0"])
    with pytest.raises(_lib.GWError):
        thomas_I_minus_A(d, d, cache, 1.0, "x")
    with pytest.raises(_lib.GWError):
        rhs_diffusion_z(d, d, cache, 0.0)


@pytest.mark.parametrize("case", ["small_const", "two_wells_layers_hx", "example", "2mm"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_overlapped_step_is_bitwise_the_in_line_step(case, precision, gwlib):
    """The step with its pipe passes on a second stream (gw_set_overlap) gives
    exactly the in-line step's field and outlet series."""
    from geothermalwells_gb300 import _lib
    w = {"small_const": lambda: W.small_case(), "two_wells_layers_hx": lambda: W.small_case(n_layers=3, inlet="hx", nbh=2),
         "example": W.example_single_borehole, "2mm": W.single_well_2mm}[case]()
    L = _lib.load()
    out = []
    for on in (1, 0):
        cache = create_cache(backend=GB300(precision=precision), gridx=w["gridx"], gridy=w["gridy"],
                             gridz=w["gridz"], materials=w["materials"], boreholes=w["boreholes"],
                             inlet_model=w["inlet_model"])
        _lib.check(L.gw_set_overlap(cache.ctx, on))
        info = _lib.Info()
        _lib.check(L.gw_get_info(cache.ctx, info))
        assert info.overlap == on
        sol = gpu_run(w, cache, 3)
        out.append((sol.u[-1], sol.T_outlet))
        cache.close()
    assert np.array_equal(out[0][0], out[1][0])
    assert np.array_equal(out[0][1], out[1][1])


def test_lincomb(gwlib, torch_cuda):
    """gw_lincomb: dst = sum of weighted fields, dst aliasing a source."""
    from geothermalwells_gb300.solver import lincomb
    torch = torch_cuda
    w = W.small_case()
    cache, _ = make(w)
    rng = np.random.default_rng(9)
    fields = [rng.uniform(-5, 5, cache.N) for _ in range(5)]
    dev = [torch.from_numpy(f.copy()).cuda() for f in fields]
    coeffs = [0.5, -1.25, 3.0, 1e-3, -2.0]
    out = torch.zeros(cache.N, dtype=torch.float64, device="cuda")
    lincomb(out, coeffs, dev, cache)
    ref = sum(c * f for c, f in zip(coeffs, fields))
    assert np.max(np.abs(out.cpu().numpy() - ref)) <= 1e-13 * np.max(np.abs(ref))
    lincomb(dev[0], [2.0, 1.0], [dev[0], dev[1]], cache)   # in place
    assert np.max(np.abs(dev[0].cpu().numpy() - (2 * fields[0] + fields[1]))) <= 1e-13 * 20
