"""Schedule inlet (GW_INLET_SCHEDULE): the CustomInlet form
(bh, T_outlet, t) -> T_in(t), piecewise linear, that crosses the C ABI.

CPU: the oracle's schedule with one point is the constant inlet.
GPU: fused steps and the fine-grained advection against the oracle (FP64,
1e-10 / 1e-12), the mixed path against FP64 (1e-3 K), the overlapped step
and the ensemble against the in-line single context (bitwise), and the
adjoint's refusal."""
import numpy as np
import pytest

from geothermalwells_gb300 import (GB300, ConstantInlet, ScheduleInlet, ODEProblem, ROCK2, create_cache,
                                   eigen_estimator, rhs_diffusion_z, rock2, solve, advection)
from geothermalwells_gb300 import workloads as W
from geothermalwells_gb300 import _lib
import oracle as O

SCHED = ScheduleInlet([0.0, 100.0, 150.0, 220.0], [10.0, 14.0, 6.0, 9.0])


def case(inlet=SCHED, **kw):
    w = W.small_case(**kw)
    return dict(w, inlet_model=inlet)


def oracle_run(w, nsteps):
    orc = O.Oracle(w["gridx"], w["gridy"], w["gridz"], w["boreholes"], w["materials"], w["inlet_model"])
    s, _ = rock2.choose_stages(w["dt"], orc.eigen_estimate())
    u = w["T0"].copy(order="F")
    out = orc.simulate(u, 0.0, w["dt"], nsteps, s, rock2.coefficients(s))
    orc.close()
    return u, out


def test_schedule_inlet_validation():
    with pytest.raises(ValueError):
        ScheduleInlet([0.0, 0.0], [1.0, 2.0])
    with pytest.raises(ValueError):
        ScheduleInlet([0.0, 1.0], [1.0])
    assert abs(SCHED(0, None, 125.0) - 10.0) < 1e-12   # halfway from 14 down to 6
    assert SCHED(0, None, -5.0) == 10.0 and SCHED(0, None, 500.0) == 9.0


def test_oracle_one_point_schedule_is_the_constant_inlet():
    u1, o1 = oracle_run(case(ScheduleInlet([50.0], [12.5])), 4)
    u2, o2 = oracle_run(case(ConstantInlet(12.5)), 4)
    assert np.array_equal(u1, u2) and np.array_equal(o1, o2)


def gpu(w, precision="fp64", nsteps=6, overlap=None):
    cache = create_cache(backend=GB300(precision=precision), gridx=w["gridx"], gridy=w["gridy"],
                         gridz=w["gridz"], materials=w["materials"], boreholes=w["boreholes"],
                         inlet_model=w["inlet_model"])
    if overlap is not None:
        _lib.check(_lib.load().gw_set_overlap(cache.ctx, overlap))
    sol = solve(ODEProblem(rhs_diffusion_z, w["T0"], (0.0, nsteps * w["dt"]), cache),
                ROCK2(max_stages=100, eigen_est=eigen_estimator), dt=w["dt"])
    return cache, sol


def rel(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / np.max(np.abs(np.asarray(b))))


@pytest.mark.gpu
@pytest.mark.parametrize("kw", [dict(), dict(n_layers=3, nbh=2)])
def test_fused_steps_with_schedule_match_oracle(kw, gwlib):
    w = case(**kw)
    u_ref, out_ref = oracle_run(w, 6)
    cache, sol = gpu(w)
    assert rel(sol.u[-1], u_ref) < 1e-10
    assert rel(sol.T_outlet, out_ref) < 1e-10


@pytest.mark.gpu
def test_advection_with_schedule_matches_oracle(gwlib, torch_cuda):
    torch = torch_cuda
    w = case()
    cache, _ = gpu(w, nsteps=0)
    orc = O.Oracle(w["gridx"], w["gridy"], w["gridz"], w["boreholes"], w["materials"], w["inlet_model"])
    phi = np.asfortranarray(w["T0"] + np.random.default_rng(4).uniform(-3, 3, w["T0"].shape))
    for t in (30.0, 125.0, 400.0):
        ref = phi.copy(order="F")
        orc.advection(ref, w["dt"] / 2, t)
        d = torch.from_numpy(phi.ravel(order="F").copy()).cuda()
        advection(d, w["dt"] / 2, t, cache)
        assert rel(d.cpu().numpy().reshape(phi.shape, order="F"), ref) < 1e-12


@pytest.mark.gpu
def test_mixed_with_schedule_against_fp64(gwlib):
    w = case(n_layers=2)
    _, s64 = gpu(w, "fp64")
    _, s32 = gpu(w, "mixed")
    assert np.max(np.abs(s32.T_outlet - s64.T_outlet)) < 1e-3


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_overlapped_step_with_schedule_is_bitwise(precision, gwlib):
    w = case(n_layers=3, nbh=2)
    _, a = gpu(w, precision, overlap=1)
    _, b = gpu(w, precision, overlap=0)
    assert np.array_equal(a.u[-1], b.u[-1]) and np.array_equal(a.T_outlet, b.T_outlet)


@pytest.mark.gpu
def test_ensemble_with_schedule_equals_single(gwlib):
    from geothermalwells_gb300.ensemble import Ensemble
    ds = [case(), case(n_layers=3, nbh=2)]
    ens = Ensemble(ds, precision="mixed")
    ens.step(40.0, 3)
    ens.step(40.0, 3)          # time continues across calls
    for d, (design, c) in enumerate(zip(ds, ens.caches)):
        _, sol = gpu(design, "mixed", nsteps=6)
        assert np.array_equal(c.get_field(), sol.u[-1])
    ens.close()


@pytest.mark.gpu
def test_adjoint_refuses_schedule(gwlib):
    from geothermalwells_gb300 import adjoint as A
    w = case()
    cache, _ = gpu(w, nsteps=0)
    with pytest.raises(_lib.GWError) as e:
        A.adjoint(cache, w["T0"], w["dt"], 2)
    assert e.value.code == _lib.GW_ERR_UNSUPPORTED
