"""Expression inlet (GW_INLET_EXPRESSION): a CustomInlet whose closure
(bh, T_outlet, t) -> T_in is arithmetic in the borehole's outlet
temperature, t, the borehole index and a schedule -- the outlet-dependent
control laws of heat-pump operation, e.g. max(T_min, T_out - dT(t)).

CPU: the compiler, and the oracle's program evaluation against the three
fixed inlet models it generalises (bitwise).  GPU: fused steps, the
fine-grained advection, the mixed path, the overlapped step and the
ensemble against the oracle or the in-line single context, and the entry
points that refuse a program."""
import ctypes

import numpy as np
import pytest

from geothermalwells_gb300 import (GB300, ConstantInlet, ExpressionInlet, HeatExchangerInlet, ODEProblem,
                                   ROCK2, ScheduleInlet, advection, create_cache, eigen_estimator,
                                   rhs_diffusion_z, rock2, solve)
from geothermalwells_gb300 import _lib
from geothermalwells_gb300 import physics as P
from geothermalwells_gb300 import workloads as W
import oracle as O

SCHED = ([0.0, 100.0, 150.0, 220.0], [3.0, 6.0, 1.0, 4.0])
# a heat pump taking dT(t) out of the outlet, never cooling the inlet below 12
HEAT_PUMP = ExpressionInlet("max(12.0, T_out - sched(t))", schedule=SCHED)
# borehole-dependent and nonlinear in the outlet
MIXED_LAW = ExpressionInlet("min(T_out - 1.5 - 0.25 * bh, 0.02 * T_out * T_out + t / 1000.0)")


def case(inlet, **kw):
    return dict(W.small_case(**kw), inlet_model=inlet)


def oracle_run(w, nsteps):
    orc = O.Oracle(w["gridx"], w["gridy"], w["gridz"], w["boreholes"], w["materials"], w["inlet_model"])
    s, _ = rock2.choose_stages(w["dt"], orc.eigen_estimate())
    u = w["T0"].copy(order="F")
    out = orc.simulate(u, 0.0, w["dt"], nsteps, s, rock2.coefficients(s))
    orc.close()
    return u, out


def test_compiler():
    assert HEAT_PUMP.ops == (P.OP_CONST, P.OP_TOUT, P.OP_TIME, P.OP_SCHED, P.OP_SUB, P.OP_MAX)
    assert HEAT_PUMP.args[0] == 12.0
    assert ExpressionInlet("-(T_out) + 2").ops == (P.OP_TOUT, P.OP_NEG, P.OP_CONST, P.OP_ADD)
    assert ExpressionInlet("max(1, 2, bh)").ops == (P.OP_CONST, P.OP_CONST, P.OP_MAX, P.OP_BH, P.OP_MAX)
    assert HEAT_PUMP(0, [20.0], 125.0) == max(12.0, 20.0 - 3.5)
    for bad in ("T_out ** 2", "foo(t)", "T_in", "sched(t)", "1 if t else 2", "T_out > 3"):
        with pytest.raises(ValueError):
            ExpressionInlet(bad)


@pytest.mark.parametrize("expr,fixed", [("20.0", ConstantInlet(20.0)),
                                        ("T_out - 3.0", HeatExchangerInlet(3.0)),
                                        ("sched(t)", ScheduleInlet(*SCHED))])
def test_oracle_programs_reproduce_the_fixed_models(expr, fixed):
    prog = ExpressionInlet(expr, schedule=SCHED if "sched" in expr else None)
    u1, o1 = oracle_run(case(prog, nbh=2), 4)
    u2, o2 = oracle_run(case(fixed, nbh=2), 4)
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
@pytest.mark.parametrize("law", [HEAT_PUMP, MIXED_LAW], ids=["heat_pump", "mixed_law"])
@pytest.mark.parametrize("kw", [dict(nbh=2), dict(n_layers=3, nbh=3)])
def test_fused_steps_match_oracle(law, kw, gwlib):
    w = case(law, **kw)
    u_ref, out_ref = oracle_run(w, 6)
    cache, sol = gpu(w)
    assert rel(sol.u[-1], u_ref) < 1e-10
    assert rel(sol.T_outlet, out_ref) < 1e-10
    cache.close()


@pytest.mark.gpu
def test_advection_matches_oracle(gwlib, torch_cuda):
    torch = torch_cuda
    w = case(HEAT_PUMP, nbh=2)
    cache, _ = gpu(w, nsteps=0)
    orc = O.Oracle(w["gridx"], w["gridy"], w["gridz"], w["boreholes"], w["materials"], w["inlet_model"])
    phi = np.asfortranarray(w["T0"] + np.random.default_rng(4).uniform(-3, 3, w["T0"].shape))
    for t in (30.0, 125.0, 400.0):
        ref = phi.copy(order="F")
        orc.advection(ref, w["dt"] / 2, t)
        d = torch.from_numpy(phi.ravel(order="F").copy()).cuda()
        advection(d, w["dt"] / 2, t, cache)
        assert rel(d.cpu().numpy().reshape(phi.shape, order="F"), ref) < 1e-12
        assert rel(cache.T_outlet, orc.outlet()) < 1e-12
    orc.close()
    cache.close()


@pytest.mark.gpu
def test_mixed_against_fp64(gwlib):
    w = case(HEAT_PUMP, n_layers=2, nbh=2)
    c1, s64 = gpu(w, "fp64")
    c2, s32 = gpu(w, "mixed")
    assert np.max(np.abs(s32.T_outlet - s64.T_outlet)) < 1e-3
    c1.close(); c2.close()


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_overlapped_step_is_bitwise(precision, gwlib):
    w = case(MIXED_LAW, n_layers=3, nbh=2)
    ca, a = gpu(w, precision, overlap=1)
    cb, b = gpu(w, precision, overlap=0)
    assert np.array_equal(a.u[-1], b.u[-1]) and np.array_equal(a.T_outlet, b.T_outlet)
    ca.close(); cb.close()


@pytest.mark.gpu
def test_ensemble_equals_single(gwlib):
    from geothermalwells_gb300.ensemble import Ensemble
    ds = [case(HEAT_PUMP), case(MIXED_LAW, n_layers=3, nbh=2)]
    ens = Ensemble(ds, precision="mixed")
    ens.step(40.0, 3)
    ens.step(40.0, 3)
    for design, c in zip(ds, ens.caches):
        cs, sol = gpu(design, "mixed", nsteps=6)
        assert np.array_equal(c.get_field(), sol.u[-1])
        cs.close()
    ens.close()


@pytest.mark.gpu
def test_program_validation_and_refusals(gwlib, torch_cuda):
    L = _lib.load()
    w = case(HEAT_PUMP, nbh=2)
    cache, _ = gpu(w, nsteps=0)

    def setp(ops, args=None):
        ops = np.ascontiguousarray(ops, dtype=np.int32)
        args = np.ascontiguousarray(args if args is not None else np.zeros(len(ops)), dtype=np.float64)
        return L.gw_set_inlet_program(cache.ctx, len(ops), ops.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                      _lib.dptr(args))

    assert setp([P.OP_ADD]) == _lib.GW_ERR_ARG                       # operand missing
    assert setp([P.OP_TOUT, P.OP_TIME]) == _lib.GW_ERR_ARG           # two values left
    assert setp([99]) == _lib.GW_ERR_ARG                             # unknown operation
    assert setp([P.OP_CONST], [np.inf]) == _lib.GW_ERR_ARG           # non-finite constant
    assert setp([P.OP_CONST] * 17 + [P.OP_ADD] * 16) == _lib.GW_ERR_ARG   # stack deeper than 16
    assert setp(list(HEAT_PUMP.ops), list(HEAT_PUMP.args)) == _lib.GW_OK
    d = torch_cuda.zeros(cache.N, dtype=torch_cuda.float64, device="cuda")
    out = torch_cuda.zeros(cache.N_bh, dtype=torch_cuda.float64, device="cuda")
    assert L.gw_advection_noalloc(cache.ctx, d.data_ptr(), 1.0, 0.0, out.data_ptr()) == _lib.GW_ERR_UNSUPPORTED
    from geothermalwells_gb300 import adjoint as A
    with pytest.raises(_lib.GWError) as e:
        A.adjoint(cache, w["T0"], w["dt"], 2)
    assert e.value.code == _lib.GW_ERR_UNSUPPORTED
    cache.close()
