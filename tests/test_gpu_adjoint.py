"""Adjoint (gw_adjoint, gw_step_vjp) on the GPU against

* central finite differences of the FP64 CPU oracle (the reference's own
  step): |g_adj - g_fd| <= 1e-4 |g_fd| per parameter, the bar the gradient
  is held to (the FD's own error at these cases is below 1e-5 relative,
  tests/test_adjoint_oracle.py);
* exact identities of the step map, which is affine in the field for fixed
  parameters: <dJ/du^0, v> = J(u^0 + v) - J(u^0), and the one-step VJP
  against the one-step map, both to rounding (1e-9 relative);
* checkpoint-interval invariance (1e-12 relative).
"""
import numpy as np
import pytest

from geothermalwells_gb300 import GB300, create_cache, rock2
from geothermalwells_gb300 import adjoint as A
from geothermalwells_gb300 import workloads as W
from geothermalwells_gb300 import _lib
import fd_oracle as FD

pytestmark = pytest.mark.gpu

FD_RTOL = 1e-4
EXACT_RTOL = 1e-9

CASES = {
    "const_layers": (dict(n_layers=3), dict(w_energy=1.0, w_outlet=0.0)),
    "hx_two_wells": (dict(n_layers=2, inlet="hx", nbh=2), dict(w_energy=0.0, w_outlet=1.0)),
    "many_stages": (dict(n_layers=2, backfill_quirk=True), dict(w_energy=1.0, w_outlet=2.0)),
}


def fp64_cache(w):
    return create_cache(backend=GB300(precision="fp64"), gridx=w["gridx"], gridy=w["gridy"],
                        gridz=w["gridz"], materials=w["materials"], boreholes=w["boreholes"],
                        inlet_model=w["inlet_model"])


@pytest.mark.parametrize("name", list(CASES))
def test_adjoint_matches_oracle_fd(name, gwlib):
    kw, obj = CASES[name]
    w = W.adjoint_small(**kw)
    cache = fp64_cache(w)
    r = A.adjoint(cache, w["T0"], w["dt"], w["nsteps"], checkpoint_every=5, **obj)
    p = FD.params(w)
    J = FD.objective(w, p, w["nsteps"], **obj)
    assert abs(r.objective - J) <= 1e-10 * abs(J)
    g_fd = FD.central_fd(w, w["nsteps"], rel=1e-4, **obj)
    g = r.grad
    err = np.abs(g - g_fd)
    assert np.all(err <= FD_RTOL * np.abs(g_fd) + 1e-12 * np.max(np.abs(g_fd))), (g, g_fd, err / np.abs(g_fd))


def test_stage_count_of_many_stages_case(gwlib):
    w = W.adjoint_small(**CASES["many_stages"][0])
    cache = fp64_cache(w)
    r = A.adjoint(cache, w["T0"], w["dt"], 2)
    assert r.stages > 8


@pytest.mark.parametrize("name", list(CASES))
def test_checkpoint_interval_invariance(name, gwlib):
    kw, obj = CASES[name]
    w = W.adjoint_small(**kw)
    cache = fp64_cache(w)
    ref = A.adjoint(cache, w["T0"], w["dt"], w["nsteps"], checkpoint_every=w["nsteps"], **obj)
    for K in (1, 4, 7):
        r = A.adjoint(cache, w["T0"], w["dt"], w["nsteps"], checkpoint_every=K, **obj)
        assert r.checkpoints == -(-w["nsteps"] // K)
        assert r.objective == ref.objective
        assert np.max(np.abs(r.grad - ref.grad)) <= 1e-12 * np.max(np.abs(ref.grad))


@pytest.mark.parametrize("name", list(CASES))
def test_initial_field_gradient_is_exact(name, gwlib, torch_cuda):
    """J is affine in u^0: <dJ/du^0, v> = J(u^0 + v) - J(u^0) up to rounding."""
    kw, obj = CASES[name]
    w = W.adjoint_small(**kw)
    cache = fp64_cache(w)
    n = 6
    r = A.adjoint(cache, w["T0"], w["dt"], n, checkpoint_every=4, want_T0=True, **obj)
    v = np.asfortranarray(np.random.default_rng(3).uniform(-1.0, 1.0, w["T0"].shape))
    r2 = A.adjoint(cache, w["T0"] + v, w["dt"], n, checkpoint_every=4, **obj)
    lhs = float(np.sum(r.dT0 * v))
    rhs = r2.objective - r.objective
    assert abs(lhs - rhs) <= EXACT_RTOL * abs(r.objective)
    assert abs(lhs - rhs) <= 1e-6 * abs(rhs)


@pytest.mark.parametrize("name", list(CASES))
def test_step_vjp_against_step_map(name, gwlib, torch_cuda):
    """(du^{n+1}/du^n)^T lam + dJ_n/du^n against the fused step: for random u,
    v, lam, <vjp, v> = Phi(u + v) - Phi(u) with Phi(u) = <lam, F(u)> + J_n(u)."""
    torch = torch_cuda
    kw, obj = CASES[name]
    w = W.adjoint_small(**kw)
    cache = fp64_cache(w)
    rng = np.random.default_rng(11)
    u = np.asfortranarray(w["T0"] + rng.uniform(-2.0, 2.0, w["T0"].shape))
    v = np.asfortranarray(rng.uniform(-1.0, 1.0, w["T0"].shape))
    lam = np.asfortranarray(rng.uniform(-1.0, 1.0, w["T0"].shape))
    L = _lib.load()

    def phi(field):
        cache.set_field(field)
        _lib.check(L.gw_reset_energy(cache.ctx))
        _lib.check(L.gw_step(cache.ctx, 0.0, w["dt"], 1, 100))
        E = np.zeros(cache.N_bh)
        _lib.check(L.gw_get_energy(cache.ctx, _lib.dptr(E)))
        return float(np.sum(lam * cache.get_field()) + obj["w_energy"] * E.sum()
                     + obj["w_outlet"] * cache.T_outlet.sum())

    d_u = torch.from_numpy(u.ravel(order="F").copy()).cuda()
    d_l = torch.from_numpy(lam.ravel(order="F").copy()).cuda()
    A.step_vjp(cache, d_u, d_l, w["dt"], **obj)
    vjp = d_l.cpu().numpy().reshape(u.shape, order="F")
    lhs = float(np.sum(vjp * v))
    rhs = phi(u + v) - phi(u)
    assert abs(lhs - rhs) <= EXACT_RTOL * max(abs(phi(u)), 1.0)


def test_step_vjp_parameters_against_gpu_fd(gwlib, torch_cuda):
    """Parameter part of one step's VJP against central differences of the
    fused FP64 step (new caches per perturbed parameter)."""
    torch = torch_cuda
    w = W.adjoint_small(n_layers=3)
    rng = np.random.default_rng(5)
    u = np.asfortranarray(w["T0"] + rng.uniform(-2.0, 2.0, w["T0"].shape))
    lam = np.asfortranarray(rng.uniform(-1.0, 1.0, w["T0"].shape))
    L = _lib.load()

    def phi(p):
        c = fp64_cache(FD.with_params(w, p))
        try:
            c.set_field(u)
            _lib.check(L.gw_reset_energy(c.ctx))
            _lib.check(L.gw_step(c.ctx, 0.0, w["dt"], 1, 100))
            E = np.zeros(c.N_bh)
            _lib.check(L.gw_get_energy(c.ctx, _lib.dptr(E)))
            return float(np.sum(lam * c.get_field()) + E.sum())
        finally:
            c.close()

    cache = fp64_cache(w)
    d_u = torch.from_numpy(u.ravel(order="F").copy()).cuda()
    d_l = torch.from_numpy(lam.ravel(order="F").copy()).cuda()
    g = A.step_vjp(cache, d_u, d_l, w["dt"], w_energy=1.0, w_outlet=0.0)
    p0 = FD.params(w)
    for i in range(len(p0)):
        hs = 1e-4 * abs(p0[i])
        pp, pm = p0.copy(), p0.copy()
        pp[i] += hs
        pm[i] -= hs
        fd = (phi(pp) - phi(pm)) / (pp[i] - pm[i])
        assert abs(g[i] - fd) <= 1e-5 * abs(fd) + 1e-9 * np.max(np.abs(g)), (i, g[i], fd)


def test_autograd_function(gwlib, torch_cuda):
    """extracted_heat as a torch.autograd.Function: backward gives the
    adjoint gradient."""
    torch = torch_cuda
    w = W.adjoint_small(n_layers=3, nsteps=4)
    d = A.Design(w["gridx"], w["gridy"], w["gridz"], w["boreholes"], w["materials"], w["inlet_model"],
                 w["T0"], w["dt"], w["nsteps"], checkpoint_every=2)
    p = FD.params(w)
    k = torch.tensor(p[:3], dtype=torch.float64, requires_grad=True)
    m = torch.tensor(p[3:4], dtype=torch.float64, requires_grad=True)
    t = torch.tensor(p[4], dtype=torch.float64, requires_grad=True)
    J = A.extracted_heat(d, k, m, t)
    J.backward()
    r = d.run(p[:3], p[3:4], p[4])
    # two separate solves: the gradient sums use atomics, so equal to rounding
    assert abs(J.item() - r.objective) <= 1e-12 * abs(r.objective)
    assert np.allclose(k.grad.numpy(), r.dk_layers, rtol=1e-12, atol=0)
    assert np.allclose(m.grad.numpy(), r.dmdot, rtol=1e-12, atol=0)
    assert abs(float(t.grad) - r.dinlet) <= 1e-12 * abs(r.dinlet)


def mixed_cache(w):
    return create_cache(backend=GB300(precision="mixed"), gridx=w["gridx"], gridy=w["gridy"],
                        gridz=w["gridz"], materials=w["materials"], boreholes=w["boreholes"],
                        inlet_model=w["inlet_model"])


MIXED_RTOL = 1e-3   # float adjoint fields over the mixed step, against the double adjoint


@pytest.mark.parametrize("name", list(CASES))
def test_mixed_adjoint_against_fp64_adjoint(name, gwlib):
    """The mixed path's adjoint (float fields, double sums) against the FP64
    GPU adjoint and the oracle's central differences."""
    kw, obj = CASES[name]
    w = W.adjoint_small(**kw)
    r64 = A.adjoint(fp64_cache(w), w["T0"], w["dt"], w["nsteps"], checkpoint_every=5, **obj)
    r32 = A.adjoint(mixed_cache(w), w["T0"], w["dt"], w["nsteps"], checkpoint_every=5, **obj)
    scale = np.max(np.abs(r64.grad))
    err = np.abs(r32.grad - r64.grad)
    assert np.all(err <= MIXED_RTOL * np.abs(r64.grad) + 1e-6 * scale), (r32.grad, r64.grad, err / np.abs(r64.grad))
    assert abs(r32.objective - r64.objective) <= 1e-5 * abs(r64.objective)


def test_mixed_initial_field_gradient(gwlib, torch_cuda):
    """dJ/du^0 of the mixed adjoint against the FP64 one."""
    w = W.adjoint_small(n_layers=3)
    r64 = A.adjoint(fp64_cache(w), w["T0"], w["dt"], 6, checkpoint_every=4, want_T0=True)
    r32 = A.adjoint(mixed_cache(w), w["T0"], w["dt"], 6, checkpoint_every=4, want_T0=True)
    assert np.max(np.abs(r32.dT0 - r64.dT0)) <= 1e-3 * np.max(np.abs(r64.dT0))


def test_step_vjp_needs_fp64_context(gwlib, torch_cuda):
    torch = torch_cuda
    w = W.adjoint_small()
    cache = mixed_cache(w)
    d = torch.zeros(cache.N, dtype=torch.float64, device="cuda")
    with pytest.raises(_lib.GWError) as e:
        A.step_vjp(cache, d, d.clone(), w["dt"])
    assert e.value.code == _lib.GW_ERR_UNSUPPORTED
