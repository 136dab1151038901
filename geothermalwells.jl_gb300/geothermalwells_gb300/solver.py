"""Time-step entry points, mirroring ``src/solver.jl`` and the integrator
calls of ``examples/single_borehole_basic.jl:116-139``.

Fine-grained calls (``rhs_diffusion_z`` etc.) take device fields: CUDA
``torch.Tensor``s of float64 with ``Nx*Ny*Nz`` contiguous elements in the
reference's order (z fastest), or raw device addresses as ``int``.  They are
for driving the hot path from an external integrator.

:func:`solve` is the fused path: it keeps the state on the device and runs
ROCK2 + ADI + advection steps as one captured CUDA graph per step.
"""
import ctypes
import math

import numpy as np

from . import _lib
from .cache import Cache, SimulationCallback


def _devptr(x, cache):
    if isinstance(x, int):
        return x
    if hasattr(x, "data_ptr") and hasattr(x, "is_cuda"):
        import torch
        if not x.is_cuda or x.dtype != torch.float64 or not x.is_contiguous():
            raise ValueError("device fields must be contiguous CUDA float64 tensors")
        if x.numel() != cache.N:
            raise ValueError("field has %d values, grid has %d" % (x.numel(), cache.N))
        torch.cuda.current_stream(x.device).synchronize()
        return x.data_ptr()
    raise TypeError("expected a CUDA tensor or a device address, got %r" % type(x))


def rhs_diffusion_z(dphi, phi, cache, t):
    """``rhs_diffusion_z!(dphi, phi, cache, t)``, ``src/solver.jl:23-31``:
    dphi = A_z phi (vertical diffusion, Neumann ends)."""
    _lib.check(_lib.load().gw_rhs_diffusion_z(cache.ctx, _devptr(dphi, cache), _devptr(phi, cache)))


def diffusion_1d(dphi, phi, cache, dt, direction, plus_I):
    """``diffusion_1D!``, ``src/solver.jl:34-58``."""
    _lib.check(_lib.load().gw_diffusion_1d(cache.ctx, _devptr(dphi, cache), _devptr(phi, cache),
                                           float(dt), _lib.DIRS[direction], int(bool(plus_I))))


def thomas_I_minus_A(U, RHS, cache, dt, direction):
    """``thomas_I_minus_A!``, ``src/solver.jl:111-232``: (I - dt A_dir) U = RHS."""
    if direction not in ("x", "y"):
        raise ValueError("Invalid direction chosen")
    _lib.check(_lib.load().gw_thomas(cache.ctx, _devptr(U, cache), _devptr(RHS, cache), float(dt),
                                     _lib.DIRS[direction]))


def advection(phi, dt, t, cache):
    """``advection!``, ``src/solver.jl:250-264`` (updates phi and T_outlet)."""
    _lib.check(_lib.load().gw_advection(cache.ctx, _devptr(phi, cache), float(dt), float(t)))


def lincomb(dst, coeffs, srcs, cache):
    """dst = sum_i coeffs[i] * srcs[i] on device fields (up to 8; dst may be
    one of the sources): the vector updates of an integrator's stages."""
    import ctypes
    n = len(srcs)
    if n != len(coeffs):
        raise ValueError("one coefficient per source field")
    w = np.ascontiguousarray(coeffs, dtype=np.float64)
    ptrs = (ctypes.c_void_p * max(n, 1))(*[_devptr(x, cache) for x in srcs])
    _lib.check(_lib.load().gw_lincomb(cache.ctx, _devptr(dst, cache), n, _lib.dptr(w), ptrs))


def ADI_and_ADV_callback(u, temp, t, dt, cache):
    """``ADI_and_ADV_callback!``, ``src/solver.jl:432-464``, with the
    integrator's ``u``, ``uprev`` (as scratch), ``t`` and ``t - tprev``."""
    _lib.check(_lib.load().gw_adi_adv(cache.ctx, _devptr(u, cache), _devptr(temp, cache), float(t),
                                      float(dt)))


def eigen_estimator(integrator):
    """``src/solver.jl:495``: the constant 8 d_max / dz_min^2 estimate."""
    integrator.eigen_est = integrator.p.eigen_estimate
    return integrator.eigen_est


class ROCK2:
    """Second-order stabilised Runge-Kutta-Chebyshev method for the z part.
    The stage count is the smallest s >= 3 whose stability interval covers
    dt * eigen_est, capped at ``max_stages``."""

    def __init__(self, max_stages=100, eigen_est=None):
        self.max_stages = int(max_stages)
        self.eigen_est = eigen_est


class ODEProblem:
    """``ODEProblem(rhs_diffusion_z!, T0, tspan, cache)``."""

    def __init__(self, f, u0, tspan, p):
        self.f, self.u0, self.tspan, self.p = f, u0, (float(tspan[0]), float(tspan[1])), p


class Solution:
    def __init__(self, t, u, outlet_t, outlet, energy, stages, stages_covered):
        self.t = t
        self.u = u
        self.outlet_t = outlet_t       # time after each step
        self.T_outlet = outlet         # (nsteps, N_bh) outlet temperature after each step
        self.energy = energy           # extracted heat per borehole [J]
        self.stages = stages
        self.stages_covered = stages_covered


class _Integrator:
    def __init__(self, p):
        self.p = p
        self.eigen_est = None


def _steps_for(t, t0, dt, what):
    n = (t - t0) / dt
    r = round(n)
    if abs(n - r) > 1e-9 * max(1.0, abs(n)):
        raise ValueError("%s time %r is not on the fixed-step grid (t0=%r, dt=%r)" % (what, t, t0, dt))
    return int(r)


def solve(prob, alg, *, dt, adaptive=False, save_everystep=False, callback=None, maxiters=None):
    """Fixed-step integration on the device (``adaptive=false``, as every
    reference example uses).  Each step: ROCK2 on u' = A_z u, then the
    ADI/advection split of ``ADI_and_ADV_callback!``; saving and printing as
    the callback set of ``get_simulation_callback`` asks."""
    cache = prob.p
    if not isinstance(cache, Cache):
        raise TypeError("prob.p must be a cache from create_cache(backend=GB300(), ...)")
    if adaptive:
        raise ValueError("only fixed steps (adaptive=false) are supported, as in the reference")
    if not isinstance(alg, ROCK2):
        raise TypeError("alg must be ROCK2(...)")
    if prob.f is not rhs_diffusion_z:
        raise ValueError("the fused path integrates rhs_diffusion_z")
    if callback is not None and not isinstance(callback, SimulationCallback):
        raise TypeError("callback must come from get_simulation_callback")
    L = _lib.load()
    integ = _Integrator(cache)
    if alg.eigen_est is not None:
        alg.eigen_est(integ)
    dt = float(dt)
    t0, t1 = prob.tspan
    nsteps = _steps_for(t1, t0, dt, "final")
    if maxiters is not None and nsteps > maxiters:
        raise ValueError("nsteps %d exceeds maxiters" % nsteps)
    s = ctypes_int()
    cov = ctypes_int()
    _lib.check(L.gw_rock2_stages(cache.ctx, dt, alg.max_stages, s.ref(), cov.ref()))
    cache.set_field(prob.u0)
    _lib.check(L.gw_reset_energy(cache.ctx))
    stops = {nsteps}
    save_steps = {}
    if callback is not None:
        for ts in callback.saveat:
            if t0 <= ts <= t1:
                save_steps.setdefault(_steps_for(ts, t0, dt, "saveat"), ts)
        stops |= set(save_steps)
        if callback.print_every_n > 0:
            stops |= set(range(callback.print_every_n, nsteps + 1, callback.print_every_n))
    # saved fields: float snapshots converted on the device and copied to
    # pinned host buffers on a second stream while the next steps run; they
    # are handed to the callback once every copy has landed
    snaps = []

    def snapshot(ts):
        ptr = ctypes.c_void_p()
        _lib.check(L.gw_snapshot_host_alloc(cache.ctx, ctypes.byref(ptr)))
        snaps.append((ts, ptr))
        _lib.check(L.gw_snapshot(cache.ctx, ptr))

    if 0 in save_steps:
        snapshot(save_steps[0])
    series = []
    done = 0
    for stop in sorted(x for x in stops if x > 0):
        n = stop - done
        _lib.check(L.gw_step(cache.ctx, t0 + done * dt, dt, n, alg.max_stages))
        buf = np.zeros(n * cache.N_bh)
        _lib.check(L.gw_get_outlet_series(cache.ctx, _lib.dptr(buf), n))
        series.append(buf.reshape(n, cache.N_bh))
        done = stop
        t = t0 + done * dt
        if callback is not None:
            if callback.print_every_n > 0 and done % callback.print_every_n == 0:
                callback.print_step(done, t)
            if done in save_steps:
                snapshot(save_steps[done])
    if snaps:
        _lib.check(L.gw_snapshot_wait(cache.ctx))
        for ts, ptr in snaps:
            host = np.ctypeslib.as_array(ctypes.cast(ptr, ctypes.POINTER(ctypes.c_float)), shape=(cache.N,))
            callback.save(ts, host.reshape(cache.shape, order="F").copy(order="F"))
            _lib.check(L.gw_snapshot_host_free(cache.ctx, ptr))
    energy = np.zeros(cache.N_bh)
    _lib.check(L.gw_get_energy(cache.ctx, _lib.dptr(energy)))
    outlet = np.concatenate(series) if series else np.zeros((0, cache.N_bh))
    u_end = cache.get_field()
    return Solution([t0, t1], [np.asarray(prob.u0), u_end],
                    t0 + dt * np.arange(1, nsteps + 1), outlet, energy, s.value, bool(cov.value))


class ctypes_int:
    def __init__(self):
        import ctypes
        self._v = ctypes.c_int(0)

    def ref(self):
        import ctypes
        return ctypes.byref(self._v)

    @property
    def value(self):
        return self._v.value
