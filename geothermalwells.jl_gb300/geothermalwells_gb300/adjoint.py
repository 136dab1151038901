"""Gradients of the solve: ``gw_adjoint`` / ``gw_step_vjp`` of the C ABI.

The reference has no derivatives.  This module gives the objective

    J = sum_b [ w_energy * E_b + w_outlet * T_out,b(last step) ],
    E_b = sum_n mdot_b * c_w * (T_out,b^n - T_in,b^n) * dt,

and dJ/dp for p = (rock layer conductivities, flow rate per borehole, inlet
parameter), computed by the library's adjoint kernels with checkpointing.
:class:`ExtractedHeat` wraps it as a ``torch.autograd.Function``, the Python
counterpart of a ChainRulesCore ``rrule`` over the solve.
"""
import ctypes
from dataclasses import dataclass

import numpy as np

from . import _lib
from .cache import GB300, create_cache
from .physics import (ConstantInlet, HeatExchangerInlet, StratifiedMaterialProperties)


@dataclass
class AdjointResult:
    objective: float
    dk_layers: np.ndarray      # dJ / d k_rock_layers
    dmdot: np.ndarray          # dJ / d mdot per borehole
    dinlet: float              # dJ / d T_const (constant inlet) or dT (heat-exchanger inlet)
    dT0: object                # dJ / d u^0 as an (Nz, Ny, Nx) array, or None
    stages: int
    checkpoints: int
    forward_ms: float
    reverse_ms: float
    peak_bytes: int

    @property
    def grad(self):
        return np.concatenate([self.dk_layers, self.dmdot, [self.dinlet]])


def _split(cache, g):
    nl = len(cache.materials.k_rock_layers)
    return g[:nl].copy(), g[nl:nl + cache.N_bh].copy(), float(g[nl + cache.N_bh])


def adjoint(cache, T0, dt, nsteps, *, max_stages=100, checkpoint_every=64, w_energy=1.0,
            w_outlet=0.0, want_T0=False):
    """J and its gradient over ``nsteps`` steps of size ``dt`` from the field
    ``T0`` (host array, (Nz, Ny, Nx)).  FP64 caches run the adjoint in double,
    mixed caches with float adjoint fields over the mixed step.  The cache is
    left at the final state, as after the forward solve."""
    L = _lib.load()
    cache.set_field(T0)
    npar = len(cache.materials.k_rock_layers) + cache.N_bh + 1
    g = np.zeros(npar)
    info = _lib.AdjointInfo()
    dT0 = None
    buf = None
    if want_T0:
        import torch   # device buffer for dJ/du^0 (plumbing only)
        buf = torch.zeros(cache.N, dtype=torch.float64, device="cuda:%d" % cache.backend.device)
    _lib.check(L.gw_adjoint(cache.ctx, float(dt), int(nsteps), int(max_stages), int(checkpoint_every),
                            float(w_energy), float(w_outlet), _lib.dptr(g),
                            ctypes.c_void_p(buf.data_ptr()) if buf is not None else None,
                            ctypes.byref(info)))
    if buf is not None:
        dT0 = buf.cpu().numpy().reshape(cache.shape, order="F")
    dk, dm, di = _split(cache, g)
    return AdjointResult(info.objective, dk, dm, di, dT0, info.stages, info.checkpoints,
                         info.forward_ms, info.reverse_ms, info.peak_bytes)


def step_vjp(cache, u_dev, lam_dev, dt, *, max_stages=100, w_energy=1.0, w_outlet=0.0):
    """One step's vector-Jacobian product on device buffers (torch tensors
    or integer device addresses): lam <- (du^{n+1}/du^n)^T lam + d J_n/du^n;
    returns d(<lam, u^{n+1}> + J_n)/dp as a host vector."""
    L = _lib.load()
    npar = len(cache.materials.k_rock_layers) + cache.N_bh + 1
    g = np.zeros(npar)
    up = u_dev.data_ptr() if hasattr(u_dev, "data_ptr") else int(u_dev)
    lp = lam_dev.data_ptr() if hasattr(lam_dev, "data_ptr") else int(lam_dev)
    _lib.check(L.gw_step_vjp(cache.ctx, ctypes.c_void_p(up), ctypes.c_void_p(lp), float(dt),
                             int(max_stages), float(w_energy), float(w_outlet), _lib.dptr(g)))
    return g


class Design:
    """A well design whose rock layer conductivities, flow rates and inlet
    parameter are the inputs of a differentiable solve: grids, borehole and
    material templates, inlet kind, initial field and step schedule."""

    def __init__(self, gridx, gridy, gridz, boreholes, materials, inlet_model, T0, dt, nsteps,
                 device=0, checkpoint_every=64, w_energy=1.0, w_outlet=0.0, max_stages=100,
                 precision="fp64"):
        self.gridx, self.gridy, self.gridz = gridx, gridy, gridz
        self.boreholes = tuple(boreholes)
        self.materials = materials
        self.inlet_model = inlet_model
        self.T0 = T0
        self.dt, self.nsteps = float(dt), int(nsteps)
        self.device = int(device)
        self.checkpoint_every = int(checkpoint_every)
        self.w_energy, self.w_outlet = float(w_energy), float(w_outlet)
        self.max_stages = int(max_stages)
        self.precision = precision

    def cache(self, k_layers, mdot, inlet_param):
        m = self.materials
        mat = StratifiedMaterialProperties(tuple(float(v) for v in k_layers), m.rho_c_rock_layers,
                                           m.layer_depths, *m.fixed())
        bhs = tuple(b.with_flow(float(q)) for b, q in zip(self.boreholes, mdot))
        inlet = (ConstantInlet(float(inlet_param)) if self.inlet_model.kind == 0
                 else HeatExchangerInlet(float(inlet_param)))
        return create_cache(backend=GB300(device=self.device, precision=self.precision), gridx=self.gridx,
                            gridy=self.gridy, gridz=self.gridz, materials=mat, boreholes=bhs,
                            inlet_model=inlet)

    def run(self, k_layers, mdot, inlet_param):
        c = self.cache(k_layers, mdot, inlet_param)
        try:
            return adjoint(c, self.T0, self.dt, self.nsteps, max_stages=self.max_stages,
                           checkpoint_every=self.checkpoint_every, w_energy=self.w_energy,
                           w_outlet=self.w_outlet)
        finally:
            c.close()


def _make_function():
    import torch

    class ExtractedHeat(torch.autograd.Function):
        """J(k_layers, mdot, inlet_param) for a :class:`Design`; backward
        returns the adjoint gradient (the rrule pullback)."""

        @staticmethod
        def forward(ctx, k_layers, mdot, inlet_param, design):
            r = design.run(k_layers.detach().cpu().double().numpy(),
                           mdot.detach().cpu().double().numpy(),
                           float(inlet_param.detach().cpu()))
            dev = k_layers.device
            ctx.save_for_backward(torch.from_numpy(r.dk_layers).to(dev),
                                  torch.from_numpy(r.dmdot).to(dev),
                                  torch.tensor(r.dinlet, dtype=torch.float64, device=dev))
            return torch.tensor(r.objective, dtype=torch.float64, device=dev)

        @staticmethod
        def backward(ctx, gJ):
            dk, dm, di = ctx.saved_tensors
            return gJ * dk, gJ * dm, gJ * di, None

    return ExtractedHeat


_fn = None


def extracted_heat(design, k_layers, mdot, inlet_param):
    """Differentiable J (a 0-d float64 tensor) of the design's solve."""
    global _fn
    if _fn is None:
        _fn = _make_function()
    return _fn.apply(k_layers, mdot, inlet_param, design)
