"""``create_cache`` and the simulation callbacks, mirroring ``src/cache.jl``.

``create_cache(; backend=GB300(), ...)`` builds a device context through the
C ABI (``gw_create``): the material model, the advection index lists
(``src/cache.jl:9-44``), the state and scratch buffers.  The returned
:class:`Cache` carries the same fields the reference's NamedTuple does
(``src/cache.jl:83-113``) plus the context handle.
"""
import ctypes
import os

import numpy as np

from . import _lib
from .physics import CustomInlet


class GB300:
    """Backend value selecting the GB300 library (the reference's
    ``backend = CPU()`` / ``CUDABackend()`` plug point).

    ``precision``: ``"fp64"`` (plain double) or ``"mixed"`` (float storage and
    Thomas sweeps, double ROCK2 accumulation and energy balance) for the
    fused :func:`solve` path.  The fine-grained entry points are always
    double."""

    def __init__(self, device=0, precision="fp64"):
        if precision not in ("fp64", "mixed"):
            raise ValueError("precision must be 'fp64' or 'mixed'")
        self.device = int(device)
        self.precision = precision

    def __repr__(self):
        return "GB300(device=%d, precision=%r)" % (self.device, self.precision)


class Cache:
    """The ODE parameter ``p``: grids, materials, boreholes, inlet and the
    device context.  ``T_outlet`` reads the device's current outlet values."""

    def __init__(self, backend, gridx, gridy, gridz, materials, boreholes, inlet_model):
        if not isinstance(backend, GB300):
            raise TypeError("this package provides the GB300 backend only; got %r" % (backend,))
        if isinstance(inlet_model, CustomInlet) or getattr(inlet_model, "kind", -1) not in (0, 1, 2, 3):
            raise ValueError("CustomInlet closures cannot cross the C ABI: use ConstantInlet, "
                             "HeatExchangerInlet, ScheduleInlet or ExpressionInlet")
        L = _lib.load()
        self.backend = backend
        self.gridx = np.ascontiguousarray(gridx, dtype=np.float64)
        self.gridy = np.ascontiguousarray(gridy, dtype=np.float64)
        self.gridz = np.ascontiguousarray(gridz, dtype=np.float64)
        self.Nx, self.Ny, self.Nz = len(self.gridx), len(self.gridy), len(self.gridz)
        self.boreholes = tuple(boreholes)
        self.N_bh = len(self.boreholes)
        self.materials = materials
        self.inlet_model = inlet_model
        kl, rl, dl = (np.ascontiguousarray(v, dtype=np.float64) for v in materials.layers())
        bh = (_lib.BoreholeDesc * self.N_bh)(*[_lib.BoreholeDesc(*b.args()) for b in self.boreholes])
        md = _lib.MaterialDesc(len(kl), _lib.dptr(kl), _lib.dptr(rl), _lib.dptr(dl), *materials.fixed())
        prec = _lib.GW_PREC_MIXED if backend.precision == "mixed" else _lib.GW_PREC_FP64
        desc = _lib.Desc(self.Nx, self.Ny, self.Nz, _lib.dptr(self.gridx), _lib.dptr(self.gridy),
                         _lib.dptr(self.gridz), self.N_bh, bh, md, inlet_model.kind,
                         inlet_model.param, prec, backend.device)
        h = ctypes.c_void_p()
        _lib.check(L.gw_create(ctypes.byref(desc), ctypes.byref(h)))
        self.ctx = h
        sched = inlet_model if inlet_model.kind == 2 else getattr(inlet_model, "schedule", None)
        if sched is not None:
            st = np.ascontiguousarray(sched.times, dtype=np.float64)
            sv = np.ascontiguousarray(sched.values, dtype=np.float64)
            _lib.check(L.gw_set_inlet_schedule(self.ctx, len(st), _lib.dptr(st), _lib.dptr(sv)))
        if inlet_model.kind == 3:
            ops = np.ascontiguousarray(inlet_model.ops, dtype=np.int32)
            args = np.ascontiguousarray(inlet_model.args, dtype=np.float64)
            _lib.check(L.gw_set_inlet_program(self.ctx, len(ops), ops.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                              _lib.dptr(args)))
        info = _lib.Info()
        _lib.check(L.gw_get_info(self.ctx, ctypes.byref(info)))
        self.countxy_inner = info.countxy_inner
        self.countxy_outer = info.countxy_outer
        self.countz = info.countz
        self.eigen_estimate = info.eigen_estimate
        self.n_zclass = info.n_zclass
        self.n_profiles = info.n_profiles
        self.device_bytes = info.device_bytes

    @property
    def shape(self):
        return (self.Nz, self.Ny, self.Nx)

    @property
    def N(self):
        return self.Nx * self.Ny * self.Nz

    @property
    def T_outlet(self):
        out = np.zeros(self.N_bh)
        _lib.check(_lib.load().gw_get_outlet(self.ctx, _lib.dptr(out)))
        return out

    def set_field(self, T):
        T = np.asarray(T, dtype=np.float64)
        if T.size != self.N:
            raise ValueError("field has %d values, grid has %d" % (T.size, self.N))
        buf = np.ascontiguousarray(T.reshape(self.shape, order="F").ravel(order="F"))
        _lib.check(_lib.load().gw_set_field(self.ctx, _lib.dptr(buf)))

    def init_thermal_gradient(self, T_surface, gradient):
        """u = T_surface + gradient * z filled on the device
        (``initial_condition_thermal_gradient``, ``src/physics.jl:333-348``,
        without an N-cell host array)."""
        _lib.check(_lib.load().gw_init_thermal_gradient(self.ctx, float(T_surface), float(gradient)))

    def get_field(self, dtype=np.float64):
        buf = np.zeros(self.N)
        _lib.check(_lib.load().gw_get_field(self.ctx, _lib.dptr(buf)))
        return buf.reshape(self.shape, order="F").astype(dtype, copy=False)

    def close(self):
        if getattr(self, "ctx", None):
            _lib.load().gw_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def create_cache(*, backend, gridx, gridy, gridz, materials, boreholes, inlet_model):
    """``src/cache.jl:55-116``."""
    return Cache(backend, gridx, gridy, gridz, materials, boreholes, inlet_model)


class SavedValues:
    """``DiffEqCallbacks.SavedValues``: ``t`` and ``saveval`` lists."""

    def __init__(self, dtype=np.float32):
        self.t = []
        self.saveval = []
        self.dtype = dtype


class SimulationCallback:
    """The reference's ``CallbackSet(ADI_and_ADV, print_cb, save_cb)``
    (``src/cache.jl:224-237``).  The ADI + advection part runs on the device
    inside every step of :func:`geothermalwells_gb300.solve`; this object holds
    the saving and printing schedule."""

    def __init__(self, saveat, print_every_n, write_to_jld, data_folder_dir, saved_values):
        self.saveat = sorted(float(t) for t in np.atleast_1d(np.asarray(saveat, dtype=np.float64)))
        self.print_every_n = int(print_every_n)
        self.write_to_jld = bool(write_to_jld)
        self.data_folder_dir = data_folder_dir
        self.saved_values = saved_values
        self.file_counter = 0

    def save(self, t, field):
        self.saved_values.t.append(float(t))
        arr = np.asarray(field, dtype=self.saved_values.dtype, order="F")
        self.saved_values.saveval.append(arr)
        if self.write_to_jld:
            # src/cache.jl:163-167 writes checkpoint_N.jld2; the host format here is .npy
            self.file_counter += 1
            np.save(os.path.join(self.data_folder_dir, "checkpoint_%d.npy" % self.file_counter),
                    np.asfortranarray(arr))

    def print_step(self, naccept, t):
        """``src/cache.jl:140-149`` print_affect!"""
        if t > 3600 * 24 * 365:
            print("Step %d, t = %s s, or %s years" % (naccept, t, round(t / 31536000, 4)), flush=True)
        elif t > 3600 * 24:
            print("Step %d, t = %s s, or %s days" % (naccept, t, round(t / 86400, 2)), flush=True)
        else:
            print("Step %d, t = %s s, or %s hours" % (naccept, t, round(t / 3600, 2)), flush=True)


def get_simulation_callback(*, saveat, print_every_n=1000, write_to_jld=False, data_folder_dir=""):
    """``src/cache.jl:224-237``: returns ``(callback, saved_values)``."""
    if write_to_jld and not data_folder_dir:
        raise ValueError("When `write_to_jld` is true, `data_folder_dir` must be provided and "
                         "cannot be an empty string")
    if write_to_jld and not os.path.isdir(data_folder_dir):
        os.mkdir(data_folder_dir)
    sv = SavedValues(np.float32)
    return SimulationCallback(saveat, print_every_n, write_to_jld, data_folder_dir, sv), sv
