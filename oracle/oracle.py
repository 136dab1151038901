"""ctypes front end of the CPU FP64 oracle (``oracle/gw_oracle.c``).

TEST INFRASTRUCTURE ONLY.  Imported by ``tests/``, ``__graft_entry__.smoke()``
and the CPU-baseline leg of ``bench.py`` as the checker; the product never
imports it.  ``simulate`` restates the reference's driver loop
(``examples/single_borehole_basic.jl:116-139`` + ``src/cache.jl:224-237``):
one ROCK2 step of ``rhs_diffusion_z!`` followed by ``ADI_and_ADV_callback!``
per time step, with f evaluated fresh at each step start.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "build", "libgw_oracle.so")

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_lib = None


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(os.path.join(HERE, "gw_oracle.c")):
            build()
        L = ctypes.CDLL(LIB)
        L.ogw_create.restype = ctypes.c_void_p
        L.ogw_create.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, _dp, _dp, _dp,
                                 ctypes.c_int, _dp, ctypes.c_int, _dp, _dp, _dp, _dp,
                                 ctypes.c_int, ctypes.c_double]
        L.ogw_destroy.argtypes = [ctypes.c_void_p]
        L.ogw_counts.argtypes = [ctypes.c_void_p, _ip]
        L.ogw_index_lists.argtypes = [ctypes.c_void_p, _ip]
        L.ogw_velocities.argtypes = [ctypes.c_void_p, _dp]
        L.ogw_material.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_double,
                                   ctypes.c_double, _dp, _dp]
        L.ogw_eigen_estimate.restype = ctypes.c_double
        L.ogw_eigen_estimate.argtypes = [ctypes.c_void_p]
        L.ogw_diffusion_1d.argtypes = [ctypes.c_void_p, _dp, _dp, ctypes.c_double, ctypes.c_int, ctypes.c_int]
        L.ogw_thomas.argtypes = [ctypes.c_void_p, _dp, _dp, ctypes.c_double, ctypes.c_int]
        L.ogw_advection.argtypes = [ctypes.c_void_p, _dp, ctypes.c_double, ctypes.c_double]
        L.ogw_adi_adv.argtypes = [ctypes.c_void_p, _dp, _dp, ctypes.c_double, ctypes.c_double]
        L.ogw_rock2_step.argtypes = [ctypes.c_void_p, _dp, ctypes.c_double, ctypes.c_int, _dp, _dp, _dp,
                                     ctypes.c_double, ctypes.c_double, _dp]
        L.ogw_get_outlet.argtypes = [ctypes.c_void_p, _dp]
        L.ogw_initial_condition.argtypes = [ctypes.c_void_p, _dp, ctypes.c_double, ctypes.c_double]
        _lp = ctypes.POINTER(ctypes.c_longlong)
        L.ogw_tridiag_batch.argtypes = [ctypes.c_int, _lp, _ip, _dp, _dp, _dp, _dp, _dp]
        L.ogw_set_schedule.argtypes = [ctypes.c_void_p, ctypes.c_int, _dp, _dp]
        L.ogw_set_program.restype = ctypes.c_int
        L.ogw_set_program.argtypes = [ctypes.c_void_p, ctypes.c_int, _ip, _dp]
        L.ogw_set_threads.restype = ctypes.c_int
        L.ogw_set_threads.argtypes = [ctypes.c_int]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(_dp)


def _field_ok(a, shape):
    if not (isinstance(a, np.ndarray) and a.dtype == np.float64 and a.shape == shape
            and a.flags.f_contiguous):
        raise ValueError("oracle fields are Fortran-ordered float64 arrays of shape (Nz, Ny, Nx)")


class Oracle:
    """One reference-equivalent simulation cache on the CPU."""

    def __init__(self, gridx, gridy, gridz, boreholes, materials, inlet_model):
        L = lib()
        self.gx = np.ascontiguousarray(gridx, dtype=np.float64)
        self.gy = np.ascontiguousarray(gridy, dtype=np.float64)
        self.gz = np.ascontiguousarray(gridz, dtype=np.float64)
        self.nx, self.ny, self.nz = len(self.gx), len(self.gy), len(self.gz)
        self.shape = (self.nz, self.ny, self.nx)
        bh = np.array([b.args() for b in boreholes], dtype=np.float64).ravel()
        kl, rl, dl = (np.array(v, dtype=np.float64) for v in materials.layers())
        m8 = np.array(materials.fixed(), dtype=np.float64)
        if inlet_model.kind not in (0, 1, 2, 3):
            raise ValueError("oracle supports ConstantInlet, HeatExchangerInlet, ScheduleInlet and "
                             "ExpressionInlet")
        self.nbh = len(boreholes)
        self._keep = (bh, kl, rl, dl, m8)
        self.h = L.ogw_create(self.nx, self.ny, self.nz, _p(self.gx), _p(self.gy), _p(self.gz),
                              self.nbh, _p(bh), len(kl), _p(kl), _p(rl), _p(dl), _p(m8),
                              inlet_model.kind, inlet_model.param)
        sched = inlet_model if inlet_model.kind == 2 else getattr(inlet_model, "schedule", None)
        if sched is not None:
            st = np.ascontiguousarray(sched.times, dtype=np.float64)
            sv = np.ascontiguousarray(sched.values, dtype=np.float64)
            L.ogw_set_schedule(self.h, len(st), _p(st), _p(sv))
        if inlet_model.kind == 3:
            ops = np.ascontiguousarray(inlet_model.ops, dtype=np.int32)
            args = np.ascontiguousarray(inlet_model.args, dtype=np.float64)
            if L.ogw_set_program(self.h, len(ops), ops.ctypes.data_as(_ip), _p(args)) != 0:
                raise ValueError("malformed inlet program")
        self.temp = np.zeros(self.shape, order="F")
        self._work = None

    def close(self):
        if self.h:
            lib().ogw_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def counts(self):
        out = (ctypes.c_int * 4)()
        lib().ogw_counts(self.h, out)
        return dict(countxy_inner=out[0], countxy_outer=out[1], countz=out[2], nbh=out[3])

    def index_lists(self):
        c = self.counts()
        n = c["countxy_inner"] + c["countxy_outer"]
        out = np.zeros(3 * max(n, 1), dtype=np.int32)
        lib().ogw_index_lists(self.h, out.ctypes.data_as(_ip))
        return out[:3 * n].reshape(n, 3)

    def velocities(self):
        out = np.zeros(2 * self.nbh)
        lib().ogw_velocities(self.h, _p(out))
        return out.reshape(self.nbh, 2)

    def material(self, x, y, z):
        k, r = ctypes.c_double(), ctypes.c_double()
        lib().ogw_material(self.h, x, y, z, ctypes.byref(k), ctypes.byref(r))
        return k.value, r.value

    def eigen_estimate(self):
        return lib().ogw_eigen_estimate(self.h)

    def diffusion_1d(self, dphi, phi, dt, direction, plus_I):
        _field_ok(dphi, self.shape); _field_ok(phi, self.shape)
        lib().ogw_diffusion_1d(self.h, _p(dphi), _p(phi), dt, "xyz".index(direction), int(plus_I))

    def rhs_diffusion_z(self, dphi, phi):
        self.diffusion_1d(dphi, phi, 0.0, "z", False)

    def thomas(self, U, RHS, dt, direction):
        _field_ok(U, self.shape); _field_ok(RHS, self.shape)
        lib().ogw_thomas(self.h, _p(U), _p(RHS), dt, "xy".index(direction))

    def advection(self, phi, dt, t):
        _field_ok(phi, self.shape)
        lib().ogw_advection(self.h, _p(phi), dt, t)

    def adi_adv(self, u, t, dt):
        _field_ok(u, self.shape)
        lib().ogw_adi_adv(self.h, _p(u), _p(self.temp), t, dt)

    def rock2_step(self, u, dt, s, coeffs):
        _field_ok(u, self.shape)
        mu, nu, kappa, sigma, tau = coeffs
        if self._work is None:
            self._work = np.zeros(5 * u.size)
        mu = np.ascontiguousarray(mu, dtype=np.float64) if len(mu) else np.zeros(1)
        nu = np.ascontiguousarray(nu, dtype=np.float64) if len(nu) else np.zeros(1)
        kappa = np.ascontiguousarray(kappa, dtype=np.float64) if len(kappa) else np.zeros(1)
        lib().ogw_rock2_step(self.h, _p(u), dt, s, _p(mu), _p(nu), _p(kappa), sigma, tau,
                             _p(self._work))

    def outlet(self):
        out = np.zeros(self.nbh)
        lib().ogw_get_outlet(self.h, _p(out))
        return out

    def simulate(self, u, t0, dt, nsteps, s, coeffs, record=None):
        """Advance u in place by nsteps fixed steps; returns the outlet
        temperature after every step as an (nsteps, nbh) array."""
        out = np.zeros((nsteps, self.nbh))
        t = t0
        for n in range(nsteps):
            self.rock2_step(u, dt, s, coeffs)
            t_new = t + dt
            self.adi_adv(u, t_new, t_new - t)
            t = t_new
            out[n] = self.outlet()
            if record is not None:
                record(n, t, u)
        return out


def set_threads(n):
    return lib().ogw_set_threads(int(n))


def tridiag_batch(w):
    """Solve a batch from workloads.tridiagonal_batch on the CPU (FP64)."""
    L = lib()
    goff = np.ascontiguousarray(w["group_off"], dtype=np.int64)
    glen = np.ascontiguousarray(w["group_len"], dtype=np.int32)
    x = np.zeros(w["n"])
    arr = [np.ascontiguousarray(w[k], dtype=np.float64) for k in "abcd"]
    L.ogw_tridiag_batch(w["ngroups"], goff.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong)),
                        glen.ctypes.data_as(_ip), *[_p(v) for v in arr], _p(x))
    return x


def tridiag_residual(w, x):
    """max |d - A x| / max |d| in the grouped interleaved layout."""
    a, b, c, d = (w[k] for k in "abcd")
    xm = np.roll(x, 32)
    xp = np.roll(x, -32)
    r = d - (a * xm + b * x + c * xp)
    return float(np.max(np.abs(r)) / np.max(np.abs(d)))
