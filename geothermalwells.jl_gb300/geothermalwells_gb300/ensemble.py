"""Ensembles: many well designs advanced together on one GPU.

Each design gets its own cache (``create_cache``); the batch advances all of
them with one CUDA-graph launch per step in which the designs' fused steps
run concurrently (``gw_batch_*`` in ``include/gw_gb300.h``).  An autotuner
picks each design's half-step tiling by timing the candidates.
"""
import ctypes

import numpy as np

from . import _lib
from .cache import GB300, create_cache

# (lines per block, rows per chunk) of the tiled half step (mixed path: the
# forward-elimination values in tensor memory where they fit); entry 6 is the
# segmented half step (2 lines per block, 8 segments of up to 32 rows); 7-12
# are the row tiles of 0-5 with the forward values in global memory
_ROWS = ((4, 16), (8, 16), (8, 8), (4, 32), (2, 16), (8, 32))
TILINGS = _ROWS + ((2, "seg8x32"),) + tuple((hw, hr, "global") for hw, hr in _ROWS)


class Ensemble:
    def __init__(self, designs, precision="mixed", device=0, initial_field=None,
                 initial_gradient=None):
        """designs: dicts with gridx, gridy, gridz, boreholes, materials,
        inlet_model.  The initial field is, in this order of preference:
        initial_gradient(design) -> (T_surface, gradient), filled on the
        device; initial_field(design) -> (Nz, Ny, Nx) host array; the
        design's "T0"."""
        L = _lib.load()
        self.caches = []
        for d in designs:
            c = create_cache(backend=GB300(device=device, precision=precision), gridx=d["gridx"],
                             gridy=d["gridy"], gridz=d["gridz"], materials=d["materials"],
                             boreholes=d["boreholes"], inlet_model=d["inlet_model"])
            self.caches.append(c)
            if initial_gradient is not None:
                c.init_thermal_gradient(*initial_gradient(d))
            else:
                c.set_field(initial_field(d) if initial_field else d["T0"])
        arr = (ctypes.c_void_p * len(self.caches))(*[c.ctx for c in self.caches])
        h = ctypes.c_void_p()
        _lib.check(L.gw_batch_create(arr, len(self.caches), ctypes.byref(h)))
        self.batch = h
        self.cells = sum(c.N for c in self.caches)

    def set_tiling(self, t):
        _lib.check(_lib.load().gw_batch_set_tiling(self.batch, int(t)))

    def autotune(self, dt, reps=3):
        out = (ctypes.c_int * len(self.caches))()
        _lib.check(_lib.load().gw_batch_autotune(self.batch, float(dt), int(reps), out))
        return list(out)

    def step(self, dt, nsteps, max_stages=100):
        """Advance every design by nsteps steps of dt; returns device ms."""
        L = _lib.load()
        _lib.check(L.gw_batch_step(self.batch, float(dt), int(nsteps), int(max_stages)))
        ms = ctypes.c_double()
        _lib.check(L.gw_batch_get_last_step_time(self.batch, ctypes.byref(ms)))
        return ms.value

    def outlet_series(self, d, nsteps):
        c = self.caches[d]
        buf = np.zeros(nsteps * c.N_bh)
        _lib.check(_lib.load().gw_get_outlet_series(c.ctx, _lib.dptr(buf), nsteps))
        return buf.reshape(nsteps, c.N_bh)

    def close(self):
        if getattr(self, "batch", None):
            _lib.load().gw_batch_destroy(self.batch)
            self.batch = None
        for c in self.caches:
            c.close()
        self.caches = []

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
