"""CPU tests of the C ABI boundary: the library loads, exports every symbol
include/gw_gb300.h declares, and rejects bad arguments before touching the
device (no compute call runs here)."""
import ctypes
import os
import re

import numpy as np
import pytest

from geothermalwells_gb300 import _lib
from geothermalwells_gb300 import workloads as W

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include",
                      "gw_gb300.h")


def declared_symbols():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(gw_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_bound_symbols():
    assert set(declared_symbols()) == set(_lib.SIGNATURES)


def test_library_exports_every_declared_symbol(gwlib):
    for name in declared_symbols():
        assert hasattr(gwlib, name), name


def test_version(gwlib):
    assert b"sm_103a" in gwlib.gw_version()


def _desc(w, **over):
    gx, gy, gz = (np.ascontiguousarray(w[k], dtype=np.float64) for k in ("gridx", "gridy", "gridz"))
    kl, rl, dl = (np.ascontiguousarray(v, dtype=np.float64) for v in w["materials"].layers())
    bh = (_lib.BoreholeDesc * len(w["boreholes"]))(*[_lib.BoreholeDesc(*b.args()) for b in w["boreholes"]])
    md = _lib.MaterialDesc(len(kl), _lib.dptr(kl), _lib.dptr(rl), _lib.dptr(dl), *w["materials"].fixed())
    args = dict(nx=len(gx), ny=len(gy), nz=len(gz), gridx=_lib.dptr(gx), gridy=_lib.dptr(gy),
                gridz=_lib.dptr(gz), n_boreholes=len(w["boreholes"]), boreholes=bh, materials=md,
                inlet_kind=w["inlet_model"].kind, inlet_param=w["inlet_model"].param, precision=0,
                device=0)
    args.update(over)
    d = _lib.Desc(**args)
    return d, (gx, gy, gz, kl, rl, dl, bh)


@pytest.mark.parametrize("over,code", [
    (dict(nx=1), _lib.GW_ERR_ARG),
    (dict(n_boreholes=0), _lib.GW_ERR_ARG),
    (dict(inlet_kind=7), _lib.GW_ERR_UNSUPPORTED),
    (dict(precision=9), _lib.GW_ERR_ARG),
])
def test_create_rejects_bad_descriptors(gwlib, over, code):
    w = W.small_case()
    d, keep = _desc(w, **over)
    h = ctypes.c_void_p()
    rc = gwlib.gw_create(ctypes.byref(d), ctypes.byref(h))
    assert rc == code and not h.value
    assert gwlib.gw_last_error()


def test_create_rejects_unsorted_grid(gwlib):
    w = W.small_case()
    w = dict(w, gridx=w["gridx"][::-1].copy())
    d, keep = _desc(w)
    h = ctypes.c_void_p()
    assert gwlib.gw_create(ctypes.byref(d), ctypes.byref(h)) == _lib.GW_ERR_ARG
    assert b"increasing" in gwlib.gw_last_error()


def test_null_arguments(gwlib):
    assert gwlib.gw_create(None, None) == _lib.GW_ERR_ARG
    assert gwlib.gw_get_info(None, None) == _lib.GW_ERR_ARG
    assert gwlib.gw_step(None, 0.0, 1.0, 1, 100) == _lib.GW_ERR_ARG
    assert gwlib.gw_destroy(None) == _lib.GW_OK


def test_custom_inlet_is_rejected_by_the_host_mirror():
    from geothermalwells_gb300 import CustomInlet, GB300, create_cache
    w = W.small_case()
    with pytest.raises(ValueError):
        create_cache(backend=GB300(), gridx=w["gridx"], gridy=w["gridy"], gridz=w["gridz"],
                     materials=w["materials"], boreholes=w["boreholes"],
                     inlet_model=CustomInlet(lambda b, T, t: 20.0))
