"""ctypes binding of ``libgw_gb300.so`` (declarations: ``include/gw_gb300.h``).

This is the Python counterpart of the ``ccall`` layer a Julia backend uses.
The library is the only compute path: if it cannot be loaded, every entry
point raises instead of falling back to anything else.
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
PKG_ROOT = os.path.dirname(_HERE)
# GW_LIB selects another build of the library (the bounds-checking debug
# build, lib/libgw_gb300_debug.so)
LIB_PATH = os.environ.get("GW_LIB") or os.path.join(PKG_ROOT, "lib", "libgw_gb300.so")

GW_OK, GW_ERR_ARG, GW_ERR_CUDA, GW_ERR_NONFINITE, GW_ERR_TIMEOUT, GW_ERR_UNSUPPORTED = range(6)
GW_PREC_FP64, GW_PREC_MIXED = 0, 1
GW_INLET_CONSTANT, GW_INLET_HEAT_EXCHANGER, GW_INLET_SCHEDULE, GW_INLET_EXPRESSION = 0, 1, 2, 3
GW_MODULAR_NZ, GW_MODULAR_SHARED_COLUMN = 1, 2
GW_MIXED_ROCK2_F64, GW_MIXED_REFINE = 1, 2
DIRS = {"x": 0, "y": 1, "z": 2}

# Every symbol include/gw_gb300.h declares, with (restype, argtypes).
_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_vp = ctypes.c_void_p
_i, _d = ctypes.c_int, ctypes.c_double


class BoreholeDesc(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in
                ("xc", "yc", "h", "r_inner", "t_inner", "r_outer", "t_outer", "r_backfill",
                 "mdot", "insulation_depth")]


class MaterialDesc(ctypes.Structure):
    _fields_ = [("n_layers", ctypes.c_int), ("k_rock_layers", _dp),
                ("rho_c_rock_layers", _dp), ("layer_depths", _dp)] + \
               [(n, ctypes.c_double) for n in
                ("k_water", "rho_c_water", "k_steel", "rho_c_steel", "k_insulating",
                 "rho_c_insulating", "k_backfill", "rho_c_backfill")]


class Desc(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
                ("gridx", _dp), ("gridy", _dp), ("gridz", _dp),
                ("n_boreholes", ctypes.c_int), ("boreholes", ctypes.POINTER(BoreholeDesc)),
                ("materials", MaterialDesc), ("inlet_kind", ctypes.c_int),
                ("inlet_param", ctypes.c_double), ("precision", ctypes.c_int),
                ("device", ctypes.c_int)]


class AdjointInfo(ctypes.Structure):
    _fields_ = [("objective", ctypes.c_double), ("n_params", ctypes.c_int), ("stages", ctypes.c_int),
                ("checkpoints", ctypes.c_int), ("forward_ms", ctypes.c_double),
                ("reverse_ms", ctypes.c_double), ("peak_bytes", ctypes.c_longlong)]


class Info(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int) for n in
                ("nx", "ny", "nz", "n_boreholes", "countxy_inner", "countxy_outer", "countz",
                 "n_zclass", "n_profiles")] + \
               [("eigen_estimate", ctypes.c_double), ("device_bytes", ctypes.c_longlong),
                ("overlap", ctypes.c_int), ("fused", ctypes.c_int), ("modular_reason", ctypes.c_int),
                ("tiling", ctypes.c_int), ("mixed_options", ctypes.c_int), ("step_order", ctypes.c_int)]


SIGNATURES = {
    "gw_last_error": (ctypes.c_char_p, []),
    "gw_version": (ctypes.c_char_p, []),
    "gw_create": (_i, [ctypes.POINTER(Desc), ctypes.POINTER(_vp)]),
    "gw_destroy": (_i, [_vp]),
    "gw_get_info": (_i, [_vp, ctypes.POINTER(Info)]),
    "gw_set_field": (_i, [_vp, _dp]),
    "gw_get_field": (_i, [_vp, _dp]),
    "gw_init_thermal_gradient": (_i, [_vp, _d, _d]),
    "gw_rhs_diffusion_z": (_i, [_vp, _vp, _vp]),
    "gw_lincomb": (_i, [_vp, _vp, _i, _dp, ctypes.POINTER(_vp)]),
    "gw_field_alloc": (_i, [_vp, ctypes.POINTER(_vp)]),
    "gw_field_free": (_i, [_vp, _vp]),
    "gw_field_copy": (_i, [_vp, _vp, _vp]),
    "gw_set_inlet_schedule": (_i, [_vp, _i, _dp, _dp]),
    "gw_set_inlet_program": (_i, [_vp, _i, _ip, _dp]),
    "gw_diffusion_1d": (_i, [_vp, _vp, _vp, _d, _i, _i]),
    "gw_thomas": (_i, [_vp, _vp, _vp, _d, _i]),
    "gw_advection": (_i, [_vp, _vp, _d, _d]),
    "gw_adi_adv": (_i, [_vp, _vp, _vp, _d, _d]),
    "gw_step": (_i, [_vp, _d, _d, _i, _i]),
    "gw_set_overlap": (_i, [_vp, _i]),
    "gw_set_tiling": (_i, [_vp, _i]),
    "gw_set_mixed_options": (_i, [_vp, _i]),
    "gw_rock2_stages": (_i, [_vp, _d, _i, _ip, _ip]),
    "gw_snapshot_host_alloc": (_i, [_vp, ctypes.POINTER(_vp)]),
    "gw_snapshot_host_free": (_i, [_vp, _vp]),
    "gw_snapshot": (_i, [_vp, _vp]),
    "gw_snapshot_wait": (_i, [_vp]),
    "gw_get_outlet": (_i, [_vp, _dp]),
    "gw_get_outlet_series": (_i, [_vp, _dp, _i]),
    "gw_get_energy": (_i, [_vp, _dp]),
    "gw_reset_energy": (_i, [_vp]),
    "gw_check_finite": (_i, [_vp]),
    "gw_get_last_step_time": (_i, [_vp, _dp]),
    "gw_profile_kernels": (_i, [_vp, _d, _i, _dp]),
    "gw_advection_noalloc": (_i, [_vp, _vp, _d, _d, _vp]),
    "gw_batch_create": (_i, [ctypes.POINTER(_vp), _i, ctypes.POINTER(_vp)]),
    "gw_batch_destroy": (_i, [_vp]),
    "gw_batch_set_tiling": (_i, [_vp, _i]),
    "gw_batch_autotune": (_i, [_vp, _d, _i, _ip]),
    "gw_batch_step": (_i, [_vp, _d, _i, _i]),
    "gw_batch_get_last_step_time": (_i, [_vp, _dp]),
    "gw_tridiag_batch": (_i, [_i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, ctypes.c_longlong, _vp]),
    "gw_adjoint": (_i, [_vp, _d, _i, _i, _i, _d, _d, _dp, _vp, ctypes.POINTER(AdjointInfo)]),
    "gw_step_vjp": (_i, [_vp, _vp, _vp, _d, _i, _d, _d, _dp]),
}
KERNELS = ("rock2_columns", "half_step_x", "half_step_y", "pipe")

_lib = None


class GWError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("gw_gb300 error %d: %s" % (code, msg))
        self.code = code


def load(path=None):
    """Load the library (once).  Raises if it is missing: there is no
    fallback compute path."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError("libgw_gb300.so is not built (%s); run __graft_entry__.build()" % p)
    L = ctypes.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def check(rc):
    if rc != GW_OK:
        raise GWError(rc, load().gw_last_error().decode())
    return rc


def dptr(a):
    return a.ctypes.data_as(_dp)
