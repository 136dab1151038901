"""Geometry, materials and inlet models, mirroring ``src/physics.jl``.

These are plain parameter records.  The device-side material model is built
from them by the library when a cache is created (``gw_create``); the
lookups below exist for host-side checks and follow the reference's
branch order exactly.
"""
from dataclasses import dataclass, field
import math

import numpy as np

RHO_WATER = 998.2  # kg/m^3, src/physics.jl:49


class Borehole:
    """Coaxial borehole heat exchanger, ``src/physics.jl:30-61``.

    ``Borehole(xc, yc, h, r_inner, t_inner, r_outer, t_outer, r_backfill,
    mdot, insulation_depth)``; fluid flows down the annulus and up the inner
    pipe.  Squared radii and the plug-flow velocities are derived exactly as
    the reference's constructor does (``src/physics.jl:48-59``)."""

    __slots__ = ("xc", "yc", "h", "r_inner", "t_inner", "r_and_t_inner_sq", "r_outer",
                 "r_outer_sq", "t_outer", "r_and_t_outer_sq", "r_backfill", "r_backfill_sq",
                 "mdot", "v_inner", "v_outer", "insulation_depth")

    def __init__(self, xc, yc, h, r_inner, t_inner, r_outer, t_outer, r_backfill, mdot,
                 insulation_depth):
        f = float
        self.xc, self.yc, self.h = f(xc), f(yc), f(h)
        self.r_inner, self.t_inner = f(r_inner), f(t_inner)
        self.r_outer, self.t_outer = f(r_outer), f(t_outer)
        self.r_backfill, self.mdot = f(r_backfill), f(mdot)
        self.insulation_depth = f(insulation_depth)
        rti = self.r_inner + self.t_inner
        self.r_and_t_inner_sq = rti * rti
        self.r_outer_sq = self.r_outer * self.r_outer
        rto = self.r_outer + self.t_outer
        self.r_and_t_outer_sq = rto * rto
        self.r_backfill_sq = self.r_backfill * self.r_backfill
        a_inner = math.pi * (self.r_inner * self.r_inner)
        a_outer = math.pi * self.r_outer_sq - math.pi * self.r_and_t_inner_sq
        self.v_inner = self.mdot / (a_inner * RHO_WATER)
        self.v_outer = self.mdot / (a_outer * RHO_WATER)

    def args(self):
        """The ten constructor arguments, in order (the C-ABI record)."""
        return (self.xc, self.yc, self.h, self.r_inner, self.t_inner, self.r_outer,
                self.t_outer, self.r_backfill, self.mdot, self.insulation_depth)

    def with_flow(self, mdot):
        a = list(self.args())
        a[8] = mdot
        return Borehole(*a)

    def __repr__(self):
        return "Borehole(%s)" % ", ".join(repr(v) for v in self.args())


@dataclass
class StratifiedMaterialProperties:
    """``src/physics.jl:81-94``: rock layers with ``z <= layer_depths[i]``
    selecting layer i (deepest layer below all), plus pipe/fluid/grout."""
    k_rock_layers: tuple
    rho_c_rock_layers: tuple
    layer_depths: tuple
    k_water: float
    rho_c_water: float
    k_steel: float
    rho_c_steel: float
    k_insulating: float
    rho_c_insulating: float
    k_backfill: float
    rho_c_backfill: float

    def __post_init__(self):
        n = len(self.k_rock_layers)
        if n < 1 or len(self.rho_c_rock_layers) != n or len(self.layer_depths) != n:
            raise ValueError("rock layer tuples must be non-empty and of equal length")
        self.k_rock_layers = tuple(float(v) for v in self.k_rock_layers)
        self.rho_c_rock_layers = tuple(float(v) for v in self.rho_c_rock_layers)
        self.layer_depths = tuple(float(v) for v in self.layer_depths)

    def layers(self):
        return self.k_rock_layers, self.rho_c_rock_layers, self.layer_depths

    def fixed(self):
        return (self.k_water, self.rho_c_water, self.k_steel, self.rho_c_steel,
                self.k_insulating, self.rho_c_insulating, self.k_backfill, self.rho_c_backfill)

    # src/physics.jl:102-125
    def rock_k(self, z):
        for k, d in zip(self.k_rock_layers, self.layer_depths):
            if z <= d:
                return k
        return self.k_rock_layers[-1]

    def rock_rho_c(self, z):
        for r, d in zip(self.rho_c_rock_layers, self.layer_depths):
            if z <= d:
                return r
        return self.rho_c_rock_layers[-1]

    def d_max(self):
        """``src/physics.jl:134-149`` eigen_estimator_get_dmax."""
        d = 0.0
        for k, r in zip(self.k_rock_layers, self.rho_c_rock_layers):
            d = max(d, k / r)
        return max(d, self.k_water / self.rho_c_water, self.k_steel / self.rho_c_steel,
                   self.k_insulating / self.rho_c_insulating,
                   self.k_backfill / self.rho_c_backfill)


class HomogenousMaterialProperties(StratifiedMaterialProperties):
    """``src/physics.jl:159-175``: uniform rock.  Identical in every lookup to
    a one-layer stratified model (the deepest-layer fallback returns the same
    values), which is how it crosses the C ABI."""

    def __init__(self, k_rock, rho_c_rock, k_water, rho_c_water, k_steel, rho_c_steel,
                 k_insulating, rho_c_insulating, k_backfill, rho_c_backfill):
        super().__init__((float(k_rock),), (float(rho_c_rock),), (math.inf,),
                         float(k_water), float(rho_c_water), float(k_steel), float(rho_c_steel),
                         float(k_insulating), float(rho_c_insulating), float(k_backfill),
                         float(rho_c_backfill))

    @property
    def k_rock(self):
        return self.k_rock_layers[0]

    @property
    def rho_c_rock(self):
        return self.rho_c_rock_layers[0]


def get_thermal_conductivity(x, y, z, boreholes, materials):
    """``src/physics.jl:199-233`` (host copy of the device lookup)."""
    k = materials.rock_k(z)
    for bh in boreholes:
        r_sq = (x - bh.xc) * (x - bh.xc) + (y - bh.yc) * (y - bh.yc)
        if r_sq > bh.r_backfill_sq:
            continue
        if z <= bh.h:
            if r_sq < bh.r_inner * bh.r_inner:
                k = materials.k_water
            elif r_sq < bh.r_and_t_inner_sq:
                k = materials.k_insulating
            elif r_sq < bh.r_outer_sq:
                k = materials.k_water
            elif r_sq < bh.r_and_t_outer_sq:
                k = materials.k_insulating if z <= bh.insulation_depth else materials.k_steel
            else:
                k = materials.k_backfill
        elif z <= bh.h + 3:
            k = materials.k_steel
    return k


def get_volumetric_heat_capacity(x, y, z, boreholes, materials):
    """``src/physics.jl:243-274`` (host copy of the device lookup)."""
    rc = materials.rock_rho_c(z)
    for bh in boreholes:
        r_sq = (x - bh.xc) * (x - bh.xc) + (y - bh.yc) * (y - bh.yc)
        if r_sq > bh.r_and_t_outer_sq:
            continue
        if z <= bh.h:
            if r_sq < bh.r_inner * bh.r_inner:
                rc = materials.rho_c_water
            elif r_sq < bh.r_and_t_inner_sq:
                rc = materials.rho_c_insulating
            elif r_sq < bh.r_outer_sq:
                rc = materials.rho_c_water
            else:
                rc = materials.rho_c_insulating if z <= bh.insulation_depth else materials.rho_c_steel
        elif z <= bh.h + 3:
            rc = materials.rho_c_steel
    return rc


class ConstantInlet:
    """``src/physics.jl:290-293``: inlet temperature ``T_const``."""
    kind = 0

    def __init__(self, T_const):
        self.T_const = float(T_const)

    @property
    def param(self):
        return self.T_const

    def __call__(self, bh_idx, T_outlet_values, t):
        return self.T_const


class HeatExchangerInlet:
    """``src/physics.jl:303-306``: inlet = outlet of the same borehole - dT."""
    kind = 1

    def __init__(self, dT):
        self.dT = float(dT)

    @property
    def param(self):
        return self.dT

    def __call__(self, bh_idx, T_outlet_values, t):
        return T_outlet_values[bh_idx] - self.dT


class ScheduleInlet:
    """A ``CustomInlet`` (``src/physics.jl:315-318``) whose closure is a
    piecewise-linear schedule ``(bh, T_outlet, t) -> T_in(t)``: linear between
    the points, held constant before the first and after the last.  The form
    of custom inlet that crosses the C ABI (``GW_INLET_SCHEDULE``)."""
    kind = 2

    def __init__(self, times, values):
        self.times = tuple(float(v) for v in times)
        self.values = tuple(float(v) for v in values)
        if len(self.times) < 1 or len(self.times) != len(self.values):
            raise ValueError("one value per schedule time, at least one point")
        if any(b <= a for a, b in zip(self.times, self.times[1:])):
            raise ValueError("schedule times must be strictly increasing")

    @property
    def param(self):
        return 0.0

    def __call__(self, bh_idx, T_outlet_values, t):
        return float(np.interp(t, self.times, self.values))


class CustomInlet:
    """``src/physics.jl:315-318``: an arbitrary host function.  The GB300
    backend evaluates the inlet on the device, so a Python callable cannot
    cross the C ABI; :func:`create_cache` rejects it with ``ValueError``."""
    kind = -1

    def __init__(self, func):
        self.func = func

    def __call__(self, bh_idx, T_outlet_values, t):
        return self.func(bh_idx, T_outlet_values, t)


def initial_condition_thermal_gradient(backend, Float_used, gridx, gridy, gridz, *,
                                       T_surface, gradient):
    """``src/physics.jl:333-348``: ``T = T_surface + gradient * z`` as an
    ``(Nz, Ny, Nx)`` array in Julia (column-major) order, i.e. a Fortran-ordered
    numpy array so that ``T0[k, j, i]`` indexes like the reference."""
    nx, ny, nz = len(gridx), len(gridy), len(gridz)
    col = float(T_surface) + float(gradient) * np.asarray(gridz, dtype=np.float64)
    T0 = np.empty((nz, ny, nx), dtype=np.float64, order="F")
    T0[...] = col[:, None, None]
    return T0.astype(Float_used, order="F", copy=False)
