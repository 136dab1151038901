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


# GW_OP_* codes of include/gw_gb300.h (the inlet program of GW_INLET_EXPRESSION)
OP_CONST, OP_TOUT, OP_TIME, OP_BH, OP_SCHED, OP_NEG = 0, 1, 2, 3, 4, 5
OP_ADD, OP_SUB, OP_MUL, OP_DIV, OP_MIN, OP_MAX = 6, 7, 8, 9, 10, 11


class ExpressionInlet:
    """A ``CustomInlet`` (``src/physics.jl:315-318``) whose closure
    ``(bh, T_outlet, t) -> T_in`` is arithmetic, written as an expression
    string over ``T_out`` (the borehole's outlet temperature,
    ``T_outlet[bh]``), ``t``, ``bh`` (0-based), numbers, ``+ - * /``,
    unary ``-``, ``min(a, b)``, ``max(a, b)`` and ``sched(x)`` (the optional
    piecewise-linear ``schedule=(times, values)`` at ``x``).  For example a
    heat pump that takes ``dT(t)`` out of the outlet but never cools the inlet
    below 5 degrees: ``ExpressionInlet("max(5.0, T_out - sched(t))",
    schedule=([0, 3600], [3.0, 6.0]))``.

    It is compiled to the postfix program of ``GW_INLET_EXPRESSION``, which the
    GPU evaluates per borehole where the reference calls the inlet model
    (``src/solver.jl:349-350``), each operation one correctly rounded double
    operation; calling the object evaluates the same program on the host."""
    kind = 3

    def __init__(self, expr, schedule=None):
        import ast
        self.expr = str(expr)
        self.schedule = None
        if schedule is not None:
            self.schedule = ScheduleInlet(*schedule)
        ops, args = [], []

        def emit(op, a=0.0):
            ops.append(op)
            args.append(float(a))

        bin_ops = {ast.Add: OP_ADD, ast.Sub: OP_SUB, ast.Mult: OP_MUL, ast.Div: OP_DIV}
        names = {"T_out": OP_TOUT, "t": OP_TIME, "bh": OP_BH}

        def walk(n):
            if isinstance(n, ast.Expression):
                return walk(n.body)
            if isinstance(n, ast.Constant) and isinstance(n.value, (int, float)) and not isinstance(n.value, bool):
                return emit(OP_CONST, n.value)
            if isinstance(n, ast.Name) and n.id in names:
                return emit(names[n.id])
            if isinstance(n, ast.UnaryOp) and isinstance(n.op, (ast.USub, ast.UAdd)):
                walk(n.operand)
                if isinstance(n.op, ast.USub):
                    emit(OP_NEG)
                return None
            if isinstance(n, ast.BinOp) and type(n.op) in bin_ops:
                walk(n.left)
                walk(n.right)
                return emit(bin_ops[type(n.op)])
            if isinstance(n, ast.Call) and isinstance(n.func, ast.Name) and not n.keywords:
                f, a = n.func.id, n.args
                if f in ("min", "max") and len(a) >= 2:
                    walk(a[0])
                    for x in a[1:]:
                        walk(x)
                        emit(OP_MIN if f == "min" else OP_MAX)
                    return None
                if f == "sched" and len(a) == 1:
                    if self.schedule is None:
                        raise ValueError("sched(...) needs ExpressionInlet(..., schedule=(times, values))")
                    walk(a[0])
                    return emit(OP_SCHED)
            raise ValueError("unsupported element in the inlet expression %r: %s"
                             % (self.expr, ast.dump(n)))

        walk(ast.parse(self.expr, mode="eval"))
        depth, top = 0, 0
        for o in ops:
            depth += 1 if o <= OP_BH else (0 if o <= OP_NEG else -1)
            top = max(top, depth)
        if len(ops) > 64 or top > 16:
            raise ValueError("inlet expression too long (at most 64 operations, stack depth 16)")
        self.ops = tuple(ops)
        self.args = tuple(args)

    @property
    def param(self):
        return 0.0

    def __call__(self, bh_idx, T_outlet_values, t):
        st = []
        for o, a in zip(self.ops, self.args):
            if o == OP_CONST:
                st.append(a)
            elif o == OP_TOUT:
                st.append(float(T_outlet_values[bh_idx]))
            elif o == OP_TIME:
                st.append(float(t))
            elif o == OP_BH:
                st.append(float(bh_idx))
            elif o == OP_SCHED:
                st[-1] = self.schedule(bh_idx, T_outlet_values, st[-1])
            elif o == OP_NEG:
                st[-1] = -st[-1]
            else:
                b = st.pop()
                x = st[-1]
                st[-1] = {OP_ADD: x + b, OP_SUB: x - b, OP_MUL: x * b, OP_DIV: x / b if b else np.inf,
                          OP_MIN: min(x, b), OP_MAX: max(x, b)}[o]
        return st[0]


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
