"""Objective of the FP64 CPU oracle for central finite differences (test
helper, imported by the adjoint tests).

J(p) = sum_b [ w_energy * E_b + w_outlet * T_out,b(last step) ] with
E_b = sum_n mdot_b c_w (T_out,b^n - T_in,b^n) dt, c_w = rho_c_water / 998.2,
for p = (rock layer conductivities, flow rates, inlet parameter) of a
workload dict (``geothermalwells_gb300.workloads``).  The oracle runs the
reference's step (ROCK2 of rhs_diffusion_z! then ADI_and_ADV_callback!) on
the CPU, so these differences are the reference's own derivatives.
"""
import numpy as np

from geothermalwells_gb300 import (ConstantInlet, HeatExchangerInlet, StratifiedMaterialProperties,
                                   rock2)
from geothermalwells_gb300.physics import RHO_WATER
import oracle as O


def params(w):
    m = w["materials"]
    return np.concatenate([np.asarray(m.k_rock_layers, dtype=np.float64),
                           [b.mdot for b in w["boreholes"]], [w["inlet_model"].param]])


def with_params(w, p):
    m = w["materials"]
    nl = len(m.k_rock_layers)
    nb = len(w["boreholes"])
    mat = StratifiedMaterialProperties(tuple(p[:nl]), m.rho_c_rock_layers, m.layer_depths, *m.fixed())
    bhs = tuple(b.with_flow(q) for b, q in zip(w["boreholes"], p[nl:nl + nb]))
    inlet = ConstantInlet(p[-1]) if w["inlet_model"].kind == 0 else HeatExchangerInlet(p[-1])
    return dict(w, materials=mat, boreholes=bhs, inlet_model=inlet)


def objective(w, p, nsteps, w_energy=1.0, w_outlet=0.0, T0=None):
    v = with_params(w, p)
    orc = O.Oracle(v["gridx"], v["gridy"], v["gridz"], v["boreholes"], v["materials"], v["inlet_model"])
    try:
        s, _ = rock2.choose_stages(v["dt"], orc.eigen_estimate())
        u = (w["T0"] if T0 is None else T0).copy(order="F")
        out = orc.simulate(u, v.get("t0", 0.0), v["dt"], nsteps, s, rock2.coefficients(s))
    finally:
        orc.close()
    c_w = v["materials"].rho_c_water / RHO_WATER
    mdot = np.array([b.mdot for b in v["boreholes"]])
    T_in = p[-1] if v["inlet_model"].kind == 0 else out - p[-1]
    E = (mdot * c_w * (out - T_in) * v["dt"]).sum(axis=0)
    return float(w_energy * E.sum() + w_outlet * out[-1].sum())


def central_fd(w, nsteps, rel=1e-4, **kw):
    """Central differences with step rel * |p_i| in every parameter."""
    p0 = params(w)
    g = np.zeros_like(p0)
    for i in range(len(p0)):
        h = rel * abs(p0[i])
        pp, pm = p0.copy(), p0.copy()
        pp[i] += h
        pm[i] -= h
        g[i] = (objective(w, pp, nsteps, **kw) - objective(w, pm, nsteps, **kw)) / (pp[i] - pm[i])
    return g
