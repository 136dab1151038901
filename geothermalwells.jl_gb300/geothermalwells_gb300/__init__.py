"""GB300 (sm_103a) backend for the time-step hot path of GeothermalWells.jl.

The public names mirror the reference's exports (``src/GeothermalWells.jl:21-48``)
that a simulation script uses, with ``GB300()`` as the backend value:

    cache = create_cache(backend=GB300(), gridx=..., gridy=..., gridz=...,
                         materials=..., boreholes=..., inlet_model=...)
    prob = ODEProblem(rhs_diffusion_z, T0, tspan, cache)
    callback, saved_values = get_simulation_callback(saveat=..., print_every_n=...)
    sol = solve(prob, ROCK2(max_stages=100, eigen_est=eigen_estimator),
                dt=dt, adaptive=False, callback=callback)

All computation runs in ``lib/libgw_gb300.so`` (C ABI, ``include/gw_gb300.h``).
"""
from .physics import (Borehole, HomogenousMaterialProperties, StratifiedMaterialProperties,
                      ConstantInlet, HeatExchangerInlet, ScheduleInlet, ExpressionInlet, CustomInlet,
                      initial_condition_thermal_gradient, get_thermal_conductivity,
                      get_volumetric_heat_capacity)
from .grids import (compute_domain, create_uniform_gridz_with_borehole_depths,
                    create_adaptive_grid_1d, julia_range, julia_colon)
from .cache import GB300, Cache, create_cache, get_simulation_callback, SavedValues
from .solver import (rhs_diffusion_z, diffusion_1d, thomas_I_minus_A, advection,
                     ADI_and_ADV_callback, eigen_estimator, ROCK2, ODEProblem, solve, Solution)
from . import rock2

__all__ = [
    "Borehole", "HomogenousMaterialProperties", "StratifiedMaterialProperties", "ConstantInlet",
    "HeatExchangerInlet", "ScheduleInlet", "ExpressionInlet", "CustomInlet", "initial_condition_thermal_gradient",
    "get_thermal_conductivity", "get_volumetric_heat_capacity", "compute_domain",
    "create_uniform_gridz_with_borehole_depths", "create_adaptive_grid_1d", "julia_range",
    "julia_colon", "GB300", "Cache", "create_cache", "get_simulation_callback", "SavedValues",
    "rhs_diffusion_z", "diffusion_1d", "thomas_I_minus_A", "advection", "ADI_and_ADV_callback",
    "eigen_estimator", "ROCK2", "ODEProblem", "solve", "Solution", "rock2",
]
