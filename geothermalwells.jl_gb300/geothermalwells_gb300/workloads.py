"""Named simulation set-ups: the reference's two examples and the single-well
benchmark configurations.  Each returns a dict with gridx, gridy, gridz,
boreholes, materials, inlet_model, T0 (initial field), dt and nsteps.

The coaxial benchmark well: 2000 m deep, inner pipe r = 0.0625 m with a
0.01 m wall, casing inner radius 0.088 m with a 0.01 m steel wall, grout to
0.108 m; rock k = 2.5 W/m/K, rho*c = 2.2e6; water 0.6 / 4.18e6; inner-pipe
wall 0.4 W/m/K (insulating), steel casing 45 W/m/K; 5 kg/s, ConstantInlet
20 degC; T0 = 2.29 + 0.035 z.  The reference's x/y generator cannot produce
the 61 / 201 points such configurations quote at 2 mm refinement, so the
grid parameters are pinned here and the resulting counts stated:
  single_well_2mm:   dx_fine 2 mm, growth 1.15, dx_max 10 m over +-50 m
                     -> 225 x 225 x 402 (z: 400 cells of 5.5 m + h)
  single_well_large: dx_fine 3 mm, growth 1.15, dx_max 5 m over +-100 m
                     -> 205 x 205 x 2002 (z: 2000 cells of 1.1 m + h)
"""
import numpy as np

from .grids import create_adaptive_grid_1d, create_uniform_gridz_with_borehole_depths
from .physics import (Borehole, ConstantInlet, HeatExchangerInlet, HomogenousMaterialProperties,
                      StratifiedMaterialProperties, initial_condition_thermal_gradient)


def _xy(lo, hi, dx_fine, growth, dx_max, bhs):
    gx = create_adaptive_grid_1d(xmin=lo, xmax=hi, dx_fine=dx_fine, growth_factor=growth,
                                 dx_max=dx_max, boreholes=bhs, direction="x")
    gy = create_adaptive_grid_1d(xmin=lo, xmax=hi, dx_fine=dx_fine, growth_factor=growth,
                                 dx_max=dx_max, boreholes=bhs, direction="y")
    return gx, gy


def example_single_borehole():
    """``examples/single_borehole_basic.jl``: the set-up behind the
    reference's integration test (``test/test_integration.jl:17``)."""
    mat = HomogenousMaterialProperties(2.88, 2.17e6, 0.6, 4.18e6, 44.5, 3.73e6, 0.26, 1.96e6,
                                       1.0, 1.0)
    bhs = (Borehole(0.0, 0.0, 350.0, 0.0381, 0.01, 0.0889, 0.01, 0.0989, 10.0, 100.0),)
    gx, gy = _xy(-100.0, 100.0, 0.0025, 1.3, 10.0, bhs)
    gz = create_uniform_gridz_with_borehole_depths(zmin=0.0, zmax=370.0, dz=10.0, boreholes=bhs)
    T0 = initial_condition_thermal_gradient(None, np.float64, gx, gy, gz, T_surface=2.29,
                                            gradient=0.35)
    return dict(name="example_single_borehole", gridx=gx, gridy=gy, gridz=gz, boreholes=bhs,
                materials=mat, inlet_model=ConstantInlet(20.0), T0=T0, dt=80.0, nsteps=10,
                t0=0.0)


def example_well_array():
    """``examples/well_array_basic.jl``: 2 x 2 array, HeatExchangerInlet(5)."""
    mat = HomogenousMaterialProperties(2.5, 2.0e6, 0.6, 4.18e6, 44.5, 3.73e6, 0.26, 1.96e6,
                                       1.5, 1.76e6)
    bhs = tuple(Borehole(xc, yc, 350.0, 0.0381, 0.01, 0.0889, 0.01, 0.0989, 10.0, 100.0)
                for yc in (-15.0, 15.0) for xc in (-15.0, 15.0))  # Julia's (xc in XC, yc in YC) order
    gx, gy = _xy(-80.0, 80.0, 0.0025, 1.3, 10.0, bhs)
    gz = create_uniform_gridz_with_borehole_depths(zmin=0.0, zmax=370.0, dz=10.0, boreholes=bhs)
    T0 = initial_condition_thermal_gradient(None, np.float64, gx, gy, gz, T_surface=10.0,
                                            gradient=0.35)
    return dict(name="example_well_array", gridx=gx, gridy=gy, gridz=gz, boreholes=bhs,
                materials=mat, inlet_model=HeatExchangerInlet(5.0), T0=T0, dt=80.0, nsteps=10,
                t0=0.0)


def coaxial_materials():
    return HomogenousMaterialProperties(2.5, 2.2e6, 0.6, 4.18e6, 45.0, 3.73e6, 0.4, 1.96e6,
                                        1.5, 1.76e6)


def coaxial_borehole(xc=0.0, yc=0.0, h=2000.0, mdot=5.0):
    return Borehole(xc, yc, h, 0.0625, 0.01, 0.088, 0.01, 0.108, mdot, 0.0)


def single_well_2mm():
    """Plain FP64 single well: 225 x 225 x 402, dt 60 s, 1 simulated hour."""
    bhs = (coaxial_borehole(),)
    gx, gy = _xy(-50.0, 50.0, 0.002, 1.15, 10.0, bhs)
    gz = create_uniform_gridz_with_borehole_depths(zmin=0.0, zmax=2200.0, dz=5.5, boreholes=bhs)
    T0 = initial_condition_thermal_gradient(None, np.float64, gx, gy, gz, T_surface=2.29,
                                            gradient=0.035)
    return dict(name="single_well_2mm_225x225x402", gridx=gx, gridy=gy, gridz=gz, boreholes=bhs,
                materials=coaxial_materials(), inlet_model=ConstantInlet(20.0), T0=T0, dt=60.0,
                nsteps=60, t0=0.0)


def single_well_large():
    """Plain vs mixed single well: 205 x 205 x 2002 (8.4e7 cells), dt 300 s,
    30 simulated days (8640 steps)."""
    bhs = (coaxial_borehole(),)
    gx, gy = _xy(-100.0, 100.0, 0.003, 1.15, 5.0, bhs)
    gz = create_uniform_gridz_with_borehole_depths(zmin=0.0, zmax=2200.0, dz=1.1, boreholes=bhs)
    T0 = initial_condition_thermal_gradient(None, np.float64, gx, gy, gz, T_surface=2.29,
                                            gradient=0.035)
    return dict(name="single_well_large_205x205x2002", gridx=gx, gridy=gy, gridz=gz,
                boreholes=bhs, materials=coaxial_materials(), inlet_model=ConstantInlet(20.0),
                T0=T0, dt=300.0, nsteps=8640, t0=0.0)


def small_case(n_layers=1, inlet="constant", nbh=1, nz_cells=12, spacing=0.6, h=60.0,
               insulation_depth=20.0, backfill_quirk=False, dt=40.0):
    """A few-thousand-cell well (or row of wells) for element-wise parity
    checks: coarse x/y around the pipes, every material class present,
    layered rock optional, both inlet kinds.  ``backfill_quirk`` gives the
    grout the reference example's placeholder k = rho*c = 1 (diffusivity 1),
    which only inflates the eigenvalue estimate and so the ROCK2 stage count,
    as in ``examples/single_borehole_basic.jl:25-26``."""
    xs = [spacing * (b - (nbh - 1) / 2) for b in range(nbh)]
    bhs = tuple(Borehole(x, 0.0, h - 7.0 * b, 0.0381, 0.01, 0.0889, 0.01, 0.0989, 3.0 + b,
                         insulation_depth) for b, x in enumerate(xs))
    gx, gy = _xy(-1.0 - spacing * nbh, 1.0 + spacing * nbh, 0.012, 1.6, 0.5, bhs)
    gz = create_uniform_gridz_with_borehole_depths(zmin=0.0, zmax=h * 1.25, dz=h * 1.25 / nz_cells,
                                                   boreholes=bhs)
    kb, rb = (1.0, 1.0) if backfill_quirk else (1.5, 1.76e6)
    if n_layers == 1:
        mat = HomogenousMaterialProperties(2.5, 2.2e6, 0.6, 4.18e6, 45.0, 3.73e6, 0.4, 1.96e6,
                                           kb, rb)
    else:
        depths = tuple(float(d) for d in np.linspace(h * 1.25 / n_layers, h * 1.25, n_layers))
        ks = tuple(1.8 + 0.3 * q for q in range(n_layers))
        rcs = tuple(2.0e6 + 1e5 * q for q in range(n_layers))
        mat = StratifiedMaterialProperties(ks, rcs, depths, 0.6, 4.18e6, 45.0, 3.73e6, 0.4,
                                           1.96e6, kb, rb)
    T0 = initial_condition_thermal_gradient(None, np.float64, gx, gy, gz, T_surface=5.0,
                                            gradient=0.5)
    im = ConstantInlet(10.0) if inlet == "constant" else HeatExchangerInlet(3.0)
    return dict(name="small", gridx=gx, gridy=gy, gridz=gz, boreholes=bhs, materials=mat,
                inlet_model=im, T0=T0, dt=float(dt), nsteps=6, t0=0.0)


def tridiagonal_batch(nsys=262144, lmin=32, lmax=1024, seed=20261203):
    """Batched Thomas microbenchmark: nsys independent systems with lengths
    uniform in [lmin, lmax]; a_i, c_i ~ -U(0.1, 1), b_i = 1 + |a_i| + |c_i| +
    U(0, 2) (strictly diagonally dominant, like the ADI implicit step),
    d_i ~ U(0, 100); seeded.  Returned in the grouped interleaved layout of
    gw_tridiag_batch: systems sorted by length (longest first) in groups of
    32, row r of lane l of group g at group_off[g] + 32 r + l, identity rows
    as padding, a_0 = c_{len-1} = 0.  Also returns the true lengths per slot
    and the permutation (slot -> original system index)."""
    rng = np.random.default_rng(seed)
    lengths = rng.integers(lmin, lmax + 1, size=nsys)
    ngroups = (nsys + 31) // 32
    order = np.argsort(-lengths, kind="stable")
    slot_len = np.zeros(ngroups * 32, dtype=np.int64)
    slot_len[:nsys] = lengths[order]
    glen = slot_len.reshape(ngroups, 32).max(axis=1)
    goff = np.zeros(ngroups + 1, dtype=np.int64)
    goff[1:] = np.cumsum(glen * 32)
    n = int(goff[-1])
    a = -rng.uniform(0.1, 1.0, n)
    c = -rng.uniform(0.1, 1.0, n)
    b = 1.0 + np.abs(a) + np.abs(c) + rng.uniform(0.0, 2.0, n)
    d = rng.uniform(0.0, 100.0, n)
    for g in range(ngroups):
        sl = slice(goff[g], goff[g + 1])
        lens = slot_len[32 * g:32 * g + 32]
        rows = np.arange(glen[g])[:, None]
        pad = rows >= lens[None, :]
        last = rows == (lens[None, :] - 1)
        ag, bg, cg, dg = (v[sl].reshape(glen[g], 32) for v in (a, b, c, d))
        ag[pad] = 0.0; cg[pad] = 0.0; bg[pad] = 1.0; dg[pad] = 0.0
        ag[0, :] = 0.0
        cg[last] = 0.0
    return dict(name="tridiagonal_batch_%d_len%d-%d" % (nsys, lmin, lmax), a=a, b=b, c=c, d=d,
                group_off=goff[:-1].copy(), group_len=glen.astype(np.int32), n=n,
                ngroups=ngroups, unknowns=int(lengths.sum()), slot_len=slot_len, order=order)


def array_design(rng, n_cells, dt=3600.0, years=10.0, spacing=None, h=None, mdot=None):
    """One 3 x 3 coaxial well array for the ensemble: spacing U(10, 40) m,
    depth U(1500, 3000) m (snapped to the z grid so no sliver cell appears
    at h), flow U(2, 8) kg/s, rock k per 100 m layer U(1.8, 3.5) W/m/K.
    The x/y refinement (4 mm to 1 cm at the wells, so every inner pipe and
    annulus holds grid columns; growth 1.6 to cells of at most 20 m) and nz
    (300 to 1500) are chosen so the grid has about n_cells cells.  Resolving
    the pipes of a 3 x 3 array needs at least ~150 points per direction."""
    spacing = float(rng.uniform(10.0, 40.0)) if spacing is None else spacing
    h = float(rng.uniform(1500.0, 3000.0)) if h is None else h
    mdot = float(rng.uniform(2.0, 8.0)) if mdot is None else mdot
    zmax = h + 200.0
    nlay = int(np.ceil(zmax / 100.0))
    ks = tuple(float(v) for v in rng.uniform(1.8, 3.5, nlay))
    depths = tuple(100.0 * (q + 1) for q in range(nlay))
    mat = StratifiedMaterialProperties(ks, (2.2e6,) * nlay, depths, 0.6, 4.18e6, 45.0, 3.73e6,
                                       0.4, 1.96e6, 1.5, 1.76e6)
    # nz and nxy: nz in [300, 1500], nxy in [81, 241], nxy^2 nz ~ n_cells
    nz_target = int(np.clip(rng.uniform(300, 1500), 300, 1500))
    nxy_target = int(np.clip(np.sqrt(n_cells / nz_target), 81, 241))
    nz_target = int(np.clip(n_cells / nxy_target ** 2, 300, 1500))
    dz = zmax / nz_target
    h = round(h / dz) * dz
    pos = (-spacing, 0.0, spacing)
    bhs = tuple(Borehole(x, y, h, 0.0625, 0.01, 0.088, 0.01, 0.108, mdot, 0.0)
                for y in pos for x in pos)
    lo, hi = -spacing - 100.0, spacing + 100.0
    # coarsest refinement (at most 1 cm, so the 15 mm annulus and the inner
    # pipe hold grid columns) whose grid reaches the target point count
    f_lo, f_hi = 0.004, 0.01
    for _ in range(30):
        f = np.sqrt(f_lo * f_hi)
        n = len(create_adaptive_grid_1d(xmin=lo, xmax=hi, dx_fine=f, growth_factor=1.6,
                                        dx_max=20.0, boreholes=bhs, direction="x"))
        if n > nxy_target:
            f_lo = f
        else:
            f_hi = f
    gx, gy = _xy(lo, hi, f_hi, 1.6, 20.0, bhs)
    # keep the design's cell budget: refit nz to the x/y count obtained
    nz_target = int(np.clip(n_cells / len(gx) ** 2, 300, 1500))
    dz = zmax / nz_target
    h = round(bhs[0].h / dz) * dz
    bhs = tuple(Borehole(b.xc, b.yc, h, 0.0625, 0.01, 0.088, 0.01, 0.108, mdot, 0.0) for b in bhs)
    gz = create_uniform_gridz_with_borehole_depths(zmin=0.0, zmax=zmax, dz=dz, boreholes=bhs)
    return dict(name="array3x3", gridx=gx, gridy=gy, gridz=gz, boreholes=bhs, materials=mat,
                inlet_model=ConstantInlet(15.0), dt=dt, nsteps=int(round(years * 365 * 86400 / dt)),
                t0=0.0, T_surface=8.0, gradient=0.03, spacing=spacing, h=h, mdot=mdot)


def ensemble(n_designs=64, total_cells=1.5e9, seed=20261204):
    """The heterogeneous ensemble: n_designs 3 x 3 arrays whose grids (81^2 x
    300 up to 241^2 x 1500) add up to about total_cells.  Initial fields are
    built per design on demand (initial_field) to keep host memory small."""
    rng = np.random.default_rng(seed)
    w = rng.lognormal(0.0, 0.8, n_designs)
    w *= total_cells / w.sum()
    w = np.clip(w, 81 ** 2 * 300, 241 ** 2 * 1500)
    return [array_design(rng, float(cells)) for cells in w]


def initial_field(d):
    """T0 = T_surface + gradient z for one design (Fortran order, (Nz, Ny, Nx))."""
    return initial_condition_thermal_gradient(None, np.float64, d["gridx"], d["gridy"], d["gridz"],
                                              T_surface=d["T_surface"], gradient=d["gradient"])


def initial_gradient(d):
    """(T_surface, gradient) of one design, for the device-side initial field."""
    return d["T_surface"], d["gradient"]


def adjoint_small(inlet="constant", nbh=1, n_layers=3, backfill_quirk=False, dt=200.0, nsteps=12):
    """A few-thousand-cell well for checking gradients against central
    differences of the oracle: the small_case geometry at low flow (0.6 kg/s,
    + 0.3 per further borehole, so inner cells both interpolate within the
    pipe and turn around at the bottom) run long enough (12 steps of 200 s)
    for every rock layer to shape the outlet temperature."""
    w = small_case(n_layers=n_layers, inlet=inlet, nbh=nbh, backfill_quirk=backfill_quirk, dt=dt)
    bhs = tuple(b.with_flow(0.6 + 0.3 * q) for q, b in enumerate(w["boreholes"]))
    return dict(w, name="adjoint_small", boreholes=bhs, nsteps=int(nsteps))


def adjoint_well(seed=20261205):
    """Gradient workload: the single_well_large grid (205 x 205 x 2002) with 22
    rock layers of 100 m, k ~ U(1.8, 3.5) W/m/K (seeded), rho*c 2.2e6, 5 kg/s,
    ConstantInlet 20 degC, 7 simulated days, checkpoints every 64 steps.
    The step is 200 s (3024 steps): at 300 s the reference's splitting
    diverges on this z grid (from about step 90, starting at the casing at
    z = h), which its own CPU restatement reproduces."""
    w = single_well_large()
    rng = np.random.default_rng(seed)
    ks = tuple(float(v) for v in rng.uniform(1.8, 3.5, 22))
    depths = tuple(100.0 * (q + 1) for q in range(22))
    mat = StratifiedMaterialProperties(ks, (2.2e6,) * 22, depths, 0.6, 4.18e6, 45.0, 3.73e6, 0.4,
                                       1.96e6, 1.5, 1.76e6)
    return dict(w, name="adjoint_well_205x205x2002_22layers", materials=mat, dt=200.0,
                nsteps=3024, checkpoint_every=64)
