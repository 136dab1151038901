/*
 * gw_gb300.h -- C ABI of the GB300 (sm_103a) backend for the time-step hot
 * path of GeothermalWells.jl.
 *
 * The reference's plugin point is the KernelAbstractions `backend` value
 * passed to `create_cache` (src/cache.jl:55); every device-side call then
 * dispatches on `cache.backend` (src/solver.jl:24,28,256-261,444-461).  This
 * library is what a GB300 backend value dispatches to: plain C, plain
 * pointers and sizes, int status codes.
 *
 * Conventions
 *  - Fields are Nz x Ny x Nx arrays of double in the reference's layout
 *    (Julia column-major, z fastest): element (k, j, i) sits at
 *    k + Nz * (j + Ny * i), all indices 0-based here.
 *  - Functions taking `double *` field arguments whose names end in `_dev`
 *    take device pointers; all others take host pointers.
 *  - Every call is synchronous with respect to the host unless stated.
 *  - A context owns one CUDA stream and its device buffers; calls on one
 *    context must not overlap (the reference's cache is not re-entrant
 *    either: T_outlet and u_tmp are shared, src/cache.jl:41,62).
 *  - Return value 0 (GW_OK) on success; otherwise an error code, with a
 *    message available from gw_last_error() on the calling thread.
 */
#ifndef GW_GB300_H
#define GW_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#define GW_OK 0
#define GW_ERR_ARG 1          /* invalid argument or size */
#define GW_ERR_CUDA 2         /* a CUDA call failed */
#define GW_ERR_NONFINITE 3    /* NaN/Inf found in the state by gw_check_finite */
#define GW_ERR_TIMEOUT 4      /* a bounded device wait expired */
#define GW_ERR_UNSUPPORTED 5  /* a feature the device path does not offer */

#define GW_PREC_FP64 0        /* all storage and arithmetic in double */
#define GW_PREC_MIXED 1       /* float theta = T - T_ref(z) storage, ROCK2 stages (as increments,
                                 rounded into the field once per step) and Thomas sweeps; double
                                 outlet / annulus means, pipe interpolation offsets, energy balance */

#define GW_INLET_CONSTANT 0        /* ConstantInlet, src/physics.jl:290-293 */
#define GW_INLET_HEAT_EXCHANGER 1  /* HeatExchangerInlet, src/physics.jl:303-306 */
#define GW_INLET_SCHEDULE 2        /* a CustomInlet (src/physics.jl:315-318) of the form
                                      (bh, T_outlet, t) -> T_in(t): a piecewise-linear
                                      schedule, set with gw_set_inlet_schedule */
#define GW_INLET_EXPRESSION 3      /* a CustomInlet whose closure is arithmetic in the
                                      borehole's outlet temperature, t, the borehole index
                                      and the schedule: a program set with
                                      gw_set_inlet_program */

#define GW_DIR_X 0
#define GW_DIR_Y 1
#define GW_DIR_Z 2

/* Borehole constructor arguments, src/physics.jl:30-61 (the derived squared
 * radii and plug-flow velocities are computed inside, as physics.jl:48-59). */
typedef struct gw_borehole_desc {
    double xc, yc, h, r_inner, t_inner, r_outer, t_outer, r_backfill, mdot, insulation_depth;
} gw_borehole_desc;

/* StratifiedMaterialProperties, src/physics.jl:81-94.  A
 * HomogenousMaterialProperties (physics.jl:159-170) is n_layers = 1. */
typedef struct gw_material_desc {
    int n_layers;
    const double *k_rock_layers;
    const double *rho_c_rock_layers;
    const double *layer_depths;
    double k_water, rho_c_water, k_steel, rho_c_steel;
    double k_insulating, rho_c_insulating, k_backfill, rho_c_backfill;
} gw_material_desc;

/* Everything create_cache(; backend, gridx, gridy, gridz, materials,
 * boreholes, inlet_model) receives (src/cache.jl:55). */
typedef struct gw_desc {
    int nx, ny, nz;
    const double *gridx, *gridy, *gridz;   /* strictly increasing, host */
    int n_boreholes;
    const gw_borehole_desc *boreholes;
    gw_material_desc materials;
    int inlet_kind;        /* GW_INLET_*; CustomInlet closures cannot cross the ABI */
    double inlet_param;    /* T_const or DeltaT */
    int precision;         /* GW_PREC_* (the fused gw_step path) */
    int device;            /* CUDA device ordinal */
} gw_desc;

/* Sizes the reference keeps in its cache (src/cache.jl:28-39,57-58,65). */
typedef struct gw_info_t {
    int nx, ny, nz, n_boreholes;
    int countxy_inner, countxy_outer, countz;
    int n_zclass, n_profiles;
    double eigen_estimate;           /* src/solver.jl:474-488 */
    long long device_bytes;          /* device memory held by the context */
    int overlap;                     /* pipe passes on a second stream (gw_set_overlap) */
    int fused;                       /* 1: gw_step runs the fused graph-captured step;
                                        0: the modular reference-shaped kernels (several
                                        times slower; GW_PREC_FP64 only) */
    int modular_reason;              /* why fused == 0: GW_MODULAR_* bits, 0 when fused */
    int tiling;                      /* half-step kernel (gw_set_tiling) */
    int mixed_options;               /* GW_MIXED_* flags (gw_set_mixed_options) */
    int step_order;                  /* launch order of the overlapped step that gw_step
                                        chose by timing for the last step size: 0 ROCK2
                                        of the pipe rows first, 1 of the pipe columns
                                        first on the second stream (same state bitwise) */
} gw_info_t;

/* gw_info_t.modular_reason bits */
#define GW_MODULAR_NZ 1               /* nz beyond the fused ROCK2 column kernels' shared memory */
#define GW_MODULAR_SHARED_COLUMN 2    /* a pipe column belongs to two boreholes (the later one
                                         overrides, src/physics.jl:204-229) */

typedef struct gw_ctx gw_ctx;

const char *gw_last_error(void);
const char *gw_version(void);

/* create_cache (src/cache.jl:55-116): builds the material model, the advection
 * index lists (src/cache.jl:9-44) and all buffers on the device. */
int gw_create(const gw_desc *desc, gw_ctx **out);
int gw_destroy(gw_ctx *ctx);
int gw_get_info(gw_ctx *ctx, gw_info_t *out);

/* The solution state u owned by the context (the integrator's u). */
int gw_set_field(gw_ctx *ctx, const double *T);
int gw_get_field(gw_ctx *ctx, double *T);
/* initial_condition_thermal_gradient (src/physics.jl:333-348) into u. */
int gw_init_thermal_gradient(gw_ctx *ctx, double T_surface, double gradient);

/* ---- device fields for hosts without a CUDA binding ----
 * No single counterpart in the reference, where KernelAbstractions'
 * `allocate(backend, ...)` / `adapt(backend, ...)` make the device arrays
 * (src/cache.jl:41, src/physics.jl:333-348).  A host language that binds only
 * this library (e.g. Julia through ccall, without CUDA.jl) allocates the
 * fields of the fine-grained entry points here.  Each field holds the
 * context's N = nx*ny*nz doubles on its device and is owned by the caller;
 * free it with gw_field_free before gw_destroy. */
/* A new N-cell double field on the context's device, set to zero. */
int gw_field_alloc(gw_ctx *ctx, double **field_dev);
int gw_field_free(gw_ctx *ctx, double *field_dev);
/* Copy N doubles between host and device memory, or within either (the
 * direction follows from the pointers); returns when the copy is done. */
int gw_field_copy(gw_ctx *ctx, double *dst, const double *src);

/* ---- fine-grained entry points on caller-owned device fields (double) ---- */
/* rhs_diffusion_z!(dphi, phi, cache, t), src/solver.jl:23-31 */
int gw_rhs_diffusion_z(gw_ctx *ctx, double *dphi_dev, const double *phi_dev);
/* diffusion_1D!(dphi, phi, ..., dt, Val(dir), Val(plus_I)), src/solver.jl:34-58 */
int gw_diffusion_1d(gw_ctx *ctx, double *dphi_dev, const double *phi_dev, double dt, int dir,
                    int plus_I);
/* thomas_I_minus_A!(U, RHS, ..., dt, ..., Val(dir)), src/solver.jl:111-232; dir X or Y */
int gw_thomas(gw_ctx *ctx, double *U_dev, const double *RHS_dev, double dt, int dir);
/* advection!(phi, dt, t, cache, boreholes), src/solver.jl:250-264 */
int gw_advection(gw_ctx *ctx, double *phi_dev, double dt, double t);
/* ADI_and_ADV_callback!(integrator), src/solver.jl:432-464: u = integrator.u,
 * temp = integrator.uprev (clobbered), t = integrator.t, dt = t - tprev. */
int gw_adi_adv(gw_ctx *ctx, double *u_dev, double *temp_dev, double t, double dt);

/* Inlet temperature schedule of a GW_INLET_SCHEDULE context (or the schedule
 * a GW_INLET_EXPRESSION program reads with GW_OP_SCHED): T_in(t) linear
 * between the n points (times strictly increasing), held constant before the
 * first and after the last.  Evaluated where the reference calls
 * inlet_model(bh, T_outlet, t) (src/solver.jl:349-350): at the step's end time
 * in the first advection and half a step later in the second. */
int gw_set_inlet_schedule(gw_ctx *ctx, int n, const double *times, const double *values);

/* Inlet program of a GW_INLET_EXPRESSION context: a postfix sequence of n
 * operations (n <= GW_PROGRAM_MAX) evaluated for every borehole wherever the
 * reference calls inlet_model(bh, T_outlet, t) (src/solver.jl:349-350), each
 * operation one correctly rounded double operation.  Operands go on a stack
 * (depth <= 16); the program must leave exactly one value, the inlet
 * temperature.  GW_OP_SCHED reads the context's schedule
 * (gw_set_inlet_schedule, which GW_INLET_EXPRESSION contexts also take).
 * Example, T_in = max(5, T_out - dT(t)):
 *   CONST 5, TOUT, TIME, SCHED, SUB, MAX. */
#define GW_PROGRAM_MAX 64
#define GW_OP_CONST 0   /* push args[i] */
#define GW_OP_TOUT 1    /* push T_outlet of the borehole (cache.T_outlet[bh]) */
#define GW_OP_TIME 2    /* push t */
#define GW_OP_BH 3      /* push the borehole index (0-based) */
#define GW_OP_SCHED 4   /* x -> schedule(x) */
#define GW_OP_NEG 5     /* x -> -x */
#define GW_OP_ADD 6     /* a b -> a + b */
#define GW_OP_SUB 7     /* a b -> a - b */
#define GW_OP_MUL 8     /* a b -> a * b */
#define GW_OP_DIV 9     /* a b -> a / b */
#define GW_OP_MIN 10    /* a b -> min(a, b) */
#define GW_OP_MAX 11    /* a b -> max(a, b) */
int gw_set_inlet_program(gw_ctx *ctx, int n, const int *ops, const double *args);

/* dst = sum_i coeffs[i] * srcs[i] over the context's N = nx*ny*nz cells, n <= 8
 * device fields (dst may be one of them).  The vector updates an ODE
 * integrator's stages make (the `@..` broadcasts of ROCK2's perform_step!)
 * for callers that hold the state on the device and use no other GPU
 * library. */
int gw_lincomb(gw_ctx *ctx, double *dst_dev, int n, const double *coeffs,
               const double *const *srcs_dev);

/* ---- fused step on the context's own state ---- */
/* Advance u by nsteps fixed steps of size dt from time t0: per step one
 * ROCK2 step of rhs_diffusion_z! (stage count from the eigenvalue estimate,
 * src/solver.jl:495, capped at max_stages) then ADI_and_ADV_callback!.  The
 * step is captured once in CUDA graphs (of one step, and of eight for calls
 * of at least eight steps) and replayed.  Records the outlet
 * temperature and extracted heat after every step.  When the step runs its
 * pipe passes on a second stream (gw_info_t.overlap), the first call for a
 * new step size (or after a setter) times the step's two launch orders on 64
 * trial steps, restores the field, outlet and energy values, and keeps the
 * faster order (gw_info_t.step_order); both give the same state bitwise. */
int gw_step(gw_ctx *ctx, double t0, double dt, int nsteps, int max_stages);
/* Run the step's two pipe passes (and the x-lines through the pipes) on a
 * second stream, overlapping the rest of the step (on = 1; the default where
 * the rows holding pipe columns are at most half of the domain), or in line
 * (on = 0).  Both give bitwise identical results.  gw_get_info reports the
 * setting (overlap). */
int gw_set_overlap(gw_ctx *ctx, int on);
/* Options of the mixed step (GW_PREC_MIXED contexts; 0 = the default form):
 *  GW_MIXED_ROCK2_F64  ROCK2 stages accumulated in double over the float
 *                      field, rounded into it once per step (the FP64 pipe
 *                      makes the column kernel several times slower);
 *  GW_MIXED_REFINE     after each float line solve, the residual of the
 *                      half step's equation in double and one correction
 *                      solve (a second pass over the field per half step).
 * No counterpart in the reference, which runs in one precision. */
#define GW_MIXED_ROCK2_F64 1
#define GW_MIXED_REFINE 2
int gw_set_mixed_options(gw_ctx *ctx, int flags);

/* Half-step kernel of this context (0 .. GW_TILINGS-1, see GW_TILINGS); all
 * give the same field bitwise except the segmented tiling 6.  gw_create picks
 * 0, except for mixed contexts whose half steps of tiling 0 would keep their
 * forward values in global memory (fewer than four rounds of blocks per
 * half step): those start with 9 (8 lines x 8 rows, global memory).
 * gw_get_info reports the setting (tiling). */
int gw_set_tiling(gw_ctx *ctx, int tiling);
/* Stage count gw_step uses for dt (and whether its interval covers dt*lambda). */
int gw_rock2_stages(gw_ctx *ctx, double dt, int max_stages, int *stages, int *covered);

/* ---- snapshots: asynchronous float copies of the state ----
 * save_and_print_callback's SavingCallback (src/cache.jl:132-184) copies u to
 * the host at every saveat time and keeps it as Float32.  gw_snapshot
 * converts the context's u to float temperatures on the device and starts
 * the copy into host_dst (N floats, (k, j, i) order) on a second stream; it
 * returns once the conversion is done (a fraction of a step) without waiting
 * for the copy, which overlaps the gw_step calls that follow.  host_dst must
 * stay untouched until gw_snapshot_wait returns.  Two device staging buffers
 * alternate; a third snapshot started before the first copy has landed makes
 * the device (not the host) wait for it.  The overlap needs pinned host
 * memory (gw_snapshot_host_alloc); with pageable memory the copy completes
 * before gw_snapshot returns. */
int gw_snapshot_host_alloc(gw_ctx *ctx, float **host);
int gw_snapshot_host_free(gw_ctx *ctx, float *host);
int gw_snapshot(gw_ctx *ctx, float *host_dst);
int gw_snapshot_wait(gw_ctx *ctx);

/* cache.T_outlet after the last advection (src/solver.jl:253-257). */
int gw_get_outlet(gw_ctx *ctx, double *T_outlet);
/* Outlet temperature after each of the last gw_step call's steps, nsteps x nbh. */
int gw_get_outlet_series(gw_ctx *ctx, double *T_series, int nsteps);
/* Extracted heat per borehole integrated over all gw_step steps so far [J]:
 * sum over steps of mdot * c_w * (T_outlet - T_inlet) * dt, c_w = rho_c_water / 998.2. */
int gw_get_energy(gw_ctx *ctx, double *E);
int gw_reset_energy(gw_ctx *ctx);
/* GW_ERR_NONFINITE if the context's u holds a NaN or Inf. */
int gw_check_finite(gw_ctx *ctx);

/* Device time of the last gw_step call's replay loop [ms], from CUDA events
 * recorded on the context's stream around the graph launches. */
int gw_get_last_step_time(gw_ctx *ctx, double *ms);

/* Kernel timing for the roofline: runs each kernel class of the fused step
 * of size dt (in the context's precision) `reps` times on the context's
 * buffers (the state u is restored afterwards) and writes the mean device
 * time per launch [ms] into ms_out[GW_KERNEL_COUNT], indexed by GW_KERNEL_*.
 * Each launch is bracketed by CUDA events on the context's stream. */
#define GW_KERNEL_ROCK2 0      /* all ROCK2 stages of the z-diffusion, whole columns */
#define GW_KERNEL_HALF_X 1     /* explicit y-sweep + pipe values + x-line Thomas */
#define GW_KERNEL_HALF_Y 2     /* explicit x-sweep + pipe values + y-line Thomas */
#define GW_KERNEL_PIPE 3       /* pipe columns: sweep, outlet/annulus means, advection */
#define GW_KERNEL_COUNT 4
int gw_profile_kernels(gw_ctx *ctx, double dt, int reps, double *ms_out);

/* ---- ensembles: many well designs advanced together ---- */
/* Configuration 4 of the benchmark set (no single counterpart in the
 * reference, which runs one cache per solve): a batch advances the contexts
 * of many designs -- each created by gw_create with GW_PREC_MIXED or
 * GW_PREC_FP64 on one device -- with CUDA-graph launches of 32 steps (one
 * step for the remainder) in which the designs' fused steps run
 * concurrently.  The contexts stay owned
 * by the caller and must outlive the batch; per-design state, outlet series
 * and energies are read with the single-context getters. */
typedef struct gw_batch gw_batch;
#define GW_TILINGS 13  /* half-step kernels: 0-5 row tiles (lines per block, rows per chunk)
                          of the mixed path keeping the forward-elimination values in tensor
                          memory where the block's lines fit (blocks of 4 or 8 lines, lines
                          of up to 512 / 256 rows); 6 lines split into register-resident
                          segments; 7-12 the row tiles of 0-5 with the forward values in
                          global memory (more resident blocks per SM, which pays when many
                          designs run at once).  FP64 contexts: 7-12 are 0-5. */
int gw_batch_create(gw_ctx *const *ctxs, int n, gw_batch **out);
int gw_batch_destroy(gw_batch *batch);
/* Use one tiling (0 .. GW_TILINGS-1) for every design (0 is the default). */
int gw_batch_set_tiling(gw_batch *batch, int tiling);
/* Pick the half-step tiling of every design: each design's fastest tiling
 * alone (`reps` timed launches), then the real concurrent ensemble step
 * timed for every uniform tiling and for those per-design choices; the
 * fastest assignment is kept (tiling_out[n]).  The designs' states, outlet
 * and energy values are restored afterwards. */
int gw_batch_autotune(gw_batch *batch, double dt, int reps, int *tiling_out);
/* nsteps fixed steps of size dt for every design (as gw_step per context). */
int gw_batch_step(gw_batch *batch, double dt, int nsteps, int max_stages);
int gw_batch_get_last_step_time(gw_batch *batch, double *ms);

/* Batched independent tridiagonal solves A_s x_s = d_s (the elimination of
 * thomas_I_minus_A!, src/solver.jl:207-218, on arbitrary systems), all
 * arrays on the device in the grouped interleaved layout: systems sorted by
 * length in groups of 32; row r of the group's lane l at
 * group_off[g] + 32 r + l; group_len[g] rows per group (shorter systems
 * padded with identity rows, a_0 = 0 and c_{len-1} = 0).  n_elements = total
 * stored rows * 32.  precision GW_PREC_FP64: double elimination, scratch of
 * 8 * n_elements bytes; GW_PREC_MIXED: float elimination plus one residual
 * correction (residual in double), scratch of 12 * n_elements bytes.  stream
 * is a cudaStream_t (NULL: the default stream); returns when done. */
int gw_tridiag_batch(int precision, int ngroups, const long long *group_off, const int *group_len,
                     const double *a, const double *b, const double *c, const double *d,
                     double *x, void *scratch, long long n_elements, void *stream);

/* advection! (same result as gw_advection) for callers that must not make
 * the library allocate device memory.  No counterpart in the reference.
 *
 * Who needs it: a host integrator that owns every device buffer itself --
 * e.g. a Julia caller whose arrays come from its own pool allocator and must
 * keep the device footprint fixed after set-up, or a process that reserves
 * its share of a GPU shared with other jobs once at start-up and may not
 * grow it during the run.  This entry point calls no cudaMalloc, cudaFree or
 * allocating library routine, and waits for its own work on the context's
 * stream before it returns.
 *
 * Its scratch (outlet means and per-level annulus means) lives in one
 * file-scope device array of 65536 doubles (512 KiB) that every GPU which
 * loads the library holds until the process exits; each pipe column is
 * advected inside one thread block's shared memory, so no column buffer is
 * needed.  Limits: n_boreholes * (nz + 1) <= 65536 and at most 12288 levels
 * at or above the deepest borehole bottom; larger problems get GW_ERR_ARG.
 * T_outlet_dev (device, n_boreholes doubles) receives cache.T_outlet.
 *
 * The first call on a device looks up the array's device address and sets
 * the kernel's shared-memory limit for that device; make that first call
 * before any stream capture.  All calls share the one array (every value a
 * call reads is first written by the same call, so nothing needs clearing
 * between calls); calls that overlap on the GPU -- from two contexts or two
 * threads at once -- race on it and must be serialised by the caller. */
int gw_advection_noalloc(gw_ctx *ctx, double *phi_dev, double dt, double t, double *T_outlet_dev);

/* ---- adjoint: reverse-mode gradients of the time-step map ----
 * No counterpart in the reference, which has no derivatives: these are the
 * kernels a ChainRulesCore rrule over the solve (the Julia side of a
 * torch.autograd.Function) calls.  GW_PREC_FP64 contexts run it in double;
 * GW_PREC_MIXED contexts keep float adjoint fields over the float states of
 * the mixed step (gradient sums in double). 
 *
 * Objective over the steps n = 0 .. nsteps-1 of size dt:
 *   J = sum_b [ w_energy * E_b + w_outlet * T_out,b(last step) ],
 *   E_b = sum_n mdot_b c_w (T_out,b^n - T_in,b^n) dt   (as gw_get_energy).
 * Parameters, in this order in grad[]:
 *   k_rock_layers[0 .. n_layers-1], mdot[0 .. n_boreholes-1], inlet_param
 *   (T_const of the constant inlet, or dT of the heat-exchanger inlet).
 * The derivative holds the branch structure of the advection fixed (which
 * cells turn around or take the inlet value, the outlet window's levels),
 * as the derivative of a piecewise map does. */
typedef struct {
    double objective;      /* J */
    int n_params;          /* n_layers + n_boreholes + 1 */
    int stages;            /* ROCK2 stages per step */
    int checkpoints;       /* states kept by the forward sweep */
    double forward_ms;     /* forward sweep with checkpoints, device time */
    double reverse_ms;     /* recomputation + reverse sweep, device time */
    long long peak_bytes;  /* device memory held during the call: context + adjoint */
} gw_adjoint_info_t;

/* Gradient of J over nsteps steps from the context's current field u^0.
 * The forward sweep keeps u every checkpoint_every steps; the reverse sweep
 * recomputes each segment's states and each step's intermediates.  grad
 * receives n_params values; grad_T0_dev (device, N doubles, may be NULL)
 * receives dJ/du^0.  Afterwards the context's field, outlet and energy are
 * as after gw_step(ctx, 0, dt, nsteps, max_stages). */
int gw_adjoint(gw_ctx *ctx, double dt, int nsteps, int max_stages, int checkpoint_every,
               double w_energy, double w_outlet, double *grad, double *grad_T0_dev,
               gw_adjoint_info_t *info);

/* One step's vector-Jacobian product: with u_dev = u^n and lam_dev =
 * dJ/du^{n+1} on entry, lam_dev = dJ/du^n on return, where J includes this
 * step's objective terms (w_energy * its energy, w_outlet * its outlet
 * temperature); grad[n_params] is accumulated into (+=).  The context's
 * field is not touched.  For callers that drive the time loop themselves;
 * double fields, GW_PREC_FP64 contexts. */
int gw_step_vjp(gw_ctx *ctx, const double *u_dev, double *lam_dev, double dt, int max_stages,
                double w_energy, double w_outlet, double *grad);

#ifdef __cplusplus
}
#endif
#endif /* GW_GB300_H */
