// gw_internal.h -- device context and kernel launch interface shared by the
// translation units of libgw_gb300.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <string>
#include <vector>

#include "../../include/gw_gb300.h"

// Borehole record with the derived values of src/physics.jl:48-59.
struct GwBorehole {
    double xc, yc, h, r_inner, t_inner, r_and_t_inner_sq, r_outer, r_outer_sq;
    double t_outer, r_and_t_outer_sq, r_backfill, r_backfill_sq, mdot;
    double v_inner, v_outer, insulation_depth;
};

// One departure record of the semi-Lagrangian advection (see k_adv_table):
// per (borehole, level, inner pipe / annulus), for a half step.
enum : int { kAdvKeep = 0, kAdvInterp = 1, kAdvTurn = 2, kAdvInlet = 3 };
struct GwAdvRec {
    double alpha;
    double dref;   // mixed path: alpha T_ref(ir) + (1 - alpha) T_ref(il) - T_ref(k)
    int il, ir, type, pad;
};

// Per-borehole data the advection kernels read (one small device array).
struct GwBhDev {
    double h, v_inner, v_outer, mdot;
    int inner_begin, inner_count;   // range in the pipe-column list
    int outer_begin, outer_count;
};

// Thomas factorisation of one direction's (I - h A) lines, per (zclass, line, row):
//   forward  y_l = (b_l - a_l * y_{l-1}) * ib_l
//   backward x_l = y_l - cu_l * x_{l+1}
template <typename T>
struct GwFactors {
    T *a = nullptr, *ib = nullptr, *cu = nullptr;
};

template <typename T>
struct GwCoefTables {
    // x: [zc][j][i], y: [zc][i][j] (row index fastest); z: [profile][k]
    T *cxm = nullptr, *cxp = nullptr, *cym = nullptr, *cyp = nullptr;
    T *czm = nullptr, *czp = nullptr;
    GwFactors<T> fx, fy;   // for h = dt/2 of the current step size
    // fused half steps, per (zc, line, row) of x-lines (hx) and y-lines (hy):
    // 4 values {e0, ep, em, a} * ib folding the explicit sweep of the other
    // direction into the forward elimination (see gw_build_half_tables)
    T *hx = nullptr, *hy = nullptr;
};

struct gw_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    int nx = 0, ny = 0, nz = 0, nbh = 0, precision = GW_PREC_FP64;
    std::vector<double> gx, gy, gz;
    std::vector<GwBorehole> bh;
    // materials (one-layer stratified == homogeneous)
    std::vector<double> k_layers, rhoc_layers, depths;
    double k_water, rho_c_water, k_steel, rho_c_steel, k_insulating, rho_c_insulating;
    double k_backfill, rho_c_backfill;
    int inlet_kind = 0;
    double inlet_param = 0.0;
    // GW_INLET_SCHEDULE: T_in(t) piecewise linear; d_sched = times then values
    std::vector<double> sched_t, sched_T;
    double *d_sched = nullptr;
    int n_sched = 0;
    // GW_INLET_EXPRESSION: the inlet program (gw_set_inlet_program)
    std::vector<int> prog_op;
    std::vector<double> prog_arg;
    int *d_prog_op = nullptr;
    double *d_prog_arg = nullptr;
    int n_prog = 0;
    bool prog_sched = false;          // the program reads the schedule
    double *d_time = nullptr;         // [2]: start time of the current gw_step call, dt
    double *d_inlet = nullptr;        // [nbh]: inlet value of the last pipe pass
    double t_now = 0.0;               // end time of the last step taken
    double eigen_estimate = 0.0;

    // host-side material model
    int n_zclass = 0, n_profiles = 0;
    std::vector<int> zclass;          // [nz]
    std::vector<int> colprof;         // [nx*ny] (i*ny + j)
    int n_inner = 0, n_outer = 0, countz = 0;
    std::vector<int> pipe_i, pipe_j, pipe_b;   // inner list then outer list

    // device: grids, tables, lists
    double *d_gz = nullptr;
    int *d_zclass = nullptr, *d_colprof = nullptr;
    int *d_colorder = nullptr;        // columns sorted by profile
    // Overlap of the pipe passes with the bulk of the step: the rows jlo..jhi
    // hold every pipe column; d_colorder_ab lists the columns of rows
    // jlo-1..jhi+1 (ncol_a, the ones the pipe passes and the x-lines through
    // the pipes read) and then the rest (ncol_b), each sorted by profile.
    int *d_colorder_ab = nullptr;
    int ncol_a = 0, ncol_b = 0, jlo = -1, jhi = -1;
    int ncol_p = 0;   // of the ncol_a: the pipe columns and their y-neighbours, first
    int step_order = 0;           // launch order of the overlapped step (0 / 1, gw_fused.cu fused_step)
    int step_order_fixed = -1;    // -1: chosen by timing when gw_step captures a new graph
    int ilo = -1, ihi = -1;           // columns (i) holding pipe columns
    bool overlap = false;
    cudaStream_t stream2 = nullptr;   // the pipe passes' stream inside the step graph
    cudaEvent_t ev_a = nullptr, ev_px = nullptr, ev_p = nullptr, ev_q = nullptr;
    int *d_pipe_i = nullptr, *d_pipe_j = nullptr, *d_pipe_b = nullptr;
    GwBhDev *d_bh = nullptr;
    GwCoefTables<double> c64;
    GwCoefTables<float> c32;
    double factors_h = -1.0;          // h for which c64.fx/fy (and c32) are valid

    // device state and scratch (double path)
    double *d_u = nullptr, *d_temp = nullptr, *d_g1 = nullptr, *d_g2 = nullptr;
    double *d_utmp = nullptr;         // [ncol][countz] (k fastest)
    double *d_annmean = nullptr;      // [nbh][nz]
    double *d_outlet = nullptr;       // [nbh]
    double *d_energy = nullptr;       // [nbh]
    double *d_series = nullptr;       // [series_cap][nbh]
    int *d_step_counter = nullptr;
    int *d_flag = nullptr;
    int series_cap = 0;
    int last_nsteps = 0;
    // fused step (both precisions)
    int *d_pipe_of = nullptr;         // [nx*ny] pipe-column index or -1
    int *d_pipe_lx = nullptr;         // [ny][nx] pipe index along x-lines (j, i), then [ny] line flags
    int *d_pipe_ly = nullptr;         // [nx][ny] pipe index along y-lines (i, j), then [nx] line flags
    int4 *d_pipe_chunks = nullptr;    // pipe-column chunks: (borehole, q0, q1, outer)
    int *d_bchunk = nullptr;          // [nbh][4]: chunk ranges (inner, outer) per borehole
    double *d_pipepart = nullptr;     // [chunk][nz] column sums of the swept pipe values
    int n_pipe_chunks = 0;
    GwAdvRec *d_advtab = nullptr;     // [nbh][countz][2] departure table for dt/2
    int *d_nlev = nullptr;            // [nbh] outlet window of that step size: levels with z <= v_inner dt/2
    double *d_stage = nullptr;        // ROCK2 stage coefficients of the captured step
    float *f_stage = nullptr;         // the same, rounded to float (mixed path)
    double *d_tp = nullptr;           // double path: [ncol][nz] swept pipe columns
    double *d_pp = nullptr;           // double path: [ncol][countz] advected pipe values
    int rock2_grid = 0;
    int rock2_nt = 256;               // threads per block of the ROCK2 column kernel
    int sms = 0;                      // multiprocessors of the context's GPU
    int pz = 0;                       // level pitch of the fused fields: nz (FP64), nz rounded up to 4 (mixed)
    // mixed path: 3-D tensor maps of the half-step tiles, [source: f_u, f_temp][x-, y-lines][tiling]
    CUtensorMap tmaps[2][2][6];
    CUtensorMap qmaps[2][6];          // their row-coefficient quads, [x-, y-lines][tiling]
    bool tma_ok = false;              // maps encoded (else the half step copies with cp.async)
    bool half_tmem = false;           // tensor-map half steps keep their forward values in TMEM
    bool half_split = false;          // ... rows beyond 128 in shared memory where that runs more blocks
    bool half_tm_force = false;       // ... also for half steps of fewer than four rounds of blocks
    int smem_per_sm = 0;              // shared memory per SM (bytes)
    int *d_err = nullptr;             // set by a kernel whose bounded wait ran out
    int rock2w_per_sm[9] = {};        // resident blocks per SM of the window ROCK2 kernel, by LPT
    bool rock2_block = false;         // mixed ROCK2 on the block kernel (GW_ROCK2_BLOCK), not by windows
    bool refine_f64 = false;          // GW_MIXED_REFINE residual in double (GW_REFINE_F64), not double-float
    float4 *f_rq[2] = {nullptr, nullptr};   // refinement tables per direction (x, y): h c_m, h c_p as double-float
    float2 *f_rg[2] = {nullptr, nullptr};   //   and 1 + h (c_m + c_p)
    double rq_h = -1.0;               // step size those tables hold
    int half_cfg = 0;                 // half-step tiling (gw_fused.cu kTileHW/kTileHR)
    bool fused = false;
    bool host_setup = false;          // tables built on the host (GW_HOST_SETUP), else on the GPU
    int modular_reason = 0;           // GW_MODULAR_* bits when !fused
    // mixed path state (GW_PREC_MIXED): theta = T - T_ref(z) in float
    float *f_u = nullptr, *f_temp = nullptr, *f_g1 = nullptr, *f_tp = nullptr, *f_pp = nullptr;
    float *f_fref = nullptr;          // [profile][nz] A_z T_ref
    double *d_fref64 = nullptr;       // the same in double (FP64 ROCK2 stage accumulation)
    int mixed_flags = 0;              // GW_MIXED_* options of the mixed step
    int rock2_nt64 = 0, rock2_grid64 = 0;   // column kernel with double stages over float storage
    double *d_Tref = nullptr;         // [nz]
    std::vector<double> Tref;         // host copy
    std::vector<double> h_czm, h_czp; // host copies of the z coefficients

    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    double last_step_ms = 0.0;
    // asynchronous snapshots (gw_snapshot): two float staging buffers, the
    // copy stream and per-buffer events (converted, copied)
    float *d_snap[2] = {nullptr, nullptr};
    cudaStream_t snap_stream = nullptr;
    cudaEvent_t ev_conv[2] = {nullptr, nullptr}, ev_copy[2] = {nullptr, nullptr};
    bool snap_pending[2] = {false, false};
    int snap_next = 0;
    // graph cache for gw_step
    cudaGraphExec_t graph = nullptr;
    cudaGraphExec_t graph_k = nullptr;   // several steps per launch (calls of at least that many)
    double graph_dt = -1.0;
    int graph_s = -1;
    int graph_gen = -1;               // series_gen the graph was captured with
    int series_gen = 0;               // bumped when d_series is reallocated
    double tables_dt = -1.0;          // step size of the loaded stage/advection tables
    int tables_s = -1;

    long long device_bytes = 0;
    std::vector<void *> allocations;
    struct GwAdj *adj = nullptr;      // adjoint tables (gw_adjoint.cu), built on first use
};

// debug build (GW_DEBUG): device allocations registered for the kernels'
// bounds checks (gw_debug.cuh); no-ops in the normal build
void gw_debug_register(int device, const void *p, size_t bytes);
void gw_debug_unregister(int device, const void *p);
// GW_ERR_ARG if a bounds check failed since the last call (and clears it)
int gw_debug_status(int device);

// error reporting
// slots of one fused-step field: nx ny columns, pz apart
inline size_t gw_field_slots(const gw_ctx *c) { return (size_t)c->nx * c->ny * c->pz; }
int gw_dalloc_f(gw_ctx *c, float **p, size_t n);
int gw_fail(int code, const std::string &msg);
int gw_cuda_fail(cudaError_t e, const char *what);
#define GW_CUDA(call)                                                    \
    do {                                                                 \
        cudaError_t _e = (call);                                         \
        if (_e != cudaSuccess) return gw_cuda_fail(_e, #call);           \
    } while (0)

// setup (gw_setup.cpp)
int gw_setup_host(gw_ctx *c, const gw_desc *d);
void gw_build_profiles(gw_ctx *c);   // host path of the column profiles
void gw_build_coefs(const gw_ctx *c, std::vector<double> &cxm, std::vector<double> &cxp,
                    std::vector<double> &cym, std::vector<double> &cyp,
                    std::vector<double> &czm, std::vector<double> &czp);
void gw_build_factors(const gw_ctx *c, double h, int dir, const std::vector<double> &cm,
                      const std::vector<double> &cp, std::vector<double> &a,
                      std::vector<double> &ib, std::vector<double> &cu);
void gw_build_half_table(const gw_ctx *c, double h, int dir, const std::vector<double> &ecm,
                         const std::vector<double> &ecp, const std::vector<double> &a,
                         const std::vector<double> &ib, std::vector<double> &out4);
void gw_build_adjoint_tables(const gw_ctx *c, std::vector<double> &wxm, std::vector<double> &wxp,
                             std::vector<double> &wym, std::vector<double> &wyp,
                             std::vector<double> &wzm, std::vector<double> &wzp,
                             std::vector<unsigned char> &rock, std::vector<int> &layer);
void gw_adjoint_release(gw_ctx *c);
// gw_setup_dev.cu: column profiles, coefficient tables (c64, owned by the
// context; cx/cy/cz receive the (m, p) pointers), Thomas factors and half
// tables on the GPU, bitwise the host builders' values.
int gw_setup_tables_device(gw_ctx *c, double **cx, double **cy, double **cz);
int gw_tables_to_float(gw_ctx *c, float *dst, const double *src, size_t n);
int gw_factors_device(gw_ctx *c, double h);
int gw_rock2_choose(double dt, double eigen_est, int max_stages, int *s, int *covered);
void gw_rock2_coefs(int s, const double **mu, const double **nu, const double **kappa,
                    double *sigma, double *tau);

// launches (gw_kernels.cu); all enqueue on c->stream
int gw_launch_zstage(gw_ctx *c, double *out, const double *x, const double *y, double hmu,
                     double kap, int rhs_only);
int gw_launch_explicit(gw_ctx *c, double *dst, const double *src, double h, int dir);
int gw_launch_thomas(gw_ctx *c, double *U, const double *RHS, int dir);
int gw_launch_advection(gw_ctx *c, double *phi, double dt, double t = 0.0);
// T_in(t) of the context's schedule (host); the same formula as the device.
double gw_schedule_at(const gw_ctx *c, double t);
// on stream st (NULL: the context's stream)
int gw_launch_record(gw_ctx *c, double dt, cudaStream_t st = nullptr);
int gw_launch_check_finite(gw_ctx *c, const double *u, size_t n);
int gw_launch_lincomb(gw_ctx *c, double *dst, int n, const double *w, const double *const *src);
// u = col[k] in every column (col: nz device doubles)
int gw_launch_broadcast_column(gw_ctx *c, double *u, const double *col);
// dst = float(T) of the context's state (theta + T_ref in the mixed path)
int gw_launch_snapshot(gw_ctx *c, float *dst);
int gw_ensure_factors(gw_ctx *c, double h);
int gw_set_step_time(gw_ctx *c, double t0, double dt);
int gw_prepare_step(gw_ctx *c, double dt, int s, int nsteps);

#define GW_STAGE_TABLE 208   // doubles: 2 per recurrence stage (<= 98) + 3
