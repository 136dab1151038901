/*
 * gw_oracle.c -- CPU FP64 restatement of the GeothermalWells.jl time-step
 * hot path.  TEST INFRASTRUCTURE ONLY: the parity tests, the smoke check and
 * the CPU-baseline leg of the benchmark use it as the checker.  Nothing in
 * the product links or calls it.
 *
 * It follows the reference operation by operation (file:line cited per
 * function), including its O(N_inner * N_outer) turnaround mean and its
 * per-cell material lookups, so it is also the timed CPU baseline.  Where the
 * reference's @muladd turns `a*b + c` into a fused multiply-add, fma() is
 * used, so that the branch decisions of the semi-Lagrangian advection
 * (departure point vs. h, vs. 0) round as on FMA hardware.
 *
 * Build: see oracle/Makefile (plain gcc, OpenMP, -ffp-contract=off so the
 * results are identical on x86-64 and aarch64).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct {
    /* src/physics.jl:30-61 (Borehole fields, derived values as in 48-59) */
    double xc, yc, h, r_inner, t_inner, r_and_t_inner_sq, r_outer, r_outer_sq;
    double t_outer, r_and_t_outer_sq, r_backfill, r_backfill_sq, mdot;
    double v_inner, v_outer, insulation_depth;
} obh_t;

typedef struct {
    int nx, ny, nz;
    double *gx, *gy, *gz;
    int nbh;
    obh_t *bh;
    /* materials: stratified rock (homogeneous == one layer), physics.jl:81-125,159-175 */
    int nlayers;
    double *k_layers, *rhoc_layers, *depths;
    double k_water, rho_c_water, k_steel, rho_c_steel;
    double k_insulating, rho_c_insulating, k_backfill, rho_c_backfill;
    int inlet_kind;      /* 0 = ConstantInlet, 1 = HeatExchangerInlet, 2 = schedule T_in(t) */
    double inlet_param;  /* T_const or DeltaT */
    int sched_n;         /* kind 2: piecewise-linear T_in(t), constant outside the points */
    double *sched_t, *sched_T;
    /* advection index lists, cache.jl:9-44 (0-based i, j, bh) */
    int n_inner, n_outer, countz;
    int *idx;            /* 3 * (n_inner + n_outer): inner list then outer list */
    unsigned char *last; /* 1 where entry q is the last one of its (i, j) column */
    int prog_n;          /* kind 3: inlet program, postfix GW_OP_* codes and constants */
    int *prog_op;
    double *prog_arg;
    double *u_tmp;       /* (n_inner + n_outer) x countz, ij fastest (cache.jl:41) */
    double *T_outlet;    /* nbh */
    long *T_outlet_counter;
} octx_t;

#define IDX(c, k, j, i) ((size_t)(k) + (size_t)(c)->nz * ((size_t)(j) + (size_t)(c)->ny * (size_t)(i)))

/* physics.jl:102-110 / 117-125 (and the homogeneous dispatch 173-175) */
static double rock_k(const octx_t *c, double z) {
    for (int i = 0; i < c->nlayers; ++i)
        if (z <= c->depths[i]) return c->k_layers[i];
    return c->k_layers[c->nlayers - 1];
}
static double rock_rhoc(const octx_t *c, double z) {
    for (int i = 0; i < c->nlayers; ++i)
        if (z <= c->depths[i]) return c->rhoc_layers[i];
    return c->rhoc_layers[c->nlayers - 1];
}

/* physics.jl:199-233 get_thermal_conductivity */
static double mat_k(const octx_t *c, double x, double y, double z) {
    double k = rock_k(c, z);
    for (int b = 0; b < c->nbh; ++b) {
        const obh_t *bh = &c->bh[b];
        double dx = x - bh->xc, dy = y - bh->yc;
        double r_sq = dx * dx + dy * dy;
        if (r_sq > bh->r_backfill_sq) continue;
        if (z <= bh->h) {
            if (r_sq < bh->r_inner * bh->r_inner) k = c->k_water;
            else if (r_sq < bh->r_and_t_inner_sq) k = c->k_insulating;
            else if (r_sq < bh->r_outer_sq) k = c->k_water;
            else if (r_sq < bh->r_and_t_outer_sq) k = (z <= bh->insulation_depth) ? c->k_insulating : c->k_steel;
            else k = c->k_backfill;
        } else if (z <= bh->h + 3) {
            k = c->k_steel;
        }
    }
    return k;
}

/* physics.jl:243-274 get_volumetric_heat_capacity */
static double mat_rhoc(const octx_t *c, double x, double y, double z) {
    double rc = rock_rhoc(c, z);
    for (int b = 0; b < c->nbh; ++b) {
        const obh_t *bh = &c->bh[b];
        double dx = x - bh->xc, dy = y - bh->yc;
        double r_sq = dx * dx + dy * dy;
        if (r_sq > bh->r_and_t_outer_sq) continue;
        if (z <= bh->h) {
            if (r_sq < bh->r_inner * bh->r_inner) rc = c->rho_c_water;
            else if (r_sq < bh->r_and_t_inner_sq) rc = c->rho_c_insulating;
            else if (r_sq < bh->r_outer_sq) rc = c->rho_c_water;
            else rc = (z <= bh->insulation_depth) ? c->rho_c_insulating : c->rho_c_steel;
        } else if (z <= bh->h + 3) {
            rc = c->rho_c_steel;
        }
    }
    return rc;
}

void ogw_destroy(void *h) {
    octx_t *c = (octx_t *)h;
    if (!c) return;
    free(c->gx); free(c->gy); free(c->gz); free(c->bh);
    free(c->k_layers); free(c->rhoc_layers); free(c->depths);
    free(c->idx); free(c->last); free(c->u_tmp); free(c->T_outlet); free(c->T_outlet_counter);
    free(c->sched_t); free(c->sched_T); free(c->prog_op); free(c->prog_arg);
    free(c);
}

/* bh10: per borehole xc, yc, h, r_inner, t_inner, r_outer, t_outer,
 * r_backfill, mdot, insulation_depth (the Borehole constructor arguments).
 * mat8: k_water, rho_c_water, k_steel, rho_c_steel, k_insulating,
 * rho_c_insulating, k_backfill, rho_c_backfill. */
void *ogw_create(int nx, int ny, int nz, const double *gx, const double *gy, const double *gz,
                 int nbh, const double *bh10, int nlayers, const double *k_layers,
                 const double *rhoc_layers, const double *depths, const double *mat8,
                 int inlet_kind, double inlet_param) {
    octx_t *c = (octx_t *)calloc(1, sizeof(octx_t));
    c->nx = nx; c->ny = ny; c->nz = nz;
    c->gx = (double *)malloc(sizeof(double) * nx); memcpy(c->gx, gx, sizeof(double) * nx);
    c->gy = (double *)malloc(sizeof(double) * ny); memcpy(c->gy, gy, sizeof(double) * ny);
    c->gz = (double *)malloc(sizeof(double) * nz); memcpy(c->gz, gz, sizeof(double) * nz);
    c->nbh = nbh;
    c->bh = (obh_t *)calloc(nbh, sizeof(obh_t));
    const double pi = 3.141592653589793;  /* Float64(pi) */
    for (int b = 0; b < nbh; ++b) {
        const double *p = bh10 + 10 * b;
        obh_t *o = &c->bh[b];
        /* physics.jl:48-59 */
        double rho_water = 998.2;
        o->xc = p[0]; o->yc = p[1]; o->h = p[2]; o->r_inner = p[3]; o->t_inner = p[4];
        o->r_outer = p[5]; o->t_outer = p[6]; o->r_backfill = p[7]; o->mdot = p[8];
        o->insulation_depth = p[9];
        double rti = o->r_inner + o->t_inner;
        o->r_and_t_inner_sq = rti * rti;
        o->r_outer_sq = o->r_outer * o->r_outer;
        double rto = o->r_outer + o->t_outer;
        o->r_and_t_outer_sq = rto * rto;
        o->r_backfill_sq = o->r_backfill * o->r_backfill;
        double A_inner = pi * (o->r_inner * o->r_inner);
        double A_outer = pi * o->r_outer_sq - pi * o->r_and_t_inner_sq;
        o->v_inner = o->mdot / (A_inner * rho_water);
        o->v_outer = o->mdot / (A_outer * rho_water);
    }
    c->nlayers = nlayers;
    c->k_layers = (double *)malloc(sizeof(double) * nlayers); memcpy(c->k_layers, k_layers, sizeof(double) * nlayers);
    c->rhoc_layers = (double *)malloc(sizeof(double) * nlayers); memcpy(c->rhoc_layers, rhoc_layers, sizeof(double) * nlayers);
    c->depths = (double *)malloc(sizeof(double) * nlayers); memcpy(c->depths, depths, sizeof(double) * nlayers);
    c->k_water = mat8[0]; c->rho_c_water = mat8[1]; c->k_steel = mat8[2]; c->rho_c_steel = mat8[3];
    c->k_insulating = mat8[4]; c->rho_c_insulating = mat8[5]; c->k_backfill = mat8[6]; c->rho_c_backfill = mat8[7];
    c->inlet_kind = inlet_kind; c->inlet_param = inlet_param;

    /* cache.jl:9-44 create_advection_index_lists */
    int cap = 1024, ni = 0, no = 0;
    int *inner = (int *)malloc(sizeof(int) * 3 * cap);
    int capo = 1024;
    int *outer = (int *)malloc(sizeof(int) * 3 * capo);
    for (int b = 0; b < nbh; ++b) {
        const obh_t *bh = &c->bh[b];
        for (int i = 0; i < nx; ++i)
            for (int j = 0; j < ny; ++j) {
                double dx = c->gx[i] - bh->xc, dy = c->gy[j] - bh->yc;
                double r_sq = dx * dx + dy * dy;
                double rti = bh->r_inner + bh->t_inner;
                if (r_sq < bh->r_inner * bh->r_inner) {
                    if (ni == cap) { cap *= 2; inner = (int *)realloc(inner, sizeof(int) * 3 * cap); }
                    inner[3 * ni] = i; inner[3 * ni + 1] = j; inner[3 * ni + 2] = b; ++ni;
                } else if (rti * rti <= r_sq && r_sq < bh->r_outer * bh->r_outer) {
                    if (no == capo) { capo *= 2; outer = (int *)realloc(outer, sizeof(int) * 3 * capo); }
                    outer[3 * no] = i; outer[3 * no + 1] = j; outer[3 * no + 2] = b; ++no;
                }
            }
    }
    c->n_inner = ni; c->n_outer = no;
    c->idx = (int *)malloc(sizeof(int) * 3 * (size_t)(ni + no + 1));
    memcpy(c->idx, inner, sizeof(int) * 3 * ni);
    memcpy(c->idx + 3 * ni, outer, sizeof(int) * 3 * no);
    free(inner); free(outer);
    /* boreholes whose pipes share a column list it more than once; the
     * reference's copy-back (solver.jl:391-396) then writes it from several
     * work items in parallel.  Restated deterministically, as a sequential
     * run of that loop leaves it: the later list entry wins. */
    c->last = (unsigned char *)malloc((size_t)(ni + no + 1));
    {
        int *lastq = (int *)malloc(sizeof(int) * (size_t)nx * ny);
        for (size_t e = 0; e < (size_t)nx * ny; ++e) lastq[e] = -1;
        for (int q = 0; q < ni + no; ++q) lastq[(size_t)c->idx[3 * q] * ny + c->idx[3 * q + 1]] = q;
        for (int q = 0; q < ni + no; ++q)
            c->last[q] = lastq[(size_t)c->idx[3 * q] * ny + c->idx[3 * q + 1]] == q;
        free(lastq);
    }
    double max_h = -INFINITY;
    for (int b = 0; b < nbh; ++b) if (c->bh[b].h > max_h) max_h = c->bh[b].h;
    int cz = 0;
    for (int k = 0; k < nz; ++k) if (c->gz[k] <= max_h) ++cz;
    c->countz = cz;
    c->u_tmp = (double *)calloc((size_t)(ni + no + 1) * (size_t)(cz + 1), sizeof(double));
    c->T_outlet = (double *)calloc(nbh, sizeof(double));
    c->T_outlet_counter = (long *)calloc(nbh, sizeof(long));
    return c;
}

void ogw_counts(void *h, int *out4) {
    octx_t *c = (octx_t *)h;
    out4[0] = c->n_inner; out4[1] = c->n_outer; out4[2] = c->countz; out4[3] = c->nbh;
}

void ogw_index_lists(void *h, int *out) {
    octx_t *c = (octx_t *)h;
    memcpy(out, c->idx, sizeof(int) * 3 * (size_t)(c->n_inner + c->n_outer));
}

void ogw_velocities(void *h, double *out2) {
    octx_t *c = (octx_t *)h;
    for (int b = 0; b < c->nbh; ++b) { out2[2 * b] = c->bh[b].v_inner; out2[2 * b + 1] = c->bh[b].v_outer; }
}

void ogw_material(void *h, double x, double y, double z, double *k, double *rhoc) {
    octx_t *c = (octx_t *)h;
    *k = mat_k(c, x, y, z);
    *rhoc = mat_rhoc(c, x, y, z);
}

/* solver.jl:474-488 eigen_estimator_pre_calculation with physics.jl:134-149 */
double ogw_eigen_estimate(void *h) {
    octx_t *c = (octx_t *)h;
    double dzmin = INFINITY;
    for (int k = 0; k + 1 < c->nz; ++k) { double d = c->gz[k + 1] - c->gz[k]; if (d < dzmin) dzmin = d; }
    double dmax = 0.0;
    for (int i = 0; i < c->nlayers; ++i) { double d = c->k_layers[i] / c->rhoc_layers[i]; if (d > dmax) dmax = d; }
    double cand[4] = {c->k_water / c->rho_c_water, c->k_steel / c->rho_c_steel,
                      c->k_insulating / c->rho_c_insulating, c->k_backfill / c->rho_c_backfill};
    for (int i = 0; i < 4; ++i) if (cand[i] > dmax) dmax = cand[i];
    return 8 * dmax / (dzmin * dzmin);
}

/* solver.jl:34-109 diffusion_1D! with idx_and_Δ_and_k_helper; dir 0=x,1=y,2=z */
void ogw_diffusion_1d(void *h, double *dphi, const double *phi, double dt, int dir, int plus_I) {
    octx_t *c = (octx_t *)h;
    const int nx = c->nx, ny = c->ny, nz = c->nz;
    const double half = 0.5;
#pragma omp parallel for schedule(static) collapse(2)
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j < ny; ++j)
            for (int k = 0; k < nz; ++k) {
                double x = c->gx[i], y = c->gy[j], z = c->gz[k];
                double rho_c = mat_rhoc(c, x, y, z);
                double k_center = mat_k(c, x, y, z);
                size_t ip, im;
                double dp, dm, kp, km;
                if (dir == 0) {
                    int ipl = (i == nx - 1) ? i : i + 1, imi = (i == 0) ? i : i - 1;
                    ip = IDX(c, k, j, ipl); im = IDX(c, k, j, imi);
                    dp = (i == nx - 1) ? (c->gx[i] - c->gx[i - 1]) : (c->gx[i + 1] - c->gx[i]);
                    dm = (i == 0) ? dp : (c->gx[i] - c->gx[i - 1]);
                    kp = mat_k(c, c->gx[ipl], y, z); km = mat_k(c, c->gx[imi], y, z);
                } else if (dir == 1) {
                    int jpl = (j == ny - 1) ? j : j + 1, jmi = (j == 0) ? j : j - 1;
                    ip = IDX(c, k, jpl, i); im = IDX(c, k, jmi, i);
                    dp = (j == ny - 1) ? (c->gy[j] - c->gy[j - 1]) : (c->gy[j + 1] - c->gy[j]);
                    dm = (j == 0) ? dp : (c->gy[j] - c->gy[j - 1]);
                    kp = mat_k(c, x, c->gy[jpl], z); km = mat_k(c, x, c->gy[jmi], z);
                } else {
                    int kpl = (k == nz - 1) ? k : k + 1, kmi = (k == 0) ? k : k - 1;
                    ip = IDX(c, kpl, j, i); im = IDX(c, kmi, j, i);
                    dp = (k == nz - 1) ? (c->gz[k] - c->gz[k - 1]) : (c->gz[k + 1] - c->gz[k]);
                    dm = (k == 0) ? dp : (c->gz[k] - c->gz[k - 1]);
                    kp = mat_k(c, x, y, c->gz[kpl]); km = mat_k(c, x, y, c->gz[kmi]);
                }
                double p = phi[IDX(c, k, j, i)];
                double val = (((kp + k_center) * half * (phi[ip] - p) / dp
                               - (k_center + km) * half * (p - phi[im]) / dm)
                              / ((dp + dm) * half)) / rho_c;
                dphi[IDX(c, k, j, i)] = plus_I ? fma(dt, val, p) : val;
            }
}

/* solver.jl:111-232 thomas_I_minus_A!; dir 0 = x-lines (U[k,ij,l]), 1 = y-lines (U[k,l,ij]) */
void ogw_thomas(void *h, double *U, const double *RHS, double dt, int dir) {
    octx_t *c = (octx_t *)h;
    const int N = dir == 0 ? c->nx : c->ny;
    const int nij = dir == 0 ? c->ny : c->nx;
    const double *grid = dir == 0 ? c->gx : c->gy;
    const double half = 0.5, one = 1.0;
#pragma omp parallel
    {
        double *b = (double *)malloc(sizeof(double) * N);
        double *lower = (double *)malloc(sizeof(double) * N);
        double *diag = (double *)malloc(sizeof(double) * N);
        double *upper = (double *)malloc(sizeof(double) * N);
#pragma omp for schedule(static) collapse(2)
        for (int ij = 0; ij < nij; ++ij)
            for (int k = 0; k < c->nz; ++k) {
                double z = c->gz[k];
#define PX(l) (dir == 0 ? grid[l] : c->gx[ij])
#define PY(l) (dir == 0 ? c->gy[ij] : grid[l])
#define SLOT(l) (dir == 0 ? IDX(c, k, ij, l) : IDX(c, k, l, ij))
                for (int l = 0; l < N; ++l) b[l] = RHS[SLOT(l)];
                double dp = grid[1] - grid[0];
                double rho_c = mat_rhoc(c, PX(0), PY(0), z);
                double kc = mat_k(c, PX(0), PY(0), z);
                double kp = mat_k(c, PX(1), PY(1), z);
                double factor_left = -dt * half * ((kc + kp) / rho_c) / (dp * dp);
                diag[0] = -factor_left + one;
                upper[0] = factor_left;
                for (int l = 1; l < N - 1; ++l) {
                    double dm = grid[l] - grid[l - 1];
                    dp = grid[l + 1] - grid[l];
                    double factor = -dt * 2 / (dm + dp);
                    rho_c = mat_rhoc(c, PX(l), PY(l), z);
                    double km = mat_k(c, PX(l - 1), PY(l - 1), z);
                    kc = mat_k(c, PX(l), PY(l), z);
                    kp = mat_k(c, PX(l + 1), PY(l + 1), z);
                    lower[l - 1] = factor * half * (kc + km) / (dm * rho_c);
                    diag[l] = fma(-factor, (half * (kc + kp) / (dp * rho_c) + half * (kc + km) / (dm * rho_c)), one);
                    upper[l] = factor * half * (kc + kp) / (dp * rho_c);
                }
                double dm = grid[N - 1] - grid[N - 2];
                rho_c = mat_rhoc(c, PX(N - 1), PY(N - 1), z);
                double km = mat_k(c, PX(N - 2), PY(N - 2), z);
                kc = mat_k(c, PX(N - 1), PY(N - 1), z);
                double factor_right = -dt * half * ((kc + km) / rho_c) / (dm * dm);
                lower[N - 2] = factor_right;
                diag[N - 1] = -factor_right + one;
                for (int l = 1; l < N; ++l) {
                    double w = lower[l - 1] / diag[l - 1];
                    diag[l] = fma(-w, upper[l - 1], diag[l]);
                    b[l] = fma(-w, b[l - 1], b[l]);
                }
                lower[N - 1] = b[N - 1] / diag[N - 1];
                for (int l = N - 2; l >= 0; --l)
                    lower[l] = fma(-upper[l], lower[l + 1], b[l]) / diag[l];
                for (int l = 0; l < N; ++l) U[SLOT(l)] = lower[l];
#undef PX
#undef PY
#undef SLOT
            }
        free(b); free(lower); free(diag); free(upper);
    }
}

/* solver.jl:379-389 gpu_searchsortedfirst (0-based: first index with arr[i] >= x) */
static int searchsortedfirst(const double *arr, double x, int lo, int hi) {
    while (lo < hi) {
        int mid = lo + (hi - lo) / 2;
        if (arr[mid] < x) lo = mid + 1; else hi = mid;
    }
    return lo;
}

/* solver.jl:362-376 interpolation_helper (0-based indices) */
static void interp_helper(const double *grid, int n, double dep, int *il, int *ir, double *alpha) {
    int r = searchsortedfirst(grid, dep, 0, n - 1);
    int l = r - 1;
    if (l < 0) l = 0;
    if (r > n - 1) r = n - 1;
    *il = l; *ir = r;
    *alpha = (dep - grid[l]) / (grid[r] - grid[l]);
}

/* physics.jl:290-306 inlet models; kind 2 is a CustomInlet (physics.jl:315-318)
 * whose closure is the piecewise-linear schedule T_in(t) */
static double schedule_at(const octx_t *c, double t) {
    const int n = c->sched_n;
    if (n == 0) return 0.0;
    if (t <= c->sched_t[0]) return c->sched_T[0];
    if (t >= c->sched_t[n - 1]) return c->sched_T[n - 1];
    int lo = 0, hi = n - 1;
    while (hi - lo > 1) {
        int mid = (lo + hi) / 2;
        if (c->sched_t[mid] <= t) lo = mid; else hi = mid;
    }
    double a = (t - c->sched_t[lo]) / (c->sched_t[hi] - c->sched_t[lo]);
    return fma(a, c->sched_T[hi] - c->sched_T[lo], c->sched_T[lo]);
}

/* kind 3: a CustomInlet whose closure (bh, T_outlet, t) -> T_in is given as a
 * postfix program: 0 push constant, 1 push T_outlet[bh], 2 push t, 3 push bh,
 * 4 x -> schedule(x), 5 x -> -x, 6..11 a b -> a+b, a-b, a*b, a/b, fmin, fmax
 * (the codes of include/gw_gb300.h's GW_OP_*).  The program is checked when it
 * is set, so the stack stays within its 16 slots. */
static double program_at(const octx_t *c, int bh, double t) {
    double st[16];
    int sp = 0;
    for (int i = 0; i < c->prog_n; ++i) {
        switch (c->prog_op[i]) {
            case 0: st[sp++] = c->prog_arg[i]; break;
            case 1: st[sp++] = c->T_outlet[bh]; break;
            case 2: st[sp++] = t; break;
            case 3: st[sp++] = (double)bh; break;
            case 4: st[sp - 1] = schedule_at(c, st[sp - 1]); break;
            case 5: st[sp - 1] = -st[sp - 1]; break;
            case 6: --sp; st[sp - 1] = st[sp - 1] + st[sp]; break;
            case 7: --sp; st[sp - 1] = st[sp - 1] - st[sp]; break;
            case 8: --sp; st[sp - 1] = st[sp - 1] * st[sp]; break;
            case 9: --sp; st[sp - 1] = st[sp - 1] / st[sp]; break;
            case 10: --sp; st[sp - 1] = fmin(st[sp - 1], st[sp]); break;
            case 11: --sp; st[sp - 1] = fmax(st[sp - 1], st[sp]); break;
            default: break;
        }
    }
    return st[0];
}

static double inlet_value(const octx_t *c, int bh, double t) {
    if (c->inlet_kind == 2) return schedule_at(c, t);
    if (c->inlet_kind == 3) return program_at(c, bh, t);
    return c->inlet_kind == 0 ? c->inlet_param : c->T_outlet[bh] - c->inlet_param;
}

/* Returns 0, or -1 if the program is malformed (the library's own checks). */
int ogw_set_program(void *h, int n, const int *op, const double *arg) {
    octx_t *c = (octx_t *)h;
    int depth = 0;
    if (n < 1 || n > 64) return -1;
    for (int i = 0; i < n; ++i) {
        if (op[i] < 0 || op[i] > 11) return -1;
        if (op[i] <= 3) ++depth;
        else if (op[i] <= 5) { if (depth < 1) return -1; }
        else { if (depth < 2) return -1; --depth; }
        if (depth > 16) return -1;
    }
    if (depth != 1) return -1;
    free(c->prog_op); free(c->prog_arg);
    c->prog_op = (int *)malloc(sizeof(int) * n);
    c->prog_arg = (double *)malloc(sizeof(double) * n);
    memcpy(c->prog_op, op, sizeof(int) * n);
    memcpy(c->prog_arg, arg, sizeof(double) * n);
    c->prog_n = n;
    return 0;
}

void ogw_set_schedule(void *h, int n, const double *t, const double *T) {
    octx_t *c = (octx_t *)h;
    free(c->sched_t); free(c->sched_T);
    c->sched_n = n;
    c->sched_t = (double *)malloc(sizeof(double) * (n > 0 ? n : 1));
    c->sched_T = (double *)malloc(sizeof(double) * (n > 0 ? n : 1));
    memcpy(c->sched_t, t, sizeof(double) * n);
    memcpy(c->sched_T, T, sizeof(double) * n);
}

/* solver.jl:250-396 advection! with kernel_accumulate_outlet!, kernel_advection!,
 * kernel_copy_advection! */
void ogw_advection(void *h, double *phi, double dt, double t) {
    octx_t *c = (octx_t *)h;
    const int ni = c->n_inner, no = c->n_outer, ncol = ni + no, cz = c->countz;
    /* solver.jl:253-257 */
    for (int b = 0; b < c->nbh; ++b) { c->T_outlet[b] = 0; c->T_outlet_counter[b] = 0; }
    for (int q = 0; q < ni; ++q) {
        int i = c->idx[3 * q], j = c->idx[3 * q + 1], b = c->idx[3 * q + 2];
        double z_max = c->bh[b].v_inner * dt;
        for (int k = 0; k < c->nz; ++k)
            if (c->gz[k] <= z_max) { c->T_outlet[b] += phi[IDX(c, k, j, i)]; c->T_outlet_counter[b] += 1; }
    }
    for (int b = 0; b < c->nbh; ++b) c->T_outlet[b] /= (double)c->T_outlet_counter[b];
    /* solver.jl:285-360 */
#pragma omp parallel for schedule(dynamic, 16)
    for (int q = 0; q < ncol; ++q) {
        int i = c->idx[3 * q], j = c->idx[3 * q + 1], b = c->idx[3 * q + 2];
        const obh_t *bh = &c->bh[b];
        for (int k = 0; k < cz; ++k) {
            double z = c->gz[k];
            double *out = &c->u_tmp[(size_t)q + (size_t)ncol * k];
            if (z > bh->h) { *out = phi[IDX(c, k, j, i)]; continue; }
            if (q < ni) {
                double zd = fma(bh->v_inner, dt, z);
                if (zd > bh->h) {
                    double dt1 = (bh->h - z) / bh->v_inner;
                    double dt2 = dt - dt1;
                    double zd2 = fma(-bh->v_outer, dt2, bh->h);
                    int kl, kr; double a;
                    interp_helper(c->gz, c->nz, zd2, &kl, &kr, &a);
                    double ml = 0, mr = 0; long cnt = 0;
                    for (int o = ni; o < ncol; ++o) {
                        if (c->idx[3 * o + 2] != b) continue;
                        int io = c->idx[3 * o], jo = c->idx[3 * o + 1];
                        ml += phi[IDX(c, kl, jo, io)];
                        mr += phi[IDX(c, kr, jo, io)];
                        cnt += 1;
                    }
                    ml /= (double)cnt; mr /= (double)cnt;
                    *out = fma(a, mr, (1 - a) * ml);
                } else {
                    int kl, kr; double a;
                    interp_helper(c->gz, c->nz, zd, &kl, &kr, &a);
                    *out = fma(a, phi[IDX(c, kr, j, i)], (1 - a) * phi[IDX(c, kl, j, i)]);
                }
            } else {
                double zd = fma(-bh->v_outer, dt, z);
                if (zd <= 0.0) {
                    *out = inlet_value(c, b, t);
                } else {
                    int kl, kr; double a;
                    interp_helper(c->gz, c->nz, zd, &kl, &kr, &a);
                    *out = fma(a, phi[IDX(c, kr, j, i)], (1 - a) * phi[IDX(c, kl, j, i)]);
                }
            }
        }
    }
    /* solver.jl:391-396 */
#pragma omp parallel for schedule(static)
    for (int q = 0; q < ncol; ++q) {
        if (!c->last[q]) continue;
        int i = c->idx[3 * q], j = c->idx[3 * q + 1];
        for (int k = 0; k < cz; ++k) phi[IDX(c, k, j, i)] = c->u_tmp[(size_t)q + (size_t)ncol * k];
    }
}

/* solver.jl:432-464 ADI_and_ADV_callback!: t = integrator.t (end of the step),
 * dt = t - tprev; temp is the scratch the reference takes from integrator.uprev */
void ogw_adi_adv(void *h, double *u, double *temp, double t, double dt) {
    ogw_diffusion_1d(h, temp, u, dt / 2, 1, 1);
    ogw_advection(h, temp, dt / 2, t);
    ogw_thomas(h, u, temp, dt / 2, 0);
    ogw_diffusion_1d(h, temp, u, dt / 2, 0, 1);
    ogw_advection(h, temp, dt / 2, t + dt / 2);
    ogw_thomas(h, u, temp, dt / 2, 1);
}

/* One ROCK2 step of u' = A_z u (rhs_diffusion_z!, solver.jl:23-31) in the
 * published stage form: recurrence g_j = h mu_j f(g_{j-1}) - nu_j g_{j-1}
 * - kappa_j g_{j-2} for j = 1..s-2, then the two-stage finishing procedure
 * with sigma, tau.  work holds 5 field-sized buffers. */
void ogw_rock2_step(void *hctx, double *u, double h, int s, const double *mu, const double *nu,
                    const double *kappa, double sigma, double tau, double *work) {
    octx_t *c = (octx_t *)hctx;
    size_t N = (size_t)c->nx * c->ny * c->nz;
    double *gm = work, *g = work + N, *gn = work + 2 * N, *F1 = work + 3 * N, *F2 = work + 4 * N;
    memcpy(g, u, sizeof(double) * N);
    memcpy(gm, u, sizeof(double) * N);
    for (int j = 1; j <= s - 2; ++j) {
        ogw_diffusion_1d(c, F1, g, 0.0, 2, 0);
        if (j == 1) {
#pragma omp parallel for schedule(static)
            for (size_t q = 0; q < N; ++q) gn[q] = g[q] + h * mu[0] * F1[q];
        } else {
            double m = mu[j - 1], n_ = nu[j - 1], kk = kappa[j - 1];
#pragma omp parallel for schedule(static)
            for (size_t q = 0; q < N; ++q) gn[q] = h * m * F1[q] - n_ * g[q] - kk * gm[q];
        }
        double *tmp = gm; gm = g; g = gn; gn = tmp;
    }
    /* finishing procedure: g = g_{s-2} */
    ogw_diffusion_1d(c, F1, g, 0.0, 2, 0);
#pragma omp parallel for schedule(static)
    for (size_t q = 0; q < N; ++q) gn[q] = g[q] + h * sigma * F1[q];
    ogw_diffusion_1d(c, F2, gn, 0.0, 2, 0);
    double cfin = h * sigma * (1 - tau / (sigma * sigma));
#pragma omp parallel for schedule(static)
    for (size_t q = 0; q < N; ++q) {
        double gstar = gn[q] + h * sigma * F2[q];
        u[q] = gstar - cfin * (F2[q] - F1[q]);
    }
}

void ogw_get_outlet(void *h, double *out) {
    octx_t *c = (octx_t *)h;
    memcpy(out, c->T_outlet, sizeof(double) * c->nbh);
}

/* physics.jl:333-348 initial_condition_thermal_gradient */
void ogw_initial_condition(void *h, double *phi, double T_surface, double gradient) {
    octx_t *c = (octx_t *)h;
    for (int i = 0; i < c->nx; ++i)
        for (int j = 0; j < c->ny; ++j)
            for (int k = 0; k < c->nz; ++k) phi[IDX(c, k, j, i)] = T_surface + gradient * c->gz[k];
}

int ogw_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
    return omp_get_max_threads();
#else
    (void)n;
    return 1;
#endif
}

/* Batched independent tridiagonal systems in the grouped interleaved layout
 * (row r of lane l of group g at goff[g] + 32 r + l; glen[g] rows), solved
 * one by one with the elimination of thomas_I_minus_A! (solver.jl:207-218):
 * w = lower/diag; diag -= w upper; rhs -= w rhs_prev; then back substitution
 * x_l = (rhs_l - upper_l x_{l+1}) / diag_l.  The sub-diagonal entry of row r
 * is a[r], the super-diagonal c[r]. */
void ogw_tridiag_batch(int ngroups, const long long *goff, const int *glen, const double *a,
                       const double *b, const double *c, const double *d, double *x) {
#pragma omp parallel
    {
        int cap = 0;
        double *dg = NULL, *rh = NULL;
#pragma omp for schedule(dynamic, 4)
        for (long long s = 0; s < 32LL * ngroups; ++s) {
            long long g = s / 32, l = s % 32;
            int L = glen[g];
            if (L > cap) { cap = L; dg = (double *)realloc(dg, sizeof(double) * cap); rh = (double *)realloc(rh, sizeof(double) * cap); }
            long long o = goff[g] + l;
            for (int r = 0; r < L; ++r) { dg[r] = b[o + 32LL * r]; rh[r] = d[o + 32LL * r]; }
            for (int r = 1; r < L; ++r) {
                double w = a[o + 32LL * r] / dg[r - 1];
                dg[r] = fma(-w, c[o + 32LL * (r - 1)], dg[r]);
                rh[r] = fma(-w, rh[r - 1], rh[r]);
            }
            double xn = rh[L - 1] / dg[L - 1];
            x[o + 32LL * (L - 1)] = xn;
            for (int r = L - 2; r >= 0; --r) {
                xn = fma(-c[o + 32LL * r], xn, rh[r]) / dg[r];
                x[o + 32LL * r] = xn;
            }
        }
        free(dg); free(rh);
    }
}
