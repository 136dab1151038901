// gw_kernels.cu -- sm_103a kernels of the time-step hot path (double path).
//
// Layout: field element (k, j, i) at k + Nz*(j + Ny*i) (z fastest, as the
// reference's phi[k,j,i]).  Every kernel maps consecutive threads to
// consecutive k, so each warp access is one contiguous run of the field.
// The material model is read from small coefficient tables (per z-class and
// column, see gw_setup.cpp) instead of being re-evaluated per cell.
#include <cuda_runtime.h>

#include "gw_inlet.cuh"
#include "gw_internal.h"

namespace {

constexpr int kBlock = 256;

inline unsigned grid_for(long long n, int block) {
    return (unsigned)((n + block - 1) / block);
}

// One ROCK2 stage on the z-operator (rhs_diffusion_z!, src/solver.jl:23-58 in
// the z direction):  az = (A_z x)_c
//   rhs_only: out = az
//   else      out = x + hmu * az + kap * (x - y)
// which is the recurrence g_j = g_{j-1} + h mu_j A g_{j-1} + kappa_j (g_{j-1} - g_{j-2})
// (equal to h mu_j f(g_{j-1}) - nu_j g_{j-1} - kappa_j g_{j-2} since -nu_j - kappa_j = 1)
// and both finishing stages.  out may alias y (read at c only), not x.
__global__ void __launch_bounds__(kBlock) k_zstage(double *out,
                                                   const double *__restrict__ x,
                                                   const double *y, const int *__restrict__ colprof,
                                                   const double *__restrict__ czm,
                                                   const double *__restrict__ czp, int nz,
                                                   long long ncell, double hmu, double kap,
                                                   int rhs_only) {
    long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncell) return;
    int k = (int)(c % nz);
    long long col = c / nz;
    int p = __ldg(colprof + col);
    double cm = __ldg(czm + (size_t)p * nz + k), cp = __ldg(czp + (size_t)p * nz + k);
    double xc = x[c];
    double xp = (k < nz - 1) ? x[c + 1] : xc;
    double xm = (k > 0) ? x[c - 1] : xc;
    double az = cp * (xp - xc) - cm * (xc - xm);
    if (rhs_only) {
        out[c] = az;
    } else {
        double v = fma(hmu, az, xc);
        if (kap != 0.0) v = fma(kap, xc - y[c], v);
        out[c] = v;
    }
}

// Explicit half step (I + h A_dir) phi, src/solver.jl:34-58 with plus_I.
// dir 0: x (stride Nz*Ny, table [zc][j][i]); dir 1: y (stride Nz, table [zc][i][j]).
__global__ void __launch_bounds__(kBlock) k_explicit(double *__restrict__ dst,
                                                     const double *__restrict__ src,
                                                     const int *__restrict__ zclass,
                                                     const double *__restrict__ cmt,
                                                     const double *__restrict__ cpt, int nx, int ny,
                                                     int nz, long long ncell, double h, int dir) {
    long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncell) return;
    int k = (int)(c % nz);
    long long r = c / nz;
    int j = (int)(r % ny), i = (int)(r / ny);
    int zc = __ldg(zclass + k);
    double xc = src[c], xp, xm;
    size_t q;
    if (dir == 0) {
        long long s = (long long)nz * ny;
        xp = (i < nx - 1) ? src[c + s] : xc;
        xm = (i > 0) ? src[c - s] : xc;
        q = ((size_t)zc * ny + j) * nx + i;
    } else {
        xp = (j < ny - 1) ? src[c + nz] : xc;
        xm = (j > 0) ? src[c - nz] : xc;
        q = ((size_t)zc * nx + i) * ny + j;
    }
    double a = __ldg(cpt + q) * (xp - xc) - __ldg(cmt + q) * (xc - xm);
    dst[c] = fma(h, a, xc);
}

// (I - h A_dir) U = RHS along every x- or y-line with the precomputed LU
// factors (src/solver.jl:111-232).  One thread per line; consecutive threads
// take consecutive k, so each row access of a warp is contiguous.  The
// forward sweep stores y_l in U, the backward sweep overwrites it with x_l.
__global__ void __launch_bounds__(128) k_thomas(double *__restrict__ U,
                                                const double *__restrict__ R,
                                                const int *__restrict__ zclass,
                                                const double *__restrict__ fa,
                                                const double *__restrict__ fib,
                                                const double *__restrict__ fcu, int nx, int ny,
                                                int nz, int dir) {
    const int nl = dir == 0 ? ny : nx;          // lines per level
    const int N = dir == 0 ? nx : ny;           // line length
    long long L = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (L >= (long long)nz * nl) return;
    int k = (int)(L % nz);
    int m = (int)(L / nz);
    int zc = __ldg(zclass + k);
    size_t fb = ((size_t)zc * nl + m) * N;
    long long stride, off0;
    if (dir == 0) {  // x-line at (k, j=m): element (k, m, l)
        stride = (long long)nz * ny;
        off0 = k + (long long)nz * m;
    } else {         // y-line at (k, i=m): element (k, l, m)
        stride = nz;
        off0 = k + (long long)nz * ny * m;
    }
    double y = 0.0;
    for (int l = 0; l < N; ++l) {
        long long o = off0 + l * stride;
        y = (R[o] - __ldg(fa + fb + l) * y) * __ldg(fib + fb + l);
        U[o] = y;
    }
    double x = y;
    for (int l = N - 2; l >= 0; --l) {
        long long o = off0 + l * stride;
        x = U[o] - __ldg(fcu + fb + l) * x;
        U[o] = x;
    }
}

// kernel_accumulate_outlet! (src/solver.jl:267-282) + the division of 257:
// mean of phi over the borehole's inner-pipe cells with z <= v_inner * dt.
// One block per borehole, fixed-order reduction (deterministic, unlike the
// reference's float atomics).
__global__ void __launch_bounds__(256) k_outlet(double *__restrict__ outlet,
                                                const double *__restrict__ phi,
                                                const double *__restrict__ gz,
                                                const int *__restrict__ pi,
                                                const int *__restrict__ pj,
                                                const GwBhDev *__restrict__ bh, int ny, int nz,
                                                double dt) {
    const int b = blockIdx.x;
    const GwBhDev B = bh[b];
    const double zmax = B.v_inner * dt;
    __shared__ int s_nlev;
    __shared__ double s_red[256];
    if (threadIdx.x == 0) {
        int lo = 0, hi = nz;  // gz sorted: levels with gz <= zmax are a prefix
        while (lo < hi) {
            int mid = (lo + hi) >> 1;
            if (gz[mid] <= zmax) lo = mid + 1; else hi = mid;
        }
        s_nlev = lo;
    }
    __syncthreads();
    const int nlev = s_nlev;
    const long long tot = (long long)B.inner_count * nlev;
    double acc = 0.0;
    for (long long e = threadIdx.x; e < tot; e += blockDim.x) {
        int q = B.inner_begin + (int)(e / nlev);
        int k = (int)(e % nlev);
        acc += phi[k + (long long)nz * (pj[q] + (long long)ny * pi[q])];
    }
    s_red[threadIdx.x] = acc;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) s_red[threadIdx.x] += s_red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) outlet[b] = s_red[0] / (double)tot;
}

// Per borehole and level, the annulus mean that every turnaround cell of the
// reference recomputes by looping over all annulus cells
// (src/solver.jl:322-335).  Summed in the same list order.
__global__ void __launch_bounds__(128) k_annulus_mean(double *__restrict__ mean,
                                                      const double *__restrict__ phi,
                                                      const int *__restrict__ pi,
                                                      const int *__restrict__ pj,
                                                      const GwBhDev *__restrict__ bh, int ny,
                                                      int nz) {
    // every level: a departure index can reach any of them (src/solver.jl:366-368)
    const int b = blockIdx.y;
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nz) return;
    const GwBhDev B = bh[b];
    double s = 0.0;
    for (int q = B.outer_begin; q < B.outer_begin + B.outer_count; ++q)
        s += phi[k + (long long)nz * (pj[q] + (long long)ny * pi[q])];
    mean[(size_t)b * nz + k] = s / (double)B.outer_count;
}

// gpu_searchsortedfirst + interpolation_helper (src/solver.jl:362-389), 0-based.
__device__ __forceinline__ void interp(const double *__restrict__ g, int n, double dep, int &il,
                                       int &ir, double &alpha) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        int mid = lo + ((hi - lo) >> 1);
        if (g[mid] < dep) lo = mid + 1; else hi = mid;
    }
    ir = lo;
    il = lo - 1;
    if (il < 0) il = 0;
    if (ir > n - 1) ir = n - 1;
    double xl = g[il], xr = g[ir];
    alpha = __ddiv_rn(__dsub_rn(dep, xl), __dsub_rn(xr, xl));
}

// kernel_advection! (src/solver.jl:285-360): one thread per (level < countz,
// pipe column), k fastest.  Reads phi, writes utmp[q][k].  The departure
// points use fused multiply-adds as the reference's @muladd does, so branch
// decisions (turnaround, inlet) match it exactly.
__global__ void __launch_bounds__(256) k_advect(double *__restrict__ utmp,
                                                const double *__restrict__ phi,
                                                const double *__restrict__ gz,
                                                const int *__restrict__ pi,
                                                const int *__restrict__ pj,
                                                const int *__restrict__ pb,
                                                const GwBhDev *__restrict__ bh,
                                                const double *__restrict__ ann_mean,
                                                const double *__restrict__ outlet, int n_inner,
                                                int ncol, int ny, int nz, int countz, double dt,
                                                int inlet_kind, double inlet_param,
                                                const double *__restrict__ inlet_v) {
    long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (long long)ncol * countz) return;
    const int k = (int)(e % countz);
    const int q = (int)(e / countz);
    const int b = pb[q];
    const GwBhDev B = bh[b];
    const long long col = (long long)nz * (pj[q] + (long long)ny * pi[q]);
    const double z = gz[k];
    double v;
    if (z > B.h) {
        v = phi[col + k];
    } else if (q < n_inner) {
        double zd = __fma_rn(B.v_inner, dt, z);
        if (zd > B.h) {
            double dt1 = __ddiv_rn(__dsub_rn(B.h, z), B.v_inner);
            double dt2 = __dsub_rn(dt, dt1);
            double zd2 = __fma_rn(-B.v_outer, dt2, B.h);
            int il, ir; double a;
            interp(gz, nz, zd2, il, ir, a);
            const double *m = ann_mean + (size_t)b * nz;
            v = __fma_rn(a, m[ir], __dmul_rn(__dsub_rn(1.0, a), m[il]));
        } else {
            int il, ir; double a;
            interp(gz, nz, zd, il, ir, a);
            v = __fma_rn(a, phi[col + ir], __dmul_rn(__dsub_rn(1.0, a), phi[col + il]));
        }
    } else {
        double zd = __fma_rn(-B.v_outer, dt, z);
        if (zd <= 0.0) {
            v = inlet_kind == GW_INLET_CONSTANT ? inlet_param
              : inlet_kind == GW_INLET_EXPRESSION ? inlet_v[b] : outlet[b] - inlet_param;
        } else {
            int il, ir; double a;
            interp(gz, nz, zd, il, ir, a);
            v = __fma_rn(a, phi[col + ir], __dmul_rn(__dsub_rn(1.0, a), phi[col + il]));
        }
    }
    utmp[(size_t)q * countz + k] = v;
}

// The inlet program of every borehole at time t (GW_INLET_EXPRESSION), with
// the outlet temperatures of the advection's k_outlet.
__global__ void k_inlet_program(double *__restrict__ inlet_v, const int *__restrict__ op,
                                const double *__restrict__ arg, int nprog,
                                const double *__restrict__ outlet, const double *__restrict__ sched, int ns,
                                double t, int nbh) {
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < nbh; b += gridDim.x * blockDim.x)
        inlet_v[b] = gw_program_eval(op, arg, nprog, outlet[b], t, b, sched, ns);
}

// kernel_copy_advection! (src/solver.jl:391-396).  A column listed for two
// boreholes (their pipes overlap) is written by its last list entry only,
// as a sequential run of the reference's loop leaves it (pipe_of holds the
// last entry of every column).
__global__ void __launch_bounds__(256) k_scatter(double *__restrict__ phi,
                                                 const double *__restrict__ utmp,
                                                 const int *__restrict__ pi,
                                                 const int *__restrict__ pj,
                                                 const int *__restrict__ pipe_of, int ncol, int ny,
                                                 int nz, int countz) {
    long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (long long)ncol * countz) return;
    const int k = (int)(e % countz);
    const int q = (int)(e / countz);
    if (pipe_of[(size_t)pi[q] * ny + pj[q]] != q) return;
    phi[k + (long long)nz * (pj[q] + (long long)ny * pi[q])] = utmp[e];
}

// After each fused step: outlet series and the extracted-heat integral,
// Q = mdot * c_w * (T_out - T_in), c_w = rho_c_water / 998.2 (double).
__global__ void k_record(double *__restrict__ series, double *__restrict__ energy,
                         int *__restrict__ counter, const double *__restrict__ outlet,
                         const GwBhDev *__restrict__ bh, int nbh, int cap, double dt,
                         double c_w, int inlet_kind, double inlet_param,
                         const double *__restrict__ inlet_v) {
    const int b = threadIdx.x;
    const int n = *counter;
    __syncthreads();
    if (b < nbh) {
        double to = outlet[b];
        double ti = inlet_kind == GW_INLET_CONSTANT ? inlet_param
                  : inlet_kind >= GW_INLET_SCHEDULE ? inlet_v[b] : to - inlet_param;
        if (n < cap) series[(size_t)n * nbh + b] = to;
        energy[b] += bh[b].mdot * c_w * (to - ti) * dt;
    }
    __syncthreads();
    if (b == 0) *counter = n + 1;
}

// dst = sum_i w_i src_i (up to 8 sources), grid-stride over the cells.
struct LinComb {
    const double *src[8];
    double w[8];
    int n;
};

__global__ void __launch_bounds__(256) k_lincomb(double *dst, LinComb lc, size_t ncell) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < ncell; i += stride) {
        double v = 0.0;
#pragma unroll
        for (int q = 0; q < 8; ++q)
            if (q < lc.n) v = fma(lc.w[q], lc.src[q][i], v);
        dst[i] = v;
    }
}

// u[k, j, i] = col[k]: one z profile copied into every column (z fastest).
__global__ void __launch_bounds__(256) k_broadcast_column(double *__restrict__ u, const double *__restrict__ col,
                                                          size_t ncell, int nz) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < ncell; i += stride)
        u[i] = col[i % (size_t)nz];
}

__global__ void k_check_finite(const double *__restrict__ u, size_t n, int *__restrict__ flag) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    size_t s = (size_t)gridDim.x * blockDim.x;
    bool bad = false;
    for (; i < n; i += s) bad |= !isfinite(u[i]);
    if (__syncthreads_or(bad) && threadIdx.x == 0) atomicExch(flag, 1);
}

}  // namespace

int gw_launch_zstage(gw_ctx *c, double *out, const double *x, const double *y, double hmu,
                     double kap, int rhs_only) {
    long long n = (long long)c->nx * c->ny * c->nz;
    k_zstage<<<grid_for(n, kBlock), kBlock, 0, c->stream>>>(out, x, y, c->d_colprof, c->c64.czm,
                                                            c->c64.czp, c->nz, n, hmu, kap,
                                                            rhs_only);
    GW_CUDA(cudaGetLastError());
    return GW_OK;
}

int gw_launch_explicit(gw_ctx *c, double *dst, const double *src, double h, int dir) {
    long long n = (long long)c->nx * c->ny * c->nz;
    const double *cm = dir == GW_DIR_X ? c->c64.cxm : c->c64.cym;
    const double *cp = dir == GW_DIR_X ? c->c64.cxp : c->c64.cyp;
    k_explicit<<<grid_for(n, kBlock), kBlock, 0, c->stream>>>(dst, src, c->d_zclass, cm, cp, c->nx,
                                                              c->ny, c->nz, n, h, dir);
    GW_CUDA(cudaGetLastError());
    return GW_OK;
}

int gw_launch_thomas(gw_ctx *c, double *U, const double *R, int dir) {
    long long lines = (long long)c->nz * (dir == GW_DIR_X ? c->ny : c->nx);
    const GwFactors<double> &f = dir == GW_DIR_X ? c->c64.fx : c->c64.fy;
    k_thomas<<<grid_for(lines, 128), 128, 0, c->stream>>>(U, R, c->d_zclass, f.a, f.ib, f.cu, c->nx,
                                                          c->ny, c->nz, dir);
    GW_CUDA(cudaGetLastError());
    return GW_OK;
}

int gw_launch_advection(gw_ctx *c, double *phi, double dt, double t) {
    // a schedule inlet is a known value at the call's time t
    const bool sched = c->inlet_kind == GW_INLET_SCHEDULE;
    const int ikind = sched ? GW_INLET_CONSTANT : c->inlet_kind;
    const double iparam = sched ? gw_schedule_at(c, t) : c->inlet_param;
    const int ncol = c->n_inner + c->n_outer;
    k_outlet<<<c->nbh, 256, 0, c->stream>>>(c->d_outlet, phi, c->d_gz, c->d_pipe_i, c->d_pipe_j,
                                            c->d_bh, c->ny, c->nz, dt);
    GW_CUDA(cudaGetLastError());
    if (ncol == 0 || c->countz == 0) return GW_OK;
    if (c->inlet_kind == GW_INLET_EXPRESSION) {
        // the program reads this advection's outlet temperatures
        k_inlet_program<<<1, 128, 0, c->stream>>>(c->d_inlet, c->d_prog_op, c->d_prog_arg, c->n_prog,
                                                  c->d_outlet, c->d_sched, c->n_sched, t, c->nbh);
        GW_CUDA(cudaGetLastError());
    }
    dim3 g(grid_for(c->nz, 128), c->nbh);
    k_annulus_mean<<<g, 128, 0, c->stream>>>(c->d_annmean, phi, c->d_pipe_i, c->d_pipe_j, c->d_bh,
                                             c->ny, c->nz);
    GW_CUDA(cudaGetLastError());
    long long n = (long long)ncol * c->countz;
    k_advect<<<grid_for(n, 256), 256, 0, c->stream>>>(
        c->d_utmp, phi, c->d_gz, c->d_pipe_i, c->d_pipe_j, c->d_pipe_b, c->d_bh, c->d_annmean,
        c->d_outlet, c->n_inner, ncol, c->ny, c->nz, c->countz, dt, ikind, iparam, c->d_inlet);
    GW_CUDA(cudaGetLastError());
    k_scatter<<<grid_for(n, 256), 256, 0, c->stream>>>(phi, c->d_utmp, c->d_pipe_i, c->d_pipe_j,
                                                        c->d_pipe_of, ncol, c->ny, c->nz, c->countz);
    GW_CUDA(cudaGetLastError());
    return GW_OK;
}

int gw_launch_record(gw_ctx *c, double dt, cudaStream_t st) {
    int threads = ((c->nbh + 31) / 32) * 32;
    k_record<<<1, threads, 0, st ? st : c->stream>>>(c->d_series, c->d_energy, c->d_step_counter, c->d_outlet,
                                           c->d_bh, c->nbh, c->series_cap, dt,
                                           c->rho_c_water / 998.2, c->inlet_kind, c->inlet_param, c->d_inlet);
    GW_CUDA(cudaGetLastError());
    return GW_OK;
}

int gw_launch_lincomb(gw_ctx *c, double *dst, int n, const double *w, const double *const *src) {
    LinComb lc{};
    for (int q = 0; q < n; ++q) { lc.src[q] = src[q]; lc.w[q] = w[q]; }
    lc.n = n;
    const size_t N = (size_t)c->nx * c->ny * c->nz;
    k_lincomb<<<152 * 8, 256, 0, c->stream>>>(dst, lc, N);
    GW_CUDA(cudaGetLastError());
    return GW_OK;
}

// Snapshot conversion: float temperatures of the state, rounded once from
// the double value (theta + T_ref in the mixed path).
__global__ void k_snapshot_f64(float *__restrict__ dst, const double *__restrict__ u, size_t n) {
    for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x)
        dst[q] = (float)u[q];
}
// theta: columns pz floats apart (pz >= nz); dst: nz levels per column
__global__ void k_snapshot_theta(float *__restrict__ dst, const float *__restrict__ th,
                                 const double *__restrict__ Tref, size_t n, int nz, int pz) {
    for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x) {
        const size_t col = q / nz, k = q - col * nz;
        dst[q] = (float)((double)th[col * pz + k] + Tref[k]);
    }
}

int gw_launch_snapshot(gw_ctx *c, float *dst) {
    const size_t N = (size_t)c->nx * c->ny * c->nz;
    if (c->precision == GW_PREC_MIXED)
        k_snapshot_theta<<<152 * 8, 256, 0, c->stream>>>(dst, c->f_u, c->d_Tref, N, c->nz, c->pz);
    else
        k_snapshot_f64<<<152 * 8, 256, 0, c->stream>>>(dst, c->d_u, N);
    GW_CUDA(cudaGetLastError());
    return GW_OK;
}

int gw_launch_broadcast_column(gw_ctx *c, double *u, const double *col) {
    const size_t N = (size_t)c->nx * c->ny * c->nz;
    k_broadcast_column<<<152 * 8, 256, 0, c->stream>>>(u, col, N, c->nz);
    GW_CUDA(cudaGetLastError());
    return GW_OK;
}

int gw_launch_check_finite(gw_ctx *c, const double *u, size_t n) {
    GW_CUDA(cudaMemsetAsync(c->d_flag, 0, sizeof(int), c->stream));
    k_check_finite<<<1216, 256, 0, c->stream>>>(u, n, c->d_flag);
    GW_CUDA(cudaGetLastError());
    return GW_OK;
}
