// gw_setup_dev.cu -- the context's tables built on the GPU: the material
// model per (z-class, column), the column profiles, the coefficient tables
// of A_x, A_y, A_z, and per step size the Thomas factors of (I - h A) with
// the folded half-step tables.
//
// These are what create_cache and the first step of each step size cost:
// on the host they take ~0.3 s for a 239 x 239 x 1501 well array, about a
// thousand steps' worth of GPU time across an ensemble.  Every value here is
// bitwise the host path's (gw_setup.cpp, compiled with -ffp-contract=off):
// each double operation is one correctly rounded intrinsic, so nothing is
// contracted, and the material model makes the reference's comparisons
// (src/physics.jl:199-274) in the reference's order.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <unordered_map>
#include <vector>

#include "gw_internal.h"

namespace {

// material description on the device
struct MatDev {
    const double *depths, *kl, *rl;
    int nl;
    double k_water, rho_c_water, k_steel, rho_c_steel, k_ins, rho_c_ins, k_bf, rho_c_bf;
    const GwBorehole *bh;
    int nbh;
};

// src/physics.jl:102-125 (homogeneous == one layer)
__device__ int d_layer(const MatDev &m, double z) {
    for (int i = 0; i < m.nl; ++i)
        if (z <= m.depths[i]) return i;
    return m.nl - 1;
}

__device__ __forceinline__ double d_rsq(double x, double y, const GwBorehole &b) {
    const double dx = __dsub_rn(x, b.xc), dy = __dsub_rn(y, b.yc);
    return __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
}

// src/physics.jl:199-233 get_thermal_conductivity
__device__ double d_mat_k(const MatDev &m, double x, double y, double z) {
    double k = m.kl[d_layer(m, z)];
    for (int q = 0; q < m.nbh; ++q) {
        const GwBorehole &b = m.bh[q];
        const double r_sq = d_rsq(x, y, b);
        if (r_sq > b.r_backfill_sq) continue;
        if (z <= b.h) {
            if (r_sq < __dmul_rn(b.r_inner, b.r_inner)) k = m.k_water;
            else if (r_sq < b.r_and_t_inner_sq) k = m.k_ins;
            else if (r_sq < b.r_outer_sq) k = m.k_water;
            else if (r_sq < b.r_and_t_outer_sq) k = (z <= b.insulation_depth) ? m.k_ins : m.k_steel;
            else k = m.k_bf;
        } else if (z <= __dadd_rn(b.h, 3.0)) {
            k = m.k_steel;
        }
    }
    return k;
}

// src/physics.jl:243-274 get_volumetric_heat_capacity
__device__ double d_mat_rhoc(const MatDev &m, double x, double y, double z) {
    double rc = m.rl[d_layer(m, z)];
    for (int q = 0; q < m.nbh; ++q) {
        const GwBorehole &b = m.bh[q];
        const double r_sq = d_rsq(x, y, b);
        if (r_sq > b.r_and_t_outer_sq) continue;
        if (z <= b.h) {
            if (r_sq < __dmul_rn(b.r_inner, b.r_inner)) rc = m.rho_c_water;
            else if (r_sq < b.r_and_t_inner_sq) rc = m.rho_c_ins;
            else if (r_sq < b.r_outer_sq) rc = m.rho_c_water;
            else rc = (z <= b.insulation_depth) ? m.rho_c_ins : m.rho_c_steel;
        } else if (z <= __dadd_rn(b.h, 3.0)) {
            rc = m.rho_c_steel;
        }
    }
    return rc;
}

// K and R at every (z-class, column): [zc][i][j], zrep = z of the class's first level
__global__ void k_mat(double *__restrict__ K, double *__restrict__ R, const double *__restrict__ gx,
                      const double *__restrict__ gy, const double *__restrict__ zrep, MatDev m, int nx,
                      int ny, int nzc) {
    const long long n = (long long)nzc * nx * ny;
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n;
         q += (long long)gridDim.x * blockDim.x) {
        const int j = (int)(q % ny);
        const long long r = q / ny;
        const int i = (int)(r % nx), zc = (int)(r / nx);
        K[q] = d_mat_k(m, gx[i], gy[j], zrep[zc]);
        R[q] = d_mat_rhoc(m, gx[i], gy[j], zrep[zc]);
    }
}

// 64-bit FNV-1a of a column's material sequence (K, R per z-class, bit patterns)
__global__ void k_col_hash(unsigned long long *__restrict__ hash, const double *__restrict__ K,
                           const double *__restrict__ R, long long ncol, int nzc) {
    for (long long col = (long long)blockIdx.x * blockDim.x + threadIdx.x; col < ncol;
         col += (long long)gridDim.x * blockDim.x) {
        unsigned long long h = 1469598103934665603ull;
        for (int zc = 0; zc < nzc; ++zc) {
            const unsigned long long a = (unsigned long long)__double_as_longlong(K[zc * ncol + col]);
            const unsigned long long b = (unsigned long long)__double_as_longlong(R[zc * ncol + col]);
            for (int s = 0; s < 64; s += 8) { h ^= (a >> s) & 0xffull; h *= 1099511628211ull; }
            for (int s = 0; s < 64; s += 8) { h ^= (b >> s) & 0xffull; h *= 1099511628211ull; }
        }
        hash[col] = h;
    }
}

// every column's material sequence equals its profile representative's
__global__ void k_col_verify(int *__restrict__ bad, const int *__restrict__ colprof,
                             const int *__restrict__ repcol, const double *__restrict__ K,
                             const double *__restrict__ R, long long ncol, int nzc) {
    for (long long col = (long long)blockIdx.x * blockDim.x + threadIdx.x; col < ncol;
         col += (long long)gridDim.x * blockDim.x) {
        const long long rc = repcol[colprof[col]];
        for (int zc = 0; zc < nzc; ++zc)
            if (__double_as_longlong(K[zc * ncol + col]) != __double_as_longlong(K[zc * ncol + rc]) ||
                __double_as_longlong(R[zc * ncol + col]) != __double_as_longlong(R[zc * ncol + rc]))
                atomicExch(bad, 1);
    }
}

// the coefficient formula of gw_build_coefs: face conductivity (k_l + k_l+-1)/2,
// Neumann ends (cm = 0 at the first point, cp = 0 at the last)
__device__ __forceinline__ void d_coef(const double *__restrict__ g, int n, int l, double kc, double km,
                                       double kp, double rc, double *cm, double *cp) {
    const double dp = (l == n - 1) ? __dsub_rn(g[l], g[l - 1]) : __dsub_rn(g[l + 1], g[l]);
    const double dm = (l == 0) ? dp : __dsub_rn(g[l], g[l - 1]);
    const double mid = __dmul_rn(__dadd_rn(dp, dm), 0.5);
    *cp = (l == n - 1) ? 0.0 : __ddiv_rn(__ddiv_rn(__ddiv_rn(__dmul_rn(__dadd_rn(kp, kc), 0.5), dp), mid), rc);
    *cm = (l == 0) ? 0.0 : __ddiv_rn(__ddiv_rn(__ddiv_rn(__dmul_rn(__dadd_rn(kc, km), 0.5), dm), mid), rc);
}

// x: [zc][j][i]; y: [zc][i][j] (row index fastest)
__global__ void k_coef_xy(double *__restrict__ cxm, double *__restrict__ cxp, double *__restrict__ cym,
                          double *__restrict__ cyp, const double *__restrict__ K, const double *__restrict__ R,
                          const double *__restrict__ gx, const double *__restrict__ gy, int nx, int ny, int nzc) {
    const long long n = (long long)nzc * nx * ny;
    auto KI = [&](int zc, int i, int j) { return K[((long long)zc * nx + i) * ny + j]; };
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n;
         q += (long long)gridDim.x * blockDim.x) {
        {   // x entry q = (zc * ny + j) * nx + i
            const int i = (int)(q % nx);
            const long long r = q / nx;
            const int j = (int)(r % ny), zc = (int)(r / ny);
            const int ipl = i == nx - 1 ? i : i + 1, imi = i == 0 ? i : i - 1;
            d_coef(gx, nx, i, KI(zc, i, j), KI(zc, imi, j), KI(zc, ipl, j),
                   R[((long long)zc * nx + i) * ny + j], &cxm[q], &cxp[q]);
        }
        {   // y entry q = (zc * nx + i) * ny + j
            const int j = (int)(q % ny);
            const long long r = q / ny;
            const int i = (int)(r % nx), zc = (int)(r / nx);
            const int jpl = j == ny - 1 ? j : j + 1, jmi = j == 0 ? j : j - 1;
            d_coef(gy, ny, j, KI(zc, i, j), KI(zc, i, jmi), KI(zc, i, jpl), R[q], &cym[q], &cyp[q]);
        }
    }
}

// z: [profile][k] from the profile's representative column
__global__ void k_coef_z(double *__restrict__ czm, double *__restrict__ czp, const double *__restrict__ K,
                         const double *__restrict__ R, const double *__restrict__ gz,
                         const int *__restrict__ zclass, const int *__restrict__ repcol, long long ncol,
                         int nz, int np) {
    const long long n = (long long)np * nz;
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n;
         q += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(q % nz), p = (int)(q / nz);
        const long long col = repcol[p];
        const int kpl = k == nz - 1 ? k : k + 1, kmi = k == 0 ? k : k - 1;
        d_coef(gz, nz, k, K[zclass[k] * ncol + col], K[zclass[kmi] * ncol + col], K[zclass[kpl] * ncol + col],
               R[zclass[k] * ncol + col], &czm[q], &czp[q]);
    }
}

__global__ void k_to_float(float *__restrict__ dst, const double *__restrict__ src, size_t n) {
    for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x)
        dst[q] = (float)src[q];
}

// Thomas factors of (I - h A) along every (z-class, line) -- one thread per
// line, rows in sequence (gw_build_factors) -- with the folded half-step
// table of that line (gw_build_half_table; ecm/ecp the other direction's
// coefficients, [zc][row][line]).  Writes the double tables and, when the
// float pointers are set, their float roundings (mixed path: the half table
// only in float).
__global__ void k_factors(double *__restrict__ fa, double *__restrict__ fib, double *__restrict__ fcu,
                          double *__restrict__ h4, float *__restrict__ ga, float *__restrict__ gib,
                          float *__restrict__ gcu, float *__restrict__ g4, const double *__restrict__ cmt,
                          const double *__restrict__ cpt, const double *__restrict__ ecm,
                          const double *__restrict__ ecp, int nzc, int nl, int N, double h) {
    const long long nline = (long long)nzc * nl;
    for (long long line = (long long)blockIdx.x * blockDim.x + threadIdx.x; line < nline;
         line += (long long)gridDim.x * blockDim.x) {
        const int zc = (int)(line / nl), mline = (int)(line % nl);
        double dprev = 0.0, uprev = 0.0;
        for (int l = 0; l < N; ++l) {
            const size_t q = (size_t)line * N + l;
            const double m_ = cmt[q], p_ = cpt[q];
            const double lower = -__dmul_rn(h, m_);
            double diag = __dadd_rn(1.0, __dmul_rn(h, __dadd_rn(m_, p_)));
            const double upper = -__dmul_rn(h, p_);
            if (l > 0) diag = __dsub_rn(diag, __dmul_rn(__ddiv_rn(lower, dprev), uprev));
            const double a = (l > 0) ? lower : 0.0;
            const double ib = __ddiv_rn(1.0, diag);
            const double cu = __ddiv_rn(upper, diag);
            fa[q] = a; fib[q] = ib; fcu[q] = cu;
            const size_t e = ((size_t)zc * N + l) * nl + mline;
            const double cm = ecm[e], cp = ecp[e];
            const double v0 = __dmul_rn(__dsub_rn(1.0, __dmul_rn(h, __dadd_rn(cp, cm))), ib);
            const double v1 = __dmul_rn(__dmul_rn(h, cp), ib);
            const double v2 = __dmul_rn(__dmul_rn(h, cm), ib);
            const double v3 = __dmul_rn(a, ib);
            if (ga) {
                ga[q] = (float)a; gib[q] = (float)ib; gcu[q] = (float)cu;
                g4[4 * q] = (float)v0; g4[4 * q + 1] = (float)v1; g4[4 * q + 2] = (float)v2; g4[4 * q + 3] = (float)v3;
            } else {
                h4[4 * q] = v0; h4[4 * q + 1] = v1; h4[4 * q + 2] = v2; h4[4 * q + 3] = v3;
            }
            dprev = diag;
            uprev = upper;
        }
    }
}

inline unsigned blocks(long long n, int b = 256) {
    long long g = (n + b - 1) / b;
    return (unsigned)(g < 152 * 16 ? (g > 0 ? g : 1) : 152 * 16);
}

// device scratch freed at scope exit
struct Scratch {
    std::vector<void *> p;
    template <typename T>
    cudaError_t get(T **out, size_t n) {
        void *q = nullptr;
        cudaError_t e = cudaMalloc(&q, (n ? n : 1) * sizeof(T));
        if (e == cudaSuccess) p.push_back(q);
        *out = (T *)q;
        return e;
    }
    template <typename T>
    cudaError_t put(T **out, const std::vector<T> &v) {
        cudaError_t e = get(out, v.size());
        if (e == cudaSuccess && !v.empty()) e = cudaMemcpy(*out, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
        return e;
    }
    ~Scratch() {
        for (void *q : p) cudaFree(q);
    }
};

#define SCR(call)                                                          \
    do {                                                                   \
        cudaError_t _e = (call);                                           \
        if (_e != cudaSuccess) return gw_cuda_fail(_e, #call);             \
    } while (0)

}  // namespace

int gw_setup_tables_device(gw_ctx *c, double **cx, double **cy, double **cz) {
    const int nx = c->nx, ny = c->ny, nz = c->nz, nzc = c->n_zclass;
    const long long ncol = (long long)nx * ny;
    Scratch s;
    std::vector<double> zrep(nzc, 0.0);
    {
        std::vector<int> rep(nzc, -1);
        for (int k = 0; k < nz; ++k)
            if (rep[c->zclass[k]] < 0) rep[c->zclass[k]] = k;
        for (int zc = 0; zc < nzc; ++zc) zrep[zc] = c->gz[rep[zc]];
    }
    double *gx, *gy, *gz, *dz, *K, *R, *depths, *kl, *rl;
    int *zclass;
    GwBorehole *bh;
    SCR(s.put(&gx, c->gx)); SCR(s.put(&gy, c->gy)); SCR(s.put(&gz, c->gz)); SCR(s.put(&dz, zrep));
    SCR(s.put(&depths, c->depths)); SCR(s.put(&kl, c->k_layers)); SCR(s.put(&rl, c->rhoc_layers));
    SCR(s.put(&zclass, c->zclass)); SCR(s.put(&bh, c->bh));
    SCR(s.get(&K, (size_t)nzc * ncol)); SCR(s.get(&R, (size_t)nzc * ncol));
    MatDev m{depths, kl, rl, (int)c->depths.size(), c->k_water, c->rho_c_water, c->k_steel, c->rho_c_steel,
             c->k_insulating, c->rho_c_insulating, c->k_backfill, c->rho_c_backfill, bh, c->nbh};
    k_mat<<<blocks((long long)nzc * ncol), 256, 0, c->stream>>>(K, R, gx, gy, dz, m, nx, ny, nzc);
    SCR(cudaGetLastError());
    // column profiles: grouped by the hash of their material sequence, ids in
    // order of first appearance (i then j, as the host numbering), then every
    // column checked against its group's representative
    unsigned long long *hash;
    SCR(s.get(&hash, (size_t)ncol));
    k_col_hash<<<blocks(ncol), 256, 0, c->stream>>>(hash, K, R, ncol, nzc);
    SCR(cudaGetLastError());
    std::vector<unsigned long long> hh((size_t)ncol);
    SCR(cudaMemcpyAsync(hh.data(), hash, ncol * sizeof(unsigned long long), cudaMemcpyDeviceToHost, c->stream));
    SCR(cudaStreamSynchronize(c->stream));
    std::unordered_map<unsigned long long, int> ids;
    std::vector<int> repcol;
    c->colprof.assign((size_t)ncol, 0);
    for (long long col = 0; col < ncol; ++col) {
        auto it = ids.find(hh[col]);
        int id;
        if (it == ids.end()) {
            id = (int)repcol.size();
            ids.emplace(hh[col], id);
            repcol.push_back((int)col);
        } else {
            id = it->second;
        }
        c->colprof[col] = id;
    }
    int *dprof, *drep, *bad;
    SCR(s.put(&dprof, c->colprof)); SCR(s.put(&drep, repcol)); SCR(s.get(&bad, 1));
    SCR(cudaMemsetAsync(bad, 0, sizeof(int), c->stream));
    k_col_verify<<<blocks(ncol), 256, 0, c->stream>>>(bad, dprof, drep, K, R, ncol, nzc);
    SCR(cudaGetLastError());
    int hbad = 0;
    SCR(cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    SCR(cudaStreamSynchronize(c->stream));
    if (hbad) return gw_fail(GW_ERR_UNSUPPORTED, "column profile hash collision");   // the caller groups on the host
    c->n_profiles = (int)repcol.size();
    // coefficient tables, owned by the context from here on
    const size_t nxy = (size_t)nzc * ncol, nzp = (size_t)c->n_profiles * nz;
    double *cxm, *cxp, *cym, *cyp, *czm, *czp;
    SCR(cudaMalloc((void **)&cxm, nxy * sizeof(double))); c->allocations.push_back(cxm);
    SCR(cudaMalloc((void **)&cxp, nxy * sizeof(double))); c->allocations.push_back(cxp);
    SCR(cudaMalloc((void **)&cym, nxy * sizeof(double))); c->allocations.push_back(cym);
    SCR(cudaMalloc((void **)&cyp, nxy * sizeof(double))); c->allocations.push_back(cyp);
    SCR(cudaMalloc((void **)&czm, nzp * sizeof(double))); c->allocations.push_back(czm);
    SCR(cudaMalloc((void **)&czp, nzp * sizeof(double))); c->allocations.push_back(czp);
    c->device_bytes += (long long)((4 * nxy + 2 * nzp) * sizeof(double));
    for (double *t : {cxm, cxp, cym, cyp}) gw_debug_register(c->device, t, nxy * sizeof(double));
    for (double *t : {czm, czp}) gw_debug_register(c->device, t, nzp * sizeof(double));
    k_coef_xy<<<blocks((long long)nxy), 256, 0, c->stream>>>(cxm, cxp, cym, cyp, K, R, gx, gy, nx, ny, nzc);
    SCR(cudaGetLastError());
    k_coef_z<<<blocks((long long)nzp), 256, 0, c->stream>>>(czm, czp, K, R, gz, zclass, drep, ncol, nz,
                                                           c->n_profiles);
    SCR(cudaGetLastError());
    c->h_czm.resize(nzp);
    c->h_czp.resize(nzp);
    SCR(cudaMemcpyAsync(c->h_czm.data(), czm, nzp * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    SCR(cudaMemcpyAsync(c->h_czp.data(), czp, nzp * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    SCR(cudaStreamSynchronize(c->stream));   // before the scratch is freed
    c->c64.cxm = cxm; c->c64.cxp = cxp; c->c64.cym = cym; c->c64.cyp = cyp; c->c64.czm = czm; c->c64.czp = czp;
    cx[0] = cxm; cx[1] = cxp; cy[0] = cym; cy[1] = cyp; cz[0] = czm; cz[1] = czp;
    return GW_OK;
}

int gw_tables_to_float(gw_ctx *c, float *dst, const double *src, size_t n) {
    k_to_float<<<blocks((long long)n), 256, 0, c->stream>>>(dst, src, n);
    SCR(cudaGetLastError());
    return GW_OK;
}

int gw_factors_device(gw_ctx *c, double h) {
    const bool mix = c->precision == GW_PREC_MIXED;
    for (int dir = GW_DIR_X; dir <= GW_DIR_Y; ++dir) {
        const int nl = dir == GW_DIR_X ? c->ny : c->nx, N = dir == GW_DIR_X ? c->nx : c->ny;
        const GwFactors<double> &f = dir == GW_DIR_X ? c->c64.fx : c->c64.fy;
        const GwFactors<float> &g = dir == GW_DIR_X ? c->c32.fx : c->c32.fy;
        const double *cm = dir == GW_DIR_X ? c->c64.cxm : c->c64.cym, *cp = dir == GW_DIR_X ? c->c64.cxp : c->c64.cyp;
        // x-lines fold the explicit y sweep, y-lines the explicit x sweep
        const double *em = dir == GW_DIR_X ? c->c64.cym : c->c64.cxm, *ep = dir == GW_DIR_X ? c->c64.cyp : c->c64.cxp;
        double *h4 = mix ? nullptr : (dir == GW_DIR_X ? c->c64.hx : c->c64.hy);
        float *g4 = mix ? (dir == GW_DIR_X ? c->c32.hx : c->c32.hy) : nullptr;
        k_factors<<<blocks((long long)c->n_zclass * nl, 128), 128, 0, c->stream>>>(
            f.a, f.ib, f.cu, h4, mix ? g.a : nullptr, mix ? g.ib : nullptr, mix ? g.cu : nullptr, g4, cm, cp, em,
            ep, c->n_zclass, nl, N, h);
        SCR(cudaGetLastError());
    }
    SCR(cudaStreamSynchronize(c->stream));
    return GW_OK;
}
