// gw_adjoint.cu -- reverse-mode gradient of the time-step map, for the double
// path (GW_PREC_FP64) and the mixed path (GW_PREC_MIXED: float adjoint fields
// over the float theta = T - T_ref(z) states, double gradient sums).
//
// The reference has no derivatives; this is the differentiation layer a
// ChainRulesCore rrule (or a torch.autograd.Function) binds.  Objective:
//   J = sum_b [ w_E E_b + w_T T_out,b(last step) ],
//   E_b = sum_n mdot_b c_w (T_out,b^n - T_in,b^n) dt      (as gw_get_energy),
// parameters p = (k_rock_layers[0..L-1], mdot[0..nbh-1], inlet_param).
//
// For fixed p the step u^n -> u^{n+1} (one ROCK2 step of rhs_diffusion_z!,
// src/solver.jl:23-31, then ADI_and_ADV_callback!, src/solver.jl:432-464) is
// affine in u, so its transpose is assembled from the transposes of its parts:
//   ROCK2 = P(dt A_z), a polynomial in A_z  -> the stage recurrence run
//                                              backwards on A_z^T
//   explicit sweep (I + h A)                -> (I + h A^T)
//   line solve (I - h A)^{-1}               -> (I - h A)^{-T}: the same LU
//                                              factors swept as U^T, then L^T
//   semi-Lagrangian advection (gather and   -> scatter-add of the interpolation
//   interpolate, src/solver.jl:285-376)        weights, the turnaround means and
//                                              the outlet window
// Parameter derivatives: conductivity face terms summed per level (then per
// rock layer), departure-point derivatives (flow rate through v_inner and
// v_outer, src/physics.jl:49-57), inlet cells and the energy balance.  In the
// mixed path T = theta + T_ref(z): A_x and A_y annihilate T_ref, so theta's
// adjoint is T's, and the z face terms add T_ref's differences.
//
// Memory: the forward sweep keeps the state every K steps (checkpoints); the
// reverse sweep recomputes one segment's states with the fused step, then
// per step the step's intermediates (double: the modular kernels; mixed: the
// fused kernels, whose pipe passes leave the pre-advection values of the
// pipe columns in a compact buffer) and runs the step's adjoint.  The branch
// structure of the advection (which cells turn around, which take the inlet
// value, the outlet window's levels) is held fixed, as any derivative of a
// piecewise map is.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "gw_fused.h"
#include "gw_internal.h"

struct GwAdj {
    double *wxm = nullptr, *wxp = nullptr, *wym = nullptr, *wyp = nullptr;
    double *wzm = nullptr, *wzp = nullptr;
    float *fxm = nullptr, *fxp = nullptr, *fym = nullptr, *fyp = nullptr;   // the same, float
    float *fzm = nullptr, *fzp = nullptr;
    unsigned char *rock = nullptr;
    std::vector<int> layer;     // rock layer of each level
    double *G = nullptr;        // [nz] conductivity derivative per level
    double *sc = nullptr;       // [nbh][4]: dJ/dv_inner, dJ/dv_outer, inlet adjoint of
                                //           the current advection, its sum over calls
    double *osum = nullptr;     // [nbh] sum over steps of T_out - T_in
    double *mbar = nullptr;     // [nbh][nz] adjoint of the turnaround annulus means
    double *tmp = nullptr;      // [ncol][countz] adjoint of the advected pipe values (8 B slots)
    double *S = nullptr;        // [nbh][countz] its sum over each borehole's inner columns
    std::vector<void *> allocs;
    long long bytes = 0;
};

namespace {

constexpr int kB = 256;
constexpr double kRhoWater = 998.2;   // src/physics.jl:48

inline unsigned nblocks(long long n, int b) { return (unsigned)((n + b - 1) / b); }

template <typename T>
int adj_alloc(GwAdj *a, T **p, size_t n) {
    if (n == 0) n = 1;
    cudaError_t e = cudaMalloc((void **)p, n * sizeof(T));
    if (e != cudaSuccess) return gw_cuda_fail(e, "cudaMalloc (adjoint tables)");
    a->allocs.push_back((void *)*p);
    a->bytes += (long long)(n * sizeof(T));
    return GW_OK;
}

template <typename T>
int adj_upload(GwAdj *a, T **p, const std::vector<T> &v) {
    int rc = adj_alloc(a, p, v.size());
    if (rc) return rc;
    if (!v.empty()) GW_CUDA(cudaMemcpy(*p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
    return GW_OK;
}

// ---------------------------------------------------------------------------
// transposed operators

// out = a1 lam + hmu (A_z^T lam) + a2 w.  A_z row k: cm_k at k-1, -(cm_k + cp_k)
// at k, cp_k at k+1 (cm_0 = cp_{nz-1} = 0), so (A_z^T lam)_k = cp_{k-1} lam_{k-1}
// - (cm_k + cp_k) lam_k + cm_{k+1} lam_{k+1}.  w is read at the cell only, so
// out may alias w (not lam).
template <typename T>
__global__ void __launch_bounds__(kB) k_zstage_t(T *out, const T *__restrict__ lam, const T *w,
                                                 const int *__restrict__ colprof,
                                                 const T *__restrict__ czm, const T *__restrict__ czp,
                                                 int nz, long long ncol, T a1, T hmu, T a2) {
    // block: kB levels (blockIdx.y) of every gridDim.x-th column
    const int k = blockIdx.y * kB + threadIdx.x;
    if (k >= nz) return;
    for (long long col = blockIdx.x; col < ncol; col += gridDim.x) {
        const long long c = col * nz + k;
        const size_t base = (size_t)__ldg(colprof + col) * nz;
        const T lc = lam[c];
        T at = -(__ldg(czm + base + k) + __ldg(czp + base + k)) * lc;
        if (k > 0) at = fma(__ldg(czp + base + k - 1), lam[c - 1], at);
        if (k < nz - 1) at = fma(__ldg(czm + base + k + 1), lam[c + 1], at);
        T v = fma(hmu, at, a1 * lc);
        if (a2 != T(0)) v = fma(a2, w[c], v);
        out[c] = v;
    }
}

// Mixed path, forward: one ROCK2 stage on theta = T - T_ref with the source
// fref = A_z T_ref (per profile and level):
//   out = x + hmu (A_z x + fref) + kap (x - y)      (out may alias y, not x)
__global__ void __launch_bounds__(kB) k_zstage_theta(float *out, const float *__restrict__ x,
                                                     const float *y, const int *__restrict__ colprof,
                                                     const float *__restrict__ czm,
                                                     const float *__restrict__ czp,
                                                     const float *__restrict__ fref, int nz, long long ncol,
                                                     float hmu, float kap) {
    const int k = blockIdx.y * kB + threadIdx.x;
    if (k >= nz) return;
    for (long long col = blockIdx.x; col < ncol; col += gridDim.x) {
        const long long c = col * nz + k;
        const size_t q = (size_t)__ldg(colprof + col) * nz + k;
        const float xc = x[c];
        const float xp = k < nz - 1 ? x[c + 1] : xc;
        const float xm = k > 0 ? x[c - 1] : xc;
        const float a = __ldg(czp + q) * (xp - xc) - __ldg(czm + q) * (xc - xm) + __ldg(fref + q);
        float v = fmaf(hmu, a, xc);
        if (kap != 0.f) v = fmaf(kap, xc - y[c], v);
        out[c] = v;
    }
}

// dst = src + h A^T src along x (dir 0, table [zc][j][i]) or y (dir 1, [zc][i][j]).
template <typename T>
__global__ void __launch_bounds__(kB) k_explicit_t(T *__restrict__ dst, const T *__restrict__ src,
                                                   const int *__restrict__ zclass,
                                                   const T *__restrict__ cmt, const T *__restrict__ cpt,
                                                   int nx, int ny, int nz, T h, int dir) {
    const int k = blockIdx.y * kB + threadIdx.x;
    if (k >= nz) return;
    const int zc = __ldg(zclass + k);
    const int ncol = nx * ny;
    for (int col = blockIdx.x; col < ncol; col += gridDim.x) {
        const int j = col % ny, i = col / ny;
        const long long c = (long long)col * nz + k;
        size_t q;
        long long s;
        int l, n;
        if (dir == 0) { q = ((size_t)zc * ny + j) * nx + i; s = (long long)nz * ny; l = i; n = nx; }
        else { q = ((size_t)zc * nx + i) * ny + j; s = nz; l = j; n = ny; }
        const T lc = src[c];
        T at = -(__ldg(cmt + q) + __ldg(cpt + q)) * lc;
        if (l > 0) at = fma(__ldg(cpt + q - 1), src[c - s], at);
        if (l < n - 1) at = fma(__ldg(cmt + q + 1), src[c + s], at);
        dst[c] = fma(h, at, lc);
    }
}

// (I - h A_dir)^T U = R on every line.  The factors give M = Lt Ut with Lt
// lower bidiagonal (diagonal 1/ib_l, sub-diagonal a_l) and Ut unit upper
// (super-diagonal cu_l), so M^T = Ut^T Lt^T:
//   forward  z_l = R_l - cu_{l-1} z_{l-1}
//   backward x_l = (z_l - a_{l+1} x_{l+1}) ib_l
template <typename T, bool PARAM>
__global__ void __launch_bounds__(128) k_thomas_t(T *__restrict__ U, const T *__restrict__ R,
                                                  const int *__restrict__ zclass, const T *__restrict__ fa,
                                                  const T *__restrict__ fib, const T *__restrict__ fcu,
                                                  int nx, int ny, int nz, int dir, double *__restrict__ G,
                                                  const T *__restrict__ phi, const T *__restrict__ lam2,
                                                  const T *__restrict__ wm, const T *__restrict__ wp,
                                                  const unsigned char *__restrict__ rock, double beta) {
    const int nl = dir == 0 ? ny : nx;
    const int N = dir == 0 ? nx : ny;
    long long L = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (L >= (long long)nz * nl) return;
    const int k = (int)(L % nz);
    const int m = (int)(L / nz);
    const int zc = __ldg(zclass + k);
    const size_t fb = ((size_t)zc * nl + m) * N;
    long long stride, off0;
    if (dir == 0) { stride = (long long)nz * ny; off0 = k + (long long)nz * m; }
    else { stride = nz; off0 = k + (long long)nz * ny * m; }
    T z = T(0), cprev = T(0);
    for (int l = 0; l < N; ++l) {
        const long long o = off0 + l * stride;
        z = fma(-cprev, z, R[o]);
        U[o] = z;
        cprev = __ldg(fcu + fb + l);
    }
    // rock flags along the line: rock[(zc * nx + i) * ny + j]
    const unsigned char *rk = rock + (size_t)zc * nx * ny;
    const long long rst = dir == 0 ? (long long)ny : 1;
    const long long r0 = dir == 0 ? m : (long long)m * ny;
    const long long oN = off0 + (long long)(N - 1) * stride;
    T x = z * __ldg(fib + fb + N - 1);
    U[oN] = x;
    T acc = T(0), lnext = T(0), fnext = T(0);
    int rnext = 0;
    if (PARAM) {
        lnext = x + (lam2 ? lam2[oN] : T(0));
        fnext = phi[oN];
        rnext = __ldg(rk + r0 + (N - 1) * rst);
    }
    for (int l = N - 2; l >= 0; --l) {
        const long long o = off0 + l * stride;
        x = fma(-__ldg(fa + fb + l + 1), x, U[o]) * __ldg(fib + fb + l);
        U[o] = x;
        if (PARAM) {
            // face (l, l+1): (phi_{l+1} - phi_l)(L_l wp_l - L_{l+1} wm_{l+1}), both cells' rock flags
            const T lc = x + (lam2 ? lam2[o] : T(0));
            const T fc = phi[o];
            const int rc = __ldg(rk + r0 + l * rst);
            acc += T(rc + rnext) * ((fnext - fc) * (lc * __ldg(wp + fb + l) - lnext * __ldg(wm + fb + l + 1)));
            lnext = lc;
            fnext = fc;
            rnext = rc;
        }
    }
    if (PARAM && acc != T(0)) atomicAdd(G + k, beta * (double)acc);
}

// ---------------------------------------------------------------------------
// conductivity derivatives: G[k] += beta * d(lambda^T A phi)/dk summed over the
// rock cells of level k (the face terms of gw_build_adjoint_tables).  One
// thread per level, looping over a strided share of the columns; one atomic
// per thread.  Face terms are formed and summed per thread in the storage
// type (a few hundred columns each); the per-level totals are double.
// Tref (mixed path, z only): phi is theta and T_ref's differences are added.

template <typename T>
__global__ void __launch_bounds__(128) k_param_z(double *__restrict__ G, const T *__restrict__ lam,
                                                 const T *__restrict__ phi, const double *__restrict__ Tref,
                                                 const int *__restrict__ colprof, const T *__restrict__ wzm,
                                                 const T *__restrict__ wzp, const int *__restrict__ zclass,
                                                 const unsigned char *__restrict__ rock, long long ncol,
                                                 int nz, double beta) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nz) return;
    const unsigned char *rk = rock + (size_t)__ldg(zclass + k) * ncol;   // [(zc * nx + i) * ny + j]
    const T dtp = (Tref && k < nz - 1) ? T(Tref[k + 1] - Tref[k]) : T(0);
    const T dtm = (Tref && k > 0) ? T(Tref[k] - Tref[k - 1]) : T(0);
    T acc = T(0);
    for (long long col = blockIdx.y; col < ncol; col += gridDim.y) {
        if (!__ldg(rk + col)) continue;
        const long long c = col * nz + k;
        const size_t pb = (size_t)__ldg(colprof + col) * nz + k;
        const T lk = lam[c], fk = phi[c];
        T d = T(0);
        if (k < nz - 1) d = (phi[c + 1] - fk + dtp) * (lk * __ldg(wzp + pb) - lam[c + 1] * __ldg(wzm + pb + 1));
        if (k > 0) d += (fk - phi[c - 1] + dtm) * (lam[c - 1] * __ldg(wzp + pb - 1) - lk * __ldg(wzm + pb));
        acc += d;
    }
    if (acc != T(0)) atomicAdd(G + k, beta * (double)acc);
}

// x (dir 0) and y (dir 1): each face (l, l+1) of the level counted once, its
// term attributed to both cells (same level).
template <typename T>
__global__ void __launch_bounds__(128) k_param_xy(double *__restrict__ G, const T *__restrict__ lam,
                                                  const T *__restrict__ phi, const int *__restrict__ zclass,
                                                  const T *__restrict__ wm, const T *__restrict__ wp,
                                                  const unsigned char *__restrict__ rock, int nx, int ny,
                                                  int nz, double beta, int dir) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nz) return;
    const long long ncol = (long long)nx * ny;
    const int zc = __ldg(zclass + k);
    const unsigned char *rk = rock + (size_t)zc * ncol;
    T acc = T(0);
    constexpr int U = 4;
    for (long long c0 = blockIdx.y; c0 < ncol; c0 += (long long)U * gridDim.y) {
        T d[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const long long col = c0 + (long long)u * gridDim.y;
            const int i = (int)(col / ny), j = (int)(col % ny);
            // the face (l, l+1) exists when l is not the last point of the line
            const bool ok = col < ncol && (dir == 0 ? i < nx - 1 : j < ny - 1);
            const long long cc = ok ? col : 0;
            const long long col2 = ok ? (dir == 0 ? cc + ny : cc + 1) : 0;
            const int ii = ok ? i : 0, jj = ok ? j : 0;
            const size_t q = dir == 0 ? ((size_t)zc * ny + jj) * nx + ii : ((size_t)zc * nx + ii) * ny + jj;
            const long long c = cc * nz + k, c2 = col2 * nz + k;
            const T r = ok ? T((int)__ldg(rk + cc) + (int)__ldg(rk + col2)) : T(0);
            d[u] = r * ((phi[c2] - phi[c]) * (lam[c] * __ldg(wp + q) - lam[c2] * __ldg(wm + q + 1)));
        }
#pragma unroll
        for (int u = 0; u < U; ++u) acc += d[u];
    }
    if (acc != T(0)) atomicAdd(G + k, beta * (double)acc);
}

// ---------------------------------------------------------------------------
// advection transpose

// The field the forward advection read, at pipe column q and level k, as an
// absolute temperature: from the full field (double path) or from the compact
// swept pipe columns [q][nz] plus T_ref (mixed path).
template <typename T>
struct PipeField {
    const T *full;        // full field, or null
    const T *tp;          // [ncol][nz], or null
    const double *Tref;   // with tp
    const int *pi, *pj;
    int ny, nz;
    __device__ __forceinline__ double at(int q, int k) const {
        if (tp) return (double)tp[(size_t)q * nz + k] + Tref[k];
        return (double)full[k + (long long)nz * (pj[q] + (long long)ny * pi[q])];
    }
};

// The advected cells (pipe columns, levels < countz, z <= h) take no part of
// their own old value: move their adjoint to tmp and clear it in the field.
template <typename T>
__global__ void __launch_bounds__(kB) k_adv_t_gather(double *__restrict__ tmp, T *__restrict__ a,
                                                     const double *__restrict__ gz, const int *__restrict__ pi,
                                                     const int *__restrict__ pj, const int *__restrict__ pb,
                                                     const GwBhDev *__restrict__ bh, int ncol, int ny, int nz,
                                                     int countz) {
    long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (long long)ncol * countz) return;
    const int k = (int)(e % countz);
    const int q = (int)(e / countz);
    if (gz[k] > bh[pb[q]].h) { tmp[e] = 0.0; return; }
    const long long cell = k + (long long)nz * (pj[q] + (long long)ny * pi[q]);
    tmp[e] = (double)a[cell];
    a[cell] = T(0);
}

__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Scatter-add of every advected value's adjoint onto the cells it was
// interpolated from, plus the derivatives with respect to v_inner / v_outer
// (through the departure points) and the inlet adjoint, with the departure
// records of the forward (k_adv_table).  phi is the field the forward
// advection read.  Turnaround cells are left to k_turn_apply.
template <typename T>
__global__ void __launch_bounds__(kB) k_adv_t_scatter(
    T *__restrict__ a, const double *__restrict__ tmp, PipeField<T> phi, const GwAdvRec *__restrict__ tab,
    const double *__restrict__ gz, const int *__restrict__ pi, const int *__restrict__ pj,
    const int *__restrict__ pb, double *__restrict__ sc, int n_inner, int ncol, int ny, int nz, int countz,
    double dt) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    double dvi = 0.0, dvo = 0.0, ib = 0.0;
    int b = -1;
    if (e < (long long)ncol * countz) {
        const int k = (int)(e % countz);
        const int q = (int)(e / countz);
        b = pb[q];
        const double ab = tmp[e];
        const bool inner = q < n_inner;
        const GwAdvRec r = tab[((size_t)b * countz + k) * 2 + (inner ? 0 : 1)];
        if (ab != 0.0) {
            if (r.type == kAdvInlet) {
                ib += ab;
            } else if (r.type == kAdvInterp) {
                const long long col = (long long)nz * (pj[q] + (long long)ny * pi[q]);
                atomicAdd(a + col + r.ir, T(r.alpha * ab));
                atomicAdd(a + col + r.il, T((1.0 - r.alpha) * ab));
                if (r.ir != r.il) {
                    const double s = (phi.at(q, r.ir) - phi.at(q, r.il)) / (gz[r.ir] - gz[r.il]) * ab * dt;
                    if (inner) dvi += s;   // d zd / d v_inner = dt
                    else dvo -= s;         // d zd / d v_outer = -dt
                }
            }
            // kAdvTurn: summed over the inner columns per level (k_turn_apply); kAdvKeep: z > h
        }
    }
    const int b0 = __shfl_sync(0xffffffffu, b, 0);
    if (__all_sync(0xffffffffu, b == b0 || b < 0)) {
        dvi = warp_sum(dvi);
        dvo = warp_sum(dvo);
        ib = warp_sum(ib);
        if ((threadIdx.x & 31) == 0 && b0 >= 0) {
            if (dvi != 0.0) atomicAdd(sc + 4 * b0 + 0, dvi);
            if (dvo != 0.0) atomicAdd(sc + 4 * b0 + 1, dvo);
            if (ib != 0.0) atomicAdd(sc + 4 * b0 + 2, ib);
        }
    } else if (b >= 0) {
        if (dvi != 0.0) atomicAdd(sc + 4 * b + 0, dvi);
        if (dvo != 0.0) atomicAdd(sc + 4 * b + 1, dvo);
        if (ib != 0.0) atomicAdd(sc + 4 * b + 2, ib);
    }
}

// Annulus cells take their share of the turnaround means' adjoint; inner
// cells in the outlet window (z <= v_inner dt, src/solver.jl:273-281) their
// share of the outlet adjoint  ob_scale * mdot_b + ob_add  plus, for the
// heat-exchanger inlet (T_in = T_out - dT), the inlet adjoint of this call.
template <typename T>
__global__ void __launch_bounds__(kB) k_adv_t_fin(T *__restrict__ a, const double *__restrict__ mbar,
                                                  const double *__restrict__ sc, const double *__restrict__ gz,
                                                  const int *__restrict__ pi, const int *__restrict__ pj,
                                                  const int *__restrict__ pb, const GwBhDev *__restrict__ bh,
                                                  int n_inner, int ncol, int ny, int nz, double dt,
                                                  int inlet_kind, double ob_scale, double ob_add) {
    long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (long long)ncol * nz) return;
    const int k = (int)(e % nz);
    const int q = (int)(e / nz);
    const int b = pb[q];
    const GwBhDev B = bh[b];
    const long long cell = k + (long long)nz * (pj[q] + (long long)ny * pi[q]);
    if (q < n_inner) {
        const double zmax = B.v_inner * dt;
        if (gz[k] > zmax) return;
        int lo = 0, hi = nz;   // levels with gz <= zmax are a prefix
        while (lo < hi) {
            int mid = (lo + hi) >> 1;
            if (gz[mid] <= zmax) lo = mid + 1; else hi = mid;
        }
        double ob = ob_scale * B.mdot + ob_add;
        if (inlet_kind == GW_INLET_HEAT_EXCHANGER) ob += sc[4 * b + 2];
        if (ob != 0.0) a[cell] += T(ob / ((double)B.inner_count * (double)lo));
    } else {
        const double mb = mbar[(size_t)b * nz + k];
        if (mb != 0.0) a[cell] += T(mb / (double)B.outer_count);
    }
}

// Close one advection call: accumulate its inlet adjoint.
__global__ void k_adv_t_close(double *sc, int nbh) {
    const int b = threadIdx.x;
    if (b < nbh) {
        sc[4 * b + 3] += sc[4 * b + 2];
        sc[4 * b + 2] = 0.0;
    }
}

// Per step: sum of T_out - T_in (the flow-rate derivative of the energy).
__global__ void k_osum(double *osum, const double *outlet, int nbh, int inlet_kind, double inlet_param) {
    const int b = threadIdx.x;
    if (b < nbh) {
        const double to = outlet[b];
        const double ti = inlet_kind == GW_INLET_CONSTANT ? inlet_param : to - inlet_param;
        osum[b] += to - ti;
    }
}

// Annulus means per borehole and level of the field the forward advection
// read: 32 levels x 8 column groups per block, then a sum over the groups.
template <typename T>
__global__ void __launch_bounds__(256) k_ann_mean(double *__restrict__ mean, PipeField<T> phi,
                                                  const GwBhDev *__restrict__ bh, int nz) {
    __shared__ double red[8][32];
    const int b = blockIdx.y;
    const int lane = threadIdx.x & 31, grp = threadIdx.x >> 5;
    const int k = blockIdx.x * 32 + lane;
    const GwBhDev B = bh[b];
    double s = 0.0;
    if (k < nz)
        for (int q = B.outer_begin + grp; q < B.outer_begin + B.outer_count; q += 8) s += phi.at(q, k);
    red[grp][lane] = s;
    __syncthreads();
    if (grp == 0 && k < nz) {
        double t = 0.0;
#pragma unroll
        for (int g = 0; g < 8; ++g) t += red[g][lane];
        mean[(size_t)b * nz + k] = t / (double)B.outer_count;
    }
}

// Sum over a borehole's inner columns of the advected values' adjoint, per
// level (the turnaround cells of one level share their interpolation).
__global__ void __launch_bounds__(256) k_inner_sum(double *__restrict__ S, const double *__restrict__ tmp,
                                                   const GwBhDev *__restrict__ bh, int countz) {
    __shared__ double red[8][32];
    const int b = blockIdx.y;
    const int lane = threadIdx.x & 31, grp = threadIdx.x >> 5;
    const int k = blockIdx.x * 32 + lane;
    const GwBhDev B = bh[b];
    double s = 0.0;
    if (k < countz)
        for (int q = B.inner_begin + grp; q < B.inner_begin + B.inner_count; q += 8) s += tmp[(size_t)q * countz + k];
    red[grp][lane] = s;
    __syncthreads();
    if (grp == 0 && k < countz) {
        double t = 0.0;
#pragma unroll
        for (int g = 0; g < 8; ++g) t += red[g][lane];
        S[(size_t)b * countz + k] = t;
    }
}

// Turnaround cells, per borehole and level: the level's summed adjoint goes
// to the annulus means it was interpolated from, and the v_inner / v_outer
// derivatives through the turnaround departure point.
__global__ void k_turn_apply(double *__restrict__ mbar, double *__restrict__ sc, const double *__restrict__ S,
                             const double *__restrict__ mean, const GwAdvRec *__restrict__ tab,
                             const double *__restrict__ gz, const GwBhDev *__restrict__ bh, int nz, int countz,
                             double dt) {
    const int b = blockIdx.y;
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    double dvi = 0.0, dvo = 0.0;
    if (k < countz) {
        const GwAdvRec r = tab[((size_t)b * countz + k) * 2];
        const double ab = S[(size_t)b * countz + k];
        if (r.type == kAdvTurn && ab != 0.0) {
            const GwBhDev B = bh[b];
            const double dt1 = __ddiv_rn(__dsub_rn(B.h, gz[k]), B.v_inner);
            const double dt2 = __dsub_rn(dt, dt1);
            atomicAdd(mbar + (size_t)b * nz + r.ir, r.alpha * ab);
            atomicAdd(mbar + (size_t)b * nz + r.il, (1.0 - r.alpha) * ab);
            if (r.ir != r.il) {
                const double *m = mean + (size_t)b * nz;
                const double sl = (m[r.ir] - m[r.il]) / (gz[r.ir] - gz[r.il]) * ab;
                dvo = -sl * dt2;                           // d zd2 / d v_outer = -dt2
                dvi = -sl * B.v_outer * dt1 / B.v_inner;   // d zd2 / d v_inner
            }
        }
    }
    dvi = warp_sum(dvi);
    dvo = warp_sum(dvo);
    if ((threadIdx.x & 31) == 0) {
        if (dvi != 0.0) atomicAdd(sc + 4 * b + 0, dvi);
        if (dvo != 0.0) atomicAdd(sc + 4 * b + 1, dvo);
    }
}

__global__ void k_to_double(double *__restrict__ out, const float *__restrict__ in, long long n) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = (double)in[i];
}

// ---------------------------------------------------------------------------
// host side

int ensure_adj(gw_ctx *c) {
    if (c->adj) return GW_OK;
    GwAdj *a = new GwAdj();
    c->adj = a;
    std::vector<double> wxm, wxp, wym, wyp, wzm, wzp;
    std::vector<unsigned char> rock;
    gw_build_adjoint_tables(c, wxm, wxp, wym, wyp, wzm, wzp, rock, a->layer);
    auto f = [](const std::vector<double> &v) { return std::vector<float>(v.begin(), v.end()); };
    const int ncol = c->n_inner + c->n_outer;
    int rc;
    if ((rc = adj_upload(a, &a->wxm, wxm)) || (rc = adj_upload(a, &a->wxp, wxp)) ||
        (rc = adj_upload(a, &a->wym, wym)) || (rc = adj_upload(a, &a->wyp, wyp)) ||
        (rc = adj_upload(a, &a->wzm, wzm)) || (rc = adj_upload(a, &a->wzp, wzp)) ||
        (rc = adj_upload(a, &a->fxm, f(wxm))) || (rc = adj_upload(a, &a->fxp, f(wxp))) ||
        (rc = adj_upload(a, &a->fym, f(wym))) || (rc = adj_upload(a, &a->fyp, f(wyp))) ||
        (rc = adj_upload(a, &a->fzm, f(wzm))) || (rc = adj_upload(a, &a->fzp, f(wzp))) ||
        (rc = adj_upload(a, &a->rock, rock)) || (rc = adj_alloc(a, &a->G, (size_t)c->nz)) ||
        (rc = adj_alloc(a, &a->sc, (size_t)4 * c->nbh)) || (rc = adj_alloc(a, &a->osum, (size_t)c->nbh)) ||
        (rc = adj_alloc(a, &a->mbar, (size_t)c->nbh * c->nz)) ||
        (rc = adj_alloc(a, &a->tmp, (size_t)std::max(ncol, 1) * std::max(c->countz, 1))) ||
        (rc = adj_alloc(a, &a->S, (size_t)c->nbh * std::max(c->countz, 1)))) {
        gw_adjoint_release(c);
        return rc;
    }
    return GW_OK;
}

int zero_acc(gw_ctx *c) {
    GwAdj *a = c->adj;
    GW_CUDA(cudaMemsetAsync(a->G, 0, sizeof(double) * c->nz, c->stream));
    GW_CUDA(cudaMemsetAsync(a->sc, 0, sizeof(double) * 4 * c->nbh, c->stream));
    GW_CUDA(cudaMemsetAsync(a->osum, 0, sizeof(double) * c->nbh, c->stream));
    return GW_OK;
}

// per-cell kernels: blocks of kB levels (y) walking a strided share of the
// columns (x), about 8 resident blocks per SM
dim3 cell_grid(const gw_ctx *c) {
    const int by = (c->nz + kB - 1) / kB;
    long long bx = std::max(1LL, (152LL * 8) / by);
    bx = std::min(bx, (long long)c->nx * c->ny);
    return dim3((unsigned)bx, (unsigned)by);
}

dim3 param_grid(const gw_ctx *c) {
    const long long ncol = (long long)c->nx * c->ny;
    const int bx = (c->nz + 127) / 128;
    long long by = std::max(1LL, (152LL * 2048) / ((long long)bx * 128));
    by = std::min(by, ncol);
    by = std::min(by, 65535LL);
    return dim3((unsigned)bx, (unsigned)by);
}

// Per-precision views of the context's tables.
template <typename T>
struct Tabs {
    const GwCoefTables<T> *ct;
    const T *wxm, *wxp, *wym, *wyp, *wzm, *wzp;
    const double *Tref;    // mixed path: T_ref, for the z face terms
};
Tabs<double> tabs(gw_ctx *c, double *) {
    GwAdj *a = c->adj;
    return {&c->c64, a->wxm, a->wxp, a->wym, a->wyp, a->wzm, a->wzp, nullptr};
}
Tabs<float> tabs(gw_ctx *c, float *) {
    GwAdj *a = c->adj;
    return {&c->c32, a->fxm, a->fxp, a->fym, a->fyp, a->fzm, a->fzp, c->d_Tref};
}

template <typename T>
int launch_param(gw_ctx *c, const T *lam, const T *phi, double beta, int dir) {
    GwAdj *a = c->adj;
    Tabs<T> tb = tabs(c, (T *)nullptr);
    dim3 g = param_grid(c);
    if (dir == GW_DIR_Z)
        k_param_z<T><<<g, 128, 0, c->stream>>>(a->G, lam, phi, tb.Tref, c->d_colprof, tb.wzm, tb.wzp,
                                               c->d_zclass, a->rock, (long long)c->nx * c->ny, c->nz, beta);
    else
        k_param_xy<T><<<g, 128, 0, c->stream>>>(a->G, lam, phi, c->d_zclass, dir == GW_DIR_X ? tb.wxm : tb.wym,
                                                dir == GW_DIR_X ? tb.wxp : tb.wyp, a->rock, c->nx, c->ny,
                                                c->nz, beta, dir);
    GW_CUDA(cudaGetLastError());
    return GW_OK;
}

template <typename T>
int launch_zstage_t(gw_ctx *c, T *out, const T *lam, const T *w, double a1, double hmu, double a2) {
    Tabs<T> tb = tabs(c, (T *)nullptr);
    k_zstage_t<T><<<cell_grid(c), kB, 0, c->stream>>>(out, lam, w, c->d_colprof, tb.ct->czm, tb.ct->czp, c->nz,
                                                     (long long)c->nx * c->ny, (T)a1, (T)hmu, (T)a2);
    GW_CUDA(cudaGetLastError());
    return GW_OK;
}

template <typename T>
int launch_explicit_t(gw_ctx *c, T *dst, const T *src, double h, int dir) {
    Tabs<T> tb = tabs(c, (T *)nullptr);
    const T *cm = dir == GW_DIR_X ? tb.ct->cxm : tb.ct->cym;
    const T *cp = dir == GW_DIR_X ? tb.ct->cxp : tb.ct->cyp;
    k_explicit_t<T><<<cell_grid(c), kB, 0, c->stream>>>(dst, src, c->d_zclass, cm, cp, c->nx, c->ny, c->nz,
                                                       (T)h, dir);
    GW_CUDA(cudaGetLastError());
    return GW_OK;
}

template <typename T>
int launch_thomas_t(gw_ctx *c, T *U, const T *R, int dir, const T *phi = nullptr, const T *lam2 = nullptr,
                    double beta = 0.0) {
    const long long lines = (long long)c->nz * (dir == GW_DIR_X ? c->ny : c->nx);
    Tabs<T> tb = tabs(c, (T *)nullptr);
    const GwFactors<T> &f = dir == GW_DIR_X ? tb.ct->fx : tb.ct->fy;
    const T *wm = dir == GW_DIR_X ? tb.wxm : tb.wym;
    const T *wp = dir == GW_DIR_X ? tb.wxp : tb.wyp;
    // with phi: the conductivity face terms of (lambda + lam2)^T A phi along the lines, lambda the solution
    if (phi)
        k_thomas_t<T, true><<<nblocks(lines, 128), 128, 0, c->stream>>>(
            U, R, c->d_zclass, f.a, f.ib, f.cu, c->nx, c->ny, c->nz, dir, c->adj->G, phi, lam2, wm, wp,
            c->adj->rock, beta);
    else
        k_thomas_t<T, false><<<nblocks(lines, 128), 128, 0, c->stream>>>(
            U, R, c->d_zclass, f.a, f.ib, f.cu, c->nx, c->ny, c->nz, dir, nullptr, nullptr, nullptr, nullptr,
            nullptr, nullptr, 0.0);
    GW_CUDA(cudaGetLastError());
    return GW_OK;
}

// Transpose of one advection call (half step h) in place on a; phi = the
// field the forward call read.
template <typename T>
int advection_t(gw_ctx *c, T *a, PipeField<T> phi, double h, double ob_scale, double ob_add) {
    GwAdj *ad = c->adj;
    const int ncol = c->n_inner + c->n_outer;
    if (ncol == 0) return GW_OK;
    dim3 gm((c->nz + 31) / 32, c->nbh);
    k_ann_mean<T><<<gm, 256, 0, c->stream>>>(c->d_annmean, phi, c->d_bh, c->nz);
    GW_CUDA(cudaGetLastError());
    GW_CUDA(cudaMemsetAsync(ad->mbar, 0, sizeof(double) * c->nbh * c->nz, c->stream));
    if (c->countz > 0) {
        const long long n = (long long)ncol * c->countz;
        k_adv_t_gather<T><<<nblocks(n, kB), kB, 0, c->stream>>>(ad->tmp, a, c->d_gz, c->d_pipe_i, c->d_pipe_j,
                                                               c->d_pipe_b, c->d_bh, ncol, c->ny, c->nz,
                                                               c->countz);
        GW_CUDA(cudaGetLastError());
        k_inner_sum<<<dim3((c->countz + 31) / 32, c->nbh), 256, 0, c->stream>>>(ad->S, ad->tmp, c->d_bh, c->countz);
        GW_CUDA(cudaGetLastError());
        k_adv_t_scatter<T><<<nblocks(n, kB), kB, 0, c->stream>>>(
            a, ad->tmp, phi, c->d_advtab, c->d_gz, c->d_pipe_i, c->d_pipe_j, c->d_pipe_b, ad->sc, c->n_inner,
            ncol, c->ny, c->nz, c->countz, h);
        GW_CUDA(cudaGetLastError());
        k_turn_apply<<<dim3((c->countz + 127) / 128, c->nbh), 128, 0, c->stream>>>(
            ad->mbar, ad->sc, ad->S, c->d_annmean, c->d_advtab, c->d_gz, c->d_bh, c->nz, c->countz, h);
        GW_CUDA(cudaGetLastError());
    }
    const long long nf = (long long)ncol * c->nz;
    k_adv_t_fin<T><<<nblocks(nf, kB), kB, 0, c->stream>>>(a, ad->mbar, ad->sc, c->d_gz, c->d_pipe_i,
                                                         c->d_pipe_j, c->d_pipe_b, c->d_bh, c->n_inner, ncol,
                                                         c->ny, c->nz, h, c->inlet_kind, ob_scale, ob_add);
    GW_CUDA(cudaGetLastError());
    k_adv_t_close<<<1, ((c->nbh + 31) / 32) * 32, 0, c->stream>>>(ad->sc, c->nbh);
    GW_CUDA(cudaGetLastError());
    return GW_OK;
}

// Buffers of one step's forward intermediates.
template <typename T>
struct StepStore {
    std::vector<T *> g;   // ROCK2 stages g_1 .. g_{s-2}, then g_q (s - 1 fields)
    T *ustar, *u1;        // after ROCK2, after the x half step
    T *tA, *tC, *work;    // double path: the fields the two advections read, scratch
    T *tpA, *tpC;         // mixed path: those fields at the pipe columns ([ncol][nz])
    PipeField<T> pA, pC;
};

int launch_osum(gw_ctx *c) {
    k_osum<<<1, ((c->nbh + 31) / 32) * 32, 0, c->stream>>>(c->adj->osum, c->d_outlet, c->nbh, c->inlet_kind,
                                                          c->inlet_param);
    GW_CUDA(cudaGetLastError());
    return GW_OK;
}

// Double path: recompute the step from un with the modular kernels, keeping
// what the adjoint reads: the ROCK2 stages, u* (after ROCK2), tA (before the
// first advection), u1 (after the x solve), tC (before the second
// advection).  un1 (optional) receives u^{n+1}.  Adds the step's T_out - T_in
// to osum.
int forward_store(gw_ctx *c, const double *un, StepStore<double> &S, double dt, int s, double *un1) {
    const double *mu, *nu, *kappa;
    double sigma, tau;
    gw_rock2_coefs(s, &mu, &nu, &kappa, &sigma, &tau);
    const size_t bytes = (size_t)c->nx * c->ny * c->nz * sizeof(double);
    int rc;
    const double *gm2 = nullptr, *gm1 = un;
    for (int j = 1; j <= s - 2; ++j) {
        double *out = S.g[j - 1];
        if ((rc = gw_launch_zstage(c, out, gm1, gm2, dt * mu[j - 1], j == 1 ? 0.0 : kappa[j - 1], 0)))
            return rc;
        gm2 = gm1;
        gm1 = out;
    }
    double *gq = S.g[s - 2];
    if ((rc = gw_launch_zstage(c, gq, gm1, nullptr, dt * sigma, 0.0, 0)) ||
        (rc = gw_launch_zstage(c, S.ustar, gq, gm1, dt * tau / sigma, 1.0 - tau / (sigma * sigma), 0)))
        return rc;
    const double h = dt / 2;
    if ((rc = gw_launch_explicit(c, S.tA, S.ustar, h, GW_DIR_Y))) return rc;
    GW_CUDA(cudaMemcpyAsync(S.work, S.tA, bytes, cudaMemcpyDeviceToDevice, c->stream));
    if ((rc = gw_launch_advection(c, S.work, h)) || (rc = gw_launch_thomas(c, S.u1, S.work, GW_DIR_X)) ||
        (rc = gw_launch_explicit(c, S.tC, S.u1, h, GW_DIR_X)))
        return rc;
    GW_CUDA(cudaMemcpyAsync(S.work, S.tC, bytes, cudaMemcpyDeviceToDevice, c->stream));
    if ((rc = gw_launch_advection(c, S.work, h)) || (rc = launch_osum(c))) return rc;
    if (un1 && (rc = gw_launch_thomas(c, un1, S.work, GW_DIR_Y))) return rc;
    return GW_OK;
}

// The context's state keeps its columns pz apart (the mixed path's padded
// level pitch), the adjoint's buffers nz apart: states cross with pitched
// copies (a plain copy when the pitches agree, as in FP64).
template <typename T>
int state_copy(gw_ctx *c, T *dst, int dpitch, const T *src, int spitch) {
    GW_CUDA(cudaMemcpy2DAsync(dst, (size_t)dpitch * sizeof(T), src, (size_t)spitch * sizeof(T),
                              (size_t)c->nz * sizeof(T), (size_t)c->nx * c->ny, cudaMemcpyDeviceToDevice,
                              c->stream));
    return GW_OK;
}

// Mixed path: the ROCK2 stages of theta from un (for the conductivity terms),
// then the fused ROCK2 columns and first half step on the context's state
// (u* and u1 copied out, the pipe columns of the two advections' inputs kept
// in tpA / tpC).
int forward_store(gw_ctx *c, const float *un, StepStore<float> &S, double dt, int s, float *) {
    const double *mu, *nu, *kappa;
    double sigma, tau;
    gw_rock2_coefs(s, &mu, &nu, &kappa, &sigma, &tau);
    const long long n = (long long)c->nx * c->ny * c->nz;
    const size_t bytes = (size_t)n * sizeof(float);
    const dim3 nb = cell_grid(c);
    const float *gm2 = nullptr, *gm1 = un;
    for (int j = 1; j <= s - 2; ++j) {
        float *out = S.g[j - 1];
        k_zstage_theta<<<nb, kB, 0, c->stream>>>(out, gm1, gm2, c->d_colprof, c->c32.czm, c->c32.czp, c->f_fref,
                                                 c->nz, (long long)c->nx * c->ny, (float)(dt * mu[j - 1]),
                                                 (float)(j == 1 ? 0.0 : kappa[j - 1]));
        GW_CUDA(cudaGetLastError());
        gm2 = gm1;
        gm1 = out;
    }
    k_zstage_theta<<<nb, kB, 0, c->stream>>>(S.g[s - 2], gm1, nullptr, c->d_colprof, c->c32.czm, c->c32.czp,
                                             c->f_fref, c->nz, (long long)c->nx * c->ny, (float)(dt * sigma), 0.f);
    GW_CUDA(cudaGetLastError());
    int rc;
    if ((rc = state_copy(c, c->f_u, c->pz, un, c->nz)) || (rc = gw_fused_adjoint_store(c, dt, s, S.tpA, S.tpC)) ||
        (rc = state_copy(c, S.ustar, c->nz, (const float *)c->f_u, c->pz)) ||
        (rc = state_copy(c, S.u1, c->nz, (const float *)c->f_temp, c->pz)))
        return rc;
    return launch_osum(c);
}

// Adjoint of one step.  B[0] holds dJ/du^{n+1} on entry; B[1], B[2] are
// scratch.  On return *res is the index of the buffer holding dJ/du^n.
// un = u^n, un1 = u^{n+1}; ob_scale / ob_add: the second advection's outlet
// adjoint (energy and final-outlet terms).
template <typename T>
int adjoint_step(gw_ctx *c, const T *un, const T *un1, StepStore<T> &S, T *B[3], double dt, int s,
                 double ob_scale, double ob_add, int *res) {
    const double *mu, *nu, *kappa;
    double sigma, tau;
    gw_rock2_coefs(s, &mu, &nu, &kappa, &sigma, &tau);
    const double h = dt / 2;
    int rc;
    // u^{n+1} = (I - h A_y)^{-1} t4  (face terms of t4bar^T A_y u^{n+1} in the same sweep)
    if ((rc = launch_thomas_t<T>(c, B[1], B[0], GW_DIR_Y, un1, (const T *)nullptr, h))) return rc;
    // t4 = advection(tC)
    if ((rc = advection_t<T>(c, B[1], S.pC, h, ob_scale, ob_add))) return rc;
    // tC = (I + h A_x) u1 ; u1 = (I - h A_x)^{-1} t2: both with A_x applied to u1,
    // so one sweep sums the face terms of (t2bar + tCbar)^T A_x u1
    if ((rc = launch_explicit_t<T>(c, B[2], B[1], h, GW_DIR_X)) ||
        (rc = launch_thomas_t<T>(c, B[0], B[2], GW_DIR_X, S.u1, B[1], h)))
        return rc;
    // t2 = advection(tA)
    if ((rc = advection_t<T>(c, B[0], S.pA, h, 0.0, 0.0))) return rc;
    // tA = (I + h A_y) u*
    if ((rc = launch_explicit_t<T>(c, B[1], B[0], h, GW_DIR_Y)) ||
        (rc = launch_param<T>(c, B[0], S.ustar, h, GW_DIR_Y)))
        return rc;
    // ROCK2: u* = gq + (dt tau/sigma) A gq + cc (gq - gp);  gq = gp + dt sigma A gp
    const double cc = 1.0 - tau / (sigma * sigma);
    const T *gq = S.g[s - 2];
    const T *gp = S.g[s - 3];
    if ((rc = launch_zstage_t<T>(c, B[2], B[1], nullptr, 1.0 + cc, dt * tau / sigma, 0.0)) ||
        (rc = launch_param<T>(c, B[1], gq, dt * tau / sigma, GW_DIR_Z)) ||
        (rc = launch_zstage_t<T>(c, B[1], B[2], B[1], 1.0, dt * sigma, -cc)) ||
        (rc = launch_param<T>(c, B[2], gp, dt * sigma, GW_DIR_Z)))
        return rc;
    // recurrence g_j = (1 + kappa_j) g_{j-1} + dt mu_j A g_{j-1} - kappa_j g_{j-2}, backwards
    int cur = 1, old = 2;
    for (int j = s - 2; j >= 1; --j) {
        const T *gprev = j == 1 ? un : S.g[j - 2];
        const double kj = j == 1 ? 0.0 : kappa[j - 1];
        if ((rc = launch_param<T>(c, B[cur], gprev, dt * mu[j - 1], GW_DIR_Z))) return rc;
        if (j == s - 2) rc = launch_zstage_t<T>(c, B[old], B[cur], nullptr, 1.0 + kj, dt * mu[j - 1], 0.0);
        else rc = launch_zstage_t<T>(c, B[old], B[cur], B[old], 1.0 + kj, dt * mu[j - 1], -kappa[j]);
        if (rc) return rc;
        std::swap(cur, old);
    }
    *res = cur;
    return GW_OK;
}

// Gradient from the accumulators: per-layer conductivities, flow rates,
// inlet parameter (nsteps: steps covered; wE: energy weight).
int finish_grad(gw_ctx *c, double dt, int nsteps, double wE, double *grad) {
    GwAdj *a = c->adj;
    std::vector<double> G(c->nz), sc(4 * (size_t)c->nbh), osum(c->nbh);
    GW_CUDA(cudaMemcpyAsync(G.data(), a->G, sizeof(double) * c->nz, cudaMemcpyDeviceToHost, c->stream));
    GW_CUDA(cudaMemcpyAsync(sc.data(), a->sc, sizeof(double) * sc.size(), cudaMemcpyDeviceToHost, c->stream));
    GW_CUDA(cudaMemcpyAsync(osum.data(), a->osum, sizeof(double) * c->nbh, cudaMemcpyDeviceToHost, c->stream));
    GW_CUDA(cudaStreamSynchronize(c->stream));
    const int nl = (int)c->k_layers.size();
    for (int k = 0; k < c->nz; ++k) grad[a->layer[k]] += G[k];
    const double pi = 3.141592653589793;
    const double c_w = c->rho_c_water / kRhoWater;
    double msum = 0.0, ibsum = 0.0;
    for (int b = 0; b < c->nbh; ++b) {
        const GwBorehole &B = c->bh[b];
        const double A_inner = pi * (B.r_inner * B.r_inner);
        const double A_outer = pi * B.r_outer_sq - pi * B.r_and_t_inner_sq;
        grad[nl + b] += sc[4 * b] / (A_inner * kRhoWater) + sc[4 * b + 1] / (A_outer * kRhoWater) +
                        wE * c_w * dt * osum[b];
        msum += B.mdot;
        ibsum += sc[4 * b + 3];
    }
    const double e = wE * c_w * dt * msum * nsteps;
    grad[nl + c->nbh] += c->inlet_kind == GW_INLET_CONSTANT ? ibsum - e : e - ibsum;
    return GW_OK;
}

int check_common(gw_ctx *c, double dt, int max_stages, int *s) {
    if (!(dt > 0) || !std::isfinite(dt)) return gw_fail(GW_ERR_ARG, "dt must be positive and finite");
    if (c->inlet_kind == GW_INLET_SCHEDULE || c->inlet_kind == GW_INLET_EXPRESSION)
        return gw_fail(GW_ERR_UNSUPPORTED, "the adjoint takes constant or heat-exchanger inlets");
    if (c->modular_reason & GW_MODULAR_SHARED_COLUMN)
        return gw_fail(GW_ERR_UNSUPPORTED, "the adjoint needs every pipe column in one borehole");
    int covered, rc;
    GW_CUDA(cudaSetDevice(c->device));
    if ((rc = gw_rock2_choose(dt, c->eigen_estimate, max_stages, s, &covered))) return rc;
    if ((rc = ensure_adj(c)) || (rc = gw_ensure_factors(c, dt / 2))) return rc;
    // the half step's departure table (gw_step keeps it for its own dt)
    return gw_fused_set_dt(c, dt);
}

struct DevBlock {
    void *p = nullptr;
    ~DevBlock() { if (p) cudaFree(p); }
};

template <typename T>
T *state_of(gw_ctx *c);
template <>
double *state_of<double>(gw_ctx *c) { return c->d_u; }
template <>
float *state_of<float>(gw_ctx *c) { return c->f_u; }

// The checkpointed adjoint for one storage type (see gw_adjoint).
template <typename T>
int adjoint_run(gw_ctx *c, double dt, int nsteps, int max_stages, int s, int checkpoint_every, double w_energy,
                double w_outlet, double *grad, double *grad_T0, gw_adjoint_info_t *info) {
    const size_t N = (size_t)c->nx * c->ny * c->nz;
    const size_t bytes = N * sizeof(T);
    const bool mix = sizeof(T) == 4;
    const int ncol = c->n_inner + c->n_outer;
    const size_t tpn = (size_t)std::max(ncol, 1) * c->nz;
    const int K = std::min(checkpoint_every, nsteps);
    const int nseg = (nsteps + K - 1) / K;
    // checkpoints, one segment's states, the step store, adjoint buffers, final state
    const size_t nbuf = (size_t)nseg + (K + 1) + (s - 1) + (mix ? 2 : 5) + 3 + 1;
    const size_t total = nbuf * bytes + (mix ? 2 * tpn * sizeof(T) : 0);
    DevBlock blk;
    cudaError_t e = cudaMalloc(&blk.p, total);
    if (e != cudaSuccess) return gw_cuda_fail(e, "cudaMalloc (adjoint checkpoints and buffers)");
    T *p = (T *)blk.p;
    std::vector<T *> ckpt(nseg), seg(K + 1);
    for (int q = 0; q < nseg; ++q, p += N) ckpt[q] = p;
    for (int q = 0; q <= K; ++q, p += N) seg[q] = p;
    StepStore<T> S;
    for (int q = 0; q < s - 1; ++q, p += N) S.g.push_back(p);
    S.ustar = p; p += N; S.u1 = p; p += N;
    if (!mix) { S.tA = p; p += N; S.tC = p; p += N; S.work = p; p += N; }
    else { S.tA = S.tC = S.work = nullptr; }
    T *B[3] = {p, p + N, p + 2 * N};
    p += 3 * N;
    T *uN = p;
    p += N;
    S.tpA = mix ? p : nullptr;
    S.tpC = mix ? p + tpn : nullptr;
    S.pA = {S.tA, S.tpA, mix ? c->d_Tref : nullptr, c->d_pipe_i, c->d_pipe_j, c->ny, c->nz};
    S.pC = {S.tC, S.tpC, mix ? c->d_Tref : nullptr, c->d_pipe_i, c->d_pipe_j, c->ny, c->nz};
    T *u = state_of<T>(c);

    cudaEvent_t e0, e1, e2;
    GW_CUDA(cudaEventCreate(&e0));
    GW_CUDA(cudaEventCreate(&e1));
    GW_CUDA(cudaEventCreate(&e2));
    struct EvGuard { cudaEvent_t a, b, c; ~EvGuard() { cudaEventDestroy(a); cudaEventDestroy(b); cudaEventDestroy(c); } } eg{e0, e1, e2};

    // forward sweep with checkpoints
    std::vector<double> E0(c->nbh), E(c->nbh), O(c->nbh);
    GW_CUDA(cudaMemcpyAsync(E0.data(), c->d_energy, sizeof(double) * c->nbh, cudaMemcpyDeviceToHost, c->stream));
    GW_CUDA(cudaStreamSynchronize(c->stream));
    GW_CUDA(cudaMemsetAsync(c->d_energy, 0, sizeof(double) * c->nbh, c->stream));
    GW_CUDA(cudaEventRecord(e0, c->stream));
    int rc;
    for (int q = 0; q < nseg; ++q) {
        if ((rc = state_copy(c, ckpt[q], c->nz, (const T *)u, c->pz))) return rc;
        const int n = std::min(K, nsteps - q * K);
        if ((rc = gw_step(c, (double)q * K * dt, dt, n, max_stages))) return rc;
    }
    if ((rc = state_copy(c, uN, c->nz, (const T *)u, c->pz))) return rc;
    GW_CUDA(cudaEventRecord(e1, c->stream));
    GW_CUDA(cudaMemcpyAsync(E.data(), c->d_energy, sizeof(double) * c->nbh, cudaMemcpyDeviceToHost, c->stream));
    GW_CUDA(cudaMemcpyAsync(O.data(), c->d_outlet, sizeof(double) * c->nbh, cudaMemcpyDeviceToHost, c->stream));
    GW_CUDA(cudaStreamSynchronize(c->stream));
    double J = 0.0;
    for (int b = 0; b < c->nbh; ++b) J += w_energy * E[b] + w_outlet * O[b];

    // reverse sweep
    if ((rc = zero_acc(c))) return rc;
    GW_CUDA(cudaMemsetAsync(B[0], 0, bytes, c->stream));
    const double c_w = c->rho_c_water / kRhoWater;
    const double ob_scale = c->inlet_kind == GW_INLET_CONSTANT ? w_energy * c_w * dt : 0.0;
    for (int q = nseg - 1; q >= 0; --q) {
        const int n = std::min(K, nsteps - q * K);
        GW_CUDA(cudaMemcpyAsync(seg[0], ckpt[q], bytes, cudaMemcpyDeviceToDevice, c->stream));
        if ((rc = state_copy(c, u, c->pz, (const T *)ckpt[q], c->nz))) return rc;
        for (int m = 1; m <= n; ++m) {
            if ((rc = gw_step(c, (double)(q * K + m - 1) * dt, dt, 1, max_stages)) ||
                (rc = state_copy(c, seg[m], c->nz, (const T *)u, c->pz)))
                return rc;
        }
        for (int m = n - 1; m >= 0; --m) {
            const bool last = q * K + m == nsteps - 1;
            int res = 0;
            if ((rc = forward_store(c, seg[m], S, dt, s, (T *)nullptr)) ||
                (rc = adjoint_step<T>(c, seg[m], seg[m + 1], S, B, dt, s, ob_scale, last ? w_outlet : 0.0, &res)))
                return rc;
            if (res != 0) std::swap(B[0], B[res]);
        }
    }
    GW_CUDA(cudaEventRecord(e2, c->stream));
    if (grad_T0) {
        if (mix) {
            k_to_double<<<nblocks((long long)N, kB), kB, 0, c->stream>>>(grad_T0, (const float *)B[0], (long long)N);
            GW_CUDA(cudaGetLastError());
        } else {
            GW_CUDA(cudaMemcpyAsync(grad_T0, B[0], bytes, cudaMemcpyDeviceToDevice, c->stream));
        }
    }
    // leave the context as gw_step over nsteps would (field, outlet, energy)
    if ((rc = state_copy(c, u, c->pz, (const T *)uN, c->nz))) return rc;
    for (int b = 0; b < c->nbh; ++b) E[b] += E0[b];
    GW_CUDA(cudaMemcpyAsync(c->d_energy, E.data(), sizeof(double) * c->nbh, cudaMemcpyHostToDevice, c->stream));
    GW_CUDA(cudaMemcpyAsync(c->d_outlet, O.data(), sizeof(double) * c->nbh, cudaMemcpyHostToDevice, c->stream));
    const int npar = (int)c->k_layers.size() + c->nbh + 1;
    for (int q = 0; q < npar; ++q) grad[q] = 0.0;
    if ((rc = finish_grad(c, dt, nsteps, w_energy, grad))) return rc;
    if (info) {
        float f_ms = 0.f, r_ms = 0.f;
        GW_CUDA(cudaEventElapsedTime(&f_ms, e0, e1));
        GW_CUDA(cudaEventElapsedTime(&r_ms, e1, e2));
        info->objective = J;
        info->n_params = npar;
        info->stages = s;
        info->checkpoints = nseg;
        info->forward_ms = f_ms;
        info->reverse_ms = r_ms;
        info->peak_bytes = c->device_bytes + c->adj->bytes + (long long)total;
    }
    return GW_OK;
}

}  // namespace

void gw_adjoint_release(gw_ctx *c) {
    if (!c || !c->adj) return;
    for (void *p : c->adj->allocs) if (p) cudaFree(p);
    delete c->adj;
    c->adj = nullptr;
}

extern "C" int gw_step_vjp(gw_ctx *c, const double *u, double *lam, double dt, int max_stages,
                           double w_energy, double w_outlet, double *grad) {
    if (!c || !u || !lam || !grad) return gw_fail(GW_ERR_ARG, "NULL argument");
    if ((const void *)u == (const void *)lam) return gw_fail(GW_ERR_ARG, "lam must not alias u");
    if (c->precision != GW_PREC_FP64)
        return gw_fail(GW_ERR_UNSUPPORTED, "gw_step_vjp works on double fields of a GW_PREC_FP64 context");
    int s, rc;
    if ((rc = check_common(c, dt, max_stages, &s))) return rc;
    const size_t N = (size_t)c->nx * c->ny * c->nz;
    const int nbuf = (s - 1) + 5 + 2 + 1;
    DevBlock blk;
    cudaError_t e = cudaMalloc(&blk.p, (size_t)nbuf * N * sizeof(double));
    if (e != cudaSuccess) return gw_cuda_fail(e, "cudaMalloc (step adjoint buffers)");
    double *p = (double *)blk.p;
    StepStore<double> S;
    for (int q = 0; q < s - 1; ++q, p += N) S.g.push_back(p);
    S.ustar = p; p += N; S.tA = p; p += N; S.u1 = p; p += N; S.tC = p; p += N; S.work = p; p += N;
    S.tpA = S.tpC = nullptr;
    S.pA = {S.tA, nullptr, nullptr, c->d_pipe_i, c->d_pipe_j, c->ny, c->nz};
    S.pC = {S.tC, nullptr, nullptr, c->d_pipe_i, c->d_pipe_j, c->ny, c->nz};
    double *B[3] = {lam, p, p + N};
    double *un1 = p + 2 * N;
    if ((rc = zero_acc(c)) || (rc = forward_store(c, u, S, dt, s, un1))) return rc;
    const double c_w = c->rho_c_water / kRhoWater;
    const double ob_scale = c->inlet_kind == GW_INLET_CONSTANT ? w_energy * c_w * dt : 0.0;
    int res = 0;
    if ((rc = adjoint_step<double>(c, u, un1, S, B, dt, s, ob_scale, w_outlet, &res))) return rc;
    if (res != 0) GW_CUDA(cudaMemcpyAsync(lam, B[res], N * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    return finish_grad(c, dt, 1, w_energy, grad);
}

extern "C" int gw_adjoint(gw_ctx *c, double dt, int nsteps, int max_stages, int checkpoint_every,
                          double w_energy, double w_outlet, double *grad, double *grad_T0,
                          gw_adjoint_info_t *info) {
    if (!c || !grad) return gw_fail(GW_ERR_ARG, "NULL argument");
    if (nsteps < 1) return gw_fail(GW_ERR_ARG, "nsteps must be >= 1");
    if (checkpoint_every < 1) return gw_fail(GW_ERR_ARG, "checkpoint_every must be >= 1");
    int s, rc;
    if ((rc = check_common(c, dt, max_stages, &s))) return rc;
    if (c->mixed_flags)
        return gw_fail(GW_ERR_UNSUPPORTED, "the adjoint transposes the default mixed step: "
                                           "gw_set_mixed_options(ctx, 0) first");
    if (c->precision == GW_PREC_MIXED)
        return adjoint_run<float>(c, dt, nsteps, max_stages, s, checkpoint_every, w_energy, w_outlet, grad,
                                  grad_T0, info);
    return adjoint_run<double>(c, dt, nsteps, max_stages, s, checkpoint_every, w_energy, w_outlet, grad, grad_T0,
                               info);
}
