// gw_tridiag.cu -- batched independent tridiagonal solves (the line solve of
// thomas_I_minus_A!, src/solver.jl:207-218, on arbitrary systems).
//
// Layout ("grouped interleaved"): systems are sorted by length and packed in
// groups of 32; group g holds rows 0..len_g-1 of its 32 systems with row r
// of lane l at off_g + 32 r + l, so thread l of a warp reads every row of
// its system in one coalesced 32-wide access.  Systems shorter than their
// group's length are padded with identity rows (a = c = 0, b = 1, d = 0);
// a_0 = 0 and c_{len-1} = 0 in every system.
//
// FP64: one thread per system, forward elimination writing c' to scratch
// and d' to x, back substitution over them (as src/solver.jl:208-218).
// Mixed: the same elimination in float (scratch: c', 1/den and d' as
// floats), then one correction: the residual r = d - A x in double, the
// correction A e = r solved with the float factors, x + e returned in double.
#include <cuda_runtime.h>

#include "gw_internal.h"

namespace {

// Rows are processed in batches of kB: a batch's loads (independent of the
// recurrences) issue together ahead of the dependent chain.
constexpr int kB = 8;

__global__ void __launch_bounds__(128) k_tri_f64(const double *__restrict__ a, const double *__restrict__ b,
                                                 const double *__restrict__ c, const double *__restrict__ d,
                                                 double *__restrict__ x, double *__restrict__ cs,
                                                 const long long *__restrict__ goff,
                                                 const int *__restrict__ glen, int ngroups) {
    const int g = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (g >= ngroups) return;
    const int lane = threadIdx.x & 31;
    const long long o = goff[g] + lane;
    const int L = glen[g];
    double cp = 0.0, dp = 0.0;
    for (int r0 = 0; r0 < L; r0 += kB) {
        double av[kB], bv[kB], cv[kB], dv[kB];
#pragma unroll
        for (int u = 0; u < kB; ++u)
            if (r0 + u < L) {
                const long long e = o + 32LL * (r0 + u);
                av[u] = a[e]; bv[u] = b[e]; cv[u] = c[e]; dv[u] = d[e];
            }
#pragma unroll
        for (int u = 0; u < kB; ++u)
            if (r0 + u < L) {
                const long long e = o + 32LL * (r0 + u);
                const double rden = 1.0 / fma(-av[u], cp, bv[u]);
                cp = cv[u] * rden;
                dp = fma(-av[u], dp, dv[u]) * rden;
                cs[e] = cp;
                x[e] = dp;
            }
    }
    double xn = dp;
    for (int r0 = L - 2; r0 >= 0; r0 -= kB) {
        double cv[kB], xv[kB];
#pragma unroll
        for (int u = 0; u < kB; ++u)
            if (r0 - u >= 0) {
                const long long e = o + 32LL * (r0 - u);
                cv[u] = cs[e]; xv[u] = x[e];
            }
#pragma unroll
        for (int u = 0; u < kB; ++u)
            if (r0 - u >= 0) {
                xn = fma(-cv[u], xn, xv[u]);
                x[o + 32LL * (r0 - u)] = xn;
            }
    }
}

// Mixed, pass 1: float factorisation and solve; x <- x32 (as double).
// fs: [3][n] floats (c', 1/den, d').
__global__ void __launch_bounds__(128) k_tri_mix1(const double *__restrict__ a, const double *__restrict__ b,
                                                  const double *__restrict__ c, const double *__restrict__ d,
                                                  double *__restrict__ x, float *__restrict__ fs,
                                                  long long n, const long long *__restrict__ goff,
                                                  const int *__restrict__ glen, int ngroups) {
    const int g = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (g >= ngroups) return;
    const int lane = threadIdx.x & 31;
    const long long o = goff[g] + lane;
    const int L = glen[g];
    float *fc = fs, *fr = fs + n, *fd = fs + 2 * n;
    float cp = 0.f, dp = 0.f;
    for (int r0 = 0; r0 < L; r0 += kB) {
        float av[kB], bv[kB], cv[kB], dv[kB];
#pragma unroll
        for (int u = 0; u < kB; ++u)
            if (r0 + u < L) {
                const long long e = o + 32LL * (r0 + u);
                av[u] = (float)a[e]; bv[u] = (float)b[e]; cv[u] = (float)c[e]; dv[u] = (float)d[e];
            }
#pragma unroll
        for (int u = 0; u < kB; ++u)
            if (r0 + u < L) {
                const long long e = o + 32LL * (r0 + u);
                const float rden = 1.0f / fmaf(-av[u], cp, bv[u]);
                cp = cv[u] * rden;
                dp = fmaf(-av[u], dp, dv[u]) * rden;
                fc[e] = cp;
                fr[e] = rden;
                fd[e] = dp;
            }
    }
    float xn = dp;
    x[o + 32LL * (L - 1)] = (double)xn;
    for (int r0 = L - 2; r0 >= 0; r0 -= kB) {
        float cv[kB], dv[kB];
#pragma unroll
        for (int u = 0; u < kB; ++u)
            if (r0 - u >= 0) {
                const long long e = o + 32LL * (r0 - u);
                cv[u] = fc[e]; dv[u] = fd[e];
            }
#pragma unroll
        for (int u = 0; u < kB; ++u)
            if (r0 - u >= 0) {
                xn = fmaf(-cv[u], xn, dv[u]);
                x[o + 32LL * (r0 - u)] = (double)xn;
            }
    }
}

// Mixed, pass 2: residual in double, correction with the float factors.
__global__ void __launch_bounds__(128) k_tri_mix2(const double *__restrict__ a, const double *__restrict__ b,
                                                  const double *__restrict__ c, const double *__restrict__ d,
                                                  double *__restrict__ x, float *__restrict__ fs,
                                                  long long n, const long long *__restrict__ goff,
                                                  const int *__restrict__ glen, int ngroups) {
    const int g = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (g >= ngroups) return;
    const int lane = threadIdx.x & 31;
    const long long o = goff[g] + lane;
    const int L = glen[g];
    const float *fc = fs, *fr = fs + n;
    float *fe = fs + 2 * n;   // reuses the d' slot for the correction's forward values
    double xm = 0.0, xc = x[o];
    float ep = 0.f;
    for (int r0 = 0; r0 < L; r0 += kB) {
        double av[kB], bv[kB], cv[kB], dv[kB], xp[kB];
        float rv[kB];
#pragma unroll
        for (int u = 0; u < kB; ++u)
            if (r0 + u < L) {
                const long long e = o + 32LL * (r0 + u);
                av[u] = a[e]; bv[u] = b[e]; cv[u] = c[e]; dv[u] = d[e]; rv[u] = fr[e];
                xp[u] = r0 + u + 1 < L ? x[e + 32] : 0.0;
            }
#pragma unroll
        for (int u = 0; u < kB; ++u)
            if (r0 + u < L) {
                const double res = dv[u] - fma(av[u], xm, fma(bv[u], xc, cv[u] * xp[u]));
                ep = fmaf(-(float)av[u], ep, (float)res) * rv[u];
                fe[o + 32LL * (r0 + u)] = ep;
                xm = xc;
                xc = xp[u];
            }
    }
    float en = ep;
    x[o + 32LL * (L - 1)] += (double)en;
    for (int r0 = L - 2; r0 >= 0; r0 -= kB) {
        float cv[kB], ev[kB];
        double xv[kB];
#pragma unroll
        for (int u = 0; u < kB; ++u)
            if (r0 - u >= 0) {
                const long long e = o + 32LL * (r0 - u);
                cv[u] = fc[e]; ev[u] = fe[e]; xv[u] = x[e];
            }
#pragma unroll
        for (int u = 0; u < kB; ++u)
            if (r0 - u >= 0) {
                en = fmaf(-cv[u], en, ev[u]);
                x[o + 32LL * (r0 - u)] = xv[u] + (double)en;
            }
    }
}

}  // namespace

extern "C" int gw_tridiag_batch(int precision, int ngroups, const long long *group_off,
                                const int *group_len, const double *a, const double *b,
                                const double *c, const double *d, double *x, void *scratch,
                                long long n_elements, void *stream) {
    if (ngroups < 0 || n_elements < 0) return gw_fail(GW_ERR_ARG, "negative size");
    if (ngroups == 0) return GW_OK;
    if (!group_off || !group_len || !a || !b || !c || !d || !x || !scratch)
        return gw_fail(GW_ERR_ARG, "NULL argument");
    if (precision != GW_PREC_FP64 && precision != GW_PREC_MIXED)
        return gw_fail(GW_ERR_ARG, "precision must be GW_PREC_FP64 or GW_PREC_MIXED");
    cudaStream_t s = (cudaStream_t)stream;
    const int wpb = 4;   // warps (groups) per block
    const unsigned grid = (unsigned)((ngroups + wpb - 1) / wpb);
    if (precision == GW_PREC_FP64) {
        k_tri_f64<<<grid, 32 * wpb, 0, s>>>(a, b, c, d, x, (double *)scratch, group_off, group_len, ngroups);
    } else {
        k_tri_mix1<<<grid, 32 * wpb, 0, s>>>(a, b, c, d, x, (float *)scratch, n_elements, group_off,
                                             group_len, ngroups);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return gw_cuda_fail(e, "k_tri_mix1");
        k_tri_mix2<<<grid, 32 * wpb, 0, s>>>(a, b, c, d, x, (float *)scratch, n_elements, group_off,
                                             group_len, ngroups);
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return gw_cuda_fail(e, "gw_tridiag_batch launch");
    e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return gw_cuda_fail(e, "gw_tridiag_batch");
    return GW_OK;
}
