// gw_fused.cu -- the fused time step used by gw_step, for both precisions.
//
// Per step the field crosses HBM three times:
//   1. k_rock2_col: every ROCK2 stage of the z-diffusion for one z-column,
//      the column held in shared memory (the z-stencil only couples levels
//      of one column, so all stages run without touching HBM in between);
//   2. k_half_tile (x-lines): explicit y-sweep + advected pipe values +
//      Thomas x-solve, one thread per line, the explicit sweep evaluated on
//      the fly while the forward elimination streams the line;
//   3. k_half_tile (y-lines): explicit x-sweep + pipe values + Thomas y-solve.
// Before each half step the pipe columns (5-9 % of the columns) get the
// explicit sweep into a compact [column][level] buffer on which the outlet
// mean, the per-level annulus means and the semi-Lagrangian advection run.
//
// Storage type T: double (GW_PREC_FP64) or float (GW_PREC_MIXED).  The mixed
// path stores theta = T - T_ref(z) (T_ref = the initial field's first
// column), so far-field cells carry small numbers whose increments are not
// absorbed by float rounding; A_x and A_y annihilate T_ref, A_z T_ref enters
// as a per-(column profile, level) source term, and the pipe advection
// converts to absolute temperature in double.  ROCK2 in the mixed path
// accumulates its stages as increments over the column's start value, so the
// stored field is rounded once per step.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <mutex>

#include "gw_internal.h"
#include "gw_fused.h"
#include "gw_inlet.cuh"
#include "gw_debug.cuh"

namespace {

inline unsigned grid_for(long long n, int block) { return (unsigned)((n + block - 1) / block); }

// cp.async (4/8-byte, zero-fill when pred is false) and its group fences
template <int BYTES>
__device__ __forceinline__ void cp_async(void *smem, const void *gmem, bool pred) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    const int n = pred ? BYTES : 0;   // 0: zero-fill, nothing is read
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2, %3;\n" ::"r"(s), "l"(gmem), "n"(BYTES),
                 "r"(n));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N)); }

// mbarrier and 3-D tensor-map tile copies (cp.async.bulk.tensor)
__device__ __forceinline__ void mbar_init(unsigned long long *mb, unsigned count) {
    const unsigned a = (unsigned)__cvta_generic_to_shared(mb);
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(a), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long *mb, unsigned bytes) {
    const unsigned a = (unsigned)__cvta_generic_to_shared(mb);
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(a), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try(unsigned long long *mb, unsigned parity) {
    const unsigned a = (unsigned)__cvta_generic_to_shared(mb);
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(a), "r"(parity)
        : "memory");
    return ok != 0;
}
// bounded: after the limit the flag is set and the caller goes on (the step
// then reports an error; no thread leaves the block's barriers)
__device__ __forceinline__ void mbar_wait(unsigned long long *mb, unsigned parity, int *err) {
    for (int i = 0; i < (1 << 24); ++i)
        if (mbar_try(mb, parity)) return;
    atomicExch(err, 1);
}
__device__ __forceinline__ void tma_tile3(void *dst, const CUtensorMap *map, int c0, int c1, int c2,
                                          unsigned long long *mb) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst), m = (unsigned)__cvta_generic_to_shared(mb);
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];\n" ::"r"(d),
        "l"((unsigned long long)map), "r"(c0), "r"(c1), "r"(c2), "r"(m)
        : "memory");
}

// Tensor memory (TMEM, 128 lanes x 512 32-bit columns per SM) as a scratch
// store of the half step's forward-elimination values.  Allocation by one
// warp (the address lands in shared memory), freed by the same warp before
// the block exits; a warp reaches only its lane quarter (lanes
// 32 (warp % 4) ..), one lane per thread with the 32x32b shapes.
__device__ __forceinline__ void tm_alloc(unsigned *slot, unsigned ncols) {
    const unsigned a = (unsigned)__cvta_generic_to_shared(slot);
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(a), "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
}
__device__ __forceinline__ void tm_dealloc(unsigned taddr, unsigned ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tm_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void tm_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void tm_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;\n" ::: "memory"); }
// 8 / 16 consecutive columns of this thread's lane
__device__ __forceinline__ void tm_st8(unsigned ta, const float *v) {
    asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};\n" ::"r"(ta),
                 "f"(v[0]), "f"(v[1]), "f"(v[2]), "f"(v[3]), "f"(v[4]), "f"(v[5]), "f"(v[6]), "f"(v[7])
                 : "memory");
}
__device__ __forceinline__ void tm_st16(unsigned ta, const float *v) {
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15, %16};\n" ::"r"(ta),
        "f"(v[0]), "f"(v[1]), "f"(v[2]), "f"(v[3]), "f"(v[4]), "f"(v[5]), "f"(v[6]), "f"(v[7]), "f"(v[8]), "f"(v[9]),
        "f"(v[10]), "f"(v[11]), "f"(v[12]), "f"(v[13]), "f"(v[14]), "f"(v[15])
        : "memory");
}
__device__ __forceinline__ void tm_ld16(unsigned ta, float *v) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];\n"
        : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3]), "=f"(v[4]), "=f"(v[5]), "=f"(v[6]), "=f"(v[7]),
          "=f"(v[8]), "=f"(v[9]), "=f"(v[10]), "=f"(v[11]), "=f"(v[12]), "=f"(v[13]), "=f"(v[14]), "=f"(v[15])
        : "r"(ta)
        : "memory");
}
// the registers of the loads before it hold their values only after this
// wait: they pass through it, so no use of them moves above it
__device__ __forceinline__ void tm_wait_ld(float *v) {
    asm volatile("tcgen05.wait::ld.sync.aligned;\n"
                 : "+f"(v[0]), "+f"(v[1]), "+f"(v[2]), "+f"(v[3]), "+f"(v[4]), "+f"(v[5]), "+f"(v[6]), "+f"(v[7]),
                   "+f"(v[8]), "+f"(v[9]), "+f"(v[10]), "+f"(v[11]), "+f"(v[12]), "+f"(v[13]), "+f"(v[14]),
                   "+f"(v[15])
                 :
                 : "memory");
}

// ---------------------------------------------------------------------------
// 1. ROCK2 on whole columns
// sc: per recurrence stage j = 1..s-2: (h mu_j, kappa_j); then (h sigma,
// h tau / sigma, 1 - tau / sigma^2).
template <typename T, bool INC>
__global__ void __launch_bounds__(256) k_rock2_col(T *__restrict__ u, const int *__restrict__ colprof,
                                                   const T *__restrict__ czm,
                                                   const T *__restrict__ czp,
                                                   const T *__restrict__ fref,
                                                   const double *__restrict__ sc, int s, int nz,
                                                   int pz, long long ncols) {
    // shared memory: base (the column at the step start), b0, and for the
    // increment form F0 = A base (+ source) and b1.  A stage reads its input
    // as a stencil and the stage before it only at its own level, so each
    // stage overwrites the older of the two.
    extern __shared__ unsigned char smem_raw[];
    T *base = reinterpret_cast<T *>(smem_raw);
    T *b0 = base + nz;
    T *F0 = b0 + nz;
    T *b1 = F0 + nz;
    const int nrec = s - 2;
    for (long long col = blockIdx.x; col < ncols; col += gridDim.x) {
        const int p = colprof[col];
        const T *cmc = czm + (size_t)p * nz;
        const T *cpc = czp + (size_t)p * nz;
        T *uc = u + col * pz;
        for (int k = threadIdx.x; k < nz; k += blockDim.x) base[k] = uc[k];
        __syncthreads();
        // A_z on a column in shared memory; Neumann ends (src/solver.jl:95-109)
        auto A = [&](const T *g, int k) {
            T gc = g[k];
            T gp = k < nz - 1 ? g[k + 1] : gc;
            T gm = k > 0 ? g[k - 1] : gc;
            return __ldg(cpc + k) * (gp - gc) - __ldg(cmc + k) * (gc - gm);
        };
        T *prev, *cur;
        if (INC) {
            for (int k = threadIdx.x; k < nz; k += blockDim.x) {
                T f = A(base, k);
                if (fref) f += __ldg(fref + (size_t)p * nz + k);
                F0[k] = f;
                b0[k] = T(0);
                b1[k] = T(0);
            }
            prev = b0;
            cur = b1;
            __syncthreads();
        } else {
            prev = nullptr;
            cur = base;
        }
        // recurrence g_j = g_{j-1} + h mu_j A g_{j-1} + kappa_j (g_{j-1} - g_{j-2})
        for (int j = 0; j < nrec; ++j) {
            const T hmu = (T)sc[2 * j], kap = (T)sc[2 * j + 1];
            T *out = prev ? prev : b0;
            for (int k = threadIdx.x; k < nz; k += blockDim.x) {
                T gc = cur[k];
                T a = A(cur, k);
                if (INC) a += F0[k];
                T gp = prev ? prev[k] : gc;
                out[k] = gc + hmu * a + kap * (gc - gp);
            }
            __syncthreads();
            prev = cur;
            cur = out;
        }
        // finishing procedure: gq = gp + h sigma A gp;
        // y = gq + (h tau / sigma) A gq + (1 - tau / sigma^2) (gq - gp)
        const T hs = (T)sc[2 * nrec], hts = (T)sc[2 * nrec + 1], c3 = (T)sc[2 * nrec + 2];
        T *q = prev ? prev : b0;
        for (int k = threadIdx.x; k < nz; k += blockDim.x) {
            T a = A(cur, k);
            if (INC) a += F0[k];
            q[k] = cur[k] + hs * a;
        }
        __syncthreads();
        for (int k = threadIdx.x; k < nz; k += blockDim.x) {
            T gq = q[k];
            T a = A(q, k);
            if (INC) a += F0[k];
            T y = gq + hts * a + c3 * (gq - cur[k]);
            uc[k] = INC ? base[k] + y : y;
        }
        __syncthreads();
    }
}

// Register-resident variant for nz <= 256 * LPT: thread t owns the LPT
// consecutive levels [t LPT, t LPT + LPT) in registers; a stage only
// exchanges the two end values of each thread's run through shared memory
// (double-buffered, one barrier per stage).  Blocks walk the columns in an
// order sorted by column profile, so the coefficient rows (the same for every
// column of a profile) stay in registers and are reloaded only when the
// profile changes.  The next column is copied into shared memory with
// coalesced cp.async while the current one runs its stages.
// Staging index of level k: one pad word per 32, so the coalesced copies
// (consecutive k per lane) and the per-thread runs (k = LPT t + i) are both
// free of shared-memory bank conflicts.
__device__ __forceinline__ int spad(int k) { return k + (k >> 5); }

// C is the arithmetic type of the stages (the storage type T by default;
// double over float storage for the mixed path's FP64 stage accumulation,
// where the column is rounded to float once, when it is stored).
template <typename T, bool INC, int LPT, typename C = T>
__global__ void __launch_bounds__(256, LPT <= 8 ? (sizeof(C) == 4 ? 3 : 2) : 1) k_rock2_reg(T *__restrict__ u, const int *__restrict__ order,
                                                   const int *__restrict__ colprof,
                                                   const C *__restrict__ czm,
                                                   const C *__restrict__ czp,
                                                   const C *__restrict__ fref,
                                                   const C *__restrict__ sc, int s, int nz,
                                                   int pz, long long ncols) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    // nt = blockDim.x threads (a multiple of 32, at most 256), LPT levels each
    const int nt = blockDim.x;
    T *stage = reinterpret_cast<T *>(smem_raw);   // [2][spad(nt * LPT)]
    const int nzs = spad(nt * LPT);
    // run ends of every thread, shifted by one slot so thread t reads its
    // neighbours at [t] (left, from s_hi) and [t + 1] (right, from s_lo)
    // without predicates; the outer slots hold zeros.
    __shared__ C s_lo[2][257], s_hi[2][257];
    const int t = threadIdx.x;
    const int kb = t * LPT;
    const int nrec = s - 2;
    int xb = 0;
    // The column is padded to nt * LPT levels: pad levels start at zero and
    // have zero coefficients, so they never feed a real level (the real
    // bottom level's cp is 0) and every thread owns exactly LPT levels.
    for (int k = nz + t; k < nt * LPT; k += nt) {
        if (GW_OK_D(stage + nzs + spad(k), smem_raw, 201)) { stage[spad(k)] = T(0); stage[nzs + spad(k)] = T(0); }
    }
    if (t < 2 && GW_OK_I(nt, 257, 202)) { s_hi[t][0] = C(0); s_lo[t][nt] = C(0); }
    // thread t copies levels t + nt i, whose padded slots are spad(t) + nts i
    const int st0 = spad(t), nts = nt + nt / 32;
    auto fetch = [&](long long col, int buf) {
        T *d = stage + (size_t)buf * nzs + st0;
        const T *g = u + col * pz + t;
#pragma unroll
        for (int i = 0; i < LPT; ++i)
            if (t + nt * i < nz && GW_OK_D(d + nts * i, smem_raw, 203) && GW_OK_G(g + nt * i, 204))
                cp_async<sizeof(T)>(d + nts * i, g + nt * i, true);
        cp_async_commit();
    };
    auto exchange = [&](const C (&v)[LPT], C &left, C &right) {
        if (GW_OK_I(t + 1, 257, 205)) { s_lo[xb][t] = v[0]; s_hi[xb][t + 1] = v[LPT - 1]; }
        __syncthreads();
        left = GW_OK_I(t + 1, 257, 205) ? s_hi[xb][t] : C(0);
        right = GW_OK_I(t + 1, 257, 205) ? s_lo[xb][t + 1] : C(0);
        xb ^= 1;
    };
    auto apply = [&](const C (&v)[LPT], const C (&cm)[LPT], const C (&cp)[LPT], int i, C left,
                     C right) {
        const C gc = v[i];
        const C gm = i == 0 ? left : v[i > 0 ? i - 1 : 0];
        const C gp = i + 1 < LPT ? v[i + 1 < LPT ? i + 1 : i] : right;
        return cp[i] * (gp - gc) - cm[i] * (gc - gm);
    };
    C cm[LPT], cp[LPT], fr[LPT];
    int pcur = -1;
    long long it = blockIdx.x;
    int buf = 0;
    // column indices and profiles run one column ahead of their use, so their
    // loads are not on the per-column chain
    long long col = it < ncols && GW_OK_G(order + it, 206) ? order[it] : 0;
    long long col_n = it + gridDim.x < ncols && GW_OK_G(order + it + gridDim.x, 206) ? order[it + gridDim.x] : 0;
    int p_cur = it < ncols && GW_OK_G(colprof + col, 207) ? colprof[col] : 0;
    if (it < ncols) fetch(col, 0);
    for (; it < ncols; it += gridDim.x, buf ^= 1) {
        const long long nxt = it + gridDim.x;
        const int p = p_cur;
        long long col_nn = 0;
        if (nxt < ncols) {
            fetch(col_n, buf ^ 1);
            if (nxt + gridDim.x < ncols && GW_OK_G(order + nxt + gridDim.x, 206)) col_nn = order[nxt + gridDim.x];
            p_cur = GW_OK_G(colprof + col_n, 207) ? colprof[col_n] : 0;
            cp_async_wait<1>();
        } else {
            cp_async_wait<0>();
        }
        if (p != pcur) {   // block-uniform
            pcur = p;
#pragma unroll
            for (int i = 0; i < LPT; ++i) {
                const bool ok = kb + i < nz;
                const size_t q = (size_t)p * nz + kb + i;
                cm[i] = ok && GW_OK_G(czm + q, 208) ? __ldg(czm + q) : C(0);
                cp[i] = ok && GW_OK_G(czp + q, 208) ? __ldg(czp + q) : C(0);
                fr[i] = (INC && fref && ok && GW_OK_G(fref + q, 209)) ? __ldg(fref + q) : C(0);
            }
        }
        __syncthreads();
        T *st = stage + (size_t)buf * nzs;
        C base[LPT], F0[LPT], prev[LPT], cur[LPT];
#pragma unroll
        for (int i = 0; i < LPT; ++i) base[i] = GW_OK_D(st + spad(kb + i), smem_raw, 210) ? (C)st[spad(kb + i)] : C(0);
        C left, right;
        exchange(base, left, right);
        if (INC) {
#pragma unroll
            for (int i = 0; i < LPT; ++i) {
                F0[i] = fr[i] + apply(base, cm, cp, i, left, right);
                prev[i] = C(0);
                cur[i] = C(0);
            }
        } else {
#pragma unroll
            for (int i = 0; i < LPT; ++i) { F0[i] = C(0); prev[i] = base[i]; cur[i] = base[i]; }
        }
        // recurrence g_j = g_{j-1} + h mu_j A g_{j-1} + kappa_j (g_{j-1} - g_{j-2});
        // in the increment form g = base + delta and A g = F0 + A delta
        for (int j = 0; j < nrec; ++j) {
            const C hmu = sc[2 * j], kap = sc[2 * j + 1];
            if (INC && j == 0) {
#pragma unroll
                for (int i = 0; i < LPT; ++i) { prev[i] = cur[i]; cur[i] = hmu * F0[i]; }
                continue;
            }
            exchange(cur, left, right);
            C out[LPT];
#pragma unroll
            for (int i = 0; i < LPT; ++i) {
                C a = apply(cur, cm, cp, i, left, right);
                if (INC) a += F0[i];
                out[i] = cur[i] + hmu * a + kap * (cur[i] - prev[i]);
            }
#pragma unroll
            for (int i = 0; i < LPT; ++i) { prev[i] = cur[i]; cur[i] = out[i]; }
        }
        // finishing procedure: gq = gp + h sigma A gp;
        // y = gq + (h tau / sigma) A gq + (1 - tau / sigma^2) (gq - gp)
        const C hs = sc[2 * nrec], hts = sc[2 * nrec + 1], c3 = sc[2 * nrec + 2];
        C q[LPT];
        if (INC && nrec == 0) {
#pragma unroll
            for (int i = 0; i < LPT; ++i) q[i] = hs * F0[i];
        } else {
            exchange(cur, left, right);
#pragma unroll
            for (int i = 0; i < LPT; ++i) {
                C a = apply(cur, cm, cp, i, left, right);
                if (INC) a += F0[i];
                q[i] = cur[i] + hs * a;
            }
        }
        exchange(q, left, right);
        // results go back through the staging buffer for a coalesced store
#pragma unroll
        for (int i = 0; i < LPT; ++i) {
            C a = apply(q, cm, cp, i, left, right);
            if (INC) a += F0[i];
            const C y = q[i] + hts * a + c3 * (q[i] - cur[i]);
            if (GW_OK_D(st + spad(kb + i), smem_raw, 210)) st[spad(kb + i)] = (T)(INC ? base[i] + y : y);
        }
        __syncthreads();
        T *uc = u + col * pz + t;
#pragma unroll
        for (int i = 0; i < LPT; ++i)
            if (t + nt * i < nz && GW_OK_G(uc + nt * i, 211) && GW_OK_D(st + st0 + nts * i, smem_raw, 212))
                uc[nt * i] = st[st0 + nts * i];
        __syncthreads();   // this buffer is refilled by the next iteration's fetch
        col = col_n;
        col_n = col_nn;
    }
}

// Mixed path, ROCK2 by windows: the same stages as k_rock2_reg<float, true>,
// level for level the same arithmetic, without block barriers.  A warp owns a
// window of W = 32 LPT consecutive levels of a column (lane l: levels
// ws + l LPT + i) and exchanges run ends with warp shuffles.  A window's
// outermost level has no neighbour outside the window; the error that leaves
// there reaches one level further inward per A evaluation, i.e. s - 1 levels
// over the s evaluations of an s-stage step (F0 and the stages reuse the
// start value).  So interior windows overlap by 2 s levels and store only
// their levels at least s from an interior edge.  Window w starts at level
// w (W - 2 s); the last window reaches the column's end (padding levels are
// zero-filled with zero coefficients, as in k_rock2_reg).
// A block holds whole column slots: blockDim / (32 nwin) slots of nwin
// warps (nwin <= 8), warp wib owning window wib % nwin of its slot's
// columns (every slots-th of the profile-sorted order, so the window's
// coefficient rows stay in registers), streamed through a private ring of NB
// staging buffers (NB - 1 windows in flight) with cp.async.  The halo levels
// a window reads are levels its neighbour windows store, in place, so a
// slot's warps meet at a named barrier once per column, after every
// window's copy of that column has landed and before any window stores it.
// (Without it a window fetching late, e.g. in a block started after its
// neighbour's when another stream's kernels held the SMs, read stored values
// as halo.  An mbarrier per ring buffer, arrived on when a copy lands and
// waited on just before the store, measured no faster.)
// S3: the instance for s = 3 (one recurrence stage, no g_{j-2} to keep).
template <int LPT, int NB, bool S3>
__global__ void __launch_bounds__(256, 3) k_rock2_win(float *__restrict__ u, const int *__restrict__ order,
                                                      const int *__restrict__ colprof,
                                                      const float *__restrict__ czm,
                                                      const float *__restrict__ czp,
                                                      const float *__restrict__ fref,
                                                      const float *__restrict__ sc, int s, int nz,
                                                      int pz, int ncols, int nwin) {
    constexpr int W = 32 * LPT;
    constexpr int WS = W + W / 32;   // padded slots of one staging buffer
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int spb = (blockDim.x >> 5) / nwin;               // column slots per block (blockDim: whole slots)
    const int slots = gridDim.x * spb;
    const int w = wib % nwin;
    const int slot = blockIdx.x * spb + wib / nwin;
    const unsigned bar_id = 1 + wib / nwin, bar_n = 32 * nwin;   // the slot's named barrier
    float *ring = reinterpret_cast<float *>(smem_raw) + (size_t)wib * NB * WS;
    const int ws = w * (W - 2 * s);                      // first level of the window
    const int lo = w == 0 ? 0 : ws + s;                  // stored levels [lo, hi)
    const int hi = w == nwin - 1 ? nz : ws + W - s;
    const int kb = ws + lane * LPT;                      // this lane's run
    const int nrec = S3 ? 1 : s - 2;
    const unsigned FULL = 0xffffffffu;
    // lane l copies window levels l + 32 i into slots spad(l + 32 i)
    auto fetch = [&](int col, int buf) {
        float *d = ring + (size_t)buf * WS;
        const float *gcol = u + (size_t)col * pz;
#pragma unroll
        for (int i = 0; i < LPT; ++i) {
            const int j = lane + 32 * i, k = ws + j;
            const bool ok = k < nz;
            if (GW_OK_D(d + spad(j), smem_raw, 220) && (!ok || GW_OK_G(gcol + k, 221)))
                cp_async<4>(d + spad(j), ok ? (const void *)(gcol + k) : (const void *)gcol, ok);
        }
    };
    auto exchange = [&](const float (&v)[LPT], float &left, float &right) {
        const float a = __shfl_up_sync(FULL, v[LPT - 1], 1);
        const float b = __shfl_down_sync(FULL, v[0], 1);
        left = lane == 0 ? 0.f : a;
        right = lane == 31 ? 0.f : b;
    };
    auto apply = [&](const float (&v)[LPT], const float (&cm)[LPT], const float (&cp)[LPT], int i,
                     float left, float right) {
        const float gc = v[i];
        const float gm = i == 0 ? left : v[i > 0 ? i - 1 : 0];
        const float gp = i + 1 < LPT ? v[i + 1 < LPT ? i + 1 : i] : right;
        return cp[i] * (gp - gc) - cm[i] * (gc - gm);
    };
    const int stride = slots;
    int it = slot;
    // columns (and profiles) of the items it + q stride, q < NB; the column of
    // item it + NB stride is read one item ahead of its fetch
    int cq[NB];
    int pq[NB];
#pragma unroll
    for (int q = 0; q < NB; ++q) {
        const long long iq = it + (long long)q * stride;
        cq[q] = iq < ncols && GW_OK_G(order + iq, 222) ? order[iq] : -1;
    }
#pragma unroll
    for (int q = 0; q < NB - 1; ++q) {
        pq[q] = cq[q] >= 0 && GW_OK_G(colprof + cq[q], 223) ? colprof[cq[q]] : 0;
        if (cq[q] >= 0) fetch(cq[q], q);
        cp_async_commit();
    }
    float cm[LPT], cp[LPT], fr[LPT];
    int pcur = -1, buf = 0, bnext = NB - 1;
    for (; it < ncols; it += stride) {
        // the item NB - 1 ahead goes into the buffer the previous item used
        __syncwarp();
        if (cq[NB - 1] >= 0) fetch(cq[NB - 1], bnext);
        cp_async_commit();
        pq[NB - 1] = cq[NB - 1] >= 0 && GW_OK_G(colprof + cq[NB - 1], 223) ? colprof[cq[NB - 1]] : 0;
        const long long iahead = it + (long long)NB * stride;
        const int cahead = iahead < ncols && GW_OK_G(order + iahead, 222) ? order[iahead] : -1;
        const int col = cq[0];
        const int p = pq[0];
        if (p != pcur) {   // warp-uniform
            pcur = p;
#pragma unroll
            for (int i = 0; i < LPT; ++i) {
                const bool ok = kb + i < nz;
                const size_t q = (size_t)p * nz + kb + i;
                cm[i] = ok && GW_OK_G(czm + q, 224) ? __ldg(czm + q) : 0.f;
                cp[i] = ok && GW_OK_G(czp + q, 224) ? __ldg(czp + q) : 0.f;
                fr[i] = fref && ok && GW_OK_G(fref + q, 225) ? __ldg(fref + q) : 0.f;
            }
        }
        cp_async_wait<NB - 1>();
        __syncwarp();
        // every window of the slot holds this column before any stores it
        if (nwin > 1) asm volatile("bar.sync %0, %1;" ::"r"(bar_id), "r"(bar_n) : "memory");
        float *st = ring + (size_t)buf * WS;
        float F0[LPT], prev[LPT], cur[LPT];
        float left, right;
        {   // the start values are read again from st at the end
            float base[LPT];
#pragma unroll
            for (int i = 0; i < LPT; ++i)
                base[i] = GW_OK_D(st + spad(lane * LPT + i), smem_raw, 226) ? st[spad(lane * LPT + i)] : 0.f;
            exchange(base, left, right);
#pragma unroll
            for (int i = 0; i < LPT; ++i) {
                F0[i] = fr[i] + apply(base, cm, cp, i, left, right);
                prev[i] = 0.f;
                cur[i] = 0.f;
            }
        }
        // increment form: g = base + delta, A g = F0 + A delta
        for (int j = 0; j < nrec; ++j) {
            const float hmu = sc[2 * j], kap = sc[2 * j + 1];
            if (j == 0) {
#pragma unroll
                for (int i = 0; i < LPT; ++i) { prev[i] = cur[i]; cur[i] = hmu * F0[i]; }
                continue;
            }
            exchange(cur, left, right);
            float out[LPT];
#pragma unroll
            for (int i = 0; i < LPT; ++i) {
                float a = apply(cur, cm, cp, i, left, right);
                a += F0[i];
                out[i] = cur[i] + hmu * a + kap * (cur[i] - prev[i]);
            }
#pragma unroll
            for (int i = 0; i < LPT; ++i) { prev[i] = cur[i]; cur[i] = out[i]; }
        }
        const float hs = sc[2 * nrec], hts = sc[2 * nrec + 1], c3 = sc[2 * nrec + 2];
        float q[LPT];
        if (nrec == 0) {
#pragma unroll
            for (int i = 0; i < LPT; ++i) q[i] = hs * F0[i];
        } else {
            exchange(cur, left, right);
#pragma unroll
            for (int i = 0; i < LPT; ++i) {
                float a = apply(cur, cm, cp, i, left, right);
                a += F0[i];
                q[i] = cur[i] + hs * a;
            }
        }
        exchange(q, left, right);
        // each lane updates its own run's slots: start value + increment
#pragma unroll
        for (int i = 0; i < LPT; ++i) {
            float a = apply(q, cm, cp, i, left, right);
            a += F0[i];
            const float y = q[i] + hts * a + c3 * (q[i] - cur[i]);
            if (GW_OK_D(st + spad(lane * LPT + i), smem_raw, 226))
                st[spad(lane * LPT + i)] = st[spad(lane * LPT + i)] + y;
        }
        __syncwarp();
        float *uc = u + (size_t)col * pz;
#pragma unroll
        for (int i = 0; i < LPT; ++i) {
            const int j = lane + 32 * i, k = ws + j;
            if (k >= lo && k < hi && GW_OK_G(uc + k, 227) && GW_OK_D(st + spad(j), smem_raw, 226))
                uc[k] = st[spad(j)];
        }
#pragma unroll
        for (int q2 = 0; q2 < NB - 1; ++q2) { cq[q2] = cq[q2 + 1]; pq[q2] = pq[q2 + 1]; }
        cq[NB - 1] = cahead;
        buf = buf + 1 == NB ? 0 : buf + 1;
        bnext = bnext + 1 == NB ? 0 : bnext + 1;
    }
    cp_async_wait<0>();
}

// ---------------------------------------------------------------------------
// 2. pipe columns

// absolute temperature of a pipe value (theta + T_ref in the mixed path)
template <typename T>
__device__ __forceinline__ double absT(T v, const double *Tref, int k) {
    return Tref ? (double)v + Tref[k] : (double)v;
}

// Pipe pass in two launches before the advection: k_pipe_sweep applies the
// explicit sweep to the pipe columns of one chunk (a run of at most 16
// columns of one borehole's inner pipe or annulus) for 128 levels, stores the
// swept values and the chunk's column sum per level; k_pipe_reduce turns the
// sums into the outlet mean (src/solver.jl:267-282, 257) and the per-level
// annulus means (src/solver.jl:322-335).  Every sum runs in a fixed order
// (per warp, then across warps in warp order): the results do not depend on
// scheduling.

// Pipe kernels put the chunks on the grid's y dimension (at most 65535),
// continued on z for more chunks.
constexpr int kChunkRows = 65535;
inline dim3 chunk_grid(int kblocks, int nchunks) {
    return dim3(kblocks, std::min(nchunks, kChunkRows), (nchunks + kChunkRows - 1) / kChunkRows);
}

// PR columns per round (8: large well pipe pass 0.0596 -> 0.0544 ms, 2 mm
// well 0.0437 -> 0.0402 ms against 4; 16: 0.0571 / 0.0415)
template <typename T, int PR = 8>
__global__ void __launch_bounds__(128) k_pipe_sweep(T *__restrict__ tp, double *__restrict__ part,
                                                    const T *__restrict__ src,
                                                    const int4 *__restrict__ chunks,
                                                    const int *__restrict__ pi,
                                                    const int *__restrict__ pj,
                                                    const int *__restrict__ zclass,
                                                    const T *__restrict__ cmt,
                                                    const T *__restrict__ cpt,
                                                    const double *__restrict__ Tref, int nx, int ny,
                                                    int nz, int pz, double h, int dir, int nchunks) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int ch = blockIdx.y + kChunkRows * blockIdx.z;   // chunk rows of at most 65535
    if (k >= nz || ch >= nchunks) return;
    if (!GW_OK_G(chunks + ch, 301) || !GW_OK_G(zclass + k, 302)) return;
    const int4 C = chunks[ch];   // (borehole, first column, end column, outer?)
    const int zc = zclass[k];
    const T hh = (T)h;
    // debug build: every global load checked (nothing in the normal build)
    auto ld = [&](const T *p) -> T { return GW_OK_G(p, 304) ? *p : T(0); };
    auto sweep = [&](int q) {
        const int i = GW_OK_G(pi + q, 303) ? pi[q] : 0, j = GW_OK_G(pj + q, 303) ? pj[q] : 0;
        const long long c = k + (long long)pz * (j + (long long)ny * i);
        const T xc = ld(src + c);
        T xp, xm;
        size_t t;
        if (dir == GW_DIR_X) {
            const long long st = (long long)pz * ny;
            xp = (i < nx - 1) ? ld(src + c + st) : xc;
            xm = (i > 0) ? ld(src + c - st) : xc;
            t = ((size_t)zc * ny + j) * nx + i;
        } else {
            xp = (j < ny - 1) ? ld(src + c + pz) : xc;
            xm = (j > 0) ? ld(src + c - pz) : xc;
            t = ((size_t)zc * nx + i) * ny + j;
        }
        const T a = (GW_OK_G(cpt + t, 305) ? __ldg(cpt + t) : T(0)) * (xp - xc) -
                    (GW_OK_G(cmt + t, 305) ? __ldg(cmt + t) : T(0)) * (xc - xm);
        return fma(hh, a, xc);
    };
    // kPR columns per round: their loads are independent and overlap; the
    // sum still runs over the columns in order
    constexpr int kPR = PR;
    double acc = 0.0;
    int q = C.y;
    for (; q + kPR <= C.z; q += kPR) {
        T v[kPR];
#pragma unroll
        for (int u = 0; u < kPR; ++u) v[u] = sweep(q + u);
#pragma unroll
        for (int u = 0; u < kPR; ++u) {
            if (GW_OK_G(tp + (size_t)(q + u) * nz + k, 306)) tp[(size_t)(q + u) * nz + k] = v[u];
            acc += (double)v[u];
        }
    }
    for (; q < C.z; ++q) {
        const T v = sweep(q);
        if (GW_OK_G(tp + (size_t)q * nz + k, 306)) tp[(size_t)q * nz + k] = v;
        acc += (double)v;
    }
    // absolute temperature: add T_ref once per column summed
    if (Tref && GW_OK_G(Tref + k, 308)) acc += (double)(C.z - C.y) * Tref[k];
    if (GW_OK_G(part + (size_t)ch * nz + k, 307)) part[(size_t)ch * nz + k] = acc;
}

constexpr int kReduceWarps = 8;   // warps of k_pipe_reduce, splitting a borehole's chunks

// grid (ceil(nz / 32), nbh), block 32 * kReduceWarps: annulus means per
// level (lane = level, warps split the chunks); the first block of a
// borehole also reduces its inner-pipe chunks over the outlet window.
__global__ void __launch_bounds__(32 * kReduceWarps) k_pipe_reduce(double *__restrict__ outlet,
                                                     double *__restrict__ mean,
                                                     const double *__restrict__ part,
                                                     const int *__restrict__ bchunk,
                                                     const int *__restrict__ nlev_b,
                                                     const GwBhDev *__restrict__ bh, int nz) {
    __shared__ double s_red[32 * kReduceWarps];
    const int b = blockIdx.y;
    if (!GW_OK_G(bh + b, 311) || !GW_OK_GB(bchunk + 4 * b, 4 * sizeof(int), 312)) return;
    const GwBhDev B = bh[b];
    // chunks of b: inner [bchunk[4b], bchunk[4b+1]), outer [bchunk[4b+2], bchunk[4b+3])
    const int i0 = bchunk[4 * b], i1 = bchunk[4 * b + 1], o0 = bchunk[4 * b + 2], o1 = bchunk[4 * b + 3];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int k = blockIdx.x * 32 + lane;
    // four running sums (chunks w, w + 8, w + 16, w + 24 of each round of 32),
    // so four loads are in flight; they are added in a fixed order
    double sacc = 0.0;
    if (k < nz) {
        auto ld = [&](int ch) { return GW_OK_G(part + (size_t)ch * nz + k, 313) ? part[(size_t)ch * nz + k] : 0.0; };
        double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
        int ch = o0 + w;
        for (; ch + 3 * kReduceWarps < o1; ch += 4 * kReduceWarps) {
            a0 += ld(ch);
            a1 += ld(ch + kReduceWarps);
            a2 += ld(ch + 2 * kReduceWarps);
            a3 += ld(ch + 3 * kReduceWarps);
        }
        for (; ch < o1; ch += kReduceWarps) a0 += ld(ch);
        sacc = (a0 + a1) + (a2 + a3);
    }
    s_red[threadIdx.x] = sacc;
    __syncthreads();
    if (w == 0 && k < nz) {
        double m = s_red[lane];
#pragma unroll
        for (int q = 1; q < kReduceWarps; ++q) m += s_red[32 * q + lane];
        if (GW_OK_G(mean + (size_t)b * nz + k, 314)) mean[(size_t)b * nz + k] = m / (double)B.outer_count;
    }
    if (blockIdx.x != 0) return;   // the whole block: the outlet is block 0's
    __syncthreads();   // every read of s_red above is done
    const int nlev = GW_OK_G(nlev_b + b, 315) ? nlev_b[b] : 0;
    // (chunk, level) elements, level fastest (coalesced), spread over the
    // block; each thread keeps four running sums (four loads in flight),
    // added in a fixed order
    const int total = nlev * (i1 - i0);
    auto ld = [&](int e) {
        const size_t q = (size_t)(i0 + e / nlev) * nz + e % nlev;
        return GW_OK_G(part + q, 313) ? part[q] : 0.0;
    };
    const int bd = blockDim.x;
    double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
    int e = threadIdx.x;
    for (; e + 3 * bd < total; e += 4 * bd) {
        a0 += ld(e);
        a1 += ld(e + bd);
        a2 += ld(e + 2 * bd);
        a3 += ld(e + 3 * bd);
    }
    for (; e < total; e += bd) a0 += ld(e);
    const double acc = (a0 + a1) + (a2 + a3);
    s_red[threadIdx.x] = acc;
    __syncthreads();
    for (int r = blockDim.x / 2; r > 0; r >>= 1) {
        if (threadIdx.x < r) s_red[threadIdx.x] += s_red[threadIdx.x + r];
        __syncthreads();
    }
    if (threadIdx.x == 0 && GW_OK_G(outlet + b, 316)) outlet[b] = s_red[0] / (double)((long long)B.inner_count * nlev);
}

// Outlet window of kernel_accumulate_outlet! (src/solver.jl:273-281) for a
// step size: the number of levels with z <= v_inner dt (gz is sorted, so
// they are a prefix), per borehole.
__global__ void k_outlet_levels(int *__restrict__ nlev, const double *__restrict__ gz,
                                const GwBhDev *__restrict__ bh, int nbh, int nz, double dt) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nbh) return;
    const double zmax = bh[b].v_inner * dt;
    int lo = 0, hi = nz;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (gz[mid] <= zmax) lo = mid + 1; else hi = mid;
    }
    nlev[b] = lo;
}

// Departure table of kernel_advection! (src/solver.jl:285-360): for every
// borehole b, level k < countz and pipe (0 inner, 1 annulus) the branch
// taken, the two interpolation levels and the weight.  It depends only on
// the grid, the velocities and dt, so it is built once per step size with the
// same floating-point operations (fused multiply-adds as the reference's
// @muladd) the per-cell evaluation would use.

__global__ void k_adv_table(GwAdvRec *__restrict__ tab, const double *__restrict__ gz,
                            const GwBhDev *__restrict__ bh, const double *__restrict__ Tref, int nbh,
                            int nz, int countz, double dt) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nbh * countz * 2) return;
    const int pipe = e & 1, k = (e >> 1) % countz, b = (e >> 1) / countz;
    const GwBhDev B = bh[b];
    const double z = gz[k];
    GwAdvRec r;
    r.type = kAdvKeep; r.il = k; r.ir = k; r.alpha = 0.0; r.dref = 0.0; r.pad = 0;
    if (z <= B.h) {
        double dep;
        if (pipe == 0) {
            double zd = __fma_rn(B.v_inner, dt, z);
            if (zd > B.h) {
                double dt1 = __ddiv_rn(__dsub_rn(B.h, z), B.v_inner);
                double dt2 = __dsub_rn(dt, dt1);
                dep = __fma_rn(-B.v_outer, dt2, B.h);
                r.type = kAdvTurn;
            } else {
                dep = zd;
                r.type = kAdvInterp;
            }
        } else {
            dep = __fma_rn(-B.v_outer, dt, z);
            r.type = dep <= 0.0 ? kAdvInlet : kAdvInterp;
        }
        if (r.type != kAdvInlet) {
            int lo = 0, hi = nz - 1;   // gpu_searchsortedfirst + interpolation_helper
            while (lo < hi) {
                int mid = lo + ((hi - lo) >> 1);
                if (gz[mid] < dep) lo = mid + 1; else hi = mid;
            }
            int ir = lo, il = lo - 1;
            if (il < 0) il = 0;
            if (ir > nz - 1) ir = nz - 1;
            r.il = il; r.ir = ir;
            r.alpha = __ddiv_rn(__dsub_rn(dep, gz[il]), __dsub_rn(gz[ir], gz[il]));
            if (Tref)
                r.dref = r.alpha * Tref[ir] + (1.0 - r.alpha) * Tref[il] - Tref[k];
        }
    }
    tab[e] = r;
}

// Time-dependent inlets at t = t0 + (n + 1 + off) dt for the step n the
// counter holds (off 0: first advection, 1/2: second): the schedule
// (nprog = 0), or the inlet program of every borehole with the outlet
// temperatures of this pipe pass (GW_INLET_EXPRESSION).
__global__ void k_inlet_eval(double *__restrict__ inlet_v, const double *__restrict__ sched, int ns,
                             const double *__restrict__ time, const int *__restrict__ counter, double off,
                             int nbh, const int *__restrict__ op, const double *__restrict__ arg, int nprog,
                             const double *__restrict__ outlet) {
    const double t = __fma_rn((double)(*counter) + 1.0 + off, time[1], time[0]);
    if (nprog > 0) {
        for (int b = threadIdx.x; b < nbh; b += blockDim.x)
            inlet_v[b] = gw_program_eval(op, arg, nprog, outlet[b], t, b, sched, ns);
        return;
    }
    const double v = gw_sched_eval(sched, ns, t);
    for (int b = threadIdx.x; b < nbh; b += blockDim.x) inlet_v[b] = v;
}

// kernel_advection! on the compact buffer with the departure table; the
// result (minus T_ref in the mixed path) goes to pp[q][k], k < countz.
// grid (ceil(countz / 128), chunks): a thread takes one level of every
// column of one pipe chunk (the columns of one borehole's inner pipe or
// annulus share the departure record of that level), so the record is read
// once per chunk; turnaround and inlet values do not depend on the column
// and are computed once.
template <typename T>
__global__ void __launch_bounds__(128) k_advect_c(T *__restrict__ pp, const T *__restrict__ tp,
                                                  const GwAdvRec *__restrict__ tab,
                                                  const int4 *__restrict__ chunks,
                                                  const double *__restrict__ ann_mean,
                                                  const double *__restrict__ outlet,
                                                  const double *__restrict__ Tref, int nz, int countz,
                                                  int inlet_kind, double inlet_param,
                                                  const double *__restrict__ inlet_v, int nchunks) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int ch = blockIdx.y + kChunkRows * blockIdx.z;
    if (k >= countz || ch >= nchunks) return;
    if (!GW_OK_G(chunks + ch, 321)) return;
    const int4 C = chunks[ch];   // (borehole, first column, end column, annulus?)
    const int b = C.x;
    if (!GW_OK_G(tab + ((size_t)b * countz + k) * 2 + C.w, 322)) return;
    const GwAdvRec r = tab[((size_t)b * countz + k) * 2 + C.w];
    T *out = pp + k;
    if (r.type == kAdvInlet || r.type == kAdvTurn) {
        double v;
        if (r.type == kAdvInlet) {
            v = inlet_kind == GW_INLET_CONSTANT ? inlet_param
              : inlet_kind >= GW_INLET_SCHEDULE ? inlet_v[b] : outlet[b] - inlet_param;
        } else {
            const double *m = ann_mean + (size_t)b * nz;
            v = __fma_rn(r.alpha, m[r.ir], __dmul_rn(__dsub_rn(1.0, r.alpha), m[r.il]));
        }
        const T o = (T)(Tref ? v - Tref[k] : v);
        for (int q = C.y; q < C.z; ++q)
            if (GW_OK_G(out + (size_t)q * countz, 325)) out[(size_t)q * countz] = o;
        return;
    }
    if (r.type == kAdvKeep) {
        for (int q = C.y; q < C.z; ++q) {
            if (!GW_OK_G(tp + (size_t)q * nz + k, 326) || !GW_OK_G(out + (size_t)q * countz, 325)) continue;
            const double v = absT(tp[(size_t)q * nz + k], Tref, k);
            out[(size_t)q * countz] = (T)(Tref ? v - Tref[k] : v);
        }
        return;
    }
    if (sizeof(T) == 4) {
        // mixed path: interpolate theta in float, the T_ref part is the
        // tabulated double offset
        const float a = (float)r.alpha, a1 = 1.0f - a, dref = (float)r.dref;
        for (int q = C.y; q < C.z; ++q) {
            const T *col = tp + (size_t)q * nz;
            if (!GW_OK_G(col + r.ir, 326) || !GW_OK_G(col + r.il, 326) || !GW_OK_G(out + (size_t)q * countz, 325))
                continue;
            out[(size_t)q * countz] = (T)(fmaf(a, (float)col[r.ir], a1 * (float)col[r.il]) + dref);
        }
        return;
    }
    const double a1 = __dsub_rn(1.0, r.alpha);
    for (int q = C.y; q < C.z; ++q) {
        const T *col = tp + (size_t)q * nz;
        if (!GW_OK_G(col + r.ir, 326) || !GW_OK_G(col + r.il, 326) || !GW_OK_G(out + (size_t)q * countz, 325))
            continue;
        const double v = __fma_rn(r.alpha, absT(col[r.ir], Tref, r.ir), __dmul_rn(a1, absT(col[r.il], Tref, r.il)));
        out[(size_t)q * countz] = (T)(Tref ? v - Tref[k] : v);
    }
}

// ---------------------------------------------------------------------------
// 3. half step: explicit sweep in the other direction + advected pipe values
//    + Thomas along the line direction.  XL: x-lines (explicit y), else
//    y-lines (explicit x).
//
// A block owns 32 consecutive levels (one per lane) of HW neighbouring lines
// (one warp each).  Rows are streamed in chunks of HR: the block copies the
// chunk's rows of its kHW lines plus the two neighbouring lines (which the
// explicit sweep needs) into shared memory with cp.async, double-buffered so
// the next chunk is in flight while the current one is eliminated.  The
// forward sweep stores y_l in dst; the backward sweep reads it back in
// batches loaded ahead of their use and overwrites it with x_l.  The x_l are
// streaming stores (st.global.cs, evict-first): no kernel reads them back
// from L2, while the y_l of every resident line (up to ~96 MB) wait there
// for their backward sweep (large well: half steps 1-2 % faster).
// Tilings (lines per block HW, rows per chunk HR); the autotuner picks one
// per context, the default is the first.
// 7 .. 12 are the row tiles of 0 .. 5 with the forward values in global memory.
constexpr int kTilings = 13;   // 6 is the segmented kernel (k_half_seg)
constexpr int kTileHW[kTilings] = {4, 8, 8, 4, 2, 8, 2, 4, 8, 8, 4, 2, 8};
constexpr int kTileHR[kTilings] = {16, 16, 8, 32, 16, 32, 16, 16, 16, 8, 32, 16, 32};
constexpr int kSegCfg = 6;
constexpr int kGlobalCfg = 7;   // first tiling with the forward values in global memory
static_assert(kTilings == GW_TILINGS, "tiling count of the C ABI");
constexpr int kSegS = 8, kSegR = 32;   // segments per line, rows per segment (lines up to 256)
constexpr int kHG = 4;    // rows whose coefficients are loaded together
constexpr int kHB = 16;    // rows per backward batch


template <typename T>
struct alignas(4 * sizeof(T)) Quad {
    T x, y, z, w;
};

// TMA (float field, columns pz apart, pz a multiple of 4): the chunk of the
// HW + 2 lines is one 3-D tensor-map tile (32 levels x lines x rows, levels
// beyond nz, lines outside 0..nl-1 and rows beyond N zero-filled, as the
// cp.async copies fill them), issued by one thread into a ring of NB buffers
// and awaited on the buffer's mbarrier.  Tile layout: [row][line][32] for the
// x-lines and the cp.async path, [line][row][32] for TMA y-lines (the tensor's
// dimensions are levels, j, i).
//
// TM (with TMA; blocks of 4 or 8 lines): the forward values stay on chip, in
// tensor memory.  The block allocates tm_cw columns (a power of two >= N) per
// line slot -- a warp uses its TMEM lane quarter (warp % 4), warps w and w + 4
// the column blocks 0 and tm_cw -- after its first tiles are in flight (the
// allocation waits while other blocks of the SM hold the 512 columns; those
// blocks, resident with their first tiles loaded, start at once when it is
// freed).  Each chunk's y_l of a lane go to its TMEM lane as HR consecutive
// columns; the backward sweep reads them 16 at a time, the next batch and
// its coefficients in flight, and writes x_l.  With tm_cw < N (the split
// form: 128 columns, a ring of two) rows tm_cw .. N - 1 go to the block's
// shared memory instead, which lets three blocks of 205-row lines work per
// SM where whole lines in TMEM let two.  The field then crosses HBM
// once per direction plus the halo lines, with no y_l round trip through L2,
// and the values and their order of operations are those of the global-memory
// form: bitwise the same field.
template <typename T, bool XL, int HW, int HR, int NB = 2, bool TMA = false, bool TM = false>
__global__ void __launch_bounds__(32 * HW) k_half_tile(T *__restrict__ dst, const T *__restrict__ src,
                                                        const T *__restrict__ pp,
                                                        const int *__restrict__ pipe_line,
                                                        const int *__restrict__ zclass,
                                                        const Quad<T> *__restrict__ hq,
                                                        const T *__restrict__ fib,
                                                        const T *__restrict__ fcu, int nx, int ny,
                                                        int nz, int pz, int countz, int m_begin, int m_end,
                                                        const __grid_constant__ CUtensorMap tmap,
                                                        const __grid_constant__ CUtensorMap qmap, int *err,
                                                        int tm_cw = 0, int prow_lo = 0, int prow_hi = 0x7fffffff) {
    static_assert(!TMA || sizeof(T) == 4, "tensor-map tiles: float fields only");
    static_assert(TMA || NB == 2, "the cp.async path double-buffers");
    static_assert(!TM || (TMA && (HR == 8 || HR == 16 || HR == 32)), "TMEM forward values: TMA tiles of 8-32 rows");
    extern __shared__ __align__(128) unsigned char smem_raw[];
    T *tile = reinterpret_cast<T *>(smem_raw);   // [NB][tile]
    constexpr int kRow = (HW + 2) * 32;
    constexpr int kTile = HR * kRow;
    constexpr int kRowS = (TMA && !XL) ? 32 : kRow;        // rows apart in a tile
    constexpr int kSlotS = (TMA && !XL) ? HR * 32 : 32;    // line slots apart in a tile
    // TMA: the chunk's row coefficients of the block's lines for the block's
    // z-class ([line][row] quads) arrive with the tile, on its mbarrier
    constexpr int kQ = HW * HR;
    Quad<T> *qtile = reinterpret_cast<Quad<T> *>(smem_raw + (size_t)NB * kTile * sizeof(T));
    unsigned long long *mbar = reinterpret_cast<unsigned long long *>(
        smem_raw + (size_t)NB * kTile * sizeof(T) + (TMA ? (size_t)NB * kQ * sizeof(Quad<T>) : 0));
    unsigned *tslot = reinterpret_cast<unsigned *>(mbar + NB);   // TM: the TMEM allocation's address
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nl = XL ? ny : nx;   // lines per level
    const int N = XL ? nx : ny;    // line length
    const int k0 = blockIdx.x * 32, m0 = m_begin + blockIdx.y * HW;   // lines m_begin .. m_end - 1
    const int k = k0 + lane, m = m0 + warp;
    const bool kok = k < nz;
    const bool active = kok && m < m_end;
    const int kc = kok ? k : nz - 1, mc = m < m_end ? m : m_end - 1;   // clamped for table reads
    // element (k, line m, row l): x-lines (k, j=m, i=l), y-lines (k, i=m, j=l)
    const long long mst = XL ? (long long)pz : (long long)pz * ny;
    const long long rst = XL ? (long long)pz * ny : (long long)pz;
    const int zcl = GW_OK_G(zclass + kc, 112) ? zclass[kc] : 0;
    const size_t fb = ((size_t)zcl * nl + mc) * N;
    // the block's z-class (its first level's): lanes of another class, at a
    // class boundary, read their coefficients from global memory
    const int kb0 = k0 < nz ? k0 : nz - 1;
    const int zcb = GW_OK_G(zclass + kb0, 112) ? zclass[kb0] : 0;
    const bool qs_ok = TMA && zcl == zcb;
    const int *pline = pipe_line + (size_t)mc * N;
    // lines through no pipe column skip the per-row pipe lookup (most lines)
    const bool pipe_levels = k < countz && GW_OK_G(pipe_line + (size_t)nl * N + mc, 113) &&
                             __ldg(pipe_line + (size_t)nl * N + mc) != 0;
    const Quad<T> *hql = hq + fb;
    T *dl = dst + k + m * mst;   // row 0 of this thread's line
    const int nchunk = (N + HR - 1) / HR;

    // this warp copies neighbour-line slots mm = warp and warp + HW of each
    // row; slot pointers and validity are fixed for the whole line
    const T *gs[2];
    bool sok[2];
#pragma unroll
    for (int rep = 0; rep < 2; ++rep) {
        const int mm = warp + rep * HW;
        const int gm = m0 - 1 + mm;
        sok[rep] = mm < HW + 2 && kok && gm >= 0 && gm < nl;
        gs[rep] = sok[rep] ? src + k + (long long)gm * mst : src;
    }
    // debug build: tile copies and tile reads checked (nothing in the normal build)
    auto tile_copy = [&](T *ds, const T *gp, bool ok) {
        if (!GW_OK_D(ds, smem_raw, 101)) return;
        ok = ok && GW_OK_G(gp, 102);
        cp_async<sizeof(T)>(ds, ok ? (const void *)gp : (const void *)src, ok);
    };
    auto rd = [&](const T *p) -> T { return GW_OK_D(p, smem_raw, 103) ? *p : T(0); };
    auto load_chunk = [&](int ch, int buf) {
        T *t = tile + buf * kTile;
        const int l0 = ch * HR;
        if constexpr (TMA) {
            if (threadIdx.x == 0) {
                // the buffer's previous chunk was read through the generic proxy
                asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
                mbar_expect_tx(mbar + buf, (unsigned)(kTile * sizeof(T) + kQ * sizeof(Quad<T>)));
                if (XL)
                    tma_tile3(t, &tmap, k0, m0 - 1, l0, mbar + buf);
                else
                    tma_tile3(t, &tmap, k0, l0, m0 - 1, mbar + buf);
                tma_tile3(qtile + buf * kQ, &qmap, 4 * l0, m0, zcb, mbar + buf);
            }
            return;
        }
        const bool full = l0 + HR <= N;
#pragma unroll
        for (int rep = 0; rep < 2; ++rep) {
            if (warp + rep * HW >= HW + 2) break;
            const T *g = gs[rep] + (long long)l0 * rst;
            T *d = t + (warp + rep * HW) * 32 + lane;
            if (full) {
#pragma unroll
                for (int r = 0; r < HR; ++r) tile_copy(d + r * kRow, g + r * rst, sok[rep]);
            } else {
                for (int r = 0; r < HR; ++r) {
                    tile_copy(d + r * kRow, g + r * rst, sok[rep] && l0 + r < N);
                }
            }
        }
        cp_async_commit();
    };
    // warp-uniform: does this line cross a pipe column at any level?
    const bool line_pipe = GW_OK_G(pipe_line + (size_t)nl * N + mc, 113) &&
                           __ldg(pipe_line + (size_t)nl * N + mc) != 0;

    T y = T(0);
    T *dr = dl;
    const unsigned tm_cols = TM ? (unsigned)tm_cw * ((HW + 3) / 4) : 0u;
    unsigned tbase = 0, taddr = 0;
    T yb[TM ? HR : 1];   // TM: the chunk's forward values of this lane
    // TM with tm_cw < N: rows tm_cw .. of each line in shared memory after the
    // ring, [warp][row - tm_cw][32]
    constexpr size_t kYsOff = ((size_t)NB * kTile * sizeof(T) + (TMA ? (size_t)NB * kQ * sizeof(Quad<T>) : 0) +
                               8 * NB + 16 + 15) / 16 * 16;
    const int ys_rows = TM ? max(0, nchunk * HR - tm_cw) : 0;
    float *ysw = reinterpret_cast<float *>(smem_raw + kYsOff) + (size_t)warp * ys_rows * 32 + lane;
    // TM: the line's backward-sweep coefficients cu_l of the block's z-class,
    // copied to shared memory while the forward sweep runs ([warp][row])
    const int cu_rows = TM ? (N + 31) / 32 * 32 : 0;
    T *cus = reinterpret_cast<T *>(smem_raw + kYsOff + (size_t)HW * ys_rows * 32 * sizeof(float)) +
             (size_t)warp * cu_rows;
    if constexpr (TMA) {
        if (threadIdx.x < NB) mbar_init(mbar + threadIdx.x, 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        __syncthreads();
        for (int b = 0; b < NB - 1 && b < nchunk; ++b) load_chunk(b, b);
        if constexpr (TM) {
            const T *cub = fcu + ((size_t)zcb * nl + mc) * N;   // the block class's row of this line
            for (int r = lane; r < cu_rows; r += 32)
                tile_copy(cus + r, cub + r, r < N);
            cp_async_commit();
            if (warp == 0) {
                __syncwarp();
                tm_alloc(tslot, tm_cols);
            }
            tm_fence_before();
            __syncthreads();
            tm_fence_after();
            tbase = *tslot;
            taddr = tbase + ((unsigned)(32 * (warp & 3)) << 16) + (unsigned)((warp >> 2) * tm_cw);
        }
    } else {
        load_chunk(0, 0);
    }
    auto put = [&](int r, T v) {
        if constexpr (TM) {
            yb[r] = v;
        } else {
            (void)r;
            if (active && GW_OK_G(dr, 108)) *dr = v;
            dr += rst;
        }
    };
    for (int ch = 0; ch < nchunk; ++ch) {
        const int buf = TMA ? ch % NB : ch & 1;
        if constexpr (TMA) {
            if (ch + NB - 1 < nchunk) load_chunk(ch + NB - 1, (ch + NB - 1) % NB);
            mbar_wait(mbar + buf, (unsigned)((ch / NB) & 1), err);
        } else {
            if (ch + 1 < nchunk) {
                load_chunk(ch + 1, (ch + 1) & 1);
                cp_async_wait<1>();
            } else {
                cp_async_wait<0>();
            }
            __syncthreads();
        }
        const T *row = tile + buf * kTile + warp * kSlotS + lane;
        const int l0 = ch * HR;
        const Quad<T> *qc = hql + l0;
        const Quad<T> *qsm = qtile + buf * kQ + warp * HR;   // this line's staged quads (TMA)
        auto quad = [&](int r) -> Quad<T> {
            if (qs_ok) return GW_OK_D(qsm + r, smem_raw, 114) ? qsm[r] : Quad<T>{};
            return GW_OK_G(qc + r, 104) ? qc[r] : Quad<T>{};
        };
        // pipe columns lie in rows prow_lo .. prow_hi of every line
        const bool chunk_pipe = line_pipe && l0 + HR > prow_lo && l0 <= prow_hi;
        if (l0 + HR <= N && !chunk_pipe) {
            // full chunk, no pipe column in it: straight-line rows
#pragma unroll
            for (int r0 = 0; r0 < HR; r0 += kHG) {
                Quad<T> q[kHG];
                T xm[kHG], xc[kHG], xp[kHG];
#pragma unroll
                for (int g = 0; g < kHG; ++g) {
                    q[g] = quad(r0 + g);
                    const T *rw = row + (r0 + g) * kRowS;
                    xm[g] = rd(rw); xc[g] = rd(rw + kSlotS); xp[g] = rd(rw + 2 * kSlotS);
                }
#pragma unroll
                for (int g = 0; g < kHG; ++g) {
                    y = fma(q[g].x, xc[g], fma(q[g].y, xp[g], fma(q[g].z, xm[g], -q[g].w * y)));
                    put(r0 + g, y);
                }
            }
        } else if (l0 + HR <= N) {
            // full chunk of a line through pipe columns: the same grouped rows,
            // with the advected pipe value (times ib) in place of the explicit
            // sweep at the pipe rows
#pragma unroll
            for (int r0 = 0; r0 < HR; r0 += kHG) {
                Quad<T> q[kHG];
                T xm[kHG], xc[kHG], xp[kHG], pv[kHG], iv[kHG];
                int pq[kHG];
#pragma unroll
                for (int g = 0; g < kHG; ++g) {
                    q[g] = quad(r0 + g);
                    const T *rw = row + (r0 + g) * kRowS;
                    xm[g] = rd(rw); xc[g] = rd(rw + kSlotS); xp[g] = rd(rw + 2 * kSlotS);
                    pq[g] = pipe_levels && GW_OK_G(pline + l0 + r0 + g, 105) ? __ldg(pline + l0 + r0 + g) : -1;
                }
#pragma unroll
                for (int g = 0; g < kHG; ++g) {
                    pv[g] = pq[g] >= 0 && GW_OK_G(pp + (size_t)pq[g] * countz + k, 106) ? pp[(size_t)pq[g] * countz + k] : T(0);
                    iv[g] = pq[g] >= 0 && GW_OK_G(fib + fb + l0 + r0 + g, 107) ? __ldg(fib + fb + l0 + r0 + g) : T(0);
                }
#pragma unroll
                for (int g = 0; g < kHG; ++g) {
                    const T ay = q[g].w * y;
                    y = pq[g] >= 0 ? fma(pv[g], iv[g], -ay) : fma(q[g].x, xc[g], fma(q[g].y, xp[g], fma(q[g].z, xm[g], -ay)));
                    put(r0 + g, y);
                }
            }
        } else {
            const int rmax = min(HR, N - l0);
            auto row_step = [&](int r) {
                const int l = l0 + r;
                const Quad<T> q = quad(r);
                const T *rw = row + r * kRowS;
                const T ay = q.w * y;
                T yn = fma(q.x, rd(rw + kSlotS), fma(q.y, rd(rw + 2 * kSlotS), fma(q.z, rd(rw), -ay)));
                const int pq = pipe_levels && GW_OK_G(pline + l, 105) ? __ldg(pline + l) : -1;
                if (pq >= 0)
                    yn = fma(GW_OK_G(pp + (size_t)pq * countz + k, 106) ? pp[(size_t)pq * countz + k] : T(0),
                             GW_OK_G(fib + fb + l, 107) ? __ldg(fib + fb + l) : T(0), -ay);
                y = yn;
            };
            if constexpr (TM) {
#pragma unroll
                for (int r = 0; r < HR; ++r) {
                    if (r < rmax) row_step(r);
                    yb[r] = y;
                }
            } else {
                for (int r = 0; r < rmax; ++r) {
                    row_step(r);
                    put(r, y);
                }
            }
        }
        if constexpr (TM) {
            __syncwarp();
            if (l0 < tm_cw) {
                // columns l0 .. l0 + HR - 1 of this lane (tm_cw is a multiple of HR)
                if (GW_OK_I(l0 + HR - 1, tm_cw, 115)) {
                    if constexpr (HR == 8) {
                        tm_st8(taddr + l0, yb);
                    } else {
                        tm_st16(taddr + l0, yb);
                        if constexpr (HR == 32) tm_st16(taddr + l0 + 16, yb + 16);
                    }
                }
            } else {
#pragma unroll
                for (int r = 0; r < HR; ++r) {
                    float *p = ysw + (size_t)(l0 - tm_cw + r) * 32;
                    if (GW_OK_D(p, smem_raw, 117)) *p = yb[r];
                }
            }
        }
        __syncthreads();   // the buffer is refilled NB - 1 chunks later
    }
    if constexpr (TM) {
        tm_wait_st();
        if (m < m_end) {
            const T *cuf = fcu + fb;
            // cu_l from shared memory where every lane is of the block's class
            cp_async_wait<0>();
            __syncwarp();
            const bool wq = __all_sync(0xffffffffu, qs_ok);
            auto cu_at = [&](int l) -> T {
                if (wq) return GW_OK_D(cus + l, smem_raw, 119) ? cus[l] : T(0);
                return GW_OK_G(cuf + l, 110) ? __ldg(cuf + l) : T(0);
            };
            if (kok && GW_OK_G(dl + (long long)(N - 1) * rst, 111)) __stcs(dl + (long long)(N - 1) * rst, y);
            T x = y;
            if (N >= 2) {
                int cb = (N - 2) >> 4;
                float cur[16], nxt[16];
                T cuc[16], cun[16];
                // rows rb .. rb + 15 from TMEM or, at and beyond tm_cw, from
                // shared memory (tm_cw is a multiple of 16)
                auto load_batch = [&](int rb, float *v) {
                    if (rb < tm_cw) {
                        if (GW_OK_I(rb + 15, tm_cw, 116)) tm_ld16(taddr + rb, v);
                        return;
                    }
#pragma unroll
                    for (int j = 0; j < 16; ++j) {
                        const float *p = ysw + (size_t)(rb - tm_cw + j) * 32;
                        v[j] = GW_OK_D(p, smem_raw, 118) ? *p : 0.f;
                    }
                };
                load_batch(16 * cb, cur);
#pragma unroll
                for (int j = 0; j < 16; ++j)
                    cuc[j] = 16 * cb + j < N ? cu_at(16 * cb + j) : T(0);
                tm_wait_ld(cur);   // (no TMEM load pending: returns at once)
                for (;;) {
                    const int r0 = 16 * cb;
                    if (cb > 0) {
                        load_batch(r0 - 16, nxt);
#pragma unroll
                        for (int j = 0; j < 16; ++j)
                            cun[j] = cu_at(r0 - 16 + j);
                    }
                    T *pc = dl + (long long)r0 * rst;
                    if (r0 + 15 <= N - 2) {
#pragma unroll
                        for (int j = 15; j >= 0; --j) {
                            x = cur[j] - cuc[j] * x;
                            if (kok && GW_OK_G(pc + (long long)j * rst, 111)) __stcs(pc + (long long)j * rst, x);
                        }
                    } else {
#pragma unroll
                        for (int j = 15; j >= 0; --j) {
                            if (r0 + j <= N - 2) {
                                x = cur[j] - cuc[j] * x;
                                if (kok && GW_OK_G(pc + (long long)j * rst, 111))
                                    __stcs(pc + (long long)j * rst, x);
                            }
                        }
                    }
                    if (cb == 0) break;
                    tm_wait_ld(nxt);
#pragma unroll
                    for (int j = 0; j < 16; ++j) { cur[j] = nxt[j]; cuc[j] = cun[j]; }
                    --cb;
                }
            }
        }
        tm_fence_before();
        __syncthreads();
        tm_fence_after();
        if (warp == 0) {
            __syncwarp();
            tm_dealloc(tbase, tm_cols);
        }
        return;
    }
    if (!active) return;
    // backward sweep: batches of kHB rows are loaded before the previous
    // batch is processed, so the loads overlap the dependent chain
    T x = y;
    const T *cuf = fcu + fb;
    T *pc = dl + (long long)(N - 2) * rst;   // row l = N - 2
    int l = N - 2;
    // full batches: rows l .. l - kHB + 1 all exist
    if (l - kHB + 1 >= 0) {
        T cur[kHB], cuc[kHB];
#pragma unroll
        for (int b = 0; b < kHB; ++b) {
            cur[b] = GW_OK_G(pc - (long long)b * rst, 109) ? pc[-(long long)b * rst] : T(0);
            cuc[b] = GW_OK_G(cuf + l - b, 110) ? __ldg(cuf + l - b) : T(0);
        }
        while (l - kHB + 1 >= 0) {
            const bool more = l - 2 * kHB + 1 >= 0;
            T nxt[kHB], cun[kHB];
            if (more) {
#pragma unroll
                for (int b = 0; b < kHB; ++b) {
                    nxt[b] = GW_OK_G(pc - (long long)(b + kHB) * rst, 109) ? pc[-(long long)(b + kHB) * rst] : T(0);
                    cun[b] = GW_OK_G(cuf + l - kHB - b, 110) ? __ldg(cuf + l - kHB - b) : T(0);
                }
            }
#pragma unroll
            for (int b = 0; b < kHB; ++b) {
                x = cur[b] - cuc[b] * x;
                if (GW_OK_G(pc - (long long)b * rst, 111)) __stcs(pc - (long long)b * rst, x);
            }
            pc -= (long long)kHB * rst;
            l -= kHB;
            if (!more) break;
#pragma unroll
            for (int b = 0; b < kHB; ++b) { cur[b] = nxt[b]; cuc[b] = cun[b]; }
        }
    }
    for (; l >= 0; --l) {
        x = (GW_OK_G(pc, 109) ? *pc : T(0)) - (GW_OK_G(cuf + l, 110) ? __ldg(cuf + l) : T(0)) * x;
        if (GW_OK_G(pc, 111)) __stcs(pc, x);
        pc -= rst;
    }
}

// 3b. the same half step with each line split into S segments, one warp per
//     (line, segment), 32 levels per warp.  The forward elimination
//     y_l = b_l + alpha_l y_{l-1} (alpha_l = -a_l ib_l, b_l the explicit
//     sweep folded with ib_l) and the back substitution x_l = y_l + delta_l
//     x_{l+1} (delta_l = -cu_l) are first-order linear recurrences: every
//     segment runs them from a zero start value, keeping its rows in
//     registers, and the true start values follow from a scan over the
//     segments' end values and end propagators (products of alpha or delta
//     over the segment), exchanged through shared memory:
//       y_l = y0_l + (prod_{s0..l} alpha) Y_in,   x_l = x0_l + (prod_{l..s1-1} delta) X_in.
//     The forward values never leave the registers, so the field crosses
//     HBM once in each direction; the neighbour lines of the explicit sweep
//     are read straight from global memory (L1/L2 serve the reuse).
template <typename T, bool XL, int HW, int S, int RMAX>
__global__ void __launch_bounds__(32 * HW * S) k_half_seg(T *__restrict__ dst, const T *__restrict__ src,
                                                          const T *__restrict__ pp,
                                                          const int *__restrict__ pipe_line,
                                                          const int *__restrict__ zclass,
                                                          const Quad<T> *__restrict__ hq,
                                                          const T *__restrict__ fib,
                                                          const T *__restrict__ fcu, int nx, int ny,
                                                          int nz, int pz, int countz, int m_begin, int m_end) {
    __shared__ T s_end[HW][S][32], s_prop[HW][S][32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int lw = warp / S, sg = warp % S;
    const int nl = XL ? ny : nx;
    const int N = XL ? nx : ny;
    const int k = blockIdx.x * 32 + lane;
    const int m = m_begin + blockIdx.y * HW + lw;
    const bool kok = k < nz;
    const bool active = kok && m < m_end;
    const int kc = kok ? k : nz - 1, mc = m < m_end ? m : m_end - 1;
    const long long mst = XL ? (long long)pz : (long long)pz * ny;
    const long long rst = XL ? (long long)pz * ny : (long long)pz;
    const int R = (N + S - 1) / S;                 // rows per segment (<= RMAX)
    const int s0 = sg * R;
    const int len = max(0, min(R, N - s0));
    const size_t fb = ((size_t)zclass[kc] * nl + mc) * N + s0;
    const Quad<T> *q = hq + fb;
    const T *cu = fcu + fb;
    // the line and its neighbours (clamped at the domain edge: the folded
    // coefficient of a missing neighbour is zero)
    const T *xc = src + kc + (long long)mc * mst + (long long)s0 * rst;
    const T *xm = mc > 0 ? xc - mst : xc;
    const T *xp = mc + 1 < nl ? xc + mst : xc;
    const bool line_pipe = __ldg(pipe_line + (size_t)nl * N + mc) != 0;
    const bool pipe_levels = line_pipe && k < countz;
    const int *pline = pipe_line + (size_t)mc * N + s0;

    // forward, local: y0 with a zero start value; P = prod of alpha
    T v[RMAX];
    T y = T(0), P = T(1);
    if (!line_pipe) {
#pragma unroll
        for (int r = 0; r < RMAX; ++r) {
            if (r < len) {
                const Quad<T> c = q[r];
                const long long o = (long long)r * rst;
                y = fma(c.x, xc[o], fma(c.y, xp[o], fma(c.z, xm[o], -c.w * y)));
                P *= -c.w;
                v[r] = y;
            }
        }
    } else {
#pragma unroll
        for (int r = 0; r < RMAX; ++r) {
            if (r < len) {
                const Quad<T> c = q[r];
                const long long o = (long long)r * rst;
                const int pq = pipe_levels ? __ldg(pline + r) : -1;
                const T b = pq >= 0 ? pp[(size_t)pq * countz + k] * __ldg(fib + fb + r)
                                    : fma(c.x, xc[o], fma(c.y, xp[o], c.z * xm[o]));
                y = fma(-c.w, y, b);
                P *= -c.w;
                v[r] = y;
            }
        }
    }
    s_end[lw][sg][lane] = y;
    s_prop[lw][sg][lane] = P;
    __syncthreads();
    T Y = T(0);
    for (int g = 0; g < sg; ++g) Y = fma(s_prop[lw][g][lane], Y, s_end[lw][g][lane]);
    // forward correction and local back substitution from a zero end value
    T Pl = T(1);
#pragma unroll
    for (int r = 0; r < RMAX; ++r) {
        if (r < len) {
            Pl *= -q[r].w;
            v[r] = fma(Pl, Y, v[r]);
        }
    }
    __syncthreads();   // s_end / s_prop are reused below
    T x = T(0), Q = T(1);
#pragma unroll
    for (int r = RMAX - 1; r >= 0; --r) {
        if (r < len) {
            const T d = -__ldg(cu + r);
            x = fma(d, x, v[r]);
            Q *= d;
            v[r] = x;
        }
    }
    s_end[lw][sg][lane] = x;     // x0 at the segment's first row
    s_prop[lw][sg][lane] = Q;    // prod of delta over the segment
    __syncthreads();
    T X = T(0);
    for (int g = S - 1; g > sg; --g) X = fma(s_prop[lw][g][lane], X, s_end[lw][g][lane]);
    if (!active) return;
    T *out = dst + k + (long long)m * mst + (long long)s0 * rst;
    T Ql = T(1);
#pragma unroll
    for (int r = RMAX - 1; r >= 0; --r) {
        if (r < len) {
            Ql *= -__ldg(cu + r);
            out[(long long)r * rst] = fma(Ql, X, v[r]);
        }
    }
}

// Mixed path, GW_MIXED_REFINE: one residual correction of a half step's
// line solves.  The float solve left x in dst for (I - h A_line) x = b, b the
// explicit sweep (I + h A_other) of src (the advected pipe value at pipe
// rows).  Per line, in double: r = b - (I - h A_line) x with the double
// coefficient tables, then (I - h A_line) d = r with the same LU factors the
// float solve used, and x <- x + d, rounded to float once.  One thread per
// line (lanes = levels, so every row access of a warp is contiguous); the
// forward values of the correction solve go to the scratch field yb.
// Coefficient layouts: line direction [zc][line][row] (lcm, lcp and the
// factors), the other direction [zc][row][line] (ecm, ecp).
template <bool XL>
__global__ void __launch_bounds__(128) k_half_refine(float *__restrict__ x, float *__restrict__ yb,
                                                     const float *__restrict__ src,
                                                     const float *__restrict__ pp,
                                                     const int *__restrict__ pipe_line,
                                                     const int *__restrict__ zclass,
                                                     const double *__restrict__ lcm,
                                                     const double *__restrict__ lcp,
                                                     const double *__restrict__ ecm,
                                                     const double *__restrict__ ecp,
                                                     const float *__restrict__ fa,
                                                     const float *__restrict__ fib,
                                                     const float *__restrict__ fcu, int nx, int ny,
                                                     int nz, int pz, int countz, double h) {
    const int nl = XL ? ny : nx, N = XL ? nx : ny;
    const int k = blockIdx.x * 32 + (threadIdx.x & 31);
    const int m = blockIdx.y * 4 + (threadIdx.x >> 5);
    if (k >= nz || m >= nl) return;
    const long long mst = XL ? (long long)pz : (long long)pz * ny;
    const long long rst = XL ? (long long)pz * ny : (long long)pz;
    const int zc = zclass[k];
    const size_t lb = ((size_t)zc * nl + m) * N;   // line-direction tables
    const bool pipe_levels = k < countz && __ldg(pipe_line + (size_t)nl * N + m) != 0;
    const int *pline = pipe_line + (size_t)m * N;
    const long long e0 = k + m * mst;
    auto b_at = [&](int l) -> double {   // right-hand side of row l, in double
        const long long e = e0 + l * rst;
        const int pq = pipe_levels ? __ldg(pline + l) : -1;
        if (pq >= 0) return (double)pp[(size_t)pq * countz + k];
        const double uc = src[e];
        const double up = m + 1 < nl ? (double)src[e + mst] : uc;
        const double um = m > 0 ? (double)src[e - mst] : uc;
        const size_t q = ((size_t)zc * N + l) * nl + m;
        return fma(h, __ldg(ecp + q) * (up - uc) - __ldg(ecm + q) * (uc - um), uc);
    };
    // rows in batches of kRB: the batch's loads are independent of the
    // recurrence and issue together, ahead of it
    constexpr int kRB = 8;
    double xm = 0.0, xc = x[e0], y = 0.0;
    for (int l0 = 0; l0 < N; l0 += kRB) {
        double xn[kRB], bb[kRB], cm[kRB], cp[kRB], fa_[kRB], fi_[kRB];
#pragma unroll
        for (int r = 0; r < kRB; ++r) {
            const int l = l0 + r;
            if (l < N) {
                xn[r] = l + 1 < N ? (double)x[e0 + (l + 1) * rst] : 0.0;
                bb[r] = b_at(l);
                cm[r] = __ldg(lcm + lb + l); cp[r] = __ldg(lcp + lb + l);
                fa_[r] = (double)__ldg(fa + lb + l); fi_[r] = (double)__ldg(fib + lb + l);
            }
        }
#pragma unroll
        for (int r = 0; r < kRB; ++r) {
            const int l = l0 + r;
            if (l < N) {
                const double xp = xn[r];
                double ax = (1.0 + h * (cm[r] + cp[r])) * xc;
                if (l > 0) ax -= h * cm[r] * xm;
                if (l + 1 < N) ax -= h * cp[r] * xp;
                y = (bb[r] - ax - fa_[r] * y) * fi_[r];
                yb[e0 + l * rst] = (float)y;
                xm = xc;
                xc = xp;
            }
        }
    }
    // back substitution of the correction, added to x (x_{N-1} first)
    double d = y;
    long long e = e0 + (long long)(N - 1) * rst;
    x[e] = (float)((double)x[e] + d);
    for (int l1 = N - 2; l1 >= 0; l1 -= kRB) {
        float yv[kRB], xv[kRB];
        double cu[kRB];
#pragma unroll
        for (int r = 0; r < kRB; ++r) {
            const int l = l1 - r;
            if (l >= 0) {
                const long long el = e0 + (long long)l * rst;
                yv[r] = yb[el]; xv[r] = x[el]; cu[r] = (double)__ldg(fcu + lb + l);
            }
        }
#pragma unroll
        for (int r = 0; r < kRB; ++r) {
            const int l = l1 - r;
            if (l >= 0) {
                d = (double)yv[r] - cu[r] * d;
                x[e0 + (long long)l * rst] = (float)((double)xv[r] + d);
            }
        }
    }
}

// GW_MIXED_REFINE on the FP32 pipe.  The residual r = b - (I - h A_line) x
// of k_half_refine, computed in double-float arithmetic (a value as an
// unevaluated sum hi + lo of two floats: about 44 bits) instead of double:
// GB300 runs float arithmetic at many times its FP64 rate.  Products with a
// float are exact through fmaf, sums use two-sum (Knuth, Dekker); every
// operation is a correctly rounded intrinsic, never contracted, so the
// error-free transformations hold.  The residual depends only on the float
// solution x and on b, so it is formed for a batch of rows ahead of the
// correction's recurrence, which runs in float (the correction is small
// against x: its own rounding is below the float rounding of x + d).
struct Df {
    float hi, lo;
};
__device__ __forceinline__ Df df_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b), bb = __fsub_rn(s, a);
    return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
__device__ __forceinline__ Df df_fast(float a, float b) {   // |a| >= |b| or a == 0
    const float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ Df df_mul_f(Df a, float b) {
    const float p = __fmul_rn(a.hi, b);
    return df_fast(p, __fmaf_rn(a.lo, b, __fmaf_rn(a.hi, b, -p)));
}
__device__ __forceinline__ Df df_mul(Df a, Df b) {
    const float p = __fmul_rn(a.hi, b.hi);
    return df_fast(p, __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, __fmaf_rn(a.hi, b.hi, -p))));
}
__device__ __forceinline__ Df df_add(Df a, Df b) {
    const Df s = df_two_sum(a.hi, b.hi);
    return df_fast(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}
__device__ __forceinline__ Df df_neg(Df a) { return {-a.hi, -a.lo}; }

// Per step size: h c_m, h c_p (float4: hi, lo, hi, lo) and 1 + h (c_m + c_p)
// (float2) of one direction's double coefficient table, as double-float.
__global__ void k_refine_tables(float4 *__restrict__ hmp, float2 *__restrict__ dg,
                                const double *__restrict__ cm, const double *__restrict__ cp, double h,
                                size_t n) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    auto split = [](double v, float &hi, float &lo) {
        hi = __double2float_rn(v);
        lo = __double2float_rn(__dsub_rn(v, (double)hi));
    };
    const double a = __dmul_rn(h, cm[i]), b = __dmul_rn(h, cp[i]);
    const double d = __dadd_rn(1.0, __dmul_rn(h, __dadd_rn(cm[i], cp[i])));
    float4 q;
    float2 g;
    split(a, q.x, q.y);
    split(b, q.z, q.w);
    split(d, g.x, g.y);
    hmp[i] = q;
    dg[i] = g;
}

// Line-direction tables lq/lg at [zc][line][row], the other direction's eq at
// [zc][row][line] (the coefficient layouts of k_half_refine).
template <bool XL>
__global__ void __launch_bounds__(128) k_half_refine_df(float *__restrict__ x, float *__restrict__ yb,
                                                        const float *__restrict__ src,
                                                        const float *__restrict__ pp,
                                                        const int *__restrict__ pipe_line,
                                                        const int *__restrict__ zclass,
                                                        const float4 *__restrict__ lq,
                                                        const float2 *__restrict__ lg,
                                                        const float4 *__restrict__ eq,
                                                        const float *__restrict__ fa,
                                                        const float *__restrict__ fib,
                                                        const float *__restrict__ fcu, int nx, int ny,
                                                        int nz, int pz, int countz) {
    const int nl = XL ? ny : nx, N = XL ? nx : ny;
    const int k = blockIdx.x * 32 + (threadIdx.x & 31);
    const int m = blockIdx.y * 4 + (threadIdx.x >> 5);
    if (k >= nz || m >= nl) return;
    const long long mst = XL ? (long long)pz : (long long)pz * ny;
    const long long rst = XL ? (long long)pz * ny : (long long)pz;
    const int zc = zclass[k];
    const size_t lb = ((size_t)zc * nl + m) * N;   // line-direction tables
    const bool pipe_levels = k < countz && __ldg(pipe_line + (size_t)nl * N + m) != 0;
    const int *pline = pipe_line + (size_t)m * N;
    const long long e0 = k + m * mst;
    constexpr int kRB = 4;
    float xm = 0.f, xc = x[e0], y = 0.f;
    for (int l0 = 0; l0 < N; l0 += kRB) {
        float xn[kRB], uc[kRB], up[kRB], um[kRB], pv[kRB], fa_[kRB], fi_[kRB];
        float4 L[kRB], E[kRB];
        float2 G[kRB];
        int pq[kRB];
#pragma unroll
        for (int r = 0; r < kRB; ++r) {   // the batch's loads, ahead of the arithmetic
            const int l = l0 + r;
            if (l < N) {
                const long long e = e0 + (long long)l * rst;
                xn[r] = l + 1 < N ? x[e + rst] : 0.f;
                pq[r] = pipe_levels ? __ldg(pline + l) : -1;
                pv[r] = pq[r] >= 0 ? pp[(size_t)pq[r] * countz + k] : 0.f;
                uc[r] = src[e];
                up[r] = m + 1 < nl ? src[e + mst] : uc[r];
                um[r] = m > 0 ? src[e - mst] : uc[r];
                E[r] = __ldg(eq + ((size_t)zc * N + l) * nl + m);
                L[r] = __ldg(lq + lb + l);
                G[r] = __ldg(lg + lb + l);
                fa_[r] = __ldg(fa + lb + l);
                fi_[r] = __ldg(fib + lb + l);
            }
        }
        float rr[kRB];
#pragma unroll
        for (int r = 0; r < kRB; ++r) {   // residuals: depend on x and b only
            const int l = l0 + r;
            if (l < N) {
                Df b;
                if (pq[r] >= 0) {
                    b = {pv[r], 0.f};
                } else {   // b = u + h c_p (u+ - u) - h c_m (u - u-)
                    const Df t1 = df_mul({E[r].z, E[r].w}, df_two_sum(up[r], -uc[r]));
                    const Df t2 = df_mul({E[r].x, E[r].y}, df_two_sum(uc[r], -um[r]));
                    b = df_add(Df{uc[r], 0.f}, df_add(t1, df_neg(t2)));
                }
                Df ax = df_mul_f({G[r].x, G[r].y}, xc);   // (1 + h (c_m + c_p)) x_l
                if (l > 0) ax = df_add(ax, df_neg(df_mul_f({L[r].x, L[r].y}, xm)));
                if (l + 1 < N) ax = df_add(ax, df_neg(df_mul_f({L[r].z, L[r].w}, xn[r])));
                const Df res = df_add(b, df_neg(ax));
                rr[r] = __fadd_rn(res.hi, res.lo);
                xm = xc;
                xc = xn[r];
            }
        }
#pragma unroll
        for (int r = 0; r < kRB; ++r) {   // the correction's forward elimination
            const int l = l0 + r;
            if (l < N) {
                y = (rr[r] - fa_[r] * y) * fi_[r];
                yb[e0 + (long long)l * rst] = y;
            }
        }
    }
    // back substitution of the correction, added to x (x_{N-1} first)
    float d = y;
    long long e = e0 + (long long)(N - 1) * rst;
    x[e] = x[e] + d;
    constexpr int kBB = 8;
    for (int l1 = N - 2; l1 >= 0; l1 -= kBB) {
        float yv[kBB], xv[kBB], cu[kBB];
#pragma unroll
        for (int r = 0; r < kBB; ++r) {
            const int l = l1 - r;
            if (l >= 0) {
                const long long el = e0 + (long long)l * rst;
                yv[r] = yb[el]; xv[r] = x[el]; cu[r] = __ldg(fcu + lb + l);
            }
        }
#pragma unroll
        for (int r = 0; r < kBB; ++r) {
            const int l = l1 - r;
            if (l >= 0) {
                d = yv[r] - cu[r] * d;
                x[e0 + (long long)l * rst] = xv[r] + d;
            }
        }
    }
}

// mixed path field conversion: theta = T - T_ref(z) and back
// (T: nz levels per column; theta: columns pz floats apart, pz >= nz)
__global__ void k_to_theta(float *__restrict__ th, const double *__restrict__ T,
                           const double *__restrict__ Tref, size_t n, int nz, int pz) {
    for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x) {
        const size_t col = q / nz, k = q - col * nz;
        th[col * pz + k] = (float)(T[q] - Tref[k]);
    }
}
__global__ void k_from_theta(double *__restrict__ T, const float *__restrict__ th,
                             const double *__restrict__ Tref, size_t n, int nz, int pz) {
    for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x) {
        const size_t col = q / nz, k = q - col * nz;
        T[q] = (double)th[col * pz + k] + Tref[k];
    }
}

template <typename T>
__global__ void k_finite(const T *__restrict__ u, size_t n, int *__restrict__ flag) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    size_t s = (size_t)gridDim.x * blockDim.x;
    bool bad = false;
    for (; i < n; i += s) bad |= !isfinite((double)u[i]);
    if (__syncthreads_or(bad) && threadIdx.x == 0) atomicExch(flag, 1);
}

template <typename T>
struct Bufs {
    T *u, *temp, *tp, *pp;
    const GwCoefTables<T> *ct;
    const T *fref;
    const double *Tref;
};

template <typename T>
Bufs<T> bufs(gw_ctx *c);
template <>
Bufs<double> bufs<double>(gw_ctx *c) {
    return {c->d_u, c->d_temp, c->d_tp, c->d_pp, &c->c64, nullptr, nullptr};
}
template <>
Bufs<float> bufs<float>(gw_ctx *c) {
    return {c->f_u, c->f_temp, c->f_tp, c->f_pp, &c->c32, c->f_fref, c->d_Tref};
}

template <typename T>
size_t rock2_smem(int nz) {
    const bool inc = sizeof(T) == 4;   // the float path runs the increment form
    return (size_t)nz * sizeof(T) * (inc ? 4 : 2);
}

// largest shared-memory block of the column kernel k_rock2_col
constexpr size_t kColumnSmemMax = 200 * 1024;

template <typename T>
size_t reg_smem(int lpt, int nt = 256) { return 2 * (size_t)(nt * lpt + nt * lpt / 32) * sizeof(T); }

// levels per thread of the register-resident ROCK2 kernel (0: use the
// shared-memory kernel).  Float columns of up to 2048 levels take 4 to 8 per
// thread: few threads per column leave more columns, each an independent
// chain of stages and barriers, in flight per SM (nz = 402: 0.329 -> 0.308 ms
// per step with 8 against 2 per thread), and among 4..8 the count that pads
// the column least (nt LPT levels, nt a multiple of 32) does the least
// work: nz = 402 takes 7 (448 levels, not 512), nz = 301 takes 5 (320, not
// 512).  Double columns keep 2 / 4 / 8, which the FP64 pipe prefers.
inline int rock2_lpt(int nz, bool f32) {
    if (f32 && nz <= 2048) {
        int best = 8, pad = ((nz + 7) / 8 + 31) / 32 * 32 * 8;
        for (int L = 7; L >= 4; --L) {
            const int nt = ((nz + L - 1) / L + 31) / 32 * 32;
            if (nt <= 256 && nt * L < pad) { best = L; pad = nt * L; }
        }
        return best;
    }
    if (nz <= 512) return 2;
    if (nz <= 1024) return 4;
    if (nz <= 2048) return 8;
    if (nz <= 4096) return 16;
    return 0;
}

template <typename T>
const T *stage_table(gw_ctx *c);
template <>
const double *stage_table<double>(gw_ctx *c) { return c->d_stage; }
template <>
const float *stage_table<float>(gw_ctx *c) { return c->f_stage; }

// Window kernel: staging buffers per warp, warps per block.
constexpr int kWinNB = 3, kWinWarps = 8;
inline size_t win_smem(int lpt) { return (size_t)kWinWarps * kWinNB * (32 * lpt + lpt) * sizeof(float); }

// Levels per lane and window count of k_rock2_win for nz levels and s stages:
// among 4..8 levels per lane, the fewest padded levels (windows x W); 0 when
// the halo (s levels per interior edge) would exceed a quarter of the window
// or a column would need more windows than a block has warps (its windows
// share a block; deeper columns take the block kernel).
inline int rock2_win_lpt(int nz, int s, int *nwin) {
    int best = 0, bn = 0;
    long long bw = 0;
    for (int L = 8; L >= 4; --L) {
        const int W = 32 * L;
        if (8 * s > W) continue;
        const int n = nz <= W ? 1 : 1 + (nz - W + (W - 2 * s) - 1) / (W - 2 * s);
        if (n > kWinWarps) continue;
        if (!best || (long long)n * W < bw) { best = L; bn = n; bw = (long long)n * W; }
    }
    *nwin = bn;
    return best;
}

template <int LPT>
int launch_rock2_win(gw_ctx *c, int s, int nwin, float *u, const float *czm, const float *czp,
                     const float *fref, const int *order, long long ncols, cudaStream_t st) {
    auto kern = s == 3 ? k_rock2_win<LPT, kWinNB, true> : k_rock2_win<LPT, kWinNB, false>;
    // blocks of whole column slots: spb slots of nwin warps (nwin <= kWinWarps)
    const int spb = kWinWarps / nwin, warps = spb * nwin;
    // resident blocks per SM: those of kWinWarps warps, scaled to this size
    const long long per_sm =
        std::max(1LL, (long long)(c->rock2w_per_sm[LPT] > 0 ? c->rock2w_per_sm[LPT] : 1) * kWinWarps / warps);
    const long long need = (ncols + spb - 1) / spb;
    const long long grid = std::max(1LL, std::min(per_sm * c->sms, need));
    const size_t smem = (size_t)warps * kWinNB * (32 * LPT + LPT) * sizeof(float);
    kern<<<(unsigned)grid, 32 * warps, smem, st>>>(
        u, order, c->d_colprof, czm, czp, fref, c->f_stage, s, c->nz, c->pz, (int)ncols, nwin);
    GW_CUDA(cudaGetLastError());
    return GW_OK;
}

template <typename T, bool INC>
int launch_rock2_t(gw_ctx *c, int s, T *u, const T *czm, const T *czp, const T *fref,
                   const int *order = nullptr, long long ncols = -1, cudaStream_t st = nullptr) {
    if (!st) st = c->stream;
    if (!order) order = c->d_colorder;
    if (ncols < 0) ncols = (long long)c->nx * c->ny;
    if (ncols == 0) return GW_OK;
    if constexpr (sizeof(T) == 4 && INC) {
        int nwin = 0;
        const int wl = c->rock2_block ? 0 : rock2_win_lpt(c->nz, s, &nwin);
        switch (wl) {
            case 4: return launch_rock2_win<4>(c, s, nwin, u, czm, czp, fref, order, ncols, st);
            case 5: return launch_rock2_win<5>(c, s, nwin, u, czm, czp, fref, order, ncols, st);
            case 6: return launch_rock2_win<6>(c, s, nwin, u, czm, czp, fref, order, ncols, st);
            case 7: return launch_rock2_win<7>(c, s, nwin, u, czm, czp, fref, order, ncols, st);
            case 8: return launch_rock2_win<8>(c, s, nwin, u, czm, czp, fref, order, ncols, st);
            default: break;
        }
    }
    const int lpt = rock2_lpt(c->nz, sizeof(T) == 4);
    unsigned grid = (unsigned)(ncols < (long long)c->rock2_grid ? ncols : c->rock2_grid);
    switch (lpt) {
        case 2: k_rock2_reg<T, INC, 2><<<grid, c->rock2_nt, reg_smem<T>(2, c->rock2_nt), st>>>(u, order, c->d_colprof, czm, czp, fref, stage_table<T>(c), s, c->nz, c->pz, ncols); break;
        case 4: k_rock2_reg<T, INC, 4><<<grid, c->rock2_nt, reg_smem<T>(4, c->rock2_nt), st>>>(u, order, c->d_colprof, czm, czp, fref, stage_table<T>(c), s, c->nz, c->pz, ncols); break;
        case 5: if constexpr (sizeof(T) == 4) k_rock2_reg<T, INC, 5><<<grid, c->rock2_nt, reg_smem<T>(5, c->rock2_nt), st>>>(u, order, c->d_colprof, czm, czp, fref, stage_table<T>(c), s, c->nz, c->pz, ncols); break;
        case 6: if constexpr (sizeof(T) == 4) k_rock2_reg<T, INC, 6><<<grid, c->rock2_nt, reg_smem<T>(6, c->rock2_nt), st>>>(u, order, c->d_colprof, czm, czp, fref, stage_table<T>(c), s, c->nz, c->pz, ncols); break;
        case 7: if constexpr (sizeof(T) == 4) k_rock2_reg<T, INC, 7><<<grid, c->rock2_nt, reg_smem<T>(7, c->rock2_nt), st>>>(u, order, c->d_colprof, czm, czp, fref, stage_table<T>(c), s, c->nz, c->pz, ncols); break;
        case 8: k_rock2_reg<T, INC, 8><<<grid, c->rock2_nt, reg_smem<T>(8, c->rock2_nt), st>>>(u, order, c->d_colprof, czm, czp, fref, stage_table<T>(c), s, c->nz, c->pz, ncols); break;
        case 16: k_rock2_reg<T, INC, 16><<<grid, c->rock2_nt, reg_smem<T>(16, c->rock2_nt), st>>>(u, order, c->d_colprof, czm, czp, fref, stage_table<T>(c), s, c->nz, c->pz, ncols); break;
        default:
            k_rock2_col<T, INC><<<grid, 256, rock2_smem<T>(c->nz), st>>>(u, c->d_colprof, czm, czp, fref,
                                                                            c->d_stage, s, c->nz, c->pz, ncols);
    }
    GW_CUDA(cudaGetLastError());
    return GW_OK;
}

// GW_MIXED_ROCK2_F64: the column kernel with double stages over the float
// field (double tables, the double A_z T_ref source), LPT by the double rule.
int launch_rock2_f64(gw_ctx *c, int s, const int *order, long long ncols, cudaStream_t st = nullptr) {
    if (!st) st = c->stream;
    if (!order) order = c->d_colorder;
    if (ncols < 0) ncols = (long long)c->nx * c->ny;
    if (ncols == 0) return GW_OK;
    const int lpt = rock2_lpt(c->nz, false), nt = c->rock2_nt64;
    const unsigned grid = (unsigned)(ncols < (long long)c->rock2_grid64 ? ncols : c->rock2_grid64);
    const double *czm = c->c64.czm, *czp = c->c64.czp, *fr = c->d_fref64, *sc = c->d_stage;
    switch (lpt) {
        case 2: k_rock2_reg<float, true, 2, double><<<grid, nt, reg_smem<float>(2, nt), st>>>(c->f_u, order, c->d_colprof, czm, czp, fr, sc, s, c->nz, c->pz, ncols); break;
        case 4: k_rock2_reg<float, true, 4, double><<<grid, nt, reg_smem<float>(4, nt), st>>>(c->f_u, order, c->d_colprof, czm, czp, fr, sc, s, c->nz, c->pz, ncols); break;
        case 8: k_rock2_reg<float, true, 8, double><<<grid, nt, reg_smem<float>(8, nt), st>>>(c->f_u, order, c->d_colprof, czm, czp, fr, sc, s, c->nz, c->pz, ncols); break;
        case 16: k_rock2_reg<float, true, 16, double><<<grid, nt, reg_smem<float>(16, nt), st>>>(c->f_u, order, c->d_colprof, czm, czp, fr, sc, s, c->nz, c->pz, ncols); break;
        default: return gw_fail(GW_ERR_UNSUPPORTED, "GW_MIXED_ROCK2_F64 supports nz <= 4096");
    }
    GW_CUDA(cudaGetLastError());
    return GW_OK;
}

template <typename T>
int launch_rock2(gw_ctx *c, int s, const int *order = nullptr, long long ncols = -1, cudaStream_t st = nullptr) {
    if (sizeof(T) == 4 && (c->mixed_flags & GW_MIXED_ROCK2_F64)) return launch_rock2_f64(c, s, order, ncols, st);
    Bufs<T> B = bufs<T>(c);
    if (sizeof(T) == 4)
        return launch_rock2_t<float, true>(c, s, (float *)B.u, (const float *)B.ct->czm,
                                           (const float *)B.ct->czp, (const float *)B.fref, order, ncols, st);
    return launch_rock2_t<double, false>(c, s, (double *)B.u, (const double *)B.ct->czm,
                                         (const double *)B.ct->czp, nullptr, order, ncols, st);
}

// explicit sweep along edir at the pipe columns, outlet/annulus means, advection
template <typename T>
int launch_pipe(gw_ctx *c, const T *src, int edir, double h, cudaStream_t st = nullptr) {
    Bufs<T> B = bufs<T>(c);
    if (!st) st = c->stream;
    const T *cm = edir == GW_DIR_X ? B.ct->cxm : B.ct->cym;
    const T *cp = edir == GW_DIR_X ? B.ct->cxp : B.ct->cyp;
    if (c->n_pipe_chunks > 0) {
        const dim3 g = chunk_grid(grid_for(c->nz, 128), c->n_pipe_chunks);
        k_pipe_sweep<T><<<g, 128, 0, st>>>(B.tp, c->d_pipepart, src, c->d_pipe_chunks,
                                                  c->d_pipe_i, c->d_pipe_j, c->d_zclass, cm, cp,
                                                  B.Tref, c->nx, c->ny, c->nz, c->pz, h, edir, c->n_pipe_chunks);
        GW_CUDA(cudaGetLastError());
    }
    dim3 gr((c->nz + 31) / 32, c->nbh);
    k_pipe_reduce<<<gr, 32 * kReduceWarps, 0, st>>>(c->d_outlet, c->d_annmean, c->d_pipepart, c->d_bchunk,
                                                    c->d_nlev, c->d_bh, c->nz);
    GW_CUDA(cudaGetLastError());
    if (c->inlet_kind == GW_INLET_SCHEDULE || c->inlet_kind == GW_INLET_EXPRESSION) {
        // first advection of the step at its end time, the second half a step later
        const bool prog = c->inlet_kind == GW_INLET_EXPRESSION;
        k_inlet_eval<<<1, 32, 0, st>>>(c->d_inlet, c->d_sched, c->n_sched, c->d_time, c->d_step_counter,
                                       edir == GW_DIR_Y ? 0.0 : 0.5, c->nbh, c->d_prog_op, c->d_prog_arg,
                                       prog ? c->n_prog : 0, c->d_outlet);
        GW_CUDA(cudaGetLastError());
    }
    if (c->n_pipe_chunks > 0 && c->countz > 0) {
        const dim3 ga = chunk_grid((c->countz + 127) / 128, c->n_pipe_chunks);
        k_advect_c<T><<<ga, 128, 0, st>>>(B.pp, B.tp, c->d_advtab, c->d_pipe_chunks, c->d_annmean,
                                          c->d_outlet, B.Tref, c->nz, c->countz, c->inlet_kind,
                                          c->inlet_param, c->d_inlet, c->n_pipe_chunks);
        GW_CUDA(cudaGetLastError());
    }
    return GW_OK;
}

template <typename T>
size_t half_smem(int cfg) { return 2 * (size_t)kTileHR[cfg] * (kTileHW[cfg] + 2) * 32 * sizeof(T); }

// tensor-map tiles: ring depth per tiling (the two largest tiles stay at two),
// shared memory with the ring's mbarriers
constexpr int kTileNB[6] = {3, 3, 3, 2, 3, 2};
template <int HW, int HR, int NB>
constexpr size_t tma_smem() {
    return (size_t)NB * HR * (HW + 2) * 32 * sizeof(float) + (size_t)NB * HW * HR * 4 * sizeof(float) + 8 * NB + 16;
}

// TMEM columns per line slot of the TM half step: a power of two >= N (and
// >= 32, the smallest allocation); 0 for blocks of fewer than four lines
// (half of the TMEM lanes would stay unused) or whose slots would not fit the
// SM's 512 columns: the forward values then go through global memory
// shared memory of the TM half step's staged backward-sweep coefficients
inline size_t tm_cu_smem(int N, int HW) { return (size_t)HW * ((N + 31) / 32 * 32) * sizeof(float); }

inline int tm_columns(int N, int HW) {
    if (HW < 4) return 0;
    int cw = 32;
    while (cw < N) cw *= 2;
    return cw * ((HW + 3) / 4) <= 512 ? cw : 0;
}

// the tensor map of src's tiles, or null (another buffer, or no maps)
inline const CUtensorMap *tile_map(const gw_ctx *c, const void *src, int xlines, int cfg) {
    if (!c->tma_ok || cfg < 0 || cfg >= 6) return nullptr;
    const int b = src == (const void *)c->f_u ? 0 : src == (const void *)c->f_temp ? 1 : -1;
    return b < 0 ? nullptr : &c->tmaps[b][xlines ? 0 : 1][cfg];
}

// Where the mixed half step of HW-line x HR-row tensor-map tiles keeps its
// forward values: 0 global memory, 1 whole lines in TMEM (*cw columns per
// block), 2 the split form (rows 0..127 in TMEM, the rest in shared memory;
// *sm2 bytes of shared memory per block).
template <int HW, int HR>
int half_tm_mode(const gw_ctx *c, int xlines, int *cw, size_t *sm2) {
    const int N = xlines ? c->nx : c->ny;
    // forward values in TMEM where the block's lines fit the SM's columns
    *cw = tm_columns(N, HW);
    // ... and where the whole half step (every line of the direction, over
    // however many launches the step splits it into) has at least four
    // rounds of the blocks an SM runs with them: with fewer, the last round
    // leaves SMs idle for a block's whole line, and the global-memory form,
    // five or more resident blocks per SM, does the step in fewer rounds
    const long long full_blocks = (long long)((c->nz + 31) / 32) * (((xlines ? c->ny : c->nx) + HW - 1) / HW);
    auto enough = [&](int active) { return c->half_tm_force || full_blocks >= 4LL * active * c->sms; };
    if constexpr (HW == 4 && HR == 16) {
        // rows 0..127 in TMEM, the rest in the block's shared memory (ring
        // of two), where that keeps more blocks per SM at work than whole
        // lines in TMEM (512 / cw blocks): e.g. 205-row lines, 3 against 2
        if (*cw > 128 && c->half_split && c->smem_per_sm > 0) {
            const size_t ys = (size_t)HW * (((N + HR - 1) / HR) * HR - 128) * 32 * sizeof(float);
            *sm2 = (tma_smem<HW, HR, 2>() + 15) / 16 * 16 + ys + tm_cu_smem(N, HW);
            const int fit = c->smem_per_sm / (int)(*sm2 + 1024);
            if (std::min(4, fit) > 512 / *cw && enough(std::min(4, fit))) return 2;
        }
    }
    return *cw > 0 && enough(512 / (*cw * ((HW + 3) / 4))) ? 1 : 0;
}

template <typename T, int HW, int HR, int NB>
void half_launch(gw_ctx *c, cudaStream_t st, T *dst, const T *src, int xlines, const Quad<T> *hq,
                 const GwFactors<T> &f, const T *pp, size_t smem, int mb, int me, const CUtensorMap *map,
                 const CUtensorMap *qmap, bool tm) {
    static const CUtensorMap kNoMap = {};
    dim3 grid((c->nz + 31) / 32, (me - mb + HW - 1) / HW);
    // rows along the lines that hold pipe columns (chunks outside take the fast path)
    const int plo = xlines ? c->ilo : c->jlo, phi = xlines ? c->ihi : c->jhi;
    if constexpr (sizeof(T) == 4) {
        int cw = 0;
        size_t sm2 = 0;
        const int mode = tm && map && qmap ? half_tm_mode<HW, HR>(c, xlines, &cw, &sm2) : 0;
        if constexpr (HW == 4 && HR == 16) {
            if (mode == 2) {
                const CUtensorMap &qm = *qmap;
                if (xlines)
                    k_half_tile<T, true, HW, HR, 2, true, true><<<grid, 32 * HW, sm2, st>>>(
                        dst, src, pp, c->d_pipe_lx, c->d_zclass, hq, f.ib, f.cu, c->nx, c->ny, c->nz, c->pz,
                        c->countz, mb, me, *map, qm, c->d_err, 128, plo, phi);
                else
                    k_half_tile<T, false, HW, HR, 2, true, true><<<grid, 32 * HW, sm2, st>>>(
                        dst, src, pp, c->d_pipe_ly, c->d_zclass, hq, f.ib, f.cu, c->nx, c->ny, c->nz, c->pz,
                        c->countz, mb, me, *map, qm, c->d_err, 128, plo, phi);
                return;
            }
        }
        if (mode == 1) {
            const CUtensorMap &qm = *qmap;
            const size_t smt = (tma_smem<HW, HR, NB>() + 15) / 16 * 16 + tm_cu_smem(xlines ? c->nx : c->ny, HW);
            if (xlines)
                k_half_tile<T, true, HW, HR, NB, true, true><<<grid, 32 * HW, smt, st>>>(
                    dst, src, pp, c->d_pipe_lx, c->d_zclass, hq, f.ib, f.cu, c->nx, c->ny, c->nz, c->pz, c->countz,
                    mb, me, *map, qm, c->d_err, cw, plo, phi);
            else
                k_half_tile<T, false, HW, HR, NB, true, true><<<grid, 32 * HW, smt, st>>>(
                    dst, src, pp, c->d_pipe_ly, c->d_zclass, hq, f.ib, f.cu, c->nx, c->ny, c->nz, c->pz, c->countz,
                    mb, me, *map, qm, c->d_err, cw, plo, phi);
            return;
        }
        if (map && qmap) {
            const CUtensorMap &qm = *qmap;
            if (xlines)
                k_half_tile<T, true, HW, HR, NB, true><<<grid, 32 * HW, tma_smem<HW, HR, NB>(), st>>>(
                    dst, src, pp, c->d_pipe_lx, c->d_zclass, hq, f.ib, f.cu, c->nx, c->ny, c->nz, c->pz, c->countz,
                    mb, me, *map, qm, c->d_err, 0, plo, phi);
            else
                k_half_tile<T, false, HW, HR, NB, true><<<grid, 32 * HW, tma_smem<HW, HR, NB>(), st>>>(
                    dst, src, pp, c->d_pipe_ly, c->d_zclass, hq, f.ib, f.cu, c->nx, c->ny, c->nz, c->pz, c->countz,
                    mb, me, *map, qm, c->d_err, 0, plo, phi);
            return;
        }
    }
    if (xlines)
        k_half_tile<T, true, HW, HR><<<grid, 32 * HW, smem, st>>>(
            dst, src, pp, c->d_pipe_lx, c->d_zclass, hq, f.ib, f.cu, c->nx, c->ny, c->nz, c->pz, c->countz, mb, me,
            kNoMap, kNoMap, c->d_err, 0, plo, phi);
    else
        k_half_tile<T, false, HW, HR><<<grid, 32 * HW, smem, st>>>(
            dst, src, pp, c->d_pipe_ly, c->d_zclass, hq, f.ib, f.cu, c->nx, c->ny, c->nz, c->pz, c->countz, mb, me,
            kNoMap, kNoMap, c->d_err, 0, plo, phi);
}

template <typename T>
int launch_half(gw_ctx *c, T *dst, const T *src, int xlines, double h, int mb = 0, int me = -1,
                cudaStream_t st = nullptr) {
    (void)h;   // folded into the half-step tables
    Bufs<T> B = bufs<T>(c);
    const GwFactors<T> &f = xlines ? B.ct->fx : B.ct->fy;
    const Quad<T> *hq = reinterpret_cast<const Quad<T> *>(xlines ? B.ct->hx : B.ct->hy);
    const int nl = xlines ? c->ny : c->nx;
    if (me < 0) me = nl;                       // lines mb .. me - 1
    if (!st) st = c->stream;
    if (me <= mb) return GW_OK;
    int cfg = c->half_cfg;
    const int N = xlines ? c->nx : c->ny;
    // tilings 7..12: the row tiles 0..5 with the forward values in global memory
    const bool tm = c->half_tmem && cfg < kSegCfg;
    if (cfg >= kGlobalCfg) cfg -= kGlobalCfg;
    if (cfg == kSegCfg) {
        if (N <= kSegS * kSegR) {
            dim3 grid((c->nz + 31) / 32, (me - mb + 1) / 2);
            if (xlines)
                k_half_seg<T, true, 2, kSegS, kSegR><<<grid, 32 * 2 * kSegS, 0, st>>>(
                    dst, src, B.pp, c->d_pipe_lx, c->d_zclass, hq, f.ib, f.cu, c->nx, c->ny, c->nz, c->pz, c->countz,
                    mb, me);
            else
                k_half_seg<T, false, 2, kSegS, kSegR><<<grid, 32 * 2 * kSegS, 0, st>>>(
                    dst, src, B.pp, c->d_pipe_ly, c->d_zclass, hq, f.ib, f.cu, c->nx, c->ny, c->nz, c->pz, c->countz,
                    mb, me);
            GW_CUDA(cudaGetLastError());
            return GW_OK;
        }
        cfg = 0;   // lines longer than the segments hold: the tiled kernel
    }
    const size_t sm = half_smem<T>(cfg);
    const CUtensorMap *map = sizeof(T) == 4 ? tile_map(c, src, xlines, cfg) : nullptr;
    const CUtensorMap *qmap = map ? &c->qmaps[xlines ? 0 : 1][cfg] : nullptr;

    switch (cfg) {
        case 1: half_launch<T, 8, 16, kTileNB[1]>(c, st, dst, src, xlines, hq, f, B.pp, sm, mb, me, map, qmap, tm); break;
        case 2: half_launch<T, 8, 8, kTileNB[2]>(c, st, dst, src, xlines, hq, f, B.pp, sm, mb, me, map, qmap, tm); break;
        case 3: half_launch<T, 4, 32, kTileNB[3]>(c, st, dst, src, xlines, hq, f, B.pp, sm, mb, me, map, qmap, tm); break;
        case 4: half_launch<T, 2, 16, kTileNB[4]>(c, st, dst, src, xlines, hq, f, B.pp, sm, mb, me, map, qmap, tm); break;
        case 5: half_launch<T, 8, 32, kTileNB[5]>(c, st, dst, src, xlines, hq, f, B.pp, sm, mb, me, map, qmap, tm); break;
        default: half_launch<T, 4, 16, kTileNB[0]>(c, st, dst, src, xlines, hq, f, B.pp, sm, mb, me, map, qmap, tm); break;
    }
    GW_CUDA(cudaGetLastError());
    return GW_OK;
}

// GW_MIXED_REFINE: the residual correction of the half step that left its
// solution in x (src: the explicit sweep's input; pp: the pipe values).
int launch_refine(gw_ctx *c, float *x, const float *src, int xlines, double h) {
    const int nl = xlines ? c->ny : c->nx;
    dim3 grid((c->nz + 31) / 32, (nl + 3) / 4);
    const GwFactors<float> &f = xlines ? c->c32.fx : c->c32.fy;
    if (!c->refine_f64) {
        // tables allocated by gw_fused_prepare_refine and filled for this
        // step size by gw_fused_refine_tables, both before any capture
        if (!c->f_rq[0] || c->rq_h != h) return gw_fail(GW_ERR_ARG, "refinement tables not prepared for this step size");
        const int dl = xlines ? 0 : 1;
        if (xlines)
            k_half_refine_df<true><<<grid, 128, 0, c->stream>>>(x, c->f_g1, src, c->f_pp, c->d_pipe_lx, c->d_zclass,
                                                                c->f_rq[dl], c->f_rg[dl], c->f_rq[1 - dl], f.a, f.ib,
                                                                f.cu, c->nx, c->ny, c->nz, c->pz, c->countz);
        else
            k_half_refine_df<false><<<grid, 128, 0, c->stream>>>(x, c->f_g1, src, c->f_pp, c->d_pipe_ly, c->d_zclass,
                                                                 c->f_rq[dl], c->f_rg[dl], c->f_rq[1 - dl], f.a, f.ib,
                                                                 f.cu, c->nx, c->ny, c->nz, c->pz, c->countz);
        GW_CUDA(cudaGetLastError());
        return GW_OK;
    }
    if (xlines)
        k_half_refine<true><<<grid, 128, 0, c->stream>>>(x, c->f_g1, src, c->f_pp, c->d_pipe_lx, c->d_zclass,
                                                         c->c64.cxm, c->c64.cxp, c->c64.cym, c->c64.cyp, f.a,
                                                         f.ib, f.cu, c->nx, c->ny, c->nz, c->pz, c->countz, h);
    else
        k_half_refine<false><<<grid, 128, 0, c->stream>>>(x, c->f_g1, src, c->f_pp, c->d_pipe_ly, c->d_zclass,
                                                          c->c64.cym, c->c64.cyp, c->c64.cxm, c->c64.cxp, f.a,
                                                          f.ib, f.cu, c->nx, c->ny, c->nz, c->pz, c->countz, h);
    GW_CUDA(cudaGetLastError());
    return GW_OK;
}

template <typename T, int HW, int HR, int NB>
cudaError_t half_attr() {
    const int sm = (int)(2 * (size_t)HR * (HW + 2) * 32 * sizeof(T));
    cudaError_t e = cudaFuncSetAttribute(k_half_tile<T, true, HW, HR>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
    if (e != cudaSuccess) return e;
    if ((e = cudaFuncSetAttribute(k_half_tile<T, false, HW, HR>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm)))
        return e;
    if constexpr (sizeof(T) == 4) {
        const int st = (int)tma_smem<HW, HR, NB>();
        if ((e = cudaFuncSetAttribute(k_half_tile<T, true, HW, HR, NB, true>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, st)))
            return e;
        // with the staged coefficients of lines up to 512 (4 lines) or 256 rows (8)
        const int stm = (st + 15) / 16 * 16 + (int)tm_cu_smem(HW <= 4 ? 512 : 256, HW);
        if ((e = cudaFuncSetAttribute(k_half_tile<T, true, HW, HR, NB, true, true>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, stm)))
            return e;
        if ((e = cudaFuncSetAttribute(k_half_tile<T, false, HW, HR, NB, true, true>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, stm)))
            return e;
        return cudaFuncSetAttribute(k_half_tile<T, false, HW, HR, NB, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    st);
    }
    return cudaSuccess;
}

template <typename T>
cudaError_t half_attrs() {
    cudaError_t e;
    if constexpr (sizeof(T) == 4) {
        // the split TMEM / shared-memory form takes up to the per-block maximum
        int dev = 0, mx = 0;
        if ((e = cudaGetDevice(&dev)) ||
            (e = cudaDeviceGetAttribute(&mx, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev)) ||
            (e = cudaFuncSetAttribute(k_half_tile<float, true, 4, 16, 2, true, true>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, mx)) ||
            (e = cudaFuncSetAttribute(k_half_tile<float, false, 4, 16, 2, true, true>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, mx)))
            return e;
    }
    if ((e = half_attr<T, 8, 16, kTileNB[1]>()) != cudaSuccess ||
        (e = half_attr<T, 4, 16, kTileNB[0]>()) != cudaSuccess ||
        (e = half_attr<T, 8, 8, kTileNB[2]>()) != cudaSuccess ||
        (e = half_attr<T, 4, 32, kTileNB[3]>()) != cudaSuccess ||
        (e = half_attr<T, 2, 16, kTileNB[4]>()) != cudaSuccess ||
        (e = half_attr<T, 8, 32, kTileNB[5]>()) != cudaSuccess)
        return e;
    return cudaSuccess;
}

// cuTensorMapEncodeTiled, from the driver through the runtime (no link to
// the driver library)
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiledFn encode_tiled() {
    static EncodeTiledFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
    });
    return fn;
}

// The mixed path's half-step tensor maps: per source buffer (f_u, f_temp),
// line direction and tiling, the field as a (levels, j, i) tensor with the
// padded column pitch, box 32 levels x (lines + 2) x rows for the x-lines and
// 32 x rows x (lines + 2) for the y-lines, out-of-range elements read as 0.
// Without the driver's encoder (or a map it rejects) the half step keeps its
// cp.async copies.
void encode_tile_maps(gw_ctx *c) {
    c->tma_ok = false;
    EncodeTiledFn enc = encode_tiled();
    if (!enc || c->precision != GW_PREC_MIXED || c->pz % 4) return;
    const cuuint64_t dims[3] = {(cuuint64_t)c->nz, (cuuint64_t)c->ny, (cuuint64_t)c->nx};
    const cuuint64_t strides[2] = {(cuuint64_t)c->pz * sizeof(float), (cuuint64_t)c->pz * c->ny * sizeof(float)};
    const cuuint32_t es[3] = {1, 1, 1};
    float *bufs[2] = {c->f_u, c->f_temp};
    for (int b = 0; b < 2; ++b)
        for (int d = 0; d < 2; ++d)
            for (int cfg = 0; cfg < 6; ++cfg) {
                const cuuint32_t lines = (cuuint32_t)kTileHW[cfg] + 2, rows = (cuuint32_t)kTileHR[cfg];
                const cuuint32_t box[3] = {32, d == 0 ? lines : rows, d == 0 ? rows : lines};
                if (enc(&c->tmaps[b][d][cfg], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, bufs[b], dims, strides, box, es,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
                    return;
            }
    // the half-step coefficient quads, [z-class][line][row] float4: a tensor of
    // (4 floats x rows, lines, z-classes); box: a chunk's rows x the block's lines
    for (int d = 0; d < 2; ++d) {
        const int nl = d == 0 ? c->ny : c->nx, N = d == 0 ? c->nx : c->ny;
        const cuuint64_t qd[3] = {(cuuint64_t)4 * N, (cuuint64_t)nl, (cuuint64_t)c->n_zclass};
        const cuuint64_t qs[2] = {(cuuint64_t)N * 4 * sizeof(float), (cuuint64_t)nl * N * 4 * sizeof(float)};
        float *tab = d == 0 ? c->c32.hx : c->c32.hy;
        for (int cfg = 0; cfg < 6; ++cfg) {
            const cuuint32_t box[3] = {(cuuint32_t)(4 * kTileHR[cfg]), (cuuint32_t)kTileHW[cfg], 1};
            if (enc(&c->qmaps[d][cfg], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, tab, qd, qs, box, es,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
                return;
        }
    }
    c->tma_ok = true;
}

template <typename T>
int fused_step(gw_ctx *c, double dt, int s) {
    Bufs<T> B = bufs<T>(c);
    int rc;
    // GW_MIXED_REFINE corrects each half step right after its solve, while
    // the pipe values it used are still in pp: the in-line order
    const bool refine = sizeof(T) == 4 && (c->mixed_flags & GW_MIXED_REFINE);
    if (c->overlap && rock2_lpt(c->nz, sizeof(T) == 4) > 0 && !refine) {
        // The pipe passes need only the rows around the pipes.  Order 0:
        // ROCK2 first does the columns of rows jlo-1..jhi+1; then a second
        // stream runs the y pipe pass, the x-lines through the pipes (rows
        // jlo..jhi) and the x pipe pass while the first finishes ROCK2 and
        // the other x-lines; the y-lines wait for both.  Order 1: the second
        // stream starts at once with ROCK2 of the pipe columns and their
        // y-neighbours (all the y pipe pass reads) and the y pipe pass, while
        // the first does ROCK2 of the rest of rows jlo-1..jhi+1 (which the
        // x-lines through the pipes wait for), then of the other rows, then
        // the other x-lines (which wait for the pipe columns' ROCK2).  Both
        // give the same field bitwise; gw_step times them.
        const int *ab = c->d_colorder_ab;
        cudaStream_t s1 = c->stream, s2 = c->stream2;
        if (c->step_order == 1) {
            GW_CUDA(cudaEventRecord(c->ev_a, s1));
            GW_CUDA(cudaStreamWaitEvent(s2, c->ev_a, 0));
            if ((rc = launch_rock2<T>(c, s, ab, c->ncol_p, s2))) return rc;
            GW_CUDA(cudaEventRecord(c->ev_p, s2));
            if ((rc = launch_pipe<T>(c, B.u, GW_DIR_Y, dt / 2, s2))) return rc;
            if ((rc = launch_rock2<T>(c, s, ab + c->ncol_p, c->ncol_a - c->ncol_p, s1))) return rc;
            GW_CUDA(cudaEventRecord(c->ev_q, s1));
            GW_CUDA(cudaStreamWaitEvent(s2, c->ev_q, 0));
            if ((rc = launch_half<T>(c, B.temp, B.u, 1, dt / 2, c->jlo, c->jhi + 1, s2)) ||
                (rc = launch_pipe<T>(c, B.temp, GW_DIR_X, dt / 2, s2)) || (rc = gw_launch_record(c, dt, s2)))
                return rc;
            GW_CUDA(cudaEventRecord(c->ev_px, s2));
            if ((rc = launch_rock2<T>(c, s, ab + c->ncol_a, c->ncol_b, s1))) return rc;
            GW_CUDA(cudaStreamWaitEvent(s1, c->ev_p, 0));
            if ((rc = launch_half<T>(c, B.temp, B.u, 1, dt / 2, 0, c->jlo, s1)) ||
                (rc = launch_half<T>(c, B.temp, B.u, 1, dt / 2, c->jhi + 1, c->ny, s1)))
                return rc;
            GW_CUDA(cudaStreamWaitEvent(s1, c->ev_px, 0));
            return launch_half<T>(c, B.u, B.temp, 0, dt / 2);
        }
        if ((rc = launch_rock2<T>(c, s, ab, c->ncol_a))) return rc;
        GW_CUDA(cudaEventRecord(c->ev_a, s1));
        GW_CUDA(cudaStreamWaitEvent(s2, c->ev_a, 0));
        // the step's record needs only the second pipe pass's outlet (and
        // inlet) values, so it runs here, beside the other x-lines and ROCK2
        if ((rc = launch_pipe<T>(c, B.u, GW_DIR_Y, dt / 2, s2)) ||
            (rc = launch_half<T>(c, B.temp, B.u, 1, dt / 2, c->jlo, c->jhi + 1, s2)) ||
            (rc = launch_pipe<T>(c, B.temp, GW_DIR_X, dt / 2, s2)) || (rc = gw_launch_record(c, dt, s2)))
            return rc;
        GW_CUDA(cudaEventRecord(c->ev_px, s2));
        if ((rc = launch_rock2<T>(c, s, ab + c->ncol_a, c->ncol_b)) ||
            (rc = launch_half<T>(c, B.temp, B.u, 1, dt / 2, 0, c->jlo, s1)) ||
            (rc = launch_half<T>(c, B.temp, B.u, 1, dt / 2, c->jhi + 1, c->ny, s1)))
            return rc;
        GW_CUDA(cudaStreamWaitEvent(s1, c->ev_px, 0));
        return launch_half<T>(c, B.u, B.temp, 0, dt / 2);
    }
    if ((rc = launch_rock2<T>(c, s))) return rc;
    if ((rc = launch_pipe<T>(c, B.u, GW_DIR_Y, dt / 2))) return rc;
    if ((rc = launch_half<T>(c, B.temp, B.u, 1, dt / 2))) return rc;
    if (refine && (rc = launch_refine(c, (float *)B.temp, (const float *)B.u, 1, dt / 2))) return rc;
    if ((rc = launch_pipe<T>(c, B.temp, GW_DIR_X, dt / 2))) return rc;
    if ((rc = launch_half<T>(c, B.u, B.temp, 0, dt / 2))) return rc;
    if (refine && (rc = launch_refine(c, (float *)B.u, (const float *)B.temp, 0, dt / 2))) return rc;
    return gw_launch_record(c, dt);
}

template <typename T>
int time_part(gw_ctx *c, double dt, int s, int part) {
    Bufs<T> B = bufs<T>(c);
    switch (part) {
        case GW_KERNEL_ROCK2: return launch_rock2<T>(c, s);
        case GW_KERNEL_HALF_X: return launch_half<T>(c, B.temp, B.u, 1, dt / 2);
        case GW_KERNEL_HALF_Y: return launch_half<T>(c, B.temp, B.u, 0, dt / 2);
        default: return launch_pipe<T>(c, B.u, GW_DIR_Y, dt / 2);
    }
}

}  // namespace

int gw_fused_supported(const gw_ctx *c) {
    const size_t need = c->precision == GW_PREC_MIXED ? rock2_smem<float>(c->nz) : rock2_smem<double>(c->nz);
    return need <= kColumnSmemMax;
}

// The shared-memory limit is an attribute of the kernel, shared by every
// context: set it to the largest block (256 threads) of that LPT, and size
// the occupancy query by this context's block.
template <typename K>
static cudaError_t occupancy(int *n, K kernel, size_t smem, int nt = 256, size_t smem_max = 0) {
    cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)std::max(smem, smem_max));
    if (e != cudaSuccess) return e;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(n, kernel, nt, smem);
}

int gw_fused_prepare(gw_ctx *c) {
    // shared-memory opt-in for the column kernel.  The limit belongs to the
    // kernel (per device), not to the context, so it is set to the largest
    // block any context may use (kColumnSmemMax, the bound gw_fused_supported
    // checks): a later context with fewer levels must not lower it under an
    // earlier one.
    cudaError_t e;
    if (c->precision == GW_PREC_MIXED)
        e = cudaFuncSetAttribute(k_rock2_col<float, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)kColumnSmemMax);
    else
        e = cudaFuncSetAttribute(k_rock2_col<double, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)kColumnSmemMax);
    if (e != cudaSuccess) return gw_cuda_fail(e, "cudaFuncSetAttribute(k_rock2_col)");
    if ((e = (c->precision == GW_PREC_MIXED ? half_attrs<float>() : half_attrs<double>())) != cudaSuccess)
        return gw_cuda_fail(e, "cudaFuncSetAttribute(k_half_tile)");
    // the column kernels loop over columns: one resident wave of blocks
    int per_sm = 0;
    const bool mix = c->precision == GW_PREC_MIXED;
    // threads per column block: the fewest multiples of 32 that cover nz at
    // LPT levels each (at most 256)
    const int lpt = rock2_lpt(c->nz, mix);
    c->rock2_nt = lpt > 0 ? std::min(256, ((c->nz + lpt - 1) / lpt + 31) / 32 * 32) : 256;
    const int nt = c->rock2_nt;
    switch (lpt) {
        case 2: e = mix ? occupancy(&per_sm, k_rock2_reg<float, true, 2>, reg_smem<float>(2, nt), nt, reg_smem<float>(2)) : occupancy(&per_sm, k_rock2_reg<double, false, 2>, reg_smem<double>(2, nt), nt, reg_smem<double>(2)); break;
        case 4: e = mix ? occupancy(&per_sm, k_rock2_reg<float, true, 4>, reg_smem<float>(4, nt), nt, reg_smem<float>(4)) : occupancy(&per_sm, k_rock2_reg<double, false, 4>, reg_smem<double>(4, nt), nt, reg_smem<double>(4)); break;
        case 5: e = occupancy(&per_sm, k_rock2_reg<float, true, 5>, reg_smem<float>(5, nt), nt, reg_smem<float>(5)); break;   // float only
        case 6: e = occupancy(&per_sm, k_rock2_reg<float, true, 6>, reg_smem<float>(6, nt), nt, reg_smem<float>(6)); break;
        case 7: e = occupancy(&per_sm, k_rock2_reg<float, true, 7>, reg_smem<float>(7, nt), nt, reg_smem<float>(7)); break;
        case 8: e = mix ? occupancy(&per_sm, k_rock2_reg<float, true, 8>, reg_smem<float>(8, nt), nt, reg_smem<float>(8)) : occupancy(&per_sm, k_rock2_reg<double, false, 8>, reg_smem<double>(8, nt), nt, reg_smem<double>(8)); break;
        case 16: e = mix ? occupancy(&per_sm, k_rock2_reg<float, true, 16>, reg_smem<float>(16, nt), nt, reg_smem<float>(16)) : occupancy(&per_sm, k_rock2_reg<double, false, 16>, reg_smem<double>(16, nt), nt, reg_smem<double>(16)); break;
        default:
            e = mix ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_rock2_col<float, true>, 256,
                                                                    rock2_smem<float>(c->nz))
                    : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_rock2_col<double, false>, 256,
                                                                    rock2_smem<double>(c->nz));
    }
    if (e != cudaSuccess) return gw_cuda_fail(e, "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
    int sms = 0;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device);
    if (e != cudaSuccess) return gw_cuda_fail(e, "cudaDeviceGetAttribute");
    c->rock2_grid = (per_sm > 0 ? per_sm : 1) * sms;
    c->sms = sms;
    if (mix) {   // the window kernel, per levels-per-lane instance
        auto occ = [&](auto kern, int L) {
            int n = 0;
            const cudaError_t r = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kern, 32 * kWinWarps, win_smem(L));
            c->rock2w_per_sm[L] = n;
            return r;
        };
        if ((e = occ(k_rock2_win<4, kWinNB, false>, 4)) || (e = occ(k_rock2_win<5, kWinNB, false>, 5)) ||
            (e = occ(k_rock2_win<6, kWinNB, false>, 6)) || (e = occ(k_rock2_win<7, kWinNB, false>, 7)) ||
            (e = occ(k_rock2_win<8, kWinNB, false>, 8)))
            return gw_cuda_fail(e, "cudaOccupancyMaxActiveBlocksPerMultiprocessor(k_rock2_win)");
    }
    // tensor-map tiles for the mixed half steps (GW_HALF_CPASYNC=1 keeps cp.async)
    const char *hc = std::getenv("GW_HALF_CPASYNC");
    if (!(hc && *hc && *hc != '0')) encode_tile_maps(c);
    // forward values of the tensor-map half steps in TMEM (GW_HALF_GLOBAL=1
    // keeps them in global memory)
    const char *hg = std::getenv("GW_HALF_GLOBAL");
    c->half_tmem = !(hg && *hg && *hg != '0');
    // rows beyond 128 in shared memory where that runs more blocks per SM
    // (GW_HALF_TMEM_SPLIT=0 keeps whole lines in TMEM)
    const char *hs = std::getenv("GW_HALF_TMEM_SPLIT");
    c->half_split = !(hs && *hs == '0');
    // on-chip forward values also for half steps of fewer than four rounds of
    // blocks (GW_HALF_TMEM_FORCE=1: the tests' small grids)
    const char *hf = std::getenv("GW_HALF_TMEM_FORCE");
    c->half_tm_force = hf && *hf && *hf != '0';
    // launch order of the overlapped step: chosen by timing (unset), or fixed
    // (GW_STEP_ORDER=0: the pipe rows' ROCK2 columns first; 1: the pipe
    // columns and their y-neighbours first on the second stream)
    const char *so = std::getenv("GW_STEP_ORDER");
    c->step_order_fixed = so && (*so == '0' || *so == '1') ? *so - '0' : -1;
    if (c->step_order_fixed >= 0) c->step_order = c->step_order_fixed;
    if ((e = cudaDeviceGetAttribute(&c->smem_per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, c->device)))
        return gw_cuda_fail(e, "cudaDeviceGetAttribute(shared memory per SM)");
    // default tiling: 4 lines x 16 rows (0); where neither direction's half
    // step of that tiling keeps its forward values on chip (fewer than four
    // rounds of blocks), 8 lines x 8 rows with the values in global memory
    // (9), whose blocks carry 8 lines beside 2 halo lines instead of 4
    // (225 x 225 x 402: 0.227 against 0.237 ms per step)
    if (c->tma_ok && c->half_tmem) {
        int cw;
        size_t sm2;
        if (!half_tm_mode<4, 16>(c, 1, &cw, &sm2) && !half_tm_mode<4, 16>(c, 0, &cw, &sm2))
            c->half_cfg = kGlobalCfg + 2;
    }

    return GW_OK;
}

int gw_fused_set_dt(gw_ctx *c, double dt) {
    const int n = c->nbh * c->countz * 2;
    if (n > 0) {
        k_adv_table<<<grid_for(n, 128), 128, 0, c->stream>>>(
            c->d_advtab, c->d_gz, c->d_bh, c->precision == GW_PREC_MIXED ? c->d_Tref : nullptr, c->nbh,
            c->nz, c->countz, dt / 2);
        GW_CUDA(cudaGetLastError());
    }
    if (c->nbh > 0) {
        k_outlet_levels<<<grid_for(c->nbh, 64), 64, 0, c->stream>>>(c->d_nlev, c->d_gz, c->d_bh, c->nbh, c->nz, dt / 2);
        GW_CUDA(cudaGetLastError());
    }
    GW_CUDA(cudaStreamSynchronize(c->stream));
    return GW_OK;
}

// The first half of a step for the adjoint's forward store: ROCK2 columns on
// u (u <- u*), the pipe pass of the explicit y sweep, the x half step into
// temp (temp <- u1) and the pipe pass of the explicit x sweep (outlet of
// the step's second advection); the swept pipe columns of both passes
// ([column][level], as k_pipe_sweep leaves them) are copied to tpA / tpC.
template <typename T>
int adjoint_store(gw_ctx *c, double dt, int s, T *tpA, T *tpC) {
    Bufs<T> B = bufs<T>(c);
    const size_t tb = (size_t)(c->n_inner + c->n_outer) * c->nz * sizeof(T);
    int rc;
    if ((rc = launch_rock2<T>(c, s)) || (rc = launch_pipe<T>(c, B.u, GW_DIR_Y, dt / 2))) return rc;
    if (tb) GW_CUDA(cudaMemcpyAsync(tpA, B.tp, tb, cudaMemcpyDeviceToDevice, c->stream));
    if ((rc = launch_half<T>(c, B.temp, B.u, 1, dt / 2)) || (rc = launch_pipe<T>(c, B.temp, GW_DIR_X, dt / 2)))
        return rc;
    if (tb) GW_CUDA(cudaMemcpyAsync(tpC, B.tp, tb, cudaMemcpyDeviceToDevice, c->stream));
    return GW_OK;
}

int gw_fused_adjoint_store(gw_ctx *c, double dt, int s, void *tpA, void *tpC) {
    return c->precision == GW_PREC_MIXED ? adjoint_store<float>(c, dt, s, (float *)tpA, (float *)tpC)
                                         : adjoint_store<double>(c, dt, s, (double *)tpA, (double *)tpC);
}

int gw_fused_step(gw_ctx *c, double dt, int s) {
    return c->precision == GW_PREC_MIXED ? fused_step<float>(c, dt, s) : fused_step<double>(c, dt, s);
}

int gw_fused_time_part(gw_ctx *c, double dt, int s, int part) {
    return c->precision == GW_PREC_MIXED ? time_part<float>(c, dt, s, part)
                                         : time_part<double>(c, dt, s, part);
}

int gw_fused_check_finite(gw_ctx *c) {
    // every slot of the field, padding levels (always 0) included
    size_t n = (size_t)c->nx * c->ny * c->pz;
    GW_CUDA(cudaMemsetAsync(c->d_flag, 0, sizeof(int), c->stream));
    if (c->precision == GW_PREC_MIXED)
        k_finite<float><<<1216, 256, 0, c->stream>>>(c->f_u, n, c->d_flag);
    else
        k_finite<double><<<1216, 256, 0, c->stream>>>(c->d_u, n, c->d_flag);
    GW_CUDA(cudaGetLastError());
    return GW_OK;
}

int gw_fused_set_theta(gw_ctx *c, const double *T_host) {
    const size_t n = (size_t)c->nx * c->ny * c->nz;
    double *stage = reinterpret_cast<double *>(c->f_temp);   // f_temp and f_g1: 8 n bytes
    GW_CUDA(cudaMemcpyAsync(stage, T_host, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    k_to_theta<<<1216, 256, 0, c->stream>>>(c->f_u, stage, c->d_Tref, n, c->nz, c->pz);
    GW_CUDA(cudaGetLastError());
    GW_CUDA(cudaStreamSynchronize(c->stream));
    return GW_OK;
}

int gw_fused_get_theta(gw_ctx *c, double *T_host) {
    const size_t n = (size_t)c->nx * c->ny * c->nz;
    double *stage = reinterpret_cast<double *>(c->f_temp);
    k_from_theta<<<1216, 256, 0, c->stream>>>(stage, c->f_u, c->d_Tref, n, c->nz, c->pz);
    GW_CUDA(cudaGetLastError());
    GW_CUDA(cudaMemcpyAsync(T_host, stage, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    GW_CUDA(cudaStreamSynchronize(c->stream));
    return GW_OK;
}

int gw_fused_prepare_rock2_f64(gw_ctx *c) {
    if (c->precision != GW_PREC_MIXED || !c->fused)
        return gw_fail(GW_ERR_ARG, "GW_MIXED_ROCK2_F64 needs a fused GW_PREC_MIXED context");
    const int lpt = rock2_lpt(c->nz, false);
    if (lpt <= 0) return gw_fail(GW_ERR_UNSUPPORTED, "GW_MIXED_ROCK2_F64 supports nz <= 4096");
    const int nt = std::min(256, ((c->nz + lpt - 1) / lpt + 31) / 32 * 32);
    int per_sm = 0;
    cudaError_t e;
    switch (lpt) {
        case 2: e = occupancy(&per_sm, k_rock2_reg<float, true, 2, double>, reg_smem<float>(2, nt), nt, reg_smem<float>(2)); break;
        case 4: e = occupancy(&per_sm, k_rock2_reg<float, true, 4, double>, reg_smem<float>(4, nt), nt, reg_smem<float>(4)); break;
        case 8: e = occupancy(&per_sm, k_rock2_reg<float, true, 8, double>, reg_smem<float>(8, nt), nt, reg_smem<float>(8)); break;
        default: e = occupancy(&per_sm, k_rock2_reg<float, true, 16, double>, reg_smem<float>(16, nt), nt, reg_smem<float>(16)); break;
    }
    if (e != cudaSuccess) return gw_cuda_fail(e, "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
    int sms = 0;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device)) != cudaSuccess)
        return gw_cuda_fail(e, "cudaDeviceGetAttribute");
    c->rock2_nt64 = nt;
    c->rock2_grid64 = (per_sm > 0 ? per_sm : 1) * sms;
    return GW_OK;
}

int gw_fused_prepare_refine(gw_ctx *c) {
    if (c->precision != GW_PREC_MIXED || !c->fused)
        return gw_fail(GW_ERR_ARG, "GW_MIXED_REFINE needs a fused GW_PREC_MIXED context");
    if (c->refine_f64 || c->f_rq[0]) return GW_OK;
    const size_t n = (size_t)c->n_zclass * c->nx * c->ny;
    for (int d = 0; d < 2; ++d) {
        float *a = nullptr, *g = nullptr;
        int rc;
        if ((rc = gw_dalloc_f(c, &a, 4 * n)) || (rc = gw_dalloc_f(c, &g, 2 * n))) return rc;
        c->f_rq[d] = reinterpret_cast<float4 *>(a);
        c->f_rg[d] = reinterpret_cast<float2 *>(g);
    }
    c->rq_h = -1.0;
    return GW_OK;
}

// the double-float refinement tables for half-step size h (no-op when
// GW_MIXED_REFINE is off, runs in double, or the tables hold h already)
int gw_fused_refine_tables(gw_ctx *c, double h) {
    if (!(c->mixed_flags & GW_MIXED_REFINE) || c->refine_f64 || c->rq_h == h) return GW_OK;
    if (!c->f_rq[0]) return gw_fail(GW_ERR_ARG, "refinement tables not allocated");
    const size_t n = (size_t)c->n_zclass * c->nx * c->ny;
    k_refine_tables<<<grid_for((long long)n, 256), 256, 0, c->stream>>>(c->f_rq[0], c->f_rg[0], c->c64.cxm,
                                                                        c->c64.cxp, h, n);
    k_refine_tables<<<grid_for((long long)n, 256), 256, 0, c->stream>>>(c->f_rq[1], c->f_rg[1], c->c64.cym,
                                                                        c->c64.cyp, h, n);
    GW_CUDA(cudaGetLastError());
    c->rq_h = h;
    return GW_OK;
}

// GW_ERR_CUDA if a kernel's bounded wait ran out since the last check
int gw_fused_status(gw_ctx *c) {
    if (!c->d_err) return GW_OK;
    int flag = 0;
    GW_CUDA(cudaMemcpy(&flag, c->d_err, sizeof(int), cudaMemcpyDeviceToHost));
    if (!flag) return GW_OK;
    GW_CUDA(cudaMemset(c->d_err, 0, sizeof(int)));
    return gw_fail(GW_ERR_CUDA, "a half-step tile did not arrive within its wait limit");
}

// debug build: point this translation unit's checks at the allocation registry
GW_DEBUG_BIND(gw_debug_bind_fused)
