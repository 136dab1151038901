// gw_noalloc.cu -- advection that needs no device memory from its caller or
// from the allocator: gw_advection_noalloc.
//
// gw_advection keeps its scratch (the advected pipe columns, the per-level
// annulus means, the outlet means) in buffers gw_create allocated for the
// context.  This variant keeps the small scratch it needs -- outlet means and
// per-level annulus means -- in one file-scope device array, and processes
// each pipe column inside one thread block's shared memory, so it needs no
// column-sized buffer at all.  The array exists once per device that loads
// the library and is held until the process exits.
#include <cuda_runtime.h>

#include <mutex>

#include "gw_internal.h"

// Largest nbh * (nz + 1) the array holds: 65536 doubles (512 KiB).
#define GW_NOALLOC_SCRATCH_DOUBLES 65536
// Largest column (levels <= max h) a block holds in shared memory: 96 KiB.
#define GW_NOALLOC_MAX_COUNTZ 12288
#define GW_NOALLOC_MAX_DEVICES 64

static __device__ __align__(256) double g_noalloc_scratch[GW_NOALLOC_SCRATCH_DOUBLES];

namespace {

// Device address of g_noalloc_scratch per device, filled on the first call
// made with that device current.
double *g_scratch_addr[GW_NOALLOC_MAX_DEVICES] = {nullptr};
std::mutex g_setup_mutex;

// Outlet mean of one borehole (src/solver.jl:267-282, 257) into out[b].
__global__ void __launch_bounds__(256) na_outlet(double *__restrict__ out,
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
        int lo = 0, hi = nz;
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
    if (threadIdx.x == 0) out[b] = s_red[0] / (double)tot;
}

// Annulus mean per borehole and level (src/solver.jl:322-335), list order.
__global__ void __launch_bounds__(128) na_annulus_mean(double *__restrict__ mean,
                                                       const double *__restrict__ phi,
                                                       const int *__restrict__ pi,
                                                       const int *__restrict__ pj,
                                                       const GwBhDev *__restrict__ bh, int ny,
                                                       int nz) {
    const int b = blockIdx.y;
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nz) return;
    const GwBhDev B = bh[b];
    double s = 0.0;
    for (int q = B.outer_begin; q < B.outer_begin + B.outer_count; ++q)
        s += phi[k + (long long)nz * (pj[q] + (long long)ny * pi[q])];
    mean[(size_t)b * nz + k] = s / (double)B.outer_count;
}

__device__ __forceinline__ void na_interp(const double *__restrict__ g, int n, double dep, int &il,
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
    alpha = __ddiv_rn(__dsub_rn(dep, g[il]), __dsub_rn(g[ir], g[il]));
}

// kernel_advection! + kernel_copy_advection! (src/solver.jl:285-396) for one
// pipe column per block: the column's old values are staged in shared
// memory, new values are written straight back into phi.  Departure levels
// beyond the staged column (possible only when h is not a grid point) are
// read from phi, which no other block writes (each block owns its column).
__global__ void __launch_bounds__(256) na_advect_column(
    double *__restrict__ phi, const double *__restrict__ gz, const int *__restrict__ pi,
    const int *__restrict__ pj, const int *__restrict__ pb, const GwBhDev *__restrict__ bh,
    const double *__restrict__ ann_mean, const double *__restrict__ outlet, int n_inner, int ny,
    int nz, int countz, double dt, int inlet_kind, double inlet_param) {
    extern __shared__ double s_col[];
    const int q = blockIdx.x;
    const int b = pb[q];
    const GwBhDev B = bh[b];
    double *col = phi + (long long)nz * (pj[q] + (long long)ny * pi[q]);
    for (int k = threadIdx.x; k < countz; k += blockDim.x) s_col[k] = col[k];
    __syncthreads();
    auto old = [&](int k) { return k < countz ? s_col[k] : col[k]; };
    for (int k = threadIdx.x; k < countz; k += blockDim.x) {
        const double z = gz[k];
        double v;
        if (z > B.h) {
            v = s_col[k];
        } else if (q < n_inner) {
            double zd = __fma_rn(B.v_inner, dt, z);
            if (zd > B.h) {
                double dt1 = __ddiv_rn(__dsub_rn(B.h, z), B.v_inner);
                double dt2 = __dsub_rn(dt, dt1);
                double zd2 = __fma_rn(-B.v_outer, dt2, B.h);
                int il, ir; double a;
                na_interp(gz, nz, zd2, il, ir, a);
                const double *m = ann_mean + (size_t)b * nz;
                v = __fma_rn(a, m[ir], __dmul_rn(__dsub_rn(1.0, a), m[il]));
            } else {
                int il, ir; double a;
                na_interp(gz, nz, zd, il, ir, a);
                v = __fma_rn(a, old(ir), __dmul_rn(__dsub_rn(1.0, a), old(il)));
            }
        } else {
            double zd = __fma_rn(-B.v_outer, dt, z);
            if (zd <= 0.0) {
                v = inlet_kind == GW_INLET_CONSTANT ? inlet_param : outlet[b] - inlet_param;
            } else {
                int il, ir; double a;
                na_interp(gz, nz, zd, il, ir, a);
                v = __fma_rn(a, old(ir), __dmul_rn(__dsub_rn(1.0, a), old(il)));
            }
        }
        // reads come from the staged copy (or levels >= countz, never written),
        // so writing the new value straight into phi cannot race
        col[k] = v;
    }
}

// Once per device, with that device current: look up the device address of
// the file-scope scratch array and raise the kernel's shared-memory limit.
int noalloc_setup(int dev, double **addr) {
    if (dev < 0 || dev >= GW_NOALLOC_MAX_DEVICES)
        return gw_fail(GW_ERR_ARG, "gw_advection_noalloc supports device ordinals below 64");
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_addr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return gw_cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
        e = cudaFuncSetAttribute(na_advect_column, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 GW_NOALLOC_MAX_COUNTZ * (int)sizeof(double));
        if (e != cudaSuccess) return gw_cuda_fail(e, "cudaFuncSetAttribute(na_advect_column)");
        g_scratch_addr[dev] = (double *)p;
    }
    *addr = g_scratch_addr[dev];
    return GW_OK;
}

}  // namespace

extern "C" int gw_advection_noalloc(gw_ctx *c, double *phi, double dt, double t,
                                    double *T_outlet_dev) {
    (void)t;
    if (!c || !phi || !T_outlet_dev) return gw_fail(GW_ERR_ARG, "NULL argument");
    const long long need = (long long)c->nbh * ((long long)c->nz + 1);
    if (need > GW_NOALLOC_SCRATCH_DOUBLES)
        return gw_fail(GW_ERR_ARG, "gw_advection_noalloc: n_boreholes * (nz + 1) exceeds the "
                                   "65536-double scratch limit");
    if (c->countz > GW_NOALLOC_MAX_COUNTZ)
        return gw_fail(GW_ERR_ARG, "gw_advection_noalloc: more than 12288 levels above the "
                                   "deepest borehole bottom");
    if (c->inlet_kind == GW_INLET_EXPRESSION)
        return gw_fail(GW_ERR_UNSUPPORTED, "gw_advection_noalloc: inlet programs run in gw_advection");
    if (c->modular_reason & GW_MODULAR_SHARED_COLUMN)   // one block per list entry writes its column
        return gw_fail(GW_ERR_UNSUPPORTED, "gw_advection_noalloc: a pipe column belongs to two boreholes");
    cudaError_t e = cudaSetDevice(c->device);
    if (e != cudaSuccess) return gw_cuda_fail(e, "cudaSetDevice");
    double *scratch = nullptr;
    int rc = noalloc_setup(c->device, &scratch);
    if (rc) return rc;
    double *outlet = scratch;              // [nbh]
    double *ann = scratch + c->nbh;        // [nbh][nz]
    na_outlet<<<c->nbh, 256, 0, c->stream>>>(outlet, phi, c->d_gz, c->d_pipe_i, c->d_pipe_j,
                                             c->d_bh, c->ny, c->nz, dt);
    if ((e = cudaGetLastError()) != cudaSuccess) return gw_cuda_fail(e, "na_outlet");
    const int ncol = c->n_inner + c->n_outer;
    if (ncol > 0 && c->countz > 0) {
        dim3 g((c->nz + 127) / 128, c->nbh);
        na_annulus_mean<<<g, 128, 0, c->stream>>>(ann, phi, c->d_pipe_i, c->d_pipe_j, c->d_bh,
                                                   c->ny, c->nz);
        if ((e = cudaGetLastError()) != cudaSuccess) return gw_cuda_fail(e, "na_annulus_mean");
        na_advect_column<<<ncol, 256, (size_t)c->countz * sizeof(double), c->stream>>>(
            phi, c->d_gz, c->d_pipe_i, c->d_pipe_j, c->d_pipe_b, c->d_bh, ann, outlet, c->n_inner,
            c->ny, c->nz, c->countz, dt, c->inlet_kind == GW_INLET_SCHEDULE ? GW_INLET_CONSTANT : c->inlet_kind,
            c->inlet_kind == GW_INLET_SCHEDULE ? gw_schedule_at(c, t) : c->inlet_param);
        if ((e = cudaGetLastError()) != cudaSuccess) return gw_cuda_fail(e, "na_advect_column");
    }
    e = cudaMemcpyAsync(T_outlet_dev, outlet, c->nbh * sizeof(double), cudaMemcpyDeviceToDevice,
                        c->stream);
    if (e != cudaSuccess) return gw_cuda_fail(e, "cudaMemcpyAsync(T_outlet)");
    e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return gw_cuda_fail(e, "cudaStreamSynchronize");
    return GW_OK;
}
