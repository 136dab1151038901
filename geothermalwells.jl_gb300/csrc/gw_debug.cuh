// gw_debug.cuh -- device bounds checks of the debug build (-DGW_DEBUG).
//
// The fused step's kernels run their global and shared-memory accesses
// through these checks in the debug build, and through nothing in the
// normal build.  Global addresses are looked up in a registry of every
// device allocation the contexts hold (registered by gw_create's allocator);
// dynamic shared memory is checked against the block's %dynamic_smem_size.
// A failed check does not trap: it records the first failing site and
// address in the registry, the access is skipped (a load yields 0), and the
// host entry point that launched the work returns GW_ERR_ARG with the site.
// It stands in for a memory checker on hardware where none may run.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>

#define GW_DBG_MAX_ALLOC 8192

struct GwDbgRegistry {
    unsigned int count;        // registered allocations
    unsigned int fail;         // 0, or 1 + the site of the first failed check
    unsigned long long addr;   // the address (global) or offset (shared) that failed
    unsigned long long base[GW_DBG_MAX_ALLOC], end[GW_DBG_MAX_ALLOC];
};

#ifdef GW_DEBUG
// one copy per translation unit, pointed at the one registry by gw_debug_bind_*
static __constant__ GwDbgRegistry *c_gw_dbg;

__device__ __forceinline__ void gw_dbg_record(unsigned site, unsigned long long a) {
    GwDbgRegistry *r = c_gw_dbg;
    if (atomicCAS(&r->fail, 0u, site + 1u) == 0u) r->addr = a;
}

__device__ __forceinline__ bool gw_dbg_global(const void *p, size_t bytes, unsigned site) {
    const GwDbgRegistry *r = c_gw_dbg;
    if (!r) return true;
    const unsigned long long a = (unsigned long long)p, e = a + bytes;
    for (unsigned i = 0; i < r->count; ++i)
        if (a >= r->base[i] && e <= r->end[i]) return true;
    gw_dbg_record(site, a);
    return false;
}

// p within [base, base + the block's dynamic shared memory)
__device__ __forceinline__ bool gw_dbg_dyn(const void *p, size_t bytes, const void *base, unsigned site) {
    unsigned dyn;
    asm volatile("mov.u32 %0, %%dynamic_smem_size;" : "=r"(dyn));
    const char *cp = (const char *)p, *cb = (const char *)base;
    if (cp >= cb && (size_t)(cp - cb) + bytes <= dyn) return true;
    if (c_gw_dbg) gw_dbg_record(site, (unsigned long long)(cp - cb));
    return false;
}

// an index into a fixed-size array
__device__ __forceinline__ bool gw_dbg_idx(long long i, long long n, unsigned site) {
    if (i >= 0 && i < n) return true;
    if (c_gw_dbg) gw_dbg_record(site, (unsigned long long)i);
    return false;
}
#define GW_OK_G(p, site) gw_dbg_global((p), sizeof(*(p)), (site))
#define GW_OK_GB(p, bytes, site) gw_dbg_global((p), (bytes), (site))
#define GW_OK_D(p, base, site) gw_dbg_dyn((p), sizeof(*(p)), (base), (site))
#define GW_OK_I(i, n, site) gw_dbg_idx((long long)(i), (long long)(n), (site))
#define GW_DEBUG_BIND(name)                                                           \
    int name(GwDbgRegistry *r) {                                                      \
        return cudaMemcpyToSymbol(c_gw_dbg, &r, sizeof(r)) == cudaSuccess ? 0 : 1;     \
    }
#else
#define GW_OK_G(p, site) true
#define GW_OK_GB(p, bytes, site) true
#define GW_OK_D(p, base, site) true
#define GW_OK_I(i, n, site) true
#define GW_DEBUG_BIND(name) \
    int name(GwDbgRegistry *) { return 0; }
#endif
