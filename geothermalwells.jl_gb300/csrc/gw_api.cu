// gw_api.cu -- the extern "C" entry points declared in include/gw_gb300.h.
#include <cuda_runtime.h>

#include <cstdlib>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "gw_fused.h"
#include "gw_internal.h"
#include "gw_debug.cuh"

namespace {
thread_local std::string g_err;

template <typename T>
int dalloc(gw_ctx *c, T **p, size_t n) {
    if (n == 0) n = 1;
    cudaError_t e = cudaMalloc((void **)p, n * sizeof(T));
    if (e != cudaSuccess) return gw_cuda_fail(e, "cudaMalloc");
    c->allocations.push_back((void *)*p);
    c->device_bytes += (long long)(n * sizeof(T));
    gw_debug_register(c->device, *p, n * sizeof(T));
    return GW_OK;
}

template <typename T>
int upload(gw_ctx *c, T **p, const std::vector<T> &v) {
    int rc = dalloc(c, p, v.size());
    if (rc) return rc;
    if (!v.empty()) GW_CUDA(cudaMemcpy(*p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
    return GW_OK;
}

template <typename T>
int copy_to(T *dst, const std::vector<T> &v) {
    if (!v.empty()) {
        GW_CUDA(cudaMemcpy(dst, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
        // a pageable copy may return before its DMA lands; the context's
        // stream is non-blocking, so wait for it here
        GW_CUDA(cudaStreamSynchronize(0));
    }
    return GW_OK;
}

std::vector<float> to_float(const std::vector<double> &v) {
    std::vector<float> f(v.size());
    for (size_t i = 0; i < v.size(); ++i) f[i] = (float)v[i];
    return f;
}

size_t ncell(const gw_ctx *c) { return (size_t)c->nx * c->ny * c->nz; }

int set_device(gw_ctx *c) {
    GW_CUDA(cudaSetDevice(c->device));
    return GW_OK;
}

int sync(gw_ctx *c) {
    GW_CUDA(cudaStreamSynchronize(c->stream));
    return GW_OK;
}

bool mixed(const gw_ctx *c) { return c->precision == GW_PREC_MIXED; }

// One ROCK2 step on u with the modular kernels (buffers {u, g1, spare}).
// Each stage reads its stencil input and, pointwise, the stage before it, so
// the output may overwrite the older stage; the last stage lands in u.
int rock2_step(gw_ctx *c, double *u, double *g1, double *spare, double dt, int s) {
    const double *mu, *nu, *kappa;
    double sigma, tau;
    gw_rock2_coefs(s, &mu, &nu, &kappa, &sigma, &tau);
    double *pool[3] = {u, g1, spare};
    int cur = 0, prev = -1, rc;
    auto pick = [&](int a, int b) {
        for (int q = 0; q < 3; ++q)
            if (q != a && q != b) return q;
        return -1;
    };
    for (int j = 1; j <= s - 2; ++j) {
        int out = prev >= 0 ? prev : pick(cur, 0);
        double kap = j == 1 ? 0.0 : kappa[j - 1];
        rc = gw_launch_zstage(c, pool[out], pool[cur], prev >= 0 ? pool[prev] : nullptr,
                              dt * mu[j - 1], kap, 0);
        if (rc) return rc;
        prev = cur;
        cur = out;
    }
    int gp = cur;
    int gq = pick(gp, 0);
    rc = gw_launch_zstage(c, pool[gq], pool[gp], nullptr, dt * sigma, 0.0, 0);
    if (rc) return rc;
    return gw_launch_zstage(c, pool[0], pool[gq], pool[gp], dt * tau / sigma,
                            1.0 - tau / (sigma * sigma), 0);
}

// ADI_and_ADV_callback! (src/solver.jl:432-464) with the modular kernels.
// The Thomas factors for h = dt/2 must be current (gw_ensure_factors).
// t is the callback's time (the step's end): the advections see t and
// t + dt/2 (src/solver.jl:447,458).
int adi_adv(gw_ctx *c, double *u, double *temp, double dt, double t = 0.0) {
    int rc;
    if ((rc = gw_launch_explicit(c, temp, u, dt / 2, GW_DIR_Y))) return rc;
    if ((rc = gw_launch_advection(c, temp, dt / 2, t))) return rc;
    if ((rc = gw_launch_thomas(c, u, temp, GW_DIR_X))) return rc;
    if ((rc = gw_launch_explicit(c, temp, u, dt / 2, GW_DIR_X))) return rc;
    if ((rc = gw_launch_advection(c, temp, dt / 2, t + dt / 2))) return rc;
    return gw_launch_thomas(c, u, temp, GW_DIR_Y);
}

int check_field_ptrs(const void *a, const void *b) {
    if (!a || !b) return gw_fail(GW_ERR_ARG, "field pointer is NULL");
    return GW_OK;
}

// ROCK2 stage table for the fused column kernel (layout in gw_fused.cu)
int upload_stages(gw_ctx *c, double dt, int s) {
    const double *mu, *nu, *kappa;
    double sigma, tau;
    gw_rock2_coefs(s, &mu, &nu, &kappa, &sigma, &tau);
    std::vector<double> sc;
    for (int j = 0; j < s - 2; ++j) {
        sc.push_back(dt * mu[j]);
        sc.push_back(j == 0 ? 0.0 : kappa[j]);
    }
    sc.push_back(dt * sigma);
    sc.push_back(dt * tau / sigma);
    sc.push_back(1.0 - tau / (sigma * sigma));
    if ((int)sc.size() > GW_STAGE_TABLE) return gw_fail(GW_ERR_ARG, "stage table too long");
    GW_CUDA(cudaMemcpy(c->d_stage, sc.data(), sc.size() * sizeof(double), cudaMemcpyHostToDevice));
    std::vector<float> sf(sc.begin(), sc.end());
    GW_CUDA(cudaMemcpy(c->f_stage, sf.data(), sf.size() * sizeof(float), cudaMemcpyHostToDevice));
    return GW_OK;
}

// Mixed path: T_ref = the field's first column (i = j = 0), and the source
// A_z T_ref per column profile.
int set_reference_profile(gw_ctx *c, const double *T) {
    const int nz = c->nz;
    c->Tref.assign(T, T + nz);
    std::vector<double> f((size_t)c->n_profiles * nz);
    for (int p = 0; p < c->n_profiles; ++p)
        for (int k = 0; k < nz; ++k) {
            double tc = c->Tref[k];
            double tp = k < nz - 1 ? c->Tref[k + 1] : tc;
            double tm = k > 0 ? c->Tref[k - 1] : tc;
            size_t q = (size_t)p * nz + k;
            f[q] = c->h_czp[q] * (tp - tc) - c->h_czm[q] * (tc - tm);
        }
    int rc;
    if ((rc = copy_to(c->d_Tref, c->Tref)) || (rc = copy_to(c->d_fref64, f))) return rc;
    return copy_to(c->f_fref, to_float(f));
}
}  // namespace

// a device float array owned by the context (freed by gw_destroy; counted in
// device_bytes; registered with the debug build's bounds checks)
int gw_dalloc_f(gw_ctx *c, float **p, size_t n) { return dalloc(c, p, n); }

int gw_fail(int code, const std::string &msg) {
    g_err = msg;
    return code;
}

int gw_cuda_fail(cudaError_t e, const char *what) {
    g_err = std::string(what) + ": " + cudaGetErrorString(e);
    return GW_ERR_CUDA;
}

// the instrumented translation units' registry binders (gw_debug.cuh)
int gw_debug_bind_fused(GwDbgRegistry *r);

#ifdef GW_DEBUG
// The allocation registry of the debug build, one per device: a host list
// mirrored into a device GwDbgRegistry whose address every instrumented
// translation unit holds in constant memory.
namespace {
std::mutex g_dbg_mutex;
struct DbgDevice {
    GwDbgRegistry *reg = nullptr;
    std::vector<std::pair<unsigned long long, unsigned long long>> ranges;
};
DbgDevice g_dbg[64];

void dbg_sync(int dev) {   // with g_dbg_mutex held and dev current
    DbgDevice &D = g_dbg[dev];
    if (!D.reg) {
        if (cudaMalloc((void **)&D.reg, sizeof(GwDbgRegistry)) != cudaSuccess) { D.reg = nullptr; return; }
        cudaMemset(D.reg, 0, sizeof(GwDbgRegistry));
        gw_debug_bind_fused(D.reg);
    }
    const unsigned n = (unsigned)std::min<size_t>(D.ranges.size(), GW_DBG_MAX_ALLOC);
    std::vector<unsigned long long> b(n), e(n);
    for (unsigned i = 0; i < n; ++i) { b[i] = D.ranges[i].first; e[i] = D.ranges[i].second; }
    cudaDeviceSynchronize();   // no instrumented kernel reads the registry meanwhile
    cudaMemcpy(&D.reg->count, &n, sizeof(n), cudaMemcpyHostToDevice);
    if (n) {
        cudaMemcpy(D.reg->base, b.data(), n * sizeof(unsigned long long), cudaMemcpyHostToDevice);
        cudaMemcpy(D.reg->end, e.data(), n * sizeof(unsigned long long), cudaMemcpyHostToDevice);
    }
}
}  // namespace

void gw_debug_register(int dev, const void *p, size_t bytes) {
    if (dev < 0 || dev >= 64 || !p) return;
    std::lock_guard<std::mutex> lock(g_dbg_mutex);
    const unsigned long long a = (unsigned long long)p;
    g_dbg[dev].ranges.emplace_back(a, a + bytes);
    dbg_sync(dev);
}

void gw_debug_unregister(int dev, const void *p) {
    if (dev < 0 || dev >= 64 || !p) return;
    std::lock_guard<std::mutex> lock(g_dbg_mutex);
    auto &r = g_dbg[dev].ranges;
    for (size_t i = 0; i < r.size(); ++i)
        if (r[i].first == (unsigned long long)p) { r.erase(r.begin() + (long)i); break; }
    dbg_sync(dev);
}

int gw_debug_status(int dev) {
    if (dev < 0 || dev >= 64 || !g_dbg[dev].reg) return GW_OK;
    unsigned fail = 0;
    unsigned long long addr = 0;
    GwDbgRegistry *r = g_dbg[dev].reg;
    GW_CUDA(cudaDeviceSynchronize());
    GW_CUDA(cudaMemcpy(&fail, &r->fail, sizeof(fail), cudaMemcpyDeviceToHost));
    GW_CUDA(cudaMemcpy(&addr, &r->addr, sizeof(addr), cudaMemcpyDeviceToHost));
    if (!fail) return GW_OK;
    const unsigned zero = 0;
    GW_CUDA(cudaMemcpy(&r->fail, &zero, sizeof(unsigned), cudaMemcpyHostToDevice));
    char msg[160];
    std::snprintf(msg, sizeof msg, "debug bounds check failed: site %u, address/offset 0x%llx", fail - 1, addr);
    return gw_fail(GW_ERR_ARG, msg);
}
#else
void gw_debug_register(int, const void *, size_t) {}
void gw_debug_unregister(int, const void *) {}
int gw_debug_status(int) { return GW_OK; }
#endif

// Recompute the Thomas factors of (I - h A_x) and (I - h A_y) when h changes
// (in double; the mixed path gets them rounded to float).
// Start time and step size of the steps about to run, read on the device by
// the schedule inlet (with the step counter).
int gw_set_step_time(gw_ctx *c, double t0, double dt) {
    const double v[2] = {t0, dt};
    GW_CUDA(cudaMemcpyAsync(c->d_time, v, sizeof(v), cudaMemcpyHostToDevice, c->stream));
    return GW_OK;
}

double gw_schedule_at(const gw_ctx *c, double t) {
    const std::vector<double> &ts = c->sched_t, &vs = c->sched_T;
    const int n = (int)ts.size();
    if (n == 0) return 0.0;
    if (t <= ts[0]) return vs[0];
    if (t >= ts[n - 1]) return vs[n - 1];
    int lo = 0, hi = n - 1;   // ts[lo] <= t < ts[hi]
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (ts[mid] <= t) lo = mid; else hi = mid;
    }
    const double a = (t - ts[lo]) / (ts[hi] - ts[lo]);
    return std::fma(a, vs[hi] - vs[lo], vs[lo]);
}

int gw_ensure_factors(gw_ctx *c, double h) {
    if (h == c->factors_h) return GW_OK;
    if (!c->host_setup) {
        GW_CUDA(cudaStreamSynchronize(c->stream));
        int rc = gw_factors_device(c, h);
        if (rc) return rc;
        c->factors_h = h;
        return GW_OK;
    }
    std::vector<double> cxm, cxp, cym, cyp, czm, czp;
    gw_build_coefs(c, cxm, cxp, cym, cyp, czm, czp);
    std::vector<double> a, ib, cu;
    GW_CUDA(cudaStreamSynchronize(c->stream));
    int rc;
    std::vector<double> h4;
    for (int dir = GW_DIR_X; dir <= GW_DIR_Y; ++dir) {
        gw_build_factors(c, h, dir, dir == GW_DIR_X ? cxm : cym, dir == GW_DIR_X ? cxp : cyp, a, ib, cu);
        // x-lines fold the explicit y sweep, y-lines the explicit x sweep
        gw_build_half_table(c, h, dir, dir == GW_DIR_X ? cym : cxm, dir == GW_DIR_X ? cyp : cxp, a, ib, h4);
        GwFactors<double> &f = dir == GW_DIR_X ? c->c64.fx : c->c64.fy;
        if ((rc = copy_to(f.a, a)) || (rc = copy_to(f.ib, ib)) || (rc = copy_to(f.cu, cu))) return rc;
        if (mixed(c)) {
            GwFactors<float> &g = dir == GW_DIR_X ? c->c32.fx : c->c32.fy;
            if ((rc = copy_to(g.a, to_float(a))) || (rc = copy_to(g.ib, to_float(ib))) ||
                (rc = copy_to(g.cu, to_float(cu))) ||
                (rc = copy_to(dir == GW_DIR_X ? c->c32.hx : c->c32.hy, to_float(h4))))
                return rc;
        } else if ((rc = copy_to(dir == GW_DIR_X ? c->c64.hx : c->c64.hy, h4))) {
            return rc;
        }
    }
    c->factors_h = h;
    return GW_OK;
}

// Everything a step of size dt with s stages needs before its graph runs:
// the outlet-series capacity, the step counter, the Thomas factors, and for
// the fused step the stage and advection tables.
int gw_prepare_step(gw_ctx *c, double dt, int s, int nsteps) {
    int rc;
    if (nsteps > c->series_cap) {
        GW_CUDA(cudaStreamSynchronize(c->stream));
        if (c->d_series) {
            cudaFree(c->d_series);
            for (auto &p : c->allocations) if (p == c->d_series) p = nullptr;
            c->d_series = nullptr;
        }
        if ((rc = dalloc(c, &c->d_series, (size_t)nsteps * c->nbh))) return rc;
        c->series_cap = nsteps;
        ++c->series_gen;
    }
    GW_CUDA(cudaMemsetAsync(c->d_step_counter, 0, sizeof(int), c->stream));
    c->last_nsteps = nsteps;
    if (nsteps == 0) return GW_OK;
    if ((rc = gw_ensure_factors(c, dt / 2))) return rc;
    if (c->fused && mixed(c) && (rc = gw_fused_refine_tables(c, dt / 2))) return rc;
    if (c->fused && (c->tables_dt != dt || c->tables_s != s)) {
        if ((rc = upload_stages(c, dt, s)) || (rc = gw_fused_set_dt(c, dt))) return rc;
        c->tables_dt = dt;
        c->tables_s = s;
    }
    return GW_OK;
}

extern "C" {

const char *gw_last_error(void) { return g_err.c_str(); }

const char *gw_version(void) { return "gw_gb300 0.2 (sm_103a)"; }

int gw_create(const gw_desc *desc, gw_ctx **out) {
    if (!out) return gw_fail(GW_ERR_ARG, "out is NULL");
    *out = nullptr;
    gw_ctx *c = new gw_ctx();
    // tables on the GPU unless GW_HOST_SETUP is set (the host builders give
    // the same values bitwise; tests compare the two paths)
    const char *hs = std::getenv("GW_HOST_SETUP");
    c->host_setup = hs && *hs && *hs != '0';
    // the mixed step's ROCK2 on the block kernel instead of the window kernel
    // (the two give the same field bitwise; tests compare them)
    const char *rb = std::getenv("GW_ROCK2_BLOCK");
    c->rock2_block = rb && *rb && *rb != '0';
    // the refinement's residual in double (k_half_refine) instead of double-float
    const char *rf = std::getenv("GW_REFINE_F64");
    c->refine_f64 = rf && *rf && *rf != '0';
    int rc = gw_setup_host(c, desc);
    if (rc) { delete c; return rc; }
    if (c->nbh > 1024) { delete c; return gw_fail(GW_ERR_ARG, "at most 1024 boreholes"); }
    c->device = desc->device;
    auto fail = [&](int r) { gw_destroy(c); return r; };
    if ((rc = set_device(c))) return fail(rc);
    cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) return fail(gw_cuda_fail(e, "cudaStreamCreate"));
    if ((e = cudaEventCreate(&c->ev0)) != cudaSuccess || (e = cudaEventCreate(&c->ev1)) != cudaSuccess)
        return fail(gw_cuda_fail(e, "cudaEventCreate"));

    // material model as coefficient tables (double always: the fine-grained
    // entry points work on double fields), built on the GPU, or on the host
    // (GW_HOST_SETUP, or if the GPU's column grouping met a hash collision)
    const size_t ntab = (size_t)c->n_zclass * c->nx * c->ny;   // x and y tables
    {
        double *cx[2], *cy[2], *cz[2];
        if (!c->host_setup && (rc = gw_setup_tables_device(c, cx, cy, cz)) != GW_OK) {
            if (rc != GW_ERR_UNSUPPORTED) return fail(rc);
            c->host_setup = true;   // two material sequences with one hash: group exactly on the host
            gw_build_profiles(c);
        }
    }
    if (c->host_setup) {
        std::vector<double> cxm, cxp, cym, cyp, czm, czp;
        gw_build_coefs(c, cxm, cxp, cym, cyp, czm, czp);
        c->h_czm = czm;
        c->h_czp = czp;
        if ((rc = upload(c, &c->c64.cxm, cxm)) || (rc = upload(c, &c->c64.cxp, cxp)) ||
            (rc = upload(c, &c->c64.cym, cym)) || (rc = upload(c, &c->c64.cyp, cyp)) ||
            (rc = upload(c, &c->c64.czm, czm)) || (rc = upload(c, &c->c64.czp, czp)))
            return fail(rc);
    }
    const size_t nztab = (size_t)c->n_profiles * c->nz;
    if ((rc = dalloc(c, &c->c64.fx.a, ntab)) || (rc = dalloc(c, &c->c64.fx.ib, ntab)) ||
        (rc = dalloc(c, &c->c64.fx.cu, ntab)) || (rc = dalloc(c, &c->c64.fy.a, ntab)) ||
        (rc = dalloc(c, &c->c64.fy.ib, ntab)) || (rc = dalloc(c, &c->c64.fy.cu, ntab)))
        return fail(rc);
    std::vector<int> order((size_t)c->nx * c->ny);
    for (size_t q = 0; q < order.size(); ++q) order[q] = (int)q;
    std::stable_sort(order.begin(), order.end(),
                     [&](int x, int y) { return c->colprof[x] < c->colprof[y]; });
    if ((rc = upload(c, &c->d_colorder, order))) return fail(rc);
    {
        // rows holding pipe columns; their +-1 neighbourhood first
        const int ncol = c->n_inner + c->n_outer;
        if (ncol > 0) {
            c->jlo = *std::min_element(c->pipe_j.begin(), c->pipe_j.end());
            c->jhi = *std::max_element(c->pipe_j.begin(), c->pipe_j.end());
            c->ilo = *std::min_element(c->pipe_i.begin(), c->pipe_i.end());
            c->ihi = *std::max_element(c->pipe_i.begin(), c->pipe_i.end());
        }
        std::vector<int> ab;
        ab.reserve(order.size());
        auto in_a = [&](int q) {
            const int j = q % c->ny;
            return ncol > 0 && j >= c->jlo - 1 && j <= c->jhi + 1;
        };
        // within rows jlo-1..jhi+1: the pipe columns and their y-neighbours
        // (what the y pipe pass reads) first, ncol_p of them
        std::vector<char> in_p((size_t)c->nx * c->ny, 0);
        for (int q = 0; q < ncol; ++q) {
            const size_t col = (size_t)c->pipe_i[q] * c->ny + c->pipe_j[q];
            in_p[col] = 1;
            if (c->pipe_j[q] > 0) in_p[col - 1] = 1;
            if (c->pipe_j[q] < c->ny - 1) in_p[col + 1] = 1;
        }
        for (int q : order) if (in_p[q]) ab.push_back(q);
        c->ncol_p = (int)ab.size();
        for (int q : order) if (in_a(q) && !in_p[q]) ab.push_back(q);
        c->ncol_a = (int)ab.size();
        for (int q : order) if (!in_a(q)) ab.push_back(q);
        c->ncol_b = (int)ab.size() - c->ncol_a;
        if ((rc = upload(c, &c->d_colorder_ab, ab))) return fail(rc);
        // worth it when the pipe rows are a minority of the domain
        c->overlap = ncol > 0 && 2 * (long long)c->ncol_a <= (long long)order.size();
        if ((e = cudaStreamCreateWithFlags(&c->stream2, cudaStreamNonBlocking)) != cudaSuccess ||
            (e = cudaEventCreateWithFlags(&c->ev_a, cudaEventDisableTiming)) != cudaSuccess ||
            (e = cudaEventCreateWithFlags(&c->ev_px, cudaEventDisableTiming)) != cudaSuccess ||
            (e = cudaEventCreateWithFlags(&c->ev_p, cudaEventDisableTiming)) != cudaSuccess ||
            (e = cudaEventCreateWithFlags(&c->ev_q, cudaEventDisableTiming)) != cudaSuccess)
            return fail(gw_cuda_fail(e, "stream / event"));
    }
    if ((rc = upload(c, &c->d_gz, c->gz)) || (rc = upload(c, &c->d_zclass, c->zclass)) ||
        (rc = upload(c, &c->d_colprof, c->colprof)) || (rc = upload(c, &c->d_pipe_i, c->pipe_i)) ||
        (rc = upload(c, &c->d_pipe_j, c->pipe_j)) || (rc = upload(c, &c->d_pipe_b, c->pipe_b)))
        return fail(rc);
    std::vector<GwBhDev> bhd(c->nbh);
    for (int b = 0; b < c->nbh; ++b) {
        bhd[b].h = c->bh[b].h; bhd[b].v_inner = c->bh[b].v_inner; bhd[b].v_outer = c->bh[b].v_outer;
        bhd[b].mdot = c->bh[b].mdot;
        bhd[b].inner_begin = bhd[b].outer_begin = -1;
        bhd[b].inner_count = bhd[b].outer_count = 0;
    }
    const int ncol = c->n_inner + c->n_outer;
    std::vector<int> pipe_of((size_t)c->nx * c->ny, -1);
    bool unique_cols = true;
    for (int q = 0; q < ncol; ++q) {
        GwBhDev &B = bhd[c->pipe_b[q]];
        if (q < c->n_inner) { if (B.inner_begin < 0) B.inner_begin = q; B.inner_count++; }
        else { if (B.outer_begin < 0) B.outer_begin = q; B.outer_count++; }
        int &slot = pipe_of[(size_t)c->pipe_i[q] * c->ny + c->pipe_j[q]];
        if (slot >= 0) unique_cols = false;   // overlapping boreholes
        slot = q;
    }
    for (auto &B : bhd) { if (B.inner_begin < 0) B.inner_begin = 0; if (B.outer_begin < 0) B.outer_begin = 0; }
    // chunks of at most kPipeChunk pipe columns, never spanning two boreholes
    // or pipes (16: the sweep's per-thread column loop is short enough to
    // fill the GPU on a single well; 2 mm well step 0.280 -> 0.270 ms
    // against 32, and 8 is slower again)
    constexpr int kPipeChunk = 16;
    std::vector<int4> chunks;
    std::vector<int> bchunk(4 * (size_t)c->nbh, 0);
    for (int b = 0; b < c->nbh; ++b)
        for (int outer = 0; outer < 2; ++outer) {
            const int q0 = outer ? bhd[b].outer_begin : bhd[b].inner_begin;
            const int n = outer ? bhd[b].outer_count : bhd[b].inner_count;
            bchunk[4 * b + 2 * outer] = (int)chunks.size();
            for (int q = q0; q < q0 + n; q += kPipeChunk) chunks.push_back(make_int4(b, q, std::min(q + kPipeChunk, q0 + n), outer));
            bchunk[4 * b + 2 * outer + 1] = (int)chunks.size();
        }
    c->n_pipe_chunks = (int)chunks.size();
    if ((rc = upload(c, &c->d_pipe_chunks, chunks)) || (rc = upload(c, &c->d_bchunk, bchunk)) ||
        (rc = dalloc(c, &c->d_pipepart, (size_t)std::max(c->n_pipe_chunks, 1) * c->nz)))
        return fail(rc);
    // per line direction: pipe index along each line, then one flag per line
    // telling whether the line crosses any pipe column
    std::vector<int> plx((size_t)c->ny * c->nx + c->ny, 0), ply((size_t)c->nx * c->ny + c->nx, 0);
    for (int i = 0; i < c->nx; ++i)
        for (int j = 0; j < c->ny; ++j) {
            const int q = pipe_of[(size_t)i * c->ny + j];
            plx[(size_t)j * c->nx + i] = q;
            ply[(size_t)i * c->ny + j] = q;
            if (q >= 0) {
                plx[(size_t)c->ny * c->nx + j] = 1;
                ply[(size_t)c->nx * c->ny + i] = 1;
            }
        }
    if ((rc = upload(c, &c->d_bh, bhd)) || (rc = upload(c, &c->d_pipe_of, pipe_of)) ||
        (rc = upload(c, &c->d_pipe_lx, plx)) || (rc = upload(c, &c->d_pipe_ly, ply)))
        return fail(rc);
    const size_t N = ncell(c);
    if ((rc = dalloc(c, &c->d_utmp, (size_t)ncol * c->countz)) ||
        (rc = dalloc(c, &c->d_annmean, (size_t)c->nbh * c->nz)) ||
        (rc = dalloc(c, &c->d_advtab, (size_t)c->nbh * c->countz * 2)) ||
        (rc = dalloc(c, &c->d_nlev, c->nbh)) ||
        (rc = dalloc(c, &c->d_outlet, c->nbh)) || (rc = dalloc(c, &c->d_energy, c->nbh)) ||
        (rc = dalloc(c, &c->d_stage, GW_STAGE_TABLE)) || (rc = dalloc(c, &c->f_stage, GW_STAGE_TABLE)) ||
        (rc = dalloc(c, &c->d_step_counter, 1)) || (rc = dalloc(c, &c->d_flag, 1)) || (rc = dalloc(c, &c->d_err, 1)) ||
        (rc = dalloc(c, &c->d_time, 2)) || (rc = dalloc(c, &c->d_inlet, c->nbh)))
        return fail(rc);
    // the mixed path's float fields keep columns pz = nz rounded up to 4 apart,
    // so every column starts on 16 bytes (tensor-map tiles need 16-byte
    // strides); the padding levels stay 0 and no kernel reads them
    c->pz = mixed(c) ? (c->nz + 3) / 4 * 4 : c->nz;
    const size_t NF = gw_field_slots(c);
    if (mixed(c)) {
        // f_temp and f_g1 are one block, so together they can stage a double field
        if ((rc = dalloc(c, &c->f_u, NF)) || (rc = dalloc(c, &c->f_temp, 2 * NF)) ||
            (rc = dalloc(c, &c->f_tp, (size_t)ncol * c->nz)) ||
            (rc = dalloc(c, &c->f_pp, (size_t)ncol * c->countz)) ||
            (rc = dalloc(c, &c->f_fref, (size_t)c->n_profiles * c->nz)) ||
            (rc = dalloc(c, &c->d_fref64, (size_t)c->n_profiles * c->nz)) ||
            (rc = dalloc(c, &c->d_Tref, c->nz)))
            return fail(rc);
        if ((rc = dalloc(c, &c->c32.cxm, ntab)) || (rc = dalloc(c, &c->c32.cxp, ntab)) ||
            (rc = dalloc(c, &c->c32.cym, ntab)) || (rc = dalloc(c, &c->c32.cyp, ntab)) ||
            (rc = dalloc(c, &c->c32.czm, nztab)) || (rc = dalloc(c, &c->c32.czp, nztab)) ||
            (rc = gw_tables_to_float(c, c->c32.cxm, c->c64.cxm, ntab)) ||
            (rc = gw_tables_to_float(c, c->c32.cxp, c->c64.cxp, ntab)) ||
            (rc = gw_tables_to_float(c, c->c32.cym, c->c64.cym, ntab)) ||
            (rc = gw_tables_to_float(c, c->c32.cyp, c->c64.cyp, ntab)) ||
            (rc = gw_tables_to_float(c, c->c32.czm, c->c64.czm, nztab)) ||
            (rc = gw_tables_to_float(c, c->c32.czp, c->c64.czp, nztab)))
            return fail(rc);
        if ((rc = dalloc(c, &c->c32.fx.a, ntab)) || (rc = dalloc(c, &c->c32.fx.ib, ntab)) ||
            (rc = dalloc(c, &c->c32.fx.cu, ntab)) || (rc = dalloc(c, &c->c32.fy.a, ntab)) ||
            (rc = dalloc(c, &c->c32.fy.ib, ntab)) || (rc = dalloc(c, &c->c32.fy.cu, ntab)) ||
            (rc = dalloc(c, &c->c32.hx, 4 * ntab)) || (rc = dalloc(c, &c->c32.hy, 4 * ntab)))
            return fail(rc);
        c->f_g1 = c->f_temp + NF;
        GW_CUDA(cudaMemset(c->f_u, 0, NF * sizeof(float)));
        GW_CUDA(cudaMemset(c->f_temp, 0, 2 * NF * sizeof(float)));
        std::vector<double> zero(c->nz, 0.0);
        if ((rc = set_reference_profile(c, zero.data()))) return fail(rc);
    } else {
        if ((rc = dalloc(c, &c->c64.hx, 4 * ntab)) || (rc = dalloc(c, &c->c64.hy, 4 * ntab)))
            return fail(rc);
        if ((rc = dalloc(c, &c->d_u, N)) || (rc = dalloc(c, &c->d_temp, N)) || (rc = dalloc(c, &c->d_g1, N)) ||
            (rc = dalloc(c, &c->d_tp, (size_t)ncol * c->nz)) ||
            (rc = dalloc(c, &c->d_pp, (size_t)ncol * c->countz)))
            return fail(rc);
        GW_CUDA(cudaMemset(c->d_u, 0, N * sizeof(double)));
    }
    GW_CUDA(cudaMemset(c->d_outlet, 0, c->nbh * sizeof(double)));
    GW_CUDA(cudaMemset(c->d_err, 0, sizeof(int)));
    GW_CUDA(cudaMemset(c->d_energy, 0, c->nbh * sizeof(double)));
    c->modular_reason = (gw_fused_supported(c) ? 0 : GW_MODULAR_NZ) |
                        (unique_cols ? 0 : GW_MODULAR_SHARED_COLUMN);
    c->fused = c->modular_reason == 0;
    if (c->fused && (rc = gw_fused_prepare(c))) return fail(rc);
    if (mixed(c) && !c->fused)
        return fail(gw_fail(GW_ERR_UNSUPPORTED, (c->modular_reason & GW_MODULAR_NZ)
                                                    ? "GW_PREC_MIXED needs the fused step: nz too large"
                                                    : "GW_PREC_MIXED needs the fused step: a pipe column "
                                                      "shared by two boreholes"));
    *out = c;
    return GW_OK;
}

int gw_destroy(gw_ctx *c) {
    if (!c) return GW_OK;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    if (c->graph) cudaGraphExecDestroy(c->graph);
    if (c->graph_k) cudaGraphExecDestroy(c->graph_k);
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev1) cudaEventDestroy(c->ev1);
    if (c->ev_a) cudaEventDestroy(c->ev_a);
    if (c->ev_px) cudaEventDestroy(c->ev_px);
    if (c->ev_p) cudaEventDestroy(c->ev_p);
    if (c->ev_q) cudaEventDestroy(c->ev_q);
    if (c->stream2) { cudaStreamSynchronize(c->stream2); cudaStreamDestroy(c->stream2); }
    if (c->snap_stream) { cudaStreamSynchronize(c->snap_stream); cudaStreamDestroy(c->snap_stream); }
    for (int b = 0; b < 2; ++b) {
        if (c->ev_conv[b]) cudaEventDestroy(c->ev_conv[b]);
        if (c->ev_copy[b]) cudaEventDestroy(c->ev_copy[b]);
    }
    gw_adjoint_release(c);
    for (void *p : c->allocations) if (p) { gw_debug_unregister(c->device, p); cudaFree(p); }
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return GW_OK;
}

int gw_get_info(gw_ctx *c, gw_info_t *o) {
    if (!c || !o) return gw_fail(GW_ERR_ARG, "NULL argument");
    o->nx = c->nx; o->ny = c->ny; o->nz = c->nz; o->n_boreholes = c->nbh;
    o->countxy_inner = c->n_inner; o->countxy_outer = c->n_outer; o->countz = c->countz;
    o->n_zclass = c->n_zclass; o->n_profiles = c->n_profiles;
    o->eigen_estimate = c->eigen_estimate;
    o->device_bytes = c->device_bytes;
    o->overlap = c->overlap ? 1 : 0;
    o->fused = c->fused ? 1 : 0;
    o->modular_reason = c->modular_reason;
    o->tiling = c->half_cfg;
    o->mixed_options = c->mixed_flags;
    o->step_order = c->step_order;
    return GW_OK;
}

int gw_set_tiling(gw_ctx *c, int tiling) {
    if (!c) return gw_fail(GW_ERR_ARG, "NULL context");
    if (tiling < 0 || tiling >= GW_TILINGS) return gw_fail(GW_ERR_ARG, "tiling out of range");
    c->half_cfg = tiling;
    c->graph_dt = -1.0;   // recapture the step graph
    return GW_OK;
}

int gw_set_mixed_options(gw_ctx *c, int flags) {
    if (!c) return gw_fail(GW_ERR_ARG, "NULL context");
    if (flags & ~(GW_MIXED_ROCK2_F64 | GW_MIXED_REFINE)) return gw_fail(GW_ERR_ARG, "unknown GW_MIXED_* flag");
    if (!mixed(c)) return flags ? gw_fail(GW_ERR_ARG, "GW_MIXED_* options need a GW_PREC_MIXED context") : GW_OK;
    int rc = set_device(c);
    if (rc) return rc;
    if ((flags & GW_MIXED_ROCK2_F64) && (rc = gw_fused_prepare_rock2_f64(c))) return rc;
    if ((flags & GW_MIXED_REFINE) && (rc = gw_fused_prepare_refine(c))) return rc;
    c->mixed_flags = flags;
    c->graph_dt = -1.0;   // recapture the step graph
    return GW_OK;
}

int gw_set_overlap(gw_ctx *c, int on) {
    if (!c) return gw_fail(GW_ERR_ARG, "NULL context");
    if (on && c->n_inner + c->n_outer == 0) return gw_fail(GW_ERR_ARG, "no pipe columns to overlap");
    c->overlap = on != 0;
    c->graph_dt = -1.0;   // recapture the step graph
    return GW_OK;
}

int gw_set_field(gw_ctx *c, const double *T) {
    if (!c || !T) return gw_fail(GW_ERR_ARG, "NULL argument");
    int rc = set_device(c);
    if (rc) return rc;
    if (mixed(c)) {
        if ((rc = set_reference_profile(c, T))) return rc;
        c->tables_dt = -1.0;   // the advection table depends on T_ref
        return gw_fused_set_theta(c, T);
    }
    GW_CUDA(cudaMemcpyAsync(c->d_u, T, ncell(c) * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    return sync(c);
}

int gw_get_field(gw_ctx *c, double *T) {
    if (!c || !T) return gw_fail(GW_ERR_ARG, "NULL argument");
    int rc = set_device(c);
    if (rc) return rc;
    if (mixed(c)) return gw_fused_get_theta(c, T);
    GW_CUDA(cudaMemcpyAsync(T, c->d_u, ncell(c) * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    return sync(c);
}

int gw_init_thermal_gradient(gw_ctx *c, double T_surface, double gradient) {
    if (!c) return gw_fail(GW_ERR_ARG, "NULL argument");
    if (!std::isfinite(T_surface) || !std::isfinite(gradient))
        return gw_fail(GW_ERR_ARG, "T_surface and gradient must be finite");
    int rc = set_device(c);
    if (rc) return rc;
    // one column on the host, T_surface + gradient * z_k, as gw_set_field would
    // receive it; the field is then filled on the device (no N-cell host array)
    std::vector<double> col(c->nz);
    for (int k = 0; k < c->nz; ++k) col[k] = T_surface + gradient * c->gz[k];
    if (mixed(c)) {
        // T_ref is the first column, so theta = T - T_ref is exactly 0 everywhere
        if ((rc = set_reference_profile(c, col.data()))) return rc;
        c->tables_dt = -1.0;
        GW_CUDA(cudaMemsetAsync(c->f_u, 0, gw_field_slots(c) * sizeof(float), c->stream));
        return sync(c);
    }
    GW_CUDA(cudaMemcpyAsync(c->d_temp, col.data(), c->nz * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    if ((rc = gw_launch_broadcast_column(c, c->d_u, c->d_temp))) return rc;
    return sync(c);
}

int gw_set_inlet_program(gw_ctx *c, int n, const int *ops, const double *args) {
    if (!c || !ops || !args) return gw_fail(GW_ERR_ARG, "NULL argument");
    if (c->inlet_kind != GW_INLET_EXPRESSION)
        return gw_fail(GW_ERR_ARG, "the context's inlet kind is not GW_INLET_EXPRESSION");
    if (n < 1 || n > GW_PROGRAM_MAX) return gw_fail(GW_ERR_ARG, "an inlet program has 1 to 64 operations");
    // the stack never underflows or grows beyond 16, and one value is left
    int depth = 0;
    bool uses_sched = false;
    for (int i = 0; i < n; ++i) {
        const int o = ops[i];
        if (o < GW_OP_CONST || o > GW_OP_MAX) return gw_fail(GW_ERR_ARG, "unknown GW_OP_* in the inlet program");
        if (o == GW_OP_CONST && !std::isfinite(args[i]))
            return gw_fail(GW_ERR_ARG, "inlet program constants must be finite");
        if (o <= GW_OP_BH) ++depth;                      // pushes
        else if (o == GW_OP_SCHED || o == GW_OP_NEG) {   // unary
            if (depth < 1) return gw_fail(GW_ERR_ARG, "inlet program: operand missing");
            uses_sched |= o == GW_OP_SCHED;
        } else {                                         // binary
            if (depth < 2) return gw_fail(GW_ERR_ARG, "inlet program: operand missing");
            --depth;
        }
        if (depth > 16) return gw_fail(GW_ERR_ARG, "inlet program: stack deeper than 16");
    }
    if (depth != 1) return gw_fail(GW_ERR_ARG, "inlet program must leave exactly one value");
    int rc = set_device(c);
    if (rc) return rc;
    if (!c->d_prog_op) {
        if ((rc = dalloc(c, &c->d_prog_op, GW_PROGRAM_MAX)) || (rc = dalloc(c, &c->d_prog_arg, GW_PROGRAM_MAX)))
            return rc;
    }
    c->prog_op.assign(ops, ops + n);
    c->prog_arg.assign(args, args + n);
    c->prog_sched = uses_sched;
    GW_CUDA(cudaStreamSynchronize(c->stream));
    if ((rc = copy_to(c->d_prog_op, c->prog_op)) || (rc = copy_to(c->d_prog_arg, c->prog_arg))) return rc;
    c->n_prog = n;
    c->graph_dt = -1.0;   // the captured step reads the program's length
    return GW_OK;
}

int gw_set_inlet_schedule(gw_ctx *c, int n, const double *times, const double *values) {
    if (!c || !times || !values) return gw_fail(GW_ERR_ARG, "NULL argument");
    if (c->inlet_kind != GW_INLET_SCHEDULE && c->inlet_kind != GW_INLET_EXPRESSION)
        return gw_fail(GW_ERR_ARG, "the context's inlet kind is not GW_INLET_SCHEDULE or GW_INLET_EXPRESSION");
    if (n < 1) return gw_fail(GW_ERR_ARG, "a schedule needs at least one point");
    for (int q = 0; q < n; ++q) {
        if (!std::isfinite(times[q]) || !std::isfinite(values[q]))
            return gw_fail(GW_ERR_ARG, "schedule values must be finite");
        if (q > 0 && !(times[q] > times[q - 1]))
            return gw_fail(GW_ERR_ARG, "schedule times must be strictly increasing");
    }
    int rc = set_device(c);
    if (rc) return rc;
    c->sched_t.assign(times, times + n);
    c->sched_T.assign(values, values + n);
    if (n > c->n_sched) {
        GW_CUDA(cudaStreamSynchronize(c->stream));
        if ((rc = dalloc(c, &c->d_sched, 2 * (size_t)n))) return rc;   // the old one is freed at gw_destroy
    }
    c->n_sched = n;
    std::vector<double> tv(times, times + n);
    tv.insert(tv.end(), values, values + n);
    return copy_to(c->d_sched, tv);
}

int gw_field_alloc(gw_ctx *c, double **out) {
    if (!c || !out) return gw_fail(GW_ERR_ARG, "NULL argument");
    *out = nullptr;
    int rc = set_device(c);
    if (rc) return rc;
    double *p = nullptr;
    GW_CUDA(cudaMalloc((void **)&p, ncell(c) * sizeof(double)));
    cudaError_t e = cudaMemsetAsync(p, 0, ncell(c) * sizeof(double), c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) {
        cudaFree(p);
        return gw_cuda_fail(e, "cudaMemsetAsync(field)");
    }
    *out = p;
    return GW_OK;
}

int gw_field_free(gw_ctx *c, double *p) {
    if (!c) return gw_fail(GW_ERR_ARG, "NULL context");
    if (!p) return GW_OK;
    int rc = set_device(c);
    if (rc || (rc = sync(c))) return rc;
    GW_CUDA(cudaFree(p));
    return GW_OK;
}

int gw_field_copy(gw_ctx *c, double *dst, const double *src) {
    if (!c || !dst || !src) return gw_fail(GW_ERR_ARG, "NULL argument");
    int rc = set_device(c);
    if (rc) return rc;
    if (dst == src) return GW_OK;
    GW_CUDA(cudaMemcpyAsync(dst, src, ncell(c) * sizeof(double), cudaMemcpyDefault, c->stream));
    return sync(c);
}

int gw_lincomb(gw_ctx *c, double *dst, int n, const double *coeffs, const double *const *srcs) {
    if (!c || !dst || (n > 0 && (!coeffs || !srcs))) return gw_fail(GW_ERR_ARG, "NULL argument");
    if (n < 0 || n > 8) return gw_fail(GW_ERR_ARG, "gw_lincomb takes 0 to 8 sources");
    for (int q = 0; q < n; ++q)
        if (!srcs[q]) return gw_fail(GW_ERR_ARG, "source field pointer is NULL");
    int rc = set_device(c);
    if (rc || (rc = gw_launch_lincomb(c, dst, n, coeffs, srcs))) return rc;
    return sync(c);
}

int gw_rhs_diffusion_z(gw_ctx *c, double *dphi, const double *phi) {
    if (!c) return gw_fail(GW_ERR_ARG, "NULL context");
    int rc = check_field_ptrs(dphi, phi);
    if (rc || (rc = set_device(c))) return rc;
    if (dphi == phi) return gw_fail(GW_ERR_ARG, "dphi must not alias phi");
    if ((rc = gw_launch_zstage(c, dphi, phi, nullptr, 1.0, 0.0, 1))) return rc;
    return sync(c);
}

int gw_diffusion_1d(gw_ctx *c, double *dphi, const double *phi, double dt, int dir, int plus_I) {
    if (!c) return gw_fail(GW_ERR_ARG, "NULL context");
    int rc = check_field_ptrs(dphi, phi);
    if (rc || (rc = set_device(c))) return rc;
    if (dphi == phi) return gw_fail(GW_ERR_ARG, "dphi must not alias phi");
    if (dir == GW_DIR_Z) {
        if (plus_I) rc = gw_launch_zstage(c, dphi, phi, nullptr, dt, 0.0, 0);
        else rc = gw_launch_zstage(c, dphi, phi, nullptr, 1.0, 0.0, 1);
    } else if (dir == GW_DIR_X || dir == GW_DIR_Y) {
        if (plus_I) rc = gw_launch_explicit(c, dphi, phi, dt, dir);
        else return gw_fail(GW_ERR_UNSUPPORTED, "A_x/A_y without the identity is not on the path");
    } else {
        return gw_fail(GW_ERR_ARG, "Invalid direction chosen");
    }
    if (rc) return rc;
    return sync(c);
}

int gw_thomas(gw_ctx *c, double *U, const double *RHS, double dt, int dir) {
    if (!c) return gw_fail(GW_ERR_ARG, "NULL context");
    int rc = check_field_ptrs(U, RHS);
    if (rc || (rc = set_device(c))) return rc;
    if (dir != GW_DIR_X && dir != GW_DIR_Y) return gw_fail(GW_ERR_ARG, "Invalid direction chosen");
    if ((void *)U == (const void *)RHS) return gw_fail(GW_ERR_ARG, "U must not alias RHS");
    if ((rc = gw_ensure_factors(c, dt))) return rc;
    if ((rc = gw_launch_thomas(c, U, RHS, dir))) return rc;
    return sync(c);
}

// An expression inlet needs its program (and the schedule it reads).
static int inlet_ready(const gw_ctx *c) {
    if (c->inlet_kind != GW_INLET_EXPRESSION) return GW_OK;
    if (c->n_prog == 0) return gw_fail(GW_ERR_ARG, "no inlet program set (gw_set_inlet_program)");
    if (c->prog_sched && c->n_sched == 0)
        return gw_fail(GW_ERR_ARG, "the inlet program reads a schedule: gw_set_inlet_schedule first");
    return GW_OK;
}

int gw_advection(gw_ctx *c, double *phi, double dt, double t) {
    if (!c || !phi) return gw_fail(GW_ERR_ARG, "NULL argument");
    int rc = inlet_ready(c);
    if (rc) return rc;
    rc = set_device(c);
    if (rc || (rc = gw_launch_advection(c, phi, dt, t))) return rc;
    return sync(c);
}

int gw_adi_adv(gw_ctx *c, double *u, double *temp, double t, double dt) {
    if (!c) return gw_fail(GW_ERR_ARG, "NULL context");
    int rc = inlet_ready(c);
    if (rc) return rc;
    rc = check_field_ptrs(u, temp);
    if (rc || (rc = set_device(c))) return rc;
    if (u == temp) return gw_fail(GW_ERR_ARG, "temp must not alias u");
    if ((rc = gw_ensure_factors(c, dt / 2))) return rc;
    if ((rc = adi_adv(c, u, temp, dt, t))) return rc;
    return sync(c);
}

int gw_rock2_stages(gw_ctx *c, double dt, int max_stages, int *stages, int *covered) {
    if (!c || !stages || !covered) return gw_fail(GW_ERR_ARG, "NULL argument");
    return gw_rock2_choose(dt, c->eigen_estimate, max_stages, stages, covered);
}

// steps per graph launch of gw_step for calls of at least that many (the
// rest one step per launch): 8 steps trim the gaps between launches (large
// well 0.5985 -> 0.5962 ms per step, 2 mm well 0.2456 -> 0.2425; 32: the same)
constexpr int kGraphSteps = 8;

int gw_step(gw_ctx *c, double t0, double dt, int nsteps, int max_stages) {
    if (!c) return gw_fail(GW_ERR_ARG, "NULL context");
    if (nsteps < 0) return gw_fail(GW_ERR_ARG, "nsteps must be >= 0");
    if (!(dt > 0) || !std::isfinite(dt)) return gw_fail(GW_ERR_ARG, "dt must be positive and finite");
    int rc = set_device(c);
    if (rc) return rc;
    int s, covered;
    if ((rc = gw_rock2_choose(dt, c->eigen_estimate, max_stages, &s, &covered))) return rc;
    if (c->inlet_kind == GW_INLET_SCHEDULE && (!c->fused || c->n_sched == 0))
        return gw_fail(c->fused ? GW_ERR_ARG : GW_ERR_UNSUPPORTED,
                       c->fused ? "no inlet schedule set (gw_set_inlet_schedule)"
                                : "a schedule inlet needs the fused step");
    if (c->inlet_kind == GW_INLET_EXPRESSION) {
        if (!c->fused) return gw_fail(GW_ERR_UNSUPPORTED, "an inlet program needs the fused step");
        if (c->n_prog == 0) return gw_fail(GW_ERR_ARG, "no inlet program set (gw_set_inlet_program)");
        if (c->prog_sched && c->n_sched == 0)
            return gw_fail(GW_ERR_ARG, "the inlet program reads a schedule: gw_set_inlet_schedule first");
    }
    if ((rc = gw_prepare_step(c, dt, s, nsteps))) return rc;
    if ((rc = gw_set_step_time(c, t0, dt))) return rc;
    c->t_now = t0 + nsteps * dt;
    if (nsteps == 0) return sync(c);
    // one step, or kGraphSteps steps, per graph launch
    auto capture = [&](int steps, cudaGraphExec_t *out) -> int {
        cudaGraph_t g;
        GW_CUDA(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
        int r3 = GW_OK;
        for (int k = 0; k < steps && r3 == GW_OK; ++k) {
            if (c->fused) {
                r3 = gw_fused_step(c, dt, s);
            } else {
                int r1 = rock2_step(c, c->d_u, c->d_g1, c->d_temp, dt, s);
                int r2 = r1 ? r1 : adi_adv(c, c->d_u, c->d_temp, dt);
                r3 = r2 ? r2 : gw_launch_record(c, dt);
            }
        }
        cudaError_t e = cudaStreamEndCapture(c->stream, &g);
        if (r3) { if (e == cudaSuccess) cudaGraphDestroy(g); return r3; }
        if (e != cudaSuccess) return gw_cuda_fail(e, "cudaStreamEndCapture");
        e = cudaGraphInstantiate(out, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return gw_cuda_fail(e, "cudaGraphInstantiate");
        return GW_OK;
    };
    // The overlapped step's two launch orders give the same state bitwise;
    // which is faster depends on which stream's chain is the longer
    // (205 x 205 x 2002: order 1 by 4%, 225 x 225 x 402: order 0 by 5%).  A
    // new step size, stage count or setting times both as the graphs gw_step
    // launches (kGraphSteps steps each; one-step graphs hide part of the
    // difference): one warm-up launch of each, then three rounds with the
    // order inside a round alternating, the best round counting (64 trial
    // steps: 15 ms on 225 x 225 x 402, 37 ms on 205 x 205 x 2002).  The state
    // is restored (field, outlet and energy values; the step counter
    // restarts) and the faster graph kept.
    auto tune_order = [&]() -> int {
        const bool mix = mixed(c);
        const size_t bytes = gw_field_slots(c) * (mix ? sizeof(float) : sizeof(double));
        void *u = mix ? (void *)c->f_u : (void *)c->d_u, *save = mix ? (void *)c->f_g1 : (void *)c->d_g1;
        std::vector<double> outl(c->nbh), energy(c->nbh);
        GW_CUDA(cudaMemcpyAsync(save, u, bytes, cudaMemcpyDeviceToDevice, c->stream));
        GW_CUDA(cudaMemcpyAsync(outl.data(), c->d_outlet, c->nbh * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
        GW_CUDA(cudaMemcpyAsync(energy.data(), c->d_energy, c->nbh * sizeof(double), cudaMemcpyDeviceToHost,
                                c->stream));
        cudaGraphExec_t g[2] = {nullptr, nullptr};
        float best_ms[2] = {1e30f, 1e30f};
        int r = GW_OK;
        for (int o = 0; o < 2 && r == GW_OK; ++o) {
            c->step_order = o;
            r = capture(kGraphSteps, &g[o]);
        }
        cudaError_t e = cudaSuccess;
        for (int o = 0; o < 2 && r == GW_OK && e == cudaSuccess; ++o) e = cudaGraphLaunch(g[o], c->stream);
        for (int round = 0; round < 3 && r == GW_OK && e == cudaSuccess; ++round)
            for (int q = 0; q < 2 && e == cudaSuccess; ++q) {
                const int o = q ^ (round & 1);
                float ms = 0.f;
                if ((e = cudaEventRecord(c->ev0, c->stream)) != cudaSuccess) break;
                e = cudaGraphLaunch(g[o], c->stream);
                if (e == cudaSuccess) e = cudaEventRecord(c->ev1, c->stream);
                if (e == cudaSuccess) e = cudaEventSynchronize(c->ev1);
                if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, c->ev0, c->ev1);
                best_ms[o] = std::min(best_ms[o], ms);
            }
        if (r == GW_OK && e != cudaSuccess) r = gw_cuda_fail(e, "timing the step orders");
        const int best = best_ms[1] < best_ms[0] ? 1 : 0;
        if (g[1 - best]) cudaGraphExecDestroy(g[1 - best]);
        if (r != GW_OK) {
            if (g[best]) cudaGraphExecDestroy(g[best]);
            return r;
        }
        c->step_order = best;
        c->graph_k = g[best];
        GW_CUDA(cudaMemcpyAsync(u, save, bytes, cudaMemcpyDeviceToDevice, c->stream));
        GW_CUDA(cudaMemcpyAsync(c->d_outlet, outl.data(), c->nbh * sizeof(double), cudaMemcpyHostToDevice, c->stream));
        GW_CUDA(cudaMemcpyAsync(c->d_energy, energy.data(), c->nbh * sizeof(double), cudaMemcpyHostToDevice,
                                c->stream));
        GW_CUDA(cudaMemsetAsync(c->d_step_counter, 0, sizeof(int), c->stream));
        GW_CUDA(cudaStreamSynchronize(c->stream));
        return capture(1, &c->graph);
    };
    if (!c->graph || c->graph_dt != dt || c->graph_s != s || c->graph_gen != c->series_gen) {
        if (c->graph) { cudaGraphExecDestroy(c->graph); c->graph = nullptr; }
        if (c->graph_k) { cudaGraphExecDestroy(c->graph_k); c->graph_k = nullptr; }
        // timed again for a new step size, stage count or setting (each
        // setter resets graph_dt), not for a longer outlet series alone
        const bool retime = c->graph_dt != dt || c->graph_s != s;
        if (c->fused && c->overlap && c->step_order_fixed < 0 && retime) {
            if ((rc = tune_order())) return rc;
        } else if ((rc = capture(1, &c->graph))) {
            return rc;
        }
        c->graph_dt = dt;
        c->graph_s = s;
        c->graph_gen = c->series_gen;
    }
    if (nsteps >= kGraphSteps && !c->graph_k && (rc = capture(kGraphSteps, &c->graph_k))) return rc;
    GW_CUDA(cudaEventRecord(c->ev0, c->stream));
    int n = 0;
    if (c->graph_k)
        for (; n + kGraphSteps <= nsteps; n += kGraphSteps) GW_CUDA(cudaGraphLaunch(c->graph_k, c->stream));
    for (; n < nsteps; ++n) GW_CUDA(cudaGraphLaunch(c->graph, c->stream));
    GW_CUDA(cudaEventRecord(c->ev1, c->stream));
    if ((rc = sync(c)) || (rc = gw_debug_status(c->device)) || (rc = gw_fused_status(c))) return rc;
    float ms = 0.f;
    GW_CUDA(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
    c->last_step_ms = ms;
    return GW_OK;
}

int gw_get_last_step_time(gw_ctx *c, double *ms) {
    if (!c || !ms) return gw_fail(GW_ERR_ARG, "NULL argument");
    *ms = c->last_step_ms;
    return GW_OK;
}

int gw_profile_kernels(gw_ctx *c, double dt, int reps, double *ms_out) {
    if (!c || !ms_out) return gw_fail(GW_ERR_ARG, "NULL argument");
    if (reps < 1 || !(dt > 0)) return gw_fail(GW_ERR_ARG, "reps >= 1 and dt > 0 required");
    if (!c->fused) return gw_fail(GW_ERR_UNSUPPORTED, "this context runs the modular step");
    int rc = set_device(c);
    if (rc || (rc = gw_ensure_factors(c, dt / 2))) return rc;
    int s, covered;
    if ((rc = gw_rock2_choose(dt, c->eigen_estimate, 100, &s, &covered))) return rc;
    if ((rc = upload_stages(c, dt, s)) || (rc = gw_fused_set_dt(c, dt))) return rc;
    c->tables_dt = dt;
    c->tables_s = s;
    void *u = mixed(c) ? (void *)c->f_u : (void *)c->d_u;
    void *bak = mixed(c) ? (void *)c->f_g1 : (void *)c->d_g1;
    const size_t bytes = gw_field_slots(c) * (mixed(c) ? sizeof(float) : sizeof(double));
    GW_CUDA(cudaMemcpyAsync(bak, u, bytes, cudaMemcpyDeviceToDevice, c->stream));
    for (int part = 0; part < GW_KERNEL_COUNT; ++part) {
        float total = 0.f;
        for (int r = 0; r < reps; ++r) {
            GW_CUDA(cudaEventRecord(c->ev0, c->stream));
            if ((rc = gw_fused_time_part(c, dt, s, part))) return rc;
            GW_CUDA(cudaEventRecord(c->ev1, c->stream));
            if ((rc = sync(c))) return rc;
            float ms = 0.f;
            GW_CUDA(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
            total += ms;
        }
        ms_out[part] = total / reps;
    }
    GW_CUDA(cudaMemcpyAsync(u, bak, bytes, cudaMemcpyDeviceToDevice, c->stream));
    if ((rc = sync(c))) return rc;
    return gw_debug_status(c->device);
}

int gw_snapshot_host_alloc(gw_ctx *c, float **host) {
    if (!c || !host) return gw_fail(GW_ERR_ARG, "NULL argument");
    *host = nullptr;
    int rc = set_device(c);
    if (rc) return rc;
    GW_CUDA(cudaMallocHost((void **)host, ncell(c) * sizeof(float)));
    return GW_OK;
}

int gw_snapshot_host_free(gw_ctx *c, float *host) {
    if (!c) return gw_fail(GW_ERR_ARG, "NULL context");
    if (!host) return GW_OK;
    int rc = set_device(c);
    if (rc || (rc = gw_snapshot_wait(c))) return rc;
    GW_CUDA(cudaFreeHost(host));
    return GW_OK;
}

int gw_snapshot(gw_ctx *c, float *host_dst) {
    if (!c || !host_dst) return gw_fail(GW_ERR_ARG, "NULL argument");
    int rc = set_device(c);
    if (rc) return rc;
    const size_t bytes = ncell(c) * sizeof(float);
    if (!c->snap_stream) {
        GW_CUDA(cudaStreamCreateWithFlags(&c->snap_stream, cudaStreamNonBlocking));
        for (int b = 0; b < 2; ++b) {
            GW_CUDA(cudaEventCreateWithFlags(&c->ev_conv[b], cudaEventDisableTiming));
            GW_CUDA(cudaEventCreateWithFlags(&c->ev_copy[b], cudaEventDisableTiming));
            if ((rc = dalloc(c, &c->d_snap[b], ncell(c)))) return rc;
        }
    }
    const int b = c->snap_next;
    // the staging buffer may still be on its way to the host: the device waits
    if (c->snap_pending[b]) GW_CUDA(cudaStreamWaitEvent(c->stream, c->ev_copy[b], 0));
    if ((rc = gw_launch_snapshot(c, c->d_snap[b]))) return rc;
    GW_CUDA(cudaEventRecord(c->ev_conv[b], c->stream));
    GW_CUDA(cudaStreamWaitEvent(c->snap_stream, c->ev_conv[b], 0));
    GW_CUDA(cudaMemcpyAsync(host_dst, c->d_snap[b], bytes, cudaMemcpyDeviceToHost, c->snap_stream));
    GW_CUDA(cudaEventRecord(c->ev_copy[b], c->snap_stream));
    c->snap_pending[b] = true;
    c->snap_next = b ^ 1;
    // the conversion (a fraction of a step) has finished when the call
    // returns, so the caller may change the state or T_ref at once; only the
    // copy to the host runs on
    GW_CUDA(cudaEventSynchronize(c->ev_conv[b]));
    return GW_OK;
}

int gw_snapshot_wait(gw_ctx *c) {
    if (!c) return gw_fail(GW_ERR_ARG, "NULL context");
    int rc = set_device(c);
    if (rc) return rc;
    for (int b = 0; b < 2; ++b)
        if (c->snap_pending[b]) {
            GW_CUDA(cudaEventSynchronize(c->ev_copy[b]));
            c->snap_pending[b] = false;
        }
    return GW_OK;
}

int gw_get_outlet(gw_ctx *c, double *T) {
    if (!c || !T) return gw_fail(GW_ERR_ARG, "NULL argument");
    int rc = set_device(c);
    if (rc) return rc;
    GW_CUDA(cudaMemcpyAsync(T, c->d_outlet, c->nbh * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    return sync(c);
}

int gw_get_outlet_series(gw_ctx *c, double *T, int nsteps) {
    if (!c || !T) return gw_fail(GW_ERR_ARG, "NULL argument");
    if (nsteps < 0 || nsteps > c->last_nsteps) return gw_fail(GW_ERR_ARG, "nsteps exceeds the last gw_step call");
    if (nsteps == 0) return GW_OK;
    int rc = set_device(c);
    if (rc) return rc;
    GW_CUDA(cudaMemcpyAsync(T, c->d_series, (size_t)nsteps * c->nbh * sizeof(double),
                            cudaMemcpyDeviceToHost, c->stream));
    return sync(c);
}

int gw_get_energy(gw_ctx *c, double *E) {
    if (!c || !E) return gw_fail(GW_ERR_ARG, "NULL argument");
    int rc = set_device(c);
    if (rc) return rc;
    GW_CUDA(cudaMemcpyAsync(E, c->d_energy, c->nbh * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    return sync(c);
}

int gw_reset_energy(gw_ctx *c) {
    if (!c) return gw_fail(GW_ERR_ARG, "NULL argument");
    int rc = set_device(c);
    if (rc) return rc;
    GW_CUDA(cudaMemsetAsync(c->d_energy, 0, c->nbh * sizeof(double), c->stream));
    return sync(c);
}

int gw_check_finite(gw_ctx *c) {
    if (!c) return gw_fail(GW_ERR_ARG, "NULL argument");
    int rc = set_device(c);
    if (rc) return rc;
    if (mixed(c)) rc = gw_fused_check_finite(c);
    else rc = gw_launch_check_finite(c, c->d_u, ncell(c));
    if (rc) return rc;
    int flag = 0;
    GW_CUDA(cudaMemcpyAsync(&flag, c->d_flag, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    if ((rc = sync(c))) return rc;
    return flag ? gw_fail(GW_ERR_NONFINITE, "state holds NaN or Inf") : GW_OK;
}

}  // extern "C"
