// gw_batch.cu -- ensembles of well designs advanced together.
//
// A batch holds the contexts of many designs (each built by gw_create with
// its own grids, materials and boreholes).  One ensemble step is captured as
// a single CUDA graph: a fork from the batch's stream into every design's
// stream, that design's fused step (gw_fused.cu), and a join back -- so all
// designs advance with one graph launch per step and the designs' kernels
// run concurrently, which fills the GPU even for the small designs.
#include <cuda_runtime.h>

#include <vector>

#include "gw_fused.h"
#include "gw_internal.h"

struct gw_batch {
    std::vector<gw_ctx *> ctx;
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t fork = nullptr, ev0 = nullptr, ev1 = nullptr;
    std::vector<cudaEvent_t> join;
    // graph = kSteps steps of every design between one fork and one join
    // (designs do not wait for each other every step); graph1 = one step
    cudaGraphExec_t graph = nullptr, graph1 = nullptr;
    double graph_dt = -1.0;
    int graph_steps_cap = -1;
    std::vector<int> graph_s;
    std::vector<int> graph_gen;   // each context's series_gen at capture
    double last_ms = 0.0;
};

namespace {
// steps per design between the ensemble's fork and join: the designs run
// that far apart, so a slow step of one design is absorbed by the others
// (64-design ensemble: 13.77 ms per step at 4, 13.50 at 16, 13.40 at 32,
// 13.35 at 64; the graph holds designs x 10 x kSteps kernel nodes)
constexpr int kSteps = 32;

// Capture `steps` steps of every design, each design on its own stream,
// between one fork and one join on the batch stream.
int capture(gw_batch *b, double dt, const std::vector<int> &s, int steps, cudaGraphExec_t *out) {
    const int n = (int)b->ctx.size();
    cudaGraph_t g;
    GW_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    int r = GW_OK;
    cudaError_t e = cudaEventRecord(b->fork, b->stream);
    for (int d = 0; d < n && e == cudaSuccess && r == GW_OK; ++d) {
        gw_ctx *c = b->ctx[d];
        if ((e = cudaStreamWaitEvent(c->stream, b->fork, 0)) != cudaSuccess) break;
        for (int k = 0; k < steps && r == GW_OK; ++k) r = gw_fused_step(c, dt, s[d]);
        if (r != GW_OK) break;
        if ((e = cudaEventRecord(b->join[d], c->stream)) != cudaSuccess) break;
        e = cudaStreamWaitEvent(b->stream, b->join[d], 0);
    }
    cudaError_t ee = cudaStreamEndCapture(b->stream, &g);
    if (r != GW_OK || e != cudaSuccess || ee != cudaSuccess) {
        if (ee == cudaSuccess) cudaGraphDestroy(g);
        if (r != GW_OK) return r;
        return gw_cuda_fail(e != cudaSuccess ? e : ee, "ensemble step capture");
    }
    e = cudaGraphInstantiate(out, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return gw_cuda_fail(e, "cudaGraphInstantiate");
    return GW_OK;
}

int prepare(gw_ctx *c, double dt, int max_stages, int nsteps, int *s_out) {
    int s, covered, rc;
    if ((rc = gw_rock2_choose(dt, c->eigen_estimate, max_stages, &s, &covered))) return rc;
    if ((rc = gw_prepare_step(c, dt, s, nsteps))) return rc;
    *s_out = s;
    return GW_OK;
}
}  // namespace

extern "C" {

int gw_batch_step(gw_batch *b, double dt, int nsteps, int max_stages);

int gw_batch_create(gw_ctx *const *ctxs, int n, gw_batch **out) {
    if (!out || !ctxs || n < 1) return gw_fail(GW_ERR_ARG, "need at least one context");
    *out = nullptr;
    gw_batch *b = new gw_batch();
    b->device = ctxs[0]->device;
    for (int d = 0; d < n; ++d) {
        gw_ctx *c = ctxs[d];
        if (!c) { delete b; return gw_fail(GW_ERR_ARG, "NULL context in batch"); }
        if (c->device != b->device) { delete b; return gw_fail(GW_ERR_ARG, "all contexts must use one device"); }
        if (!c->fused) { delete b; return gw_fail(GW_ERR_UNSUPPORTED, "a context runs the modular step"); }
        b->ctx.push_back(c);
    }
    cudaError_t e;
    auto fail = [&](cudaError_t err, const char *what) { gw_batch_destroy(b); return gw_cuda_fail(err, what); };
    if ((e = cudaSetDevice(b->device)) != cudaSuccess) return fail(e, "cudaSetDevice");
    if ((e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking)) != cudaSuccess) return fail(e, "cudaStreamCreate");
    if ((e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming)) != cudaSuccess ||
        (e = cudaEventCreate(&b->ev0)) != cudaSuccess || (e = cudaEventCreate(&b->ev1)) != cudaSuccess)
        return fail(e, "cudaEventCreate");
    b->join.assign(n, nullptr);
    for (int d = 0; d < n; ++d)
        if ((e = cudaEventCreateWithFlags(&b->join[d], cudaEventDisableTiming)) != cudaSuccess)
            return fail(e, "cudaEventCreate");
    *out = b;
    return GW_OK;
}

int gw_batch_destroy(gw_batch *b) {
    if (!b) return GW_OK;
    cudaSetDevice(b->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->graph) cudaGraphExecDestroy(b->graph);
    if (b->graph1) cudaGraphExecDestroy(b->graph1);
    for (cudaEvent_t ev : b->join) if (ev) cudaEventDestroy(ev);
    if (b->fork) cudaEventDestroy(b->fork);
    if (b->ev0) cudaEventDestroy(b->ev0);
    if (b->ev1) cudaEventDestroy(b->ev1);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return GW_OK;
}

int gw_batch_set_tiling(gw_batch *b, int tiling) {
    if (!b) return gw_fail(GW_ERR_ARG, "NULL batch");
    if (tiling < 0 || tiling >= GW_TILINGS) return gw_fail(GW_ERR_ARG, "tiling out of range");
    for (gw_ctx *c : b->ctx) { c->half_cfg = tiling; c->graph_dt = -1.0; }
    b->graph_dt = -1.0;
    return GW_OK;
}

// Autotuning in two rounds.  Round 1: per design, time each half-step
// tiling of that design alone (x- and y-lines, `reps` launches, CUDA events
// on the design's stream) and note its fastest.  Round 2: time the real
// concurrent ensemble step (2 steps after a capture step) for every uniform
// tiling and for the per-design choices of round 1, and keep the fastest
// assignment.  Each design's state, outlet and energy are restored after.
int gw_batch_autotune(gw_batch *b, double dt, int reps, int *tiling_out) {
    if (!b || !(dt > 0) || reps < 1) return gw_fail(GW_ERR_ARG, "bad arguments");
    int rc;
    GW_CUDA(cudaSetDevice(b->device));
    const int n = (int)b->ctx.size();
    // save the states (u into the g1 scratch), the outlet / energy values and the clocks
    std::vector<std::vector<double>> outl(n), energy(n);
    std::vector<double> clock(n);
    for (int d = 0; d < n; ++d) clock[d] = b->ctx[d]->t_now;
    for (int d = 0; d < n; ++d) {
        gw_ctx *c = b->ctx[d];
        const size_t N = gw_field_slots(c);   // every slot of the state, padding included
        const bool mix = c->precision == GW_PREC_MIXED;
        GW_CUDA(cudaMemcpyAsync(mix ? (void *)c->f_g1 : (void *)c->d_g1, mix ? (void *)c->f_u : (void *)c->d_u,
                                N * (mix ? sizeof(float) : sizeof(double)), cudaMemcpyDeviceToDevice, c->stream));
        outl[d].resize(c->nbh);
        energy[d].resize(c->nbh);
        GW_CUDA(cudaMemcpyAsync(outl[d].data(), c->d_outlet, c->nbh * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
        GW_CUDA(cudaMemcpyAsync(energy[d].data(), c->d_energy, c->nbh * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
        GW_CUDA(cudaStreamSynchronize(c->stream));
    }
    // round 1
    std::vector<int> own(n, 0);
    for (int d = 0; d < n; ++d) {
        gw_ctx *c = b->ctx[d];
        int s;
        if ((rc = prepare(c, dt, 100, 1, &s))) return rc;
        float best = 1e30f;
        for (int t = 0; t < GW_TILINGS; ++t) {
            c->half_cfg = t;
            if ((rc = gw_fused_time_part(c, dt, s, GW_KERNEL_HALF_X)) ||
                (rc = gw_fused_time_part(c, dt, s, GW_KERNEL_HALF_Y)))
                return rc;
            GW_CUDA(cudaEventRecord(c->ev0, c->stream));
            for (int r = 0; r < reps; ++r)
                if ((rc = gw_fused_time_part(c, dt, s, GW_KERNEL_HALF_X)) ||
                    (rc = gw_fused_time_part(c, dt, s, GW_KERNEL_HALF_Y)))
                    return rc;
            GW_CUDA(cudaEventRecord(c->ev1, c->stream));
            GW_CUDA(cudaEventSynchronize(c->ev1));
            float ms = 0.f;
            GW_CUDA(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
            if (ms < best) { best = ms; own[d] = t; }
        }
    }
    // round 2: candidates are the uniform tilings and the round-1 choices
    std::vector<std::vector<int>> cand;
    for (int t = 0; t < GW_TILINGS; ++t) cand.push_back(std::vector<int>(n, t));
    cand.push_back(own);
    double best = 1e300;
    size_t arg = 0;
    for (size_t q = 0; q < cand.size(); ++q) {
        for (int d = 0; d < n; ++d) { b->ctx[d]->half_cfg = cand[q][d]; b->ctx[d]->graph_dt = -1.0; }
        b->graph_dt = -1.0;
        if ((rc = gw_batch_step(b, dt, 1, 100)) || (rc = gw_batch_step(b, dt, 2, 100))) return rc;
        if (b->last_ms < best) { best = b->last_ms; arg = q; }
    }
    for (int d = 0; d < n; ++d) {
        gw_ctx *c = b->ctx[d];
        c->half_cfg = cand[arg][d];
        c->graph_dt = -1.0;
        if (tiling_out) tiling_out[d] = cand[arg][d];
        const size_t N = gw_field_slots(c);   // every slot of the state, padding included
        const bool mix = c->precision == GW_PREC_MIXED;
        GW_CUDA(cudaMemcpyAsync(mix ? (void *)c->f_u : (void *)c->d_u, mix ? (void *)c->f_g1 : (void *)c->d_g1,
                                N * (mix ? sizeof(float) : sizeof(double)), cudaMemcpyDeviceToDevice, c->stream));
        GW_CUDA(cudaMemcpyAsync(c->d_outlet, outl[d].data(), c->nbh * sizeof(double), cudaMemcpyHostToDevice, c->stream));
        GW_CUDA(cudaMemcpyAsync(c->d_energy, energy[d].data(), c->nbh * sizeof(double), cudaMemcpyHostToDevice, c->stream));
        GW_CUDA(cudaStreamSynchronize(c->stream));
        c->t_now = clock[d];
    }
    b->graph_dt = -1.0;
    return GW_OK;
}

int gw_batch_step(gw_batch *b, double dt, int nsteps, int max_stages) {
    if (!b) return gw_fail(GW_ERR_ARG, "NULL batch");
    if (nsteps < 0 || !(dt > 0)) return gw_fail(GW_ERR_ARG, "nsteps >= 0 and dt > 0 required");
    GW_CUDA(cudaSetDevice(b->device));
    const int n = (int)b->ctx.size();
    std::vector<int> s(n);
    int rc;
    for (int d = 0; d < n; ++d) {
        gw_ctx *c = b->ctx[d];
        if (c->inlet_kind == GW_INLET_SCHEDULE && c->n_sched == 0)
            return gw_fail(GW_ERR_ARG, "a design has no inlet schedule set (gw_set_inlet_schedule)");
        if ((rc = prepare(c, dt, max_stages, nsteps, &s[d])) || (rc = gw_set_step_time(c, c->t_now, dt)))
            return rc;
    }
    if (nsteps == 0) return GW_OK;
    std::vector<int> gen(n);
    for (int d = 0; d < n; ++d) gen[d] = b->ctx[d]->series_gen;
    if (!b->graph1 || b->graph_dt != dt || b->graph_s != s || b->graph_gen != gen ||
        b->graph_steps_cap < nsteps) {
        if (b->graph) { cudaGraphExecDestroy(b->graph); b->graph = nullptr; }
        if (b->graph1) { cudaGraphExecDestroy(b->graph1); b->graph1 = nullptr; }
        if ((rc = capture(b, dt, s, 1, &b->graph1))) return rc;
        b->graph_dt = dt;
        b->graph_s = s;
        b->graph_gen = gen;
        b->graph_steps_cap = nsteps;
    }
    // the kSteps-step graph only for calls that use it
    if (nsteps >= kSteps && !b->graph && (rc = capture(b, dt, s, kSteps, &b->graph))) return rc;
    for (gw_ctx *c : b->ctx) GW_CUDA(cudaStreamSynchronize(c->stream));
    GW_CUDA(cudaEventRecord(b->ev0, b->stream));
    for (int k = 0; k + kSteps <= nsteps; k += kSteps) GW_CUDA(cudaGraphLaunch(b->graph, b->stream));
    for (int k = 0; k < nsteps % kSteps; ++k) GW_CUDA(cudaGraphLaunch(b->graph1, b->stream));
    GW_CUDA(cudaEventRecord(b->ev1, b->stream));
    GW_CUDA(cudaStreamSynchronize(b->stream));
    if ((rc = gw_debug_status(b->device))) return rc;
    for (gw_ctx *c : b->ctx)
        if ((rc = gw_fused_status(c))) return rc;
    float ms = 0.f;
    GW_CUDA(cudaEventElapsedTime(&ms, b->ev0, b->ev1));
    b->last_ms = ms;
    for (gw_ctx *c : b->ctx) { c->last_nsteps = nsteps; c->t_now += nsteps * dt; }
    return GW_OK;
}

int gw_batch_get_last_step_time(gw_batch *b, double *ms) {
    if (!b || !ms) return gw_fail(GW_ERR_ARG, "NULL argument");
    *ms = b->last_ms;
    return GW_OK;
}

}  // extern "C"
