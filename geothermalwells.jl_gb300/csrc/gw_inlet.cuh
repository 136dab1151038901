// gw_inlet.cuh -- device evaluation of the inlet models that depend on time
// or on the outlet temperature: the piecewise-linear schedule and the inlet
// programs (GW_INLET_EXPRESSION), shared by the fused and the modular
// advection.
//
// A program is a postfix sequence of GW_OP_* (include/gw_gb300.h) over
// T_outlet of the borehole, the time t and the borehole index, the form a
// CustomInlet closure (bh, T_outlet, t) -> T_in (src/physics.jl:315-318)
// takes when it is arithmetic.  Every operation is one correctly rounded
// double operation (no contraction), so the host oracle, evaluating the same
// sequence in C, gets the same bits.
#pragma once
#include <cuda_runtime.h>

#include "../../include/gw_gb300.h"

#define GW_PROGRAM_STACK 16

// T_in(t) of a schedule (times then values, ns points): linear between the
// points, held constant outside them.
__device__ __forceinline__ double gw_sched_eval(const double *__restrict__ sched, int ns, double t) {
    const double *ts = sched, *vs = sched + ns;
    if (ns <= 0) return 0.0;
    if (t <= ts[0]) return vs[0];
    if (t >= ts[ns - 1]) return vs[ns - 1];
    int lo = 0, hi = ns - 1;   // ts[lo] <= t < ts[hi]
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (ts[mid] <= t) lo = mid; else hi = mid;
    }
    const double a = __ddiv_rn(__dsub_rn(t, ts[lo]), __dsub_rn(ts[hi], ts[lo]));
    return __fma_rn(a, __dsub_rn(vs[hi], vs[lo]), vs[lo]);
}

// One inlet program for borehole b.  The host checked the program when it
// was set (stack never under- or overflows, one value left), so the stack
// indices stay within GW_PROGRAM_STACK.
__device__ __forceinline__ double gw_program_eval(const int *__restrict__ op, const double *__restrict__ arg,
                                                  int n, double tout, double t, int b,
                                                  const double *__restrict__ sched, int ns) {
    double st[GW_PROGRAM_STACK];
    int sp = 0;
    for (int i = 0; i < n; ++i) {
        switch (op[i]) {
            case GW_OP_CONST: st[sp++] = arg[i]; break;
            case GW_OP_TOUT: st[sp++] = tout; break;
            case GW_OP_TIME: st[sp++] = t; break;
            case GW_OP_BH: st[sp++] = (double)b; break;
            case GW_OP_SCHED: st[sp - 1] = gw_sched_eval(sched, ns, st[sp - 1]); break;
            case GW_OP_NEG: st[sp - 1] = -st[sp - 1]; break;
            case GW_OP_ADD: --sp; st[sp - 1] = __dadd_rn(st[sp - 1], st[sp]); break;
            case GW_OP_SUB: --sp; st[sp - 1] = __dsub_rn(st[sp - 1], st[sp]); break;
            case GW_OP_MUL: --sp; st[sp - 1] = __dmul_rn(st[sp - 1], st[sp]); break;
            case GW_OP_DIV: --sp; st[sp - 1] = __ddiv_rn(st[sp - 1], st[sp]); break;
            case GW_OP_MIN: --sp; st[sp - 1] = fmin(st[sp - 1], st[sp]); break;
            case GW_OP_MAX: --sp; st[sp - 1] = fmax(st[sp - 1], st[sp]); break;
            default: break;
        }
    }
    return st[0];
}
