// gw_fused.h -- the fused step (gw_fused.cu) as seen by gw_api.cu.
#pragma once
#include "gw_internal.h"

// 1 if the column kernel's shared memory fits this context's nz.
int gw_fused_supported(const gw_ctx *c);
// Per-context kernel attributes and the column kernel's grid size.
int gw_fused_prepare(gw_ctx *c);
// Mixed contexts: launch shape of the ROCK2 column kernel with double stages
// over the float field (GW_MIXED_ROCK2_F64); GW_ERR_UNSUPPORTED beyond its nz.
int gw_fused_prepare_rock2_f64(gw_ctx *c);
// Mixed contexts: check that GW_MIXED_REFINE can run (fused mixed step) and
// allocate its double-float tables (outside any stream capture).
int gw_fused_prepare_refine(gw_ctx *c);
// the double-float refinement tables for half-step size h, before the step's capture
int gw_fused_refine_tables(gw_ctx *c, double h);
// GW_ERR_CUDA if a kernel's bounded wait ran out since the last check (and clear the flag)
int gw_fused_status(gw_ctx *c);
// Build the step-size dependent tables (advection departures) for dt.
int gw_fused_set_dt(gw_ctx *c, double dt);
// Enqueue one full step (ROCK2 columns, two half steps, record) on c->stream.
// Requires the Thomas factors for dt/2 and the stage table c->d_stage for s.
int gw_fused_step(gw_ctx *c, double dt, int s);
// The adjoint's forward store: ROCK2 and the first half step on the
// context's state (u <- u*, temp <- u1), with the swept pipe columns of the
// step's two pipe passes copied to tpA / tpC ([column][level], storage type).
int gw_fused_adjoint_store(gw_ctx *c, double dt, int s, void *tpA, void *tpC);
// Enqueue one kernel class of the step (GW_KERNEL_*), for timing.
int gw_fused_time_part(gw_ctx *c, double dt, int s, int part);
// Mixed path: upload a double field as theta / download theta as a double
// field (through the 8N-byte scratch f_temp..f_g1; T_ref must be current).
int gw_fused_set_theta(gw_ctx *c, const double *T_host);
int gw_fused_get_theta(gw_ctx *c, double *T_host);
// Set c->d_flag if the state holds a NaN or Inf.
int gw_fused_check_finite(gw_ctx *c);
