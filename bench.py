#!/usr/bin/env python3
"""Benchmark of the GeothermalWells.jl time-step hot path on GB300.

Workload: the large single coaxial well, 205 x 205 x 2002 = 8.41e7 cells,
dt = 300 s (ROCK2 z-diffusion + ADI x/y line solves + semi-Lagrangian pipe
advection per step).  One bench step = one time step of the whole grid.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--precision fp64|mixed]
                  [--impl ours|reference]

The default arm times the fused device path (gw_step, graph-captured) with
CUDA events on the library's stream; `e2e` times the same steps through the
public solve() path with host buffers (field upload, steps, outlet series and
final field download).  `--impl reference` times the CPU FP64 restatement of
the reference (the oracle) on the host cores.  With N > 1 GPUs each rank runs
an independent replica of the well (the single-well step does not shard).
"""
import argparse
import json
import os
import subprocess
import tempfile
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "geothermalwells.jl_gb300"))

METRIC = "Mcell-steps/s"
WORD = {"fp64": 8, "mixed": 4}


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=500)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--precision", default="mixed", choices=["fp64", "mixed"],
                   help="path timed for `value`; the default run also times the other one")
    p.add_argument("--workload", default="large",
                   choices=["large", "2mm", "thomas", "ensemble", "adjoint"])
    p.add_argument("--fd", default="some", choices=["none", "some", "all"],
                   help="adjoint workload: parameters checked by central differences")
    p.add_argument("--adjoint-steps", type=int, default=0,
                   help="adjoint workload: number of steps (default: the workload's 2016)")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-compare", action="store_true",
                   help="skip timing the other precision beside the main one")
    p.add_argument("--cpu-sample-steps", type=int, default=1)
    p.add_argument("--cpu-threads", type=int, default=0,
                   help="reference arm: host threads for the oracle (default: all cores)")
    p.add_argument("--accuracy", type=int, default=0, metavar="NSTEPS",
                   help="run FP64 and mixed for NSTEPS steps and report their differences")
    p.add_argument("--dt", type=float, default=0.0, help="override the workload's step size [s]")
    p.add_argument("--accuracy-suite", action="store_true",
                   help="errors of every GPU path on every configuration (oracle / FP64 reference)")
    p.add_argument("--suite", default="", help="with --accuracy-suite: subset, e.g. cfg1,cfg2")
    p.add_argument("--kernels", action="store_true",
                   help="single-well workloads: only the per-kernel timing (each fused kernel "
                        "launched --steps times on the full grid, outside the step graph)")
    p.add_argument("--tiling", type=int, default=-1,
                   help="half-step tiling of the context, or of every ensemble design without autotuning "
                        "(default: the context's own; the ensemble autotunes)")
    return p.parse_args()


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def workload(name, dt=0.0):
    from geothermalwells_gb300 import workloads as W
    w = W.single_well_large() if name == "large" else W.single_well_2mm()
    if dt > 0:
        w["dt"] = float(dt)
    return w


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, gpu):
        self.proc = None
        self.path = os.path.join(tempfile.gettempdir(), "bench_clocks_%d.csv" % os.getpid())
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(gpu), "--query-gpu=clocks.sm,clocks.max.sm,power.draw,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        self.proc.wait()
        self.f.close()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0])); mx.append(float(parts[1]))
            except ValueError:
                continue
            for n, v in zip(names, parts[3:7]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)),
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_init(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
        return rank, world, local, dist
    return 0, 1, 0, None


def reduce_replicas(dist, t_ms, units, device="cuda"):
    """Whole-job figures of independent replicas (one per rank, no data
    exchange): the slowest rank's time and the units all ranks processed."""
    if not dist:
        return t_ms, float(units)
    import torch
    t = torch.tensor([t_ms], dtype=torch.float64, device=device)
    u = torch.tensor([float(units)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    return float(t.item()), float(u.item())


def cpu_baseline(w, sample_steps, threads=0):
    """The oracle (CPU FP64 restatement of the reference) on all host cores
    (or `threads` of them), timed on a bounded sample: sample_steps full time
    steps of the workload."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    from geothermalwells_gb300 import rock2
    cores = O.set_threads(threads if threads > 0 else (os.cpu_count() or 1))
    orc = O.Oracle(w["gridx"], w["gridy"], w["gridz"], w["boreholes"], w["materials"],
                   w["inlet_model"])
    s, _ = rock2.choose_stages(w["dt"], orc.eigen_estimate())
    u = w["T0"].copy(order="F")
    t0 = time.perf_counter()
    orc.simulate(u, 0.0, w["dt"], sample_steps, s, rock2.coefficients(s))
    el = time.perf_counter() - t0
    ncell = u.size
    return {"value": ncell * sample_steps / el / 1e6, "unit": METRIC, "cores": cores,
            "kind": "port",
            "sample": "%d full time step(s) of the %s workload (%d cells), oracle OpenMP"
                      % (sample_steps, w["name"], ncell),
            "seconds": el}


def run_reference(args):
    rank, world, local, dist = dist_init(args)
    if rank != 0:
        return
    w = workload(args.workload, args.dt)
    steps = max(1, min(args.steps, 2))
    cb = cpu_baseline(w, steps, args.cpu_threads)
    line = {"impl": "reference", "metric": METRIC, "value": cb["value"], "unit": METRIC,
            "n_gpus": args.gpus, "steps": steps, "warmup": 0, "ms_per_step": cb["seconds"] * 1e3 / steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": {"workload": w["name"], "cells": int(w["T0"].size),
                                            "dt_s": w["dt"], "timed_steps_of_requested": [steps, args.steps]},
            "cpu_baseline": {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")},
            "e2e": {"value": cb["value"], "unit": METRIC, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_kernels(args):
    """Per-kernel device times (CUDA events) of the fused step's kernels on
    the full grid, each launched --steps times on its own: the launches a
    single-kernel profiler capture selects."""
    import ctypes
    from geothermalwells_gb300 import _lib, create_cache, GB300
    L = _lib.load()
    w = workload(args.workload, args.dt)
    cache = create_cache(backend=GB300(precision=args.precision), gridx=w["gridx"], gridy=w["gridy"],
                         gridz=w["gridz"], materials=w["materials"], boreholes=w["boreholes"],
                         inlet_model=w["inlet_model"])
    cache.set_field(w["T0"])
    if args.tiling >= 0:
        _lib.check(L.gw_set_tiling(cache.ctx, args.tiling))
    prof = (ctypes.c_double * len(_lib.KERNELS))()
    _lib.check(L.gw_profile_kernels(cache.ctx, w["dt"], max(1, args.steps), prof))
    print(json.dumps({"workload": w.get("name", args.workload), "precision": args.precision,
                      "launches_per_kernel": max(1, args.steps),
                      "kernel_ms": dict(zip(_lib.KERNELS, list(prof)))}), flush=True)
    cache.close()


def run_ours(args):
    rank, world, local, dist = dist_init(args)
    from geothermalwells_gb300 import _lib, create_cache, GB300
    L = _lib.load()
    w = workload(args.workload, args.dt)
    cache = create_cache(backend=GB300(device=local, precision=args.precision), gridx=w["gridx"],
                         gridy=w["gridy"], gridz=w["gridz"], materials=w["materials"],
                         boreholes=w["boreholes"], inlet_model=w["inlet_model"])
    ncell = cache.N
    dt = w["dt"]
    import ctypes
    s, cov = ctypes.c_int(), ctypes.c_int()
    _lib.check(L.gw_rock2_stages(cache.ctx, dt, 100, ctypes.byref(s), ctypes.byref(cov)))
    cache.set_field(w["T0"])
    if args.tiling >= 0:
        _lib.check(L.gw_set_tiling(cache.ctx, args.tiling))
    # warm-up (also builds the CUDA graphs and, for the overlapped step, times
    # its two launch orders)
    _lib.check(L.gw_step(cache.ctx, 0.0, dt, args.warmup, 100))
    # rock2 columns, 2 half steps, 2 x 3 pipe kernels, record; the overlapped
    # step splits the x-lines in three launches and ROCK2 in two (three when
    # the pipe columns go first)
    info = _lib.Info()
    _lib.check(L.gw_get_info(cache.ctx, ctypes.byref(info)))
    launches_per_step = (14 if info.step_order == 1 else 13) if info.overlap else 10
    if dist:
        dist.barrier()
    clocks = Clocks(local)
    _lib.check(L.gw_step(cache.ctx, args.warmup * dt, dt, args.steps, 100))
    ms = ctypes.c_double()
    _lib.check(L.gw_get_last_step_time(cache.ctx, ctypes.byref(ms)))
    ck = clocks.stop()
    t_ms, units = reduce_replicas(dist, ms.value, ncell * args.steps)
    value = units / (t_ms / 1e3) / 1e6

    # per-kernel timing for the roofline of the dominant kernel
    prof = (ctypes.c_double * len(_lib.KERNELS))()
    _lib.check(L.gw_profile_kernels(cache.ctx, dt, 3, prof))
    kms = dict(zip(_lib.KERNELS, list(prof)))
    wb = WORD[args.precision]
    ncol = cache.countxy_inner + cache.countxy_outer
    # compulsory bytes per launch: each fused field kernel reads and writes the
    # field once; the pipe pass reads and writes the pipe columns
    alg = {"rock2_columns": 2 * wb * ncell, "half_step_x": 2 * wb * ncell,
           "half_step_y": 2 * wb * ncell,
           "pipe": 2 * wb * ncol * cache.Nz + 2 * wb * ncol * cache.countz}
    per_step = {"rock2_columns": 1, "half_step_x": 1, "half_step_y": 1, "pipe": 2}
    share = {k: kms[k] * per_step[k] for k in kms}
    dom = max(share, key=share.get)
    peak, peak_kind = peaks()
    achieved = alg[dom] / (kms[dom] / 1e3) / 1e9
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "traffic_per_cell.json")
    if os.path.exists(tpath):
        tr = json.load(open(tpath)).get(args.precision, {}).get(dom)
        if tr is not None:
            traffic = tr * (ncol * cache.Nz if dom == "pipe" else ncell)

    # end to end through the public path with host buffers (pinned)
    e2e = None
    try:
        import torch
        pin = torch.empty(ncell, dtype=torch.float64, pin_memory=True).numpy()
        out_pin = torch.empty(ncell, dtype=torch.float64, pin_memory=True).numpy()
    except Exception:
        pin, out_pin = np.empty(ncell), np.empty(ncell)
    pin[:] = np.asfortranarray(w["T0"]).ravel(order="F")
    out_pin[:] = 0.0   # pages resident before the timed region
    series = np.zeros(args.steps * cache.N_bh)
    t0 = time.perf_counter()
    _lib.check(L.gw_set_field(cache.ctx, _lib.dptr(pin)))
    _lib.check(L.gw_step(cache.ctx, 0.0, dt, args.steps, 100))
    _lib.check(L.gw_get_outlet_series(cache.ctx, _lib.dptr(series), args.steps))
    _lib.check(L.gw_get_field(cache.ctx, _lib.dptr(out_pin)))
    e2e_ms, e2e_units = reduce_replicas(dist, (time.perf_counter() - t0) * 1e3, ncell * args.steps)
    e2e = {"value": e2e_units / (e2e_ms / 1e3) / 1e6, "unit": METRIC,
           "h2d_bytes_per_step": 8 * ncell / args.steps,
           "d2h_bytes_per_step": (8 * ncell + 8 * args.steps * cache.N_bh) / args.steps,
           "path": "gw_set_field + gw_step(K) + gw_get_outlet_series + gw_get_field, pinned host"}
    cache.close()
    other = None
    if not args.no_compare:
        oprec = "fp64" if args.precision == "mixed" else "mixed"
        oc = create_cache(backend=GB300(device=local, precision=oprec), gridx=w["gridx"],
                          gridy=w["gridy"], gridz=w["gridz"], materials=w["materials"],
                          boreholes=w["boreholes"], inlet_model=w["inlet_model"])
        oc.set_field(w["T0"])
        _lib.check(L.gw_step(oc.ctx, 0.0, dt, args.warmup, 100))
        _lib.check(L.gw_step(oc.ctx, args.warmup * dt, dt, args.steps, 100))
        oms = ctypes.c_double()
        _lib.check(L.gw_get_last_step_time(oc.ctx, ctypes.byref(oms)))
        oc.close()
        o_ms, o_units = reduce_replicas(dist, oms.value, ncell * args.steps)
        ov = o_units / (o_ms / 1e3) / 1e6
        other = {"precision": oprec, "value": ov, "ms_per_step": oms.value / args.steps,
                 "ratio_mixed_over_fp64": (value / ov) if args.precision == "mixed" else (ov / value)}
    if rank != 0:
        return
    cb = None
    if not args.no_cpu_baseline and world == 1:
        cb = cpu_baseline(w, args.cpu_sample_steps)
        cb = {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")}
    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if args.precision == "fp64" else "f32 (f64 outlet and energy balance)", "data": "synthetic",
        "config": {"workload": w["name"], "cells": ncell, "dt_s": dt, "rock2_stages": s.value,
                   "precision": args.precision, "l2": "inputs larger than L2 (field %.0f MB)"
                   % (ncell * 8 / 1e6), "parallelism": "replicas" if world > 1 else "single",
                   "half_step_tiling": int(info.tiling), "step_order": int(info.step_order)},
        "roofline": {"kernel": dom, "bound": "hbm", "achieved": achieved, "peak": peak,
                     "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "kernel_ms": kms,
                     "alg_bytes_per_launch": alg[dom],
                     "step_share": {k: share[k] / sum(share.values()) for k in share}},
        "compare": other,
        "cpu_baseline": cb, "e2e": e2e, "gpu_launches": launches_per_step * args.steps,
        "clocks": ck,
    }
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def run_accuracy(args):
    """Mixed vs FP64 on the same workload over NSTEPS steps: max |dT| of the
    final field, the largest outlet-temperature difference over all steps and
    the relative difference of the extracted heat."""
    from geothermalwells_gb300 import (GB300, ODEProblem, ROCK2, create_cache, eigen_estimator,
                                       rhs_diffusion_z, solve)
    w = workload(args.workload, args.dt)
    res = {}
    for prec in ("fp64", "mixed"):
        cache = create_cache(backend=GB300(precision=prec), gridx=w["gridx"], gridy=w["gridy"],
                             gridz=w["gridz"], materials=w["materials"],
                             boreholes=w["boreholes"], inlet_model=w["inlet_model"])
        prob = ODEProblem(rhs_diffusion_z, w["T0"], (0.0, args.accuracy * w["dt"]), cache)
        t0 = time.perf_counter()
        sol = solve(prob, ROCK2(max_stages=100, eigen_est=eigen_estimator), dt=w["dt"])
        res[prec] = (sol, time.perf_counter() - t0)
        cache.close()
    a, b = res["fp64"][0], res["mixed"][0]
    line = {"accuracy": {"workload": w["name"], "steps": args.accuracy, "dt_s": w["dt"],
                         "simulated_days": args.accuracy * w["dt"] / 86400.0,
                         "field_max_abs_dT_K": float(np.max(np.abs(b.u[-1] - a.u[-1]))),
                         "outlet_max_abs_err_K": float(np.max(np.abs(b.T_outlet - a.T_outlet))),
                         "outlet_final_fp64_C": float(a.T_outlet[-1, 0]),
                         "outlet_final_mixed_C": float(b.T_outlet[-1, 0]),
                         "energy_fp64_J": float(a.energy[0]), "energy_mixed_J": float(b.energy[0]),
                         "energy_rel_err": float(abs(b.energy[0] - a.energy[0]) / abs(a.energy[0])),
                         "wall_s": {"fp64": res["fp64"][1], "mixed": res["mixed"][1]},
                         "reference": "the FP64 GPU path (pinned to the FP64 oracle at 1e-10 in the parity tests)"}}
    print(json.dumps(line), flush=True)


def _gpu_solve(w, precision, nsteps, flags=0, T0=None):
    """Final field, outlet series, extracted heat and wall time of a fused
    GPU solve of nsteps steps (flags: GW_MIXED_* options of a mixed run)."""
    from geothermalwells_gb300 import (GB300, ODEProblem, ROCK2, _lib, create_cache, eigen_estimator,
                                       rhs_diffusion_z, solve)
    cache = create_cache(backend=GB300(precision=precision), gridx=w["gridx"], gridy=w["gridy"],
                         gridz=w["gridz"], materials=w["materials"], boreholes=w["boreholes"],
                         inlet_model=w["inlet_model"])
    if flags:
        _lib.check(_lib.load().gw_set_mixed_options(cache.ctx, flags))
    u0 = w["T0"] if T0 is None else T0
    t0 = time.perf_counter()
    sol = solve(ODEProblem(rhs_diffusion_z, u0, (0.0, nsteps * w["dt"]), cache),
                ROCK2(max_stages=100, eigen_est=eigen_estimator), dt=w["dt"], adaptive=False)
    wall = time.perf_counter() - t0
    cache.close()
    return sol.u[-1], sol.T_outlet, sol.energy, wall


def _oracle_solve(w, nsteps, T0=None):
    """The oracle's final field and outlet series (all host threads)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    from geothermalwells_gb300 import rock2
    O.set_threads(os.cpu_count() or 1)
    orc = O.Oracle(w["gridx"], w["gridy"], w["gridz"], w["boreholes"], w["materials"], w["inlet_model"])
    s, _ = rock2.choose_stages(w["dt"], orc.eigen_estimate())
    u = (w["T0"] if T0 is None else T0).copy(order="F")
    t0 = time.perf_counter()
    out = orc.simulate(u, 0.0, w["dt"], nsteps, s, rock2.coefficients(s))
    wall = time.perf_counter() - t0
    orc.close()
    return u, out, wall


def _energy_from_outlet(w, out):
    """sum over steps of mdot c_w (T_out - T_in) dt per borehole, the balance
    gw_get_energy keeps, from an outlet series (constant or heat-exchanger inlet)."""
    from geothermalwells_gb300.physics import RHO_WATER
    c_w = w["materials"].rho_c_water / RHO_WATER
    im = w["inlet_model"]
    mdot = np.array([b.mdot for b in w["boreholes"]])
    t_in = (im.param if im.kind == 0 else out - im.param)
    return np.sum(mdot * c_w * (out - t_in) * w["dt"], axis=0)


def _errors(u, out, energy, u_ref, out_ref, energy_ref):
    return {"field_max_abs_dT_K": float(np.max(np.abs(u - u_ref))),
            "field_max_rel": float(np.max(np.abs(u - u_ref)) / np.max(np.abs(u_ref))),
            "outlet_max_abs_err_K": float(np.max(np.abs(out - out_ref))),
            "heat_rel_err": float(np.max(np.abs(energy - energy_ref) / np.abs(energy_ref)))}


def run_accuracy_suite(args):
    """Errors of the GPU paths on every configuration, against the FP64 oracle
    (the reference's algorithm in C) where it runs in seconds, else against
    the FP64 GPU path (itself pinned to the oracle at 1e-10):

      cfg1 2 mm well, 1 simulated hour (60 steps of 60 s), oracle in full;
      cfg2 large well, 24-step window of the 300 s steps against the oracle,
           and 30 days (12,960 steps of 200 s) mixed against FP64;
      cfg4 four ensemble designs, a 12-step window against the oracle and
           5 days (720 steps of 600 s) mixed against FP64;
      cfg5 the adjoint workload's forward solve (22 layers, 3024 steps of
           200 s), mixed against FP64.

    Each mixed run is repeated with the two FP64 options of the mixed step
    (GW_MIXED_ROCK2_F64, GW_MIXED_REFINE) and their wall times."""
    from geothermalwells_gb300 import _lib
    from geothermalwells_gb300 import workloads as W
    variants = {"mixed": 0, "mixed+rock2_f64": _lib.GW_MIXED_ROCK2_F64,
                "mixed+refine": _lib.GW_MIXED_REFINE,
                "mixed+both": _lib.GW_MIXED_ROCK2_F64 | _lib.GW_MIXED_REFINE}
    res = {}
    only = set(args.suite.split(",")) if args.suite else None

    def against_oracle(name, w, nsteps, T0=None):
        u_r, o_r, wall_r = _oracle_solve(w, nsteps, T0)
        e_r = _energy_from_outlet(w, o_r)
        entry = {"workload": w["name"], "cells": int(np.prod(u_r.shape)), "steps": nsteps, "dt_s": w["dt"],
                 "reference": "FP64 oracle", "oracle_wall_s": wall_r}
        u, o, e, wall = _gpu_solve(w, "fp64", nsteps, T0=T0)
        entry["fp64"] = dict(_errors(u, o, e, u_r, o_r, e_r), wall_s=wall)
        for v, f in variants.items():
            u, o, e, wall = _gpu_solve(w, "mixed", nsteps, f, T0=T0)
            entry[v] = dict(_errors(u, o, e, u_r, o_r, e_r), wall_s=wall)
        res[name] = entry
        print(json.dumps({name: entry}), flush=True)

    def against_fp64(name, w, nsteps, T0=None, vlist=None):
        u_r, o_r, e_r, wall_r = _gpu_solve(w, "fp64", nsteps, T0=T0)
        entry = {"workload": w["name"], "cells": int(np.prod(u_r.shape)), "steps": nsteps, "dt_s": w["dt"],
                 "simulated_days": nsteps * w["dt"] / 86400.0, "reference": "FP64 GPU path",
                 "fp64_wall_s": wall_r}
        for v in (vlist or variants):
            u, o, e, wall = _gpu_solve(w, "mixed", nsteps, variants[v], T0=T0)
            entry[v] = dict(_errors(u, o, e, u_r, o_r, e_r), wall_s=wall)
        res[name] = entry
        print(json.dumps({name: entry}), flush=True)

    if not only or "cfg1" in only:
        against_oracle("cfg1_2mm_1h", W.single_well_2mm(), 60)
    if not only or "cfg2" in only:
        w = W.single_well_large()
        against_oracle("cfg2_large_24steps", w, 24)
        against_fp64("cfg2_large_30days", dict(w, dt=200.0), 12960)
    if not only or "cfg4" in only:
        designs = W.ensemble()
        for q in (0, 1, 2, 3):
            d = dict(designs[q], dt=600.0, name="ensemble_design_%d" % q)
            T0 = W.initial_field(d)
            against_oracle("cfg4_design%d_12steps" % q, dict(d, T0=T0), 12)
            against_fp64("cfg4_design%d_5days" % q, dict(d, T0=T0), 720, vlist=["mixed", "mixed+both"])
    if not only or "cfg5" in only:
        w = W.adjoint_well()
        against_fp64("cfg5_adjoint_forward_7days", w, w["nsteps"])
    print(json.dumps({"accuracy_suite": res}), flush=True)


def run_thomas(args):
    """Batched tridiagonal microbenchmark: 262,144 seeded systems, lengths
    U[32, 1024]; algorithmic traffic 5 words per unknown (a, b, c, d in, x
    out).  Inputs (5.5 GB) exceed L2."""
    import torch
    from geothermalwells_gb300 import _lib
    from geothermalwells_gb300 import workloads as W
    L = _lib.load()
    w = W.tridiagonal_batch()
    prec = _lib.GW_PREC_MIXED if args.precision == "mixed" else _lib.GW_PREC_FP64
    dev = {k: torch.from_numpy(np.ascontiguousarray(w[k])).cuda() for k in "abcd"}
    goff = torch.from_numpy(w["group_off"].astype(np.int64)).cuda()
    glen = torch.from_numpy(w["group_len"].astype(np.int32)).cuda()
    x = torch.zeros(w["n"], dtype=torch.float64, device="cuda")
    scratch = torch.zeros((w["n"] * 12 + 7) // 8, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream()

    def solve():
        _lib.check(L.gw_tridiag_batch(prec, w["ngroups"], goff.data_ptr(), glen.data_ptr(),
                                      dev["a"].data_ptr(), dev["b"].data_ptr(), dev["c"].data_ptr(),
                                      dev["d"].data_ptr(), x.data_ptr(), scratch.data_ptr(), w["n"],
                                      stream.cuda_stream))
    for _ in range(args.warmup):
        solve()
    torch.cuda.synchronize()
    clocks = Clocks(0)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        solve()
    e1.record(stream)
    torch.cuda.synchronize()
    ck = clocks.stop()
    ms = e0.elapsed_time(e1) / args.steps
    # residuals in double on the device: r = d - (a x_{r-1} + b x_r + c x_{r+1})
    r = dev["d"] - (dev["a"] * torch.roll(x, 32) + dev["b"] * x + dev["c"] * torch.roll(x, -32))
    res = float(r.abs().max() / dev["d"].abs().max())
    unknowns = w["unknowns"]
    alg = 5 * 8 * unknowns
    peak, peak_kind = peaks()
    achieved = alg / (ms / 1e3) / 1e9
    line = {"metric": "Munknowns/s", "value": unknowns / (ms / 1e3) / 1e6, "unit": "Munknowns/s",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if prec == _lib.GW_PREC_FP64 else "f32+f64refine", "data": "synthetic",
            "config": {"workload": w["name"], "systems": 262144, "unknowns": unknowns,
                       "stored_rows_x32": w["n"], "l2": "inputs larger than L2 (5.5 GB)"},
            "residual_max_rel": res,
            "roofline": {"kernel": "k_tri_f64" if prec == _lib.GW_PREC_FP64 else "k_tri_mix1+2",
                         "bound": "hbm", "achieved": achieved, "peak": peak, "peak_kind": peak_kind,
                         "unit": "GB/s", "frac": achieved / peak, "traffic": None,
                         "alg_bytes_per_launch": alg},
            "gpu_launches": args.steps * (1 if prec == _lib.GW_PREC_FP64 else 2), "clocks": ck}
    print(json.dumps(line), flush=True)


def run_ensemble(args):
    """64 heterogeneous 3 x 3 well-array designs (about 1.5e9 cells in all),
    dt 3600 s, advanced together (one graph launch per step); the autotuned
    half-step tiling against the fixed default tiling."""
    from geothermalwells_gb300 import workloads as W
    from geothermalwells_gb300.ensemble import Ensemble, TILINGS
    t0 = time.perf_counter()
    designs = W.ensemble()
    t1 = time.perf_counter()
    prec = args.precision
    ens = Ensemble(designs, precision=prec, initial_gradient=W.initial_gradient)
    setup_s = time.perf_counter() - t1
    generate_s = t1 - t0
    # dt 600 s: at the configured 3600 s the reference scheme itself breaks
    # down for part of the designs (departure points above the surface at
    # high flow, divergence on fine z grids); the work per step is the same
    dt = args.dt if args.dt > 0 else 600.0
    if args.tiling >= 0:   # one tiling for every design, no autotuning
        ens.set_tiling(args.tiling)
        choice = [args.tiling] * len(designs)
    else:
        choice = ens.autotune(dt, reps=2)
    ens.step(dt, args.warmup)
    clocks = Clocks(0)
    ms_tuned = ens.step(dt, args.steps)
    ck = clocks.stop()
    ens.set_tiling(0)
    ens.step(dt, 1)
    ms_fixed = ens.step(dt, args.steps)
    cells = ens.cells
    finite = all(np.isfinite(ens.outlet_series(d, args.steps)).all() for d in range(len(designs)))
    value = cells * args.steps / (ms_tuned / 1e3) / 1e6
    wb = WORD[prec]
    peak, peak_kind = peaks()
    achieved = 6 * wb * cells * args.steps / (ms_tuned / 1e3) / 1e9   # 3 field passes of 2 words per step
    line = {"metric": METRIC, "value": value, "unit": METRIC, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_tuned / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if prec == "fp64" else "f32 (f64 outlet and energy balance)", "data": "synthetic",
            "config": {"workload": "ensemble_64_designs_3x3_arrays", "designs": len(designs),
                       "cells": cells, "dt_s": dt, "generate_s": generate_s, "setup_s": setup_s,
                       "grid_range": [min(len(d["gridx"]) for d in designs),
                                      max(len(d["gridx"]) for d in designs),
                                      min(len(d["gridz"]) for d in designs),
                                      max(len(d["gridz"]) for d in designs)],
                       "l2": "inputs larger than L2"},
            "tiling": {"autotuned_ms_per_step": ms_tuned / args.steps,
                       "fixed_ms_per_step": ms_fixed / args.steps,
                       "fixed": list(TILINGS[0]),
                       "chosen_histogram": {str(list(TILINGS[t])): choice.count(t) for t in set(choice)}},
            "roofline": {"kernel": "whole step (3 field passes)", "bound": "hbm", "achieved": achieved,
                         "peak": peak, "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": None},
            "outlet_finite": finite, "clocks": ck}
    print(json.dumps(line), flush=True)
    ens.close()


def run_adjoint(args):
    """Gradient workload: d(extracted heat over 7 days)/d(22 rock layer
    conductivities, flow rate, inlet temperature) on the 205 x 205 x 2002 well
    (3024 steps of 200 s), checkpoints every 64 steps, in the selected
    precision (mixed: float adjoint fields over the mixed step), with the FP64
    adjoint beside it (--no-compare skips it).  Reports the adjoint's device
    time as a multiple of one forward solve of the same precision, the device
    memory it holds, and central differences (h = 1e-4 relative) of the FP64
    forward solve: --fd some checks the largest and the median layer
    gradient, the flow rate, the inlet temperature and one random direction
    through all 24 parameters; --fd all checks every parameter.  Each check
    takes central differences at h = 1e-4 and h / 2 (relative) and their
    Richardson extrapolation; the adjoint must be within 1e-4 of the latter
    (plus the differences' rounding floor, 16 eps |J| / h)."""
    from geothermalwells_gb300 import _lib
    from geothermalwells_gb300 import adjoint as A
    from geothermalwells_gb300 import workloads as W
    L = _lib.load()
    w = W.adjoint_well()
    dt = args.dt if args.dt > 0 else w["dt"]
    nsteps = args.adjoint_steps or w["nsteps"]
    K = w["checkpoint_every"]

    def design(prec):
        return A.Design(w["gridx"], w["gridy"], w["gridz"], w["boreholes"], w["materials"],
                        w["inlet_model"], w["T0"], dt, nsteps, checkpoint_every=K, precision=prec)

    p0 = np.concatenate([w["materials"].k_rock_layers, [b.mdot for b in w["boreholes"]],
                         [w["inlet_model"].param]])
    nl = len(w["materials"].k_rock_layers)

    def forward(p, prec="fp64"):
        c = design(prec).cache(p[:nl], p[nl:-1], p[-1])
        try:
            c.set_field(w["T0"])
            _lib.check(L.gw_reset_energy(c.ctx))
            _lib.check(L.gw_step(c.ctx, 0.0, dt, nsteps, 100))
            E = np.zeros(c.N_bh)
            _lib.check(L.gw_get_energy(c.ctx, _lib.dptr(E)))
            ms = ctypes_double()
            _lib.check(L.gw_get_last_step_time(c.ctx, ms))
            return float(E.sum()), ms.value
        finally:
            c.close()

    def run_adj(prec):
        cache = design(prec).cache(p0[:nl], p0[nl:-1], p0[-1])
        cache.set_field(w["T0"])
        _lib.check(L.gw_step(cache.ctx, 0.0, dt, 4, 100))     # warm-up (graph capture, tables)
        J_fwd, fwd_ms = forward(p0, prec)
        clocks = Clocks(0)
        r = A.adjoint(cache, w["T0"], dt, nsteps, checkpoint_every=K)
        ck = clocks.stop()
        cache.close()
        return r, J_fwd, fwd_ms, ck

    prec = args.precision
    r, J_fwd, fwd_ms, ck = run_adj(prec)
    g = r.grad
    g64 = None
    if prec != "fp64" and not args.no_compare:
        r64, J64, fwd64_ms, _ = run_adj("fp64")
        g64 = r64.grad
    J_ref = J_fwd if g64 is None else J64
    if args.fd == "all":
        idx = list(range(len(p0)))
    elif args.fd == "some":
        order = np.argsort(np.abs(g[:nl]))
        idx = sorted({int(order[-1]), int(order[nl // 2]), nl, len(p0) - 1})
    else:
        idx = []
    eps = np.finfo(np.float64).eps

    def central(d, hs):
        """Central difference of the FP64 J along p0 * (1 + hs d)."""
        return (forward(p0 * (1 + hs * d))[0] - forward(p0 * (1 - hs * d))[0]) / (2 * hs)

    def check(d):
        """Directional derivative g . (p0 * d) against central differences at
        h = 1e-4 and h / 2 and their Richardson extrapolation (which removes
        the h^2 term: J is strongly curved in the flow rate, whose h = 1e-4
        difference alone carries a ~1e-3 truncation error)."""
        f1, f2 = central(d, 1e-4), central(d, 5e-5)
        rich = (4 * f2 - f1) / 3
        floor = 16 * eps * abs(J_ref) / 1e-4
        out = {"fd_h": f1, "fd_h2": f2, "fd_richardson": rich}
        for tag, gg in (("adjoint", g), ("adjoint_fp64", g64)):
            if gg is None:
                continue
            a = float(np.dot(gg, p0 * d))
            out[tag] = a
            out["rel_err_" + tag] = abs(a - rich) / abs(rich) if rich else None
            out["ok_" + tag] = bool(abs(a - rich) <= 1e-4 * abs(rich) + floor)
        return out

    checks = {}
    for i in idx:
        d = np.zeros(len(p0))
        d[i] = 1.0
        checks[str(i)] = check(d)
    if args.fd != "none":
        checks["direction"] = check(np.random.default_rng(7).choice([-1.0, 1.0], len(p0)))
    ok = all(v["ok_adjoint"] for v in checks.values())
    finite = bool(np.isfinite(r.objective) and np.all(np.isfinite(g)))
    cells = len(w["gridx"]) * len(w["gridy"]) * len(w["gridz"])
    adj_ms = r.forward_ms + r.reverse_ms
    compare = None
    if g64 is not None:
        rel = np.abs(g - g64) / np.maximum(np.abs(g64), 1e-300)
        big = np.abs(g64) > 1e-6 * np.max(np.abs(g64))
        compare = {"precision": "fp64", "grad": [float(v) for v in g64],
                   "objective_J": r64.objective,
                   "adjoint_ms": r64.forward_ms + r64.reverse_ms, "forward_ms": fwd64_ms,
                   "max_rel_diff_mixed_vs_fp64": float(np.max(rel[big])),
                   "peak_device_gb": r64.peak_bytes / 1e9}
    line = {"metric": "adjoint cost (multiple of one forward solve)", "value": adj_ms / fwd_ms,
            "unit": "x", "n_gpus": 1, "steps": nsteps, "higher_is_better": False,
            "vs_baseline": None, "dtype": "f64" if prec == "fp64" else "f32 (f64 outlet and energy balance)", "data": "synthetic",
            "config": {"workload": w["name"], "cells": cells, "dt_s": dt, "checkpoint_every": K,
                       "checkpoints": r.checkpoints, "stages": r.stages, "precision": prec,
                       "params": "k_rock_layers[22], mdot, T_inlet"},
            "forward_ms": fwd_ms, "adjoint_ms": adj_ms, "adjoint_forward_sweep_ms": r.forward_ms,
            "adjoint_reverse_ms": r.reverse_ms,
            "forward_mcell_steps_per_s": cells * nsteps / (fwd_ms / 1e3) / 1e6,
            "peak_device_gb": r.peak_bytes / 1e9, "objective_J": r.objective,
            "objective_forward_J": J_fwd, "grad": [float(v) for v in g],
            "fd_check": {"h_rel": 1e-4, "of": "FP64 forward solve",
                         "derivatives": "d J / d ln p (p * dJ/dp)", "checks": checks,
                         "max_rel_err_richardson": max([v["rel_err_adjoint"] for v in checks.values()
                                                        if v.get("rel_err_adjoint") is not None], default=None),
                         "within_1e-4": bool(ok)},
            "compare": compare, "finite": finite, "clocks": ck}
    print(json.dumps(line), flush=True)


def ctypes_double():
    import ctypes
    return ctypes.c_double()


def main():
    args = parse()
    if args.workload == "adjoint":
        run_adjoint(args)
        return
    if args.workload == "ensemble":
        run_ensemble(args)
        return
    if args.workload == "thomas":
        run_thomas(args)
        return
    if args.accuracy_suite:
        run_accuracy_suite(args)
        return
    if args.accuracy:
        run_accuracy(args)
        return
    if args.kernels:
        run_kernels(args)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
