"""Benchmark of the MPDATA advection step on one GB300 (or N replicas).

Workload (the headline configuration): 512x512x128 periodic grid, FP64,
infinite-gauge MPDATA with iord=3 and the nonoscillatory limiter, velocity
predictor active, time-varying deformational flow with max Courant 0.5,
psi = seeded uniform noise in [1,2] plus two Gaussian cones.  One step is:
  1. the A-grid Courant numbers at t_n (the flow is separable in time:
     pattern * cos(pi t/T); written on the device by torch, standing in for
     the dynamics that would supply them),
  2. the velocity predictor (A grid at n and n-1 -> C grid at n+1/2),
  3. one MPDATA step on psi.
Metric: Gcell-steps/s (interior cells x steps / second), whole job.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--precision 64|32] [--grid NX NY NZ] [--no-cpu-baseline]

--impl reference times the CPU oracle (the C++ restatement of the
reference's Fortran path; the Fortran build itself is unavailable: no Fortran
compiler on either machine) on the host cores, on a bounded slab of the same
workload.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "MPDATA Gcell-steps/s fwd & adjoint, 1×GB300, % HBM roofline, err vs FP64"
UNIT = "Gcell-steps/s"

# Algorithmic (compulsory) device bytes per cell per launch of each stage:
# every array a kernel must read or write, once.  Units: elements per cell.
#   upwind   r psi u1..3 h rhr                w xant hinv hmx hmy hmz   11
#   pairs    r xant                           w Sx Sy Sz                 4 (FP64 gauge only)
#   pseudo   r xant a1..3 hm1..3 (+Sx Sy Sz)  w v1..3 (+f1..3 std)      10, 13 FP64 gauge (13 std)
#   bounds   r xant psi|mx,mn h rhr F1..3     w q cp cn (+mx mn)        10..13
#   limit    r cp cn v1..3 (+xant q)          w w1..3 (+f1..3)          8 (13 std)
#   update   r q rhr h|hinv F1..3             w out                     7
#   predictor level  r o0 x3 o2 x3 h  w o1 x3 o2 x3 (the level roll)     13
#   predictor cgrid  r o1 x3          w u1..3                             6
# The fused single-precision step (periodic gauge grids):
#   fused_upwind_pseudo  r psi u1..3 h rhr     w x_in xant v1..3           11
#   fused_pseudo         r x w1..3 h           w v1..3                      8
#   fused_limit_update   r x x_in|mx,mn v1..3 h rhr  w x (w1..3) (mx mn)  11..15
def stage_elems(stage, gauge, iord, precision=64):
    """Compulsory fields read + written per cell by one launch of a stage
    (interior cells, each field once; ncu DRAM bytes agree within 4%)."""
    keep = iord > 2
    pairs = gauge and precision == 64                 # FP64 gauge: pair sums precomputed
    if stage == "upwind":
        return 11.0                                   # psi,u1..3,h,rhr -> xant,1/h,hmx,hmy,hmz
    if stage == "pair_sums":
        return 10.0                                   # xant,a1..3 -> Sx,Sy,Sz, velocity pairs C1..C3
    if stage == "pseudo_velocity":
        if not gauge:
            return 13.0                               # xant,a1..3,hm1..3 -> v1..3,f1..3
        return 16.0 if pairs else 10.0                # xant,a1..3,hm1..3 (+Sx,Sy,Sz,C1..C3) -> v1..3
    if stage == "limiter_bounds":
        first = 10.0 + (2.0 if keep else 0.0)         # xant,rhr,psi,F1..3,h -> q,cp,cn (+mx,mn kept)
        later = 13.0                                  # xant,rhr,mx,mn,F1..3,h -> q,mx,mn,cp,cn
        n = max(iord - 1, 1)
        return (first + later * (n - 1)) / n
    if stage == "limited_flux":
        return 8.0 if gauge else 13.0                 # cp,cn,v1..3 -> w1..3 (+xant,q -> f1..3 std)
    if stage == "corrective_update":
        return 7.0                                    # w1..3 (f1..3),q,h (1/h),rhr -> psi
    if stage == "predictor_level":
        return 13.0
    if stage == "predictor_cgrid":
        return 6.0
    if stage == "fused_upwind_pseudo":
        return 11.0
    if stage == "fused_pseudo":
        return 8.0
    if stage == "fused_limit_update":
        n = max(iord - 1, 1)                          # passes: first, middle..., last
        first = 7.0 + 1.0 + (3.0 + 2.0 if n > 1 else 0.0)      # + x_out, w1..3 and mx,mn when more follow
        later = 8.0 + 1.0 + 2.0 + 3.0                            # mx,mn in; x_out, mx,mn, w1..3 out
        last = 8.0 + 1.0 + 2.0                                   # mx,mn in; psi, mx,mn out
        if n == 1:
            return first
        return (first + later * (n - 2) + last) / n
    return 2.0


# Compulsory DRAM bytes per interior cell of one whole step (read psi, h, rhr
# and the six A-grid momenta of the two time levels the predictor needs;
# write psi), per element size: the floor of any implementation of the step.
STEP_COMPULSORY_ELEMS = 11.0


# DRAM bytes and FP64 instructions per cell of the dominant kernel (k_pseudo,
# gauge form), from an ncu capture of every stage kernel at 384x384x64
# (dram__bytes_read.sum + dram__bytes_write.sum, and
# smsp__sass_thread_inst_executed_op_{dadd,dmul,dfma}_pred_on.sum, per cell).
# Both grow in proportion to the cells of a launch.
NCU_PSEUDO = {64: {"dram_bytes_per_cell": 127.8, "fp64_inst_per_cell": 39.0},
              32: {"dram_bytes_per_cell": 38.2, "fp64_inst_per_cell": 0.0}}
# The same for the dominant fused single-precision kernel (the first pass's
# fused_limit_update) at 384x384x64: DRAM bytes and issued warp instructions
# per cell (smsp__inst_executed.sum * 32 / cells) and the issue-active share.
NCU_FUSED_LIMIT = {"dram_bytes_per_cell": 50.0, "inst_per_cell": 577.0, "issue_active": 0.748}
# GB300 issues 2 FP64 instructions per SM per clock (1.25 TFLOP/s nominal FMA).
FP64_INST_PER_SM_CLK = 2.0
# FP64 flops per cell of one launch of each stage (DADD and DMUL 1, DFMA 2),
# counted by ncu (smsp__sass_thread_inst_executed_op_{dadd,dmul,dfma}_pred_on.sum)
# on the deformational flow at unit density, 384x384x64, gauge iord=3.
FP64_FLOPS_PER_CELL = {"upwind": 12.4, "pair_sums": 6.0, "pseudo_velocity": 39.0, "limiter_bounds": 11.7,
                       "limited_flux": 3.0, "corrective_update": 6.2, "predictor_level": 9.0,
                       "predictor_cgrid": 3.0}
# FP32 arithmetic instructions (FADD, FMUL, FFMA) per cell of one launch of
# each fused single-precision kernel, counted by ncu
# (smsp__sass_thread_inst_executed_op_{fadd,fmul,ffma}_pred_on) on the
# deformational flow at unit density, 384x384x64; the predictor's from its
# source (per component, three adds and the product by 0.5 of the n+1/2
# momenta, one add and one product by 0.5 of the C-grid average).
FP32_INST_PER_CELL = {"fused_upwind_pseudo": 102.5, "fused_pseudo": 90.0, "fused_limit_update": 52.0,
                      "predictor_level": 12.0, "predictor_cgrid": 6.0}
FP32_LANES_PER_SM_CLK = 128.0
HBM_NOMINAL_GBS = 7900.0  # GB300 HBM3e, nominal


def step_roofs(stages, steps, ms_step, cells, precision, peak, sm_mhz, sms):
    """Step-level roofline: the compulsory bytes of the whole step against
    HBM, and the attainable floor max(HBM time, arithmetic-pipe time) with
    the pipe that binds each precision on GB300 (FP64: 2 instructions per SM
    per clock; FP32: 128 lanes per SM per clock) at the sampled SM clock."""
    elem = 8 if precision == 64 else 4
    comp = STEP_COMPULSORY_ELEMS * elem
    t = ms_step * 1e-3
    t_hbm = comp * cells / (peak * 1e9)
    if precision == 64:
        inst = sum(FP64_FLOPS_PER_CELL.get(k, 0.0) * v[1] for k, v in stages.items()) / steps
        rate, pipe = FP64_INST_PER_SM_CLK * sms * sm_mhz * 1e6, "fp64_pipe"
    else:
        inst = sum(FP32_INST_PER_CELL.get(k, 0.0) * v[1] for k, v in stages.items()) / steps
        rate, pipe = FP32_LANES_PER_SM_CLK * sms * sm_mhz * 1e6, "fp32_pipe"
    t_pipe = inst * cells / rate
    lib_ms = sum(v[0] for v in stages.values()) / steps
    return {"compulsory_bytes_per_cell": comp,
            "step_compulsory_frac": round(t_hbm / t, 4),
            "arith_inst_per_cell": round(inst, 1),
            "attainable_roof": "hbm" if t_hbm >= t_pipe else pipe,
            "attainable_ms_per_step": round(max(t_hbm, t_pipe) * 1e3, 4),
            "step_attainable_frac": round(max(t_hbm, t_pipe) / t, 4),
            "library_ms_per_step": round(lib_ms, 4),
            "note": "compulsory: read psi, h, rhr and the six A-grid momenta, write psi; attainable: "
                    "max(compulsory bytes / HBM peak, arithmetic instructions / %s rate); "
                    "library_ms_per_step: predictor + step kernels alone (profiled pass)" % pipe}


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            p = json.load(fh)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled during the timed region."""

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        import tempfile
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.fh.close()

    def summary(self):
        if self.proc is None or not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as fh:
            for line in fh:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    smax.append(float(parts[2]))
                except ValueError:
                    continue
                for n, v in zip(names, parts[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(n)
        os.remove(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None, "samples": len(sm),
                "reasons": sorted(reasons)}


def dist_init(gpus):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
        dist.init_process_group(backend=backend)
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, ws):
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if torch.cuda.is_available() else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# --------------------------------------------------------------------------
# the workload
# --------------------------------------------------------------------------

def agrid_patterns(nx, ny, nz, courant=0.5):
    """Spatial A-grid Courant-number patterns of the deformational flow (at
    t=0); u and v scale with cos(pi t/T), w is steady."""
    from advectionhpctester_gb300 import workloads as W
    return W.deformational_agrid(nx, ny, nz, 0.0, 1.0, courant)


def time_factor(step, T):
    return math.cos(math.pi * step / T)


def make_state(nx, ny, nz, dtype_np, seed=20261203, T=200.0):
    """Host arrays (Fortran layout, ih=1) of the workload."""
    from advectionhpctester_gb300 import workloads as W
    f = W.deformational(nx, ny, nz, 1, 0.5, seed, np.float64, nsteps=int(T))
    su, sv, sw = agrid_patterns(nx, ny, nz)
    sh = f.x.shape
    pats = []
    for s in (su, sv, sw):
        a = W.zeros(sh)
        W.interior(a)[...] = s
        pats.append(a.astype(dtype_np, order="F"))
    return f.astype(dtype_np), pats


class GpuArm:
    def __init__(self, nx, ny, nz, precision, T=200.0, host=None):
        import torch
        from advectionhpctester_gb300 import mpdata as M
        self.torch, self.M = torch, M
        self.nx, self.ny, self.nz, self.T = nx, ny, nz, T
        dnp = np.float64 if precision == 64 else np.float32
        self.tdtype = torch.float64 if precision == 64 else torch.float32
        f, pats = host if host is not None else make_state(nx, ny, nz, np.float64, T=T)
        f = f.astype(dnp) if f.dtype != dnp else f
        pats = [p.astype(dnp, order="F") for p in pats]
        self.host = f
        self.pats_host = pats
        dv = lambda a: M.fortran_device(a, dtype=dnp)
        self.psi, self.u1, self.u2, self.u3 = dv(f.x), dv(f.u1), dv(f.u2), dv(f.u3)
        self.h, self.rhr = dv(f.h), dv(f.rhr)
        self.pats = [dv(p) for p in pats]
        lev = f.x.shape + (3,)
        self.o = [M.fortran_empty(lev, self.tdtype) for _ in range(3)]
        # level 2 = momenta at n-1 times h (h = 1)
        for c in range(3):
            fac = time_factor(-1, T) if c < 2 else 1.0
            self.o[c][..., 2].copy_(self.pats[c] * fac)
        self.ws = M.Workspace(nx, ny, nz, 1, 1, 1, 1, iord=3, nonos=1, gauge=1, precision=precision)

    def dynamics(self, n):
        """A-grid Courant numbers at t_n into level 0 (stand-in for the dynamics)."""
        fac = time_factor(n, self.T)
        for c in range(3):
            self.torch.mul(self.pats[c], fac if c < 2 else 1.0, out=self.o[c][..., 0])

    def dynamics_from(self, n, pats):
        fac = time_factor(n, self.T)
        for c in range(3):
            self.torch.mul(pats[c], fac if c < 2 else 1.0, out=self.o[c][..., 0])

    def step(self, n):
        self.dynamics(n)
        self.ws.velprd(self.o[0], self.o[1], self.o[2], self.h, 1.0, 1.0, 1.0, 1.0, 1.0,
                       self.u1, self.u2, self.u3)
        self.ws.step(self.psi, self.u1, self.u2, self.u3, self.h, self.rhr)

    def step_on(self, n, b):
        """One step on the buffer set b (psi, pats, h, rhr), current stream."""
        self.dynamics_from(n, b["pats"])
        self.ws.velprd(self.o[0], self.o[1], self.o[2], b["h"], 1.0, 1.0, 1.0, 1.0, 1.0,
                       self.u1, self.u2, self.u3)
        self.ws.step(b["psi"], self.u1, self.u2, self.u3, b["h"], b["rhr"])


def run_ours(args, ws, rank, local):
    import torch
    from advectionhpctester_gb300 import _native, mpdata as M
    _native.load(build_if_missing=True)
    torch.cuda.set_device(local)
    nx, ny, nz = args.grid
    cells = nx * ny * nz
    host = make_state(nx, ny, nz, np.float64)
    arm = GpuArm(nx, ny, nz, args.precision, host=host)
    stream = torch.cuda.current_stream()
    mass0 = M.mass(arm.psi, arm.h)
    for n in range(args.warmup):
        arm.step(n)
    torch.cuda.synchronize()
    # timed region: inputs (268 MB per FP64 field) exceed the 129 MB L2, no flush needed
    l0 = M.launch_count()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier(ws)
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        e0.record(stream)
        for n in range(args.warmup, args.warmup + args.steps):
            arm.step(n)
        e1.record(stream)
        torch.cuda.synchronize()
    barrier(ws)
    launches = M.launch_count() - l0
    ms = e0.elapsed_time(e1)
    ms_max = max_over_ranks(ms, ws)
    clocks = clk.summary()
    # per-stage kernel times from a separate profiled pass (event pairs around
    # every launch), so that the timed region above carries no events
    stages = profiled_stages(arm, args.warmup + args.steps, args.steps)
    value = ws * cells * args.steps / (ms_max * 1e-3) / 1e9

    # roofline of the dominant kernel
    peak, peak_kind = load_peaks()
    elem = 8 if args.precision == 64 else 4
    dom = max(stages.items(), key=lambda kv: kv[1][0])
    name, (tot_ms, nl) = dom
    avg_ms = tot_ms / max(nl, 1)
    alg_bytes = stage_elems(name, True, 3, args.precision) * elem * cells
    achieved = alg_bytes / (avg_ms * 1e-3) / 1e9
    ncu = NCU_PSEUDO[args.precision] if name == "pseudo_velocity" else None
    traffic = int(ncu["dram_bytes_per_cell"] * cells) if ncu else None
    roof = {"bound": "hbm", "kernel": name, "achieved": round(achieved, 1), "peak": peak,
            "unit": "GB/s", "frac": round(achieved / peak, 4), "traffic": traffic,
            "frac_nominal": round(achieved / HBM_NOMINAL_GBS, 4),
            "peak_source": peak_kind, "alg_bytes_per_launch": int(alg_bytes),
            "avg_launch_ms": round(avg_ms, 4),
            "traffic_source": "ncu DRAM bytes per cell of this kernel at 384x384x64, scaled by cells"}
    sms = torch.cuda.get_device_properties(local).multi_processor_count
    roof.update(step_roofs(stages, args.steps, ms_max / args.steps, cells, args.precision, peak,
                           clocks.get("sm_mhz") or clocks.get("sm_max_mhz") or 2070.0, sms))
    if args.precision == 64 and ncu:
        mhz = clocks.get("sm_max_mhz") or 2070.0
        fp64_peak = FP64_INST_PER_SM_CLK * sms * mhz * 1e6 / 1e9
        fp64_ach = ncu["fp64_inst_per_cell"] * cells / (avg_ms * 1e-3) / 1e9
        step_flops = sum(FP64_FLOPS_PER_CELL.get(k, 0.0) * v[1] for k, v in stages.items()) / args.steps
        roof["fp64_pipe"] = {"achieved": round(fp64_ach, 1), "peak": round(fp64_peak, 1),
                             "unit": "G FP64 inst/s", "frac": round(fp64_ach / fp64_peak, 4),
                             "inst_per_cell": ncu["fp64_inst_per_cell"],
                             "step_fp64_flops_per_cell": round(step_flops, 1),
                             "step_achieved_gflops": round(step_flops * value, 1),
                             "note": "the binding roof: 2 FP64 instructions per SM per clock at the "
                                     "sampled maximum SM clock; DRAM runs at the hbm frac"}
    stage_json = {k: {"ms_total": round(v[0], 3), "launches": int(v[1]),
                      "share": round(v[0] / max(sum(t for t, _ in stages.values()), 1e-9), 4)}
                  for k, v in stages.items() if v[1]}
    step_alg = sum(stage_elems(k, True, 3, args.precision) * elem * cells * v[1]
                   for k, v in stages.items()) / args.steps
    result = dict(metric=METRIC, value=round(value, 4), unit=UNIT, n_gpus=ws, steps=args.steps,
                  warmup=args.warmup, ms_per_step=round(ms_max / args.steps, 4), higher_is_better=True,
                  scaling="weak", vs_baseline=None, dtype="f64" if args.precision == 64 else "f32",
                  data="synthetic (seeded deformational flow; no public data set)",
                  config={"workload": "deformational_%dx%dx%d_periodic_gauge_iord3_nonos_predictor"
                                      % (nx, ny, nz),
                          "grid": [nx, ny, nz], "bc": "periodic", "iord": 3, "gauge": True,
                          "nonos": True, "predictor": True, "courant": 0.5,
                          "precision": "fp%d" % args.precision,
                          "l2": "each field %.0f MB > 129 MB L2; no flush" % (cells * elem / 1e6),
                          "parallelism": "replicas" if ws > 1 else "single"},
                  roofline=roof, gpu_launches=int(launches), clocks=clocks, stages=stage_json,
                  stage_io={"bytes_per_step": int(step_alg),
                            "bytes_per_cell": round(step_alg / cells, 1),
                            "gbs": round(step_alg / (ms_max / args.steps * 1e-3) / 1e9, 1),
                            "note": "every stage kernel's own inputs and outputs, intermediates "
                                    "included; a traffic figure, not a roofline (the compulsory "
                                    "bytes are roofline.compulsory_bytes_per_cell)"})
    mass1 = M.mass(arm.psi, arm.h)
    result["mass_rel_drift"] = (mass1 - mass0) / mass0
    # the last step's output against the running extrema its limiter kept (h = rhr = 1 here)
    tol = 1e-12 * float(arm.psi.abs().max())
    result["limiter_bound_violations"] = {"count": arm.ws.bound_violations(arm.psi, tol), "cells": cells,
                                          "tol": tol, "step": "the last timed step"}
    # e2e directly after the device-resident measurement, so that both see the
    # GPU in the same state (the studies below run for minutes)
    if not args.no_e2e:
        barrier(ws)
        e2e = run_e2e(arm, args, local)
        ms_e2e = max_over_ranks(e2e["ms_per_step"], ws)
        e2e["value"] = round(ws * cells / (ms_e2e * 1e-3) / 1e9, 4)
        e2e["ms_per_step"] = round(ms_e2e, 4)
        result["e2e"] = e2e
    if rank == 0 and ws == 1 and not args.no_extras and args.precision == 64:
        result["fp32"] = run_fp32_study(args, host, arm, ms_max / args.steps, mass0, peak, peak_kind, sms)
    if rank == 0 and ws == 1 and not args.no_extras:
        result["variable_density"] = run_density_study(args, host, ms_max / args.steps)
    arm.ws.close()
    del arm
    if rank == 0 and ws == 1 and not args.no_extras:
        torch.cuda.empty_cache()
        result["adjoint"] = run_adjoint_study(args)
        torch.cuda.empty_cache()
        result["batch"] = run_batch_study(args)
        torch.cuda.empty_cache()
        result["precision_768x768x160"] = run_precision_study(args, nsteps=args.precision_steps)
        if not args.no_cpu_baseline:
            result["config_baselines"] = run_config_baselines(args)
    return result


def profiled_stages(arm, n0, steps):
    """Per-stage kernel times of `steps` further steps with an event pair
    around every launch; the field keeps advancing (steps n0, n0+1, ...)."""
    import torch
    torch.cuda.synchronize()
    arm.ws.profile(True)
    for n in range(n0, n0 + steps):
        arm.step(n)
    stages = arm.ws.stage_times()
    arm.ws.profile(False)
    return stages


def run_fp32_study(args, host, arm64, ms64, mass0, peak, peak_kind, sms):
    """Same workload and steps in FP32 (the precision study): speedup
    over the FP64 run, error against it, FP64-compensated mass drift, and
    the roofline of the FP32 step (its dominant kernel and the whole step)."""
    import torch
    M = arm64.M
    nx, ny, nz = args.grid
    arm = GpuArm(nx, ny, nz, 32, host=host)
    for n in range(args.warmup):
        arm.step(n)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    l0 = M.launch_count()
    with ClockSampler(torch.cuda.current_device()) as clk:
        e0.record()
        for n in range(args.warmup, args.warmup + args.steps):
            arm.step(n)
        e1.record()
        torch.cuda.synchronize()
    launches = M.launch_count() - l0
    clocks = clk.summary()
    ms = e0.elapsed_time(e1) / args.steps
    # the profiled pass also brings the field to the FP64 run's step count
    # (it ran warmup + steps timed steps and as many profiled ones)
    stages = profiled_stages(arm, args.warmup + args.steps, args.steps)
    steps_compared = args.warmup + 2 * args.steps
    linf, l2, bmax, bl2 = M.error_norms(arm.psi, arm64.psi)
    m32 = M.mass(arm.psi, arm.h)
    cells = nx * ny * nz
    dom = max(stages.items(), key=lambda kv: kv[1][0])
    name, (tot_ms, nl) = dom
    avg_ms = tot_ms / max(nl, 1)
    alg = stage_elems(name, True, 3, 32) * 4 * cells
    achieved = alg / (avg_ms * 1e-3) / 1e9
    fused = name.startswith("fused")
    roof = {"bound": "hbm", "kernel": name, "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
            "frac": round(achieved / peak, 4), "peak_source": peak_kind, "alg_bytes_per_launch": int(alg),
            "avg_launch_ms": round(avg_ms, 4),
            "traffic": int(NCU_FUSED_LIMIT["dram_bytes_per_cell"] * cells) if name == "fused_limit_update" else None,
            "traffic_source": "ncu DRAM bytes per cell of this kernel at 384x384x64, scaled by cells"}
    if name == "fused_limit_update":
        roof["issue"] = {"inst_per_cell": NCU_FUSED_LIMIT["inst_per_cell"],
                         "issue_active": NCU_FUSED_LIMIT["issue_active"],
                         "note": "ncu at 384x384x64: the kernel is bound by instruction issue "
                                 "(shared-memory loads, selects, address arithmetic), not by DRAM"}
    roof.update(step_roofs(stages, args.steps, ms, cells, 32, peak,
                           clocks.get("sm_mhz") or clocks.get("sm_max_mhz") or 2070.0, sms))
    out = {"value": round(cells / (ms * 1e-3) / 1e9, 4), "unit": UNIT, "ms_per_step": round(ms, 4),
           "speedup_vs_fp64": round(ms64 / ms, 3),
           "linf_rel_err_vs_fp64": linf / bmax, "l2_rel_err_vs_fp64": l2 / bl2,
           "steps_compared": steps_compared,
           "mass_rel_drift": (m32 - mass0) / mass0,
           "path": "fused z-marching kernels (TMA-staged tiles)" if fused else "stage kernels",
           "gpu_launches_per_step": round(launches / args.steps, 2),
           "roofline": roof, "clocks": clocks,
           "stages": {k: {"ms_per_step": round(v[0] / args.steps, 4), "launches_per_step": v[1] / args.steps}
                      for k, v in stages.items() if v[1]},
           "note": "FP32 stencil arithmetic, FP64 Neumaier-compensated mass and norms"}
    arm.ws.close()
    return out


def run_density_study(args, host, ms_unit, amp=0.1, phase=1.0):
    """The headline step with a variable fluid density.  The reference's test
    application uses unit density (advection_test_setup.f90:630-631); its
    perturbed set-up (advection_test_setup.f90:745-759) uses
    h = 1 + amp*sin(2pi i/n + phase 2pi/3)*cos(2pi j/m + 2 phase 2pi/3)*cos(2pi k/l + 3 phase 2pi/3),
    used here with rhr = 1/h.  The kernels skip multiplications and divisions by an
    exact 1.0, so this line shows the general-density throughput beside the headline."""
    import torch
    nx, ny, nz = args.grid
    arm = GpuArm(nx, ny, nz, args.precision, host=host)
    dt = arm.tdtype
    ax = lambda n, s: torch.arange(1, n + 1, device="cuda", dtype=torch.float64) * (2 * math.pi / n) + s
    tp = 2 * math.pi / 3
    noise = (torch.sin(ax(nx, phase * tp))[:, None, None] * torch.cos(ax(ny, 2 * phase * tp))[None, :, None]
             * torch.cos(ax(nz, 3 * phase * tp))[None, None, :]) * amp
    inner = lambda t: t.permute(2, 1, 0)[1:nz + 1, 1:ny + 1, 1:nx + 1].permute(2, 1, 0)
    inner(arm.h).copy_((1.0 + noise).to(dt))
    inner(arm.rhr).copy_((1.0 / (1.0 + noise)).to(dt))
    for c in range(3):
        arm.o[c][..., 2].mul_(arm.h)
    for n in range(args.warmup):
        arm.step(n)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for n in range(args.warmup, args.warmup + args.steps):
        arm.step(n)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    arm.ws.close()
    cells = nx * ny * nz
    return {"value": round(cells / (ms * 1e-3) / 1e9, 4), "unit": UNIT, "ms_per_step": round(ms, 4),
            "vs_unit_density": round(ms_unit / ms, 3),
            "density": "h = 1 + %.2f sin cos cos (reference perturbed set-up), rhr = 1/h" % amp}


class DevArm:
    """A workload built on the device: the deformational A-grid flow (u, v
    scaled by cos(pi t/T), w steady) through the predictor, psi from a
    callable, h = rhr = 1, periodic; iord and precision as given."""

    def __init__(self, nx, ny, nz, precision, iord, psi_fn, T=200.0, courant=0.5):
        import torch
        from advectionhpctester_gb300 import mpdata as M
        self.torch, self.M, self.T = torch, M, T
        dt = torch.float64 if precision == 64 else torch.float32
        sh = M.shapes(nx, ny, nz, 1)
        emp = lambda shape: M.fortran_empty(shape, dt)
        inner = lambda t: t.permute(2, 1, 0)[1:nz + 1, 1:ny + 1, 1:nx + 1].permute(2, 1, 0)
        x = (torch.arange(nx, device="cuda", dtype=torch.float64) + 0.5) / nx
        y = (torch.arange(ny, device="cuda", dtype=torch.float64) + 0.5) / ny
        z = (torch.arange(nz, device="cuda", dtype=torch.float64) + 0.5) / nz
        sc = courant / 1.1
        pat = [(torch.sin(math.pi * x) ** 2)[:, None, None] * torch.sin(2 * math.pi * y)[None, :, None] * sc,
               -(torch.sin(math.pi * y) ** 2)[None, :, None] * torch.sin(2 * math.pi * x)[:, None, None] * sc,
               0.1 * torch.sin(2 * math.pi * z)[None, None, :] * sc]
        self.pats = []
        for a in pat:
            t = emp(sh["psi"])
            t.zero_()
            inner(t).copy_(a.expand(nx, ny, nz))
            self.pats.append(t)
        self.psi = emp(sh["psi"])
        self.psi.zero_()
        inner(self.psi).copy_(psi_fn(x, y, z))
        self.h = emp(sh["psi"])
        self.h.fill_(1.0)
        self.rhr = emp(sh["psi"])
        self.rhr.fill_(1.0)
        self.u1, self.u2, self.u3 = emp(sh["u1"]), emp(sh["u2"]), emp(sh["u3"])
        for u in (self.u1, self.u2, self.u3):
            u.zero_()
        self.o = [M.fortran_empty(sh["psi"] + (3,), dt) for _ in range(3)]
        for c in range(3):
            self.o[c].zero_()
            self.o[c][..., 2].copy_(self.pats[c] * (time_factor(-1, T) if c < 2 else 1.0))
        self.ws = M.Workspace(nx, ny, nz, 1, 1, 1, 1, iord=iord, nonos=1, gauge=1, precision=precision)

    def step(self, n):
        fac = time_factor(n, self.T)
        for c in range(3):
            self.torch.mul(self.pats[c], fac if c < 2 else 1.0, out=self.o[c][..., 0])
        self.ws.velprd(self.o[0], self.o[1], self.o[2], self.h, 1.0, 1.0, 1.0, 1.0, 1.0,
                       self.u1, self.u2, self.u3)
        self.ws.step(self.psi, self.u1, self.u2, self.u3, self.h, self.rhr)

    def close(self):
        self.ws.close()


def run_precision_study(args, n=(768, 768, 160), nsteps=500):
    """FP32 against FP64 on 768x768x160 periodic, the deformational flow through
    the predictor, gauge iord=2 nonoscillatory, psi = 1 inside [0.25,0.75]^3
    and 0.1 outside plus 1e-3 U[-1,1] (seed 4): throughput of each, error of
    FP32 against FP64 after the same steps, FP64-compensated mass drift."""
    import torch
    from advectionhpctester_gb300 import mpdata as M
    nx, ny, nz = n
    gen = torch.Generator(device="cuda")
    gen.manual_seed(4)
    noise = (torch.rand((nx, ny, nz), device="cuda", dtype=torch.float64, generator=gen) * 2 - 1) * 1e-3

    def psi_fn(x, y, z):
        box = (((x >= 0.25) & (x <= 0.75))[:, None, None] & ((y >= 0.25) & (y <= 0.75))[None, :, None]
               & ((z >= 0.25) & (z <= 0.75))[None, None, :])
        return torch.where(box, 1.0, 0.1).to(torch.float64) + noise

    out = {"workload": "box_%dx%dx%d_periodic_gauge_iord2_nonos_predictor" % n, "steps": nsteps}
    arms, mass0 = {}, {}
    for prec in (64, 32):
        arm = DevArm(nx, ny, nz, prec, 2, psi_fn)
        mass0[prec] = M.mass(arm.psi, arm.h)
        arm.step(0)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for k in range(1, nsteps):
            arm.step(k)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / (nsteps - 1)
        out["fp%d_gcell_steps_per_s" % prec] = round(nx * ny * nz / (ms * 1e-3) / 1e9, 4)
        out["fp%d_ms_per_step" % prec] = round(ms, 4)
        m = M.mass(arm.psi, arm.h)
        out["fp%d_mass_rel_drift" % prec] = (m - mass0[prec]) / mass0[prec]
        arms[prec] = arm
    linf, l2, bmax, bl2 = M.error_norms(arms[32].psi, arms[64].psi)
    out["fp32_speedup"] = round(out["fp64_ms_per_step"] / out["fp32_ms_per_step"], 3)
    out["linf_rel_err_fp32_vs_fp64"] = linf / bmax
    out["l2_rel_err_fp32_vs_fp64"] = l2 / bl2
    # where the L-inf error sits: cells above each threshold, and its share
    # at the front (largest neighbour jump of the FP64 field above 5% of max)
    x64 = arms[64].psi[1:-1, 1:-1, 1:-1]
    err = (arms[32].psi[1:-1, 1:-1, 1:-1].double() - x64).abs()
    out["cells_over"] = {"%g" % t: int((err > t * bmax).sum().item()) for t in (1e-6, 1e-5)}
    jump = torch.zeros_like(x64)
    for d in range(3):
        for sgn in (1, -1):
            jump = torch.maximum(jump, (torch.roll(x64, sgn, d) - x64).abs())
    front = jump > 0.05 * bmax
    out["linf_rel_err_front"] = err[front].max().item() / bmax
    out["linf_rel_err_elsewhere"] = err[~front].max().item() / bmax
    del x64, err, jump, front
    for a in arms.values():
        a.close()
    del arms
    torch.cuda.empty_cache()
    # conditioning floor: FP64 arithmetic from the initial field and velocity
    # patterns rounded once to FP32, against the exact FP64 run
    ref = DevArm(nx, ny, nz, 64, 2, psi_fn)
    rnd = DevArm(nx, ny, nz, 64, 2, psi_fn)
    rnd.psi.copy_(rnd.psi.float().double())
    for t in rnd.pats:
        t.copy_(t.float().double())
    for k in range(nsteps):
        ref.step(k)
        rnd.step(k)
    linf_r, l2_r, bmax_r, bl2_r = M.error_norms(rnd.psi, ref.psi)
    ref.close()
    rnd.close()
    del ref, rnd
    out["linf_rel_fp64_from_fp32_rounded_input"] = linf_r / bmax_r
    out["l2_rel_fp64_from_fp32_rounded_input"] = l2_r / bl2_r
    out["diagnosis"] = ("the L-inf error comes from a few hundred cells beside the noisy front, where the "
                        "nonoscillatory limiter's branches (min(1,cp,cn), star extrema) switch under "
                        "perturbations of a few ulps; rounding only the initial data to FP32 and "
                        "computing in FP64 moves those cells by linf_rel_fp64_from_fp32_rounded_input, "
                        "so no computation that holds the field in FP32 meets 1e-5 after 500 steps; "
                        "L2 stays below 1e-6")
    torch.cuda.empty_cache()
    return out


def run_adjoint_study(args, n=(256, 256, 64), nsteps=200, iord=2, fd_dirs=32):
    """Adjoint of the gauge nonoscillatory iord=2 step on 256x256x64 periodic,
    deformational flow held fixed, Gaussian-cone psi, J = 0.5|psi_N - target|^2
    with a seeded shifted-cone target, sqrt(N) checkpointing; FP64 and FP32.
    The FP64 gradient is checked by central finite differences of J (GPU
    forward runs, eps = 1e-6) along fd_dirs seeded random directions in
    (psi_0, u1, u2, u3)."""
    import torch
    from advectionhpctester_gb300 import mpdata as M
    from advectionhpctester_gb300 import workloads as W
    nx, ny, nz = n
    f = W.Fields(nx, ny, nz, 1, 1, 1, 1)
    ua, va, wa = W.deformational_agrid(nx, ny, nz, 0.0, float(nsteps))
    W.set_c_grid_periodic(f, ua, va, wa)
    x = (np.arange(nx) + 0.5) / nx
    y = (np.arange(ny) + 0.5) / ny
    z = (np.arange(nz) + 0.5) / nz
    rng = np.random.default_rng(5)
    off = rng.uniform(-0.1, 0.1, 3)

    def cone(cx, cy, cz):
        r2 = (x - cx)[:, None, None] ** 2 + (y - cy)[None, :, None] ** 2 + (z - cz)[None, None, :] ** 2
        return 1.0 + np.exp(-r2 / (2 * 0.1 ** 2))
    W.interior(f.x)[...] = cone(0.5, 0.5, 0.5)
    tg = np.zeros_like(f.x)
    W.interior(tg)[...] = cone(0.5 + off[0], 0.5 + off[1], 0.5 + off[2])
    cells = nx * ny * nz
    out = {"workload": "adjoint_%dx%dx%d_periodic_gauge_iord%d_nonos_N%d" % (nx, ny, nz, iord, nsteps),
           "checkpoint_interval": int(math.ceil(math.sqrt(nsteps)))}
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    grads = {}
    for prec, dt in ((64, torch.float64), (32, torch.float32)):
        d = {k: M.fortran_device(getattr(f, k), dtype=np.float64 if prec == 64 else np.float32)
             for k in ("x", "u1", "u2", "u3", "h", "rhr")}
        target = M.fortran_device(tg, dtype=np.float64 if prec == 64 else np.float32)
        ws = M.Workspace(nx, ny, nz, 1, 1, 1, 1, iord=iord, nonos=1, gauge=1, precision=prec)
        psi = d["x"].clone()
        for _ in range(3):
            ws.step(psi, d["u1"], d["u2"], d["u3"], d["h"], d["rhr"])
        psi.copy_(d["x"])
        torch.cuda.synchronize()
        e0.record()
        for _ in range(nsteps):
            ws.step(psi, d["u1"], d["u2"], d["u3"], d["h"], d["rhr"])
        e1.record()
        torch.cuda.synchronize()
        fwd_ms = e0.elapsed_time(e1)
        lam = psi.clone()
        gu = [torch.zeros_like(d[k]) for k in ("u1", "u2", "u3")]
        ws.step_adjoint(d["x"], d["u1"], d["u2"], d["u3"], d["h"], d["rhr"], lam, *gu)
        torch.cuda.synchronize()
        e0.record()
        for _ in range(10):
            ws.step_adjoint(d["x"], d["u1"], d["u2"], d["u3"], d["h"], d["rhr"], lam, *gu)
        e1.record()
        torch.cuda.synchronize()
        step_adj_ms = e0.elapsed_time(e1) / 10
        psi.copy_(d["x"])
        gx = torch.zeros_like(psi)
        gu = [torch.zeros_like(d[k]) for k in ("u1", "u2", "u3")]
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        J, peak = ws.adjoint_run(nsteps, psi, d["u1"], d["u2"], d["u3"], d["h"], d["rhr"], target, gx, *gu)
        run_ms = (time.perf_counter() - t0) * 1e3
        res = {"forward_ms_per_step": round(fwd_ms / nsteps, 4), "step_adjoint_ms": round(step_adj_ms, 4),
               "step_adjoint_over_forward": round(step_adj_ms / (fwd_ms / nsteps), 3),
               "run_ms": round(run_ms, 2), "run_over_forward": round(run_ms / fwd_ms, 3),
               "adjoint_gcell_steps_per_s": round(cells * nsteps / (run_ms * 1e-3) / 1e9, 4),
               "peak_bytes": int(peak), "J": J}
        grads[prec] = [gx.double()] + [g.double() for g in gu]
        # the same run with the limiter off, where J is smooth
        ws0 = M.Workspace(nx, ny, nz, 1, 1, 1, 1, iord=iord, nonos=0, gauge=1, precision=prec)
        psi.copy_(d["x"])
        g0 = [torch.zeros_like(psi)] + [torch.zeros_like(d[k]) for k in ("u1", "u2", "u3")]
        ws0.adjoint_run(nsteps, psi, d["u1"], d["u2"], d["u3"], d["h"], d["rhr"], target, *g0)
        ws0.close()
        grads["off%d" % prec] = [g.double() for g in g0]
        del g0
        if prec == 32:
            # the FP32 gradients against the FP64 ones (central differences of
            # an FP32 J of about 1e6 resolve nothing at eps = 1e-6)
            def cmp(a32, a64):
                num = math.sqrt(sum(float(((a - b) ** 2).sum()) for a, b in zip(a32, a64)))
                den = math.sqrt(sum(float((b ** 2).sum()) for b in a64))
                lmax = max(float((a - b).abs().max()) for a, b in zip(a32, a64))
                gmax = max(float(b.abs().max()) for b in a64)
                return {"l2_rel": num / den, "linf_rel": lmax / gmax}
            res["grad_vs_fp64"] = {"limiter_off": cmp(grads["off32"], grads["off64"]),
                                   "limiter_on": cmp(grads[32], grads[64]),
                                   "note": "dJ/dpsi_0 and dJ/du1..u3 of the FP32 run against the FP64 run's; "
                                           "with the limiter on the cone's flat far field (exactly 1) ties "
                                           "the star extrema everywhere, and the two precisions take "
                                           "different branches there"}
            del grads
        if prec == 64 and fd_dirs:
            res["fd_check"] = fd_checks(M, f, tg, d, target, nsteps, fd_dirs, nx, ny, nz, iord)
        out["fp%d" % prec] = res
        ws.close()
        del d, target, psi, lam, gx, gu
        torch.cuda.empty_cache()
    return out


def fd_checks(M, f, tg, d, target, nsteps, ndirs, nx, ny, nz, iord):
    """Central differences of J against the adjoint gradient, where J is
    differentiable.  The limiter makes J piecewise smooth: wherever the
    updated field is its own star extremum (or two star values tie) the
    forward point sits on a kink, and a central difference averages the two
    one-sided slopes.  So: (1) the same flow, cone and N with the limiter
    off, (2) one step with the limiter on, the cone plus 1e-3 seeded noise
    breaking the exact ties of its flat far field."""
    import torch
    from advectionhpctester_gb300 import workloads as W
    out = {}
    ws0 = M.Workspace(nx, ny, nz, 1, 1, 1, 1, iord=iord, nonos=0, gauge=1, precision=64)
    psi = d["x"].clone()
    gx = torch.zeros_like(psi)
    gu = [torch.zeros_like(d[k]) for k in ("u1", "u2", "u3")]
    ws0.adjoint_run(nsteps, psi, d["u1"], d["u2"], d["u3"], d["h"], d["rhr"], target, gx, *gu)
    out["limiter_off_N%d" % nsteps] = adjoint_fd_check(ws0, d, target, gx, gu, nsteps, ndirs, nx, ny, nz)
    # the Taylor sweep's optimum (truncation ~ eps^2 above it, round-off ~ 1/eps below)
    out["limiter_off_N%d_eps1e-4" % nsteps] = adjoint_fd_check(ws0, d, target, gx, gu, nsteps, ndirs, nx, ny, nz,
                                                               eps=1e-4)
    ws0.close()
    noisy = f.x.copy()
    W.interior(noisy)[...] += 1e-3 * np.random.default_rng(7).random((nx, ny, nz))
    dn = dict(d)
    dn["x"] = M.fortran_device(noisy)
    ws1 = M.Workspace(nx, ny, nz, 1, 1, 1, 1, iord=iord, nonos=1, gauge=1, precision=64)
    psi = dn["x"].clone()
    gx = torch.zeros_like(psi)
    gu = [torch.zeros_like(d[k]) for k in ("u1", "u2", "u3")]
    ws1.adjoint_run(1, psi, d["u1"], d["u2"], d["u3"], d["h"], d["rhr"], target, gx, *gu)
    out["limiter_on_N1_noise1e-3"] = adjoint_fd_check(ws1, dn, target, gx, gu, 1, ndirs, nx, ny, nz)
    ws1.close()
    return out


def adjoint_fd_check(ws, d, target, gx, gu, nsteps, ndirs, nx, ny, nz, eps=1e-6):
    """Central differences (J(p + eps e) - J(p - eps e)) / (2 eps) against
    <e, grad J> along ndirs unit directions (seed 6): half in psi_0 (interior
    cells), half in the velocities (interior faces with |u| >= 1e-6, away
    from the kinks of pp, pn and |u| at u = 0).  The difference of J is
    summed cell by cell as 0.5 (psi+ - psi-)(psi+ + psi- - 2 target), which
    keeps about 7 significant digits where J(+) - J(-) would keep 4."""
    import torch
    gen = torch.Generator(device="cuda")
    gen.manual_seed(6)
    inner = lambda t: t.permute(2, 1, 0)[1:nz + 1, 1:ny + 1, 1:nx + 1].permute(2, 1, 0)

    def final(psi0, u):
        psi = psi0.clone()
        for _ in range(nsteps):
            ws.step(psi, u[0], u[1], u[2], d["h"], d["rhr"])
        return inner(psi).clone()

    errs, errs_g = [], []
    gnorm = math.sqrt(float((gx * gx).sum()) + sum(float((g * g).sum()) for g in gu))
    u0 = [d["u1"], d["u2"], d["u3"]]
    tin = inner(target)
    for n in range(ndirs):
        epsi = torch.zeros_like(d["x"])
        eu = [torch.zeros_like(t) for t in u0]
        if n % 2 == 0:
            inner(epsi).copy_(torch.randn((nx, ny, nz), device="cuda", dtype=torch.float64, generator=gen))
        else:
            for t, u in zip(eu, u0):
                r = torch.randn((nx, ny, nz), device="cuda", dtype=torch.float64, generator=gen)
                inner(t).copy_(torch.where(inner(u).abs() >= 1e-6, r, torch.zeros_like(r)))
        norm = math.sqrt(float((epsi * epsi).sum()) + sum(float((t * t).sum()) for t in eu))
        epsi /= norm
        for t in eu:
            t /= norm
        dot = float((gx * epsi).sum()) + sum(float((g * t).sum()) for g, t in zip(gu, eu))

        def shifted(sign):  # clones keep the Fortran strides; the shift is in place
            xs = d["x"].clone().add_(epsi, alpha=sign * eps)
            return xs, [a.clone().add_(b, alpha=sign * eps) for a, b in zip(u0, eu)]
        pp_, pm_ = final(*shifted(1.0)), final(*shifted(-1.0))
        fd = float((0.5 * (pp_ - pm_) * (pp_ + pm_ - 2.0 * tin)).sum()) / (2 * eps)
        errs.append(abs(fd - dot) / max(abs(dot), 1e-300))
        errs_g.append(abs(fd - dot) / max(gnorm, 1e-300))
    errs = sorted(errs)
    return {"directions": ndirs, "eps": eps, "max_rel_err": errs[-1], "median_rel_err": errs[len(errs) // 2],
            "max_err_over_grad_norm": max(errs_g)}


def batch_domains(seed=3, count=64):
    sizes = [(32, 32, 32), (64, 64, 64), (128, 128, 64), (256, 256, 64), (192, 96, 48)]
    rng = np.random.default_rng(seed)
    picks = [sizes[i] for i in rng.integers(0, len(sizes), count)]
    return picks, rng


def make_domain_device(n, rng, torch_dtype):
    """One periodic domain generated on the device: solid-body rotation about
    z or the deformational flow, Courant U[0.2,0.5], Gaussian plus noise psi."""
    import torch
    from advectionhpctester_gb300 import mpdata as M
    nx, ny, nz = n
    dev = "cuda"
    c = float(rng.uniform(0.2, 0.5))
    kind = int(rng.integers(0, 2))
    g = torch.Generator(device=dev)
    g.manual_seed(int(rng.integers(0, 2 ** 31)))
    sh = M.shapes(nx, ny, nz, 1)
    t = {k: M.fortran_empty(sh[k], torch_dtype) for k in ("u1", "u2", "u3")}
    for k in ("psi", "h", "rhr"):
        t[k] = M.fortran_empty(sh["psi"], torch_dtype)
    t["h"].fill_(1.0)
    t["rhr"].fill_(1.0)
    x = (torch.arange(nx, device=dev, dtype=torch.float64) + 0.5) / nx
    y = (torch.arange(ny, device=dev, dtype=torch.float64) + 0.5) / ny
    z = (torch.arange(nz, device=dev, dtype=torch.float64) + 0.5) / nz
    X, Y, Z = torch.meshgrid(x, y, z, indexing="ij")
    if kind == 0:  # solid body about z through the centre, on the faces
        xf = torch.arange(nx, device=dev, dtype=torch.float64) / nx
        yf = torch.arange(ny, device=dev, dtype=torch.float64) / ny
        ua = -(Y - 0.5) * torch.ones_like(X)
        va = (X - 0.5) * torch.ones_like(Y)
        u1 = -(y[None, :, None] - 0.5).expand(nx, ny, nz) + 0 * xf[:, None, None]
        u2 = (x[:, None, None] - 0.5).expand(nx, ny, nz) + 0 * yf[None, :, None]
        u3 = torch.zeros_like(X)
        s = c / 0.5
        u1, u2 = u1 * s, u2 * s
        del ua, va
    else:
        ua = torch.sin(math.pi * X) ** 2 * torch.sin(2 * math.pi * Y)
        va = -torch.sin(math.pi * Y) ** 2 * torch.sin(2 * math.pi * X)
        wa = 0.1 * torch.sin(2 * math.pi * Z)
        s = c / 1.1
        u1 = 0.5 * (ua + torch.roll(ua, 1, 0)) * s
        u2 = 0.5 * (va + torch.roll(va, 1, 1)) * s
        u3 = 0.5 * (wa + torch.roll(wa, 1, 2)) * s
    cx, cy, cz = (float(v) for v in rng.uniform(0.3, 0.7, 3))
    psi = 1.0 + torch.exp(-((X - cx) ** 2 + (Y - cy) ** 2 + (Z - cz) ** 2) / (2 * 0.1 ** 2))
    psi = psi + 0.01 * torch.rand(psi.shape, device=dev, dtype=torch.float64, generator=g)
    t["psi"][1:-1, 1:-1, 1:-1] = psi.to(torch_dtype)
    t["u1"][1:-2, 1:-1, 1:-1] = u1.to(torch_dtype)
    t["u1"][-2, 1:-1, 1:-1] = u1[0].to(torch_dtype)
    t["u2"][1:-1, 1:-2, 1:-1] = u2.to(torch_dtype)
    t["u2"][1:-1, -2, 1:-1] = u2[:, 0].to(torch_dtype)
    t["u3"][1:-1, 1:-1, 1:-2] = u3.to(torch_dtype)
    t["u3"][1:-1, 1:-1, -2] = u3[:, :, 0].to(torch_dtype)
    return t


def run_batch_study(args, steps=100):
    """Batching: 64 periodic domains of uneven sizes (seed 3) in one
    batch (one CUDA-graph launch per step, tuned tile shape) against a loop of
    per-domain steps; FP64 and FP32.  Plus 16 tracers sharing one velocity on
    256x256x64 against 16 separate steps, in the gauge and the standard form."""
    import torch
    from advectionhpctester_gb300 import mpdata as M
    out = {}

    def timed(fn, reps):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    for prec, tdt in ((64, torch.float64), (32, torch.float32)):
        picks, rng = batch_domains()
        doms = [make_domain_device(n, rng, tdt) for n in picks]
        cells = sum(a * b * c for a, b, c in picks)
        probs = [dict(np=n[0], mp=n[1], lp=n[2], gauge=1) for n in picks]
        b = M.Batch(probs, iord=2, nonos=1, precision=prec)
        for p, t in enumerate(doms):
            b.set(p, t["psi"], t["u1"], t["u2"], t["u3"], t["h"], t["rhr"])
        bx, by = b.tune()
        l0 = M.launch_count()
        b.step()
        lps = M.launch_count() - l0
        b.graph(True)
        ms_batch = timed(b.step, steps)
        wss = [M.Workspace(*n, 1, 1, 1, 1, iord=2, nonos=1, gauge=1, precision=prec) for n in picks]

        def loop():
            for w, t in zip(wss, doms):
                w.step(t["psi"], t["u1"], t["u2"], t["u3"], t["h"], t["rhr"])
        ms_loop = timed(loop, steps)
        for w in wss:
            w.close()
        b.close()
        out["domains_fp%d" % prec] = {
            "domains": len(picks), "cells": cells, "tile": [bx, by],
            "graph_gcell_steps_per_s": round(cells / (ms_batch * 1e-3) / 1e9, 4),
            "loop_gcell_steps_per_s": round(cells / (ms_loop * 1e-3) / 1e9, 4),
            "speedup_vs_loop": round(ms_loop / ms_batch, 3),
            "launches_per_step": int(lps), "graph_launches_per_step": 1}
        del doms
        torch.cuda.empty_cache()
    # 16 tracers sharing one velocity, in the gauge form and in the standard
    # form (the reference's multi-field step advects its scalars in the latter)
    tc = 16 * 256 * 256 * 64
    for gauge, key, prec in ((1, "tracers16_fp64", 64), (0, "tracers16_std_fp64", 64), (1, "tracers16_fp32", 32)):
        rng = np.random.default_rng(16)
        base = make_domain_device((256, 256, 64), rng, torch.float64 if prec == 64 else torch.float32)
        tr = [base["psi"].clone() * (1.0 + 0.01 * k) for k in range(16)]
        b = M.Batch([dict(np=256, mp=256, lp=64, gauge=gauge, velocity_group=0)] * 16, iord=2, nonos=1,
                    precision=prec)
        for p in range(16):
            b.set(p, tr[p], base["u1"], base["u2"], base["u3"], base["h"], base["rhr"])
        b.graph(True)
        ms_b = timed(b.step, steps)
        w = M.Workspace(256, 256, 64, 1, 1, 1, 1, iord=2, nonos=1, gauge=gauge, precision=prec)

        def loop16():
            for p in range(16):
                w.step(tr[p], base["u1"], base["u2"], base["u3"], base["h"], base["rhr"])
        ms_l = timed(loop16, steps)
        w.close()
        b.close()
        out[key] = {"tracer_cells": tc, "form": "gauge" if gauge else "standard",
                    "batch_gcell_steps_per_s": round(tc / (ms_b * 1e-3) / 1e9, 4),
                    "loop_gcell_steps_per_s": round(tc / (ms_l * 1e-3) / 1e9, 4),
                    "speedup_vs_loop": round(ms_l / ms_b, 3)}
        del base, tr
        torch.cuda.empty_cache()
    return out


def run_e2e(arm, args, local=0):
    """Same metric through the public API with host buffers: every step copies
    psi, the A-grid Courant numbers, h and rhr from pinned host memory and
    reads psi back.  The copies run on their own streams into two alternating
    device buffer sets, so step n's upload and step n-1's read-back overlap
    step n's compute; events order each buffer's upload, compute and
    read-back.  The timed region spans the first upload to the last
    read-back."""
    torch, M = arm.torch, arm.M
    comp = torch.cuda.current_stream()
    up, down = torch.cuda.Stream(), torch.cuda.Stream()
    pin = lambda t: t.detach().cpu().pin_memory()
    hpsi = pin(arm.psi)
    hpat = [pin(p) for p in arm.pats]
    hh, hrhr = pin(arm.h), pin(arm.rhr)
    outs = [torch.empty_like(hpsi).pin_memory() for _ in range(2)]
    cells = arm.nx * arm.ny * arm.nz
    bi = sum(t.numel() * t.element_size() for t in [hpsi, hh, hrhr] + hpat)
    bo = outs[0].numel() * outs[0].element_size()
    steps = max(6, args.steps)
    bufs = [dict(psi=arm.psi, pats=arm.pats, h=arm.h, rhr=arm.rhr),
            dict(psi=torch.empty_like(arm.psi), pats=[torch.empty_like(p) for p in arm.pats],
                 h=torch.empty_like(arm.h), rhr=torch.empty_like(arm.rhr))]
    ev_in = [torch.cuda.Event() for _ in range(2)]
    ev_done = [torch.cuda.Event() for _ in range(2)]
    ev_out = [torch.cuda.Event() for _ in range(2)]

    def issue(n):
        k = n % 2
        b = bufs[k]
        with torch.cuda.stream(up):
            up.wait_event(ev_out[k])      # step n-2 has been read back from this set
            b["psi"].copy_(hpsi, non_blocking=True)
            for c in range(3):
                b["pats"][c].copy_(hpat[c], non_blocking=True)
            b["h"].copy_(hh, non_blocking=True)
            b["rhr"].copy_(hrhr, non_blocking=True)
            ev_in[k].record(up)
        comp.wait_event(ev_in[k])
        arm.step_on(n, b)
        ev_done[k].record(comp)
        with torch.cuda.stream(down):
            down.wait_event(ev_done[k])
            outs[k].copy_(b["psi"], non_blocking=True)
            ev_out[k].record(down)

    def link_gbs():
        """Host-to-device rate of one untimed upload of the six fields (the
        host link's rate varies from run to run on a shared machine)."""
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(up):
            a.record(up)
            bufs[1]["psi"].copy_(hpsi, non_blocking=True)
            for c in range(3):
                bufs[1]["pats"][c].copy_(hpat[c], non_blocking=True)
            bufs[1]["h"].copy_(hh, non_blocking=True)
            bufs[1]["rhr"].copy_(hrhr, non_blocking=True)
            b.record(up)
        torch.cuda.synchronize()
        return round(bi / (a.elapsed_time(b) * 1e-3) / 1e9, 1)

    for n in range(2):  # warm the streams and buffers
        issue(n)
    torch.cuda.synchronize()
    gbs_before = link_gbs()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        e0.record(comp)
        up.wait_stream(comp)
        for n in range(steps):
            issue(n)
        comp.wait_stream(down)
        e1.record(comp)
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    gbs_after = link_gbs()
    return {"value": round(cells * steps / (ms * 1e-3) / 1e9, 4), "unit": UNIT,
            "h2d_bytes_per_step": int(bi), "d2h_bytes_per_step": int(bo), "steps": steps,
            "ms_per_step": round(ms / steps, 4), "clocks": clk.summary(),
            "h2d_link_gbs": {"before": gbs_before, "after": gbs_after,
                             "note": "one untimed upload of the step's six fields before and after "
                                     "the timed region; the copies hide behind the step while this "
                                     "stays near 210 GB/s"},
            "overlap": "double-buffered: upload and read-back streams beside the compute stream; "
                       "the first upload and the last read-back are not overlapped"}


# --------------------------------------------------------------------------
# CPU oracle (reference arm and cpu_baseline)
# --------------------------------------------------------------------------

def oracle_slab(nx, ny, nz_slab, precision):
    f, pats = make_state(nx, ny, nz_slab, np.float64 if precision == 64 else np.float32)
    return f, pats


def time_oracle(nx, ny, nz_slab, steps, warmup, precision, threads, budget_s=None, iord=3, psi_fn=None):
    """CPU oracle Gcell-steps/s of the predictor + gauge step on a periodic
    slab of the deformational flow; psi_fn(x, y, z) replaces the field."""
    from oracle import oracle as O
    O.lib()
    O.set_threads(threads)
    f, pats = oracle_slab(nx, ny, nz_slab, precision)
    if psi_fn is not None:
        from advectionhpctester_gb300 import workloads as W
        c = lambda n: (np.arange(n) + 0.5) / n
        W.interior(f.x)[...] = psi_fn(c(nx)[:, None, None], c(ny)[None, :, None], c(nz_slab)[None, None, :])
    g = O.grid(nx, ny, nz_slab, 1, 1, 1, 1)
    T = 200.0
    lev = f.x.shape + (3,)
    dt_np = f.x.dtype
    o = [np.zeros(lev, dtype=dt_np, order="F") for _ in range(3)]
    for c in range(3):
        o[c][..., 2] = pats[c] * (time_factor(-1, T) if c < 2 else 1.0)

    def step(n):
        for c in range(3):
            o[c][..., 0] = pats[c] * (time_factor(n, T) if c < 2 else 1.0)
        t0 = time.perf_counter()
        O.velprd(g, o[0], o[1], o[2], f.h, 1.0, 1.0, 1.0, 1.0, 1.0, f.u1, f.u2, f.u3)
        O.advec_dwarf(g, f.x, f.bcx, f.bcy, f.u1, f.u2, f.u3, f.rhr, f.h, legacyoptmode=4, t_adv=1,
                      iord=iord, nonos=1)
        return time.perf_counter() - t0

    for n in range(warmup):
        step(n)
    total, done = 0.0, 0
    for n in range(warmup, warmup + steps):
        total += step(n)
        done += 1
        if budget_s is not None and total >= budget_s:
            break
    return nx * ny * nz_slab * done / total / 1e9, done, total


def run_config_baselines(args):
    """The CPU baselines of the configurations besides the headline, with the
    GPU beside where the whole configuration fits a short run:
    - config 1: 64x64x32 periodic solid-body rotation about z (max |u| 0.4),
      psi = 1 + 4 exp(-r^2/32), standard form, iord=2, nonos, 100 steps, on the
      GPU and on the CPU oracle with one thread and with all threads;
    - config 4: the 768x768x160 box field (psi = 1 inside [0.25,0.75]^3, 0.1
      outside) in the deformational flow, iord=2 with the predictor, on the
      CPU oracle over a 768x768x16 slab."""
    import torch
    from oracle import oracle as O
    from advectionhpctester_gb300 import mpdata as M
    from advectionhpctester_gb300 import workloads as W
    out = {}
    n, steps = (64, 64, 32), 100
    f = W.solid_body_z(*n, ih=1, courant=0.4, std=True)
    d = {k: M.fortran_device(getattr(f, k)) for k in ("x", "u1", "u2", "u3", "h", "rhr")}
    ws = M.Workspace(*n, 1, 1, 1, 1, iord=2, nonos=1, gauge=0, precision=64)
    args_ = (d["x"], d["u1"], d["u2"], d["u3"], d["h"], d["rhr"])
    for _ in range(3):
        ws.step(*args_)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        ws.step(*args_)
    e1.record()
    torch.cuda.synchronize()
    ws.close()
    cells = n[0] * n[1] * n[2]
    gpu = cells * steps / (e0.elapsed_time(e1) * 1e-3) / 1e9
    cpu = {}
    for threads in (1, os.cpu_count() or 1):
        O.lib()
        O.set_threads(threads)
        g = f.copy()
        t0 = time.perf_counter()
        O.advec_dwarf(O.grid(*n, 1, 1, 1, 1), g.x, g.bcx, g.bcy, g.u1, g.u2, g.u3, g.rhr, g.h, t_adv=2,
                      iord=2, nonos=1, nsteps=steps)
        cpu[threads] = cells * steps / (time.perf_counter() - t0) / 1e9
    out["config1_64x64x32_std_iord2_100steps"] = {
        "gpu_gcell_steps_per_s": round(gpu, 4), "cpu_1_thread": round(cpu[1], 6),
        "cpu_all_threads": round(cpu[max(cpu)], 6), "cpu_threads": max(cpu),
        "note": "131072 cells: the GPU step is launch-bound at this size"}

    def box(x, y, z):
        inside = (x >= 0.25) & (x <= 0.75) & (y >= 0.25) & (y <= 0.75) & (z >= 0.25) & (z <= 0.75)
        return np.where(inside, 1.0, 0.1)
    for threads in (1, os.cpu_count() or 1):
        v, done, total = time_oracle(768, 768, 16, 3, 1, 64, threads, budget_s=10.0, iord=2, psi_fn=box)
        out.setdefault("config4_768x768x16_slab_iord2_cpu", {})[
            "cpu_1_thread" if threads == 1 else "cpu_all_threads"] = round(v, 6)
    out["config4_768x768x16_slab_iord2_cpu"]["cpu_threads"] = os.cpu_count() or 1
    out["config4_768x768x16_slab_iord2_cpu"]["gpu_full_grid"] = "precision_768x768x160.fp64_gcell_steps_per_s"
    return out


def run_reference(args, ws, rank):
    if rank != 0:
        return None
    nx, ny, nz = args.grid
    threads = os.cpu_count() or 1
    slab = min(nz, args.ref_slab)
    value, done, total = time_oracle(nx, ny, slab, args.steps, args.warmup, args.precision, threads)
    sample = ("%d steps of a %dx%dx%d periodic slab of the same workload (predictor + gauge "
              "iord=3 step), CPU oracle (C++ restatement of the reference's Fortran path; the "
              "Fortran build is unavailable: no Fortran compiler)" % (done, nx, ny, slab))
    line = dict(metric=METRIC, value=round(value, 6), unit=UNIT, n_gpus=ws, steps=done,
                warmup=args.warmup, ms_per_step=round(total / max(done, 1) * 1e3, 3),
                higher_is_better=True, scaling="weak", vs_baseline=None,
                dtype="f64" if args.precision == 64 else "f32",
                data="synthetic (seeded deformational flow; no public data set)",
                config={"workload": "deformational_%dx%dx%d_periodic_gauge_iord3_nonos_predictor"
                                    % (nx, ny, nz), "grid": [nx, ny, nz],
                        "precision": "fp%d" % args.precision},
                impl="reference",
                cpu_baseline={"value": round(value, 6), "unit": UNIT, "cores": threads, "kind": "port",
                              "sample": sample},
                e2e={"value": round(value, 6), "unit": UNIT, "h2d_bytes_per_step": 0,
                     "d2h_bytes_per_step": 0})
    return line


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--precision", type=int, choices=[32, 64], default=64)
    ap.add_argument("--grid", type=int, nargs=3, default=[512, 512, 128])
    ap.add_argument("--ref-slab", type=int, default=16)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the FP32, adjoint, batch and 768x768x160 precision studies")
    ap.add_argument("--precision-steps", type=int, default=500,
                    help="steps of the 768x768x160 FP32-vs-FP64 study")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    ws, rank, local = dist_init(args.gpus)
    if args.impl == "reference":
        line = run_reference(args, ws, rank)
        if line is not None:
            print(json.dumps(line), flush=True)
        return
    result = run_ours(args, ws, rank, local)
    if rank == 0:
        if ws == 1 and not args.no_cpu_baseline:
            nx, ny, _ = args.grid
            v, done, total = time_oracle(nx, ny, args.ref_slab, 50, 1, args.precision,
                                         os.cpu_count() or 1, budget_s=15.0)
            v1, done1, total1 = time_oracle(nx, ny, args.ref_slab, 20, 1, args.precision, 1, budget_s=8.0)
            result["cpu_baseline"] = {
                "value": round(v, 6), "unit": UNIT, "cores": os.cpu_count() or 1, "kind": "port",
                "sample": "%d steps (%.1f s) of a %dx%dx%d periodic slab of the same workload, "
                          "CPU oracle with OpenMP on all host threads" % (done, total, nx, ny, args.ref_slab),
                "single_thread": {"value": round(v1, 6), "cores": 1,
                                  "sample": "%d steps (%.1f s) of the same slab, one thread (the "
                                            "reference's CPU build is serial)" % (done1, total1)}}
        print(json.dumps(result), flush=True)


if __name__ == "__main__":
    main()
