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
#   upwind   r psi u1 u2 u3 h rhr          w xant hinv            8
#   pseudo   r xant a1 a2 a3 h             w v1 v2 v3 (+fn1..3)   8 (11 std)
#   bounds   r xant psi|mx,mn h rhr F1..3  w cp cn q (+mx mn)     9..13
#   limit    r xant v1..3 cp cn (+q)       w w1..3 (+f1..3)       9 (13 std)
#   update   r q rhr h|hinv F1..3          w out                  7
#   predictor level  r o0 x3 o2 x3 h  w o1 x3                    10
#   predictor cgrid  r o1 x3 o0 x3 h  w u1..3 o2 x3              13
def stage_elems(stage, gauge, iord):
    keep = iord > 2
    if stage == "upwind":
        return 8.0
    if stage == "pseudo_velocity":
        return 8.0 if gauge else 11.0
    if stage == "limiter_bounds":
        first = 9.0 + (2.0 if keep else 0.0)          # reads psi, writes mx/mn when kept
        later = 13.0                                  # reads and writes mx/mn
        n = max(iord - 1, 1)
        return (first + later * (n - 1)) / n
    if stage == "limited_flux":
        return 9.0 if gauge else 13.0
    if stage == "corrective_update":
        return 7.0
    if stage == "predictor_level":
        return 10.0
    if stage == "predictor_cgrid":
        return 13.0
    return 2.0


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
    def __init__(self, nx, ny, nz, precision, T=200.0):
        import torch
        from advectionhpctester_gb300 import mpdata as M
        self.torch, self.M = torch, M
        self.nx, self.ny, self.nz, self.T = nx, ny, nz, T
        dnp = np.float64 if precision == 64 else np.float32
        self.tdtype = torch.float64 if precision == 64 else torch.float32
        f, pats = make_state(nx, ny, nz, dnp, T=T)
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

    def step(self, n):
        self.dynamics(n)
        self.ws.velprd(self.o[0], self.o[1], self.o[2], self.h, 1.0, 1.0, 1.0, 1.0, 1.0,
                       self.u1, self.u2, self.u3)
        self.ws.step(self.psi, self.u1, self.u2, self.u3, self.h, self.rhr)


def run_ours(args, ws, rank, local):
    import torch
    from advectionhpctester_gb300 import _native, mpdata as M
    _native.load(build_if_missing=True)
    torch.cuda.set_device(local)
    nx, ny, nz = args.grid
    cells = nx * ny * nz
    arm = GpuArm(nx, ny, nz, args.precision)
    stream = torch.cuda.current_stream()
    for n in range(args.warmup):
        arm.step(n)
    torch.cuda.synchronize()
    # timed region: inputs (268 MB per FP64 field) exceed the 129 MB L2, no flush needed
    arm.ws.profile(True)
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
    stages = arm.ws.stage_times()
    arm.ws.profile(False)
    clocks = clk.summary()
    value = ws * cells * args.steps / (ms_max * 1e-3) / 1e9

    # roofline of the dominant kernel
    peak, peak_kind = load_peaks()
    elem = 8 if args.precision == 64 else 4
    dom = max(stages.items(), key=lambda kv: kv[1][0])
    name, (tot_ms, nl) = dom
    avg_ms = tot_ms / max(nl, 1)
    alg_bytes = stage_elems(name, True, 3) * elem * cells
    achieved = alg_bytes / (avg_ms * 1e-3) / 1e9
    roof = {"bound": "hbm", "kernel": name, "achieved": round(achieved, 1), "peak": peak,
            "unit": "GB/s", "frac": round(achieved / peak, 4), "traffic": None,
            "peak_source": peak_kind, "alg_bytes_per_launch": int(alg_bytes),
            "avg_launch_ms": round(avg_ms, 4),
            "note": "FP64-ALU bound on GB300 (FP64 ~1.2 TFLOP/s); see fp64_pipe"}
    stage_json = {k: {"ms_total": round(v[0], 3), "launches": int(v[1]),
                      "share": round(v[0] / max(sum(t for t, _ in stages.values()), 1e-9), 4)}
                  for k, v in stages.items() if v[1]}
    step_alg = sum(stage_elems(k, True, 3) * elem * cells * v[1] for k, v in stages.items()) / args.steps
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
                  step_alg_bytes=int(step_alg),
                  step_hbm_frac=round(step_alg / (ms_max / args.steps * 1e-3) / 1e9 / peak, 4))
    if rank == 0 and ws == 1 and not args.no_e2e:
        result["e2e"] = run_e2e(arm, args)
    arm.ws.close()
    return result


def run_e2e(arm, args):
    """Same metric through the public API with host buffers: every step copies
    psi, the A-grid Courant numbers, h and rhr from pinned host memory and
    reads psi back."""
    torch, M = arm.torch, arm.M
    stream = torch.cuda.current_stream()
    pin = lambda t: t.detach().cpu().pin_memory()
    hpsi = pin(arm.psi)
    hpat = [pin(p) for p in arm.pats]
    hh, hrhr = pin(arm.h), pin(arm.rhr)
    out = torch.empty_like(hpsi).pin_memory()
    cells = arm.nx * arm.ny * arm.nz
    bi = sum(t.numel() * t.element_size() for t in [hpsi, hh, hrhr] + hpat)
    bo = out.numel() * out.element_size()
    steps = max(3, args.steps // 2)

    def one(n):
        arm.psi.copy_(hpsi, non_blocking=True)
        for c in range(3):
            arm.pats[c].copy_(hpat[c], non_blocking=True)
        arm.h.copy_(hh, non_blocking=True)
        arm.rhr.copy_(hrhr, non_blocking=True)
        arm.step(n)
        out.copy_(arm.psi, non_blocking=True)

    one(0)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for n in range(steps):
        one(n)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    return {"value": round(cells * steps / (ms * 1e-3) / 1e9, 4), "unit": UNIT,
            "h2d_bytes_per_step": int(bi), "d2h_bytes_per_step": int(bo), "steps": steps,
            "ms_per_step": round(ms / steps, 4)}


# --------------------------------------------------------------------------
# CPU oracle (reference arm and cpu_baseline)
# --------------------------------------------------------------------------

def oracle_slab(nx, ny, nz_slab, precision):
    f, pats = make_state(nx, ny, nz_slab, np.float64 if precision == 64 else np.float32)
    return f, pats


def time_oracle(nx, ny, nz_slab, steps, warmup, precision, threads, budget_s=None):
    from oracle import oracle as O
    O.lib()
    O.set_threads(threads)
    f, pats = oracle_slab(nx, ny, nz_slab, precision)
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
                      iord=3, nonos=1)
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
            result["cpu_baseline"] = {
                "value": round(v, 6), "unit": UNIT, "cores": os.cpu_count() or 1, "kind": "port",
                "sample": "%d steps (%.1f s) of a %dx%dx%d periodic slab of the same workload, "
                          "CPU oracle with OpenMP on all host threads" % (done, total, nx, ny, args.ref_slab)}
        print(json.dumps(result), flush=True)


if __name__ == "__main__":
    main()
