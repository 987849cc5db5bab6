"""Runs a few MPDATA steps of one workload with the fewest device
allocations, for profilers (ncu) and quick timing.

  python -m advectionhpctester_gb300.profile_case --grid 384 384 64 --steps 2 \
      [--precision 64|32] [--std] [--iord 3] [--bc periodic|reference] \
      [--workload random|deformational|balls] [--adjoint]

random: seeded random fields with h, rhr in [0.8, 1.2]; deformational: the
periodic deformational flow with unit densities (the benchmark's fields);
balls: the same flow carrying two balls on an exactly zero background.

Prints the CUDA-event time per step and the per-stage times.  --adjoint
times the step adjoint (lambda = psi, zero velocity gradients) after the
forward steps and reports its time beside the forward step's.
"""
import argparse
import json

import numpy as np


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--grid", type=int, nargs=3, default=[384, 384, 64])
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--warmup", type=int, default=1)
    ap.add_argument("--precision", type=int, choices=[32, 64], default=64)
    ap.add_argument("--std", action="store_true", help="standard form (default: gauge)")
    ap.add_argument("--iord", type=int, default=3)
    ap.add_argument("--bc", choices=["periodic", "reference"], default="periodic")
    ap.add_argument("--workload", choices=["random", "deformational", "balls"], default="random")
    ap.add_argument("--adjoint", action="store_true", help="also time the step adjoint")
    a = ap.parse_args(argv)

    import torch

    from advectionhpctester_gb300 import _native
    from advectionhpctester_gb300 import mpdata as M
    from advectionhpctester_gb300 import workloads as W

    _native.load(build_if_missing=True)
    nx, ny, nz = a.grid
    ibc = (1, 1, 1) if a.bc == "periodic" else (0, 0, 0)
    dnp = np.float64 if a.precision == 64 else np.float32
    if a.workload in ("deformational", "balls"):
        if a.bc != "periodic":
            ap.error("the deformational workload is periodic")
        f = W.deformational(nx, ny, nz, dtype=dnp, balls=a.workload == "balls")
    else:
        f = W.random_fields(nx, ny, nz, ibc=ibc, seed=1, courant=0.25, dtype=dnp)
    d = {k: M.fortran_device(getattr(f, k)) for k in ("x", "u1", "u2", "u3", "h", "rhr", "bcx", "bcy")}
    del f
    ws = M.Workspace(nx, ny, nz, 1, *ibc, iord=a.iord, nonos=1, gauge=0 if a.std else 1,
                     precision=a.precision)
    args = (d["x"], d["u1"], d["u2"], d["u3"], d["h"], d["rhr"], d["bcx"], d["bcy"])
    for _ in range(a.warmup):
        ws.step(*args)
    torch.cuda.synchronize()
    ws.profile(True)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(a.steps):
        ws.step(*args)
    e1.record()
    torch.cuda.synchronize()
    st = ws.stage_times()
    ms = e0.elapsed_time(e1) / a.steps
    out = {"grid": a.grid, "workload": a.workload, "precision": a.precision,
           "form": "std" if a.std else "gauge",
           "iord": a.iord, "bc": a.bc, "ms_per_step": round(ms, 4),
           "gcell_steps_per_s": round(nx * ny * nz / (ms * 1e-3) / 1e9, 4),
           "stages_ms": {k: round(v[0] / a.steps, 4) for k, v in st.items() if v[1]}}
    if a.adjoint:
        lam = d["x"].clone()
        gu = [torch.zeros_like(d[k]) for k in ("u1", "u2", "u3")]
        adj = (d["x"], d["u1"], d["u2"], d["u3"], d["h"], d["rhr"], lam, *gu, d["bcx"], d["bcy"])
        for _ in range(a.warmup):
            ws.step_adjoint(*adj)
        torch.cuda.synchronize()
        e0.record()
        for _ in range(a.steps):
            ws.step_adjoint(*adj)
        e1.record()
        torch.cuda.synchronize()
        ams = e0.elapsed_time(e1) / a.steps
        out["adjoint_ms_per_step"] = round(ams, 4)
        out["adjoint_over_forward"] = round(ams / ms, 3)
    print(json.dumps(out))
    ws.close()


if __name__ == "__main__":
    main()
