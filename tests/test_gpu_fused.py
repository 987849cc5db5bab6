"""Fused single-precision step (z-marching tiles, TMA staging) against the
FP32 oracle and against the stage path, bit for bit.

The fused path serves FP32 infinite-gauge nonoscillatory steps on periodic
grids.  Grids are chosen to cover tiles whose boxes come in by TMA (inside
the grid), tiles at a periodic seam (wrapped cp.async staging), partial tiles,
grids smaller than one tile, every pass count from 2 to 4, and chunk
boundaries of the z-march (MPDATA_FUSED_KCHUNK)."""
import os

import numpy as np
import pytest

from advectionhpctester_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def M(native_lib):
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    from advectionhpctester_gb300 import mpdata
    return mpdata


class env:
    """Environment overrides read when a workspace is created."""

    def __init__(self, **kv):
        self.kv = {k: str(v) for k, v in kv.items()}

    def __enter__(self):
        self.old = {k: os.environ.get(k) for k in self.kv}
        os.environ.update(self.kv)

    def __exit__(self, *a):
        for k, v in self.old.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v


def gpu_steps(M, f, iord, steps=1, **kv):
    d = {k: M.fortran_device(getattr(f, k), dtype=f.dtype) for k in ("x", "u1", "u2", "u3", "h", "rhr")}
    with env(**kv):
        ws = M.Workspace(f.np, f.mp, f.lp, f.ih, 1, 1, 1, iord=iord, nonos=1, gauge=1,
                         precision=64 if f.dtype == np.float64 else 32)
    l0 = M.launch_count()
    for _ in range(steps):
        ws.step(d["x"], d["u1"], d["u2"], d["u3"], d["h"], d["rhr"])
    launches = M.launch_count() - l0
    out = M.to_numpy(d["x"])
    ws.close()
    return out, launches


def oracle_steps(O, f, iord, steps=1):
    g = f.copy()
    O.advec_dwarf(O.grid(g.np, g.mp, g.lp, g.ih, 1, 1, 1), g.x, g.bcx, g.bcy, g.u1, g.u2, g.u3, g.rhr, g.h,
                  legacyoptmode=4, t_adv=1, iord=iord, nonos=1, nsteps=steps)
    return g.x


CASES = [
    # (np, mp, lp, iord, steps, fields)
    (64, 64, 32, 3, 4, "deformational"),   # every tile at a seam (wrapped staging)
    (200, 96, 24, 3, 3, "random"),         # TMA tiles, seam tiles, a partial tile column
    (136, 72, 20, 4, 2, "random"),         # three passes: both ping-pong fields and extrema
    (168, 40, 12, 2, 3, "random"),         # iord=2: input psi read while psi is written
    (37, 23, 9, 3, 2, "random"),           # odd sizes, partial tiles on both axes
    (5, 3, 2, 3, 2, "random"),             # smaller than one tile: multiple wraps
]


@pytest.mark.parametrize("case", CASES, ids=lambda c: "%dx%dx%d_i%d" % c[:4])
def test_fused_matches_fp32_oracle(M, oracle, case):
    n, m, l, iord, steps, kind = case
    if kind == "deformational":
        f = W.deformational(n, m, l, dtype=np.float32)
    else:
        f = W.random_fields(n, m, l, ibc=(1, 1, 1), seed=n + m + l, courant=0.3, dtype=np.float32)
    got, launches = gpu_steps(M, f, iord, steps)
    want = oracle_steps(oracle, f, iord, steps)
    np.testing.assert_array_equal(W.interior(got), W.interior(want))
    # the fused step is one upwind+pseudo launch, then per pass a pseudo
    # launch (passes after the first) and a limiter+update launch
    assert launches == steps * (1 + 1 + 2 * (iord - 2)), launches


@pytest.mark.parametrize("kchunk", [1, 3, 7, 64])
def test_fused_chunk_boundaries(M, oracle, kchunk):
    """The z-march restarts at every chunk; its start-up planes must reproduce
    the neighbour chunk's values exactly."""
    f = W.random_fields(104, 48, 21, ibc=(1, 1, 1), seed=11, courant=0.3, dtype=np.float32)
    got, _ = gpu_steps(M, f, 3, 2, MPDATA_FUSED_KCHUNK=kchunk)
    want = oracle_steps(oracle, f, 3, 2)
    np.testing.assert_array_equal(W.interior(got), W.interior(want))


def test_fused_equals_stage_path_full_size(M):
    """The headline grid (512x512x128 deformational flow, iord=3) in FP32:
    the fused path and the stage path give the same bits after 3 steps, and
    the limiter-bound check sees the same (zero) violations."""
    f = W.deformational(512, 512, 128, dtype=np.float32)
    outs, viol = [], []
    for fused in ("1", "0"):
        d = {k: M.fortran_device(getattr(f, k), dtype=np.float32) for k in ("x", "u1", "u2", "u3", "h", "rhr")}
        with env(MPDATA_FUSED=fused):
            ws = M.Workspace(512, 512, 128, 1, 1, 1, 1, iord=3, nonos=1, gauge=1, precision=32)
        for _ in range(3):
            ws.step(d["x"], d["u1"], d["u2"], d["u3"], d["h"], d["rhr"])
        viol.append(ws.bound_violations(d["x"], 1e-6))
        outs.append(M.to_numpy(d["x"]))
        ws.close()
        del d
    np.testing.assert_array_equal(W.interior(outs[0]), W.interior(outs[1]))
    assert viol[0] == viol[1] == 0, viol


def test_fused_stage_names(M):
    """Per-stage timing reports the fused kernels under their own names."""
    f = W.random_fields(96, 48, 16, ibc=(1, 1, 1), seed=3, dtype=np.float32)
    d = {k: M.fortran_device(getattr(f, k), dtype=np.float32) for k in ("x", "u1", "u2", "u3", "h", "rhr")}
    ws = M.Workspace(96, 48, 16, 1, 1, 1, 1, iord=3, nonos=1, gauge=1, precision=32)
    ws.profile(True)
    ws.step(d["x"], d["u1"], d["u2"], d["u3"], d["h"], d["rhr"])
    st = {k: v[1] for k, v in ws.stage_times().items() if v[1]}
    ws.close()
    assert st == {"fused_upwind_pseudo": 1, "fused_pseudo": 1, "fused_limit_update": 2}, st


def bits(a):
    return np.ascontiguousarray(W.interior(a)).view(np.uint32)


def test_fused_mixed_unit_density(M, oracle):
    """Unit densities everywhere except a perturbed box: blocks and steps
    whose densities are all exactly 1 take the shortcut without products and
    quotients by them, the others the full arithmetic; every bit agrees."""
    f = W.random_fields(136, 72, 20, ibc=(1, 1, 1), seed=21, courant=0.3, dtype=np.float32)
    hi, ri = W.interior(f.h), W.interior(f.rhr)
    keep_h, keep_r = hi[40:70, 10:30, 6:9].copy(), ri[40:70, 10:30, 6:9].copy()
    hi[...] = 1.0
    ri[...] = 1.0
    hi[40:70, 10:30, 6:9] = keep_h
    ri[40:70, 10:30, 6:9] = keep_r
    got, _ = gpu_steps(M, f, 3, 3)
    want = oracle_steps(oracle, f, 3, 3)
    np.testing.assert_array_equal(bits(got), bits(want))


@pytest.mark.parametrize("fused", ["1", "0"], ids=["fused", "stages"])
def test_fp32_signed_zero_extrema(M, oracle, fused):
    """A field with blocks of +0 and -0 and a sign change: star extrema that
    are zeros take the compare-and-select fold in the reference's tree order,
    whose ties keep the earlier operand; raw bit patterns agree with the
    oracle, signs of zeros included, on the fused path and the stage path."""
    f = W.random_fields(104, 56, 12, ibc=(1, 1, 1), seed=5, courant=0.3, dtype=np.float32)
    x = W.interior(f.x)
    x[10:50, 5:30, 2:7] = 0.0
    x[60:90, 20:40, 4:10] = -0.0
    x[30:40, 40:50, :] *= -1.0
    got, _ = gpu_steps(M, f, 3, 2, MPDATA_FUSED=fused)
    want = oracle_steps(oracle, f, 3, 2)
    np.testing.assert_array_equal(bits(got), bits(want))
