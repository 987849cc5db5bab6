"""Generates the golden vectors under tests/golden/ from the CPU oracle.

Each case stores its inputs (seeded random fields in the reference's Fortran
layout) and the oracle's psi after a few steps.  The GPU parity tests compare
the CUDA path against these files; a CPU test checks that the oracle still
reproduces them.  Regenerate with:  python -m tests.golden.make_golden
"""
import os

import numpy as np

from advectionhpctester_gb300 import workloads as W

HERE = os.path.dirname(os.path.abspath(__file__))

CASES = [
    dict(name="ref_gauge_i2", n=(13, 11, 7), ih=1, ibc=(0, 0, 0), t_adv=1, iord=2, nonos=1, opt=4,
         steps=4, seed=101, signed=False, dtype="f64"),
    dict(name="ref_std_i2_signed_ih2", n=(13, 11, 7), ih=2, ibc=(0, 0, 0), t_adv=2, iord=2, nonos=1,
         opt=4, steps=4, seed=102, signed=True, dtype="f64"),
    dict(name="per_gauge_i3", n=(12, 10, 8), ih=1, ibc=(1, 1, 1), t_adv=1, iord=3, nonos=1, opt=4,
         steps=4, seed=103, signed=False, dtype="f64"),
    dict(name="per_std_i2", n=(12, 10, 8), ih=1, ibc=(1, 1, 1), t_adv=2, iord=2, nonos=1, opt=4,
         steps=4, seed=104, signed=False, dtype="f64"),
    dict(name="mixed_std_i3", n=(11, 9, 6), ih=1, ibc=(1, 0, 0), t_adv=2, iord=3, nonos=1, opt=4,
         steps=3, seed=105, signed=False, dtype="f64"),
    dict(name="mixed_gauge_i2", n=(9, 12, 5), ih=1, ibc=(0, 1, 1), t_adv=1, iord=2, nonos=1, opt=4,
         steps=3, seed=106, signed=True, dtype="f64"),
    dict(name="upwind_only_ref", n=(10, 8, 6), ih=1, ibc=(0, 0, 0), t_adv=1, iord=1, nonos=0, opt=6,
         steps=3, seed=107, signed=False, dtype="f64"),
    dict(name="per_gauge_nonos0", n=(10, 8, 6), ih=1, ibc=(1, 1, 1), t_adv=1, iord=2, nonos=0, opt=4,
         steps=3, seed=108, signed=False, dtype="f64"),
    dict(name="per_std_i2_f32", n=(12, 10, 8), ih=1, ibc=(1, 1, 1), t_adv=2, iord=2, nonos=1, opt=4,
         steps=4, seed=109, signed=False, dtype="f32"),
    dict(name="ref_gauge_i2_f32", n=(13, 11, 7), ih=1, ibc=(0, 0, 0), t_adv=1, iord=2, nonos=1, opt=4,
         steps=4, seed=110, signed=False, dtype="f32"),
]

FIELDS = ("x", "u1", "u2", "u3", "h", "rhr", "bcx", "bcy")


def build_case(case, from_file=True):
    """Inputs of a case: from the committed file when present (so platforms
    with another numpy agree), else from the seeded generator."""
    path = os.path.join(HERE, case["name"] + ".npz")
    f = W.random_fields(*case["n"], ih=case["ih"], ibc=case["ibc"], seed=case["seed"],
                        sign_change=case["signed"])
    if case["dtype"] == "f32":
        f = f.astype(np.float32)
    if from_file and os.path.exists(path):
        z = np.load(path)
        for k in FIELDS:
            getattr(f, k)[...] = z["in_" + k]
    return f


def run_oracle(O, f, case):
    g = O.grid(f.np, f.mp, f.lp, f.ih, f.ibcx, f.ibcy, f.ibcz)
    O.advec_dwarf(g, f.x, f.bcx, f.bcy, f.u1, f.u2, f.u3, f.rhr, f.h, legacyoptmode=case["opt"],
                  t_adv=case["t_adv"], iord=case["iord"], nonos=case["nonos"], nsteps=case["steps"])


def main():
    from oracle import oracle as O
    for case in CASES:
        f = build_case(case, from_file=False)
        inputs = {"in_" + k: getattr(f, k).copy(order="F") for k in FIELDS}
        run_oracle(O, f, case)
        np.savez_compressed(os.path.join(HERE, case["name"] + ".npz"), x=f.x, **inputs)
        print(case["name"], float(np.abs(f.x).max()))


if __name__ == "__main__":
    main()
