"""GPU parity of the batched step (many tracers sharing a velocity, uneven
independent domains, CUDA-graph replay, autotuned tile shapes) against the
CPU oracle run problem by problem."""
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


def dev(M, f):
    return {k: M.fortran_device(getattr(f, k)) for k in ("x", "u1", "u2", "u3", "h", "rhr", "bcx", "bcy")}


def oracle_steps(oracle, f, gauge, iord, steps, nonos=1):
    g = f.copy()
    oracle.advec_dwarf(oracle.grid(g.np, g.mp, g.lp, g.ih, g.ibcx, g.ibcy, g.ibcz), g.x, g.bcx, g.bcy,
                       g.u1, g.u2, g.u3, g.rhr, g.h, legacyoptmode=4 if iord >= 2 else 6,
                       t_adv=1 if gauge else 2, iord=max(iord, 2), nonos=nonos, nsteps=steps)
    return g.x


def tracers(n, shape, ibc, seed):
    base = W.random_fields(*shape, ibc=ibc, seed=seed)
    out = []
    for t in range(n):
        f = base.copy()
        rng = np.random.default_rng(seed + 100 + t)
        f.x[...] = rng.uniform(0.5, 1.5, f.x.shape) if t % 2 == 0 else rng.uniform(-1, 1, f.x.shape)
        f.bcx[...] = rng.uniform(0.5, 1.5, f.bcx.shape)
        f.bcy[...] = rng.uniform(0.5, 1.5, f.bcy.shape)
        out.append(f)
    return out


@pytest.mark.parametrize("ibc", [(1, 1, 1), (0, 0, 0)])
@pytest.mark.parametrize("iord", [2, 3])
def test_tracers_sharing_velocity(M, oracle, ibc, iord):
    """K tracers, one velocity group, mixed forms: each matches its own
    single-field oracle run bit for bit."""
    fs = tracers(5, (13, 11, 7), ibc, seed=21)
    forms = [1, 0, 1, 1, 0]
    probs = [dict(np=13, mp=11, lp=7, ibcx=ibc[0], ibcy=ibc[1], ibcz=ibc[2], gauge=g, velocity_group=7)
             for g in forms]
    b = M.Batch(probs, iord=iord)
    ds = [dev(M, f) for f in fs]
    shared = ds[0]
    for p, d in enumerate(ds):
        b.set(p, d["x"], shared["u1"], shared["u2"], shared["u3"], shared["h"], shared["rhr"], d["bcx"], d["bcy"])
    for _ in range(3):
        b.step()
    for p, (f, d) in enumerate(zip(fs, ds)):
        np.testing.assert_array_equal(M.to_numpy(d["x"]), oracle_steps(oracle, f, forms[p], iord, 3),
                                      err_msg="tracer %d" % p)
    b.close()


def test_uneven_domains(M, oracle):
    """Independent domains of different sizes, boundaries and forms."""
    specs = [((32, 32, 32), (1, 1, 1), 1), ((17, 9, 5), (0, 0, 0), 0), ((40, 20, 6), (1, 0, 1), 1),
             ((8, 8, 8), (0, 1, 0), 0), ((33, 3, 2), (1, 1, 1), 0), ((64, 16, 4), (0, 0, 0), 1)]
    fs = [W.random_fields(*n, ibc=ibc, seed=50 + q) for q, (n, ibc, _) in enumerate(specs)]
    probs = [dict(np=n[0], mp=n[1], lp=n[2], ibcx=ibc[0], ibcy=ibc[1], ibcz=ibc[2], gauge=g)
             for (n, ibc, g) in specs]
    b = M.Batch(probs, iord=2)
    ds = [dev(M, f) for f in fs]
    for p, d in enumerate(ds):
        b.set(p, d["x"], d["u1"], d["u2"], d["u3"], d["h"], d["rhr"], d["bcx"], d["bcy"])
    b.step()
    b.step()
    for p, (f, d) in enumerate(zip(fs, ds)):
        np.testing.assert_array_equal(M.to_numpy(d["x"]), oracle_steps(oracle, f, specs[p][2], 2, 2),
                                      err_msg="domain %d" % p)
    b.close()


def test_graph_replay_and_tuning(M, oracle):
    """Tuning leaves psi untouched; graph replay gives the same bits as eager
    launches, also after the arrays are swapped between steps."""
    import torch
    specs = [(24, 20, 12), (16, 16, 16), (30, 10, 8)]
    fs = [W.random_fields(*n, ibc=(1, 1, 1), seed=70 + q) for q, n in enumerate(specs)]
    probs = [dict(np=n[0], mp=n[1], lp=n[2], gauge=q % 2) for q, n in enumerate(specs)]
    b = M.Batch(probs, iord=3)
    ds = [dev(M, f) for f in fs]
    for p, d in enumerate(ds):
        b.set(p, d["x"], d["u1"], d["u2"], d["u3"], d["h"], d["rhr"])
    before = [d["x"].clone() for d in ds]
    bx, by = b.tune()
    assert bx * by in (128, 256) and bx >= 16
    for d, x0 in zip(ds, before):
        assert torch.equal(d["x"], x0)
    b.graph(True)
    b.step()
    b.step()
    # swap in fresh copies of the inputs: the graph reads the new pointers
    ds2 = [dev(M, f) for f in fs]
    for p, d in enumerate(ds2):
        b.set(p, d["x"], d["u1"], d["u2"], d["u3"], d["h"], d["rhr"])
    b.step()
    torch.cuda.synchronize()
    for p, (f, d, d2) in enumerate(zip(fs, ds, ds2)):
        ref2 = oracle_steps(oracle, f, p % 2, 3, 2)
        np.testing.assert_array_equal(M.to_numpy(d["x"]), ref2, err_msg="graph domain %d" % p)
        ref1 = oracle_steps(oracle, f, p % 2, 3, 1)
        np.testing.assert_array_equal(M.to_numpy(d2["x"]), ref1, err_msg="swapped domain %d" % p)
    b.close()


def test_ce_advection_mirror(M, oracle):
    """CE_advection with six dry and two moist fields, mpdata_alg_choice 0:
    th/qv/qc standard, u/v/w/tht/pstr gauge."""
    names = ["th", "u", "v", "w", "tht", "pstr", "qv", "qc"]
    fs = tracers(len(names), (12, 10, 6), (0, 0, 0), seed=90)
    ds = [dev(M, f) for f in fs]
    sh = ds[0]
    kw = {n: (d["x"], d["bcx"], d["bcy"]) for n, d in zip(names, ds)}
    M.ce_advection(0, 0, 0, 0, 0, 0, 12, 10, 6, 1, sh["rhr"], sh["h"], sh["u1"], sh["u2"], sh["u3"], **kw)
    forms = {"th": 0, "qv": 0, "qc": 0}
    for n, f, d in zip(names, fs, ds):
        ref = oracle_steps(oracle, f, forms.get(n, 1), 2, 1)
        np.testing.assert_array_equal(M.to_numpy(d["x"]), ref, err_msg=n)


def test_batch_rejects_bad_input(M):
    with pytest.raises(M.MpdataError):  # sharing a velocity needs equal grids
        M.Batch([dict(np=8, mp=8, lp=8, velocity_group=1), dict(np=9, mp=8, lp=8, velocity_group=1)])
    b = M.Batch([dict(np=8, mp=8, lp=8)])
    with pytest.raises(M.MpdataError):  # step before the arrays are set
        b.step()
    b.close()


@pytest.mark.parametrize("density", ["unit", "one_cell_off", "random"])
@pytest.mark.parametrize("shape", [(32, 4), (16, 8)])
def test_interior_tiles_velocity_group(M, oracle, shape, density):
    """Three tracers of one velocity group on an 80-wide grid: interior warps
    of the tile kernels read the group's precomputed first-pass terms and the
    pair sums, and take the unit-density bodies (h = rhr = 1, or all but one
    cell) and the block-compacted limiter ratios, for the default and the 16x8
    tile shapes.  Bit for bit against the oracle."""
    ibc = (1, 1, 1)
    fs = tracers(3, (80, 12, 8), ibc, seed=61)
    for f in fs:
        if density == "random":
            continue
        f.h[...] = 1.0
        f.rhr[...] = 1.0
        if density == "one_cell_off":
            f.h[45, 5, 4] = 1.125
            f.rhr[45, 5, 4] = 0.875
    forms = [1, 0, 1]
    probs = [dict(np=80, mp=12, lp=8, ibcx=1, ibcy=1, ibcz=1, gauge=g, velocity_group=3) for g in forms]
    b = M.Batch(probs, iord=3)
    b.shape(*shape)
    ds = [dev(M, f) for f in fs]
    shared = ds[0]
    for p, d in enumerate(ds):
        b.set(p, d["x"], shared["u1"], shared["u2"], shared["u3"], shared["h"], shared["rhr"], d["bcx"], d["bcy"])
    for _ in range(3):
        b.step()
    for p, (f, d) in enumerate(zip(fs, ds)):
        np.testing.assert_array_equal(M.to_numpy(d["x"]), oracle_steps(oracle, f, forms[p], 3, 3),
                                      err_msg="tracer %d" % p)
    b.close()


def dev32(M, f):
    return {k: M.fortran_device(getattr(f, k), dtype=np.float32) for k in
            ("x", "u1", "u2", "u3", "h", "rhr", "bcx", "bcy")}


@pytest.mark.parametrize("iord", [2, 3])
def test_fp32_batch_fused_and_tile_problems(M, oracle, iord):
    """FP32: periodic gauge problems of uneven sizes (and a velocity group of
    three tracers) run on the fused kernels, one launch per kernel for all of
    them; walls and the standard form run on the tile kernels of the same
    batch.  Tuning leaves every psi untouched; graph replay and eager steps
    give each problem the FP32 oracle's bits."""
    import torch
    specs = [((200, 40, 12), (1, 1, 1), 1, None), ((37, 23, 9), (1, 1, 1), 1, None),
             ((5, 3, 2), (1, 1, 1), 1, None), ((72, 48, 10), (1, 1, 1), 1, 4), ((72, 48, 10), (1, 1, 1), 1, 4),
             ((72, 48, 10), (1, 1, 1), 1, 4), ((24, 20, 6), (0, 0, 0), 1, None), ((30, 16, 5), (1, 1, 1), 0, None),
             ((40, 12, 6), (1, 0, 1), 1, None)]
    fs = []
    for q, (n, ibc, g, grp) in enumerate(specs):
        seed = 400 if grp is not None else 300 + q
        f = W.random_fields(*n, ibc=ibc, seed=seed, courant=0.3, dtype=np.float32)
        if grp is not None:  # tracers of one velocity: own psi, shared u, h, rhr
            f.x[...] = np.random.default_rng(500 + q).uniform(0.5, 1.5, f.x.shape).astype(np.float32)
        fs.append(f)
    probs = [dict(np=n[0], mp=n[1], lp=n[2], ibcx=ibc[0], ibcy=ibc[1], ibcz=ibc[2], gauge=g,
                  velocity_group=grp if grp is not None else 100 + q)
             for q, (n, ibc, g, grp) in enumerate(specs)]
    b = M.Batch(probs, iord=iord, nonos=1, precision=32)
    ds = [dev32(M, f) for f in fs]
    shared = ds[3]
    for p, d in enumerate(ds):
        v = shared if specs[p][3] is not None else d
        b.set(p, d["x"], v["u1"], v["u2"], v["u3"], v["h"], v["rhr"], d["bcx"], d["bcy"])
    before = [d["x"].clone() for d in ds]
    b.tune()
    for d, x0 in zip(ds, before):
        assert torch.equal(d["x"], x0)
    b.step()
    b.graph(True)
    b.step()
    b.step()
    torch.cuda.synchronize()
    for p, (f, d) in enumerate(zip(fs, ds)):
        g = f if specs[p][3] is None else fs[3]
        ref = f.copy()
        for k in ("u1", "u2", "u3", "h", "rhr"):
            getattr(ref, k)[...] = getattr(g, k)
        want = oracle_steps(oracle, ref, specs[p][2], iord, 3)
        np.testing.assert_array_equal(W.interior(M.to_numpy(d["x"])), W.interior(want), err_msg="problem %d" % p)
    b.close()


def test_fp32_batch_all_fused_launches(M, oracle):
    """A batch whose problems all take the fused kernels launches each fused
    kernel once per pass for all of them (iord=3: four launches a step)."""
    specs = [(64, 32, 16), (32, 32, 32), (96, 24, 8)]
    fs = [W.random_fields(*n, ibc=(1, 1, 1), seed=600 + q, courant=0.3, dtype=np.float32)
          for q, n in enumerate(specs)]
    b = M.Batch([dict(np=n[0], mp=n[1], lp=n[2]) for n in specs], iord=3, nonos=1, precision=32)
    ds = [dev32(M, f) for f in fs]
    for p, d in enumerate(ds):
        b.set(p, d["x"], d["u1"], d["u2"], d["u3"], d["h"], d["rhr"])
    l0 = M.launch_count()
    b.step()
    assert M.launch_count() - l0 == 4
    b.step()
    for p, (f, d) in enumerate(zip(fs, ds)):
        np.testing.assert_array_equal(W.interior(M.to_numpy(d["x"])), W.interior(oracle_steps(oracle, f, 1, 3, 2)))
    b.close()
