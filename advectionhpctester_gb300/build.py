"""Build recipe of the CUDA library (nvcc, sm_103a only, in-tree output).

Compiles every translation unit under csrc/ in parallel and links
advectionhpctester_gb300/_lib/libmpdata_gb300.so.  The stage kernels are
compiled with --fmad=false: the strict path evaluates every expression with
the reference's rounding (IEEE add/mul/div, no contraction); kernels that
want fused multiply-adds call fma() explicitly.
"""
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_lib")
LIB = os.path.join(OUT, "libmpdata_gb300.so")
INCLUDE = os.path.join(os.path.dirname(PKG), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC",
                     "-I" + INCLUDE, "-I" + CSRC]
# Extra nvcc flags for tuning sweeps (e.g. "-DMPDATA_FZ_TY=16"); a build with
# them is never up to date with a default build.
EXTRA = os.environ.get("MPDATA_NVCC_EXTRA", "").split()


def nvcc():
    exe = shutil.which("nvcc")
    if exe:
        return exe
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found; the CUDA toolkit is required to build the MPDATA library")


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _deps():
    return _sources() + sorted(glob.glob(os.path.join(CSRC, "*.cuh"))) + [os.path.join(INCLUDE, "mpdata.h")]


def up_to_date():
    if not os.path.exists(LIB) or EXTRA:
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(d) <= t for d in _deps())


def build(force=False, verbose=False):
    """Compile and link the library; returns its path."""
    if not force and up_to_date():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    exe = nvcc()
    objs = []
    cmds = []
    for src in _sources():
        obj = os.path.join(OUT, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        cmds.append([exe, *NVCC_FLAGS, *EXTRA, "-c", src, "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n%s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr)

    with cf.ThreadPoolExecutor(max_workers=max(1, len(cmds))) as ex:
        list(ex.map(run, cmds))
    tmp = LIB + ".tmp%d" % os.getpid()
    run([exe, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"])
    os.replace(tmp, LIB)
    for o in objs:
        os.remove(o)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
