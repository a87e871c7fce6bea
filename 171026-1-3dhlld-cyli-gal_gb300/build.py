"""Build recipe for lib/libmhdgpu.so (sm_103a) -- no cmake, one nvcc per file,
compiled in parallel.

Flags that matter for results:
* plain FP64 kernels and the context code: ``--fmad=false`` with IEEE
  division and square root, so every expression rounds exactly as the
  reference C (built without contraction) does;
* precision-form kernels: FP32 with multiply-add contraction and the fast
  (2-ulp) FP32 division and square root;
* host C: ``-ffp-contract=off`` (gcc contracts by default on Arm).
"""
import concurrent.futures as cf
import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OBJ = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "lib")
LIB = os.path.join(LIBDIR, "libmhdgpu.so")
HOSTEXE = os.path.join(LIBDIR, "mhd_disc")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_COMMON = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-I", INCLUDE, "-I", CSRC,
                      "-Xcompiler", "-fPIC,-ffp-contract=off", "-Xptxas", "-v"]
EXACT = ["--fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false"]
FP32 = ["--fmad=true", "-prec-div=false", "-prec-sqrt=false", "-ftz=true"]

UNITS = {
    "mhd_ctx.cu": EXACT,
    "mhd_fp64.cu": EXACT,
    "mhd_fp32.cu": FP32,
    "mhd_batch.cu": FP32,
}


def _sources():
    out = []
    for f in sorted(os.listdir(CSRC)):
        if f.endswith(".cu") or f.endswith(".c"):
            out.append(f)
    return out


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs.append(os.path.join(INCLUDE, "mhd_gpu.h"))
    return hs


def _compile(src):
    path = os.path.join(CSRC, src)
    obj = os.path.join(OBJ, src + ".o")
    if src.endswith(".c"):
        cmd = ["gcc", "-std=gnu11", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC",
               "-I", INCLUDE, "-I", CSRC, "-c", path, "-o", obj]
    else:
        cmd = ["nvcc"] + NVCC_COMMON + UNITS.get(src, EXACT) + ["-c", path, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    log = os.path.join(OBJ, src + ".log")
    with open(log, "w") as f:
        f.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
    if r.returncode != 0:
        raise RuntimeError("compile failed: %s\n%s" % (src, r.stderr[-4000:]))
    return obj


def build(force=False, verbose=False):
    """Compile csrc/ into lib/libmhdgpu.so; returns the library path."""
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    srcs = _sources()
    newest = max(os.path.getmtime(p) for p in [os.path.join(CSRC, s) for s in srcs] + _headers())
    newest = max(newest, os.path.getmtime(__file__), os.path.getmtime(os.path.join(PKG, "host", "mhd_disc_main.c")))
    if (not force and os.path.exists(LIB) and os.path.exists(HOSTEXE)
            and min(os.path.getmtime(LIB), os.path.getmtime(HOSTEXE)) >= newest):
        return LIB
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(_compile, srcs))
    cmd = ["nvcc"] + ARCH + ["-shared", "-o", LIB + ".tmp"] + objs + ["-lm"]
    subprocess.check_call(cmd)
    os.replace(LIB + ".tmp", LIB)
    # the C host program (the reference's main.c on the C-ABI), next to the library
    subprocess.check_call(["gcc", "-std=gnu11", "-O2", "-ffp-contract=off", "-I", INCLUDE,
                           os.path.join(PKG, "host", "mhd_disc_main.c"), "-o", HOSTEXE + ".tmp",
                           "-L", LIBDIR, "-lmhdgpu", "-Wl,-rpath,$ORIGIN"])
    os.replace(HOSTEXE + ".tmp", HOSTEXE)
    if verbose:
        for s in srcs:
            print(open(os.path.join(OBJ, s + ".log")).read())
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
