"""Builds the native libraries in-tree.

  aphros_gb300/_build/libaphgpu.so   the CUDA library (C ABI, include/aphgpu.h)
  aphros_gb300/_build/libaphgen.so   the synthetic workload generator (host C)
  oracle/_build/liboracle.so         the CPU oracle (test infrastructure)
  oracle/_ref/ref_harness            aphros's own code, only where the
                                     reference sources are present

Plain nvcc/gcc invocations, translation units compiled in parallel, one
-gencode for sm_103a.  Run `python -m aphros_gb300.build`.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "aphros_gb300")
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
ORACLE = os.path.join(ROOT, "oracle")
# the reference installed as sources by oracle/ref/stage_reference.sh
REFERENCE_SRC = os.environ.get(
    "APHROS_REFERENCE_SRC", os.path.join(ROOT, "baseline", "_ref", "aphros", "src"))

NVCC = os.environ.get("NVCC", shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
    "-I" + os.path.join(ROOT, "include"), "--expt-relaxed-constexpr",
]
# per translation unit extra flags: the VOF/curvature arithmetic is kept free
# of fused multiply-adds so it follows the reference's rounding
CU_UNITS = {
    "api.cu": [],
    "poisson.cu": [],
    "vof.cu": ["-fmad=false"],
    "noalloc.cu": [],
    "server.cu": [],
    "batch.cu": [],
    "dump.cu": [],
    "label.cu": [],
    "fluid.cu": ["-fmad=false"],
    "partstr.cu": ["-fmad=false"],
}


def _run(cmd, cwd=None):
    r = subprocess.run(cmd, cwd=cwd, stdout=subprocess.PIPE,
                       stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s" % (" ".join(cmd), r.stdout))
    return r.stdout


def _newer(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build_cuda(verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(ROOT, "include", "aphgpu.h"))
    objs, jobs = [], []
    for unit, extra in CU_UNITS.items():
        src = os.path.join(CSRC, unit)
        obj = os.path.join(BUILD, unit + ".o")
        objs.append(obj)
        if _newer(obj, [src] + headers):
            jobs.append([NVCC] + NVCC_FLAGS + extra + ["-c", src, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        for out in ex.map(_run, jobs):
            if verbose and out.strip():
                print(out)
    lib = os.path.join(BUILD, "libaphgpu.so")
    if _newer(lib, objs):
        # --no-undefined: a missing definition fails the build, not the load
        _run([NVCC] + ARCH + ["-shared", "-o", lib] + objs +
             ["-lcudart", "-Xlinker", "--no-undefined"])
    return lib


def build_gen():
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(CSRC, "gen.c")
    lib = os.path.join(BUILD, "libaphgen.so")
    if _newer(lib, [src]):
        _run(["gcc", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
              "-o", lib, src, "-lm"])
    return lib


def build_oracle():
    out = os.path.join(ORACLE, "_build")
    os.makedirs(out, exist_ok=True)
    srcs = [os.path.join(ORACLE, "aphros_oracle.c"), os.path.join(ORACLE, "partstr_oracle.c")]
    lib = os.path.join(out, "liboracle.so")
    if _newer(lib, srcs + [os.path.join(ORACLE, "aphros_oracle.h")]):
        _run(["gcc", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
              "-o", lib] + srcs + ["-lm"])
    return lib


def build_reference():
    """aphros's own hot-path code, only where its sources exist."""
    if not os.path.isdir(REFERENCE_SRC):
        return None
    jobs = str(min(16, os.cpu_count() or 4))
    try:
        _run(["make", "-C", os.path.join(ORACLE, "ref"), "REF=" + REFERENCE_SRC, "-j" + jobs])
    except RuntimeError as e:
        # the checker is optional: the product library does not depend on it
        print("reference harness not built: %s" % str(e)[-2000:], file=sys.stderr)
        return None
    return os.path.join(ORACLE, "_ref", "ref_harness")


def build(verbose=False):
    with cf.ThreadPoolExecutor(max_workers=4) as ex:
        futs = [ex.submit(build_cuda, verbose), ex.submit(build_gen),
                ex.submit(build_oracle), ex.submit(build_reference)]
        return [f.result() for f in futs]


if __name__ == "__main__":
    for p in build(verbose="-v" in sys.argv):
        if p:
            print(p)
