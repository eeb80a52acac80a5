"""Builds the CUDA C-ABI library in-tree:  clm.jl_gb300/lib/libclmgb.so

Each translation unit in csrc/ is compiled by nvcc for sm_103a only, in parallel,
with --fmad=false (the Float64 reference never fuses a*b+c) and -lineinfo for
ncu source attribution, then linked into one shared library with a static CUDA
runtime.  No cmake.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))   # clm.jl_gb300/
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
LIBDIR = os.path.join(PKG, "lib")
OBJDIR = os.path.join(LIBDIR, "obj")
LIB = os.path.join(LIBDIR, "libclmgb.so")
PROBE_SRC = os.path.join(PKG, "probe", "fp64_probe.cu")
PROBE_LIB = os.path.join(LIBDIR, "libclmgb_probe.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "--fmad=false", "-lineinfo", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-fno-fast-math", "--extended-lambda"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _deps():
    hdrs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hdrs.append(os.path.join(ROOT, "include", "clmgb.h"))
    return hdrs


def _git_desc():
    try:
        return subprocess.check_output(["git", "-C", ROOT, "describe", "--always", "--dirty"],
                                       stderr=subprocess.DEVNULL).decode().strip()
    except Exception:
        return "dev"


def build_probe(force=False):
    """libclmgb_probe.so: the FP64 throughput probe bench.py measures the roofline with."""
    deps = [PROBE_SRC, os.path.join(CSRC, "clm_math.h"), os.path.join(CSRC, "clm_math_tables.h"), __file__]
    if not force and os.path.exists(PROBE_LIB) and os.path.getmtime(PROBE_LIB) > max(map(os.path.getmtime, deps)):
        return PROBE_LIB
    os.makedirs(LIBDIR, exist_ok=True)
    tmp = PROBE_LIB + ".tmp%d" % os.getpid()
    subprocess.check_call([_nvcc()] + NVCC_FLAGS + ARCH + ["-shared", PROBE_SRC, "-o", tmp])
    os.replace(tmp, PROBE_LIB)
    return PROBE_LIB


def build(force=False, verbose=False, ptxas_v=False):
    build_probe(force)
    srcs = sources()
    newest = max(os.path.getmtime(p) for p in srcs + _deps() + [__file__])
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) > newest:
        return LIB
    os.makedirs(OBJDIR, exist_ok=True)
    nvcc = _nvcc()
    desc = ['-DCLMGB_GIT_DESC="%s"' % _git_desc()]

    def compile_one(src):
        obj = os.path.join(OBJDIR, os.path.basename(src) + ".o")
        cmd = [nvcc] + NVCC_FLAGS + ARCH + desc + (["-Xptxas", "-v"] if ptxas_v else []) + ["-c", src, "-o", obj]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
        out = r.stdout.decode()
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s" % (src, out))
        return obj, out

    with ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        results = list(ex.map(compile_one, srcs))
    if ptxas_v or verbose:
        for _, out in results:
            if out.strip():
                print(out)
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = [nvcc, "-shared"] + ARCH + ["-o", tmp] + [o for o, _ in results]
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv, ptxas_v="--ptxas" in sys.argv))
