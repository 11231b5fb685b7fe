"""Builds librpd_gb300.so in-tree (libmat_gb300/librpd_gb300.so).

Every CUDA translation unit is compiled for sm_103a only
(-gencode arch=compute_103a,code=sm_103a).  The clipper and the pair/kNN
kernels are compiled with -fmad=false: the reference's float and double
expressions are evaluated one IEEE rounding at a time, as its source states
them (FMA appears only where the code asks for it explicitly).  Translation
units compile in parallel; the CUDA runtime is linked statically.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "librpd_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2",
              "-Xptxas", "-O3", "-I" + os.path.join(ROOT, "include")]
CUDA_UNITS = {
    "rpd_clip.cu": ["-fmad=false"],
    "rpd_pairs.cu": ["-fmad=false"],
    "rpd_noalloc.cu": [],
    "rpd_mlp.cu": [],
    "rpd_prep.cu": [],
    "rpd_topo.cu": ["-fmad=false"],
    "rpd_poly.cu": ["-fmad=false"],
    "rpd_dist2mat.cu": ["-fmad=false"],
    "rpd_partial.cu": [],
    "rpd_sort.cu": [],
    "rpd_powercell.cu": ["-fmad=false"],
    "rpd_cc.cu": [],
}
CXX_UNITS = ["rpd_api.cpp", "rpd_mesh.cpp", "rpd_batch.cpp"]


def nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def cuda_home():
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc())))


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n%s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stdout + r.stderr


def _deps():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + \
        [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))]


def _stale(out, srcs):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(s) > t for s in srcs)


def build(force=False, verbose=False, extra_nvcc=()):
    """Compiles the library if any source changed; returns its path."""
    deps = _deps() + [__file__]
    if not force and not _stale(LIB, deps):
        return LIB
    os.makedirs(OBJ, exist_ok=True)
    nv = nvcc()
    jobs = []
    for f, extra in CUDA_UNITS.items():
        o = os.path.join(OBJ, f + ".o")
        jobs.append([nv, "-c", os.path.join(CSRC, f), "-o", o] + ARCH + NVCC_FLAGS +
                    list(extra) + list(extra_nvcc) + (["-Xptxas", "-v"] if verbose else []))
    inc = os.path.join(cuda_home(), "include")
    for f in CXX_UNITS:
        o = os.path.join(OBJ, f + ".o")
        jobs.append(["g++", "-c", os.path.join(CSRC, f), "-o", o, "-O2", "-fPIC", "-std=c++17",
                     "-I" + inc, "-I" + os.path.join(ROOT, "include")])
    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        outs = list(ex.map(_run, jobs))
    if verbose:
        for o in outs:
            if o.strip():
                print(o)
    objs = [os.path.join(OBJ, f + ".o") for f in list(CUDA_UNITS) + CXX_UNITS]
    tmp = LIB + ".tmp"
    _run([nv, "-shared", "-o", tmp] + ARCH + objs + ["-cudart", "static"])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="-f" in sys.argv, verbose="-v" in sys.argv))
