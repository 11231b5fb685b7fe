"""Builds the oracle (test infrastructure only).

* ``liboracle.so`` from rpd_oracle.c -- the CPU restatement of the reference's
  RPD path, compiled with -ffp-contract=off so every float/double operation
  is one IEEE-rounded step, as the reference's sources state them.
* ``_ref/libref.so`` -- the reference's own clipping kernel
  (src/rpd3d/convex_cell.cu) compiled for the CPU through ref_shim/, built
  only when the reference sources are present (they are not on the GPU
  machines; the tests that need it skip there).
* ``_ref/libreftopo.so`` -- the reference's own per-cell topology
  (src/rpd3d_base/voronoi_defs.cxx) behind ref_topo_driver.cpp, same
  condition.
* ``_ref/librefbgeo.so`` -- the reference's own Houdini geometry writer
  (src/IO/IO_CUDA/io_utils.cpp) behind ref_bgeo_driver.cpp, through
  ref_io_shim/ (CUDA's vector structs, an empty json header), same
  condition.
* ``_ref/librefpc.so`` -- the reference's own power-cell construction
  (src/rpd3d_base/rpd_update.cxx:1-521, fed to the compiler on its standard
  input) behind ref_powercell_driver.cpp, through ref_pc_shim/ (PowerCell,
  a surface mesh from arrays), same condition.
* ``_ref/librefd2m.so`` -- the reference's own dist2mat distance functions
  (src/dist2mat/dist2mat.cu) behind ref_dist2mat_driver.cu, same condition.

The reference sources are found through $RPD_REFERENCE_ROOT or, without it,
as a checkout named ``reference`` beside this repository.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def _reference_root():
    """The libmat source checkout: $RPD_REFERENCE_ROOT, else a checkout named
    ``reference`` beside this repository; "" (every _ref build skips) when
    neither holds libmat's sources."""
    env = os.environ.get("RPD_REFERENCE_ROOT")
    cand = env if env else os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")
    return cand if os.path.isfile(os.path.join(cand, "src", "rpd3d", "convex_cell.cu")) else ""


REF_ROOT = _reference_root()


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))


def _stale(out, srcs):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(s) > t for s in srcs)


def build_oracle(force=False):
    src = os.path.join(HERE, "rpd_oracle.c")
    hdr = os.path.join(HERE, "rpd_oracle.h")
    out = os.path.join(HERE, "liboracle.so")
    if force or _stale(out, [src, hdr]):
        _run(["gcc", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
              "-std=gnu11", "-o", out, src, "-lm"])
    return out


def build_ref(force=False):
    """Returns the path of _ref/libref.so, or None without reference sources."""
    if not REF_ROOT:
        return None
    kernel = os.path.join(REF_ROOT, "src", "rpd3d", "convex_cell.cu")
    if not os.path.exists(kernel):
        return None
    outdir = os.path.join(HERE, "_ref")
    os.makedirs(outdir, exist_ok=True)
    out = os.path.join(outdir, "libref.so")
    drv = os.path.join(HERE, "ref_driver.cpp")
    shim = os.path.join(HERE, "ref_shim", "cuda_runtime.h")
    if force or _stale(out, [drv, shim, kernel]):
        _run(["g++", "-O2", "-fPIC", "-shared", "-std=c++17", "-DNDEBUG",
              "-ffp-contract=off", "-w", "-pthread",
              "-I" + os.path.join(HERE, "ref_shim"),
              "-I" + os.path.join(REF_ROOT, "include"),
              "-I" + os.path.join(REF_ROOT, "src", "rpd3d"),
              "-I" + os.path.join(REF_ROOT, "src", "rpd3d_base"),
              "-x", "c++", drv, "-o", out])
    return out


def build_ref_topo(force=False):
    """Returns the path of _ref/libreftopo.so -- the reference's own
    ConvexCellHost topology (src/rpd3d_base/voronoi_defs.cxx) behind
    ref_topo_driver.cpp -- or None without reference sources."""
    if not REF_ROOT:
        return None
    defs = os.path.join(REF_ROOT, "src", "rpd3d_base", "voronoi_defs.cxx")
    if not os.path.exists(defs):
        return None
    outdir = os.path.join(HERE, "_ref")
    os.makedirs(outdir, exist_ok=True)
    out = os.path.join(outdir, "libreftopo.so")
    drv = os.path.join(HERE, "ref_topo_driver.cpp")
    if force or _stale(out, [drv, defs, os.path.join(HERE, "rpd_oracle.h")]):
        _run(["g++", "-O2", "-fPIC", "-shared", "-std=c++17", "-DNDEBUG",
              "-ffp-contract=off", "-w", "-pthread",
              "-I" + os.path.join(REF_ROOT, "include"),
              "-I" + os.path.join(REF_ROOT, "src", "rpd3d_base"),
              drv, defs, "-o", out])
    return out


# rpd_update.cxx up to the end of update_pc_edge_cc_info: get_all_voro_info,
# its helpers, the surface groups and the component updates; the rest of the
# file needs the sphere model and geogram
_PC_LAST_LINE = 521


def build_ref_powercell(force=False):
    """Returns the path of _ref/librefpc.so -- the reference's own power-cell
    construction (src/rpd3d_base/rpd_update.cxx:1-521, read into the
    compiler's standard input, never copied) behind ref_powercell_driver.cpp
    with ref_pc_shim/ -- or None without reference sources or when those
    lines do not end where update_pc_edge_cc_info does."""
    if not REF_ROOT:
        return None
    base = os.path.join(REF_ROOT, "src", "rpd3d_base")
    upd = os.path.join(base, "rpd_update.cxx")
    defs = os.path.join(base, "voronoi_defs.cxx")
    if not (os.path.exists(upd) and os.path.exists(defs)):
        return None
    outdir = os.path.join(HERE, "_ref")
    os.makedirs(outdir, exist_ok=True)
    out = os.path.join(outdir, "librefpc.so")
    drv = os.path.join(HERE, "ref_powercell_driver.cpp")
    shim = os.path.join(HERE, "ref_pc_shim")
    deps = [drv, upd, defs, os.path.join(HERE, "rpd_oracle.h"),
            os.path.join(shim, "medial_sphere.h"), os.path.join(shim, "input_types.h")]
    if force or _stale(out, deps):
        with open(upd) as f:
            lines = f.readlines()
        head = "".join(lines[:_PC_LAST_LINE])
        tail = "".join(lines[_PC_LAST_LINE:_PC_LAST_LINE + 3])
        if ("void update_pc_edge_cc_info(PowerCell& pcell)" not in head
                or "update_sphere_type_based_on_pcells" not in tail
                or not lines[_PC_LAST_LINE - 1].startswith("}")):
            return None
        cmd = ["g++", "-O2", "-fPIC", "-shared", "-std=c++17", "-DNDEBUG",
               "-ffp-contract=off", "-w", "-pthread", "-I" + shim,
               "-I" + os.path.join(REF_ROOT, "include"), "-I" + base,
               drv, defs, "-x", "c++", "-", "-o", out]
        r = subprocess.run(cmd, input=head, capture_output=True, text=True, cwd=outdir)
        if r.returncode != 0:
            raise RuntimeError("build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return out


def build_ref_bgeo(force=False):
    """Returns the path of _ref/librefbgeo.so -- the reference's own Houdini
    geometry writer behind ref_bgeo_driver.cpp -- or None without reference
    sources."""
    if not REF_ROOT:
        return None
    io_dir = os.path.join(REF_ROOT, "src", "IO", "IO_CUDA")
    src = os.path.join(io_dir, "io_utils.cpp")
    if not os.path.exists(src):
        return None
    outdir = os.path.join(HERE, "_ref")
    os.makedirs(outdir, exist_ok=True)
    out = os.path.join(outdir, "librefbgeo.so")
    drv = os.path.join(HERE, "ref_bgeo_driver.cpp")
    shim = os.path.join(HERE, "ref_io_shim")
    if force or _stale(out, [drv, src, os.path.join(shim, "cuda_runtime.h")]):
        _run(["g++", "-O2", "-fPIC", "-shared", "-std=c++17", "-DNDEBUG", "-w",
              "-I" + shim, "-I" + io_dir, drv, src, "-o", out])
    return out


def build_ref_dist2mat(force=False):
    """Returns the path of _ref/librefd2m.so -- the reference's own dist2mat
    distance functions (src/dist2mat/dist2mat.cu) behind
    ref_dist2mat_driver.cu, compiled by nvcc for the host -- or None without
    reference sources (or without nvcc)."""
    if not REF_ROOT:
        return None
    src_dir = os.path.join(REF_ROOT, "src", "dist2mat")
    src = os.path.join(src_dir, "dist2mat.cu")
    if not os.path.exists(src):
        return None
    import shutil
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        return None
    outdir = os.path.join(HERE, "_ref")
    os.makedirs(outdir, exist_ok=True)
    out = os.path.join(outdir, "librefd2m.so")
    drv = os.path.join(HERE, "ref_dist2mat_driver.cu")
    if force or _stale(out, [drv, src]):
        _run([nvcc, "-O2", "-shared", "-std=c++17", "-w",
              "-gencode", "arch=compute_103a,code=sm_103a",
              "-Xcompiler", "-fPIC,-ffp-contract=off",
              "-I" + os.path.join(REF_ROOT, "include"), "-I" + src_dir, drv, "-o", out])
    return out


if __name__ == "__main__":
    print(build_oracle(force="-f" in sys.argv))
    print(build_ref(force="-f" in sys.argv))
    print(build_ref_topo(force="-f" in sys.argv))
    print(build_ref_powercell(force="-f" in sys.argv))
    print(build_ref_bgeo(force="-f" in sys.argv))
    print(build_ref_dist2mat(force="-f" in sys.argv))
