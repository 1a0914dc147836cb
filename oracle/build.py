"""Build recipe for the oracle (test infrastructure only).

- ``liboracle.so``: the CPU restatement ``oracle/rt_cpu_ref.cpp``.
- ``_ref/libref.so``: the reference's own OpenCL kernels
  (``src/kernel/{bvh-builder,bvh-builder-sort,trace-bvh,shadow-trace-bvh,
  ray-shader,secondary-ray-generator,primary-ray-generator}.cl``) compiled
  unmodified for the CPU through ``ref_shim/cl_shim_body.hpp`` (the two
  work-group kernels of the LBVH build as emulated work-groups,
  ``ref_shim/ref_emit.cpp``), plus the host loop driver
  ``ref_shim/ref_driver.cpp``.  Built only where the reference
  checkout exists (``REFERENCE_ROOT``, default ``/root/reference``); its
  outputs stay in the git-ignored ``oracle/_ref/``.

Both use ``-ffp-contract=off`` so that single-precision arithmetic is not
fused, matching the CUDA path (compiled with ``--fmad=false``).
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
REFERENCE_ROOT = os.environ.get("REFERENCE_ROOT", "/root/reference")
CXX = os.environ.get("CXX", "g++")
FLAGS = ["-std=c++17", "-O3", "-fPIC", "-ffp-contract=off", "-fno-strict-aliasing", "-pthread"]

REF_UNITS = ["ref_bvh", "ref_emit", "ref_sort", "ref_trace", "ref_shadow", "ref_shade",
             "ref_secondary", "ref_primary", "ref_driver", "ref_mangle", "ref_obj", "ref_sah"]
# the reference's host sources its OBJ import and CPU SAH BVH need, compiled
# where they lie
REF_HOST_SOURCES = ["obj-loader", "cl_aux", "mesh", "vector", "material", "bbox", "bvh"]
# per-unit flags: mangler.cl has no fp64 pragma, so its constants are floats
REF_UNIT_FLAGS = {"ref_mangle": ["-fsingle-precision-constant"]}


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s" % (" ".join(cmd), r.stderr[-4000:]))


def _stale(out, srcs):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(s) > t for s in srcs)


def build_oracle(force=False):
    out = os.path.join(HERE, "liboracle.so")
    src = os.path.join(HERE, "rt_cpu_ref.cpp")
    hdr = os.path.join(HERE, "..", "include", "rt_cuda.h")
    if force or _stale(out, [src, hdr]):
        _run([CXX] + FLAGS + ["-shared", src, "-o", out])
    return out


def reference_available():
    return os.path.isdir(os.path.join(REFERENCE_ROOT, "src", "kernel"))


def build_ref(force=False):
    """Compile the reference kernels for the CPU; returns the .so path or None."""
    if not reference_available():
        return None
    kdir = os.path.join(REFERENCE_ROOT, "src", "kernel")
    shim = os.path.join(HERE, "ref_shim")
    outdir = os.path.join(HERE, "_ref")
    os.makedirs(outdir, exist_ok=True)
    so = os.path.join(outdir, "libref.so")
    deps = [os.path.join(shim, f) for f in os.listdir(shim)]
    if not force and not _stale(so, deps):
        return so
    objs = []

    def one(unit):
        src = os.path.join(shim, unit + ".cpp")
        obj = os.path.join(outdir, unit + ".o")
        extra = host_inc if unit in ("ref_obj", "ref_sah") else []
        _run([CXX] + FLAGS + REF_UNIT_FLAGS.get(unit, []) + extra +
             ["-fno-semantic-interposition", "-w", "-I", kdir, "-c", src, "-o", obj])
        return obj

    host_inc = ["-I", os.path.join(shim, "include"), "-I", os.path.join(REFERENCE_ROOT, "include")]

    def host(unit):
        obj = os.path.join(outdir, "host_" + unit + ".o")
        _run([CXX] + FLAGS + ["-w"] + host_inc +
             ["-c", os.path.join(REFERENCE_ROOT, "src", "rt", unit + ".cpp"), "-o", obj])
        return obj

    def any_unit(u):
        return one(u) if u in REF_UNITS else host(u)

    with ThreadPoolExecutor(max_workers=len(REF_UNITS) + len(REF_HOST_SOURCES)) as ex:
        objs = list(ex.map(any_unit, REF_UNITS + REF_HOST_SOURCES))
    _run([CXX] + FLAGS + ["-shared"] + objs + ["-o", so])
    return so


if __name__ == "__main__":
    print(build_oracle(force="-f" in sys.argv))
    print(build_ref(force="-f" in sys.argv))
