"""In-tree build of librt_cuda.so for sm_103a (nvcc, no cmake), and of
librt_shim.so, the drop-in C++ classes over it (g++; headers in
include/rt and include/gpu).

All CUDA translation units are compiled with ``--fmad=false`` so that the
single-precision math follows the reference kernels' operation order without
fused multiply-adds; division and square root keep nvcc's IEEE defaults.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))   # tesina-rt_gb300/
CSRC = os.path.join(PKG, "csrc")
LIB = os.path.join(PKG, "librt_cuda.so")
OBJDIR = os.path.join(PKG, "_build")
NVCC = os.environ.get("NVCC", "nvcc")
UNITS = ["lbvh", "trace", "capi", "noalloc", "batch", "batch_api", "server", "animate", "obj", "instances", "sah"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# host code as the device code: no fused multiply-add (gcc contracts by default
# where the machine has FMA, as the Arm hosts do)
FLAGS = ARCH + ["-O3", "-lineinfo", "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC",
                "-Xcompiler", "-fvisibility=hidden", "-Xcompiler", "-ffp-contract=off"]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s%s" % (" ".join(cmd), r.stdout[-3000:],
                                                         r.stderr[-6000:]))
    return r


def _sources():
    out = []
    for root, _, files in os.walk(CSRC):
        out += [os.path.join(root, f) for f in files if f.endswith((".cu", ".cuh", ".h"))]
    out.append(os.path.join(PKG, "..", "include", "rt_cuda.h"))
    return out


def stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(s) > t for s in _sources())


SHIM = os.path.join(PKG, "librt_shim.so")
SHIM_SRC = os.path.join(PKG, "shim")
INCLUDE = os.path.join(PKG, "..", "include")
CXX = os.environ.get("CXX", "g++")


def _shim_sources():
    return sorted(os.path.join(SHIM_SRC, f) for f in os.listdir(SHIM_SRC) if f.endswith(".cpp"))


def build_shim(force=False):
    """librt_shim.so: BVHBuilder, Tracer, RayShader, SecondaryRayGenerator,
    PrimaryRayGenerator, FrameBuffer, Scene, RayBundle / HitBundle and
    DeviceInterface / DeviceMemory over librt_cuda.so (found beside it)."""
    deps = _shim_sources() + [LIB]
    for d in ("rt", "gpu"):
        deps += [os.path.join(INCLUDE, d, f) for f in os.listdir(os.path.join(INCLUDE, d))]
    if not force and os.path.exists(SHIM) and all(os.path.getmtime(x) <= os.path.getmtime(SHIM)
                                                  for x in deps):
        return SHIM
    tmp = SHIM + ".tmp"
    _run([CXX, "-std=c++17", "-O2", "-fPIC", "-shared", "-Wall", "-I", INCLUDE] + _shim_sources() +
         ["-L", PKG, "-lrt_cuda", "-Wl,-rpath,$ORIGIN", "-o", tmp])
    os.replace(tmp, SHIM)
    return SHIM


def build(force=False, verbose=False):
    _build_cuda(force, verbose)
    build_shim(force)
    return LIB


def _build_cuda(force, verbose):
    if not force and not stale():
        return LIB
    os.makedirs(OBJDIR, exist_ok=True)

    def one(u):
        obj = os.path.join(OBJDIR, u + ".o")
        extra = ["-Xptxas", "-v"] if verbose else []
        r = _run([NVCC] + FLAGS + extra + ["-c", os.path.join(CSRC, u + ".cu"), "-o", obj])
        if verbose:
            sys.stderr.write(r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(one, UNITS))
    tmp = LIB + ".tmp"
    _run([NVCC] + ARCH + ["-shared", "-o", tmp] + objs)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="-f" in sys.argv, verbose="-v" in sys.argv))
