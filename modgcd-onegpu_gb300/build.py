"""Builds libmodgcd.so (CUDA kernels for sm_103a + host C ABI) and the C++ drop-in.

Outputs stay in the source tree (``lib/``); objects go to ``_build/``.  Translation units
compile in parallel.  GMP: the runtime library libgmp.so.10 is linked directly; the
project's declaration header stands in for <gmp.h> when the system has none.
Extra compiler flags for experiments: MGCD_NVCC_FLAGS (CUDA units), MGCD_CXX_FLAGS (host
units); rebuild with --force after changing them.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "lib")

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CXX = os.environ.get("CXX", "g++")

LIBNAME = "libmodgcd.so"
DROPIN_NAME = "libGmpCuda.so"


def _have_gmp_h():
    r = subprocess.run([CXX, "-E", "-x", "c++", "-include", "gmp.h", "/dev/null"],
                       stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
    return r.returncode == 0


def gmp_include_flags():
    return [] if _have_gmp_h() else ["-I" + os.path.join(CSRC, "gmp_decl")]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stdout + r.stderr


def _newer(target, deps):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs += [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))]
    return hs


def build(verbose=False, force=False):
    """Compiles everything that is out of date; returns the path of libmodgcd.so."""
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIB, exist_ok=True)
    gmpinc = gmp_include_flags()
    hdrs = _headers()
    cuda_inc = "-I" + os.path.join(CUDA_HOME, "include")
    units = []
    for f in ("mgcd_kernels.cu", "mgcd_noalloc.cu", "mgcd_radix_dev.cu", "mgcd_certify.cu"):
        src = os.path.join(CSRC, f)
        obj = os.path.join(BUILD, f + ".o")
        cmd = [NVCC] + ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xptxas", "-v"] + \
            os.environ.get("MGCD_NVCC_FLAGS", "").split() + ["-c", src, "-o", obj]
        units.append((obj, [src] + hdrs, cmd))
    for f in ("mgcd_capi.cpp", "mgcd_serve.cpp", "mgcd_moduli.cpp", "mgcd_radix.cpp", "GmpCudaDevice.cpp"):
        src = os.path.join(CSRC, f)
        obj = os.path.join(BUILD, f + ".o")
        cmd = [CXX, "-O2", "-fPIC", "-std=c++17", "-Wall", cuda_inc, "-I" + os.path.join(ROOT, "include")] + \
            os.environ.get("MGCD_CXX_FLAGS", "").split() + \
            gmpinc + ["-c", src, "-o", obj]
        units.append((obj, [src] + hdrs, cmd))

    todo = [u for u in units if force or not _newer(u[0], u[1])]
    logs = {}
    if todo:
        with ThreadPoolExecutor(max_workers=len(todo)) as ex:
            for (obj, _, _), out in zip(todo, ex.map(lambda u: _run(u[2]), todo)):
                logs[obj] = out
    if verbose:
        for k, v in logs.items():
            sys.stdout.write("%s\n%s" % (k, v))

    objs = [u[0] for u in units]
    lib = os.path.join(LIB, LIBNAME)
    core = [o for o in objs if not o.endswith("GmpCudaDevice.cpp.o")]
    if force or not _newer(lib, core):
        _run([NVCC] + ARCH + ["-shared", "-o", lib] + core + ["-l:libgmp.so.10", "-lpthread"])

    # createModuli (host tool) -> GmpCuda::moduli[] source in the reference's format
    cm = os.path.join(LIB, "createModuli")
    cm_src = [os.path.join(CSRC, "createModuli.cpp"), os.path.join(CSRC, "mgcd_moduli.cpp")]
    if force or not _newer(cm, cm_src + hdrs):
        _run([CXX, "-O2", "-std=c++17", "-o", cm] + cm_src)
    gen = os.path.join(BUILD, "GmpCudaModuli.cpp")
    if force or not _newer(gen, [cm]):
        with open(gen + ".tmp", "w") as f:
            r = subprocess.run([cm, "32", "131072", "--inverses"], stdout=f, stderr=subprocess.PIPE, text=True)
        if r.returncode != 0:
            raise RuntimeError("createModuli failed: " + r.stderr)
        os.replace(gen + ".tmp", gen)
    gen_obj = gen + ".o"
    if force or not _newer(gen_obj, [gen]):
        _run([CXX, "-O0", "-fPIC", "-std=c++17", "-I" + os.path.join(ROOT, "include")] + gmpinc +
             ["-c", gen, "-o", gen_obj])

    dropin = os.path.join(LIB, DROPIN_NAME)
    dep = [o for o in objs if o.endswith("GmpCudaDevice.cpp.o")] + [gen_obj]
    if force or not _newer(dropin, dep + [lib]):
        _run([CXX, "-shared", "-o", dropin] + dep + ["-L" + LIB, "-lmodgcd", "-Wl,-rpath,$ORIGIN",
                                                      "-l:libgmp.so.10"])
    drv = os.path.join(LIB, "testmodgcd_gb300")
    drv_src = os.path.join(CSRC, "testmodgcd_gb300.cpp")
    if force or not _newer(drv, [drv_src, dropin] + hdrs):
        _run([CXX, "-O2", "-std=c++17", "-I" + os.path.join(ROOT, "include")] + gmpinc +
             [drv_src, "-o", drv, "-L" + LIB, "-lGmpCuda", "-lmodgcd", "-Wl,-rpath," + LIB, "-l:libgmp.so.10"])
    return lib


def ptxas_report():
    """Registers / spills / shared memory of the kernels (-Xptxas -v)."""
    src = os.path.join(CSRC, "mgcd_kernels.cu")
    out = _run([NVCC] + ARCH + ["-O3", "-std=c++17", "-Xptxas", "-v", "-c", src, "-o", os.devnull])
    return out


def clean():
    shutil.rmtree(BUILD, ignore_errors=True)
    shutil.rmtree(LIB, ignore_errors=True)


if __name__ == "__main__":
    if "--clean" in sys.argv:
        clean()
    print(build(verbose="-v" in sys.argv, force="--force" in sys.argv))
