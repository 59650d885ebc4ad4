"""Builds libdvs_gb300.so in-tree for sm_103a, and the drop-in apps.

The CUDA and host C++ translation units compile in parallel and link into
one shared library exposing the C-ABI declared in include/dvs_gb300.h; the
apps bin/dvs and bin/cam (apps/main_*.cpp) link against it.  Host code and
device code are both compiled without floating-point contraction so that
every expression rounds as written.

    python -m dvsrender4deepspace_gb300.build        (or build() from Python)
"""
import fcntl
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
APPS = os.path.join(PKG, "apps")
BIN = os.path.join(ROOT, "bin")
APP_MAINS = {"dvs": "main_dvs.cpp", "cam": "main_cam.cpp", "cam_blur": "main_cam_blur.cpp"}
OUT_DIR = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libdvs_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
HOST_FLAGS = ["-O3", "-fPIC", "-fopenmp", "-ffp-contract=off", "-std=c++17", "-Wall", "-Wno-unused-function"]


def nvcc():
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    path = os.path.join(cuda, "bin", "nvcc")
    return path if os.path.exists(path) else (shutil.which("nvcc") or "nvcc")


def _sources():
    cuda_and_core = [os.path.join(CSRC, f) for f in ("kernels.cu", "batch.cu", "adaptive.cu", "capi.cu", "noalloc.cu",
                                                     "readout.cu", "bvh_build.cpp", "readout.cpp")]
    host_inputs = [os.path.join(APPS, f) for f in ("app_config.cpp", "app_scene.cpp", "app_trajectory.cpp",
                                                   "app_writers.cpp", "app_capi.cpp")]
    return cuda_and_core + host_inputs


def _headers():
    return ([os.path.join(CSRC, f) for f in ("kernels.h", "dvs_internal.h", "device_optics.cuh", "device_circuit.cuh")]
            + [os.path.join(APPS, f) for f in sorted(os.listdir(APPS)) if f.endswith(".hpp")]
            + [os.path.join(ROOT, "include", f) for f in ("dvs_gb300.h", "dvs_gb300.hpp")])


def _apps():
    return {name: os.path.join(BIN, name) for name in APP_MAINS}


def up_to_date():
    outputs = [LIB] + list(_apps().values())
    if not all(os.path.exists(p) for p in outputs):
        return False
    t = min(os.path.getmtime(p) for p in outputs)
    inputs = _sources() + _headers() + [os.path.join(APPS, f) for f in APP_MAINS.values()] + [__file__]
    return all(os.path.getmtime(p) <= t for p in inputs)


def build(force=False, verbose=False):
    """Compile the library unless it is newer than every source.  Processes
    that find it stale at the same time (parallel test workers) build it one
    at a time: the others wait on a lock file and find it fresh."""
    if not force and up_to_date():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    with open(os.path.join(OUT_DIR, "build.lock"), "w") as lock:
        fcntl.flock(lock, fcntl.LOCK_EX)
        if not force and up_to_date():
            return LIB
        return _build(verbose)


def _build(verbose):
    inc = ["-I", CSRC, "-I", APPS, "-I", os.path.join(ROOT, "include")]
    xhost = ",".join(HOST_FLAGS)
    cmds = []
    for src in _sources():
        obj = os.path.join(OUT_DIR, os.path.basename(src) + ".o")
        if src.endswith(".cu"):
            cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-prec-div=true",
                   "-prec-sqrt=true", *os.environ.get("DVS_NVCC_DEFINES", "").split(), "-Xcompiler", xhost, *inc,
                   "-c", src, "-o", obj]
        else:
            cmd = [os.environ.get("CXX", "g++"), *HOST_FLAGS, *inc, "-I",
                   os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include"), "-c", src, "-o", obj]
        cmds.append((cmd, obj))
    procs = [(subprocess.Popen(c, stdout=subprocess.PIPE, stderr=subprocess.STDOUT), c, o) for c, o in cmds]
    failed = []
    for p, c, o in procs:
        out = p.communicate()[0].decode(errors="replace")
        if p.returncode != 0:
            failed.append((" ".join(c), out))
        elif verbose and out.strip():
            print(out)
    if failed:
        msg = "\n\n".join("%s\n%s" % f for f in failed)
        raise RuntimeError("building libdvs_gb300.so failed:\n" + msg)
    tmp = LIB + ".tmp"
    link = [nvcc(), *ARCH, "-shared", "-o", tmp, *[o for _, o in cmds], "-Xcompiler", "-fopenmp", "-lgomp"]
    r = subprocess.run(link, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if r.returncode != 0:
        raise RuntimeError("linking libdvs_gb300.so failed:\n" + r.stdout.decode(errors="replace"))
    os.replace(tmp, LIB)
    build_apps()
    return LIB


def build_apps():
    """Links bin/dvs and bin/cam against the in-tree library."""
    os.makedirs(BIN, exist_ok=True)
    inc = ["-I", APPS, "-I", os.path.join(ROOT, "include")]
    procs = []
    for name, main in APP_MAINS.items():
        tmp = os.path.join(BIN, name + ".tmp")
        cmd = [os.environ.get("CXX", "g++"), *HOST_FLAGS, *inc, os.path.join(APPS, main), "-o", tmp, "-L", PKG,
               "-ldvs_gb300", "-Wl,-rpath,$ORIGIN/../dvsrender4deepspace_gb300"]
        procs.append((subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT), cmd, tmp, name))
    failed = []
    for p, cmd, tmp, name in procs:
        out = p.communicate()[0].decode(errors="replace")
        if p.returncode != 0:
            failed.append("%s\n%s" % (" ".join(cmd), out))
        else:
            os.replace(tmp, os.path.join(BIN, name))
    if failed:
        raise RuntimeError("building the apps failed:\n" + "\n\n".join(failed))


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
    print(LIB)
