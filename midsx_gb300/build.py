"""In-tree build of the native libraries (no cmake, no pip install).

* ``midsx_gb300/lib/libmidsx_gb300.so`` - CUDA kernels for sm_103a + host table builder
  + the C ABI declared in ``include/midsx_gpu.h``.
* ``midsx_gb300/lib/libmidsx_core.so`` - the C++ API of MIDSX (ComputationalDomain,
  InteractionData, PhotonSource, tallies, PhysicsEngine, runSimulation) on top of the
  C ABI, headers in ``include/MIDSX``.
* ``oracle/_build/liboracle.so`` - the CPU restatement used by tests and the CPU baseline.

Translation units compile in parallel; a unit is rebuilt only when a source it depends on
is newer than its object file.
"""
import os
import shutil
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "midsx_gb300")
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
LIBDIR = os.path.join(PKG, "lib")
OBJDIR = os.path.join(PKG, "_build")
ORACLE = os.path.join(ROOT, "oracle")
ORACLE_BUILD = os.path.join(ORACLE, "_build")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I", INCLUDE]
CXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-fopenmp", "-I", INCLUDE, "-Wall", "-Wno-unknown-pragmas"]

LIB_MAIN = os.path.join(LIBDIR, "libmidsx_gb300.so")
LIB_CORE = os.path.join(LIBDIR, "libmidsx_core.so")
LIB_ORACLE = os.path.join(ORACLE_BUILD, "liboracle.so")


def _nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def _cuda_lib_dir():
    nv = _nvcc()
    root = os.path.dirname(os.path.dirname(os.path.realpath(nv)))
    for sub in ("lib64", "lib", os.path.join("targets", "sbsa-linux", "lib"),
                os.path.join("targets", "x86_64-linux", "lib")):
        d = os.path.join(root, sub)
        if os.path.exists(os.path.join(d, "libcudart_static.a")):
            return d
    return os.path.join(root, "lib64")


def _have_zlib():
    """True when zlib's header and linkable library are installed (the C++ API then reads
    .nii.gz directly)."""
    import glob
    header = any(os.path.exists(os.path.join(d, "zlib.h")) for d in ("/usr/include", "/usr/local/include"))
    lib = bool(glob.glob("/usr/lib*/libz.so") + glob.glob("/usr/lib/*/libz.so") + glob.glob("/lib/*/libz.so") +
               glob.glob("/usr/local/lib/libz.so"))
    return header and lib


def _deps(path):
    """Sources a translation unit depends on: itself plus every header in csrc/include."""
    deps = [path]
    for d in (CSRC, INCLUDE, os.path.join(INCLUDE, "MIDSX"), os.path.join(INCLUDE, "MIDSX", "Core")):
        if os.path.isdir(d):
            deps += [os.path.join(d, f) for f in os.listdir(d) if f.endswith((".h", ".cuh", ".hpp"))]
    return deps


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _run_parallel(jobs):
    procs = []
    for cmd, target in jobs:
        procs.append((subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT), cmd, target))
    failed = []
    for p, cmd, target in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((cmd, out.decode(errors="replace")))
    if failed:
        msg = "\n\n".join(" ".join(c) + "\n" + o for c, o in failed)
        raise RuntimeError("native build failed:\n" + msg)


def build(verbose=False, with_oracle=True):
    os.makedirs(LIBDIR, exist_ok=True)
    os.makedirs(OBJDIR, exist_ok=True)
    os.makedirs(ORACLE_BUILD, exist_ok=True)
    nvcc = _nvcc()
    units = [
        ("transport.cu", [nvcc] + NVCC_FLAGS),
        ("server.cu", [nvcc] + NVCC_FLAGS),
        ("probe.cu", [nvcc] + NVCC_FLAGS),
        ("tables.cpp", ["g++"] + CXX_FLAGS),
    ]
    core_units = [f for f in sorted(os.listdir(CSRC)) if f.startswith("core_") and f.endswith(".cpp")]
    jobs = []
    objs, core_objs = [], []
    for name, cc in units:
        src = os.path.join(CSRC, name)
        obj = os.path.join(OBJDIR, name + ".o")
        objs.append(obj)
        if _stale(obj, _deps(src)):
            jobs.append((cc + ["-c", src, "-o", obj], obj))
    for name in core_units:
        src = os.path.join(CSRC, name)
        obj = os.path.join(OBJDIR, name + ".o")
        core_objs.append(obj)
        if _stale(obj, _deps(src)):
            jobs.append((["g++"] + CXX_FLAGS + ([] if _have_zlib() else ["-DMIDSX_NO_ZLIB"]) +
                         ["-c", src, "-o", obj], obj))
    oracle_src = os.path.join(ORACLE, "oracle.cpp")
    if with_oracle and _stale(LIB_ORACLE, [oracle_src, os.path.join(INCLUDE, "midsx_gpu.h")]):
        jobs.append((["g++", "-O3", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-I", INCLUDE,
                      oracle_src, "-o", LIB_ORACLE], LIB_ORACLE))
    if verbose:
        for cmd, _ in jobs:
            print(" ".join(cmd), file=sys.stderr)
    _run_parallel(jobs)
    cudalib = _cuda_lib_dir()
    link = []
    if _stale(LIB_MAIN, objs):
        link.append((["g++", "-shared", "-fopenmp", "-o", LIB_MAIN] + objs +
                     ["-L" + cudalib, "-lcudart_static", "-ldl", "-lpthread", "-lrt"], LIB_MAIN))
    if core_objs and (_stale(LIB_CORE, core_objs) or _stale(LIB_CORE, [LIB_MAIN])):
        link.append((["g++", "-shared", "-fopenmp", "-o", LIB_CORE] + core_objs +
                     ["-L" + LIBDIR, "-lmidsx_gb300", "-Wl,-rpath,$ORIGIN", "-ldl"] +
                     (["-lz"] if _have_zlib() else []), LIB_CORE))
    for cmd, target in link:
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        _run_parallel([(cmd, target)])
    # reference-style C++ programs on the C++ API
    exdir = os.path.join(PKG, "examples")
    jobs = []
    for f in sorted(os.listdir(exdir)) if os.path.isdir(exdir) else []:
        if not f.endswith(".cpp"):
            continue
        exe = os.path.join(LIBDIR, "midsx_example_" + f[:-4])
        src = os.path.join(exdir, f)
        if _stale(exe, _deps(src) + [LIB_CORE]):
            jobs.append((["g++", "-O2", "-std=c++17", "-I", INCLUDE, src, "-o", exe, "-L" + LIBDIR, "-lmidsx_core",
                          "-lmidsx_gb300", "-Wl,-rpath," + LIBDIR], exe))
    _run_parallel(jobs)
    return LIB_MAIN


if __name__ == "__main__":
    build(verbose=True)
    print(LIB_MAIN)
