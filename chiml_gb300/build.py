"""Builds the native parts in-tree: the device engine library and the CPU oracle.

The engine (``chiml_gb300/_build/libchiml_gb300.so``) is compiled for sm_103a
only. The oracle (``oracle/_build/libchiml_oracle.so``) is test infrastructure.
When the chiML sources are available, the one-process reference binary is also
built from them by ``oracle/Makefile.ref`` into ``oracle/_ref/``.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "chiml_gb300")
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
ORACLE = os.path.join(ROOT, "oracle")
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
HOST_SRCS = ["json.cpp", "inputs.cpp", "setup.cpp", "outputs.cpp", "emitters.cpp", "tfsf.cpp"]

LIB_ENGINE = os.path.join(BUILD, "libchiml_gb300.so")
LIB_ORACLE = os.path.join(ORACLE, "_build", "libchiml_oracle.so")


def _run(cmd, cwd=None):
    r = subprocess.run(cmd, cwd=cwd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r


def _newer(target, sources):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(s) <= t for s in sources)


def _sources():
    out = []
    for d, _, files in os.walk(CSRC):
        for f in files:
            if f.endswith((".cpp", ".cu", ".hpp", ".cuh", ".h")):
                out.append(os.path.join(d, f))
    out.append(os.path.join(ROOT, "include", "chiml_gpu.h"))
    return out


def build_engine(force=False):
    os.makedirs(BUILD, exist_ok=True)
    srcs = _sources()
    if not force and _newer(LIB_ENGINE, srcs):
        return LIB_ENGINE
    objs = []
    jobs = []
    for name in ("fdtd_kernels", "box_noalloc", "emitter_kernels", "tfsf_kernels", "flux_kernels"):
        cu = os.path.join(CSRC, "kernels", name + ".cu")
        o = os.path.join(BUILD, name + ".o")
        jobs.append([NVCC] + ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-c", cu, "-o", o])
        objs.append(o)
    # The host plan (cell classes, shape tests, source cells) is built without contracting
    # a*b+c into fused multiply-adds, which aarch64 gcc does by default, so that its
    # inside/outside decisions are the same on x86_64 and aarch64 hosts.
    cxx = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-fopenmp", "-I" + os.path.join(CUDA_HOME, "include")]
    for f in ["engine.cpp"] + ["host/" + h for h in HOST_SRCS]:
        o = os.path.join(BUILD, os.path.basename(f).replace(".cpp", ".o"))
        jobs.append(cxx + ["-c", os.path.join(CSRC, f), "-o", o])
        objs.append(o)
    with cf.ThreadPoolExecutor(max_workers=8) as ex:
        list(ex.map(_run, jobs))
    _run([NVCC] + ARCH + ["-shared", "-o", LIB_ENGINE] + objs + ["-Xcompiler", "-fopenmp", "-lgomp"])
    return LIB_ENGINE


def build_oracle(force=False):
    out_dir = os.path.dirname(LIB_ORACLE)
    os.makedirs(out_dir, exist_ok=True)
    srcs = [os.path.join(ORACLE, "chiml_oracle.cpp")] + [os.path.join(CSRC, "host", h) for h in HOST_SRCS]
    deps = srcs + [os.path.join(CSRC, "host", h) for h in os.listdir(os.path.join(CSRC, "host")) if h.endswith(".hpp")]
    if not force and _newer(LIB_ORACLE, deps):
        return LIB_ORACLE
    _run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-fopenmp", "-o", LIB_ORACLE] + srcs)
    return LIB_ORACLE


def build_reference(ref_dir=None):
    """One-process CPU build of the chiML sources, only where they exist (never on the GPU
    host). The checkout is ``ref_dir``, else the CHIML_REF_SRC environment variable; without
    either nothing is built."""
    ref_dir = ref_dir or os.environ.get("CHIML_REF_SRC")
    if not ref_dir or not os.path.isdir(os.path.join(ref_dir, "src")):
        return None
    if shutil.which("make") is None:
        return None
    _run(["make", "-f", "Makefile.ref", "REF=" + ref_dir, "-j8"], cwd=ORACLE)
    return os.path.join(ORACLE, "_ref", "chiml_ref")


def build_all(force=False, ref_dir=None):
    with cf.ThreadPoolExecutor(max_workers=3) as ex:
        fe = ex.submit(build_engine, force)
        fo = ex.submit(build_oracle, force)
        fr = ex.submit(build_reference, ref_dir)
        return fe.result(), fo.result(), fr.result()


if __name__ == "__main__":
    print(build_all(force=True))
