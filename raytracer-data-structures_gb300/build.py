"""Build recipe for the engine library (librq.so) — nvcc, sm_103a only.

Each .cu in csrc/ (nvcc) and each .cpp (the host C++ compiler) is compiled
to an object in parallel, then linked into librq.so next to this file.  Used by __graft_entry__.build() and by rq.py when
the library is missing.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "librq.so")
DRIVER = os.path.join(HERE, "rq_render")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Exact-arithmetic parity relies on explicit __f*_rn intrinsics; -fmad=false
# additionally keeps nvcc from contracting any remaining a*b+c.
NVFLAGS = ["-O3", "-std=c++17", "-lineinfo", "-fmad=false", "-Xcompiler", "-fPIC",
           "--expt-relaxed-constexpr", "-I", os.path.join(ROOT, "include"), "-I", CSRC]


def nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def _newest_input():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(ROOT, "include", "rq.h")]
    files += [os.path.join(HERE, "host", f) for f in os.listdir(os.path.join(HERE, "host"))]
    return max(os.path.getmtime(f) for f in files)


def build(force=False, verbose=False):
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _newest_input():
        if not os.path.exists(DRIVER):
            build_driver()
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    cc = nvcc()
    srcs = sources()

    cxx = os.environ.get("CXX") or shutil.which("g++") or "g++"

    def compile_one(src):
        obj = os.path.join(OUT_DIR, os.path.splitext(os.path.basename(src))[0] + ".o")
        if src.endswith(".cpp"):  # host-only code
            # no contraction of a*b+c, so x86 and Arm builds round alike
            cmd = [cxx, "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"),
                   "-c", src, "-o", obj]
        else:
            cmd = [cc, *ARCH, *NVFLAGS, "-c", src, "-o", obj]
        if verbose and not src.endswith(".cpp"):
            cmd.insert(1, "-Xptxas=-v")
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
        if verbose and r.stderr:
            sys.stderr.write(r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB + ".tmp"
    r = subprocess.run([cc, *ARCH, "-shared", "-o", tmp, *objs], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    build_driver()
    return LIB


def build_driver():
    """The C++ host program over the C ABI (host/rq_render_main.cpp)."""
    cxx = os.environ.get("CXX") or shutil.which("g++") or "g++"
    cmd = [cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(HERE, "host"),
           os.path.join(HERE, "host", "rq_render_main.cpp"), "-L", HERE, "-lrq", "-Wl,-rpath,$ORIGIN",
           "-o", DRIVER]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"driver build failed:\n{r.stderr}")
    return DRIVER


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(LIB)
