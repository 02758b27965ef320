"""Compile the netlk shared library (host C++ + sm_103a CUDA) in-tree.

Output: ``netrax_gb300/_build/libnetlk.so``. Sources compile in parallel, one
``-gencode`` (sm_103a), no CMake.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libnetlk.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["dag.cpp", "model.cpp", "netlk.cpp", "kernels.cu", "kernels20.cu", "kernels20tc.cu", "tangent.cu",
           "noalloc.cu", "alignment.cpp"]
HEADERS = ["internal.hpp", "kernels.cuh", "kernels_common.cuh", "tc.cuh"]


def _nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the netlk CUDA library cannot be built")
    return cand


def _stale(obj, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [
        os.path.join(HERE, "..", "include", "netlk.h")]
    common = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-lineinfo"] + ARCH
    jobs = []
    objs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + hdrs):
            extra = ["-Xptxas", "-v"] if (verbose and src.endswith(".cu")) else []
            jobs.append([nvcc, "-c", s, "-o", o] + common + extra)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        futs = [ex.submit(subprocess.run, j, capture_output=True, text=True) for j in jobs]
        for j, f in zip(jobs, futs):
            r = f.result()
            if verbose and r.stderr:
                print(r.stderr)
            if r.returncode != 0:
                raise RuntimeError("compile failed: %s\n%s\n%s" % (" ".join(j), r.stdout, r.stderr))
    if force or _stale(LIB, objs):
        tmp = LIB + ".tmp%d" % os.getpid()
        r = subprocess.run([nvcc, "-shared", "-o", tmp] + objs + ARCH, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
