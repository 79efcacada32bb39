"""Build the sm_103a CUDA library of the package (in-tree, no torch headers).

``build_library()`` compiles every ``csrc/*.cu`` with nvcc for
``-gencode arch=compute_103a,code=sm_103a`` in parallel and links
``sailor_gb300/libsailor_gb300.so``.  The library exports only the C ABI
declared in ``include/sailor_gb300.h``.
"""
import glob
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
LIB = os.path.join(HERE, "libsailor_gb300.so")
OBJ_DIR = os.path.join(HERE, "_build")

NVCC_FLAGS = [
    "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-lineinfo", "-std=c++17",
    "-Xcompiler", "-fPIC", "-fmad=false", "-Xptxas", "-O3",
]


def _nvcc():
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def sources():
    return sorted(glob.glob(os.path.join(HERE, "csrc", "*.cu")))


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build_library(force=False, verbose=False, extra_flags=()):
    srcs = sources()
    headers = glob.glob(os.path.join(HERE, "csrc", "*.cuh")) + [os.path.join(ROOT, "include", "sailor_gb300.h")]
    os.makedirs(OBJ_DIR, exist_ok=True)
    nvcc = _nvcc()
    procs, objs = [], []
    for s in srcs:
        o = os.path.join(OBJ_DIR, os.path.basename(s)[:-3] + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            cmd = [nvcc, "-c", s, "-o", o] + NVCC_FLAGS + list(extra_flags)
            if verbose:
                print(" ".join(cmd), flush=True)
            procs.append((s, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    failed = []
    for s, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append(s)
            sys.stderr.write(out.decode(errors="replace"))
        elif verbose and out:
            sys.stdout.write(out.decode(errors="replace"))
    if failed:
        raise RuntimeError("nvcc failed: " + ", ".join(os.path.basename(f) for f in failed))
    if force or procs or _stale(LIB, objs):
        cmd = [nvcc, "-shared", "-o", LIB + ".tmp"] + objs + ["-gencode", "arch=compute_103a,code=sm_103a",
                                                               "-lcudart"]
        subprocess.check_call(cmd)
        os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build_library(force="--force" in sys.argv, verbose=True,
                        extra_flags=["-Xptxas", "-v"] if "-v" in sys.argv else []))
