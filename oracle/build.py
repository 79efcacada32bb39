"""Build recipe for the oracle (test infrastructure).

``build_oracle()`` compiles ``sailor_oracle.c`` and ``octree_oracle.c`` with gcc into
``oracle/liboracle.so``; it adds no floating-point contraction of its own
(``-ffp-contract=off``) so that the explicit ``fmaf`` calls in the source are
the only fused operations, on x86-64 and aarch64 alike.

``build_reference_cubins()`` compiles the reference's own CUDA sources, read
in place from a SAILOR checkout, into sm_103a cubins under ``oracle/_ref/``.
They are launched through the CUDA driver API by ``oracle/ref_cubin.py`` to
produce golden vectors; nothing else uses them.  The recipe only runs where
the reference checkout exists.  ``python oracle/build.py <SAILOR checkout>
--fastnerf`` also builds the FastNerf inference kernels (opt-in: slow).
"""
import os
import subprocess
import sys
import sysconfig

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")
REF_KERNELS = ("fusion_kernel", "octree_kernel", "intersection_kernel",
               "sampling_kernel", "volume_rendering")


def build_oracle(force=False):
    srcs = [os.path.join(HERE, n) for n in ("sailor_oracle.c", "octree_oracle.c")]
    if (not force and os.path.exists(LIB)
            and all(os.path.getmtime(LIB) >= os.path.getmtime(s) for s in srcs)):
        return LIB
    cmd = ["gcc", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
           "-o", LIB + ".tmp"] + srcs + ["-lm"]
    subprocess.check_call(cmd)
    os.replace(LIB + ".tmp", LIB)
    return LIB


def build_reference_cubins(ref_root, force=False):
    """Compile the reference kernels (read in place) to sm_103a cubins."""
    src_dir = os.path.join(ref_root, "c_lib", "VoxelEncoding", "src")
    if not os.path.isdir(src_dir):
        return []
    import torch  # noqa: F401  (headers of the installed torch)
    tdir = os.path.dirname(torch.__file__)
    pyinc = sysconfig.get_paths()["include"]
    os.makedirs(REF_DIR, exist_ok=True)
    procs, outs = [], []
    for k in REF_KERNELS:
        src = os.path.join(src_dir, k + ".cu")
        out = os.path.join(REF_DIR, k + ".cubin")
        outs.append(out)
        if (not force and os.path.exists(out)
                and os.path.getmtime(out) >= os.path.getmtime(src)):
            continue
        cmd = ["nvcc", "-cubin", "-gencode", "arch=compute_103a,code=sm_103a",
               "-std=c++17", "-D__CUDA_NO_HALF_OPERATORS__",
               "-D__CUDA_NO_HALF_CONVERSIONS__",
               "-D__CUDA_NO_BFLOAT16_CONVERSIONS__",
               "-D__CUDA_NO_HALF2_OPERATORS__",
               "-DTORCH_EXTENSION_NAME=VoxelEncoding",
               "-I" + os.path.join(tdir, "include"),
               "-I" + os.path.join(tdir, "include", "torch", "csrc", "api", "include"),
               "-I" + pyinc, "-I/usr/local/cuda/include/cccl",
               "-o", out, src]
        procs.append(subprocess.Popen(cmd, stdout=subprocess.DEVNULL,
                                      stderr=subprocess.PIPE))
    for p in procs:
        _, err = p.communicate()
        if p.returncode != 0:
            sys.stderr.write(err.decode(errors="replace")[-2000:])
            raise RuntimeError("reference cubin build failed")
    return outs


def build_fastnerf_cubin(ref_root, force=False):
    """Compile the reference's FastNerf inference kernels
    (c_lib/FastNerf/src/infer_mlp.cu, read in place) to an sm_103a cubin for
    golden vectors of the occupancy-MLP restatement (oracle/fastnerf.py).
    Opt-in and slow (its fully unrolled per-thread MLPs take about 25 minutes
    of nvcc), so build() does not run it."""
    src = os.path.join(ref_root, "c_lib", "FastNerf", "src", "infer_mlp.cu")
    if not os.path.exists(src):
        return None
    import torch  # noqa: F401  (headers of the installed torch)
    tdir = os.path.dirname(torch.__file__)
    os.makedirs(REF_DIR, exist_ok=True)
    out = os.path.join(REF_DIR, "infer_mlp.cubin")
    if not force and os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(src):
        return out
    cmd = ["nvcc", "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-std=c++17",
           "-D__CUDA_NO_HALF_OPERATORS__", "-D__CUDA_NO_HALF_CONVERSIONS__",
           "-D__CUDA_NO_BFLOAT16_CONVERSIONS__", "-D__CUDA_NO_HALF2_OPERATORS__",
           "-DTORCH_EXTENSION_NAME=FastNerf",
           "-I" + os.path.join(tdir, "include"),
           "-I" + os.path.join(tdir, "include", "torch", "csrc", "api", "include"),
           "-I" + sysconfig.get_paths()["include"], "-I/usr/local/cuda/include/cccl",
           "-o", out, src]
    subprocess.check_call(cmd, stdout=subprocess.DEVNULL)
    return out


if __name__ == "__main__":
    print(build_oracle(force=True))
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    if args:
        print(build_reference_cubins(args[0], force=True))
        if "--fastnerf" in sys.argv:
            print(build_fastnerf_cubin(args[0], force=True))
