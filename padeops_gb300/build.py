"""Build the native library ``libpadeops_gb300.so`` in-tree with nvcc (sm_103a).

The library is plain C++/CUDA behind a C ABI (``include/padeops_gb300.h``); no torch
extension machinery is involved.  Translation units compile in parallel; a stamp file
holding a hash of the sources skips rebuilds when nothing changed.
"""
import hashlib
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT_DIR, "libpadeops_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
HOST_SOURCES = ["operators.cpp", "plan.cpp", "chunkplan.cpp", "capi.cpp", "pade6stagg.cpp"]
CUDA_SOURCES = ["kernels.cu", "kernels_df16.cu", "kernels_df32.cu", "kernels_f32.cu", "kernels_stencil.cu", "kernels_stencil_band.cu", "kernels_stencil_f32.cu",
                "kernels_stencil_stagg.cu", "kernels_reg.cu", "kernels_half.cu", "noalloc.cu", "fft.cu", "fft_df.cu",
                "spectral.cu", "fourier_coll.cu", "poisson_wall.cu", "les.cu", "mlp.cu",
                "dense_tc.cu"]
HEADERS = ["operators.h", "plan.h", "chunkplan.h", "engine.h", "dfmath.cuh", "chunk_kernel.cuh", "stencil_kernel.cuh", "reg_kernel.cuh", "half_kernel.cuh", "capi_internal.h",
           "fft.h", "spectral_internal.h", "tc_common.cuh"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def _digest():
    h = hashlib.sha256()
    for name in HOST_SOURCES + CUDA_SOURCES + HEADERS:
        with open(os.path.join(CSRC, name), "rb") as fh:
            h.update(name.encode() + fh.read())
    with open(os.path.join(ROOT, "include", "padeops_gb300.h"), "rb") as fh:
        h.update(fh.read())
    h.update(" ".join(ARCH).encode())
    return h.hexdigest()


def build(force=False, verbose=False):
    """Compile the library if its sources changed; returns the path of the .so."""
    os.makedirs(OUT_DIR, exist_ok=True)
    stamp = os.path.join(OUT_DIR, "stamp.txt")
    dig = _digest()
    if not force and os.path.exists(LIB) and os.path.exists(stamp) and open(stamp).read() == dig:
        return LIB
    nvcc = _nvcc()
    # host code: no floating-point contraction, so x86 and Arm builds round alike
    common = ["-std=c++17", "-O3", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "-I",
              os.path.join(ROOT, "include")]
    procs = []
    objs = []
    for name in HOST_SOURCES + CUDA_SOURCES:
        obj = os.path.join(OUT_DIR, name + ".o")
        cmd = [nvcc] + common + ARCH + ["-lineinfo", "-c", os.path.join(CSRC, name), "-o", obj]
        if verbose:
            print(" ".join(cmd))
        procs.append((name, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
        objs.append(obj)
    failed = []
    for name, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((name, out.decode(errors="replace")))
    if failed:
        msg = "\n".join(f"--- {n}\n{o}" for n, o in failed)
        raise RuntimeError("nvcc failed:\n" + msg)
    tmp = LIB + ".tmp"
    cmd = [nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    with open(stamp, "w") as fh:
        fh.write(dig)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
