"""Build the in-tree shared libraries:

  libsfgb.so     the CUDA kernels and the C ABI (include/sf_api.h), sm_103a
  libsfsynth.so  the synthetic sweep generator and chunk writer (host C, OpenMP)

Translation units compile in parallel; nothing is installed outside the tree.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

from . import _paths

CUDA_SOURCES = ["sf_threshold.cu", "sf_stream.cu", "sf_lattice.cu", "sf_api.cu", "sf_label.cu",
                "sf_serve.cu", "sf_refl.cu", "sf_decompress.cu", "sf_frames.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
              # No FMA contraction anywhere: the FP64/FP32 decisions must round
              # each operation as the reference does (the helpers also use
              # explicit _rn intrinsics).
              "-fmad=false", "--expt-relaxed-constexpr"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def _run(cmd, verbose):
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r.stdout + r.stderr


def build(verbose: bool = False, ptxas_info: bool = False) -> dict:
    out_dir = os.path.join(_paths.ROOT, "_build")
    os.makedirs(out_dir, exist_ok=True)
    nvcc = _nvcc()
    inc = ["-I", _paths.INCLUDE, "-I", _paths.CSRC]
    extra = ["-Xptxas", "-v"] if ptxas_info else []
    logs = {}

    def compile_one(src):
        obj = os.path.join(out_dir, os.path.splitext(src)[0] + ".o")
        logs[src] = _run([nvcc, *ARCH, *NVCC_FLAGS, *extra, *inc, "-c",
                          os.path.join(_paths.CSRC, src), "-o", obj], verbose)
        return obj

    def synth():
        tmp = _paths.synth_lib() + ".tmp"
        _run(["gcc", "-std=c11", "-O2", "-fopenmp", "-fPIC", "-shared",
              os.path.join(_paths.CSRC, "synth.c"), os.path.join(_paths.CSRC, "synth_chunk.c"),
              "-o", tmp, "-lm"], verbose)
        os.replace(tmp, _paths.synth_lib())

    with ThreadPoolExecutor(max_workers=len(CUDA_SOURCES) + 1) as ex:
        fut_synth = ex.submit(synth)
        objs = list(ex.map(compile_one, CUDA_SOURCES))
        fut_synth.result()
    tmp = _paths.core_lib() + ".tmp"
    _run([nvcc, *ARCH, "-shared", "-Xcompiler", "-fPIC", *objs, "-o", tmp,
          "-lcudart"], verbose)
    os.replace(tmp, _paths.core_lib())
    return logs


if __name__ == "__main__":
    logs = build(verbose=True, ptxas_info="-v" in sys.argv)
    for src, log in logs.items():
        if log.strip():
            print(f"== {src}\n{log}")
