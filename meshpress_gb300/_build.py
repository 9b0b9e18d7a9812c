"""In-tree build of the native libraries.

* ``libstride_gb300.so`` -- the GPU decoder: hand-written sm_103a CUDA
  kernels behind a plain C ABI (``include/stride_gb300.h``), built with nvcc
  for ``-gencode arch=compute_103a,code=sm_103a`` only.
* ``libstride_encode.so`` -- the host C++ encoder that produces test inputs.

Both land next to this file.  Loading the decoder never builds it silently on
a machine without nvcc: a missing library raises.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
REPO = os.path.dirname(HERE)
INCLUDE = os.path.join(REPO, "include")

DECODER_LIB = os.path.join(HERE, "libstride_gb300.so")
ENCODER_LIB = os.path.join(HERE, "libstride_encode.so")

CUDA_SOURCES = ["stride_kernels.cu", "stride_group.cu", "stride_api.cu", "stride_batch.cu", "stride_serve.cu", "stride_static.cu",
                "pldt5.cu"]
NVCC_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a", "-lineinfo", "-O3",
              "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2", "-Xcompiler", "-ffp-contract=off",
              "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills", "-Xptxas", "-dlcm=cg"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the STRIDE GPU decoder cannot be built")


def _stale(target: str, sources) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return hs


def build_decoder(force: bool = False, verbose: bool = False) -> str:
    srcs = [os.path.join(CSRC, s) for s in CUDA_SOURCES if os.path.exists(os.path.join(CSRC, s))]
    if not force and not _stale(DECODER_LIB, srcs + _headers()):
        return DECODER_LIB
    nvcc = _nvcc()
    objdir = os.path.join(HERE, "_objs")
    os.makedirs(objdir, exist_ok=True)

    def compile_one(src):
        obj = os.path.join(objdir, os.path.basename(src) + ".o")
        cmd = [nvcc, *NVCC_FLAGS, "-I", INCLUDE, "-I", CSRC, "-c", src, "-o", obj]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        return obj, r.stderr

    with ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        results = list(ex.map(compile_one, srcs))
    if verbose:
        for _, log in results:
            print(log)
    objs = [o for o, _ in results]
    tmp = DECODER_LIB + ".tmp"
    cmd = [nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-shared", "-Xcompiler", "-fPIC",
           *objs, "-o", tmp, "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, DECODER_LIB)
    return DECODER_LIB


def build_encoder(force: bool = False) -> str:
    src = os.path.join(CSRC, "encoder", "stride_encode.cpp")
    if not force and not _stale(ENCODER_LIB, [src]):
        return ENCODER_LIB
    tmp = ENCODER_LIB + ".tmp"
    # no contraction: the PLDT v5 writer replays the decoder's float64 arithmetic
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", src, "-o", tmp], check=True)
    os.replace(tmp, ENCODER_LIB)
    return ENCODER_LIB


def encoder_library() -> str:
    return build_encoder()


def decoder_library() -> str:
    """Path of the built decoder library; raises if it has not been built."""
    if not os.path.exists(DECODER_LIB):
        raise RuntimeError(
            f"{DECODER_LIB} is missing: build it with meshpress_gb300._build.build_decoder() "
            "(the decoder has no CPU fallback)")
    return DECODER_LIB


def build_all(force: bool = False, verbose: bool = False):
    with ThreadPoolExecutor(max_workers=2) as ex:
        f1 = ex.submit(build_encoder, force)
        f2 = ex.submit(build_decoder, force, verbose)
        return f1.result(), f2.result()
