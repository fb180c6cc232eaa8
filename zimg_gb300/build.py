"""Build the zimg_gb300 shared library in-tree with nvcc for sm_103a.

Output: zimg_gb300/_lib/libzimg_gb300.so (git-ignored). Translation units are
compiled in parallel, then linked. Host code is compiled with
-ffp-contract=off so filter tables are rounded exactly as zimg rounds them.
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT_DIR = os.path.join(PKG, "_lib")
OBJ_DIR = os.path.join(PKG, "_build")
LIB = os.path.join(OUT_DIR, "libzimg_gb300.so")

SOURCES = ["filter_plan.cpp", "capi.cu", "capi_graph.cu", "capi_batch.cu", "capi_static_tmp.cu",
           "pass_kernels.cu", "fused.cu", "fused_inst_v_f32.cu", "fused_inst_v_u16.cu", "fused_inst_h_f32.cu",
           "fused_inst_h_u16.cu", "fused_inst_v_i16.cu", "fused_inst_h_i16.cu", "mma.cu", "chain.cu", "chain_tma.cu", "wide_kernel.cu", "wide_umma.cu", "copy_kernel.cu",
           "depth_kernel.cu", "ed_kernel.cu", "alpha_kernel.cu", "capi_depth.cu", "colorspace_plan.cpp",
           "colorspace_kernel.cu", "capi_colorspace.cu", "work_chunks.cpp", "unresize_plan.cpp", "unresize_kernel.cu", "capi_unresize.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


# Per-file nvcc flags (none at present).
FILE_FLAGS: dict[str, list[str]] = {}


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _flags() -> list[str]:
    return ["-std=c++17", "-O3", "-lineinfo", *ARCH, "-Xcompiler", "-fPIC,-ffp-contract=off,-fvisibility=hidden",
            "-I", os.path.join(ROOT, "include"), "-I", CSRC, "--expt-relaxed-constexpr"]


def _headers_digest() -> str:
    h = hashlib.sha1()
    for d in (CSRC, os.path.join(ROOT, "include")):
        for f in sorted(os.listdir(d)):
            if f.endswith((".h", ".cuh", ".inc")):
                with open(os.path.join(d, f), "rb") as fh:
                    h.update(fh.read())
    return h.hexdigest()


def _compile(src: str, digest: str, verbose: bool) -> str:
    path = os.path.join(CSRC, src)
    obj = os.path.join(OBJ_DIR, src + ".o")
    stamp = obj + ".stamp"
    with open(path, "rb") as fh:
        key = hashlib.sha1(fh.read() + digest.encode() + " ".join(_flags() + FILE_FLAGS.get(src, [])).encode()).hexdigest()
    if os.path.exists(obj) and os.path.exists(stamp) and open(stamp).read() == key:
        return obj
    cmd = [_nvcc(), *_flags(), *FILE_FLAGS.get(src, []), "-c", path, "-o", obj]
    if src.endswith(".cu"):
        cmd.insert(1, "-Xptxas=-v" if verbose else "-Xptxas=-O3")
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{res.stderr[-6000:]}")
    if verbose and res.stderr:
        sys.stderr.write(res.stderr)
    with open(stamp, "w") as fh:
        fh.write(key)
    return obj


def build(verbose: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    os.makedirs(OBJ_DIR, exist_ok=True)
    digest = _headers_digest()
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, digest, verbose), SOURCES))
    newest = max(os.path.getmtime(o) for o in objs)
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < newest:
        tmp = LIB + ".tmp"
        cmd = [_nvcc(), *ARCH, "-shared", "--cudart", "shared", "-o", tmp, *objs]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"link failed:\n{res.stderr[-6000:]}")
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
