"""Build recipe for the CUDA library ``openusct_gb300/libusct_gb300.so``.

One ``-gencode`` (sm_103a), built in-tree with nvcc: the engine, the no-alloc
entry point, the model-update kernels, the TFM imaging kernels, and the
TMA-ring kernels once per
shot-channel count; the objects compile in parallel, then link.
``-fmad=false`` keeps every multiply-add unfused unless the kernels ask for
``__fmaf_rn`` explicitly, which fixes the rounding of the stencil so the CPU
restatement can reproduce it bit for bit.
"""

from __future__ import annotations

import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
LIB = os.path.join(PKG, "libusct_gb300.so")
# (source, object, extra flags): the TMA-ring kernels are built once per
# shot-channel count C, each as its own object
TMA_CHANNELS = (1, 2, 4, 8, 16, 32, 64)
SOURCES = [("usct_engine.cu", "usct_engine.o", []), ("usct_noalloc.cu", "usct_noalloc.o", []),
           ("usct_invert.cu", "usct_invert.o", []), ("usct_tfm.cu", "usct_tfm.o", [])] + [
    ("usct_tma_inst.cu", f"usct_tma_c{c}.o", [f"-DUSCT_TMA_C={c}"]) for c in TMA_CHANNELS]
DEPS = ["usct_engine.cu", "usct_noalloc.cu", "usct_invert.cu", "usct_tfm.cu", "usct_tma_inst.cu",
        "usct_kernels.cuh", "usct_plain.cuh", "usct_tma.cuh", "usct_tma2.cuh", "usct_convert.cuh"]
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libusct_gb300.so")


OBJDIR = os.path.join(PKG, "_build")


def compile_command(src: str, obj: str, verbose_ptxas: bool = False,
                    extra: list[str] | None = None) -> list[str]:
    cmd = [nvcc(), ARCH, "-O3", "-lineinfo", "-fmad=false", "-std=c++17",
           "-Xcompiler", "-fPIC", "-I", os.path.join(REPO, "include")] + list(extra or []) + [
           "-c", "-o", obj, os.path.join(CSRC, src)]
    if verbose_ptxas:
        cmd.insert(1, "-Xptxas=-v")
    return cmd


def link_command(objs: list[str], out: str) -> list[str]:
    return [nvcc(), ARCH, "-shared", "-o", out] + objs


def up_to_date(out: str = LIB) -> bool:
    if not os.path.exists(out):
        return False
    t = os.path.getmtime(out)
    deps = [os.path.join(CSRC, d) for d in DEPS] + [os.path.join(REPO, "include", "usct_gb300.h")]
    return all(os.path.getmtime(d) <= t for d in deps)


def build(force: bool = False, verbose_ptxas: bool = False) -> str:
    """Compile the library if a source is newer than it; return its path.

    The translation units compile in parallel (one nvcc each), then link."""
    if force or not up_to_date():
        os.makedirs(OBJDIR, exist_ok=True)
        objs = [os.path.join(OBJDIR, obj) for _, obj, _ in SOURCES]
        cmds = [compile_command(src, o, verbose_ptxas, extra)
                for (src, _, extra), o in zip(SOURCES, objs)]
        procs = [subprocess.Popen(c) for c in cmds]
        codes = [p.wait() for p in procs]
        for c, code in zip(cmds, codes):
            if code:
                raise subprocess.CalledProcessError(code, c)
        tmp = LIB + ".tmp"
        subprocess.run(link_command(objs, tmp), check=True)
        os.replace(tmp, LIB)
    return LIB


EXAMPLE = os.path.join(CSRC, "usct_example.cpp")


def build_example(out: str) -> str:
    """Compile the plain C++ example against the library (host compiler only)."""
    build()
    cxx = os.environ.get("CXX") or shutil.which("g++") or "c++"
    subprocess.run([cxx, "-O2", "-std=c++14", "-I", os.path.join(REPO, "include"), EXAMPLE,
                    "-L", PKG, "-lusct_gb300", f"-Wl,-rpath,{PKG}", "-o", out], check=True)
    return out


if __name__ == "__main__":
    build(force=True, verbose_ptxas=True)
