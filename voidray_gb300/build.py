"""Builds the native library libvoidray_gb300.so for sm_103a, in-tree.

Each translation unit is compiled by nvcc in parallel, then linked into
``voidray_gb300/_lib/libvoidray_gb300.so`` with the CUDA runtime linked
statically.  The tracer's device code is compiled with ``-fmad=false`` and
host code with ``-ffp-contract=off`` so that every f32 operation on the
reference-estimator path rounds separately, as the reference computes it; the
denoiser's kernels keep FMA contraction.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIBDIR = PKG / "_lib"
LIB = LIBDIR / "libvoidray_gb300.so"

SOURCES = ["vr_build.cpp", "vr_kernels.cu", "vr_capi.cu", "vr_serve.cu", "dn_kernels.cu", "dn_unet.cu", "dn_tc.cu",
           "vr_image.cpp", "vr_obj.cpp"]
# the denoiser's translation units (compiled with FMA contraction)
DENOISER = {"dn_kernels.cu", "dn_unet.cu", "dn_tc.cu"}
# host-only translation units: compiled as plain C++ (no device code)
HOST_ONLY = {"vr_image.cpp", "vr_obj.cpp"}
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the GPU library cannot be built")


def _flags(src: str) -> list[str]:
    common = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off,-fno-fast-math",
              "-I", str(CSRC), "-I", str(PKG.parent / "include")]
    # tuning knobs for sweeps, e.g. VR_NVCC_EXTRA="-DVR_TRACE_MINB=12 -DVR_DYN_FETCH=16" (rebuild with --force)
    common += os.environ.get("VR_NVCC_EXTRA", "").split()
    if src in HOST_ONLY:
        return common + ["-x", "c++"]
    if src.endswith(".cu"):
        # the tracer reproduces the reference's f32 rounding operation by
        # operation; the denoiser's kernels have no such contract and keep FMA
        fmad = [] if src in DENOISER else ["-fmad=false"]
        return ARCH + common + fmad + ["-Xptxas", "-v" if os.environ.get("VR_PTXAS_VERBOSE") else "-O3"]
    return common + ["-x", "cu"] + ARCH + ["-fmad=false"]


def _stale(obj: Path, deps: list[Path]) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    LIBDIR.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list((PKG.parent / "include").glob("*.h"))
    procs = []
    objs = []
    for src in SOURCES:
        s = CSRC / src
        o = BUILD / (src + ".o")
        objs.append(o)
        if force or _stale(o, [s, *headers, Path(__file__)]):
            cmd = [nvcc(), "-c", str(s), "-o", str(o), *_flags(src)]
            if verbose:
                print(" ".join(cmd), file=sys.stderr)
            procs.append((src, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)))
    failed = []
    for src, p in procs:
        out, _ = p.communicate()
        if out and (verbose or p.returncode):
            print(out, file=sys.stderr)
        if p.returncode:
            failed.append(src)
    if failed:
        raise RuntimeError(f"nvcc failed for {failed}")
    if force or procs or not LIB.exists():
        tmp = LIB.with_suffix(".so.tmp")
        cmd = [nvcc(), "-shared", *ARCH, "-o", str(tmp), *map(str, objs), "-Xcompiler", "-fPIC,-pthread"]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        subprocess.run(cmd, check=True)
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
    print(LIB)
