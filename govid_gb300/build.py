"""Builds the GB300 decoder library in-tree.

Compiles every CUDA translation unit for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``) and the host C++ units with
g++, in parallel, and links ``govid_gb300/_lib/libebivgpu.so`` (CUDA runtime
linked statically).  Rebuilds only what changed.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
OUT = PKG / "_lib"
OBJ = OUT / "obj"
LIB = OUT / "libebivgpu.so"

CUDA_SOURCES = ["decode_kernels.cu", "gpu_codec.cu", "rgba_kernel.cu", "batch.cu", "serve.cu", "noalloc.cu", "mvnet_kernels.cu", "altref.cu", "ingest.cu", "analysis.cu", "source.cu"]
CXX_SOURCES = ["encoder.cpp", "container.cpp", "synth.cpp", "host_api.cpp", "payload.cpp"]

GENCODE = "-gencode=arch=compute_103a,code=sm_103a"


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the GB300 decoder cannot be built")


def _headers() -> list[Path]:
    return sorted(CSRC.glob("*.h")) + sorted((PKG.parent / "include").glob("*.h"))


def _stale(obj: Path, src: Path, deps: list[Path]) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return src.stat().st_mtime > t or any(d.stat().st_mtime > t for d in deps)


def _compile(cmd: list[str]) -> tuple[list[str], int, str]:
    p = subprocess.run(cmd, capture_output=True, text=True)
    return cmd, p.returncode, p.stdout + p.stderr


def build(verbose: bool = False, jobs: int | None = None) -> Path:
    OBJ.mkdir(parents=True, exist_ok=True)
    nvcc = _nvcc()
    deps = _headers()
    cmds = []
    objs = []
    for s in CUDA_SOURCES:
        src = CSRC / s
        if not src.exists():
            continue
        obj = OBJ / (s + ".o")
        objs.append(obj)
        if _stale(obj, src, deps):
            cmds.append([nvcc, GENCODE, "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
                         "-Xcompiler", "-fPIC,-ffp-contract=off", "-Xptxas", "-v" if verbose else "-O3",
                         "-c", str(src), "-o", str(obj)])
    cxx = os.environ.get("CXX", "g++")
    for s in CXX_SOURCES:
        src = CSRC / s
        obj = OBJ / (s + ".o")
        objs.append(obj)
        if _stale(obj, src, deps):
            cmds.append([cxx, "-O2", "-std=c++17", "-fPIC", "-pthread", "-ffp-contract=off", "-Wall",
                         "-c", str(src), "-o", str(obj)])
    if cmds:
        with cf.ThreadPoolExecutor(max_workers=jobs or min(len(cmds), os.cpu_count() or 4)) as ex:
            for cmd, rc, out in ex.map(_compile, cmds):
                if verbose or rc != 0:
                    sys.stderr.write(" ".join(cmd) + "\n" + out)
                if rc != 0:
                    raise RuntimeError(f"compile failed: {cmd[-3]}")
    if cmds or not LIB.exists():
        link = [nvcc, GENCODE, "-shared", "-o", str(LIB)] + [str(o) for o in objs] + ["-lpthread"]
        cmd, rc, out = _compile(link)
        if verbose or rc != 0:
            sys.stderr.write(" ".join(cmd) + "\n" + out)
        if rc != 0:
            raise RuntimeError("link failed")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
