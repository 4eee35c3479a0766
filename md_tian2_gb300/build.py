"""Build the engine's shared library libmdt_gpu.so in-tree for sm_103a.

Each CUDA translation unit under ``csrc/`` is compiled by nvcc in parallel and linked
into ``md_tian2_gb300/libmdt_gpu.so``.  No torch headers are involved: the library is
a plain C ABI (``include/mdt_gpu.h``).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
OUT_DIR = PKG / "_build"
LIB = PKG / "libmdt_gpu.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["mdt_api.cu", "mdt_md.cu", "mdt_peak.cu", "mdt_nn.cu", "mdt_noalloc.cu", "mdt_train.cu", "mdt_train_gemm.cu",
           "mdt_nnf.cu", "mdt_nnr.cu"]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the CUDA engine cannot be built")
    return cand


def _compile(src: Path, obj: Path, extra: list[str]) -> None:
    cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off", "--expt-relaxed-constexpr",
           "-I", str(CSRC), "-I", str(PKG.parent / "include"), "-c", str(src), "-o", str(obj), *extra]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src.name}:\n{r.stdout}\n{r.stderr}")


def build(verbose: bool = False, extra: list[str] | None = None, force: bool = False) -> Path:
    """Compile every translation unit and link libmdt_gpu.so.  Returns the library path."""
    extra = list(extra or [])
    OUT_DIR.mkdir(exist_ok=True)
    srcs = [CSRC / s for s in SOURCES if (CSRC / s).exists()]
    headers = list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + [PKG.parent / "include" / "mdt_gpu.h"]
    newest_hdr = max((h.stat().st_mtime for h in headers if h.exists()), default=0.0)
    jobs = []
    for s in srcs:
        o = OUT_DIR / (s.stem + ".o")
        if force or not o.exists() or o.stat().st_mtime < max(s.stat().st_mtime, newest_hdr):
            jobs.append((s, o))
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for f in [ex.submit(_compile, s, o, extra) for s, o in jobs]:
            f.result()
    objs = [str(OUT_DIR / (s.stem + ".o")) for s in srcs]
    if jobs or not LIB.exists():
        tmp = LIB.with_suffix(".so.tmp")
        cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *objs, "-lcudart", "-lcublas"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    if verbose:
        print(f"built {LIB}", file=sys.stderr)
    return LIB


if __name__ == "__main__":
    build(verbose=True, force="--force" in sys.argv)
