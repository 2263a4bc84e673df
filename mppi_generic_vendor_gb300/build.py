"""Build libmppi_gb.so in-tree with nvcc (sm_103a only).

The translation units are compiled in parallel and linked into
``mppi_generic_vendor_gb300/_build/libmppi_gb.so``.  Device code is compiled with ``--fmad=false`` and host code with
``-ffp-contract=off`` so that the only fused multiply-adds are the ones the source writes explicitly; the rollout
arithmetic is then bit-reproducible against a CPU restatement that follows the same expression order.
"""
from __future__ import annotations

import hashlib
import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent
CSRC = PKG_DIR / "csrc"
INCLUDE = PKG_DIR.parent / "include"
BUILD_DIR = PKG_DIR / "_build"
LIB_NAME = "libmppi_gb.so"

ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3",
    "-std=c++17",
    "-lineinfo",
    "--fmad=false",
    "-Xcompiler",
    "-fPIC,-ffp-contract=off,-O2",
    "-I" + str(INCLUDE),
]


# Translation units whose parity with the CPU restatement is a tolerance rather than bit equality (the colored-noise
# FFT) are compiled with FMA contraction.
FMAD_TRUE = {"mg_colored.cu"}


def nvcc_path() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libmppi_gb.so")


def sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu"))


def _fingerprint() -> str:
    h = hashlib.sha256()
    for p in sorted(list(CSRC.glob("*")) + list(INCLUDE.glob("*.h"))):
        if p.is_file():
            h.update(p.name.encode())
            h.update(p.read_bytes())
    h.update(" ".join(ARCH_FLAGS + NVCC_FLAGS).encode())
    h.update(os.uname().machine.encode())
    return h.hexdigest()


def lib_path() -> Path:
    return BUILD_DIR / LIB_NAME


def build(force: bool = False, verbose: bool = False, jobs: int | None = None) -> Path:
    """Compile every CUDA translation unit and link the shared library; skipped when nothing changed."""
    BUILD_DIR.mkdir(parents=True, exist_ok=True)
    stamp = BUILD_DIR / "stamp.txt"
    fp = _fingerprint()
    if not force and lib_path().exists() and stamp.exists() and stamp.read_text() == fp:
        return lib_path()
    nvcc = nvcc_path()
    srcs = sources()
    objs = [BUILD_DIR / (s.stem + ".o") for s in srcs]

    def compile_one(pair):
        src, obj = pair
        flags = [("--fmad=true" if (f == "--fmad=false" and src.name in FMAD_TRUE) else f) for f in NVCC_FLAGS]
        cmd = [nvcc, *ARCH_FLAGS, *flags, "-c", str(src), "-o", str(obj)]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src.name}:\n{r.stdout}\n{r.stderr}")
        return r.stderr if verbose else ""

    n = jobs or min(len(srcs), os.cpu_count() or 4)
    with ThreadPoolExecutor(max_workers=n) as ex:
        logs = list(ex.map(compile_one, zip(srcs, objs)))
    if verbose:
        for log in logs:
            print(log)
    out = lib_path()
    tmp = out.with_suffix(".so.tmp")
    cmd = [nvcc, *ARCH_FLAGS, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, out)
    stamp.write_text(fp)
    return out


if __name__ == "__main__":
    import sys

    p = build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(p)
