"""In-tree build of libctgb.so (the CUDA kernels plus the C ABI) for sm_103a.

Every translation unit compiles in parallel with nvcc/g++; the shared library
links the CUDA runtime statically so it depends only on the driver.  Objects
and the library go to ``_build/`` next to this file.  The same pass builds
libctpeaks.so (``csrc/peaks``): the L1-load and FP32 microbenchmarks that give
the benchmark its roofline denominators; no operator uses it.
"""
from __future__ import annotations

import hashlib
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent
REPO_DIR = PKG_DIR.parent
CSRC = PKG_DIR / "csrc"
INCLUDE = REPO_DIR / "include"
BUILD_DIR = PKG_DIR / "_build"
LIB_NAME = "libctgb.so"
LIB_PATH = BUILD_DIR / LIB_NAME
PEAKS_SRC = CSRC / "peaks" / "peaks.cu"
PEAKS_PATH = BUILD_DIR / "libctpeaks.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3", "-std=c++17", "-lineinfo", "--expt-relaxed-constexpr",
    "-Xcompiler", "-fPIC,-ffp-contract=off,-O2",
    "-Xptxas", "-warn-spills",
] + ARCH
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-Wextra"]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libctgb.so")
    return cand


def _cuda_include() -> str:
    return str(Path(_nvcc()).resolve().parent.parent / "include")


def _sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))


def _headers() -> list[Path]:
    return sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + sorted(INCLUDE.glob("*.h"))


def _fingerprint(extra: str = "") -> str:
    h = hashlib.sha256(extra.encode())
    for p in _sources() + _headers():
        h.update(p.name.encode())
        h.update(p.read_bytes())
    h.update(PEAKS_SRC.read_bytes())
    h.update(" ".join(NVCC_FLAGS + CXX_FLAGS).encode())
    h.update(os.uname().machine.encode())
    return h.hexdigest()


def _compile(src: Path, out_dir: Path = BUILD_DIR, defines: tuple = ()) -> Path:
    obj = out_dir / (src.name + ".o")
    if src.suffix == ".cu":
        cmd = [_nvcc(), *NVCC_FLAGS, *defines, "-I", str(INCLUDE), "-c", str(src), "-o", str(obj)]
    else:
        cmd = ["g++", *CXX_FLAGS, *defines, "-I", str(INCLUDE), "-I", _cuda_include(), "-c",
               str(src), "-o", str(obj)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    if res.stderr.strip():
        sys.stderr.write(res.stderr)
    return obj


DEBUG_DIR = BUILD_DIR / "debug"


def build_debug(force: bool = False) -> Path:
    """The debug library (_build/debug/libctgb.so): the same sources with
    -DCT_DEBUG, whose kernels check every gather index (see dbgcheck.cuh)."""
    DEBUG_DIR.mkdir(parents=True, exist_ok=True)
    stamp = DEBUG_DIR / "stamp.txt"
    lib = DEBUG_DIR / LIB_NAME
    fp = _fingerprint("debug")
    if not force and lib.exists() and stamp.exists() and stamp.read_text() == fp:
        return lib
    srcs = _sources()
    with ThreadPoolExecutor(max_workers=max(1, min(len(srcs), os.cpu_count() or 4))) as ex:
        objs = list(ex.map(lambda p: _compile(p, DEBUG_DIR, ("-DCT_DEBUG",)), srcs))
    tmp = DEBUG_DIR / (LIB_NAME + ".tmp")
    cmd = [_nvcc(), "-shared", *ARCH, "-o", str(tmp), *map(str, objs)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, lib)
    stamp.write_text(fp)
    return lib


def build(force: bool = False, verbose: bool = False, debug: bool = False) -> Path:
    """Compiles libctgb.so unless an up-to-date build is present; returns its
    path.  debug=True builds (and returns) the index-checking debug library."""
    if debug:
        return build_debug(force)
    BUILD_DIR.mkdir(parents=True, exist_ok=True)
    stamp = BUILD_DIR / "stamp.txt"
    fp = _fingerprint()
    if (not force and LIB_PATH.exists() and PEAKS_PATH.exists() and stamp.exists()
            and stamp.read_text() == fp):
        return LIB_PATH
    srcs = _sources()
    with ThreadPoolExecutor(max_workers=max(1, min(len(srcs) + 1, os.cpu_count() or 4))) as ex:
        peaks = ex.submit(_compile, PEAKS_SRC)
        objs = list(ex.map(_compile, srcs))
        peaks_obj = peaks.result()
    tmp = BUILD_DIR / (LIB_NAME + ".tmp")
    cmd = [_nvcc(), "-shared", *ARCH, "-o", str(tmp), *map(str, objs)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB_PATH)
    tmp = BUILD_DIR / "libctpeaks.so.tmp"
    cmd = [_nvcc(), "-shared", *ARCH, "-o", str(tmp), str(peaks_obj)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, PEAKS_PATH)
    stamp.write_text(fp)
    if verbose:
        print(f"built {LIB_PATH}")
    return LIB_PATH


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
