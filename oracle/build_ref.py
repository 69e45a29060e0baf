"""Builds the executed-reference checker: the reference's own op sources,
compiled where they lie, linked against host stand-ins for TensorFlow, the
CUDA runtime (texture references included) and Intel IPP, into
``oracle/_ref/libref_{fp,bp,fbp,fdk}.so``.  TEST INFRASTRUCTURE ONLY: the
golden-vector script and the tests use these libraries as the checker; no
product code loads them.

Per op, three translation units:

* the op wrapper (``FP/transform.cc`` ...), compiled as is against the
  TensorFlow stand-in headers in ``refexec/standin``;
* the CUDA source (``FP/transform.cu`` ...), compiled as C++ with the CUDA
  stand-in force-included.  The only change to its text is the launch syntax
  ``k<<<grid, block>>>(args)``, which no C++ compiler parses: it becomes
  ``::ctref::launch(&k, grid, block)(args)``.  The rewritten text is piped to
  the compiler's standard input and never written to disk, so no copy of a
  reference source exists anywhere;
* ``refexec/harness.cpp``: the block scheduler, the op registry and the C
  ABI (``ctref_run``, ``ctref_shape``).

Nothing here runs the reference's own build system.  The reference is found at
``$CTREF_REFERENCE`` or ``/root/reference``; without it nothing is built.

usage: python oracle/build_ref.py [reference-dir]
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import re
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
STANDIN = HERE / "refexec" / "standin"
HARNESS = HERE / "refexec" / "harness.cpp"

# op -> (CUDA source, op wrapper, registered op name)
OPS = {
    "fp": ("FP/transform.cu", "FP/transform.cc", "FPFanCurve"),
    "bp": ("BP/transform.cu", "BP/transform.cc", "BPFanCurve"),
    "fbp": ("FBP/transform.cu", "FBP/transform.cc", "FBPFanCurve"),
    "fdk": ("FDK/GPURecon_GPU.cu", "FDK/FBP.cc", "BackProjection"),
}

CXX = os.environ.get("CXX", "g++")
FLAGS = ["-std=c++17", "-O2", "-fPIC", "-fopenmp", "-ffp-contract=off"]
_LAUNCH = re.compile(r"(\w+)\s*<<<(.*?)>>>")


def default_reference() -> Path:
    return Path(os.environ.get("CTREF_REFERENCE", "/root/reference"))


def rewrite_launches(text: str) -> str:
    """``k<<<g, b>>>`` -> ``::ctref::launch(&k, g, b)`` (the only text change)."""
    return _LAUNCH.sub(lambda m: f"::ctref::launch(&{m.group(1)}, {m.group(2)})", text)


def _run(cmd, stdin_text=None):
    res = subprocess.run(cmd, input=stdin_text, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("command failed: " + " ".join(map(str, cmd)) + "\n" + res.stderr[-4000:])


def _fingerprint(ref: Path) -> str:
    h = hashlib.sha256()
    for f in sorted(STANDIN.rglob("*")) + [HARNESS, HERE / "texture_rule.h", Path(__file__)]:
        if f.is_file():
            h.update(f.read_bytes())
    for cu, cc, _ in OPS.values():
        for f in (ref / cu, ref / cc):
            h.update(f.read_bytes())
    h.update(" ".join([CXX] + FLAGS).encode())
    return h.hexdigest()


def _build_op(ref: Path, op: str) -> Path:
    cu, cc, _ = OPS[op]
    obj = OUT / "obj"
    obj.mkdir(parents=True, exist_ok=True)
    src_dir = (ref / cu).parent
    o_cu, o_cc, o_h = obj / f"{op}_cu.o", obj / f"{op}_cc.o", obj / f"{op}_harness.o"
    inc = ["-I", str(STANDIN), "-iquote", str(src_dir)]
    text = f'#line 1 "{ref / cu}"\n' + rewrite_launches((ref / cu).read_text())
    _run([CXX, *FLAGS, "-w", *inc, "-DCTREF_KERNEL_SOURCE", "-include",
          str(STANDIN / "ctref_cuda.h"), "-x", "c++", "-", "-c", "-o", str(o_cu)], text)
    _run([CXX, *FLAGS, "-w", *inc, "-c", str(ref / cc), "-o", str(o_cc)])
    _run([CXX, *FLAGS, "-Wall", "-I", str(HERE / "refexec"), "-c", str(HARNESS), "-o", str(o_h)])
    lib = OUT / f"libref_{op}.so"
    _run([CXX, "-shared", "-fopenmp", "-o", str(lib), str(o_cu), str(o_cc), str(o_h)])
    return lib


def build(ref: Path | None = None, force: bool = False) -> dict[str, Path] | None:
    """Builds every op library; returns {op: path}, or None without a reference."""
    ref = Path(ref) if ref is not None else default_reference()
    if not all((ref / cu).is_file() and (ref / cc).is_file() for cu, cc, _ in OPS.values()):
        return None
    OUT.mkdir(parents=True, exist_ok=True)
    stamp = OUT / "stamp.txt"
    fp = _fingerprint(ref)
    libs = {op: OUT / f"libref_{op}.so" for op in OPS}
    if not force and stamp.exists() and stamp.read_text() == fp and all(p.exists() for p in libs.values()):
        return libs
    with cf.ThreadPoolExecutor(max_workers=len(OPS)) as ex:
        futs = {op: ex.submit(_build_op, ref, op) for op in OPS}
        libs = {op: f.result() for op, f in futs.items()}
    stamp.write_text(fp)
    return libs


if __name__ == "__main__":
    r = build(Path(sys.argv[1]) if len(sys.argv) > 1 else None, force=True)
    print(r if r else "reference sources not found: nothing built")
