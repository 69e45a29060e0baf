"""Generates tests/golden/reference_fdk_driver.json by EXECUTING the reference's
FDK training-data driver, FDK_generate of FDK/FDK_test_training.py:18-141,
from a checkout of FanBeamCTRecon_TensorflowOp.

TensorFlow, matplotlib and psutil are not installed, so stand-ins are put in
sys.modules first.  They record instead of compute:

* ``tf.load_op_library(...).BackProjection(**kw)`` records its keyword
  arguments (the projection, angle and parameter the driver builds) and
  returns an object whose ``eval()`` gives zeros of ``vol_shape``;
* ``make_tensor_proto`` / ``convert_to_tensor`` return their numpy input and
  ``tf.Session`` is an empty context manager.

The driver's module-level ``read_binary_dataset`` (which reads absolute paths
of private data) is replaced by synthetic arrays proj[s, v, c] = 1000 s + v
+ c / 1000 (+ 0.5 for the m1 file ...), and its ``np.save`` / ``open`` /
``print`` by recorders, so nothing is written.  The recorded parameter and
angle vectors, the printed view shift, the view order of the rolled
projections, the scale of the high sinogram and the file names and shapes
the driver would save are what the tests compare the batched driver against.

usage: python tests/golden/make_golden_fdk_driver.py /path/to/reference
"""
from __future__ import annotations

import importlib.util
import json
import sys
import types
from pathlib import Path

import numpy as np

CHANNEL_OFFSET = {"high": 0.0, "m1": 0.5, "m2": 0.25, "energy": 0.125, "mask": 0.0625}


def synthetic(path: str, nslice: int, nview: int, ncol: int) -> np.ndarray:
    ch = path.rsplit("_", 1)[1].split(".")[0]
    s = np.arange(nslice, dtype=np.float64)[:, None, None]
    v = np.arange(nview, dtype=np.float64)[None, :, None]
    c = np.arange(ncol, dtype=np.float64)[None, None, :]
    return (1000.0 * s + v + c / 1000.0 + CHANNEL_OFFSET[ch]).astype(np.float32)


class _Recorder:
    def __init__(self):
        self.calls, self.saves, self.raws, self.prints = [], [], [], []


def _install_stubs(rec: _Recorder) -> None:
    def mod(name, **attrs):
        m = types.ModuleType(name)
        for k, v in attrs.items():
            setattr(m, k, v)
        sys.modules[name] = m
        return m

    class _Op:
        def __init__(self, vol_shape):
            self.vol_shape = vol_shape

        def eval(self):
            return np.zeros(self.vol_shape, np.float32)

    def back_projection(**kw):
        rec.calls.append({k: (np.array(v, copy=True) if isinstance(v, np.ndarray) else v)
                          for k, v in kw.items()})
        return _Op(kw["vol_shape"])

    class _Session:
        def __init__(self, *a, **k):
            pass

        def __enter__(self):
            return self

        def __exit__(self, *a):
            return False

    contrib = types.SimpleNamespace(
        util=types.SimpleNamespace(make_tensor_proto=lambda values, dtype=None:
                                   np.array(values, copy=True)))
    mod("tensorflow", float32="float32", contrib=contrib, Session=_Session,
        convert_to_tensor=lambda x, dtype=None: x,
        load_op_library=lambda path: types.SimpleNamespace(BackProjection=back_projection))
    mpl = mod("matplotlib")
    mpl.pylab = mod("matplotlib.pylab")
    mod("psutil", virtual_memory=lambda: types.SimpleNamespace(percent=0.0))


def run_case(ref: Path, index: int, fstart: float, nview: int, nslice: int) -> dict:
    rec = _Recorder()
    _install_stubs(rec)
    spec = importlib.util.spec_from_file_location(
        "ref_fdk_driver", ref / "FDK" / "FDK_test_training.py")
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)

    m.read_binary_dataset = synthetic

    class _NpProxy:
        def __getattr__(self, k):
            return getattr(np, k)

        @staticmethod
        def save(name, arr):
            rec.saves.append((name, list(np.shape(arr)), str(np.asarray(arr).dtype),
                              float(np.asarray(arr, np.float64).sum())))

    class _File:
        def __init__(self, name, mode):
            self.name, self.n = name, 0

        def write(self, b):
            self.n += len(b)

        def close(self):
            rec.raws.append((self.name, self.n))

    m.np = _NpProxy()
    m.open = _File
    m.print = lambda *a, **k: rec.prints.append(" ".join(str(x) for x in a))
    m.FDK_generate(index, fstart, nview, nslice, folder="Training")

    first = rec.calls[0]
    proj = np.asarray(first["projection"])
    # the three channels reconstructed per slice: high / 49000, m1, m2
    per_slice = [[float(np.asarray(c["projection"], np.float64).sum()) for c in rec.calls[3 * i:3 * i + 3]]
                 for i in range(nslice)]
    return {
        "index": index, "fstart_angle": fstart, "nview_full": nview, "nslice": nslice,
        "printed_shift": rec.prints[0],
        "parameter": [float(v) for v in np.asarray(first["parameter"], np.float32)],
        "angle": [float(v) for v in np.asarray(first["angle"], np.float32)],
        "vol_shape": list(first["vol_shape"]), "proj_shape": list(first["proj_shape"]),
        # view order of the rolled high sinogram of slice 0 (channel 0 holds
        # v / 49000 there: recover v)
        "view_order": [int(round(float(x) * 49000.0)) for x in proj[0, :, 0]],
        "high_first": float(proj[0, 1, 1]),
        "projection_sums": per_slice,
        "saves": [{"name": n.split("/")[-1], "shape": s, "dtype": d, "sum": t}
                  for n, s, d, t in rec.saves],
        "raws": [{"name": n, "bytes": b} for n, b in rec.raws],
        "n_calls": len(rec.calls),
    }


def main(ref: Path) -> None:
    out = {"source": "FanBeamCTRecon_TensorflowOp FDK/FDK_test_training.py:18-141 (executed)",
           "cases": []}
    # a start angle of the driver's own list, a negative one, one on a
    # rounding half (-(-0.5 * 360/24) / (360/24) = 0.5 -> round to 0) and one
    # with no shift
    for fstart, nview in ((56.4605480091944, 40), (-127.70155229882, 36), (-7.5, 24),
                          (0.0, 30)):
        out["cases"].append(run_case(ref, 7, fstart, nview, 2))
    path = Path(__file__).resolve().parent / "reference_fdk_driver.json"
    path.write_text(json.dumps(out, indent=1))
    print(f"wrote {path}")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {Path(__file__).name} <reference checkout>")
    main(Path(sys.argv[1]))
