"""Generates tests/golden/reference_geometry.json by EXECUTING the reference's
own Python geometry code (utils.py:49-88 and config.py) from a checkout of
FanBeamCTRecon_TensorflowOp.

TensorFlow, EasyDict and matplotlib are not installed, so minimal stand-ins
are put in sys.modules first: ``make_tensor_proto`` returns the numpy array
it is given, ``load_op_library`` returns an empty namespace and EasyDict is a
dict with attribute access.  Nothing else of the reference is touched; the
angle and parameter values below are exactly what its functions compute.

usage: python tests/golden/make_golden.py /path/to/reference
"""
from __future__ import annotations

import json
import sys
import types
from pathlib import Path

import numpy as np


def _install_stubs() -> None:
    def mod(name, **attrs):
        m = types.ModuleType(name)
        for k, v in attrs.items():
            setattr(m, k, v)
        sys.modules[name] = m
        return m

    class EasyDict(dict):
        def __getattr__(self, k):
            try:
                return self[k]
            except KeyError as e:
                raise AttributeError(k) from e

        def __setattr__(self, k, v):
            self[k] = v

    mod("easydict", EasyDict=EasyDict)
    tu = mod("tensorflow.python.framework.tensor_util",
             make_tensor_proto=lambda values, dtype=None: np.array(values, copy=True))
    fw = mod("tensorflow.python.framework", ops=types.SimpleNamespace(), tensor_util=tu)
    mod("tensorflow.python", framework=fw)
    keras = mod("tensorflow.keras", models=types.SimpleNamespace(), layers=types.SimpleNamespace())
    mod("tensorflow.keras.models")
    mod("tensorflow.keras.layers")
    mod("tensorflow", float32="float32", keras=keras,
        load_op_library=lambda path: types.SimpleNamespace(path=path))
    mpl = mod("matplotlib")
    mpl.pylab = mod("matplotlib.pylab")


def main(ref: Path) -> None:
    _install_stubs()
    sys.path.insert(0, str(ref))
    import config as ref_config  # noqa: E402  (the reference's config.py)
    import utils as ref_utils  # noqa: E402  (the reference's utils.py)

    cfg = ref_config.config
    out: dict = {
        "source": "FanBeamCTRecon_TensorflowOp utils.py:49-88, config.py:9-42 (executed)",
        "config": {k: cfg[k] for k in sorted(cfg)},
        "cases": [],
    }

    def case(label, nimg, start_deg):
        old = cfg.StartAngle
        cfg.StartAngle = start_deg
        try:
            ang = np.asarray(ref_utils.angle(cfg.ProjectionsPerRotation, cfg.StartAngle),
                             dtype=np.float32)
            par = np.asarray(ref_utils.param_set(nimg), dtype=np.float32)
        finally:
            cfg.StartAngle = old
        out["cases"].append({
            "label": label, "nimg": nimg, "start_angle": start_deg,
            # float32 values written as the exact doubles they convert to
            "parameter": [float(v) for v in par],
            "angle": [float(v) for v in ang],
        })

    case("default", 1, 0)
    case("batch4", 4, 0)
    case("start30deg", 2, 30)

    # A second geometry through the same code: config.py's alternative scanner
    # (the commented values on config.py:13-18: SDD 1117.6, SAD 889, 1081 views,
    # 2001 channels) with a detector shift.
    saved = dict(cfg)
    cfg.SourceDetectorDistance = 1117.6
    cfg.SourceAxisDistance = 889
    cfg.ProjectionsPerRotation = 1081
    cfg.DetectorColumnNumber = 2001
    cfg.DetectorShift = 1.25
    case("alt_scanner_shift", 1, 0)
    cfg.clear()
    cfg.update(saved)

    path = Path(__file__).resolve().parent / "reference_geometry.json"
    path.write_text(json.dumps(out, indent=1))
    print(f"wrote {path}")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {Path(__file__).name} <reference checkout>")
    main(Path(sys.argv[1]))
