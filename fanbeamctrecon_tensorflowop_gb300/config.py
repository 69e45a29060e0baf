"""Scan / image configuration with the field names of the reference's config.py.

The reference's drivers read these names (utils.py:19-22,57-69); keeping them
lets a user point their scripts at this package unchanged.  Values are the
reference defaults (config.py:9-42).  ``AttrDict`` stands in for EasyDict.
"""
from __future__ import annotations


class AttrDict(dict):
    """dict with attribute access (the subset of EasyDict the drivers use)."""

    def __getattr__(self, name):
        try:
            return self[name]
        except KeyError as e:
            raise AttributeError(name) from e

    def __setattr__(self, name, value):
        self[name] = value

    def copy(self) -> "AttrDict":
        return AttrDict(self)


def default_config() -> AttrDict:
    c = AttrDict()
    # [File]
    c.ProjectionFilename = "./test_prj.raw"
    c.ReconstructionFilename = "./test_img.raw"
    # [Scan]
    c.SourceType = 1            # 0: parallel beam, 1: cone beam
    c.DetectorType = 1          # 0: linear, 1: curved
    c.SourceDetectorDistance = 946.73233346   # mm
    c.SourceAxisDistance = 538.52             # mm
    c.StartAngle = 0            # degrees (added to radians by angle(), as the reference does)
    c.ProjectionsPerRotation = 984
    c.DetectorColumnNumber = 888
    c.DetectorCoverage = 200.1  # mm
    c.DetectorShift = 0         # channels
    c.DetectorRowNumber = 1
    c.FanAngle = 55.0059        # degrees
    c.FullAngle = 360           # 360: full scan
    c.ParkWeighting = 0
    # [Image]
    c.NX = 512
    c.NY = 512
    c.NZ = 1
    c.FOVRadius = 200           # mm
    c.DeltaZ = 0.625            # mm
    # [Reconstruction]
    c.Algorithm = "FBP"
    c.HelicalReconMode = 1
    c.FilterType = 1            # 1: Shepp-Logan ("S-L"); 0: Ram-Lak
    return c


config = default_config()
