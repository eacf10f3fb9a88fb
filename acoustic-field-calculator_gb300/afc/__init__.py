"""afc -- Python API of the GB300 acoustic-field library (libafccapi.so).

Mirrors the reference's python/afc package (python/afc/__init__.py:14-40): same class names and
the same ctypes bindings.  The shared library is built in-tree (build_lib.py); unlike the
reference, nothing is downloaded: a missing library raises ImportError.
"""
import os

from . import nativemethods
from .afc import (AccurateCalculator, Axis, ComplexPressureFieldBuffer, CpuCalculator,
                  GpuCalculator, GridAreaBuilder, Optimizer, PowerFieldBuffer,
                  PressureFieldBuffer, ScatterArea, UniformSystem, grid_from_spec, last_error)
from .nativemethods import SphereWaveSource, T4010A1, Vector3

__all__ = [
    "UniformSystem", "CpuCalculator", "AccurateCalculator", "GpuCalculator",
    "PressureFieldBuffer", "PowerFieldBuffer", "ComplexPressureFieldBuffer", "ScatterArea",
    "GridAreaBuilder", "SphereWaveSource", "T4010A1", "Vector3", "Optimizer", "Axis",
    "grid_from_spec", "last_error",
]

_Version = "0.6.1"

PKG_DIR = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.environ.get("AFC_LIB_PATH", os.path.join(PKG_DIR, "lib", "libafccapi.so"))

if not os.path.isfile(LIB_PATH):
    raise ImportError(f"{LIB_PATH} is missing: build it with build_lib.py (no CPU fallback exists)")

DLL = nativemethods.init_dll(LIB_PATH)
