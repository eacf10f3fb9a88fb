"""Python API over libafccapi.so, mirroring the reference's python/afc/afc.py (classes, method
names, argument meaning and tags are the same; see python/afc/afc.py:24-560 of the reference).

Differences:
  * every calculator computes on the GPU; a failed native call raises RuntimeError with the
    library's message instead of aborting the process;
  * every Optimizer method runs on the GPU except ifft, which raises RuntimeError
    (unsupported: an image-file set-up step outside this library);
  * additions marked NEW: explicit wavenumber / attenuation sources, a numpy view of the source
    array, and opt-in source tracking (UniformSystem.track_sources / sources_changed) that lets
    a calculator skip re-uploading sources that have not changed.
"""
from __future__ import annotations

import ctypes
from ctypes import POINTER, byref, c_float, c_uint, c_ulong, c_void_p
from enum import IntEnum

import numpy as np

from . import nativemethods
from .nativemethods import SphereWaveSource, T4010A1, Vector3


def _dll():
    if nativemethods.AFC_DLL is None:
        raise RuntimeError("libafccapi.so is not loaded")
    return nativemethods.AFC_DLL


def last_error() -> str:
    msg = _dll().AFC_GetLastError()
    return msg.decode("utf-8") if msg else ""


def _check(before: str = ""):
    msg = last_error()
    if msg and msg != before:
        _dll().AFC_ClearLastError()
        raise RuntimeError(msg)


class Axis(IntEnum):
    X = 1
    Y = 2
    Z = 3


class UniformSystem:
    def __init__(self, temperature):
        self.handle = c_void_p()
        self.temperature = temperature
        self._source_type = -1

    def __del__(self):
        if self.handle and nativemethods.AFC_DLL is not None:
            nativemethods.AFC_DLL.AFC_FreeUniformSystem(self.handle, self._source_type)
            self.handle = c_void_p()

    def set_source_type(self, v):
        self._source_type = v

    def __check_and_init(self, source):
        if self._source_type == -1:
            self._source_type = source.get_type()
            _dll().AFC_CreateUniformSystem(byref(self.handle), self.temperature,
                                           self._source_type)
        elif self._source_type != source.get_type():
            raise TypeError("Source type error! Mixing sound source types is not allowed.")

    def sound_speed(self):
        if self.handle:
            return _dll().AFC_UniformSystemSoundSpeed(self.handle, self._source_type)
        raise TypeError("Please add sound source before.")

    def info(self):
        if self.handle:
            info = _dll().AFC_UniformSystemInfo(self.handle, self._source_type)
            print(info.decode("utf-8"))

    def info_of_source(self, idx: int):
        if self.handle:
            info = _dll().AFC_UniformSystemSourceInfo(self.handle, idx, self._source_type)
            print(info.decode("utf-8"))

    def info_string(self) -> str:
        return _dll().AFC_UniformSystemInfo(self.handle, self._source_type).decode("utf-8")

    def source_info_string(self, idx: int) -> str:
        return _dll().AFC_UniformSystemSourceInfo(self.handle, idx,
                                                  self._source_type).decode("utf-8")

    def add_wave_source(self, source):
        self.__check_and_init(source)
        if isinstance(source, SphereWaveSource):
            _dll().AFC_AddSphereWaveSource(self.handle, source)
        elif isinstance(source, T4010A1):
            _dll().AFC_AddT4010A1(self.handle, source)
        else:
            raise TypeError("Unknown source type")

    def add_wave_source_with_wavenum_atten(self, source, wavenum: float, atten: float):
        """NEW: explicit wavenumber [rad/mm] and attenuation [Np/mm]."""
        self.__check_and_init(source)
        if isinstance(source, SphereWaveSource):
            _dll().AFC_AddSphereWaveSourceWithWavenumAtten(self.handle, source, wavenum, atten)
        elif isinstance(source, T4010A1):
            _dll().AFC_AddT4010A1WithWavenumAtten(self.handle, source, wavenum, atten)
        else:
            raise TypeError("Unknown source type")

    def add_records(self, source_type: int, records: np.ndarray, wavenums=None, attens=None):
        """NEW: add many sources given as rows of the ABI layout (9 or 6 float32)."""
        cls = T4010A1 if source_type == 1 else SphereWaveSource
        records = np.ascontiguousarray(records, dtype=np.float32)
        for i, rec in enumerate(records):
            s = cls.from_buffer_copy(rec.tobytes())
            if wavenums is None:
                self.add_wave_source(s)
            else:
                self.add_wave_source_with_wavenum_atten(s, float(wavenums[i]), float(attens[i]))

    def get_wave_sources(self):
        ptr = c_void_p()
        size = _dll().AFC_GetWaveSources(self.handle, byref(ptr), self._source_type)
        if self._source_type == 0:
            return ctypes.cast(ptr, POINTER(SphereWaveSource * size)).contents
        if self._source_type == 1:
            return ctypes.cast(ptr, POINTER(T4010A1 * size)).contents
        raise TypeError("Unknown source type")

    def track_sources(self, enable: bool = True):
        """NEW, opt-in: reuse the device copy of unchanged sources between calculations.
        Writes through an array obtained earlier (get_wave_sources, records) must then be
        announced with sources_changed(); changes made through this library are seen by
        themselves."""
        if _dll().AFC_UniformSystemTrackSources(self.handle, self._source_type,
                                                1 if enable else 0) != 0:
            _check()

    def sources_changed(self):
        """NEW: announce writes made through an earlier source array (see track_sources)."""
        if _dll().AFC_UniformSystemSourcesChanged(self.handle, self._source_type) != 0:
            _check()

    def records(self) -> np.ndarray:
        """NEW: a numpy view (n x 9 or n x 6 float32) of the system's source array."""
        ptr = c_void_p()
        size = _dll().AFC_GetWaveSources(self.handle, byref(ptr), self._source_type)
        width = 9 if self._source_type == 1 else 6
        if size == 0:
            return np.zeros((0, width), np.float32)
        arr = np.ctypeslib.as_array(ctypes.cast(ptr, POINTER(c_float)), shape=(size * width,))
        return arr.reshape(size, width)


class Calculator:
    def __init__(self):
        self.handle = c_void_p()
        _dll().AFC_CreateCalculator(byref(self.handle), self.get_type())

    def __del__(self):
        if self.handle and nativemethods.AFC_DLL is not None:
            nativemethods.AFC_DLL.AFC_FreeCalculator(self.handle, self.get_type())
            self.handle = c_void_p()

    def calculate_raw(self, system, observe_area, field):
        """NEW: returns (element count, pointer) straight from AFC_Calculate."""
        ptr = c_void_p()
        _dll().AFC_ClearLastError()
        size = _dll().AFC_Calculate(self.handle, system.handle, observe_area.handle,
                                    field.handle, byref(ptr), self.get_type(),
                                    system._source_type, observe_area.get_type(),
                                    field.get_type())
        if not ptr:
            _check()
            raise RuntimeError("AFC_Calculate returned no buffer")
        return size, ptr

    def calculate(self, system, observe_area, field):
        """Returns a numpy copy of the result (the reference returns a view of the field
        buffer, which dangles once the buffer is freed or grown; a copy cannot)."""
        size, ptr = self.calculate_raw(system, observe_area, field)
        fptr = ctypes.cast(ptr, POINTER(c_float))
        if field.get_type() == 2:
            if size == 0:
                return np.zeros(0, np.complex128)
            carray = np.ctypeslib.as_array(fptr, shape=(size, 2))
            return carray.view(np.complex64).reshape(size).astype(np.complex128)
        if size == 0:
            return np.zeros(0, np.float32)
        return np.ctypeslib.as_array(fptr, shape=(size,)).copy()

    @staticmethod
    def get_type():
        raise NotImplementedError()


class CpuCalculator(Calculator):
    @staticmethod
    def get_type():
        return 0


class AccurateCalculator(Calculator):
    @staticmethod
    def get_type():
        return 1


class GpuCalculator(Calculator):
    @staticmethod
    def get_type():
        return 2


class FieldBuffer:
    def __init__(self):
        self.handle = c_void_p()

    @staticmethod
    def get_type():
        raise NotImplementedError()


class _NamedField(FieldBuffer):
    _name = ""

    def __init__(self):
        super().__init__()
        getattr(_dll(), f"AFC_Create{self._name}Field")(byref(self.handle))

    def __del__(self):
        if self.handle and nativemethods.AFC_DLL is not None:
            getattr(nativemethods.AFC_DLL, f"AFC_Free{self._name}Field")(self.handle)
            self.handle = c_void_p()


class PressureFieldBuffer(_NamedField):
    _name = "Pressure"

    @staticmethod
    def get_type():
        return 0


class PowerFieldBuffer(_NamedField):
    _name = "Power"

    @staticmethod
    def get_type():
        return 1


class ComplexPressureFieldBuffer(_NamedField):
    _name = "ComplexPressure"

    @staticmethod
    def get_type():
        return 2


class ObserveArea:
    def __init__(self):
        self.handle = c_void_p()

    @staticmethod
    def get_type():
        raise NotImplementedError()


class ScatterArea(ObserveArea):
    def __init__(self):
        super().__init__()
        _dll().AFC_CreateScatterArea(byref(self.handle))

    def __del__(self):
        if self.handle and nativemethods.AFC_DLL is not None:
            nativemethods.AFC_DLL.AFC_FreeScatterArea(self.handle)
            self.handle = c_void_p()

    def add_observe_point(self, p):
        if not isinstance(p, Vector3):
            p = Vector3(p)
        _dll().AFC_ScatterAddObservePoint(self.handle, p)

    def add_observe_points(self, pts: np.ndarray):
        """NEW: add rows of an (m, 3) array in order."""
        fn = _dll().AFC_ScatterAddObservePoint
        for x, y, z in np.asarray(pts, dtype=np.float32):
            fn(self.handle, Vector3((x, y, z)))

    @staticmethod
    def get_type():
        return 3


class GridArea(ObserveArea):
    def __del__(self):
        if self.handle and nativemethods.AFC_DLL is not None:
            nativemethods.AFC_DLL.AFC_FreeGridArea(self.handle, self.get_dimension())
            self.handle = c_void_p()

    def get_size(self):
        f, s, t = c_uint(), c_uint(), c_uint()
        _dll().AFC_GetGridSize(self.handle, self.get_dimension(), byref(f), byref(s), byref(t))
        return (f.value, s.value, t.value)

    def grid_desc(self):
        """NEW: the AfcGridDesc of this area for the device-level calls."""
        d = nativemethods.GridDesc()
        rc = _dll().AFC_GridDescFromArea(self.handle, self.get_dimension(), byref(d))
        if rc != 0:
            _check()
        return d

    @staticmethod
    def get_dimension():
        raise NotImplementedError()


class GridArea1D(GridArea):
    @staticmethod
    def get_type():
        return 0

    @staticmethod
    def get_dimension():
        return 1


class GridArea2D(GridArea):
    @staticmethod
    def get_type():
        return 1

    @staticmethod
    def get_dimension():
        return 2


class GridArea3D(GridArea):
    @staticmethod
    def get_type():
        return 2

    @staticmethod
    def get_dimension():
        return 3


class GridAreaBuilder:
    """Same state machine as python/afc/afc.py:326-441 of the reference."""

    def __init__(self):
        self.__dim_cnt = 0
        self.__ranges = []
        self.__resolution = None
        self.__axes = []

    def __add_axes(self, axis):
        if axis in self.__axes:
            raise RuntimeError(f"The axis ({axis}) is already specified.")
        self.__axes.append(axis)

    def x_at(self, pos: float):
        self.__ranges.append((pos, pos))
        self.__add_axes(Axis.X)
        return self

    def y_at(self, pos: float):
        self.__ranges.append((pos, pos))
        self.__add_axes(Axis.Y)
        return self

    def z_at(self, pos: float):
        self.__ranges.append((pos, pos))
        self.__add_axes(Axis.Z)
        return self

    def x_range(self, obs_range):
        self.__ranges.append(obs_range)
        self.__add_axes(Axis.X)
        self.__dim_cnt += 1
        return self

    def y_range(self, obs_range):
        self.__ranges.append(obs_range)
        self.__add_axes(Axis.Y)
        self.__dim_cnt += 1
        return self

    def z_range(self, obs_range):
        self.__ranges.append(obs_range)
        self.__add_axes(Axis.Z)
        self.__dim_cnt += 1
        return self

    def resolution(self, r: float):
        if self.__resolution is None:
            self.__resolution = r
        else:
            raise RuntimeError("Resolution is already specified.")
        return self

    def generate(self):
        if len(self.__ranges) != 3:
            raise RuntimeError("Some ranges is not specified.")
        if self.__resolution is None:
            raise RuntimeError("Resolution is not specified.")
        fr, sr, tr = self.__ranges
        ax = [int(a) for a in self.__axes]
        if self.__dim_cnt in (0, 1):
            area = GridArea1D()
            _dll().AFC_CreateGridArea1D(byref(area.handle), fr[0], fr[1], sr[0], tr[0],
                                        self.__resolution, *ax)
        elif self.__dim_cnt == 2:
            area = GridArea2D()
            _dll().AFC_CreateGridArea2D(byref(area.handle), fr[0], fr[1], sr[0], sr[1], tr[0],
                                        self.__resolution, *ax)
        else:
            area = GridArea3D()
            _dll().AFC_CreateGridArea3D(byref(area.handle), fr[0], fr[1], sr[0], sr[1], tr[0],
                                        tr[1], self.__resolution, *ax)
        if not area.handle:
            _check()
        return area


def grid_from_spec(spec):
    """NEW: a grid area from afc.configs.GridSpec (specification-order ranges and axes)."""
    b = GridAreaBuilder()
    for k, ((lo, hi), ax) in enumerate(zip(spec.ranges, spec.axes)):
        name = {1: "x", 2: "y", 3: "z"}[int(ax)]
        if k < spec.dim:
            getattr(b, f"{name}_range")((lo, hi))
        else:
            getattr(b, f"{name}_at")(lo)
    return b.resolution(spec.res).generate()


def _foci_args(foci, amps):
    size = len(foci)
    amps = np.ascontiguousarray(np.asarray(amps, dtype=np.float32))
    foci_array = np.ascontiguousarray(np.asarray(foci, dtype=np.float32).reshape(size * 3))
    return (foci_array, amps, size,
            foci_array.ctypes.data_as(c_void_p), amps.ctypes.data_as(POINTER(c_float)))


class Optimizer:
    """Same entry points as python/afc/afc.py:443-560 of the reference."""

    @staticmethod
    def focus(system: UniformSystem, p):
        if not isinstance(p, Vector3):
            p = Vector3(p)
        _dll().AFO_FocalPoint(system.handle, p, system._source_type)

    @staticmethod
    def bessel(system: UniformSystem, p, direction, theta_z: float):
        if not isinstance(p, Vector3):
            p = Vector3(p)
        if not isinstance(direction, Vector3):
            direction = Vector3(direction)
        _dll().AFO_BesselBeam(system.handle, p, direction, c_float(theta_z), system._source_type)

    @staticmethod
    def ifft(system: UniformSystem, path, bottom_left, top_left, bottom_right, spacing, z):
        _dll().AFC_ClearLastError()
        _dll().AFO_IFFT(system.handle, path.encode("utf-8"), bottom_left, top_left, bottom_right,
                        spacing, z, system._source_type)
        _check()

    @staticmethod
    def _multi(fn_name, system, foci, amps, *extra):
        _dll().AFC_ClearLastError()
        keep = _foci_args(foci, amps)
        getattr(_dll(), fn_name)(system.handle, keep[3], keep[4], c_ulong(keep[2]), *extra,
                                 system._source_type)
        _check()

    @staticmethod
    def gs_pat(system: UniformSystem, foci, amps):
        Optimizer._multi("AFO_GSPAT", system, foci, amps)

    @staticmethod
    def gs(system: UniformSystem, foci, amps):
        Optimizer._multi("AFO_GS", system, foci, amps)

    @staticmethod
    def naive(system: UniformSystem, foci, amps):
        Optimizer._multi("AFO_Naive", system, foci, amps)

    @staticmethod
    def horn(system: UniformSystem, foci, amps):
        Optimizer._multi("AFO_Horn", system, foci, amps)

    @staticmethod
    def long2014(system: UniformSystem, foci, amps):
        Optimizer._multi("AFO_Long", system, foci, amps)

    @staticmethod
    def apo(system: UniformSystem, foci, amps, lambda_reg: float):
        Optimizer._multi("AFO_APO", system, foci, amps, c_float(lambda_reg))

    @staticmethod
    def lm(system: UniformSystem, foci, amps):
        Optimizer._multi("AFO_LM", system, foci, amps)

    @staticmethod
    def gauss_newton(system: UniformSystem, foci, amps):
        Optimizer._multi("AFO_GaussNewton", system, foci, amps)

    @staticmethod
    def gradient_descent(system: UniformSystem, foci, amps):
        Optimizer._multi("AFO_GradientDescent", system, foci, amps)

    @staticmethod
    def greedy(system: UniformSystem, foci, amps, phase_div: int = 16):
        Optimizer._multi("AFO_Greedy", system, foci, amps, c_ulong(phase_div))
