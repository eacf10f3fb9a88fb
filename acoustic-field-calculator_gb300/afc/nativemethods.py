"""ctypes declarations of libafccapi.so.

The structures and argtypes of the reference's exports follow the reference's own Python
binding (python/afc/nativemethods.py:18-234) one for one, so code written against that binding
drives this library unchanged.  Exports marked NEW are this library's additions (include/*.h).
"""
import ctypes
from ctypes import (POINTER, Structure, c_char_p, c_double, c_float, c_int, c_int32, c_int64,
                    c_size_t, c_uint, c_uint64, c_ulong, c_void_p)


class Vector3(Structure):
    _fields_ = [("x", c_float), ("y", c_float), ("z", c_float)]

    def __init__(self, position):
        super().__init__()
        self.x = position[0]
        self.y = position[1]
        self.z = position[2]


class SphereWaveSource(Structure):
    _fields_ = [("x", c_float), ("y", c_float), ("z", c_float), ("amp", c_float),
                ("phase", c_float), ("freq", c_float)]

    def __init__(self, position, amp, phase, freq):
        super().__init__()
        self.pos = position
        self.amp = amp
        self.phase = phase
        self.freq = freq

    @property
    def pos(self):
        return (self.x, self.y, self.z)

    @pos.setter
    def pos(self, position):
        self.x = position[0]
        self.y = position[1]
        self.z = position[2]

    @staticmethod
    def get_type():
        return 0


class T4010A1(Structure):
    _fields_ = [("x", c_float), ("y", c_float), ("z", c_float), ("nx", c_float),
                ("ny", c_float), ("nz", c_float), ("amp", c_float), ("phase", c_float),
                ("freq", c_float)]

    def __init__(self, position, direction, amp, phase, freq):
        super().__init__()
        self.pos = position
        self.direction = direction
        self.amp = amp
        self.phase = phase
        self.freq = freq

    @property
    def pos(self):
        return (self.x, self.y, self.z)

    @pos.setter
    def pos(self, position):
        self.x = position[0]
        self.y = position[1]
        self.z = position[2]

    @property
    def direction(self):
        return (self.nx, self.ny, self.nz)

    @direction.setter
    def direction(self, direction):
        self.nx = direction[0]
        self.ny = direction[1]
        self.nz = direction[2]

    @staticmethod
    def get_type():
        return 1


class GridDesc(Structure):
    """NEW: AfcGridDesc of include/afc_gpu.h."""
    _fields_ = [("count", c_uint64 * 3), ("axis", c_int32 * 3), ("origin", c_float * 3),
                ("res", c_float)]


class FieldJob(Structure):
    """NEW: AfcFieldJob of include/afc_gpu.h."""
    _fields_ = [("n_sources", c_uint64), ("d_sources", c_void_p), ("d_wavenums", c_void_p),
                ("d_attens", c_void_p), ("field_type", c_int32), ("is_grid", c_int32),
                ("grid", GridDesc), ("d_points", c_void_p), ("n_points", c_uint64),
                ("d_out", c_void_p)]


class ServeConfig(Structure):
    """NEW: AfcServeConfig of include/afc_gpu.h."""
    _fields_ = [("hbm_budget_bytes", c_uint64), ("pinned_bytes", c_uint64),
                ("max_inflight", c_int32)]


class ServeStats(Structure):
    """NEW: AfcServeStats of include/afc_gpu.h."""
    _fields_ = [("completed", c_uint64), ("failed", c_uint64), ("queued", c_uint64),
                ("peak_hbm_bytes", c_uint64), ("hbm_budget_bytes", c_uint64),
                ("peak_inflight", c_int32)]


AFC_DLL = None

# Every export of include/afccapi.h and include/afc_gpu.h (checked by the symbol test).
REFERENCE_EXPORTS = [
    "AFC_CreateCalculator", "AFC_FreeCalculator", "AFC_Calculate",
    "AFC_CreatePressureField", "AFC_FreePressureField", "AFC_CreatePowerField",
    "AFC_FreePowerField", "AFC_CreateComplexPressureField", "AFC_FreeComplexPressureField",
    "AFC_CreateScatterArea", "AFC_ScatterAddObservePoint", "AFC_FreeScatterArea",
    "AFC_CreateGridArea1D", "AFC_CreateGridArea2D", "AFC_CreateGridArea3D", "AFC_FreeGridArea",
    "AFC_GetGridSize",
    "AFO_FocalPoint", "AFO_BesselBeam", "AFO_IFFT", "AFO_GSPAT", "AFO_GS", "AFO_Naive",
    "AFO_Horn", "AFO_Long", "AFO_APO", "AFO_GaussNewton", "AFO_LM", "AFO_GradientDescent",
    "AFO_Greedy",
    "AFC_CreateUniformSystem", "AFC_FreeUniformSystem", "AFC_AddSphereWaveSource",
    "AFC_AddT4010A1", "AFC_GetWaveSources", "AFC_UniformSystemSoundSpeed",
    "AFC_UniformSystemInfo", "AFC_UniformSystemSourceInfo",
]
NEW_EXPORTS = [
    "AFC_AddSphereWaveSourceWithWavenumAtten", "AFC_AddT4010A1WithWavenumAtten",
    "AFC_UniformSystemTrackSources", "AFC_UniformSystemSourcesChanged",
    "AFC_GetLastError", "AFC_ClearLastError",
    "AFC_GridDescFromArea", "AFC_FieldWorkspaceBytes", "AFC_FieldGridDevice",
    "AFC_FieldScatterDevice", "AFC_KernelLaunchCount", "AFC_CudaDeviceCount",
    "AFC_MeasurePipeRates", "AFC_SetDevice", "AFC_FieldGridDeviceNoAlloc",
    "AFC_MultiPatternWorkspaceBytes", "AFC_MultiPatternBuildG", "AFC_MultiPatternApply",
    "AFC_MultiPatternStatus", "AFC_MultiPatternApplyWaitTest", "AFC_MultiPatternDirect",
    "AFC_BatchCreate", "AFC_BatchRun",
    "AFC_BatchRunOneByOne", "AFC_BatchDescribe", "AFC_BatchDescribeKernels", "AFC_BatchFree",
    "AFC_ServeCreate",
    "AFC_ServeAddGeometry", "AFC_ServeSubmitField", "AFC_ServeSubmitGspat", "AFC_ServeWait",
    "AFC_ServeStats", "AFC_ServeDestroy",
]


def init_dll(dll_location):
    global AFC_DLL  # pylint: disable=global-statement
    AFC_DLL = ctypes.CDLL(dll_location)
    __init_calculator()
    __init_field_buffer()
    __init_observe_area()
    __init_optimizer()
    __init_system()
    __init_new()
    return AFC_DLL


def __init_calculator():
    AFC_DLL.AFC_CreateCalculator.argtypes = [POINTER(c_void_p), c_int]
    AFC_DLL.AFC_CreateCalculator.restype = None
    AFC_DLL.AFC_FreeCalculator.argtypes = [c_void_p, c_int]
    AFC_DLL.AFC_FreeCalculator.restype = None
    AFC_DLL.AFC_Calculate.argtypes = [c_void_p, c_void_p, c_void_p, c_void_p, POINTER(c_void_p),
                                      c_int, c_int, c_int, c_int]
    AFC_DLL.AFC_Calculate.restype = c_ulong


def __init_field_buffer():
    for name in ("Pressure", "Power", "ComplexPressure"):
        create = getattr(AFC_DLL, f"AFC_Create{name}Field")
        create.argtypes = [POINTER(c_void_p)]
        create.restype = None
        free = getattr(AFC_DLL, f"AFC_Free{name}Field")
        free.argtypes = [c_void_p]
        free.restype = None


def __init_observe_area():
    AFC_DLL.AFC_CreateScatterArea.argtypes = [POINTER(c_void_p)]
    AFC_DLL.AFC_CreateScatterArea.restype = None
    AFC_DLL.AFC_ScatterAddObservePoint.argtypes = [c_void_p, Vector3]
    AFC_DLL.AFC_ScatterAddObservePoint.restype = None
    AFC_DLL.AFC_FreeScatterArea.argtypes = [c_void_p]
    AFC_DLL.AFC_FreeScatterArea.restype = None
    AFC_DLL.AFC_CreateGridArea1D.argtypes = [POINTER(c_void_p), c_float, c_float, c_float,
                                             c_float, c_float, c_int, c_int, c_int]
    AFC_DLL.AFC_CreateGridArea1D.restype = None
    AFC_DLL.AFC_CreateGridArea2D.argtypes = [POINTER(c_void_p), c_float, c_float, c_float,
                                             c_float, c_float, c_float, c_int, c_int, c_int]
    AFC_DLL.AFC_CreateGridArea2D.restype = None
    AFC_DLL.AFC_CreateGridArea3D.argtypes = [POINTER(c_void_p), c_float, c_float, c_float,
                                             c_float, c_float, c_float, c_float, c_int, c_int,
                                             c_int]
    AFC_DLL.AFC_CreateGridArea3D.restype = None
    AFC_DLL.AFC_FreeGridArea.argtypes = [c_void_p, c_int]
    AFC_DLL.AFC_FreeGridArea.restype = None
    AFC_DLL.AFC_GetGridSize.argtypes = [c_void_p, c_int, POINTER(c_uint), POINTER(c_uint),
                                        POINTER(c_uint)]
    AFC_DLL.AFC_GetGridSize.restype = None


def __init_optimizer():
    AFC_DLL.AFO_FocalPoint.argtypes = [c_void_p, Vector3, c_int]
    AFC_DLL.AFO_FocalPoint.restype = None
    AFC_DLL.AFO_BesselBeam.argtypes = [c_void_p, Vector3, Vector3, c_float, c_int]
    AFC_DLL.AFO_BesselBeam.restype = None
    AFC_DLL.AFO_IFFT.argtypes = [c_void_p, c_char_p, Vector3, Vector3, Vector3, c_float, c_float,
                                 c_int]
    AFC_DLL.AFO_IFFT.restype = None
    for name in ("GSPAT", "GS", "Naive", "Horn", "Long", "GaussNewton", "LM",
                 "GradientDescent"):
        fn = getattr(AFC_DLL, f"AFO_{name}")
        fn.argtypes = [c_void_p, c_void_p, POINTER(c_float), c_ulong, c_int]
        fn.restype = None
    AFC_DLL.AFO_APO.argtypes = [c_void_p, c_void_p, POINTER(c_float), c_ulong, c_float, c_int]
    AFC_DLL.AFO_APO.restype = None
    AFC_DLL.AFO_Greedy.argtypes = [c_void_p, c_void_p, POINTER(c_float), c_ulong, c_ulong, c_int]
    AFC_DLL.AFO_Greedy.restype = None


def __init_system():
    AFC_DLL.AFC_CreateUniformSystem.argtypes = [c_void_p, c_float, c_int]
    AFC_DLL.AFC_CreateUniformSystem.restype = None
    AFC_DLL.AFC_FreeUniformSystem.argtypes = [c_void_p, c_int]
    AFC_DLL.AFC_FreeUniformSystem.restype = None
    AFC_DLL.AFC_AddSphereWaveSource.argtypes = [c_void_p, SphereWaveSource]
    AFC_DLL.AFC_AddSphereWaveSource.restype = None
    AFC_DLL.AFC_AddT4010A1.argtypes = [c_void_p, T4010A1]
    AFC_DLL.AFC_AddT4010A1.restype = None
    AFC_DLL.AFC_GetWaveSources.argtypes = [c_void_p, POINTER(c_void_p), c_int]
    AFC_DLL.AFC_GetWaveSources.restype = c_ulong
    AFC_DLL.AFC_UniformSystemSoundSpeed.argtypes = [c_void_p, c_int]
    AFC_DLL.AFC_UniformSystemSoundSpeed.restype = c_float
    AFC_DLL.AFC_UniformSystemInfo.argtypes = [c_void_p, c_int]
    AFC_DLL.AFC_UniformSystemInfo.restype = c_char_p
    AFC_DLL.AFC_UniformSystemSourceInfo.argtypes = [c_void_p, c_ulong, c_int]
    AFC_DLL.AFC_UniformSystemSourceInfo.restype = c_char_p


def __init_new():
    AFC_DLL.AFC_AddSphereWaveSourceWithWavenumAtten.argtypes = [c_void_p, SphereWaveSource,
                                                                c_float, c_float]
    AFC_DLL.AFC_AddSphereWaveSourceWithWavenumAtten.restype = None
    AFC_DLL.AFC_AddT4010A1WithWavenumAtten.argtypes = [c_void_p, T4010A1, c_float, c_float]
    AFC_DLL.AFC_AddT4010A1WithWavenumAtten.restype = None
    AFC_DLL.AFC_UniformSystemTrackSources.argtypes = [c_void_p, c_int32, c_int32]
    AFC_DLL.AFC_UniformSystemTrackSources.restype = c_int32
    AFC_DLL.AFC_UniformSystemSourcesChanged.argtypes = [c_void_p, c_int32]
    AFC_DLL.AFC_UniformSystemSourcesChanged.restype = c_int32
    AFC_DLL.AFC_GetLastError.argtypes = []
    AFC_DLL.AFC_GetLastError.restype = c_char_p
    AFC_DLL.AFC_ClearLastError.argtypes = []
    AFC_DLL.AFC_ClearLastError.restype = None
    AFC_DLL.AFC_GridDescFromArea.argtypes = [c_void_p, c_int32, POINTER(GridDesc)]
    AFC_DLL.AFC_GridDescFromArea.restype = c_int32
    AFC_DLL.AFC_FieldWorkspaceBytes.argtypes = [c_uint64]
    AFC_DLL.AFC_FieldWorkspaceBytes.restype = c_size_t
    AFC_DLL.AFC_FieldGridDevice.argtypes = [c_int32, c_int32, c_int32, c_void_p, c_void_p,
                                            c_void_p, c_uint64, POINTER(GridDesc), c_void_p,
                                            c_void_p, c_size_t, c_void_p]
    AFC_DLL.AFC_FieldGridDevice.restype = c_int32
    AFC_DLL.AFC_FieldScatterDevice.argtypes = [c_int32, c_int32, c_int32, c_void_p, c_void_p,
                                               c_void_p, c_uint64, c_void_p, c_uint64, c_void_p,
                                               c_void_p, c_size_t, c_void_p]
    AFC_DLL.AFC_FieldScatterDevice.restype = c_int32
    AFC_DLL.AFC_KernelLaunchCount.argtypes = []
    AFC_DLL.AFC_KernelLaunchCount.restype = c_uint64
    AFC_DLL.AFC_CudaDeviceCount.argtypes = []
    AFC_DLL.AFC_CudaDeviceCount.restype = c_int32
    AFC_DLL.AFC_MeasurePipeRates.argtypes = [POINTER(c_double), POINTER(c_double),
                                             POINTER(c_int32)]
    AFC_DLL.AFC_MeasurePipeRates.restype = c_int32
    AFC_DLL.AFC_SetDevice.argtypes = [c_int32]
    AFC_DLL.AFC_SetDevice.restype = c_int32
    AFC_DLL.AFC_FieldGridDeviceNoAlloc.argtypes = [c_int32, c_int32, c_int32, c_void_p, c_void_p,
                                                   c_void_p, c_uint64, POINTER(GridDesc),
                                                   c_void_p, c_void_p]
    AFC_DLL.AFC_FieldGridDeviceNoAlloc.restype = c_int32
    AFC_DLL.AFC_MultiPatternWorkspaceBytes.argtypes = [c_uint64, c_uint64, c_uint64, c_int32]
    AFC_DLL.AFC_MultiPatternWorkspaceBytes.restype = c_size_t
    AFC_DLL.AFC_MultiPatternBuildG.argtypes = [c_int32, c_int32, c_void_p, c_void_p, c_void_p,
                                               c_uint64, c_void_p, c_uint64, c_uint64, c_void_p,
                                               c_size_t, c_void_p]
    AFC_DLL.AFC_MultiPatternBuildG.restype = c_int32
    AFC_DLL.AFC_MultiPatternApply.argtypes = [c_int32, c_void_p, c_void_p, c_uint64, c_uint64,
                                              c_uint64, c_void_p, c_void_p, c_size_t, c_void_p]
    AFC_DLL.AFC_MultiPatternApply.restype = c_int32
    AFC_DLL.AFC_MultiPatternStatus.argtypes = [c_int32, c_uint64, c_uint64, c_uint64, c_void_p,
                                               c_void_p]
    AFC_DLL.AFC_MultiPatternStatus.restype = c_int32
    AFC_DLL.AFC_MultiPatternApplyWaitTest.argtypes = AFC_DLL.AFC_MultiPatternApply.argtypes
    AFC_DLL.AFC_MultiPatternApplyWaitTest.restype = c_int32
    AFC_DLL.AFC_MultiPatternDirect.argtypes = [c_int32, c_void_p, c_void_p, c_void_p, c_uint64,
                                               c_void_p, c_uint64, c_void_p, c_void_p, c_uint64,
                                               c_void_p, c_void_p, c_size_t, c_void_p]
    AFC_DLL.AFC_MultiPatternDirect.restype = c_int32
    AFC_DLL.AFC_BatchCreate.argtypes = [c_int32, POINTER(FieldJob), c_uint64, c_int32,
                                        POINTER(c_void_p), c_void_p]
    AFC_DLL.AFC_BatchCreate.restype = c_int32
    AFC_DLL.AFC_BatchRun.argtypes = [c_void_p, c_void_p]
    AFC_DLL.AFC_BatchRun.restype = c_int32
    AFC_DLL.AFC_BatchRunOneByOne.argtypes = [c_void_p, c_void_p]
    AFC_DLL.AFC_BatchRunOneByOne.restype = c_int32
    AFC_DLL.AFC_BatchDescribe.argtypes = [c_void_p, POINTER(c_int32), POINTER(c_int32),
                                          POINTER(c_uint64), POINTER(c_double)]
    AFC_DLL.AFC_BatchDescribe.restype = c_int32
    AFC_DLL.AFC_BatchDescribeKernels.argtypes = [c_void_p, POINTER(c_int32), POINTER(c_int32),
                                                 POINTER(c_uint64), POINTER(c_int32),
                                                 POINTER(c_int32), POINTER(c_uint64)]
    AFC_DLL.AFC_BatchDescribeKernels.restype = c_int32
    AFC_DLL.AFC_BatchFree.argtypes = [c_void_p]
    AFC_DLL.AFC_BatchFree.restype = None
    AFC_DLL.AFC_ServeCreate.argtypes = [POINTER(ServeConfig), POINTER(c_void_p)]
    AFC_DLL.AFC_ServeCreate.restype = c_int32
    AFC_DLL.AFC_ServeAddGeometry.argtypes = [c_void_p, c_int32, c_void_p, c_void_p, c_void_p,
                                             c_uint64, POINTER(c_int32)]
    AFC_DLL.AFC_ServeAddGeometry.restype = c_int32
    AFC_DLL.AFC_ServeSubmitField.argtypes = [c_void_p, c_int32, c_void_p, c_void_p, c_int32,
                                             c_int32, POINTER(GridDesc), c_void_p, c_uint64,
                                             c_void_p]
    AFC_DLL.AFC_ServeSubmitField.restype = c_int64
    AFC_DLL.AFC_ServeSubmitGspat.argtypes = [c_void_p, c_int32, c_void_p, c_void_p, c_uint64,
                                             POINTER(GridDesc), c_void_p, c_void_p]
    AFC_DLL.AFC_ServeSubmitGspat.restype = c_int64
    AFC_DLL.AFC_ServeWait.argtypes = [c_void_p, c_int64, POINTER(c_double), POINTER(c_double)]
    AFC_DLL.AFC_ServeWait.restype = c_int32
    AFC_DLL.AFC_ServeStats.argtypes = [c_void_p, POINTER(ServeStats)]
    AFC_DLL.AFC_ServeStats.restype = c_int32
    AFC_DLL.AFC_ServeDestroy.argtypes = [c_void_p]
    AFC_DLL.AFC_ServeDestroy.restype = None
