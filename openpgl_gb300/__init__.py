"""Python front end of libopenpgl_gb300.so, the GB300 implementation of Open
PGL's field-training and guided-query path behind the Open PGL C API.

The classes mirror the reference's C++ wrapper (openpgl/include/openpgl/cpp/:
Device, FieldConfig, Field, SampleStorage, SurfaceSamplingDistribution,
VolumeSamplingDistribution) and call the exported C functions through ctypes.
There is no fallback: if the library cannot be loaded, or no GPU is present,
constructing a Device raises.
"""

from __future__ import annotations

import ctypes
import os

import numpy as np

from .synthetic import PGL_QUERY_DTYPE, PGL_SAMPLE_DTYPE, PGL_VERTEX_DTYPE

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libopenpgl_gb300.so")

PGL_DEVICE_TYPE_CPU_4, PGL_DEVICE_TYPE_CPU_8, PGL_DEVICE_TYPE_CPU_16, PGL_DEVICE_TYPE_NONE = 0, 1, 2, 3
PGL_DEVICE_TYPE_GPU_SM103 = 4
PGL_SPATIAL_STRUCTURE_KDTREE = 0
PGL_DIRECTIONAL_DISTRIBUTION_PARALLAX_AWARE_VMM = 0
PGL_DIRECTIONAL_DISTRIBUTION_QUADTREE = 1
PGL_DIRECTIONAL_DISTRIBUTION_VMM = 2

QUERY_RESULT_DTYPE = np.dtype(
    [("ok", "<u4"), ("id", "<u4"), ("sample1d", "<f4"), ("dir", "<f4", (3,)), ("pdf", "<f4"), ("pdfLi", "<f4")]
)
assert QUERY_RESULT_DTYPE.itemsize == 32
# PGLGuidedVertexResult: per SamplePDF call k, sample[k] = (direction xyz, pdf)
VERTEX_RESULT_DTYPE = np.dtype([("ok", "<u4"), ("id", "<u4"), ("sample1d", "<f4"), ("sample", "<f4", (4, 4))])
assert VERTEX_RESULT_DTYPE.itemsize == 76


class Vec3(ctypes.Structure):
    _fields_ = [("x", ctypes.c_float), ("y", ctypes.c_float), ("z", ctypes.c_float)]


class Vec2(ctypes.Structure):
    _fields_ = [("x", ctypes.c_float), ("y", ctypes.c_float)]


class Box3(ctypes.Structure):
    _fields_ = [("lower", Vec3), ("upper", Vec3)]


class SampleData(ctypes.Structure):
    _fields_ = [("position", Vec3), ("direction", Vec3), ("weight", ctypes.c_float), ("pdf", ctypes.c_float),
                ("distance", ctypes.c_float), ("flags", ctypes.c_uint32)]


class DQTFactoryArguments(ctypes.Structure):  # PGLDQTFactoryArguments (config.h)
    _fields_ = [("leafEstimator", ctypes.c_int), ("splitMetric", ctypes.c_int), ("splitThreshold", ctypes.c_float),
                ("footprintFactor", ctypes.c_float), ("maxLevels", ctypes.c_uint32)]


class FieldArguments(ctypes.Structure):  # PGLFieldArguments (config.h)
    _fields_ = [("spatialStructureType", ctypes.c_int), ("spatialStructureArguments", ctypes.c_void_p),
                ("directionalDistributionType", ctypes.c_int), ("directionalDistributionArguments", ctypes.c_void_p),
                ("deterministic", ctypes.c_bool), ("fitRegions", ctypes.c_bool)]


class PGLString(ctypes.Structure):
    _fields_ = [("m_str", ctypes.c_char_p), ("m_size", ctypes.c_size_t)]


# Exported symbols of include/openpgl/*.h and include/openpgl_gb300.h.
C_API = {
    "pglNewDevice": (ctypes.c_void_p, [ctypes.c_int, ctypes.c_size_t]),
    "pglReleaseDevice": (None, [ctypes.c_void_p]),
    "pglDeviceNewField": (ctypes.c_void_p, [ctypes.c_void_p, FieldArguments]),
    "pglDeviceNewFieldFromFile": (ctypes.c_void_p, [ctypes.c_void_p, ctypes.c_char_p]),
    "pglFieldArgumentsSetDefaults": (None, [ctypes.POINTER(FieldArguments), ctypes.c_int, ctypes.c_int, ctypes.c_bool,
                                            ctypes.c_size_t]),
    "pglReleaseField": (None, [ctypes.c_void_p]),
    "pglFieldStoreToFile": (ctypes.c_bool, [ctypes.c_void_p, ctypes.c_char_p]),
    "pglFieldGetIteration": (ctypes.c_size_t, [ctypes.c_void_p]),
    "pglFieldSetSceneBounds": (None, [ctypes.c_void_p, Box3]),
    "pglFieldGetSceneBounds": (Box3, [ctypes.c_void_p]),
    "pglFieldUpdate": (None, [ctypes.c_void_p, ctypes.c_void_p]),
    "pglFieldUpdateSurface": (None, [ctypes.c_void_p, ctypes.c_void_p]),
    "pglFieldUpdateVolume": (None, [ctypes.c_void_p, ctypes.c_void_p]),
    "pglFieldReset": (None, [ctypes.c_void_p]),
    "pglFieldNewSurfaceSamplingDistribution": (ctypes.c_void_p, [ctypes.c_void_p]),
    "pglFieldInitSurfaceSamplingDistribution": (ctypes.c_bool, [ctypes.c_void_p, ctypes.c_void_p, Vec3,
                                                                ctypes.POINTER(ctypes.c_float)]),
    "pglFieldNewVolumeSamplingDistribution": (ctypes.c_void_p, [ctypes.c_void_p]),
    "pglFieldInitVolumeSamplingDistribution": (ctypes.c_bool, [ctypes.c_void_p, ctypes.c_void_p, Vec3,
                                                               ctypes.POINTER(ctypes.c_float)]),
    "pglFieldValidate": (ctypes.c_bool, [ctypes.c_void_p]),
    "pglFieldCompare": (ctypes.c_bool, [ctypes.c_void_p, ctypes.c_void_p]),
    "pglFieldGetSurfaceStatistics": (ctypes.c_void_p, [ctypes.c_void_p]),
    "pglFieldGetVolumeStatistics": (ctypes.c_void_p, [ctypes.c_void_p]),
    "pglReleaseFieldStatistics": (None, [ctypes.c_void_p]),
    "pglFieldStatisticsToString": (PGLString, [ctypes.c_void_p]),
    "pglFieldStatisticsHeaderCSVString": (PGLString, [ctypes.c_void_p]),
    "pglFieldStatisticsToCSVString": (PGLString, [ctypes.c_void_p]),
    "pglReleaseString": (None, [PGLString]),
    "pglNewSampleStorage": (ctypes.c_void_p, []),
    "pglNewSampleStorageFromFile": (ctypes.c_void_p, [ctypes.c_char_p]),
    "pglReleaseSampleStorage": (None, [ctypes.c_void_p]),
    "pglSampleStorageStoreToFile": (ctypes.c_bool, [ctypes.c_void_p, ctypes.c_char_p]),
    "pglSampleStorageAddSample": (None, [ctypes.c_void_p, ctypes.POINTER(SampleData)]),
    "pglSampleStorageAddSamples": (None, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t]),
    "pglSampleStorageReserve": (None, [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_size_t]),
    "pglSampleStorageClear": (None, [ctypes.c_void_p]),
    "pglSampleStorageClearSurface": (None, [ctypes.c_void_p]),
    "pglSampleStorageClearVolume": (None, [ctypes.c_void_p]),
    "pglSampleStorageGetSizeSurface": (ctypes.c_size_t, [ctypes.c_void_p]),
    "pglSampleStorageGetSizeVolume": (ctypes.c_size_t, [ctypes.c_void_p]),
    "pglSampleStorageGetSampleSurface": (SampleData, [ctypes.c_void_p, ctypes.c_int]),
    "pglSampleStorageGetSampleVolume": (SampleData, [ctypes.c_void_p, ctypes.c_int]),
    "pglSampleStorageValidate": (ctypes.c_bool, [ctypes.c_void_p]),
    "pglSampleStorageCompare": (ctypes.c_bool, [ctypes.c_void_p, ctypes.c_void_p]),
    "pglReleaseSurfaceSamplingDistribution": (None, [ctypes.c_void_p]),
    "pglSurfaceSamplingDistributionApplyCosineProduct": (None, [ctypes.c_void_p, Vec3]),
    "pglSurfaceSamplingDistributionSupportsApplyCosineProduct": (ctypes.c_bool, [ctypes.c_void_p]),
    "pglSurfaceSamplingDistributionSample": (Vec3, [ctypes.c_void_p, Vec2]),
    "pglSurfaceSamplingDistributionPDF": (ctypes.c_float, [ctypes.c_void_p, Vec3]),
    "pglSurfaceSamplingDistributionSamplePDF": (ctypes.c_float, [ctypes.c_void_p, Vec2, ctypes.POINTER(Vec3)]),
    "pglSurfaceSamplingDistributionIncomingRadiancePDF": (ctypes.c_float, [ctypes.c_void_p, Vec3]),
    "pglSurfaceSamplingDistributionGetId": (ctypes.c_uint32, [ctypes.c_void_p]),
    "pglSurfaceSamplingDistributionValidate": (ctypes.c_bool, [ctypes.c_void_p]),
    "pglSurfaceSamplingDistributionClear": (None, [ctypes.c_void_p]),
    "pglSurfaceSamplingGetRegion": (ctypes.c_void_p, [ctypes.c_void_p]),
    "pglReleaseVolumeSamplingDistribution": (None, [ctypes.c_void_p]),
    "pglVolumeSamplingDistributionSample": (Vec3, [ctypes.c_void_p, Vec2]),
    "pglVolumeSamplingDistributionPDF": (ctypes.c_float, [ctypes.c_void_p, Vec3]),
    "pglVolumeSamplingDistributionSamplePDF": (ctypes.c_float, [ctypes.c_void_p, Vec2, ctypes.POINTER(Vec3)]),
    "pglVolumeSamplingDistributionIncomingRadiancePDF": (ctypes.c_float, [ctypes.c_void_p, Vec3]),
    "pglVolumeSamplingDistributionGetId": (ctypes.c_uint32, [ctypes.c_void_p]),
    "pglVolumeSamplingDistributionValidate": (ctypes.c_bool, [ctypes.c_void_p]),
    "pglVolumeSamplingDistributionClear": (None, [ctypes.c_void_p]),
    "pglVolumeSamplingDistributionApplySingleLobeHenyeyGreensteinProduct": (None, [ctypes.c_void_p, Vec3,
                                                                                   ctypes.c_float]),
    "pglVolumeSamplingDistributionSupportsApplySingleLobeHenyeyGreensteinProduct": (ctypes.c_bool,
                                                                                    [ctypes.c_void_p]),
    "pglVolumeSamplingGetRegion": (ctypes.c_void_p, [ctypes.c_void_p]),
    "pglFieldSampleSurfaceBatch": (ctypes.c_bool, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
                                                   ctypes.c_void_p, ctypes.c_bool]),
    "pglFieldSampleVolumeBatch": (ctypes.c_bool, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
                                                  ctypes.c_void_p]),
    "pglFieldSampleBatchDevice": (ctypes.c_bool, [ctypes.c_void_p, ctypes.c_bool, ctypes.c_void_p, ctypes.c_size_t,
                                                  ctypes.c_void_p, ctypes.c_bool, ctypes.c_void_p]),
    "pglFieldSampleVolumeBatchHG": (ctypes.c_bool, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
                                                    ctypes.c_void_p]),
    "pglFieldSampleVolumeBatchHGDevice": (ctypes.c_bool, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                                          ctypes.c_size_t, ctypes.c_void_p, ctypes.c_void_p]),
    "pglSampleStorageAddSamplesDevice": (None, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t]),
    "pglFieldSampleSurfaceVertices": (ctypes.c_bool, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
                                                      ctypes.c_void_p]),
    "pglFieldSampleSurfaceVerticesDevice": (ctypes.c_bool, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
                                                            ctypes.c_void_p, ctypes.c_void_p]),
    "pglFieldStoreToBuffer": (ctypes.c_size_t, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_size_t]),
    "pglFieldGetLastUpdateTimings": (ctypes.c_bool, [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_float)]),
    "pglFieldGetLastUpdateReports": (ctypes.c_size_t, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                                       ctypes.c_size_t]),
    "pglGetLastError": (ctypes.c_char_p, []),
    "pglFieldGetLastUpdatePhases": (ctypes.c_size_t, [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                                                      ctypes.c_size_t]),
    "pglDeviceGetCudaStream": (ctypes.c_void_p, [ctypes.c_void_p]),
    "pglGetKernelLaunchCount": (ctypes.c_uint64, []),
    "pglDebugBoundedWaitRunsOut": (ctypes.c_int, [ctypes.c_uint64]),
    "pglNewGuidingServer": (ctypes.c_void_p, [ctypes.c_void_p, ctypes.c_size_t]),
    "pglNewGuidingServerEx": (ctypes.c_void_p, [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int]),
    "pglReleaseGuidingServer": (None, [ctypes.c_void_p]),
    "pglGuidingServerSubmit": (ctypes.c_uint64, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p,
                                                 ctypes.c_bool, ctypes.c_bool]),
    "pglGuidingServerWait": (ctypes.c_bool, [ctypes.c_void_p, ctypes.c_uint64, ctypes.POINTER(ctypes.c_double),
                                             ctypes.POINTER(ctypes.c_uint64)]),
    "pglGuidingServerAddSamples": (ctypes.c_bool, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t]),
    "pglGuidingServerUpdate": (ctypes.c_uint64, [ctypes.c_void_p]),
    "pglGuidingServerWaitUpdate": (ctypes.c_bool, [ctypes.c_void_p, ctypes.c_uint64]),
    "pglGuidingServerStats": (ctypes.c_bool, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)]),
    "pglGuidingServerStatsEx": (ctypes.c_size_t, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.c_size_t]),
    "pglGuidingServerResetStats": (ctypes.c_bool, [ctypes.c_void_p]),
    "pglGuidingServerAddSamplesDevice": (ctypes.c_bool, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t]),
    "pglGuidingServerSubmitVertices": (ctypes.c_uint64, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
                                                         ctypes.c_void_p]),
    "pglSplitSamplesDeviceNoAlloc": (ctypes.c_bool, [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_void_p,
                                                     ctypes.c_void_p, ctypes.c_void_p]),
    "pglFieldGetLastUpdateProfile": (ctypes.c_size_t, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_size_t]),
    "pglFieldSetEmTuning": (ctypes.c_bool, [ctypes.c_void_p, ctypes.c_void_p]),
    "pglFieldGetEmTuning": (ctypes.c_bool, [ctypes.c_void_p, ctypes.c_void_p]),
    "pglFieldAutotuneNextUpdate": (None, [ctypes.c_void_p]),
    "pglFieldSetPlainUpdate": (ctypes.c_bool, [ctypes.c_void_p, ctypes.c_bool]),
    "pglFieldGetEmTuningTrials": (ctypes.c_size_t, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t]),
    "pglNewPathSegmentStorage": (ctypes.c_void_p, []),
    "pglReleasePathSegmentStorage": (None, [ctypes.c_void_p]),
    "pglPathSegmentStorageReserve": (None, [ctypes.c_void_p, ctypes.c_size_t]),
    "pglPathSegmentStorageClear": (None, [ctypes.c_void_p]),
    "pglPathSegmentSetMaxDistance": (None, [ctypes.c_void_p, ctypes.c_float]),
    "pglPathSegmentGetMaxDistance": (ctypes.c_float, [ctypes.c_void_p]),
    "pglPathSegmentGetNumSegments": (ctypes.c_int, [ctypes.c_void_p]),
    "pglPathSegmentGetNumSamples": (ctypes.c_int, [ctypes.c_void_p]),
    "pglPathSegmentStoragePrepareSamples": (ctypes.c_size_t, [ctypes.c_void_p, ctypes.c_bool, ctypes.c_bool,
                                                              ctypes.c_bool]),
    "pglPathSegmentStorageCalculatePixelEstimate": (Vec3, [ctypes.c_void_p, ctypes.c_bool]),
    "pglPathSegmentStorageGetSamples": (ctypes.c_void_p, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_size_t)]),
    "pglPathSegmentStorageNextSegment": (ctypes.c_void_p, [ctypes.c_void_p]),
    "pglPathSegmentStorageValidateSamples": (ctypes.c_bool, [ctypes.c_void_p]),
    "pglPathSegmentStorageValidateSegments": (ctypes.c_bool, [ctypes.c_void_p]),
    "pglPathSegmentStoragePropagateSamples": (None, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_bool, ctypes.c_bool,
                                                     ctypes.c_bool]),
    "pglPathSegmentsPrepareSamplesDevice": (ctypes.c_bool, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
                                                            ctypes.c_float, ctypes.c_bool, ctypes.c_bool, ctypes.c_bool,
                                                            ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "pglPathSegmentsPropagateSamplesDevice": (ctypes.c_size_t, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
                                                                ctypes.c_float, ctypes.c_void_p, ctypes.c_bool,
                                                                ctypes.c_bool, ctypes.c_bool]),
}

_lib = None


def load(build_if_missing=True):
    """Loads the in-tree library (building it first if it is missing)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            if not build_if_missing:
                raise OSError(f"{LIB_PATH} is missing; run openpgl_gb300/build.py")
            from . import build as _b

            _b.build()
        lib = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in C_API.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def kernel_launch_count():
    """Kernels of this library launched so far by the process."""
    return int(load().pglGetKernelLaunchCount())


def bounded_wait_runs_out(limit_ns):
    """One device thread waits, with the EM kernel's bounded wait, on a flag
    that nothing sets; returns the error code the wait recorded (2: it ran out
    after limit_ns).  Raises on a CUDA error."""
    code = int(load().pglDebugBoundedWaitRunsOut(int(limit_ns)))
    if code < 0:
        raise RuntimeError(last_error())
    return code


def split_samples_device_noalloc(d_samples, n, d_surface, d_volume, d_counts, stream=None):
    """pglSplitSamplesDeviceNoAlloc: stable split of n device records into
    surface and volume records without allocating (pointers are integers)."""
    ok = load().pglSplitSamplesDeviceNoAlloc(d_samples, n, d_surface, d_volume, d_counts, stream)
    _check(ok, "pglSplitSamplesDeviceNoAlloc")


def last_error():
    return load().pglGetLastError().decode()


def _check(ok, what):
    if not ok:
        raise RuntimeError(f"{what} failed: {last_error()}")


class Device:
    def __init__(self, device_type=PGL_DEVICE_TYPE_CPU_8, num_threads=0):
        self.lib = load()
        self.h = self.lib.pglNewDevice(device_type, num_threads)
        _check(self.h, "pglNewDevice")

    def cuda_stream(self):
        """The cudaStream_t (as an int) the library launches on."""
        return self.lib.pglDeviceGetCudaStream(self.h) or 0

    def release(self):
        if self.h:
            self.lib.pglReleaseDevice(self.h)
            self.h = None


class FieldConfig:
    """FieldConfig::Init (cpp/FieldConfig.h:62-64)."""

    def __init__(self, deterministic=True, max_samples_per_leaf=32000, parallax=True, dqt=False, dqt_args=None):
        """dqt: the directional quadtree field type; dqt_args = (leafEstimator,
        splitMetric, splitThreshold, footprintFactor, maxLevels) overrides the
        factory's defaults."""
        self.args = FieldArguments()
        kind = PGL_DIRECTIONAL_DISTRIBUTION_PARALLAX_AWARE_VMM if parallax else PGL_DIRECTIONAL_DISTRIBUTION_VMM
        if dqt:
            kind = PGL_DIRECTIONAL_DISTRIBUTION_QUADTREE
        load().pglFieldArgumentsSetDefaults(ctypes.byref(self.args), PGL_SPATIAL_STRUCTURE_KDTREE, kind,
                                            deterministic, max_samples_per_leaf)
        if dqt and dqt_args:
            a = ctypes.cast(self.args.directionalDistributionArguments, ctypes.POINTER(DQTFactoryArguments)).contents
            a.leafEstimator, a.splitMetric, a.splitThreshold, a.footprintFactor, a.maxLevels = dqt_args


class SampleStorage:
    def __init__(self):
        self.lib = load()
        self.h = self.lib.pglNewSampleStorage()
        _check(self.h, "pglNewSampleStorage")

    @classmethod
    def from_file(cls, path):
        """pglNewSampleStorageFromFile: a storage from a file in the reference's layout."""
        s = cls.__new__(cls)
        s.lib = load()
        s.h = s.lib.pglNewSampleStorageFromFile(os.fsencode(path))
        _check(s.h, "pglNewSampleStorageFromFile")
        return s

    def add_samples(self, samples):
        s = np.ascontiguousarray(samples, dtype=PGL_SAMPLE_DTYPE)
        self.lib.pglSampleStorageAddSamples(self.h, s.ctypes.data, len(s))

    def add_samples_device(self, ptr, n):
        """Adds n PGLSampleData records that live in device memory at ptr."""
        self.lib.pglSampleStorageAddSamplesDevice(self.h, ptr, n)
        err = last_error()
        if err:
            raise RuntimeError(err)

    def add_sample(self, sample):
        s = np.ascontiguousarray(np.asarray([sample], dtype=PGL_SAMPLE_DTYPE))
        self.lib.pglSampleStorageAddSample(self.h, ctypes.cast(s.ctypes.data, ctypes.POINTER(SampleData)))

    def clear(self):
        self.lib.pglSampleStorageClear(self.h)

    def clear_surface(self):
        self.lib.pglSampleStorageClearSurface(self.h)

    def clear_volume(self):
        self.lib.pglSampleStorageClearVolume(self.h)

    def reserve(self, ns, nv):
        self.lib.pglSampleStorageReserve(self.h, ns, nv)

    @property
    def size_surface(self):
        return int(self.lib.pglSampleStorageGetSizeSurface(self.h))

    @property
    def size_volume(self):
        return int(self.lib.pglSampleStorageGetSizeVolume(self.h))

    def sample(self, idx, volume=False):
        fn = self.lib.pglSampleStorageGetSampleVolume if volume else self.lib.pglSampleStorageGetSampleSurface
        d = fn(self.h, idx)
        out = np.zeros(1, dtype=PGL_SAMPLE_DTYPE)
        ctypes.memmove(out.ctypes.data, ctypes.byref(d), 40)
        return out[0]

    def validate(self):
        return bool(self.lib.pglSampleStorageValidate(self.h))

    def compare(self, other):
        return bool(self.lib.pglSampleStorageCompare(self.h, other.h))

    def store(self, path):
        return bool(self.lib.pglSampleStorageStoreToFile(self.h, path.encode()))

    def release(self):
        if self.h:
            self.lib.pglReleaseSampleStorage(self.h)
            self.h = None


class Field:
    def __init__(self, device, config):
        self.lib = load()
        self.h = self.lib.pglDeviceNewField(device.h, config.args)
        _check(self.h, "pglDeviceNewField")

    @classmethod
    def from_file(cls, device, path):
        """pglDeviceNewFieldFromFile: a field from a file in the reference's layout."""
        f = cls.__new__(cls)
        f.lib = load()
        f.h = f.lib.pglDeviceNewFieldFromFile(device.h, os.fsencode(path))
        _check(f.h, "pglDeviceNewFieldFromFile")
        return f

    def update(self, storage):
        self.lib.pglFieldUpdate(self.h, storage.h)
        err = last_error()
        if err:
            raise RuntimeError(err)

    def update_surface(self, storage):
        self.lib.pglFieldUpdateSurface(self.h, storage.h)

    def update_volume(self, storage):
        self.lib.pglFieldUpdateVolume(self.h, storage.h)

    def reset(self):
        self.lib.pglFieldReset(self.h)

    @property
    def iteration(self):
        return int(self.lib.pglFieldGetIteration(self.h))

    def set_scene_bounds(self, lower, upper):
        self.lib.pglFieldSetSceneBounds(self.h, Box3(Vec3(*lower), Vec3(*upper)))

    def scene_bounds(self):
        b = self.lib.pglFieldGetSceneBounds(self.h)
        return (b.lower.x, b.lower.y, b.lower.z), (b.upper.x, b.upper.y, b.upper.z)

    def validate(self):
        return bool(self.lib.pglFieldValidate(self.h))

    def compare(self, other):
        return bool(self.lib.pglFieldCompare(self.h, other.h))

    def field_bytes(self):
        n = self.lib.pglFieldStoreToBuffer(self.h, None, 0)
        buf = ctypes.create_string_buffer(int(n))
        self.lib.pglFieldStoreToBuffer(self.h, buf, n)
        return buf.raw

    def store(self, path):
        return bool(self.lib.pglFieldStoreToFile(self.h, path.encode()))

    def timings(self, volume=False):
        out = (ctypes.c_float * 4)()
        self.lib.pglFieldGetLastUpdateTimings(self.h, int(volume), out)
        return dict(total=out[0], copy=out[1], spatial=out[2], directional=out[3])

    def set_em_tuning(self, max_helpers=4, chunk_div=1, stage_cap=8, order_by_cost=0):
        """EM schedule parameters (speed only; see pglFieldSetEmTuning)."""
        t = (ctypes.c_int * 4)(max_helpers, chunk_div, stage_cap, order_by_cost)
        if not self.lib.pglFieldSetEmTuning(self.h, t):
            raise ValueError(last_error())

    def em_tuning(self):
        t = (ctypes.c_int * 4)()
        self.lib.pglFieldGetEmTuning(self.h, t)
        return dict(max_helpers=t[0], chunk_div=t[1], stage_cap=t[2], order_by_cost=t[3])

    def set_plain_update(self, plain=True):
        """The plain form of the directional fit: one launch per region (same results)."""
        _check(self.lib.pglFieldSetPlainUpdate(self.h, bool(plain)), "pglFieldSetPlainUpdate")

    def autotune_next_update(self):
        """The next Update times candidate EM schedules first and keeps the fastest."""
        self.lib.pglFieldAutotuneNextUpdate(self.h)

    def tuning_trials(self):
        n = self.lib.pglFieldGetEmTuningTrials(self.h, None, None, 0)
        t = (ctypes.c_int * (4 * n))()
        ms = (ctypes.c_float * n)()
        if n:
            self.lib.pglFieldGetEmTuningTrials(self.h, t, ms, n)
        return [dict(max_helpers=t[4 * i], chunk_div=t[4 * i + 1], stage_cap=t[4 * i + 2],
                     order_by_cost=t[4 * i + 3], ms=ms[i]) for i in range(n)]

    def profile(self, volume=False):
        """Per-region EM profile of the last Update (see pglFieldGetLastUpdateProfile)."""
        n = self.lib.pglFieldGetLastUpdateProfile(self.h, int(volume), None, 0)
        out = np.zeros((n, 23), dtype=np.uint64)
        if n:
            self.lib.pglFieldGetLastUpdateProfile(self.h, int(volume), out.ctypes.data, out.size)
        return out

    def phases(self, volume=False):
        out = (ctypes.c_double * 8)()
        self.lib.pglFieldGetLastUpdatePhases(self.h, int(volume), out, 8)
        keys = ("total", "copy", "spatial", "directional", "gather", "em_kernel", "samples", "regions")
        return dict(zip(keys, list(out)))

    def reports(self, volume=False):
        n = self.lib.pglFieldGetLastUpdateReports(self.h, int(volume), None, 0)
        out = np.zeros((n, 5), dtype=np.uint32)
        if n:
            self.lib.pglFieldGetLastUpdateReports(self.h, int(volume), out.ctypes.data, out.size)
        return out

    def statistics_string(self, volume=False):
        s = (self.lib.pglFieldGetVolumeStatistics if volume else self.lib.pglFieldGetSurfaceStatistics)(self.h)
        p = self.lib.pglFieldStatisticsToString(s)
        text = ctypes.string_at(p.m_str).decode()
        self.lib.pglReleaseString(p)
        self.lib.pglReleaseFieldStatistics(s)
        return text

    def sample_batch(self, queries, volume=False, cosine=True, out=None):
        """Guided queries (Init + cosine product + SamplePDF + pdfLi) in one
        launch; `out` (optional) receives the results."""
        q = np.ascontiguousarray(queries, dtype=PGL_QUERY_DTYPE)
        if out is None:
            out = np.zeros(len(q), dtype=QUERY_RESULT_DTYPE)
        assert out.dtype == QUERY_RESULT_DTYPE and len(out) == len(q) and out.flags.c_contiguous
        if volume:
            ok = self.lib.pglFieldSampleVolumeBatch(self.h, q.ctypes.data, len(q), out.ctypes.data)
        else:
            ok = self.lib.pglFieldSampleSurfaceBatch(self.h, q.ctypes.data, len(q), out.ctypes.data, cosine)
        _check(ok, "pglFieldSampleBatch")
        return out

    def sample_vertices(self, vertices):
        """Path-vertex queries: Init + cosine product + four SamplePDF calls per
        vertex, in one launch (pglFieldSampleSurfaceVertices)."""
        v = np.ascontiguousarray(vertices, dtype=PGL_VERTEX_DTYPE)
        out = np.zeros(len(v), dtype=VERTEX_RESULT_DTYPE)
        _check(self.lib.pglFieldSampleSurfaceVertices(self.h, v.ctypes.data, len(v), out.ctypes.data),
               "pglFieldSampleSurfaceVertices")
        return out

    def sample_vertices_device(self, v_ptr, n, out_ptr, stream=None):
        _check(self.lib.pglFieldSampleSurfaceVerticesDevice(self.h, v_ptr, n, out_ptr, stream),
               "pglFieldSampleSurfaceVerticesDevice")

    def sample_batch_hg(self, queries, mean_cosines):
        """Volume guided queries with the Henyey-Greenstein product (the query's
        normal is the phase function's direction)."""
        q = np.ascontiguousarray(queries, dtype=PGL_QUERY_DTYPE)
        g = np.ascontiguousarray(mean_cosines, dtype=np.float32)
        if len(g) != len(q):
            raise ValueError("one mean cosine per query")
        out = np.zeros(len(q), dtype=QUERY_RESULT_DTYPE)
        _check(self.lib.pglFieldSampleVolumeBatchHG(self.h, q.ctypes.data, g.ctypes.data, len(q), out.ctypes.data),
               "pglFieldSampleVolumeBatchHG")
        return out

    def sample_batch_hg_device(self, q_ptr, g_ptr, n, out_ptr, stream=None):
        ok = self.lib.pglFieldSampleVolumeBatchHGDevice(self.h, q_ptr, g_ptr, n, out_ptr, stream)
        _check(ok, "pglFieldSampleVolumeBatchHGDevice")

    def sample_batch_device(self, q_ptr, n, out_ptr, volume=False, cosine=True, stream=None):
        ok = self.lib.pglFieldSampleBatchDevice(self.h, volume, q_ptr, n, out_ptr, cosine, stream)
        _check(ok, "pglFieldSampleBatchDevice")

    def release(self):
        if self.h:
            self.lib.pglReleaseField(self.h)
            self.h = None


class SurfaceSamplingDistribution:
    """Per-object sampling distribution (one launch chain per call)."""

    volume = False

    def __init__(self, field):
        self.lib = load()
        self.field = field
        fn = (self.lib.pglFieldNewVolumeSamplingDistribution if self.volume
              else self.lib.pglFieldNewSurfaceSamplingDistribution)
        self.h = fn(field.h)
        _check(self.h, "pglFieldNew*SamplingDistribution")
        pre = "pglVolumeSamplingDistribution" if self.volume else "pglSurfaceSamplingDistribution"
        self._sample_pdf = getattr(self.lib, pre + "SamplePDF")
        self._pdf = getattr(self.lib, pre + "PDF")
        self._pdf_li = getattr(self.lib, pre + "IncomingRadiancePDF")
        self._get_id = getattr(self.lib, pre + "GetId")

    def init(self, position, sample1d):
        s = ctypes.c_float(sample1d)
        fn = (self.lib.pglFieldInitVolumeSamplingDistribution if self.volume
              else self.lib.pglFieldInitSurfaceSamplingDistribution)
        ok = fn(self.field.h, self.h, Vec3(*position), ctypes.byref(s))
        return bool(ok), s.value

    def apply_cosine_product(self, normal):
        self.lib.pglSurfaceSamplingDistributionApplyCosineProduct(self.h, Vec3(*normal))

    def sample_pdf(self, u):
        d = Vec3()
        pdf = self._sample_pdf(self.h, Vec2(*u), ctypes.byref(d))
        return (d.x, d.y, d.z), pdf

    def pdf(self, direction):
        return self._pdf(self.h, Vec3(*direction))

    def incoming_radiance_pdf(self, direction):
        return self._pdf_li(self.h, Vec3(*direction))

    def get_id(self):
        return int(self._get_id(self.h))

    def release(self):
        if self.h:
            fn = (self.lib.pglReleaseVolumeSamplingDistribution if self.volume
                  else self.lib.pglReleaseSurfaceSamplingDistribution)
            fn(self.h)
            self.h = None


class VolumeSamplingDistribution(SurfaceSamplingDistribution):
    volume = True

    def apply_hg_product(self, direction, mean_cosine):
        self.lib.pglVolumeSamplingDistributionApplySingleLobeHenyeyGreensteinProduct(self.h, Vec3(*direction),
                                                                                     float(mean_cosine))

    def supports_hg_product(self):
        return bool(self.lib.pglVolumeSamplingDistributionSupportsApplySingleLobeHenyeyGreensteinProduct(self.h))


class PathSegmentStorage:
    """One path's segments and the samples made from them (the reference's
    PathSegmentStorage, host memory)."""

    def __init__(self, reserve=64):
        from .synthetic import PGL_SAMPLE_DTYPE

        self.lib = load()
        self._dtype = PGL_SAMPLE_DTYPE
        self.h = self.lib.pglNewPathSegmentStorage()
        _check(self.h, "pglNewPathSegmentStorage")
        self.lib.pglPathSegmentStorageReserve(self.h, reserve)

    def clear(self):
        self.lib.pglPathSegmentStorageClear(self.h)

    def set_max_distance(self, d):
        self.lib.pglPathSegmentSetMaxDistance(self.h, float(d))

    def max_distance(self):
        return self.lib.pglPathSegmentGetMaxDistance(self.h)

    def num_segments(self):
        return self.lib.pglPathSegmentGetNumSegments(self.h)

    def num_samples(self):
        return self.lib.pglPathSegmentGetNumSamples(self.h)

    def add_segments(self, segments):
        """Appends PGL_PATH_SEGMENT_DTYPE records (NextSegment, then filled)."""
        seg = np.ascontiguousarray(segments)
        for i in range(len(seg)):
            p = self.lib.pglPathSegmentStorageNextSegment(self.h)
            if not p:
                raise RuntimeError("path segment storage is full")
            ctypes.memmove(p, seg[i:i + 1].ctypes.data, seg.dtype.itemsize)

    def prepare_samples(self, use_nee_mi_weights=False, guide_direct_light=False, rr_affects_direct=True):
        return self.lib.pglPathSegmentStoragePrepareSamples(self.h, use_nee_mi_weights, guide_direct_light,
                                                            rr_affects_direct)

    def samples(self):
        n = ctypes.c_size_t(0)
        p = self.lib.pglPathSegmentStorageGetSamples(self.h, ctypes.byref(n))
        out = np.zeros(n.value, dtype=self._dtype)
        if n.value:
            ctypes.memmove(out.ctypes.data, p, n.value * self._dtype.itemsize)
        return out

    def pixel_estimate(self, rr_affects_direct=True):
        c = self.lib.pglPathSegmentStorageCalculatePixelEstimate(self.h, rr_affects_direct)
        return (c.x, c.y, c.z)

    def validate_segments(self):
        return bool(self.lib.pglPathSegmentStorageValidateSegments(self.h))

    def validate_samples(self):
        return bool(self.lib.pglPathSegmentStorageValidateSamples(self.h))

    def propagate(self, storage, guide_direct_light=False, use_nee_mi_weights=False, rr_affects_direct=True):
        self.lib.pglPathSegmentStoragePropagateSamples(self.h, storage.h, guide_direct_light, use_nee_mi_weights,
                                                       rr_affects_direct)

    def release(self):
        if self.h:
            self.lib.pglReleasePathSegmentStorage(self.h)
            self.h = None

    def __del__(self):
        try:
            self.release()
        except Exception:
            pass


def path_samples_device(d_segments, d_path_begin, num_paths, max_distance, d_samples, d_sample_begin,
                        use_nee_mi_weights=False, guide_direct_light=False, rr_affects_direct=True, stream=None):
    """pglPathSegmentsPrepareSamplesDevice on device pointers."""
    lib = load()
    _check(lib.pglPathSegmentsPrepareSamplesDevice(d_segments, d_path_begin, num_paths, float(max_distance),
                                                   use_nee_mi_weights, guide_direct_light, rr_affects_direct,
                                                   d_samples, d_sample_begin, stream),
           "pglPathSegmentsPrepareSamplesDevice")


class GuidingServer:
    """A field served while it trains (pglNewGuidingServer): submit guided
    queries from any thread, add samples, start Updates in the background."""

    def __init__(self, field, hbm_budget_bytes=1 << 30, reserved_sms=None):
        self.lib = load()
        self.field = field
        if reserved_sms is None:
            self.h = self.lib.pglNewGuidingServer(field.h, hbm_budget_bytes)
        else:
            self.h = self.lib.pglNewGuidingServerEx(field.h, hbm_budget_bytes, int(reserved_sms))
        _check(self.h, "pglNewGuidingServer")
        self._keep = {}

    def submit(self, queries, volume=False, cosine=True, out=None):
        """Queue a batch; returns (ticket, result array filled when done)."""
        q = np.ascontiguousarray(queries, dtype=PGL_QUERY_DTYPE)
        if out is None:
            out = np.zeros(len(q), dtype=QUERY_RESULT_DTYPE)
        t = self.lib.pglGuidingServerSubmit(self.h, q.ctypes.data, len(q), out.ctypes.data, volume, cosine)
        _check(t != 0, "pglGuidingServerSubmit")
        self._keep[t] = (q, out)
        return t, out

    def submit_vertices(self, vertices, out=None):
        """Queue path vertices (Init + cosine product + four SamplePDF each);
        returns (ticket, result array filled when done).  `vertices` and `out`
        are kept alive until the request is waited for."""
        v = np.ascontiguousarray(vertices, dtype=PGL_VERTEX_DTYPE)
        if out is None:
            out = np.zeros(len(v), dtype=VERTEX_RESULT_DTYPE)
        t = self.lib.pglGuidingServerSubmitVertices(self.h, v.ctypes.data, len(v), out.ctypes.data)
        _check(t != 0, "pglGuidingServerSubmitVertices")
        self._keep[t] = (v, out)
        return t, out

    def wait(self, ticket):
        """(latency ms, field iteration of the results)"""
        lat = ctypes.c_double()
        ver = ctypes.c_uint64()
        ok = self.lib.pglGuidingServerWait(self.h, ticket, ctypes.byref(lat), ctypes.byref(ver))
        self._keep.pop(ticket, None)
        _check(ok, "pglGuidingServerWait")
        return lat.value, ver.value

    def add_samples(self, samples):
        s = np.ascontiguousarray(samples, dtype=PGL_SAMPLE_DTYPE)
        _check(self.lib.pglGuidingServerAddSamples(self.h, s.ctypes.data, len(s)), "pglGuidingServerAddSamples")

    def add_samples_device(self, ptr, n):
        _check(self.lib.pglGuidingServerAddSamplesDevice(self.h, ptr, n), "pglGuidingServerAddSamplesDevice")

    def update(self):
        t = self.lib.pglGuidingServerUpdate(self.h)
        _check(t != 0, "pglGuidingServerUpdate")
        return t

    def wait_update(self, ticket):
        _check(self.lib.pglGuidingServerWaitUpdate(self.h, ticket), "pglGuidingServerWaitUpdate")

    def stats(self):
        out = (ctypes.c_double * 11)()
        _check(self.lib.pglGuidingServerStatsEx(self.h, out, 11) == 11, "pglGuidingServerStatsEx")
        keys = ("queries", "requests", "p50_ms", "p99_ms", "p999_ms", "launches", "updates", "iteration",
                "device_bytes", "budget_bytes", "launch_capacity")
        return dict(zip(keys, list(out)))

    def reset_stats(self):
        _check(self.lib.pglGuidingServerResetStats(self.h), "pglGuidingServerResetStats")

    def release(self):
        if self.h:
            self.lib.pglReleaseGuidingServer(self.h)
            self.h = None
