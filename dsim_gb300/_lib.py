"""ctypes bindings of the engine's three shared libraries.

The libraries are built in-tree (dsim_gb300/lib/) by dsim_gb300/build.py.
There is no fallback: if a library is missing or fails to load, importing the
binding raises, so no caller can silently run without the GB300 engine.
"""
import ctypes as C
import os

import numpy as np

LIB_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "lib")
NATIVE = os.path.join(LIB_DIR, "libdsim_gb300.so")
ABI3 = os.path.join(LIB_DIR, "libdsim3.so")
ABI2 = os.path.join(LIB_DIR, "libdsim2.so")


class EngineMissing(ImportError):
    pass


def _load(path):
    if not os.path.exists(path):
        raise EngineMissing(
            "GB300 engine library %s is not built; run "
            "python -c 'import __graft_entry__ as g; g.build()'" % path)
    return C.CDLL(path, mode=C.RTLD_LOCAL)


_nd = np.ctypeslib.ndpointer


class _Opt:
    """ndpointer that accepts None."""

    def __init__(self, dtype):
        self.base = _nd(dtype, flags="C_CONTIGUOUS")

    def from_param(self, obj):
        if obj is None:
            return None
        return self.base.from_param(obj)


F32 = _nd(np.float32, flags="C_CONTIGUOUS")
F64 = _nd(np.float64, flags="C_CONTIGUOUS")
U32 = _nd(np.uint32, flags="C_CONTIGUOUS")
U16 = _nd(np.uint16, flags="C_CONTIGUOUS")
U8 = _nd(np.uint8, flags="C_CONTIGUOUS")
OF32, OU32, OU16, OU8 = _Opt(np.float32), _Opt(np.uint32), _Opt(np.uint16), _Opt(np.uint8)
VP = C.c_void_p


class MeshParams(C.Structure):
    """dsim_mesh_params (include/dsim.h)."""
    _fields_ = [("stdDevs", C.c_float * 4), ("T2", C.c_float * 4), ("permeability", C.c_float),
                ("reflectionType", C.c_uint32), ("spinRadius", C.c_float),
                ("deltaTime", C.c_float), ("phaseConstant", C.c_float),
                ("maxSubsegments", C.c_uint32)]


class CylParams(C.Structure):
    """dsim_cyl_params (include/dsim.h)."""
    _fields_ = [("intraAdc", C.c_float), ("extraAdc", C.c_float), ("myelinAdc", C.c_float),
                ("spaceScale", C.c_float), ("T2fiber", C.c_float), ("T2myelin", C.c_float),
                ("T2outside", C.c_float), ("permeability", C.c_float),
                ("innerRadiusProportion", C.c_float), ("spinRadius", C.c_float),
                ("deltaTime", C.c_float), ("phaseConstant", C.c_float)]


class Float3(C.Structure):
    """The reference's float3 passed by value across its C-ABI."""
    _fields_ = [("x", C.c_float), ("y", C.c_float), ("z", C.c_float)]


def _declare_native(L):
    i32, u32, u64, f32 = C.c_int, C.c_uint32, C.c_uint64, C.c_float
    sig = {
        "dsim_last_error": (C.c_char_p, []),
        "dsim_version": (i32, []),
        "dsim_device_info": (i32, [C.c_char_p, i32, C.POINTER(i32), C.POINTER(C.c_size_t)]),
        "dsim_mesh_load": (i32, [C.c_char_p, f32, u32, C.POINTER(VP)]),
        "dsim_mesh_create": (i32, [F32, u32, U32, OU32, OU32, u32, f32, u32, C.POINTER(VP)]),
        "dsim_mesh_info": (i32, [VP, _nd(np.uint64, flags="C_CONTIGUOUS")]),
        "dsim_mesh_grid": (i32, [VP, OU32, OU32]),
        "dsim_mesh_arrays": (i32, [VP, OF32, OU32]),
        "dsim_mesh_free": (None, [VP]),
        "dsim_mesh_set_accel": (i32, [VP, u32]),
        "dsim_mesh_set_kernel": (i32, [VP, u32]),
        "dsim_mesh_set_records": (i32, [VP, u32]),
        "dsim_mesh_accel_info": (i32, [VP, _nd(np.uint64, flags="C_CONTIGUOUS")]),
        "dsim_spins_set_sort_interval": (i32, [VP, u32]),
        "dsim_cyl_load": (i32, [C.c_char_p, f32, C.POINTER(VP)]),
        "dsim_cyl_create": (i32, [F32, u32, f32, C.POINTER(VP)]),
        "dsim_cyl_info": (i32, [VP, U32, C.POINTER(f32), OU32, OU32, OF32]),
        "dsim_cyl_set_fine": (i32, [VP, u32]),
        "dsim_cyl_fine_lists": (i32, [F32, u32, u32, u32, f32, U32, U32, u32, OU32, OU32, C.c_uint64,
                                      C.POINTER(C.c_uint64)]),
        "dsim_cyl_fine_info": (i32, [VP, _nd(np.uint64, flags="C_CONTIGUOUS")]),
        "dsim_cyl_free": (None, [VP]),
        "dsim_spins_create": (i32, [u32, C.POINTER(VP)]),
        "dsim_spins_count": (u32, [VP]),
        "dsim_spins_set": (i32, [VP, OF32, OF32, OF32, OU8, OU16]),
        "dsim_spins_get": (i32, [VP, OF32, OF32, OF32, OU8, OU16]),
        "dsim_spins_set_cyl": (i32, [VP, F32, OF32, OF32, OU32, OU32]),
        "dsim_spins_get_cyl": (i32, [VP, OF32, OF32, OF32, OU32, OU32]),
        "dsim_spins_counts": (i32, [VP, OU32, i32]),
        "dsim_spins_scanned": (i32, [VP, OU32, i32]),
        "dsim_spins_status": (i32, [VP, C.POINTER(u32), i32]),
        "dsim_spins_bytes": (u64, [VP]),
        "dsim_spins_free": (None, [VP]),
        "dsim_mesh_run": (i32, [VP, VP, C.POINTER(MeshParams), OF32, OF32, u32, u64, u64, OF32, i32]),
        "dsim_cyl_run": (i32, [VP, VP, C.POINTER(CylParams), OF32, OF32, u32, u64, u64, OF32, i32]),
        "dsim_signal": (i32, [VP, C.c_double, F64]),
        "dsim_signal_noalloc": (i32, [VP, VP, u32, i32, C.c_double, VP, VP]),
        "dsim_sync": (i32, [VP]),
        "dsim_timer_start": (i32, [VP]),
        "dsim_timer_stop": (i32, [VP, C.POINTER(f32)]),
        "dsim_flush_l2": (i32, [VP, C.c_size_t]),
        "dsim_spins_launches": (i32, [VP, C.POINTER(u64), i32]),
        "dsim_spins_set_spin_base": (i32, [VP, u32]),
        "dsim_mesh_compartments": (i32, [VP, VP, u64, f32, C.POINTER(u32)]),
        "dsim_rng_draws": (i32, [u64, u32, u64, u32, u32, OU32, OF32]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    return L


class Config(C.Structure):
    """dsim_config (include/dsim_sim.h)."""
    _fields_ = [("dialect", C.c_int), ("stepsPerUpdate", C.c_uint32), ("useGpu", C.c_int),
                ("useDisplay", C.c_int), ("writeOut", C.c_int), ("numSpins", C.c_uint32), ("gamma", C.c_float),
                ("timeStep", C.c_float), ("extraAdc", C.c_float), ("intraAdc", C.c_float),
                ("myelinAdc", C.c_float), ("extraT2", C.c_float), ("intraT2", C.c_float),
                ("myelinT2", C.c_float), ("spaceScale", C.c_float), ("startBox", C.c_float),
                ("permeability", C.c_float), ("innerRadiusFraction", C.c_float),
                ("gradsFile", C.c_char * 512), ("gradsStr", C.c_char * 512), ("outFile", C.c_char * 512),
                ("fiberFile", C.c_char * 512), ("fiberRadius", C.c_float), ("fiberSpace", C.c_float),
                ("crossFraction", C.c_float)]


class JobDesc(C.Structure):
    """dsim_job_desc (include/dsim_batch.h)."""
    _fields_ = [("substrate", C.c_uint32), ("nSpins", C.c_uint32), ("steps", C.c_uint32),
                ("deltaTime", C.c_float), ("stepSd", C.c_float * 4), ("T2", C.c_float * 4),
                ("permeability", C.c_float), ("reflectionType", C.c_uint32), ("spinRadius", C.c_float),
                ("innerRadiusProportion", C.c_float), ("phaseConstant", C.c_float),
                ("waveform", C.c_uint32), ("delta", C.c_float), ("Delta", C.c_float),
                ("frequency", C.c_float), ("table", C.c_void_p), ("seed", C.c_uint64), ("flags", C.c_uint32),
                ("reserved", C.c_uint32)]


def _declare_batch(L):
    i32, u32, u64 = C.c_int, C.c_uint32, C.c_uint64
    U64 = _nd(np.uint64, flags="C_CONTIGUOUS")
    sig = {
        "dsim_batch_create": (i32, [u64, u32, C.POINTER(VP)]),
        "dsim_batch_free": (None, [VP]),
        "dsim_batch_add_mesh": (i32, [VP, VP, C.POINTER(u32)]),
        "dsim_batch_add_cyl": (i32, [VP, VP, C.POINTER(u32)]),
        "dsim_batch_submit": (i32, [VP, C.POINTER(JobDesc), F32, U8, OU32, C.POINTER(u32)]),
        "dsim_batch_configure": (i32, [VP, u32, u32, u32]),
        "dsim_batch_set_block": (i32, [VP, u32]),
        "dsim_batch_block": (i32, [VP, C.POINTER(u32)]),
        "dsim_batch_advance": (i32, [VP, u32]),
        "dsim_batch_run": (i32, [VP]),
        "dsim_batch_job_status": (i32, [VP, u32, C.POINTER(u32), C.POINTER(i32)]),
        "dsim_batch_signal": (i32, [VP, u32, F32, u32, F64]),
        "dsim_batch_signal_region": (i32, [VP, u32, F32, u32, C.c_double, F64]),
        "dsim_batch_get": (i32, [VP, u32, OF32, OF32, OF32, OU8, OU32]),
        "dsim_batch_counts": (i32, [VP, u32, U64]),
        "dsim_batch_status": (u32, [VP]),
        "dsim_batch_precision_counts": (i32, [VP, u32, U64]),
        "dsim_batch_get_precise": (i32, [VP, u32, F64, F64]),
        "dsim_batch_retire": (i32, [VP, u32]),
        "dsim_batch_compact": (i32, [VP]),
        "dsim_batch_info": (i32, [VP, U64]),
        "dsim_batch_sync": (i32, [VP]),
        "dsim_batch_autotune": (i32, [VP, u32, _nd(np.uint32, flags="C_CONTIGUOUS"), C.POINTER(C.c_float)]),
        "dsim_server_create": (i32, [u64, u32, u64, C.POINTER(VP)]),
        "dsim_server_free": (None, [VP]),
        "dsim_server_add_mesh": (i32, [VP, VP, C.POINTER(u32)]),
        "dsim_server_add_cyl": (i32, [VP, VP, C.POINTER(u32)]),
        "dsim_server_configure": (i32, [VP, u32, u32, u32]),
        "dsim_server_start": (i32, [VP]),
        "dsim_server_submit": (i32, [VP, C.POINTER(JobDesc), F32, U8, OU32, F32, u32, C.POINTER(u32)]),
        "dsim_server_poll": (i32, [VP, u32, C.POINTER(i32), _Opt(np.float64), _Opt(np.float64)]),
        "dsim_server_drain": (i32, [VP]),
        "dsim_server_stop": (i32, [VP]),
        "dsim_server_stats": (i32, [VP, F64]),
        "dsim_config_load": (i32, [C.c_char_p, C.POINTER(Config)]),
        "dsim_grads_parse_file": (i32, [C.c_char_p, OF32, u32, C.POINTER(u32)]),
        "dsim_grads_parse_string": (i32, [C.c_char_p, OF32, u32, C.POINTER(u32)]),
        "dsim_pgse_schedule": (i32, [F32, C.c_float, u32, OF32, u32, C.POINTER(u32)]),
        "dsim_tensor_fit": (i32, [F32, F64, u32, F64, F64, F32, C.POINTER(C.c_float), C.POINTER(C.c_float),
                                  C.POINTER(C.c_float)]),
        "dsim_simulate": (i32, [C.c_char_p, u64, u32, F64, u32, C.POINTER(u32), C.POINTER(C.c_double)]),
        "dsim_write_results": (i32, [C.c_char_p, C.POINTER(Config), F32, F64, u32, C.c_double]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    return L


def _declare_abi3(L):
    i32, u32, f32 = C.c_int, C.c_uint, C.c_float
    sig = {
        "checkCUDA": (None, []),
        "allocateArray": (None, [C.POINTER(VP), i32]),
        "freeArray": (None, [VP]),
        "threadSync": (None, []),
        "copyArrayFromDevice": (None, [VP, VP, u32, i32]),
        "copyArrayToDevice": (None, [VP, VP, i32, i32]),
        "copyConstantToDevice": (None, [C.c_char_p, VP, i32, i32]),
        "registerGLBufferObject": (None, [u32]),
        "unregisterGLBufferObject": (None, [u32]),
        "bindCubeCounter": (None, [VP, i32]),
        "unbindCubeCounter": (None, []),
        "bindTrianglesInCubes": (None, [VP, i32]),
        "unbindTrianglesInCubes": (None, []),
        "bindVertices": (None, [VP, i32]),
        "unbindVertices": (None, []),
        "bindTriangleHelpers": (None, [VP, i32]),
        "unbindTriangleHelpers": (None, []),
        "bindRTreeArray": (None, [VP, i32]),
        "unbindRTreeArray": (None, []),
        "bindTreeIndexArray": (None, [VP, i32]),
        "unbindTreeIndexArray": (None, []),
        "bindTriInfo": (None, [VP, i32]),
        "unbindTriInfo": (None, []),
        "integrateSystem": (None, [VP, VP, VP, f32, f32, i32, Float3, f32, u32, VP, VP]),
        "integrateSystemVBO": (None, [u32, VP, VP, f32, f32, i32, Float3, f32, u32, VP, VP]),
        "dsim3_last_error": (C.c_char_p, []),
        "dsim3_last_status": (i32, []),
        "dsim3_set_replay": (None, [VP, VP]),
        "dsim3_status": (u32, []),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    return L


def _declare_abi2(L):
    i32, u32, f32 = C.c_int, C.c_uint, C.c_float
    sig = {
        "checkCUDA": (None, []),
        "allocateArray": (None, [C.POINTER(VP), i32]),
        "freeArray": (None, [VP]),
        "threadSync": (None, []),
        "copyArrayFromDevice": (None, [VP, VP, u32, i32]),
        "copyArrayToDevice": (None, [VP, VP, i32, i32]),
        "registerGLBufferObject": (None, [u32]),
        "unregisterGLBufferObject": (None, [u32]),
        "bindFiberList": (None, [VP, i32]),
        "unbindFiberList": (None, []),
        "bindCubeList": (None, [VP, i32]),
        "unbindCubeList": (None, []),
        "integrateSystem": (None, [VP, VP, f32, VP, f32, f32, f32, f32, i32, Float3, f32, VP, VP,
                                   f32, u32, u32, f32, u32]),
        "integrateSystemVbo": (None, [u32, VP, f32, VP, f32, f32, f32, f32, i32, Float3, f32, VP,
                                      VP, f32, u32, u32, f32, u32]),
        "dsim2_last_error": (C.c_char_p, []),
        "dsim2_last_status": (i32, []),
        "dsim2_set_replay": (None, [VP, VP]),
        "dsim2_status": (u32, []),
        "dsim2_set_fine": (None, [C.c_int]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    return L


_cache = {}


def native():
    if "native" not in _cache:
        _cache["native"] = _declare_batch(_declare_native(_load(NATIVE)))
    return _cache["native"]


def abi3():
    if "abi3" not in _cache:
        _cache["abi3"] = _declare_abi3(_load(ABI3))
    return _cache["abi3"]


def abi2():
    if "abi2" not in _cache:
        _cache["abi2"] = _declare_abi2(_load(ABI2))
    return _cache["abi2"]


class DsimError(RuntimeError):
    pass


def check(rc, lib=None):
    if rc != 0:
        msg = (lib or native()).dsim_last_error()
        raise DsimError("%d: %s" % (rc, msg.decode() if msg else ""))
    return rc
