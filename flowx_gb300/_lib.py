"""ctypes binding of libflowx.so (include/flowx.h).

The library is built in-tree by ``flowx_gb300.build``. Loading fails loudly
when it is missing: there is no CPU fallback for the substep.
"""

from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libflowx.so")

FLOWX_OK = 0
ERRORS = {1: "FLOWX_ERR_ARG", 2: "FLOWX_ERR_CUDA", 3: "FLOWX_ERR_STATE", 4: "FLOWX_ERR_CAPACITY"}

BUF = {
    "positions": 0,
    "velocities": 1,
    "lambda": 2,
    "predicted": 3,
    "delta": 4,
    "normal": 5,
    "keys": 6,
    "cell_start": 7,
    "cell_end": 8,
    "surface": 9,
}
PASS = {
    "normal": 0,
    "predict": 1,
    "grid_key": 2,
    "sort": 3,
    "cell_clear": 4,
    "cell_range": 5,
    "lambda": 6,
    "delta": 7,
    "apply_delta": 8,
    "velocity": 9,
    "xsph": 10,
    "finalize": 11,
}
FLAG_KEEP_DELTA = 1
FLAG_EXACT = 2
FLAG_REFERENCE_ORDER = 4
FLAG_WARP_PASSES = 8
FLAG_THREAD_PASSES = 16
WARP_PASSES_MAX_PARTICLES = 25000


class Push(ctypes.Structure):
    """flowx_push: the 128-byte block of shaders/sph_common.glsl:10-17."""

    _fields_ = [
        ("i_layout", ctypes.c_int32 * 4),
        ("i_grid", ctypes.c_int32 * 4),
        ("i_sort", ctypes.c_int32 * 4),
        ("f_lo", ctypes.c_float * 4),
        ("f_hi", ctypes.c_float * 4),
        ("f_sph", ctypes.c_float * 4),
        ("f_sim", ctypes.c_float * 4),
        ("i_collider", ctypes.c_int32 * 4),
    ]

    @classmethod
    def from_values(cls, values: dict):
        p = cls()
        for name, _ in cls._fields_:
            vec = values.get(name)
            if vec is None and name == "i_sort":
                vec = values["i_surface"]
            getattr(p, name)[:] = tuple(vec)
        return p


class Config(ctypes.Structure):
    _fields_ = [
        ("particle_count", ctypes.c_int32),
        ("max_cells", ctypes.c_int32),
        ("max_collider_voxels", ctypes.c_int64),
        ("max_surface_samples", ctypes.c_int64),
        ("device", ctypes.c_int32),
        ("flags", ctypes.c_int32),
    ]


class Primitive(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_int32),
        ("pad", ctypes.c_int32),
        ("a", ctypes.c_double * 3),
        ("b", ctypes.c_double * 3),
        ("r", ctypes.c_double),
    ]


class Mesh(ctypes.Structure):
    _fields_ = [
        ("vertices", ctypes.POINTER(ctypes.c_float)),
        ("vertex_count", ctypes.c_int32),
        ("triangles", ctypes.POINTER(ctypes.c_int32)),
        ("triangle_count", ctypes.c_int32),
        ("matrix_world", ctypes.c_float * 16),
    ]


class AdjointConfig(ctypes.Structure):
    """flowx_adjoint_config (include/flowx.h)."""

    _fields_ = [
        ("particle_count", ctypes.c_int32),
        ("max_cells", ctypes.c_int32),
        ("max_substeps", ctypes.c_int32),
        ("max_iterations", ctypes.c_int32),
        ("max_collider_voxels", ctypes.c_int64),
        ("max_surface_samples", ctypes.c_int64),
        ("device", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
    ]


class CacheHeader(ctypes.Structure):
    """flowx_cache_header (include/flowx.h)."""

    _fields_ = [
        ("flowx_version", ctypes.c_char * 16),
        ("particle_count", ctypes.c_int32),
        ("seed_frame", ctypes.c_int32),
        ("last_frame", ctypes.c_int32),
        ("fps", ctypes.c_float),
        ("collider_count", ctypes.c_int32),
        ("collider_names", ctypes.POINTER(ctypes.c_char_p)),
        ("config_hash", ctypes.c_uint8 * 32),
    ]


class FlowxError(RuntimeError):
    def __init__(self, code, message):
        super().__init__(f"{ERRORS.get(code, code)}: {message}")
        self.code = code


_LIB = None


def load(path: str | None = None):
    """Load libflowx.so (once). Raises if the library has not been built."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise RuntimeError(
            f"{path} is missing: build it with `python -m flowx_gb300.build` "
            "(nvcc, sm_103a); the PBF substep has no CPU implementation"
        )
    lib = ctypes.CDLL(path)
    P = ctypes.POINTER
    vp = ctypes.c_void_p
    ctx = vp
    sig = {
        "flowx_create": ([P(Config), P(vp)], ctypes.c_int),
        "flowx_destroy": ([ctx], ctypes.c_int),
        "flowx_last_error": ([ctx], ctypes.c_char_p),
        "flowx_upload": ([ctx, ctypes.c_int, vp, ctypes.c_size_t], ctypes.c_int),
        "flowx_download": ([ctx, ctypes.c_int, vp, ctypes.c_size_t], ctypes.c_int),
        "flowx_set_collider": ([ctx, vp, P(ctypes.c_int32), ctypes.c_float], ctypes.c_int),
        "flowx_voxelize": ([ctx, P(Primitive), ctypes.c_int, P(ctypes.c_int32), ctypes.c_float, P(ctypes.c_float)],
                           ctypes.c_int),
        "flowx_voxelize_meshes": ([ctx, P(Mesh), ctypes.c_int, P(ctypes.c_int32), ctypes.c_float, P(ctypes.c_float)],
                                  ctypes.c_int),
        "flowx_download_collider": ([ctx, vp, ctypes.c_size_t], ctypes.c_int),
        "flowx_build_grid": ([ctx, P(Push)], ctypes.c_int),
        "flowx_substep": ([ctx, P(Push), ctypes.c_int], ctypes.c_int),
        "flowx_step": ([ctx, P(Push), ctypes.c_int, ctypes.c_int], ctypes.c_int),
        "flowx_run_pass": ([ctx, ctypes.c_int, P(Push)], ctypes.c_int),
        "flowx_splat": ([ctx, P(Push), vp, ctypes.c_size_t], ctypes.c_int),
        "flowx_synchronize": ([ctx], ctypes.c_int),
        "flowx_get_stream": ([ctx, P(vp)], ctypes.c_int),
        "flowx_time_steps": ([ctx, P(Push), ctypes.c_int, ctypes.c_int, ctypes.c_int, P(ctypes.c_float)],
                             ctypes.c_int),
        "flowx_profile_substeps": ([ctx, P(Push), ctypes.c_int, ctypes.c_int, P(ctypes.c_float), P(ctypes.c_int32)],
                                   ctypes.c_int),
        "flowx_kernel_count": ([], ctypes.c_int),
        "flowx_kernel_name": ([ctypes.c_int], ctypes.c_char_p),
        "flowx_launch_count": ([], ctypes.c_int64),
        "flowx_batch_set_scenes": ([ctx, P(Push), ctypes.c_int], ctypes.c_int),
        "flowx_batch_scene_range": ([ctx, ctypes.c_int, P(ctypes.c_int32), P(ctypes.c_int32), P(ctypes.c_int32),
                                     P(ctypes.c_int32)], ctypes.c_int),
        "flowx_batch_set_collider": ([ctx, ctypes.c_int, vp, P(ctypes.c_int32), ctypes.c_float], ctypes.c_int),
        "flowx_batch_build_grid": ([ctx], ctypes.c_int),
        "flowx_batch_substep": ([ctx, ctypes.c_int], ctypes.c_int),
        "flowx_batch_step": ([ctx, ctypes.c_int, ctypes.c_int], ctypes.c_int),
        "flowx_batch_splat": ([ctx, ctypes.c_int, P(Push), vp, ctypes.c_size_t], ctypes.c_int),
        "flowx_autotune": ([ctx, P(Push), ctypes.c_int, P(ctypes.c_int32)], ctypes.c_int),
        "flowx_set_block_sizes": ([ctx, P(ctypes.c_int32)], ctypes.c_int),
        "flowx_adjoint_create": ([P(AdjointConfig), P(vp)], ctypes.c_int),
        "flowx_adjoint_destroy": ([vp], ctypes.c_int),
        "flowx_adjoint_last_error": ([vp], ctypes.c_char_p),
        "flowx_adjoint_get_stream": ([vp, P(vp)], ctypes.c_int),
        "flowx_adjoint_set_collider": ([vp, vp, P(ctypes.c_int32), ctypes.c_float], ctypes.c_int),
        "flowx_adjoint_forward": ([vp, P(Push), ctypes.c_int, ctypes.c_int, vp, vp, vp, vp, P(Push), vp],
                                  ctypes.c_int),
        "flowx_substep_adjoint": ([vp, vp, vp, vp, vp, vp], ctypes.c_int),
        "flowx_mc_create": ([ctypes.c_int32, P(vp)], ctypes.c_int),
        "flowx_mc_destroy": ([vp], ctypes.c_int),
        "flowx_mc_last_error": ([vp], ctypes.c_char_p),
        "flowx_mc_extract": ([vp, vp, P(ctypes.c_int32), P(ctypes.c_double), ctypes.c_double, ctypes.c_double, vp,
                              P(ctypes.c_int64), P(ctypes.c_int64)], ctypes.c_int),
        "flowx_mc_download": ([vp, vp, ctypes.c_size_t, vp, ctypes.c_size_t], ctypes.c_int),
        "flowx_mc_mesh": ([vp, P(vp), P(vp)], ctypes.c_int),
        "flowx_mc_case_table": ([ctypes.c_int32, P(ctypes.c_int32), P(ctypes.c_int32)], ctypes.c_int),
        "flowx_surface_field": ([ctx, P(vp), P(ctypes.c_int64)], ctypes.c_int),
        "flowx_cache_create": ([ctypes.c_char_p, P(CacheHeader), P(vp)], ctypes.c_int),
        "flowx_cache_open": ([ctypes.c_char_p, P(vp)], ctypes.c_int),
        "flowx_cache_close": ([vp], ctypes.c_int),
        "flowx_cache_last_error": ([vp], ctypes.c_char_p),
        "flowx_cache_info": ([vp, P(CacheHeader)], ctypes.c_int),
        "flowx_cache_collider_name": ([vp, ctypes.c_int32], ctypes.c_char_p),
        "flowx_cache_write_frame": ([vp, ctx, ctypes.c_int32], ctypes.c_int),
        "flowx_cache_load_frame": ([vp, ctx, ctypes.c_int32, P(Push)], ctypes.c_int),
        "flowx_cache_write_frame_host": ([vp, ctypes.c_int32, vp, vp], ctypes.c_int),
        "flowx_cache_read_frame_host": ([vp, ctypes.c_int32, vp, vp], ctypes.c_int),
        "flowx_build_grid_static": ([vp, ctypes.c_int32, P(Push), vp, ctypes.c_int32, vp, vp, vp], ctypes.c_int),
        "flowx_build_grid_static_error": ([], ctypes.c_char_p),
    }
    for name, (args, res) in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    _LIB = lib
    return lib


def check(rc: int, ctx=None):
    if rc != FLOWX_OK:
        lib = load()
        msg = lib.flowx_last_error(ctx)
        raise FlowxError(rc, msg.decode() if msg else "")
