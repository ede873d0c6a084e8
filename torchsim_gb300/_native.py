"""ctypes binding of ``libtorchsim_gb300.so`` (the C ABI in ``include/``).

The library is the only compute path: if it is missing or cannot load, every
call raises. There is no CPU fallback.
"""

from __future__ import annotations

import ctypes
from pathlib import Path

PACKAGE = Path(__file__).resolve().parent
LIBRARY = PACKAGE / "_lib" / "libtorchsim_gb300.so"

TSG_OK = 0
TSG_ERR_ARGUMENT = -1
TSG_ERR_UNSUPPORTED = -2
TSG_ERR_CUDA = -3
TSG_ERR_CAPACITY = -4

LAYOUT_PLANES = 0
LAYOUT_COMPLEX_IJ = 1
LAYOUT_COMPLEX = 2

TANGENT_T1 = 1
TANGENT_T2 = 2
TANGENT_B1 = 4
TANGENT_INVERSION = 8


class NativeError(RuntimeError):
    """A failure reported by the CUDA library."""

    def __init__(self, code: int, message: str) -> None:
        super().__init__(f"torchsim_gb300 error {code}: {message}")
        self.code = code


class Tissue(ctypes.Structure):
    _fields_ = [(n, ctypes.c_void_p) for n in ("t1_ms", "t2_ms", "m0", "b1", "inversion")]


class Offaxis(ctypes.Structure):
    _fields_ = [(n, ctypes.c_void_p) for n in ("b1_phase_rad", "b0_hz")]


class OffaxisDirection(ctypes.Structure):
    _fields_ = [(n, ctypes.c_void_p) for n in ("b1_phase_rad", "b0_hz", "phase_rad")]


class OffaxisGradients(ctypes.Structure):
    _fields_ = [(n, ctypes.c_void_p) for n in ("b1_phase_rad", "b0_hz", "phase_rad")]


class Direction(ctypes.Structure):
    _fields_ = [(n, ctypes.c_void_p) for n in
                ("t1_ms", "t2_ms", "m0", "b1", "inversion", "duration_s", "flip_rad")]


class Gradients(ctypes.Structure):
    _fields_ = [(n, ctypes.c_void_p) for n in
                ("t1_ms", "t2_ms", "m0", "b1", "inversion", "flip_rad", "duration_s")]


class BatchSequence(ctypes.Structure):
    _fields_ = [("op_offset", ctypes.c_int32), ("op_count", ctypes.c_int32),
                ("states", ctypes.c_int32), ("lanes_per_voxel", ctypes.c_int32),
                ("outputs", ctypes.c_int32), ("voxel_count", ctypes.c_int32),
                ("voxel_offset", ctypes.c_int64), ("output_offset", ctypes.c_int64)]


class BatchUnit(ctypes.Structure):
    _fields_ = [("sequence", ctypes.c_int32), ("voxel_begin", ctypes.c_int32),
                ("voxel_count", ctypes.c_int32), ("reserved", ctypes.c_int32)]


class GNState(ctypes.Structure):
    _fields_ = [(n, ctypes.c_void_p) for n in
                ("u", "cand", "cost", "normal", "trial", "damping", "rising", "predicted", "status",
                 "flags", "iterations", "t1", "t2", "m0")]


class GNConfig(ctypes.Structure):
    _fields_ = [("low", ctypes.c_double * 3), ("high", ctypes.c_double * 3),
                ("tau", ctypes.c_double), ("gradient_tolerance", ctypes.c_double),
                ("step_tolerance", ctypes.c_double), ("max_iterations", ctypes.c_int32)]


class Launch(ctypes.Structure):
    _fields_ = [("lanes_per_voxel", ctypes.c_int), ("orders_per_lane", ctypes.c_int),
                ("warps_per_block", ctypes.c_int), ("min_blocks_per_sm", ctypes.c_int)]


_i64 = ctypes.c_int64
_vp = ctypes.c_void_p
_int = ctypes.c_int

# name -> (restype, argtypes)
SIGNATURES: dict[str, tuple] = {
    "tsg_last_error": (ctypes.c_char_p, []),
    "tsg_version": (_int, []),
    "tsg_probe_fp32": (_int, [_i64, _int, _int, _vp, _vp, ctypes.POINTER(ctypes.c_double)]),
    "tsg_probe_fp32x2": (_int, [_i64, _int, _int, _vp, _vp, ctypes.POINTER(ctypes.c_double)]),
    "tsg_program_create": (_int, [_vp, _vp, _vp, _vp, _vp, _i64, _i64, _int, _vp,
                                  ctypes.POINTER(_vp)]),
    "tsg_program_create_phased": (_int, [_vp, _vp, _vp, _vp, _vp, _vp, _i64, _i64,
                                         ctypes.POINTER(_vp)]),
    "tsg_program_destroy": (_int, [_vp]),
    "tsg_program_plan": (_int, [_vp, _vp, _vp, _vp, _vp, _i64, _i64, _int, _vp,
                                ctypes.POINTER(_i64), ctypes.POINTER(_i64), _vp, _vp, _vp, _vp,
                                _i64]),
    "tsg_program_info": (_int, [_vp, ctypes.POINTER(_i64), ctypes.POINTER(_i64),
                                ctypes.POINTER(_i64), ctypes.POINTER(_i64)]),
    "tsg_program_rebind": (_int, [_vp, _vp, _vp, _vp, _vp]),
    "tsg_program_view": (_int, [_vp, _vp, ctypes.POINTER(_vp)]),
    "tsg_sequential_sum": (_int, [_vp, _i64, _vp, _vp]),
    "tsg_epg_forward": (_int, [_vp, ctypes.POINTER(Tissue), _i64, _i64, _int, _vp, _vp,
                               ctypes.POINTER(Launch), _vp]),
    "tsg_epg_forward_complex": (_int, [_vp, ctypes.POINTER(Tissue), ctypes.POINTER(Offaxis), _i64,
                                       _i64, _int, _vp, _vp, ctypes.POINTER(Launch), _vp]),
    "tsg_epg_forward_tangents_complex": (_int, [_vp, ctypes.POINTER(Tissue), ctypes.POINTER(Offaxis),
                                                _i64, _i64, ctypes.c_uint,
                                                ctypes.POINTER(ctypes.c_int32), ctypes.c_int32,
                                                _int, _vp, _vp, _vp, _vp, ctypes.POINTER(Launch),
                                                _vp]),
    "tsg_epg_forward_tangents": (_int, [_vp, ctypes.POINTER(Tissue), _i64, _i64, ctypes.c_uint,
                                        ctypes.POINTER(ctypes.c_int32), ctypes.c_int32, _int,
                                        _vp, _vp, _vp, _vp, ctypes.POINTER(Launch), _vp]),
    "tsg_epg_tangent": (_int, [_vp, ctypes.POINTER(Tissue), _i64, _i64, ctypes.POINTER(Direction),
                               _vp, _vp, ctypes.POINTER(Launch), _vp]),
    "tsg_epg_tangent_complex": (_int, [_vp, ctypes.POINTER(Tissue), ctypes.POINTER(Offaxis), _i64,
                                       _i64, ctypes.POINTER(Direction),
                                       ctypes.POINTER(OffaxisDirection), _int, _vp, _vp,
                                       ctypes.POINTER(Launch), _vp]),
    "tsg_epg_forward_checkpointed": (_int, [_vp, ctypes.POINTER(Tissue), _i64, _i64, _int, _vp,
                                            _vp, _vp, _int, ctypes.POINTER(Launch), _vp]),
    "tsg_epg_adjoint_plan": (_int, [_vp, _i64, _i64, ctypes.POINTER(Launch), _int,
                                    ctypes.POINTER(_int), ctypes.POINTER(_i64),
                                    ctypes.POINTER(_i64)]),
    "tsg_epg_adjoint": (_int, [_vp, ctypes.POINTER(Tissue), _i64, _i64, _vp, _int, _vp, _int,
                               ctypes.POINTER(Gradients), _vp, _i64, ctypes.POINTER(Launch),
                               _vp]),
    "tsg_epg_adjoint_noalloc": (_int, [_vp, ctypes.POINTER(Tissue), _i64, _i64, _vp, _int,
                                       ctypes.POINTER(Gradients), ctypes.POINTER(Launch), _vp]),
    "tsg_static_scratch_bytes": (_i64, []),
    "tsg_epg_batched_forward": (_int, [_vp, _vp, _vp, _i64, _vp, ctypes.POINTER(Tissue), _vp, _int,
                                       _int, _int, _vp]),
    "tsg_gn_evaluate": (_int, [_vp, ctypes.POINTER(Tissue), _i64, _i64, _vp, _vp, _vp,
                               ctypes.POINTER(Launch), _vp]),
    "tsg_gn_step": (_int, [ctypes.POINTER(GNState), _i64, ctypes.POINTER(GNConfig), _vp]),
    "tsg_gn_judge": (_int, [ctypes.POINTER(GNState), _i64, ctypes.POINTER(GNConfig), _vp]),
    "tsg_gn_natural": (_int, [_vp, _i64, ctypes.POINTER(GNConfig), _vp, _vp]),
    "tsg_match_screen": (_int, [_vp, _i64, _vp, _i64, _i64, _vp, _vp, _vp, _vp]),
    "tsg_match_rescore": (_int, [_vp, _i64, _vp, _i64, _i64, _vp, _int, _vp, _vp, _vp]),
    "tsg_match_candidates": (_int, []),
    "tsg_match_screen_rows": (_int, [_i64]),
    "tsg_epg_simulate_vjp": (_int, [ctypes.POINTER(_vp), _i64, _i64, _i64, _i64, _i64, _i64,
                                    _int, _int]),
    "tsg_epg_simulate": (_int, [ctypes.POINTER(_vp), _i64, _i64, _i64, _i64, _i64, _i64, _int,
                                _int]),
    "tsg_epg_simulate_jvp": (_int, [ctypes.POINTER(_vp), _i64, _i64, _i64, _i64, _i64, _i64,
                                    _int, _int]),
    "tsg_epg_simulate_vjp_jvp": (_int, [ctypes.POINTER(_vp), _i64, _i64, _i64, _i64, _i64, _i64,
                                        _int, _int]),
    "tsg_epg_second_plan": (_int, [_vp, _i64, _i64, _int, _int, ctypes.POINTER(Launch),
                                   ctypes.POINTER(_i64), ctypes.POINTER(_i64)]),
    "tsg_epg_second_forward": (_int, [_vp, ctypes.POINTER(Tissue), _i64, _i64,
                                      ctypes.POINTER(Direction), _int, _int, _int, _vp, _vp, _vp,
                                      _vp,
                                      _vp, _vp, ctypes.POINTER(Launch), _vp]),
    "tsg_epg_complex_adjoint_plan": (_int, [_vp, _i64, _i64, ctypes.POINTER(Launch),
                                            ctypes.POINTER(_i64), ctypes.POINTER(_i64)]),
    "tsg_epg_forward_complex_trajectory": (_int, [_vp, ctypes.POINTER(Tissue),
                                                  ctypes.POINTER(Offaxis), _i64, _i64, _int, _vp,
                                                  _vp, _vp, ctypes.POINTER(Launch), _vp]),
    "tsg_epg_adjoint_complex": (_int, [_vp, ctypes.POINTER(Tissue), ctypes.POINTER(Offaxis), _i64,
                                       _i64, _vp, _vp, _int, _vp, ctypes.POINTER(Gradients),
                                       ctypes.POINTER(OffaxisGradients), _vp, _i64,
                                       ctypes.POINTER(Launch), _vp]),
    "tsg_epg_design_plan": (_int, [_vp, _i64, _i64, ctypes.c_uint, ctypes.POINTER(Launch),
                                   ctypes.POINTER(_i64), ctypes.POINTER(_i64)]),
    "tsg_epg_design_forward": (_int, [_vp, ctypes.POINTER(Tissue), _i64, _i64, ctypes.c_uint,
                                      _int, _int, _vp, _vp, _vp, _vp, _vp,
                                      ctypes.POINTER(Launch), _vp]),
    "tsg_epg_design_reverse": (_int, [_vp, ctypes.POINTER(Tissue), _i64, _i64, ctypes.c_uint,
                                      _int, _vp, _vp, _int, _vp, ctypes.POINTER(Gradients), _vp,
                                      _i64, ctypes.POINTER(Launch), _vp]),
    "tsg_epg_second_reverse": (_int, [_vp, ctypes.POINTER(Tissue), _i64, _i64,
                                      ctypes.POINTER(Direction), _int, _int, _vp, _vp, _int, _vp,
                                      ctypes.POINTER(Gradients), ctypes.POINTER(Gradients), _vp,
                                      _i64, ctypes.POINTER(Launch), _vp]),
}

_lib: ctypes.CDLL | None = None


def library() -> ctypes.CDLL:
    """Load the CUDA library (once), raising if it has not been built."""
    global _lib
    if _lib is None:
        if not LIBRARY.exists():
            raise NativeError(
                TSG_ERR_UNSUPPORTED,
                f"{LIBRARY} is missing; build it with torchsim_gb300._build.build()",
            )
        lib = ctypes.CDLL(str(LIBRARY))
        for name, (restype, argtypes) in SIGNATURES.items():
            if not hasattr(lib, name):
                continue
            fn = getattr(lib, name)
            fn.restype = restype
            fn.argtypes = argtypes
        _lib = lib
    return _lib


def check(code: int) -> None:
    """Raise the library's last error for a non-zero return code."""
    if code != TSG_OK:
        message = library().tsg_last_error()
        text = message.decode() if message else "unknown error"
        if code == TSG_ERR_ARGUMENT:
            raise ValueError(text)
        raise NativeError(code, text)


def call(name: str, *args) -> None:
    check(getattr(library(), name)(*args))


def launch_shape(shape) -> ctypes.POINTER(Launch) | None:
    """A Launch struct from a (lanes, orders, warps[, min_blocks]) tuple, or
    None for the built-in choice."""
    if shape is None:
        return None
    lanes, orders, warps = shape[:3]
    min_blocks = shape[3] if len(shape) > 3 else 0
    return ctypes.pointer(Launch(int(lanes), int(orders), int(warps), int(min_blocks)))
