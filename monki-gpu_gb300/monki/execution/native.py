"""ctypes binding of the sm_103a transport library (``libmonki_cuda.so``).

The library exports the C ABI declared in ``include/monki_cuda.h``. Loading never builds
anything and never falls back: a missing or stale library raises immediately.
"""

from __future__ import annotations

import ctypes
from pathlib import Path

LIBRARY = Path(__file__).resolve().parents[1] / "_native" / "libmonki_cuda.so"
ABI_VERSION = 1

_U32P = ctypes.POINTER(ctypes.c_uint32)
_U64P = ctypes.POINTER(ctypes.c_uint64)
_F64P = ctypes.POINTER(ctypes.c_double)
_F32P = ctypes.POINTER(ctypes.c_float)

_SIGNATURES = {
    "monki_cuda_abi_version": (ctypes.c_int, []),
    "monki_cuda_create": (
        ctypes.c_void_p,
        [ctypes.c_uint32, _F64P, ctypes.c_size_t, ctypes.c_uint32, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_size_t],
    ),
    "monki_cuda_run": (ctypes.c_int, [ctypes.c_void_p, _U32P, _F64P, ctypes.c_char_p, ctypes.c_size_t]),
    "monki_cuda_gpu_seconds": (ctypes.c_double, [ctypes.c_void_p]),
    "monki_cuda_last_timing": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_float)]),
    "monki_cuda_counters": (ctypes.c_int, [ctypes.c_void_p, _U64P]),
    "monki_cuda_stage_timing": (ctypes.c_int, [ctypes.c_void_p, _F64P, _U64P]),
    "monki_cuda_tally_count": (ctypes.c_size_t, [ctypes.c_void_p]),
    "monki_cuda_device_name": (ctypes.c_char_p, [ctypes.c_void_p]),
    "monki_cuda_close": (None, [ctypes.c_void_p]),
    "monki_cuda_inspect": (
        ctypes.c_int,
        [_F64P, ctypes.c_size_t, ctypes.c_int, ctypes.POINTER(ctypes.c_int32), _F64P, ctypes.c_size_t, ctypes.c_char_p, ctypes.c_size_t],
    ),
    "monki_cuda_inspect_rectangles": (
        ctypes.c_int,
        [_F64P, ctypes.c_size_t, ctypes.c_int, _U32P, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t), ctypes.c_char_p, ctypes.c_size_t],
    ),
    "monki_cuda_set_roulette_scale": (
        ctypes.c_int,
        [ctypes.c_void_p, _F64P, ctypes.c_size_t, ctypes.c_char_p, ctypes.c_size_t],
    ),
    "monki_cuda_importance": (
        ctypes.c_int,
        [ctypes.c_void_p, _F64P, ctypes.c_size_t, ctypes.c_int, ctypes.c_char_p, ctypes.c_size_t],
    ),
    "monki_cuda_set_importance_weights": (
        ctypes.c_int,
        [ctypes.c_void_p, _F64P, ctypes.c_size_t, ctypes.c_char_p, ctypes.c_size_t],
    ),
    "monki_cuda_run_accumulate": (
        ctypes.c_int,
        [ctypes.c_void_p, _U32P, ctypes.c_double, _F64P, ctypes.c_char_p, ctypes.c_size_t],
    ),
    "monki_cuda_run_held": (ctypes.c_int, [ctypes.c_void_p, _U32P, ctypes.c_char_p, ctypes.c_size_t]),
    "monki_cuda_fold_next": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double, _F64P, ctypes.c_char_p, ctypes.c_size_t]),
    "monki_cuda_statistics_count": (ctypes.c_size_t, [ctypes.c_void_p]),
    "monki_cuda_statistics": (
        ctypes.c_int,
        [ctypes.c_void_p, _F64P, ctypes.c_size_t, _U64P, ctypes.c_char_p, ctypes.c_size_t],
    ),
    "monki_cuda_reset_statistics": (ctypes.c_int, [ctypes.c_void_p]),
    "monki_mlp_param_count": (ctypes.c_size_t, []),
    "monki_mlp_create": (
        ctypes.c_void_p,
        [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_char_p, ctypes.c_size_t],
    ),
    "monki_mlp_set_params": (ctypes.c_int, [ctypes.c_void_p, _F32P, ctypes.c_size_t, ctypes.c_char_p, ctypes.c_size_t]),
    "monki_mlp_get_params": (ctypes.c_int, [ctypes.c_void_p, _F32P, ctypes.c_size_t, ctypes.c_char_p, ctypes.c_size_t]),
    "monki_mlp_forward": (ctypes.c_int, [ctypes.c_void_p, _F32P, ctypes.c_uint32, _F32P, ctypes.c_char_p, ctypes.c_size_t]),
    "monki_mlp_gradients": (
        ctypes.c_int,
        [ctypes.c_void_p, _F32P, _F32P, _F32P, ctypes.c_uint32, _F32P, _F32P, ctypes.c_char_p, ctypes.c_size_t],
    ),
    "monki_mlp_set_data": (
        ctypes.c_int,
        [ctypes.c_void_p, _F32P, _F32P, _F32P, ctypes.c_uint32, ctypes.c_char_p, ctypes.c_size_t],
    ),
    "monki_mlp_train": (
        ctypes.c_int,
        [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_float, _F32P, ctypes.c_char_p, ctypes.c_size_t],
    ),
    "monki_mlp_close": (None, [ctypes.c_void_p]),
    "monki_mlp_gemm_probe": (
        ctypes.c_int,
        [ctypes.c_uint32, ctypes.POINTER(ctypes.c_uint16), ctypes.POINTER(ctypes.c_uint16), ctypes.c_int, ctypes.c_int,
         ctypes.c_int, ctypes.c_int, _F32P, ctypes.c_char_p, ctypes.c_size_t],
    ),
    "monki_cuda_run_static": (
        ctypes.c_int,
        [ctypes.c_uint32, _F64P, ctypes.c_size_t, _U32P, _F64P, ctypes.c_char_p, ctypes.c_size_t],
    ),
    "monki_cuda_multi_create": (
        ctypes.c_void_p,
        [ctypes.c_uint32, ctypes.c_uint32, ctypes.POINTER(_F64P), ctypes.POINTER(ctypes.c_size_t), ctypes.c_uint32,
         ctypes.c_char_p, ctypes.c_char_p, ctypes.c_size_t],
    ),
    "monki_cuda_multi_tally_count": (ctypes.c_size_t, [ctypes.c_void_p, ctypes.c_uint32]),
    "monki_cuda_multi_run": (
        ctypes.c_int,
        [ctypes.c_void_p, _U32P, ctypes.POINTER(_F64P), ctypes.c_char_p, ctypes.c_size_t],
    ),
    "monki_cuda_multi_counters": (ctypes.c_int, [ctypes.c_void_p, _U64P]),
    "monki_cuda_multi_scene_counters": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint32, _U64P]),
    "monki_cuda_multi_last_timing": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_float)]),
    "monki_cuda_multi_close": (None, [ctypes.c_void_p]),
    "monki_cuda_probe_philox": (
        ctypes.c_int,
        [ctypes.c_uint32, _U32P, _U32P, ctypes.c_uint32, _U32P, ctypes.c_char_p, ctypes.c_size_t],
    ),
    "monki_cuda_probe_uniforms": (
        ctypes.c_int,
        [ctypes.c_uint32] * 5 + [_F32P, ctypes.c_char_p, ctypes.c_size_t],
    ),
    "monki_cuda_probe_scatter_stokes": (
        ctypes.c_int,
        [ctypes.c_uint32, ctypes.c_int, ctypes.c_double, _F64P, _F64P, ctypes.c_uint32, _F64P, ctypes.c_char_p, ctypes.c_size_t],
    ),
}

EXPORTS = tuple(_SIGNATURES)


def load(path: Path | str = LIBRARY) -> ctypes.CDLL:
    """Load the library and bind every exported signature; raise if it is missing or stale."""

    path = Path(path)

    if not path.is_file():
        raise FileNotFoundError(
            f"CUDA transport library not built: {path} (run __graft_entry__.build() or "
            "python monki-gpu_gb300/build_native.py)"
        )

    native = ctypes.CDLL(str(path))
    version = getattr(native, "monki_cuda_abi_version", None)

    if version is None or version() != ABI_VERSION:
        raise RuntimeError("Rebuild the CUDA transport library: ABI version mismatch")

    for name, (restype, argtypes) in _SIGNATURES.items():
        function = getattr(native, name)
        function.restype = restype
        function.argtypes = argtypes

    return native


def as_pointer(array, kind):
    return array.ctypes.data_as(kind)


U32P, U64P, F64P, F32P = _U32P, _U64P, _F64P, _F32P
