"""ctypes binding of the C-ABI library ``libjscc_gb300.so`` (see include/jscc_gb300.h).

The library is the only compute path of this package: there is no CPU or
pure-PyTorch fallback. Loading fails loudly when the library has not been built,
and every compute wrapper refuses non-CUDA tensors.
"""
from __future__ import annotations

import ctypes
import threading
from ctypes import POINTER, c_float, c_int, c_int32, c_int64, c_size_t, c_uint, c_ulonglong, c_void_p
from pathlib import Path

import torch

from . import build as _build

JSCC_OK = 0
JSCC_ERR_INVALID = 1
JSCC_ERR_CUDA = 2

DTYPE_F32 = 0
DTYPE_BF16 = 1

EM_PLAIN = 0
EM_SAFE = 1

CONE_STRICT = 0
CONE_LEGACY = 1
CONE_SIMPLE = 2
CONE_RECORD_FLOATS = 16

SPARSE_MATERIALIZE = 0
SPARSE_GROUPED = 1

_lib = None
_lock = threading.Lock()

# name -> (restype, argtypes); every symbol declared in include/jscc_gb300.h
_SIGNATURES: dict[str, tuple] = {
    "jscc_last_error": (ctypes.c_char_p, []),
    "jscc_abi_version": (c_int, []),
    "jscc_launch_count": (c_ulonglong, []),
    "jscc_reset_launch_count": (None, []),
    "jscc_count_graph_launches": (None, [c_ulonglong]),
    "jscc_take_bad_index_count": (c_int, [POINTER(c_uint)]),
    "jscc_kernel_timing_enable": (None, [c_int]),
    "jscc_kernel_timing_collect": (c_int, [ctypes.c_char_p, c_size_t]),
    "jscc_sc_weight_workspace_bytes": (c_size_t, [c_int64, c_int64, c_int32]),
    "jscc_sc_project": (
        c_int,
        [c_void_p, c_int32, c_int64, c_void_p, c_int64, c_int64, c_int32, c_void_p, c_void_p, c_int64, c_void_p,
         c_int64, c_void_p, c_size_t, c_void_p],
    ),
    "jscc_sc_backproject": (
        c_int,
        [c_void_p, c_int32, c_int64, c_void_p, c_int64, c_int64, c_int32, c_void_p, c_int64, c_void_p, c_int64,
         c_float, c_void_p, c_void_p, c_size_t, c_void_p],
    ),
    "jscc_compton_project": (
        c_int,
        [c_void_p, c_void_p, c_int64, c_void_p, c_int64, c_int32, c_int32, c_void_p, c_int32, c_int64, c_void_p,
         c_void_p, c_int64, c_void_p, c_void_p, c_size_t, c_void_p],
    ),
    "jscc_compton_backproject": (
        c_int,
        [c_void_p, c_void_p, c_int64, c_void_p, c_int64, c_int32, c_int32, c_void_p, c_int32, c_int64, c_void_p,
         c_void_p, c_int64, c_float, c_void_p, c_void_p, c_size_t, c_void_p],
    ),
    "jscc_sc_f64_workspace_bytes": (c_size_t, [c_int64, c_int32]),
    "jscc_sc_project_f64": (
        c_int,
        [c_void_p, c_int32, c_int64, c_void_p, c_int64, c_int64, c_int32, c_void_p, c_void_p, c_int64, c_void_p,
         c_int64, c_void_p],
    ),
    "jscc_sc_backproject_f64": (
        c_int,
        [c_void_p, c_int32, c_int64, c_void_p, c_int64, c_int64, c_int32, c_void_p, c_int64, c_void_p, c_int64,
         ctypes.c_double, c_void_p, c_void_p, c_size_t, c_void_p],
    ),
    "jscc_compton_project_f64": (
        c_int,
        [c_void_p, c_void_p, c_int64, c_void_p, c_int64, c_int32, c_void_p, c_int32, c_int64, c_void_p, c_void_p,
         c_void_p],
    ),
    "jscc_compton_backproject_f64": (
        c_int,
        [c_void_p, c_void_p, c_int64, c_void_p, c_int64, c_int32, c_void_p, c_int32, c_int64, c_void_p,
         ctypes.c_double, c_void_p, c_void_p],
    ),
    "jscc_rdp_prior_f64": (
        c_int,
        [c_void_p, c_void_p, c_void_p, c_int64, c_int32, ctypes.c_double, ctypes.c_double, ctypes.c_double,
         c_void_p, c_void_p, c_int32, c_void_p, c_size_t, c_void_p],
    ),
    "jscc_bf16_gemm_workspace_bytes": (c_size_t, [c_int64, c_int32, c_int64, c_int32]),
    "jscc_bf16_gemm_nt": (
        c_int,
        [c_void_p, c_int64, c_void_p, c_int64, c_int64, c_int32, c_int64, c_int32, c_void_p, c_int64, c_void_p,
         c_size_t, c_void_p],
    ),
    "jscc_batch_split": (c_int, [c_void_p, c_int64, c_int32, c_int32, c_int64, c_void_p, c_int64, c_void_p]),
    "jscc_batch_ratio": (
        c_int,
        [c_void_p, c_int64, c_void_p, c_int64, c_int64, c_int64, c_int32, c_int32, c_void_p, c_int64, c_void_p,
         c_int64, c_int32, c_float, c_void_p],
    ),
    "jscc_batch_em_joint": (
        c_int,
        [c_void_p, c_int64, c_int64, c_int32, c_int32, c_float, c_void_p, c_int64, c_float, c_void_p, c_int64,
         c_void_p, c_int64, c_int32, c_float, c_void_p, c_int64, c_void_p],
    ),
    "jscc_batch_weight": (
        c_int, [c_void_p, c_int64, c_int64, c_int32, c_int32, c_float, c_void_p, c_int64, c_int32, c_void_p]),
    "jscc_batch_em": (
        c_int, [c_void_p, c_int64, c_int64, c_int32, c_int32, c_void_p, c_int64, c_void_p, c_void_p, c_int64,
                c_void_p]),
    "jscc_take_gemm_timeout_count": (c_int, [POINTER(c_uint)]),
    "jscc_set_wait_limit": (c_int, [c_int64]),
    "jscc_set_fused_cluster": (c_int, [c_int32]),
    "jscc_rdp_prior_workspace_bytes": (c_size_t, [c_int64]),
    "jscc_rdp_prior": (
        c_int,
        [c_void_p, c_void_p, c_void_p, c_int64, c_int32, c_float, c_float, c_float, c_void_p, c_void_p, c_int32,
         c_void_p, c_size_t, c_void_p],
    ),
    "jscc_sc_sensitivity": (
        c_int,
        [c_void_p, c_int32, c_int64, c_void_p, c_int64, c_int64, c_int32, c_void_p, c_int64, c_void_p, c_void_p,
         c_size_t, c_void_p],
    ),
    "jscc_sc_weight": (
        c_int,
        [c_void_p, c_int32, c_int64, c_void_p, c_int64, c_int64, c_void_p, c_int64, c_int32,
         c_void_p, c_void_p, c_void_p, c_int64, c_int32, c_float, c_float, c_void_p, c_void_p,
         c_size_t, c_void_p],
    ),
    "jscc_sc_weight_noalloc": (
        c_int,
        [c_void_p, c_int32, c_int64, c_void_p, c_int64, c_int64, c_void_p, c_int64, c_int32,
         c_void_p, c_void_p, c_void_p, c_int64, c_int32, c_float, c_float, c_void_p, c_void_p],
    ),
    "jscc_compton_event_prep": (
        c_int,
        [c_void_p, c_int64, c_int64, c_void_p, c_void_p, c_void_p, c_int64, c_float, c_float, c_float, c_float,
         c_float, c_int32, c_int32, c_float, c_float, c_float, c_void_p, c_void_p, c_void_p, c_void_p],
    ),
    "jscc_compton_cone_rows": (
        c_int,
        [c_void_p, c_void_p, c_int64, c_void_p, c_int64, c_int32, c_void_p, c_int32, c_int64, c_void_p, c_void_p,
         c_void_p],
    ),
    "jscc_compton_row_stats": (
        c_int,
        [c_void_p, c_void_p, c_int64, c_void_p, c_int64, c_int32, c_int32, c_void_p, c_int32, c_int64, c_void_p,
         c_void_p, c_void_p, c_void_p],
    ),
    "jscc_compton_weight_workspace_bytes": (c_size_t, [c_int64, c_int64]),
    "jscc_compton_weight": (
        c_int,
        [c_void_p, c_void_p, c_int64, c_void_p, c_int64, c_int32, c_int32, c_void_p, c_int32, c_int64, c_void_p,
         c_void_p, c_void_p, c_int64, c_float, c_void_p, c_void_p, c_size_t, c_void_p],
    ),
    "jscc_take_bad_detector_count": (c_int, [POINTER(c_uint)]),
    "jscc_compton_batch_workspace_bytes": (c_size_t, [c_int64, c_int64, c_int64]),
    "jscc_compton_weight_batched": (
        c_int,
        [c_void_p, c_void_p, c_int64, c_void_p, c_void_p, c_void_p, c_void_p, c_int64, c_int32, c_void_p, c_int64,
         c_void_p, c_int32, c_int64, c_void_p, c_int64, c_float, c_void_p, c_int64, c_void_p, c_size_t, c_void_p],
    ),
    "jscc_take_wait_timeout_count": (c_int, [POINTER(c_uint)]),
    "jscc_sparse_map": (
        c_int,
        [c_void_p, c_int32, c_int64, c_void_p, c_int64, c_void_p, c_int64, c_void_p, c_void_p, c_void_p, c_int32,
         c_int32, c_void_p, c_void_p, c_void_p, c_int32, c_int32, c_void_p],
    ),
    "jscc_sparse_pack": (c_int, [c_void_p, c_void_p, c_int64, c_int64, c_int64, c_void_p, c_int64, c_void_p]),
    "jscc_sparse_unpack_ids": (c_int, [c_void_p, c_int64, c_int64, c_void_p, c_void_p]),
    "jscc_sparse_materialize": (
        c_int,
        [c_void_p, c_int64, c_int64, c_void_p, c_int32, c_int64, c_int64, c_void_p, c_void_p, c_int32, c_void_p,
         c_void_p, c_int32, c_int32, c_void_p, c_int64, c_void_p, c_void_p],
    ),
    "jscc_sparse_weight_workspace_bytes": (c_size_t, [c_int64, c_int64]),
    "jscc_sparse_weight": (
        c_int,
        [c_void_p, c_int64, c_int64, c_void_p, c_int32, c_int64, c_int64, c_void_p, c_void_p, c_int32, c_void_p,
         c_void_p, c_int32, c_int32, c_int32, c_void_p, c_void_p, c_void_p, c_int64, c_float, c_void_p, c_void_p,
         c_size_t, c_void_p],
    ),
    "jscc_sparse_weight_split": (
        c_int,
        [c_void_p, c_void_p, c_int32, c_int64, c_int64, c_void_p, c_int32, c_int64, c_int64, c_void_p, c_void_p,
         c_int32, c_void_p, c_void_p, c_int32, c_int32, c_int32, c_void_p, c_void_p, c_void_p, c_int64, c_float,
         c_void_p, c_void_p, c_size_t, c_void_p],
    ),
    "jscc_sparse_grouped_workspace_bytes": (c_size_t, [c_int64, c_int64, c_int64, c_int32, c_int32]),
    "jscc_sparse_weight_grouped": (
        c_int,
        [c_void_p, c_void_p, c_int32, c_int64, c_void_p, c_int64, c_void_p, c_void_p, c_void_p, c_int32, c_void_p,
         c_int32, c_void_p, c_int32, c_int64, c_int64, c_void_p, c_void_p, c_int32, c_void_p, c_void_p, c_int32,
         c_int32, c_int32, c_void_p, c_void_p, c_int32, c_int32, c_int32, c_int32, c_void_p, c_void_p, c_void_p,
         c_int64, c_float, c_void_p, c_void_p, c_size_t, c_void_p],
    ),
    "jscc_em_update": (
        c_int,
        [c_void_p, c_void_p, c_void_p, c_int32, c_float, c_void_p, c_float, c_void_p, c_int64,
         c_int32, c_float, c_void_p],
    ),
}


def library_path() -> Path:
    return _build.LIB_PATH


def load(build_if_missing: bool = False):
    """Return the loaded library (building it first only when asked)."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = library_path()
        if build_if_missing and _build.is_stale():
            _build.build()
        if not path.exists():
            raise RuntimeError(
                f"JSCC CUDA library not built ({path} missing). "
                "Run `python -c 'import __graft_entry__ as g; g.build()'` first."
            )
        lib = ctypes.CDLL(str(path))
        for name, (restype, argtypes) in _SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = restype
            fn.argtypes = argtypes
        _lib = lib
    return _lib


def check(rc: int, what: str) -> None:
    if rc == JSCC_OK:
        return
    msg = load().jscc_last_error().decode(errors="replace")
    if rc == JSCC_ERR_INVALID:
        raise ValueError(f"{what}: {msg}")
    raise RuntimeError(f"{what}: {msg}")


def launch_count() -> int:
    return int(load().jscc_launch_count())


def reset_launch_count() -> None:
    load().jscc_reset_launch_count()


def take_bad_detector_count() -> int:
    out = c_uint(0)
    check(load().jscc_take_bad_detector_count(ctypes.byref(out)), "jscc_take_bad_detector_count")
    return int(out.value)


def take_wait_timeout_count() -> int:
    """Bounded device waits (bulk-copy pipeline) that gave up since the last call."""
    out = ctypes.c_uint(0)
    check(load().jscc_take_wait_timeout_count(ctypes.byref(out)), "jscc_take_wait_timeout_count")
    return int(out.value)


def take_gemm_timeout_count() -> int:
    """Tensor-core GEMM waits that gave up since the last call."""
    out = c_uint(0)
    check(load().jscc_take_gemm_timeout_count(ctypes.byref(out)), "jscc_take_gemm_timeout_count")
    return int(out.value)


def set_wait_limit(polls: int | None) -> None:
    """Poll bound of every bounded pipeline wait (bulk sparse kernels and tensor-core GEMM)
    on the current device; None restores the default. 0 makes each wait give up at once:
    the give-up path then runs while every copy still completes."""
    check(load().jscc_set_wait_limit(-1 if polls is None else int(polls)), "jscc_set_wait_limit")


# Bumped whenever a give-up is detected: per-plan event sums computed before it may come from
# a call whose waits gave up, so ops keys its cached sums by this epoch.
timeout_epoch = 0


def set_fused_cluster(enable: bool) -> None:
    """Let the grouped sparse weight use its fused cluster kernel where it applies, or (the
    default) the separate adjoint, coefficient and scatter kernels."""
    check(load().jscc_set_fused_cluster(1 if enable else 0), "jscc_set_fused_cluster")


def check_wait_timeouts() -> None:
    """Raise RuntimeError when a bounded device wait gave up since the last check (the
    results of the calls made meanwhile are then invalid, and cached per-plan event sums are
    dropped); resets both counters."""
    global timeout_epoch
    bulk, gemm = take_wait_timeout_count(), take_gemm_timeout_count()
    if bulk or gemm:
        timeout_epoch += 1
        raise RuntimeError(f"device pipeline waits gave up: {bulk} in the bulk-copy kernels (grouped sparse "
                           f"weight, fused SC weight), {gemm} in the tensor-core GEMM; the results computed since "
                           "the last check are invalid")


def take_bad_index_count() -> int:
    out = c_uint(0)
    check(load().jscc_take_bad_index_count(ctypes.byref(out)), "jscc_take_bad_index_count")
    return int(out.value)


def kernel_timing_enable(on: bool) -> None:
    load().jscc_kernel_timing_enable(1 if on else 0)


def kernel_timing_collect() -> dict[str, tuple[int, float]]:
    """{kernel name: (launches, total ms)} since timing was enabled / last collect."""
    buf = ctypes.create_string_buffer(1 << 16)
    check(load().jscc_kernel_timing_collect(buf, len(buf)), "jscc_kernel_timing_collect")
    out = {}
    for line in buf.value.decode().splitlines():
        name, n, ms = line.split()
        out[name] = (int(n), float(ms))
    return out


# ------------------------------------------------------------------ tensor helpers
def ptr(t: torch.Tensor | None) -> int | None:
    return None if t is None else t.data_ptr()


def require_cuda(*tensors: torch.Tensor | None, what: str) -> torch.device:
    dev = None
    for t in tensors:
        if t is None:
            continue
        if not t.is_cuda:
            raise RuntimeError(
                f"{what}: the GB300 path runs on CUDA tensors only (got a {t.device} tensor); "
                "there is no CPU fallback"
            )
        if dev is None:
            dev = t.device
        elif t.device != dev:
            raise ValueError(f"{what}: tensors are on different devices ({dev} vs {t.device})")
    if dev is None:
        raise ValueError(f"{what}: no tensor arguments")
    return dev


def stream_handle(device: torch.device) -> int:
    return torch.cuda.current_stream(device).cuda_stream


class _Workspace:
    """Grow-only scratch buffers, one per (device, stream)."""

    def __init__(self) -> None:
        self._bufs: dict[tuple[int, int], torch.Tensor] = {}

    def get(self, device: torch.device, nbytes: int) -> torch.Tensor:
        key = (device.index if device.index is not None else torch.cuda.current_device(),
               stream_handle(device))
        buf = self._bufs.get(key)
        if buf is None or buf.numel() < nbytes:
            buf = torch.empty(max(nbytes, 256), dtype=torch.uint8, device=device)
            self._bufs[key] = buf
        return buf

    def clear(self) -> None:
        self._bufs.clear()


workspace = _Workspace()
