"""ctypes binding of libblaze103 (the C ABI in include/blaze_prelim.h)."""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libblaze103.so")

# The exported entry points and their C signatures (kept in step with
# include/blaze_prelim.h; tests check the two agree).
EXPORTS = (
    "blaze_status_string", "blaze_last_cuda_error", "blaze_device_count", "blaze_db_create", "blaze_db_free",
    "blaze_db_info", "blaze_query_create", "blaze_query_free", "blaze_params_default",
    "blaze_search_create", "blaze_search_free", "blaze_search_run", "blaze_search_results",
    "blaze_search_stats", "blaze_search_init_hits", "blaze_prelim_search",
    "blaze_batch_create", "blaze_batch_free", "blaze_batch_info", "blaze_search_run_batch",
    "blaze_search_batch_results", "blaze_search_set_tuning",
    "blaze_server_create", "blaze_server_submit", "blaze_server_wait", "blaze_server_take",
    "blaze_server_stats_get", "blaze_server_free", "blaze_volume_info", "blaze_volume_read", "blaze_db_open",
    "blaze_search_traceback", "blaze_search_traceback_results", "blaze_search_traceback_batch",
    "blaze_search_traceback_batch_results", "blaze_db_create_from_source",
)

HSP_DTYPE = np.dtype([
    ("oid", "<u4"), ("score", "<i4"), ("q_start", "<i4"), ("q_end", "<i4"),
    ("s_start", "<i4"), ("s_end", "<i4"), ("q_gapped_start", "<i4"), ("s_gapped_start", "<i4"),
    ("evalue", "<f8"),
])
assert HSP_DTYPE.itemsize == 40
BATCH_HSP_DTYPE = np.dtype([("query", "<u4"), ("reserved", "<u4")] + [
    (n, HSP_DTYPE.fields[n][0]) for n in HSP_DTYPE.names])
assert BATCH_HSP_DTYPE.itemsize == 48
ALIGNED_DTYPE = np.dtype([
    ("oid", "<u4"), ("score", "<i4"), ("q_start", "<i4"), ("q_end", "<i4"), ("s_start", "<i4"), ("s_end", "<i4"),
    ("length", "<i4"), ("identities", "<i4"), ("positives", "<i4"), ("mismatches", "<i4"),
    ("gap_opens", "<i4"), ("gaps", "<i4"), ("reserved", "<i4"), ("evalue", "<f8"), ("bit_score", "<f8"),
], align=True)
assert ALIGNED_DTYPE.itemsize == 72
BATCH_ALIGNED_DTYPE = np.dtype([("query", "<u4"), ("pad", "<u4")] + [
    (n, ALIGNED_DTYPE.fields[n][0]) for n in ALIGNED_DTYPE.names], align=True)
assert BATCH_ALIGNED_DTYPE.itemsize == 80 and BATCH_ALIGNED_DTYPE.fields["evalue"][1] == 64
INIT_DTYPE = np.dtype([
    ("oid", "<u4"), ("q_start", "<i4"), ("s_start", "<i4"), ("length", "<i4"), ("score", "<i4"),
    ("q_trigger", "<i4"), ("s_trigger", "<i4"),
])


class BlazeParams(ctypes.Structure):
    _fields_ = [
        ("word_threshold", ctypes.c_int32), ("window", ctypes.c_int32),
        ("ungapped_xdrop", ctypes.c_int32), ("ungapped_cutoff", ctypes.c_int32),
        ("gap_open", ctypes.c_int32), ("gap_extend", ctypes.c_int32),
        ("gapped_xdrop", ctypes.c_int32), ("gapped_cutoff", ctypes.c_int32),
        ("lambda_", ctypes.c_double), ("K", ctypes.c_double),
        ("eff_searchsp", ctypes.c_double), ("prelim_evalue", ctypes.c_double),
        ("hitlist_size", ctypes.c_int32), ("max_hsps", ctypes.c_int32),
    ]

    def as_dict(self) -> dict:
        return {(k[:-1] if k.endswith("_") else k): getattr(self, k) for k, _ in self._fields_}


class BlazeTuning(ctypes.Structure):
    _fields_ = [("stage_bytes", ctypes.c_uint32), ("tile_residues", ctypes.c_uint32),
                ("max_warps_per_block", ctypes.c_uint32), ("launch_mode", ctypes.c_uint32),
                ("batch_launch", ctypes.c_uint32)]


class BlazeStats(ctypes.Structure):
    _fields_ = [
        ("residues_scanned", ctypes.c_uint64), ("word_hits", ctypes.c_uint64),
        ("ungapped_extensions", ctypes.c_uint64), ("init_hsps", ctypes.c_uint64),
        ("gapped_extensions", ctypes.c_uint64), ("dp_cells", ctypes.c_uint64),
        ("hsps", ctypes.c_uint64), ("subjects_with_hsps", ctypes.c_uint32),
        ("reruns", ctypes.c_uint32), ("scan_ms", ctypes.c_float), ("gapped_ms", ctypes.c_float),
        ("device_ms", ctypes.c_float), ("kernel_launches", ctypes.c_uint32),
        ("h2d_bytes", ctypes.c_uint64), ("d2h_bytes", ctypes.c_uint64),
        ("graph_replays", ctypes.c_uint32), ("graph_builds", ctypes.c_uint32),
        ("traceback_ms", ctypes.c_float), ("traceback_hsps", ctypes.c_uint32),
        ("traceback_cells", ctypes.c_uint64),
    ]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class BlazeServerConfig(ctypes.Structure):
    _fields_ = [("slots", ctypes.c_uint32), ("max_batch", ctypes.c_uint32),
                ("memory_budget", ctypes.c_uint64), ("batch_window_us", ctypes.c_uint32),
                ("evalue", ctypes.c_double), ("tuning", BlazeTuning)]


class BlazeServerStats(ctypes.Structure):
    _fields_ = [
        ("submitted", ctypes.c_uint64), ("completed", ctypes.c_uint64), ("batches", ctypes.c_uint64),
        ("residues", ctypes.c_uint64), ("latency_p50_ms", ctypes.c_double),
        ("latency_p99_ms", ctypes.c_double), ("latency_max_ms", ctypes.c_double),
        ("busy_s", ctypes.c_double),
    ]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


# Callback types of blaze_seq_source (the BlastSeqSrc-shaped database source).
GET_NUM_SEQS_FN = ctypes.CFUNCTYPE(ctypes.c_int64, ctypes.c_void_p)
GET_SEQUENCE_FN = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_uint32,
                                   ctypes.POINTER(ctypes.POINTER(ctypes.c_uint8)), ctypes.POINTER(ctypes.c_uint32))
RELEASE_SEQUENCE_FN = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.c_uint32)
GET_SEQ_LEN_FN = ctypes.CFUNCTYPE(ctypes.c_int64, ctypes.c_void_p, ctypes.c_uint32)
GET_INT64_FN = ctypes.CFUNCTYPE(ctypes.c_int64, ctypes.c_void_p)


class BlazeSeqSource(ctypes.Structure):
    _fields_ = [
        ("user", ctypes.c_void_p), ("get_num_seqs", GET_NUM_SEQS_FN), ("get_sequence", GET_SEQUENCE_FN),
        ("release_sequence", RELEASE_SEQUENCE_FN), ("get_seq_len", GET_SEQ_LEN_FN),
        ("get_tot_len", GET_INT64_FN), ("get_max_seq_len", GET_INT64_FN), ("iter_next", GET_INT64_FN),
    ]


class BlazeError(RuntimeError):
    def __init__(self, status: int, what: str):
        self.status = status
        detail = ""
        if status == 2:  # BLAZE_ERR_CUDA
            try:
                detail = ": " + load().blaze_last_cuda_error().decode()
            except OSError:
                pass
        super().__init__(f"{what}: {status_string(status)} (status {status}){detail}")


_lib = None


def load(path: str | None = None):
    """Load the library. Raises OSError when it has not been built: there is
    no fallback implementation."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise OSError(f"libblaze103 is not built ({path}); run __graft_entry__.build()")
    L = ctypes.CDLL(path)
    vp, u8p = ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint8)
    u64p = ctypes.POINTER(ctypes.c_uint64)
    i32, u32 = ctypes.c_int32, ctypes.c_uint32
    L.blaze_status_string.argtypes = [ctypes.c_int]
    L.blaze_status_string.restype = ctypes.c_char_p
    L.blaze_last_cuda_error.argtypes = []
    L.blaze_last_cuda_error.restype = ctypes.c_char_p
    L.blaze_device_count.argtypes = [ctypes.POINTER(ctypes.c_int)]
    L.blaze_db_create.argtypes = [ctypes.c_int, u8p, u64p, u32, ctypes.POINTER(vp)]
    L.blaze_db_free.argtypes = [vp]
    L.blaze_db_info.argtypes = [vp, u64p, ctypes.POINTER(u32), ctypes.POINTER(u32)]
    L.blaze_query_create.argtypes = [vp, u8p, i32, i32, ctypes.POINTER(vp)]
    L.blaze_query_free.argtypes = [vp]
    L.blaze_params_default.argtypes = [i32, ctypes.c_uint64, u32, ctypes.c_double,
                                       ctypes.POINTER(BlazeParams)]
    L.blaze_search_create.argtypes = [vp, ctypes.POINTER(vp)]
    L.blaze_search_free.argtypes = [vp]
    L.blaze_search_run.argtypes = [vp, vp, ctypes.POINTER(BlazeParams), u64p]
    L.blaze_search_results.argtypes = [vp, vp, ctypes.c_uint64, u64p]
    L.blaze_search_stats.argtypes = [vp, ctypes.POINTER(BlazeStats)]
    L.blaze_search_init_hits.argtypes = [vp, vp, ctypes.c_uint64, u64p]
    L.blaze_prelim_search.argtypes = [vp, u8p, i32, ctypes.POINTER(BlazeParams), vp,
                                      ctypes.c_uint64, u64p]
    L.blaze_batch_create.argtypes = [vp, u8p, u64p, u32, i32, ctypes.POINTER(vp)]
    L.blaze_batch_free.argtypes = [vp]
    L.blaze_batch_info.argtypes = [vp, ctypes.POINTER(u32), u64p]
    L.blaze_search_run_batch.argtypes = [vp, vp, ctypes.POINTER(BlazeParams), u64p]
    L.blaze_search_batch_results.argtypes = [vp, vp, ctypes.c_uint64, u64p]
    L.blaze_search_set_tuning.argtypes = [vp, ctypes.POINTER(BlazeTuning)]
    L.blaze_server_create.argtypes = [vp, ctypes.POINTER(BlazeServerConfig), ctypes.POINTER(vp)]
    L.blaze_server_submit.argtypes = [vp, u8p, i32, u64p]
    L.blaze_server_wait.argtypes = [vp, ctypes.c_uint64, i32, u64p]
    L.blaze_server_take.argtypes = [vp, ctypes.c_uint64, vp, ctypes.c_uint64, u64p,
                                    ctypes.POINTER(ctypes.c_double)]
    L.blaze_server_stats_get.argtypes = [vp, ctypes.POINTER(BlazeServerStats)]
    L.blaze_server_free.argtypes = [vp]
    L.blaze_volume_info.argtypes = [ctypes.c_char_p, ctypes.POINTER(u32), u64p, ctypes.POINTER(u32)]
    L.blaze_volume_read.argtypes = [ctypes.c_char_p, u8p, ctypes.c_uint64, u64p]
    L.blaze_db_open.argtypes = [ctypes.c_int, ctypes.c_char_p, ctypes.POINTER(vp)]
    L.blaze_search_traceback.argtypes = [vp, vp, ctypes.POINTER(BlazeParams), i32, ctypes.c_double, u64p]
    L.blaze_search_traceback_results.argtypes = [vp, vp, ctypes.c_uint64, u64p]
    L.blaze_search_traceback_batch.argtypes = [vp, vp, ctypes.POINTER(BlazeParams), i32, ctypes.c_double, u64p]
    L.blaze_search_traceback_batch_results.argtypes = [vp, vp, ctypes.c_uint64, u64p]
    L.blaze_db_create_from_source.argtypes = [ctypes.c_int, ctypes.POINTER(BlazeSeqSource), ctypes.POINTER(vp)]
    for name in EXPORTS:
        if name not in ("blaze_status_string", "blaze_last_cuda_error"):
            getattr(L, name).restype = ctypes.c_int
    _lib = L
    return L


def status_string(status: int) -> str:
    try:
        return load().blaze_status_string(int(status)).decode()
    except OSError:
        return "library not loaded"


def check(status: int, what: str) -> None:
    if status != 0:
        raise BlazeError(status, what)


def u8ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))


def u64ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64))
