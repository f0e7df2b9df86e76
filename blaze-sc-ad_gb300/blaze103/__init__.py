"""blaze103 -- Python host side of the GB300 BLASTP preliminary search stage.

Mirrors the reference's interface for this path (181charan/BLAZE-SC-ad):

* ``SeqSrc`` plays the part of NCBI's ``BlastSeqSrc`` database source
  (BLAZE_ncbi/blast_seqsrc.c:45-134) with its getters ``num_seqs``,
  ``tot_len``, ``max_seq_len``, ``avg_seq_len``; the residues live in device
  memory, length-sorted, for the life of the object.
* ``PrelimSearch.run`` stands where ``Blast_RunPreliminarySearchWithInterruptMT``
  calls ``BLAZE_GPU`` and then re-searches the survivors on the CPU
  (BLAZE_ncbi/blast_engine.c:2962-3006); here the GPU returns every subject's
  finished HSP list (``HSPResults.hsp_lists()`` ~ the ``BlastHSPList`` objects
  written to the HSP stream at blast_engine.c:2499).
* ``default_params`` computes the cutoffs that blast_engine.c:2971-2981 takes
  from NCBI's word and hit-saving parameters.

All compute goes through libblaze103 (CUDA, sm_103a). There is no CPU
fallback: without the built library or a GPU every call raises.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass

import numpy as np

from ._lib import (ALIGNED_DTYPE, BATCH_ALIGNED_DTYPE, BATCH_HSP_DTYPE, HSP_DTYPE, INIT_DTYPE, BlazeError, BlazeParams, BlazeServerConfig,
                   BlazeServerStats, BlazeStats, BlazeTuning, check, load, u8ptr, u64ptr, status_string)

__all__ = ["SeqSrc", "PrelimSearch", "HSPResults", "QueryBatch", "Server", "BlazeParams", "BlazeTuning",
           "BlazeError", "HSP_DTYPE", "BATCH_HSP_DTYPE", "ALIGNED_DTYPE", "BATCH_ALIGNED_DTYPE", "default_params", "device_count", "load",
           "status_string"]


def device_count() -> int:
    n = ctypes.c_int(0)
    check(load().blaze_device_count(ctypes.byref(n)), "blaze_device_count")
    return n.value


def _codes(a, what: str) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.uint8)
    if a.size and (a.min() == 0 or a.max() >= 28):
        raise ValueError(f"{what}: residues must be NCBIstdaa codes 1..27")
    return a


class SeqSrc:
    """Device-resident residue database (NCBI BlastSeqSrc analog)."""

    def __init__(self, residues, offsets, device: int = 0):
        self._lib = load()
        res = _codes(residues, "database")
        off = np.ascontiguousarray(offsets, dtype=np.uint64)
        if off.ndim != 1 or off.size < 1:
            raise ValueError("offsets must be a 1-D array of n_subjects + 1 entries")
        h = ctypes.c_void_p()
        check(self._lib.blaze_db_create(int(device), u8ptr(res), u64ptr(off), off.size - 1,
                                        ctypes.byref(h)), "blaze_db_create")
        self._adopt(h, device)

    @classmethod
    def open(cls, path: str, device: int = 0) -> "SeqSrc":
        """An NCBI BLAST protein database volume (<path>.pin + <path>.psq)
        loaded straight into the resident database (blaze_db_open)."""
        self = cls.__new__(cls)
        self._lib = load()
        h = ctypes.c_void_p()
        check(self._lib.blaze_db_open(int(device), os.fsencode(path), ctypes.byref(h)), "blaze_db_open")
        self._adopt(h, device)
        return self

    @classmethod
    def from_source(cls, source, device: int = 0) -> "SeqSrc":
        """The resident database read from a BlastSeqSrc-shaped source
        (blaze_db_create_from_source). `source` provides ``num_seqs()`` and
        ``get_sequence(oid)`` (NCBIstdaa codes as a uint8 array), and may
        provide ``seq_len(oid)``, ``release_sequence(oid)``, ``tot_len()``,
        ``max_seq_len()`` and ``iter_next()`` (the next OID, negative at the
        end) -- the accessors of NCBI's BlastSeqSrc
        (BLAZE_ncbi/blast_seqsrc.c:91-130)."""
        from ._lib import (GET_INT64_FN, GET_NUM_SEQS_FN, GET_SEQ_LEN_FN, GET_SEQUENCE_FN, RELEASE_SEQUENCE_FN,
                           BlazeSeqSource)

        held = {}  # oid -> array kept alive until its release

        def get_sequence(_u, oid, res_out, len_out):
            try:
                a = np.ascontiguousarray(source.get_sequence(int(oid)), dtype=np.uint8)
            except Exception:
                return 1
            held[int(oid)] = a
            res_out[0] = a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))
            len_out[0] = a.size
            return 0

        def release(_u, oid):
            held.pop(int(oid), None)
            if hasattr(source, "release_sequence"):
                source.release_sequence(int(oid))

        def opt(name, ftype, fn):
            return ftype(fn) if hasattr(source, name) else ctypes.cast(None, ftype)

        cbs = BlazeSeqSource(
            None, GET_NUM_SEQS_FN(lambda _u: int(source.num_seqs())), GET_SEQUENCE_FN(get_sequence),
            RELEASE_SEQUENCE_FN(release),
            opt("seq_len", GET_SEQ_LEN_FN, lambda _u, oid: int(source.seq_len(int(oid)))),
            opt("tot_len", GET_INT64_FN, lambda _u: int(source.tot_len())),
            opt("max_seq_len", GET_INT64_FN, lambda _u: int(source.max_seq_len())),
            opt("iter_next", GET_INT64_FN, lambda _u: int(source.iter_next())))
        self = cls.__new__(cls)
        self._lib = load()
        h = ctypes.c_void_p()
        check(self._lib.blaze_db_create_from_source(int(device), ctypes.byref(cbs), ctypes.byref(h)),
              "blaze_db_create_from_source")
        self._adopt(h, device)
        return self

    def _adopt(self, h, device):
        self._h = h
        self.device = device
        tot, n, mx = ctypes.c_uint64(), ctypes.c_uint32(), ctypes.c_uint32()
        check(self._lib.blaze_db_info(h, ctypes.byref(tot), ctypes.byref(n), ctypes.byref(mx)),
              "blaze_db_info")
        self.tot_len, self.num_seqs, self.max_seq_len = tot.value, n.value, mx.value

    @property
    def avg_seq_len(self) -> int:
        return self.tot_len // max(self.num_seqs, 1)

    @property
    def handle(self):
        return self._h

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.blaze_db_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def default_params(query_length: int, seq_src: SeqSrc | None = None, evalue: float = 10.0, *,
                   db_residues: int | None = None, db_subjects: int | None = None) -> BlazeParams:
    """NCBI blastp defaults (BLOSUM62, gaps 11/1, word 3, T 11, window 40)."""
    if seq_src is not None:
        db_residues, db_subjects = seq_src.tot_len, seq_src.num_seqs
    p = BlazeParams()
    check(load().blaze_params_default(int(query_length), int(db_residues), int(db_subjects),
                                      float(evalue), ctypes.byref(p)), "blaze_params_default")
    return p


@dataclass
class HSPResults:
    hsps: np.ndarray  # HSP_DTYPE records grouped by OID, NCBI order within a subject
    stats: dict

    def hsp_lists(self) -> dict[int, np.ndarray]:
        """OID -> that subject's HSP records (the BlastHSPList analog)."""
        out: dict[int, np.ndarray] = {}
        if self.hsps.size == 0:
            return out
        oids = self.hsps["oid"]
        cut = np.flatnonzero(np.diff(oids)) + 1
        for chunk in np.split(self.hsps, cut):
            out[int(chunk["oid"][0])] = chunk
        return out


class Query:
    """A query's residues and word lookup resident on the device."""

    def __init__(self, seq_src: SeqSrc, query, word_threshold: int = 11):
        self._lib = load()
        q = _codes(query, "query")
        h = ctypes.c_void_p()
        check(self._lib.blaze_query_create(seq_src.handle, u8ptr(q), len(q), int(word_threshold),
                                           ctypes.byref(h)), "blaze_query_create")
        self._h = h
        self.length = len(q)

    @property
    def handle(self):
        return self._h

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.blaze_query_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class QueryBatch:
    """Many queries resident on the device for one batched launch."""

    def __init__(self, seq_src: SeqSrc, queries, word_threshold: int = 11):
        self._lib = load()
        qs = [_codes(q, "query") for q in queries]
        if not qs:
            raise ValueError("empty batch")
        off = np.zeros(len(qs) + 1, dtype=np.uint64)
        off[1:] = np.cumsum([len(q) for q in qs])
        res = np.concatenate(qs)
        h = ctypes.c_void_p()
        check(self._lib.blaze_batch_create(seq_src.handle, u8ptr(res), u64ptr(off), len(qs),
                                           int(word_threshold), ctypes.byref(h)), "blaze_batch_create")
        self._h = h
        self.lengths = [len(q) for q in qs]
        n, b = ctypes.c_uint32(), ctypes.c_uint64()
        check(self._lib.blaze_batch_info(h, ctypes.byref(n), ctypes.byref(b)), "blaze_batch_info")
        self.device_bytes = b.value

    def __len__(self):
        return len(self.lengths)

    @property
    def handle(self):
        return self._h

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.blaze_batch_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class PrelimSearch:
    """Runs the preliminary search stage against one SeqSrc (one CUDA stream)."""

    def __init__(self, seq_src: SeqSrc, autotune: bool = True):
        """autotune: batched runs take their launch shape from the committed
        autotuner table (blaze103/tuning.json, nearest shape) until
        ``set_tuning`` is called."""
        self._lib = load()
        self.seq_src = seq_src
        self._auto = autotune
        self._applied = None
        h = ctypes.c_void_p()
        check(self._lib.blaze_search_create(seq_src.handle, ctypes.byref(h)), "blaze_search_create")
        self._h = h

    def run_query(self, query: Query, params: BlazeParams) -> int:
        n = ctypes.c_uint64()
        check(self._lib.blaze_search_run(self._h, query.handle, ctypes.byref(params),
                                         ctypes.byref(n)), "blaze_search_run")
        return n.value

    def results(self) -> np.ndarray:
        n = ctypes.c_uint64()
        self._lib.blaze_search_results(self._h, None, 0, ctypes.byref(n))
        out = np.zeros(n.value, dtype=HSP_DTYPE)
        check(self._lib.blaze_search_results(self._h, out.ctypes.data_as(ctypes.c_void_p),
                                             n.value, ctypes.byref(n)), "blaze_search_results")
        return out

    def init_hits(self) -> np.ndarray:
        """Init hits of the last run (diagnostics), INIT_DTYPE records."""
        n = ctypes.c_uint64()
        self._lib.blaze_search_init_hits(self._h, None, 0, ctypes.byref(n))
        out = np.zeros(n.value, dtype=INIT_DTYPE)
        check(self._lib.blaze_search_init_hits(self._h, out.ctypes.data_as(ctypes.c_void_p),
                                               n.value, ctypes.byref(n)), "blaze_search_init_hits")
        return out

    def stats(self) -> dict:
        st = BlazeStats()
        check(self._lib.blaze_search_stats(self._h, ctypes.byref(st)), "blaze_search_stats")
        return st.as_dict()

    def run(self, query, params: BlazeParams | None = None, evalue: float = 10.0) -> HSPResults:
        q = Query(self.seq_src, query, params.word_threshold if params else 11)
        try:
            if params is None:
                params = default_params(q.length, self.seq_src, evalue)
            self.run_query(q, params)
            return HSPResults(self.results(), self.stats())
        finally:
            q.close()

    def set_tuning(self, stage_bytes: int = 0, tile_residues: int = 0, max_warps_per_block: int = 0,
                   launch_mode: int = 0, batch_launch: int = 0):
        """Launch shape (0 = library default for each); launch_mode 0: CUDA
        graph for batched runs, 1: direct launches, 2: CUDA graph always;
        batch_launch 0: by database size, 1: tiles of many queries per
        launch, 2: one scan launch per query."""
        self._auto = False
        self._set_tuning(stage_bytes, tile_residues, max_warps_per_block, launch_mode, batch_launch)

    def _set_tuning(self, stage_bytes=0, tile_residues=0, max_warps_per_block=0, launch_mode=0, batch_launch=0):
        t = BlazeTuning(int(stage_bytes), int(tile_residues), int(max_warps_per_block), int(launch_mode),
                        int(batch_launch))
        check(self._lib.blaze_search_set_tuning(self._h, ctypes.byref(t)), "blaze_search_set_tuning")

    @property
    def tuning(self) -> dict | None:
        """The autotuned launch shape applied to the last batched run, if any."""
        return self._applied

    def run_batch(self, batch: QueryBatch, params=None, evalue: float = 10.0) -> np.ndarray:
        """Every query of the batch in one batched launch; returns
        BATCH_HSP_DTYPE records grouped by query, then OID."""
        if params is None:
            params = [default_params(L, self.seq_src, evalue) for L in batch.lengths]
        if self._auto:
            from .autotune import lookup

            t = lookup("batched", len(batch), float(np.median(batch.lengths)), self.seq_src.tot_len)
            if t and t != self._applied:
                self._set_tuning(**t)
                self._applied = t
        arr = (BlazeParams * len(params))(*params)
        n = ctypes.c_uint64()
        check(self._lib.blaze_search_run_batch(self._h, batch.handle, arr, ctypes.byref(n)),
              "blaze_search_run_batch")
        out = np.zeros(n.value, dtype=BATCH_HSP_DTYPE)
        check(self._lib.blaze_search_batch_results(self._h, out.ctypes.data_as(ctypes.c_void_p),
                                                   n.value, ctypes.byref(n)),
              "blaze_search_batch_results")
        return out

    def traceback(self, query, params: BlazeParams, evalue: float | None = None,
                  final_xdrop: int = 64) -> np.ndarray:
        """Traceback stage over the last single-query run (which must have
        searched `query` with `params`): ALIGNED_DTYPE records by OID, then
        the final per-subject order, reaped at `evalue` (default: the
        preliminary E-value)."""
        q = Query(self.seq_src, query, params.word_threshold)
        try:
            n = ctypes.c_uint64()
            ev = params.prelim_evalue if evalue is None else float(evalue)
            check(self._lib.blaze_search_traceback(self._h, q.handle, ctypes.byref(params), int(final_xdrop), ev,
                                                   ctypes.byref(n)), "blaze_search_traceback")
            out = np.zeros(n.value, dtype=ALIGNED_DTYPE)
            check(self._lib.blaze_search_traceback_results(self._h, out.ctypes.data_as(ctypes.c_void_p), n.value,
                                                           ctypes.byref(n)), "blaze_search_traceback_results")
            return out[: n.value]
        finally:
            q.close()

    def traceback_batch(self, batch: QueryBatch, params, evalue: float | None = None,
                        final_xdrop: int = 64) -> np.ndarray:
        """Traceback stage over the last batched run (which must have searched
        `batch` with `params`): BATCH_ALIGNED_DTYPE records by query, then OID."""
        arr = (BlazeParams * len(params))(*params)
        ev = params[0].prelim_evalue if evalue is None else float(evalue)
        n = ctypes.c_uint64()
        check(self._lib.blaze_search_traceback_batch(self._h, batch.handle, arr, int(final_xdrop), ev,
                                                     ctypes.byref(n)), "blaze_search_traceback_batch")
        out = np.zeros(n.value, dtype=BATCH_ALIGNED_DTYPE)
        check(self._lib.blaze_search_traceback_batch_results(self._h, out.ctypes.data_as(ctypes.c_void_p), n.value,
                                                             ctypes.byref(n)), "blaze_search_traceback_batch_results")
        return out[: n.value]

    def prelim_search(self, query, params: BlazeParams, capacity: int) -> np.ndarray:
        """The one-call C-ABI path with host buffers (blaze_prelim_search)."""
        q = _codes(query, "query")
        out = np.zeros(capacity, dtype=HSP_DTYPE)
        n = ctypes.c_uint64()
        check(self._lib.blaze_prelim_search(self._h, u8ptr(q), len(q), ctypes.byref(params),
                                            out.ctypes.data_as(ctypes.c_void_p), capacity,
                                            ctypes.byref(n)), "blaze_prelim_search")
        return out[: n.value]

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.blaze_search_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Serving loop over a resident database (``blaze_server_*``): queries are
    submitted as they arrive and run in continuously formed batches, ``slots``
    batches in flight at once, admitted under ``memory_budget`` device bytes.
    Each query's result is exactly what ``PrelimSearch.run`` returns for it
    alone with ``default_params(len(query), seq_src, evalue)``."""

    def __init__(self, seq_src: SeqSrc, slots: int = 2, max_batch: int = 64, memory_budget: int = 0,
                 batch_window_us: int = 200, evalue: float = 10.0, tuning: dict | None = None):
        """tuning: launch shape of the workers' searches (BlazeTuning fields);
        None takes the autotuner's entry for batches of max_batch queries."""
        self._lib = load()
        self._src = seq_src
        if tuning is None:
            from .autotune import lookup

            tuning = lookup("batched", max_batch, 350.0, seq_src.tot_len) or {}
        self.tuning = dict(tuning)
        cfg = BlazeServerConfig(slots, max_batch, memory_budget, batch_window_us, evalue,
                                BlazeTuning(*(int(tuning.get(k, 0)) for k, _ in BlazeTuning._fields_)))
        h = ctypes.c_void_p()
        check(self._lib.blaze_server_create(seq_src.handle, ctypes.byref(cfg), ctypes.byref(h)),
              "blaze_server_create")
        self._h = h

    def submit(self, query) -> int:
        q = _codes(query, "query")
        t = ctypes.c_uint64()
        check(self._lib.blaze_server_submit(self._h, u8ptr(q), q.size, ctypes.byref(t)), "blaze_server_submit")
        return t.value

    def wait(self, ticket: int, timeout_ms: int = -1) -> np.ndarray:
        """Blocks until the ticket completed; returns its HSPs (grouped by OID)."""
        n = ctypes.c_uint64()
        check(self._lib.blaze_server_wait(self._h, ticket, timeout_ms, ctypes.byref(n)), "blaze_server_wait")
        out = np.empty(n.value, dtype=HSP_DTYPE)
        lat = ctypes.c_double()
        check(self._lib.blaze_server_take(self._h, ticket, out.ctypes.data_as(ctypes.c_void_p), n.value,
                                          ctypes.byref(n), ctypes.byref(lat)), "blaze_server_take")
        self.last_latency_ms = lat.value
        return out[: n.value]

    def stats(self) -> dict:
        st = BlazeServerStats()
        check(self._lib.blaze_server_stats_get(self._h, ctypes.byref(st)), "blaze_server_stats_get")
        return st.as_dict()

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.blaze_server_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


from . import shard, tabular, volume  # noqa: E402,F401  (submodules of the public API)
