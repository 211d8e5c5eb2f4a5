"""Python binding of libktruss_gb300 (ctypes over the C ABI in include/ktruss_gb300.h).

Mirrors the reference's k-truss interface:
    parse_args(argv)                  config.h:183-224   parseArgs
    create_coo_from_file(path)        graph.cu:37-79     createCOOFromFile
    write_coo_graph_to_file(g, path)  graph.cu:96-104    writeCOOGraphToFile
    ktruss(graph, config)             kernel.h:12        ktruss (returns the truss graph)
    verify(truss, config)             verify.cu:12-40    verify (raises KtrussError on mismatch)
and adds decompose() (per-edge truss numbers, k_max), the device-resident Engine and the
seeded generators.  Every call goes to the compiled library; there is no Python fallback:
if the library is missing, importing fails with the build command to run.
"""
from __future__ import annotations

import ctypes
import dataclasses
import os
from typing import Optional

import numpy as np

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG_DIR, "lib", "libktruss_gb300.so")
CLI_PATH = os.path.join(PKG_DIR, "bin", "ktruss")

PROCESSOR = {"cpu": 0, "gpu": 1}
DIRECTEDNESS = {"undirected": 0, "directed-by-index": 1, "directed-by-degree": 2}
INPUT_FORMAT = {"coocsr": 0, "tiled-coocsr": 1}
RECOUNT = {"all": 0, "affected": 1}

KT_OK = 0
STATUS_NAMES = {0: "KT_OK", 1: "KT_ERR_INVALID_ARG", 2: "KT_ERR_SELF_LOOP", 3: "KT_ERR_NOT_SYMMETRIC",
                4: "KT_ERR_CAPACITY", 5: "KT_ERR_UNSUPPORTED", 6: "KT_ERR_CUDA", 7: "KT_ERR_DEVICE_ALLOC",
                8: "KT_ERR_HOST_ALLOC", 9: "KT_ERR_IO", 10: "KT_ERR_MISMATCH", 11: "KT_ERR_TIMEOUT",
                12: "KT_ERR_NO_DEVICE", 13: "KT_ERR_TOO_LARGE", 14: "KT_ERR_INTERNAL"}


class KtrussError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


class _Coo(ctypes.Structure):
    _fields_ = [("num_nodes", ctypes.c_uint32), ("num_edges", ctypes.c_uint32), ("capacity", ctypes.c_uint32),
                ("src_idx", ctypes.POINTER(ctypes.c_uint32)), ("dst_idx", ctypes.POINTER(ctypes.c_uint32))]


class _Config(ctypes.Structure):
    _fields_ = [("graph_file_name", ctypes.c_char_p), ("k", ctypes.c_uint32), ("compare_file_name", ctypes.c_char_p),
                ("out_file_name", ctypes.c_char_p), ("num_warmup_runs", ctypes.c_uint32),
                ("num_timed_runs", ctypes.c_uint32), ("processor", ctypes.c_int32), ("directedness", ctypes.c_int32),
                ("input_format", ctypes.c_int32), ("num_edge_remove_iter", ctypes.c_uint32),
                ("recount", ctypes.c_int32), ("block_size", ctypes.c_uint32), ("num_tiles", ctypes.c_uint32),
                ("num_parallel_tiles", ctypes.c_uint32), ("verbosity", ctypes.c_uint32),
                ("num_nodes", ctypes.c_uint32), ("num_edges", ctypes.c_uint32)]


class _Edges(ctypes.Structure):
    _fields_ = [("num_nodes", ctypes.c_uint32), ("num_edges", ctypes.c_uint64),
                ("u", ctypes.POINTER(ctypes.c_uint32)), ("v", ctypes.POINTER(ctypes.c_uint32))]


class Stats(ctypes.Structure):
    _fields_ = [("num_nodes", ctypes.c_uint32), ("num_edges", ctypes.c_uint64), ("k_max", ctypes.c_uint32),
                ("num_levels", ctypes.c_uint32), ("num_rounds", ctypes.c_uint32), ("triangles", ctypes.c_uint64),
                ("plain_alive_sum", ctypes.c_uint64), ("plain_passes", ctypes.c_uint32),
                ("kernel_launches", ctypes.c_uint64), ("last_ms", ctypes.c_float),
                ("build_ms", ctypes.c_float), ("support_ms", ctypes.c_float), ("peel_ms", ctypes.c_float),
                ("compactions", ctypes.c_uint32), ("peel_phase_ms", ctypes.c_float * 6),
                ("peel_kernel_ms", ctypes.c_float), ("select_ms", ctypes.c_float),
                ("walk_entries", ctypes.c_uint64), ("copy_in_ms", ctypes.c_float), ("copy_out_ms", ctypes.c_float),
                ("emit_ms", ctypes.c_float)]

    PHASES = ("init", "level_scan", "collect", "compaction", "mark", "process")

    def as_dict(self) -> dict:
        d = {f: getattr(self, f) for f, _ in self._fields_}
        d["peel_phase_ms"] = dict(zip(self.PHASES, list(self.peel_phase_ms)))
        return d


class Variant(ctypes.Structure):
    """kt_variant: the reference's -d/-f/-r/-b/-t/-y switches for single-k truss calls (every
    variant gives the same k-truss; they select different kernel paths)."""
    _fields_ = [("directedness", ctypes.c_int32), ("input_format", ctypes.c_int32), ("recount", ctypes.c_int32),
                ("block_size", ctypes.c_uint32), ("num_tiles", ctypes.c_uint32),
                ("num_parallel_tiles", ctypes.c_uint32)]


class Schedule(ctypes.Structure):
    """kt_schedule: lanes per edge of the support count, row entries per peel chunk, the
    alive-edge percentage below which rows are compacted (0 = never), and the frontier share of
    the alive edges from which a round recounts the survivors instead of decrementing (0 = never).
    Results never depend on it."""
    _fields_ = [("support_group", ctypes.c_uint32), ("chunk_width", ctypes.c_uint32),
                ("compact_percent", ctypes.c_uint32), ("recount_percent", ctypes.c_uint32),
                ("peel_blocks", ctypes.c_uint32)]

    def as_tuple(self) -> tuple:
        return (self.support_group, self.chunk_width, self.compact_percent, self.recount_percent, self.peel_blocks)

    def __repr__(self) -> str:
        return ("Schedule(support_group=%d, chunk_width=%d, compact_percent=%d, recount_percent=%d, "
                "peel_blocks=%d)" % self.as_tuple())


_LIB = None
_U32P = ctypes.POINTER(ctypes.c_uint32)
_VP = ctypes.c_void_p


def lib() -> ctypes.CDLL:
    """Loads libktruss_gb300.so (built by ktruss-explorer_gb300/build.py)."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: run `python ktruss-explorer_gb300/build.py` "
                              "(or __graft_entry__.build()) to compile the CUDA library")
        L = ctypes.CDLL(LIB_PATH)
        L.kt_last_error.restype = ctypes.c_char_p
        L.kt_status_string.restype = ctypes.c_char_p
        L.kt_status_string.argtypes = [ctypes.c_int]
        L.kt_config_default.argtypes = [ctypes.POINTER(_Config)]
        L.kt_parse_args.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_char_p), ctypes.POINTER(_Config)]
        L.kt_coo_alloc.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.POINTER(_Coo)]
        L.kt_coo_free.argtypes = [ctypes.POINTER(_Coo)]
        L.kt_coo_free.restype = None
        L.kt_read_tsv.argtypes = [ctypes.c_char_p, ctypes.POINTER(_Coo)]
        L.kt_write_tsv.argtypes = [ctypes.POINTER(_Coo), ctypes.c_char_p]
        L.kt_write_truss_tsv.argtypes = [ctypes.POINTER(_Coo), _U32P, ctypes.c_char_p]
        L.kt_ktruss.argtypes = [ctypes.POINTER(_Coo), ctypes.POINTER(_Coo), ctypes.POINTER(_Config)]
        L.kt_decompose.argtypes = [ctypes.POINTER(_Coo), _U32P, _U32P, ctypes.POINTER(_Config)]
        L.kt_verify.argtypes = [ctypes.POINTER(_Coo), ctypes.POINTER(_Config)]
        L.kt_engine_create.argtypes = [ctypes.c_int, ctypes.POINTER(_VP)]
        L.kt_engine_destroy.argtypes = [_VP]
        L.kt_engine_stream.argtypes = [_VP]
        L.kt_engine_stream.restype = _VP
        L.kt_engine_reserve.argtypes = [_VP, ctypes.c_uint32, ctypes.c_uint64]
        L.kt_engine_decompose.argtypes = [_VP, _VP, _VP, ctypes.c_uint64, ctypes.c_uint32, _VP, _VP, ctypes.c_int]
        L.kt_engine_ktruss.argtypes = [_VP, _VP, _VP, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32, _VP,
                                       ctypes.c_int]
        L.kt_engine_replay.argtypes = [_VP, ctypes.c_int]
        L.kt_engine_replay_mode.argtypes = [_VP]
        L.kt_engine_stats.argtypes = [_VP, ctypes.POINTER(Stats)]
        L.kt_last_stats.argtypes = [ctypes.POINTER(Stats)]
        L.kt_engine_selftest_barrier_timeout.argtypes = [_VP, ctypes.c_uint64]
        L.kt_engine_decompose_batch.argtypes = [_VP, _VP, _VP, ctypes.c_uint64, ctypes.c_uint32, _VP, ctypes.c_uint32,
                                                _VP, _VP, ctypes.c_int]
        L.kt_decompose_batch.argtypes = [_U32P, _U32P, ctypes.c_uint64, ctypes.c_uint32, _U32P, ctypes.c_uint32,
                                         _U32P, _U32P]
        L.kt_gen_batch.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint64,
                                   ctypes.POINTER(_Edges), _U32P]
        L.kt_decompose_noalloc.argtypes = [_VP, _VP, ctypes.c_uint64, ctypes.c_uint32, _VP, _VP, _VP]
        L.kt_engine_level_log.argtypes = [_VP, _U32P, _U32P, _U32P, _U32P, ctypes.c_uint32, _U32P]
        L.kt_engine_round_log.argtypes = [_VP, _U32P, _U32P, _U32P, ctypes.c_uint32, _U32P]
        L.kt_schedule_default.restype = Schedule
        L.kt_schedule_default.argtypes = []
        L.kt_variant_default.restype = Variant
        L.kt_variant_default.argtypes = []
        L.kt_engine_set_variant.argtypes = [_VP, ctypes.POINTER(Variant)]
        L.kt_engine_get_variant.argtypes = [_VP, ctypes.POINTER(Variant)]
        L.kt_engine_set_schedule.argtypes = [_VP, ctypes.POINTER(Schedule)]
        L.kt_engine_get_schedule.argtypes = [_VP, ctypes.POINTER(Schedule)]
        L.kt_engine_set_wait_limit.argtypes = [_VP, ctypes.c_uint64, ctypes.c_uint32]
        L.kt_engine_get_wait_limit.argtypes = [_VP, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint32)]
        _FP = ctypes.POINTER(ctypes.c_float)
        L.kt_selector_create.argtypes = [ctypes.c_int, ctypes.c_uint64, ctypes.POINTER(_VP)]
        L.kt_selector_destroy.argtypes = [_VP]
        L.kt_selector_get_params.argtypes = [_VP, _FP, _FP, _FP]
        L.kt_selector_set_params.argtypes = [_VP, _FP, _FP, _FP]
        L.kt_selector_train.argtypes = [_VP, _FP, _FP, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                        ctypes.c_float, ctypes.c_uint64, _FP]
        L.kt_selector_gradient.argtypes = [_VP, _FP, _FP, ctypes.c_uint32, _FP, _FP]
        L.kt_selector_predict.argtypes = [_VP, _FP, ctypes.c_uint32, ctypes.POINTER(Schedule)]
        L.kt_engine_features.argtypes = [_VP, _VP, _VP, ctypes.c_uint64, ctypes.c_uint32, _FP]
        L.kt_engine_set_selector.argtypes = [_VP, _VP]
        L.kt_engine_tiled_coocsr.argtypes = [_VP, _VP, _VP, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32, _VP,
                                             _VP, _VP]
        L.kt_engine_symmetrize.argtypes = [_VP, _VP, _VP, ctypes.c_uint64, ctypes.c_uint32, _VP, _VP, ctypes.c_uint64,
                                           ctypes.POINTER(ctypes.c_uint64)]
        _U64P = ctypes.POINTER(ctypes.c_uint64)
        L.kt_engine_parse_tsv.argtypes = [_VP, _VP, ctypes.c_uint64, _VP, _VP, ctypes.c_uint64, _U64P, _U32P]
        L.kt_engine_read_tsv.argtypes = [_VP, ctypes.c_char_p, _VP, _VP, ctypes.c_uint64, _U64P, _U32P]
        L.kt_set_schedule.argtypes = [ctypes.POINTER(Schedule)]
        L.kt_get_schedule.argtypes = [ctypes.POINTER(Schedule)]
        L.kt_schedule_grid.argtypes = [ctypes.POINTER(Schedule), ctypes.c_uint32]
        L.kt_schedule_grid.restype = ctypes.c_uint32
        for f in ("kt_engine_autotune", "kt_engine_autotune_batch"):
            getattr(L, f).argtypes = [_VP, _VP, _VP, ctypes.c_uint64, ctypes.c_uint32, ctypes.POINTER(Schedule),
                                      ctypes.c_uint32, ctypes.c_uint32, ctypes.POINTER(ctypes.c_float),
                                      ctypes.POINTER(Schedule)]
        for g in ("kt_gen_rmat",):
            getattr(L, g).argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_double, ctypes.c_double,
                                      ctypes.c_double, ctypes.c_uint64, ctypes.POINTER(_Edges)]
        L.kt_gen_er.argtypes = [ctypes.c_uint32, ctypes.c_double, ctypes.c_uint64, ctypes.POINTER(_Edges)]
        L.kt_gen_ba.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint64, ctypes.POINTER(_Edges)]
        L.kt_gen_ws.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_double, ctypes.c_uint64,
                                ctypes.POINTER(_Edges)]
        L.kt_gen_rgg.argtypes = [ctypes.c_uint32, ctypes.c_double, ctypes.c_uint64, ctypes.POINTER(_Edges)]
        L.kt_plant_cliques.argtypes = [ctypes.c_uint32, _U32P, _U32P, ctypes.c_uint64, ctypes.c_uint32,
                                       ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint64, ctypes.POINTER(_Edges)]
        L.kt_edges_free.argtypes = [ctypes.POINTER(_Edges)]
        L.kt_edges_free.restype = None
        _LIB = L
    return _LIB


def _check(rc: int) -> None:
    if rc != KT_OK:
        raise KtrussError(rc, lib().kt_last_error().decode(errors="replace"))


# ---- configuration (config.h) -------------------------------------------------------------

@dataclasses.dataclass
class Config:
    """Fields and defaults of the reference's Config (config.h:163-199)."""
    graph_file_name: str = "data/loc-gowalla_edges_adj.tsv"
    k: int = 3
    compare_file_name: str = "data/loc-gowalla_edges_adj.tsv.3.reference.tsv"
    out_file_name: Optional[str] = None
    num_warmup_runs: int = 0
    num_timed_runs: int = 1
    processor: str = "gpu"
    directedness: str = "directed-by-degree"
    input_format: str = "coocsr"
    num_edge_remove_iter: int = 0
    recount: str = "all"
    block_size: int = 512
    num_tiles: int = 8
    num_parallel_tiles: int = 8
    verbosity: int = 1
    num_nodes: int = 0
    num_edges: int = 0

    def _c(self) -> tuple[_Config, list]:
        keep = [s.encode() if s is not None else None for s in
                (self.graph_file_name, self.compare_file_name, self.out_file_name)]
        c = _Config(keep[0], self.k & 0xFFFFFFFF, keep[1], keep[2], self.num_warmup_runs, self.num_timed_runs,
                    PROCESSOR[self.processor], DIRECTEDNESS[self.directedness], INPUT_FORMAT[self.input_format],
                    self.num_edge_remove_iter, RECOUNT[self.recount], self.block_size, self.num_tiles,
                    self.num_parallel_tiles, self.verbosity, self.num_nodes, self.num_edges)
        return c, keep


def parse_args(argv: list[str]) -> Config:
    """getopt parsing of the reference's flags; raises KtrussError on a bad option."""
    args = [a.encode() for a in (["ktruss"] + list(argv))]
    arr = (ctypes.c_char_p * len(args))(*args)
    c = _Config()
    _check(lib().kt_parse_args(len(args), arr, ctypes.byref(c)))
    inv = lambda d, v: next(k for k, x in d.items() if x == v)
    return Config(c.graph_file_name.decode(), c.k, c.compare_file_name.decode(),
                  c.out_file_name.decode() if c.out_file_name else None, c.num_warmup_runs, c.num_timed_runs,
                  inv(PROCESSOR, c.processor), inv(DIRECTEDNESS, c.directedness), inv(INPUT_FORMAT, c.input_format),
                  c.num_edge_remove_iter, inv(RECOUNT, c.recount), c.block_size, c.num_tiles, c.num_parallel_tiles,
                  c.verbosity, c.num_nodes, c.num_edges)


# ---- graphs (graph.h COOGraph) --------------------------------------------------------------

@dataclasses.dataclass
class COOGraph:
    """COOGraph (graph.h:10-16): every undirected edge once per direction, 0-based ids."""
    num_nodes: int
    src_idx: np.ndarray
    dst_idx: np.ndarray

    def __post_init__(self):
        self.src_idx = np.ascontiguousarray(self.src_idx, dtype=np.uint32)
        self.dst_idx = np.ascontiguousarray(self.dst_idx, dtype=np.uint32)
        if self.src_idx.shape != self.dst_idx.shape:
            raise ValueError("src_idx and dst_idx differ in length")

    @property
    def num_edges(self) -> int:
        return int(self.src_idx.size)

    def _c(self) -> _Coo:
        return _Coo(self.num_nodes, self.num_edges, self.num_edges, self.src_idx.ctypes.data_as(_U32P),
                    self.dst_idx.ctypes.data_as(_U32P))

    @staticmethod
    def from_undirected(num_nodes: int, u, v) -> "COOGraph":
        """Both directions of each undirected edge (u[i], v[i])."""
        u = np.asarray(u, dtype=np.uint32)
        v = np.asarray(v, dtype=np.uint32)
        return COOGraph(num_nodes, np.concatenate([u, v]), np.concatenate([v, u]))

    def canonical(self) -> np.ndarray:
        """Sorted unique (min, max) pairs as uint64 keys."""
        a = np.minimum(self.src_idx, self.dst_idx).astype(np.uint64)
        b = np.maximum(self.src_idx, self.dst_idx).astype(np.uint64)
        return np.unique((a << np.uint64(32)) | b)


def _from_c(c: _Coo) -> COOGraph:
    n = c.num_edges
    s = np.ctypeslib.as_array(c.src_idx, shape=(n,)).copy() if n else np.zeros(0, np.uint32)
    d = np.ctypeslib.as_array(c.dst_idx, shape=(n,)).copy() if n else np.zeros(0, np.uint32)
    return COOGraph(c.num_nodes, s, d)


def create_coo_from_file(path: str) -> COOGraph:
    c = _Coo()
    _check(lib().kt_read_tsv(path.encode(), ctypes.byref(c)))
    try:
        return _from_c(c)
    finally:
        lib().kt_coo_free(ctypes.byref(c))


def write_coo_graph_to_file(graph: COOGraph, path: str) -> None:
    c = graph._c()
    _check(lib().kt_write_tsv(ctypes.byref(c), path.encode()))


def write_truss_to_file(graph: COOGraph, truss_per_entry: np.ndarray, path: str) -> None:
    t = np.ascontiguousarray(truss_per_entry, dtype=np.uint32)
    c = graph._c()
    _check(lib().kt_write_truss_tsv(ctypes.byref(c), t.ctypes.data_as(_U32P), path.encode()))


# ---- the k-truss path -----------------------------------------------------------------------

def ktruss(graph: COOGraph, config: Optional[Config] = None) -> COOGraph:
    """k-truss for config.k on the GPU (kernel.h:12); returns the truss in both directions."""
    config = config or Config()
    cfg, _keep = config._c()
    cfg.num_nodes, cfg.num_edges = graph.num_nodes, graph.num_edges
    g = graph._c()
    out_s = np.empty(max(graph.num_edges, 1), np.uint32)
    out_d = np.empty(max(graph.num_edges, 1), np.uint32)
    t = _Coo(graph.num_nodes, 0, graph.num_edges, out_s.ctypes.data_as(_U32P), out_d.ctypes.data_as(_U32P))
    _check(lib().kt_ktruss(ctypes.byref(g), ctypes.byref(t), ctypes.byref(cfg)))
    return COOGraph(t.num_nodes, out_s[: t.num_edges].copy(), out_d[: t.num_edges].copy())


def decompose(graph: COOGraph, config: Optional[Config] = None,
              out: Optional[np.ndarray] = None) -> tuple[np.ndarray, int]:
    """Per-entry truss numbers and k_max on the GPU.  `out` (uint32, num_edges) may be a
    caller-owned (for example pinned) buffer to receive the result."""
    g = graph._c()
    if out is None:
        out = np.zeros(max(graph.num_edges, 1), np.uint32)
    elif out.dtype != np.uint32 or not out.flags.c_contiguous or out.size < graph.num_edges:
        raise ValueError("out must be a contiguous uint32 array with num_edges elements")
    kmax = ctypes.c_uint32(0)
    cfg = None
    keep = None
    if config is not None:
        cfg, keep = config._c()
    _check(lib().kt_decompose(ctypes.byref(g), out.ctypes.data_as(_U32P), ctypes.byref(kmax),
                              ctypes.byref(cfg) if cfg is not None else None))
    del keep
    return out[: graph.num_edges], kmax.value


def verify(truss: COOGraph, config: Config) -> None:
    """verify.cu:12-40: raises KtrussError(KT_ERR_MISMATCH) if the edge sets differ."""
    cfg, _keep = config._c()
    t = truss._c()
    _check(lib().kt_verify(ctypes.byref(t), ctypes.byref(cfg)))


class Engine:
    """Device-resident engine: graph and outputs stay in HBM (pointers are device addresses)."""

    def __init__(self, device: int = 0):
        h = _VP()
        _check(lib().kt_engine_create(device, ctypes.byref(h)))
        self._h = h

    def close(self) -> None:
        if self._h:
            lib().kt_engine_destroy(self._h)
            self._h = _VP()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def stream(self) -> int:
        return lib().kt_engine_stream(self._h) or 0

    def reserve(self, max_nodes: int, max_entries: int) -> None:
        _check(lib().kt_engine_reserve(self._h, max_nodes, max_entries))

    def decompose(self, d_src: int, d_dst: int, num_entries: int, num_nodes: int, d_truss: int,
                  d_k_max: int = 0, sync: bool = True) -> None:
        _check(lib().kt_engine_decompose(self._h, d_src, d_dst, num_entries, num_nodes, d_truss, d_k_max or None,
                                         int(sync)))

    def decompose_batch(self, d_src: int, d_dst: int, num_entries: int, num_nodes: int, d_offsets: int,
                        num_graphs: int, d_truss: int, d_k_max: int, sync: bool = True) -> None:
        _check(lib().kt_engine_decompose_batch(self._h, d_src, d_dst, num_entries, num_nodes, d_offsets, num_graphs,
                                               d_truss, d_k_max, int(sync)))

    def ktruss(self, d_src: int, d_dst: int, num_entries: int, num_nodes: int, k: int, d_keep: int,
               sync: bool = True) -> None:
        _check(lib().kt_engine_ktruss(self._h, d_src, d_dst, num_entries, num_nodes, k & 0xFFFFFFFF, d_keep,
                                      int(sync)))

    def replay(self, sync: bool = True) -> None:
        """Repeats the last decompose/ktruss call on the same (unchanged) device buffers through
        a CUDA graph of its device pipeline, captured at the first replay."""
        _check(lib().kt_engine_replay(self._h, int(sync)))

    def replay_mode(self) -> str:
        """How the next replay runs: "cuda graph", "direct launches" or "none" (not captured yet)."""
        return {1: "cuda graph", 2: "direct launches"}.get(lib().kt_engine_replay_mode(self._h), "none")

    def set_schedule(self, support_group: int = 8, chunk_width: int = 32, compact_percent: int = 85,
                     recount_percent: int = 50, peel_blocks: int = 0) -> None:
        s = Schedule(support_group, chunk_width, compact_percent, recount_percent, peel_blocks)
        _check(lib().kt_engine_set_schedule(self._h, ctypes.byref(s)))

    def set_variant(self, directedness: str = "directed-by-degree", input_format: str = "coocsr",
                    recount: str = "all", block_size: int = 512, num_tiles: int = 8,
                    num_parallel_tiles: int = 8) -> None:
        """Variant of later single-k calls, named as on the reference's command line."""
        v = Variant(DIRECTEDNESS[directedness], INPUT_FORMAT[input_format], RECOUNT[recount], block_size, num_tiles,
                    num_parallel_tiles)
        _check(lib().kt_engine_set_variant(self._h, ctypes.byref(v)))

    def variant(self) -> Variant:
        v = Variant()
        _check(lib().kt_engine_get_variant(self._h, ctypes.byref(v)))
        return v

    def set_wait_limit(self, base_ns: int, ns_per_unit: int = 8) -> None:
        """Bound of every peel barrier wait: base_ns plus ns_per_unit per unit of covered work."""
        _check(lib().kt_engine_set_wait_limit(self._h, base_ns, ns_per_unit))

    def wait_limit(self) -> tuple:
        b, u = ctypes.c_uint64(0), ctypes.c_uint32(0)
        _check(lib().kt_engine_get_wait_limit(self._h, ctypes.byref(b), ctypes.byref(u)))
        return b.value, u.value

    def schedule(self) -> Schedule:
        s = Schedule()
        _check(lib().kt_engine_get_schedule(self._h, ctypes.byref(s)))
        return s

    def autotune(self, d_src: int, d_dst: int, num_entries: int, num_nodes: int, candidates=None,
                 repeats: int = 1, batch: bool = False) -> tuple:
        """Times every candidate schedule (default: the built-in grid) on this device graph and
        keeps the fastest; returns (best Schedule, [(Schedule, ms), ...]).  batch=True times the
        candidates as decompose_batch runs them (the graph is the union of a sample batch)."""
        cands = list(candidates) if candidates is not None else schedule_grid()
        arr = (Schedule * len(cands))(*[Schedule(*c.as_tuple()) if isinstance(c, Schedule) else Schedule(*c)
                                        for c in cands])
        ms = (ctypes.c_float * len(cands))()
        best = Schedule()
        fn = lib().kt_engine_autotune_batch if batch else lib().kt_engine_autotune
        _check(fn(self._h, d_src, d_dst, num_entries, num_nodes, arr, len(cands), repeats, ms, ctypes.byref(best)))
        return best, [(arr[i], ms[i]) for i in range(len(cands))]

    def features(self, d_src: int, d_dst: int, num_entries: int, num_nodes: int) -> np.ndarray:
        """The selector's 16 features of this device graph (built on the device)."""
        out = np.zeros(SELECTOR_FEATURES, np.float32)
        _check(lib().kt_engine_features(self._h, d_src, d_dst, num_entries, num_nodes, _fp(out)))
        return out

    def parse_tsv(self, d_text: int, num_bytes: int, d_src: int, d_dst: int, capacity: int) -> tuple:
        """Parses TSV text already on the device into device entries; returns (entries, num_nodes)."""
        ne, nn = ctypes.c_uint64(0), ctypes.c_uint32(0)
        _check(lib().kt_engine_parse_tsv(self._h, d_text, num_bytes, d_src, d_dst, capacity, ctypes.byref(ne),
                                         ctypes.byref(nn)))
        return ne.value, nn.value

    def read_tsv(self, path: str, d_src: int, d_dst: int, capacity: int) -> tuple:
        """Reads a TSV file into device entries (parsed on the device); returns (entries, num_nodes)."""
        ne, nn = ctypes.c_uint64(0), ctypes.c_uint32(0)
        _check(lib().kt_engine_read_tsv(self._h, os.fsencode(path), d_src, d_dst, capacity, ctypes.byref(ne),
                                        ctypes.byref(nn)))
        return ne.value, nn.value

    def tiled_coocsr(self, d_src: int, d_dst: int, num_entries: int, num_nodes: int, tiles_per_dim: int,
                     d_tile_src_ptr: int, d_src_out: int, d_dst_out: int) -> None:
        """The reference's tiled COO/CSR layout of a device entry list (kt_engine_tiled_coocsr)."""
        _check(lib().kt_engine_tiled_coocsr(self._h, d_src, d_dst, num_entries, num_nodes, tiles_per_dim,
                                            d_tile_src_ptr, d_src_out, d_dst_out))

    def symmetrize(self, d_src: int, d_dst: int, num_entries: int, num_nodes: int, d_src_out: int, d_dst_out: int,
                   capacity: int) -> int:
        """Symmetric simple graph of a device entry list (kt_engine_symmetrize): directions merged,
        duplicates and self loops dropped; returns the number of entries written (2 per edge)."""
        out = ctypes.c_uint64(0)
        _check(lib().kt_engine_symmetrize(self._h, d_src, d_dst, num_entries, num_nodes, d_src_out, d_dst_out,
                                          capacity, ctypes.byref(out)))
        return out.value

    def set_selector(self, selector: Optional["Selector"]) -> None:
        """Attach a learned selector (its schedule is used by every decomposition) or detach (None)."""
        self._selector = selector  # keep it alive while attached
        _check(lib().kt_engine_set_selector(self._h, selector._h if selector is not None else None))

    def selftest_barrier_timeout(self, timeout_ns: int) -> int:
        """Status of a grid barrier that cannot complete (KT_ERR_TIMEOUT = 11 when correct)."""
        return lib().kt_engine_selftest_barrier_timeout(self._h, timeout_ns)

    def round_log(self, cap: int = 1 << 20) -> dict:
        """Frontier size, level and device nanoseconds of each peel round of the last call."""
        size, level, ns = (np.zeros(cap, np.uint32) for _ in range(3))
        R = ctypes.c_uint32(0)
        _check(lib().kt_engine_round_log(self._h, size.ctypes.data_as(_U32P), level.ctypes.data_as(_U32P),
                                         ns.ctypes.data_as(_U32P), cap, ctypes.byref(R)))
        c = min(cap, R.value)
        return {"size": size[:c], "level": level[:c], "ns": ns[:c], "rounds": R.value}

    def level_log(self, cap: int = 1 << 20) -> dict:
        """k, alive edges, start-of-level device nanoseconds and first frontier of each level."""
        arr = [np.zeros(cap, np.uint32) for _ in range(4)]
        L = ctypes.c_uint32(0)
        _check(lib().kt_engine_level_log(self._h, *[a.ctypes.data_as(_U32P) for a in arr], cap, ctypes.byref(L)))
        c = min(cap, L.value)
        return {"k": arr[0][:c], "alive": arr[1][:c], "ns": arr[2][:c], "frontier": arr[3][:c], "levels": L.value}

    def stats(self) -> Stats:
        s = Stats()
        _check(lib().kt_engine_stats(self._h, ctypes.byref(s)))
        return s


SELECTOR_FEATURES, SELECTOR_VARIANTS, SELECTOR_SCHEDULES, SELECTOR_PARAMS = 16, 18, 36, 6483


def _fp(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def _f32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float32)


class Selector:
    """Learned schedule selector (kt_selector): FP32 MLP 16-64-64-19 trained and run by the
    library's own CUDA kernels."""

    def __init__(self, device: int = 0, seed: int = 1):
        h = _VP()
        _check(lib().kt_selector_create(device, seed, ctypes.byref(h)))
        self._h = h

    def close(self) -> None:
        if self._h:
            lib().kt_selector_destroy(self._h)
            self._h = _VP()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def params(self) -> tuple:
        p = np.zeros(SELECTOR_PARAMS, np.float32)
        mean = np.zeros(SELECTOR_FEATURES, np.float32)
        scale = np.zeros(SELECTOR_FEATURES, np.float32)
        _check(lib().kt_selector_get_params(self._h, _fp(p), _fp(mean), _fp(scale)))
        return p, mean, scale

    def set_params(self, params=None, mean=None, scale=None) -> None:
        a = [None if x is None else _f32(x) for x in (params, mean, scale)]
        _check(lib().kt_selector_set_params(self._h, *[_fp(x) for x in a]))

    def train(self, features, times, epochs: int = 200, batch: int = 64, lr: float = 3e-3, seed: int = 1):
        """Trains on (n x 16 features, n x 36 times in ms); returns the mean loss of each epoch."""
        f, t = _f32(features), _f32(times)
        assert f.shape[1] == SELECTOR_FEATURES and t.shape == (f.shape[0], SELECTOR_SCHEDULES)
        losses = np.zeros(epochs, np.float32)
        _check(lib().kt_selector_train(self._h, _fp(f), _fp(t), f.shape[0], epochs, batch, lr, seed, _fp(losses)))
        return losses

    def gradient(self, features, times) -> tuple:
        f, t = _f32(features), _f32(times)
        g = np.zeros(SELECTOR_PARAMS, np.float32)
        loss = ctypes.c_float(0)
        _check(lib().kt_selector_gradient(self._h, _fp(f), _fp(t), f.shape[0], _fp(g), ctypes.byref(loss)))
        return loss.value, g

    def predict(self, features) -> list:
        f = _f32(features).reshape(-1, SELECTOR_FEATURES)
        out = (Schedule * max(1, f.shape[0]))()
        _check(lib().kt_selector_predict(self._h, _fp(f), f.shape[0], out))
        return [out[i] for i in range(f.shape[0])]


def schedule_index(s) -> int:
    """Position of a schedule in the autotuner's grid."""
    t = s.as_tuple() if isinstance(s, Schedule) else tuple(s)
    return [g.as_tuple() for g in schedule_grid()].index(t)


def schedule_default() -> Schedule:
    return lib().kt_schedule_default()


def set_schedule(support_group: int = 8, chunk_width: int = 32, compact_percent: int = 85,
                 recount_percent: int = 50, peel_blocks: int = 0) -> None:
    """Schedule of the engine behind the host-buffer calls (ktruss, decompose, decompose_batch)."""
    s = Schedule(support_group, chunk_width, compact_percent, recount_percent, peel_blocks)
    _check(lib().kt_set_schedule(ctypes.byref(s)))


def get_schedule() -> Schedule:
    s = Schedule()
    _check(lib().kt_get_schedule(ctypes.byref(s)))
    return s


def schedule_grid() -> list:
    """The autotuner's built-in candidate schedules."""
    n = lib().kt_schedule_grid(None, 0)
    arr = (Schedule * n)()
    lib().kt_schedule_grid(arr, n)
    return [arr[i] for i in range(n)]


def last_stats() -> Stats:
    """Statistics of the last host-buffer call (the engine behind kt_ktruss / kt_decompose /
    kt_decompose_batch)."""
    s = Stats()
    _check(lib().kt_last_stats(ctypes.byref(s)))
    return s


def decompose_batch(src, dst, num_nodes: int, vertex_offsets, out: Optional[np.ndarray] = None):
    """Batched decomposition of graphs on disjoint vertex ranges (host buffers).
    Returns (truss per entry, k_max per graph)."""
    src = np.ascontiguousarray(src, np.uint32)
    dst = np.ascontiguousarray(dst, np.uint32)
    off = np.ascontiguousarray(vertex_offsets, np.uint32)
    G = len(off) - 1
    if out is None:
        out = np.zeros(max(len(src), 1), np.uint32)
    kmax = np.zeros(G, np.uint32)
    _check(lib().kt_decompose_batch(src.ctypes.data_as(_U32P), dst.ctypes.data_as(_U32P), len(src), num_nodes,
                                    off.ctypes.data_as(_U32P), G, out.ctypes.data_as(_U32P),
                                    kmax.ctypes.data_as(_U32P)))
    return out[: len(src)], kmax


def gen_batch(num_graphs: int, n_min: int, n_max: int, seed: int = 1):
    """(num_nodes, u, v, vertex_offsets) of a seeded batch of BA / WS graphs with planted cliques."""
    e = _Edges()
    off = np.zeros(num_graphs + 1, np.uint32)
    _check(lib().kt_gen_batch(num_graphs, n_min, n_max, seed, ctypes.byref(e), off.ctypes.data_as(_U32P)))
    try:
        k = e.num_edges
        u = np.ctypeslib.as_array(e.u, shape=(k,)).copy() if k else np.zeros(0, np.uint32)
        v = np.ctypeslib.as_array(e.v, shape=(k,)).copy() if k else np.zeros(0, np.uint32)
        return e.num_nodes, u, v, off
    finally:
        lib().kt_edges_free(ctypes.byref(e))


def decompose_noalloc(d_src: int, d_dst: int, num_entries: int, num_nodes: int, d_truss: int, d_k_max: int = 0,
                      stream: int = 0) -> None:
    """kt_decompose_noalloc: the decomposition with device buffers, without any allocation by the
    library (scratch in a fixed static device array; at most 524,288 entries and 131,072
    vertices).  For callers whose device memory must not be allocated behind their back."""
    _check(lib().kt_decompose_noalloc(d_src, d_dst, num_entries, num_nodes, d_truss, d_k_max or None,
                                      stream or None))


# ---- generators -----------------------------------------------------------------------------

def _edges(fn, *args) -> tuple[int, np.ndarray, np.ndarray]:
    e = _Edges()
    _check(fn(*args, ctypes.byref(e)))
    try:
        n = e.num_edges
        u = np.ctypeslib.as_array(e.u, shape=(n,)).copy() if n else np.zeros(0, np.uint32)
        v = np.ctypeslib.as_array(e.v, shape=(n,)).copy() if n else np.zeros(0, np.uint32)
        return e.num_nodes, u, v
    finally:
        lib().kt_edges_free(ctypes.byref(e))


def gen_rmat(scale: int, edge_factor: int, a=0.57, b=0.19, c=0.19, seed: int = 1):
    return _edges(lib().kt_gen_rmat, scale, edge_factor, a, b, c, seed)


def gen_er(n: int, p: float, seed: int = 1):
    return _edges(lib().kt_gen_er, n, p, seed)


def gen_ba(n: int, m: int, seed: int = 1):
    return _edges(lib().kt_gen_ba, n, m, seed)


def gen_ws(n: int, k: int, p: float, seed: int = 1):
    return _edges(lib().kt_gen_ws, n, k, p, seed)


def gen_rgg(n: int, radius: float, seed: int = 1):
    return _edges(lib().kt_gen_rgg, n, radius, seed)


def plant_cliques(num_nodes: int, u: np.ndarray, v: np.ndarray, count: int, min_size: int, max_size: int,
                  seed: int = 1):
    u = np.ascontiguousarray(u, dtype=np.uint32)
    v = np.ascontiguousarray(v, dtype=np.uint32)
    return _edges(lib().kt_plant_cliques, num_nodes, u.ctypes.data_as(_U32P), v.ctypes.data_as(_U32P), u.size,
                  count, min_size, max_size, seed)


def coo_from_edges(num_nodes: int, u: np.ndarray, v: np.ndarray) -> COOGraph:
    return COOGraph.from_undirected(num_nodes, u, v)
