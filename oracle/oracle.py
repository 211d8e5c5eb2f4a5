"""TEST INFRASTRUCTURE ONLY: ctypes bindings of the CPU oracle (ktruss_oracle.c).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this module, as the
checker or the timed CPU baseline.  The product library never loads it.

Graphs are numpy uint32 arrays ``src``/``dst`` holding every undirected edge once per
direction (the COO convention of the reference, graph.h:10-16).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libktoracle.so")

UNDIRECTED, DIRECTED_BY_INDEX, DIRECTED_BY_DEGREE = 0, 1, 2
RECOUNT_ALL, RECOUNT_AFFECTED = 0, 1

_lib = None


class _PassLog(ctypes.Structure):
    _fields_ = [("cap", ctypes.c_uint32), ("num", ctypes.c_uint32), ("alive", ctypes.POINTER(ctypes.c_uint64)),
                ("loop_seconds", ctypes.c_double)]


class _LevelLog(ctypes.Structure):
    _fields_ = [("cap", ctypes.c_uint32), ("num", ctypes.c_uint32), ("passes", ctypes.POINTER(ctypes.c_uint32)),
                ("alive", ctypes.POINTER(ctypes.c_uint64))]


def build() -> str:
    """Compiles oracle/_build/libktoracle.so with the committed Makefile."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def _load():
    global _lib
    if _lib is None:
        src = os.path.join(HERE, "ktruss_oracle.c")
        if not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
            build()
        lib = ctypes.CDLL(LIB_PATH)
        u32p = ctypes.POINTER(ctypes.c_uint32)
        lib.ko_ktruss.argtypes = [ctypes.c_uint32, ctypes.c_uint32, u32p, u32p, ctypes.c_uint32, ctypes.c_int,
                                  ctypes.c_int, ctypes.c_uint32, u32p, u32p, u32p, ctypes.POINTER(_PassLog)]
        lib.ko_decompose_chain.argtypes = [ctypes.c_uint32, ctypes.c_uint32, u32p, u32p, u32p, u32p, u32p,
                                           ctypes.POINTER(ctypes.c_uint64)]
        lib.ko_chain_sample.argtypes = [ctypes.c_uint32, ctypes.c_uint32, u32p, u32p, ctypes.c_double, u32p,
                                        ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_double)]
        lib.ko_decompose_peel.argtypes = [ctypes.c_uint32, ctypes.c_uint32, u32p, u32p, u32p, u32p, u32p,
                                          ctypes.POINTER(ctypes.c_uint64), u32p]
        lib.ko_decompose_peel_levels.argtypes = [ctypes.c_uint32, ctypes.c_uint32, u32p, u32p, u32p, u32p, u32p,
                                                 ctypes.POINTER(ctypes.c_uint64), u32p, ctypes.POINTER(_LevelLog)]
        lib.ko_decompose_peel_mt.argtypes = [ctypes.c_uint32, ctypes.c_uint32, u32p, u32p, u32p, u32p, u32p,
                                             ctypes.POINTER(ctypes.c_uint64), u32p, ctypes.POINTER(_LevelLog),
                                             ctypes.c_uint32]
        lib.ko_ktruss_runs.argtypes = [ctypes.c_uint32, ctypes.c_uint32, u32p, u32p, ctypes.c_uint32, ctypes.c_uint32,
                                       ctypes.c_uint32, u32p, u32p, u32p, ctypes.POINTER(ctypes.c_double), u32p]
        lib.ko_gen_rmat.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_double, ctypes.c_double,
                                    ctypes.c_double, ctypes.c_uint64, u32p, u32p, ctypes.POINTER(ctypes.c_uint64)]
        _lib = lib
    return _lib


def _p(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))


def _u32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.uint32)


def ktruss(num_nodes: int, src, dst, k: int, directedness: int = DIRECTED_BY_DEGREE,
           recount: int = RECOUNT_ALL, num_edge_remove_iter: int = 0, pass_log: bool = False,
           loop_seconds: bool = False):
    """Single-k k-truss (the reference's Host path).  Returns (out_src, out_dst[, alive per pass]
    [, seconds of the count-and-prune loop, the span the reference's k-truss timer covers])."""
    lib = _load()
    src, dst = _u32(src), _u32(dst)
    n = len(src)
    os_, od = np.zeros(max(n, 1), np.uint32), np.zeros(max(n, 1), np.uint32)
    num = ctypes.c_uint32(0)
    alive = np.zeros(1 << 16, np.uint64)
    log = _PassLog(len(alive), 0, alive.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), 0.0)
    rc = lib.ko_ktruss(num_nodes, n, _p(src), _p(dst), k & 0xFFFFFFFF, directedness, recount,
                       num_edge_remove_iter, _p(os_), _p(od), ctypes.byref(num), ctypes.byref(log))
    if rc != 0:
        raise MemoryError("oracle ko_ktruss failed")
    out = (os_[: num.value].copy(), od[: num.value].copy())
    if pass_log:
        out = out + (alive[: min(log.num, len(alive))].copy(),)
    if loop_seconds:
        out = out + (log.loop_seconds,)
    return out


def decompose(num_nodes: int, src, dst, method: str = "peel", levels: bool = False, threads=None):
    """Per-entry truss numbers.  method 'chain' chains single-k runs like the reference
    would be driven; 'peel' is the exact peeling (on `threads` host threads; None: one thread
    below a million entries, else up to 16).  Returns a dict; with levels=True (peel only) also
    'level_passes' and 'level_alive': per k, the passes of the reference chain's single-k run at k
    and the sum of their alive oriented edges."""
    lib = _load()
    src, dst = _u32(src), _u32(dst)
    n = len(src)
    truss = np.zeros(max(n, 1), np.uint32)
    kmax, passes, rounds = ctypes.c_uint32(0), ctypes.c_uint32(0), ctypes.c_uint32(0)
    alive_sum = ctypes.c_uint64(0)
    out = {}
    if method == "chain":
        rc = lib.ko_decompose_chain(num_nodes, n, _p(src), _p(dst), _p(truss), ctypes.byref(kmax),
                                    ctypes.byref(passes), ctypes.byref(alive_sum))
    elif method == "peel":
        cap = (1 << 20) if levels else 0
        lp = np.zeros(max(cap, 1), np.uint32)
        la = np.zeros(max(cap, 1), np.uint64)
        log = _LevelLog(cap, 0, lp.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)),
                        la.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)))
        if threads is None:
            threads = 1 if n < 1_000_000 else min(16, os.cpu_count() or 1)
        if threads > 1:
            rc = lib.ko_decompose_peel_mt(num_nodes, n, _p(src), _p(dst), _p(truss), ctypes.byref(kmax),
                                          ctypes.byref(passes), ctypes.byref(alive_sum), ctypes.byref(rounds),
                                          ctypes.byref(log) if levels else None, threads)
        else:
            rc = lib.ko_decompose_peel_levels(num_nodes, n, _p(src), _p(dst), _p(truss), ctypes.byref(kmax),
                                              ctypes.byref(passes), ctypes.byref(alive_sum), ctypes.byref(rounds),
                                              ctypes.byref(log) if levels else None)
        if levels:
            out = {"level_passes": lp[: log.num].copy(), "level_alive": la[: log.num].copy()}
    else:
        raise ValueError(method)
    if rc != 0:
        raise MemoryError("oracle decomposition failed")
    return {"truss": truss[:n].copy(), "k_max": kmax.value, "plain_passes": passes.value,
            "plain_alive_sum": alive_sum.value, "rounds": rounds.value if method == "peel" else None, **out}


def ktruss_runs(num_nodes: int, src, dst, k: int, runs: int, threads: int = 0):
    """Repeat runs of the reference's single-k loop (directed by degree, recount all) on `threads`
    host threads (0: all, at most 64): the CSR is built once, each run restores it and times the
    count-and-prune loop alone, like the reference's -w/-x runs.  Returns (out_src, out_dst of the
    last run, seconds per run, passes per run)."""
    lib = _load()
    src, dst = _u32(src), _u32(dst)
    n = len(src)
    threads = threads or min(64, os.cpu_count() or 1)
    os_, od = np.zeros(max(n, 1), np.uint32), np.zeros(max(n, 1), np.uint32)
    num = ctypes.c_uint32(0)
    secs = np.zeros(max(runs, 1), np.float64)
    passes = np.zeros(max(runs, 1), np.uint32)
    rc = lib.ko_ktruss_runs(num_nodes, n, _p(src), _p(dst), k & 0xFFFFFFFF, runs, threads, _p(os_), _p(od),
                            ctypes.byref(num), secs.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), _p(passes))
    if rc != 0:
        raise MemoryError("oracle ko_ktruss_runs failed")
    return os_[: num.value].copy(), od[: num.value].copy(), secs[:runs].copy(), passes[:runs].copy()


def _batch_graph_job(args):
    """Worker: decompose graphs [g0, g1) of a batch held in shared memory by the reference algorithm
    (chained single-k runs) and return (graph, k_max, sha256 of its per-edge truss numbers)."""
    import hashlib
    from multiprocessing import shared_memory

    names, M, G, g0, g1, method = args
    shm = [shared_memory.SharedMemory(name=x) for x in names]
    try:
        u = np.ndarray((M,), np.uint32, buffer=shm[0].buf)
        v = np.ndarray((M,), np.uint32, buffer=shm[1].buf)
        off = np.ndarray((G + 1,), np.uint32, buffer=shm[2].buf)
        lo = np.searchsorted(u, off[g0:g1], side="left")
        hi = np.searchsorted(u, off[g0 + 1:g1 + 1], side="left")
        out = []
        for i, g in enumerate(range(g0, g1)):
            a, b = int(lo[i]), int(hi[i])
            lu, lv = u[a:b] - off[g], v[a:b] - off[g]
            r = decompose(int(off[g + 1] - off[g]), np.concatenate([lu, lv]), np.concatenate([lv, lu]), method=method,
                          threads=1)
            out.append((g, r["k_max"], hashlib.sha256(r["truss"][: b - a].astype("<u4").tobytes()).hexdigest()))
        return out
    finally:
        for x in shm:
            x.close()


def decompose_batch_processes(u, v, vertex_offsets, workers: int = 0, method: str = "chain", per_task: int = 8):
    """Every graph of a batch (canonical edges u < v, graphs on consecutive vertex ranges) decomposed
    by one single-threaded process per graph at a time, `workers` processes (spawned; the edges are
    shared through shared memory).  Returns ([(graph, k_max, truss sha256)], seconds, workers)."""
    import multiprocessing as mp
    import time
    from multiprocessing import shared_memory

    workers = workers or (len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count())
    arrays = [np.ascontiguousarray(u, np.uint32), np.ascontiguousarray(v, np.uint32),
              np.ascontiguousarray(vertex_offsets, np.uint32)]
    shm = [shared_memory.SharedMemory(create=True, size=max(a.nbytes, 1)) for a in arrays]
    try:
        for a, s_ in zip(arrays, shm):
            np.ndarray(a.shape, a.dtype, buffer=s_.buf)[:] = a
        G = len(arrays[2]) - 1
        tasks = [([x.name for x in shm], len(arrays[0]), G, g, min(g + per_task, G), method)
                 for g in range(0, G, per_task)]
        t0 = time.perf_counter()
        with mp.get_context("spawn").Pool(workers) as pool:
            parts = pool.map(_batch_graph_job, tasks, chunksize=1)
        secs = time.perf_counter() - t0
    finally:
        for x in shm:
            x.close()
            x.unlink()
    return [r for part in parts for r in part], secs, workers


def _peel_job(job):
    n, src, dst = job
    r = decompose(n, src, dst, method="peel", threads=1)
    return r["truss"], r["k_max"]


def decompose_many(jobs, workers: int = 0):
    """Peel decompositions of many graphs [(num_nodes, src, dst), ...] in a process pool started
    with spawn (safe to start after CUDA was initialised in the caller).  Returns [(truss, k_max)]."""
    import multiprocessing as mp

    workers = workers or min(16, mp.cpu_count())
    with mp.get_context("spawn").Pool(workers) as pool:
        return pool.map(_peel_job, jobs, chunksize=1)


def gen_rmat(scale: int, edge_factor: int, a: float = 0.57, b: float = 0.19, c: float = 0.19, seed: int = 1):
    """R-MAT graph of the engine's generator (same arguments, same edges), made without the product
    library.  Returns (num_nodes, u, v): canonical edges u < v sorted by (u, v)."""
    lib = _load()
    cap = edge_factor << scale
    u, v = np.zeros(cap, np.uint32), np.zeros(cap, np.uint32)
    num = ctypes.c_uint64(0)
    if lib.ko_gen_rmat(scale, edge_factor, a, b, c, seed, _p(u), _p(v), ctypes.byref(num)) != 0:
        raise ValueError("oracle ko_gen_rmat: bad arguments or out of memory")
    return 1 << scale, u[: num.value].copy(), v[: num.value].copy()


def chain_sample(num_nodes: int, src, dst, budget_s: float) -> dict:
    """Times the reference algorithm (chained count-and-prune passes) for about budget_s
    seconds; returns the passes completed, their summed alive edges and the seconds taken."""
    lib = _load()
    src, dst = _u32(src), _u32(dst)
    passes, alive, secs = ctypes.c_uint32(0), ctypes.c_uint64(0), ctypes.c_double(0)
    rc = lib.ko_chain_sample(num_nodes, len(src), _p(src), _p(dst), budget_s, ctypes.byref(passes),
                             ctypes.byref(alive), ctypes.byref(secs))
    if rc != 0:
        raise MemoryError("oracle chain sample failed")
    return {"passes": passes.value, "alive_sum": alive.value, "seconds": secs.value}


def tiled_coocsr(num_nodes: int, src, dst, tiles_per_dim: int):
    """Tiled COO/CSR of an entry list, restating coo2tiledcoocsr (graph.cu:641-706) with
    createEmptyTiledCOOCSR's tile size (graph.cu:574-586): tile_size = ceil(n / T); entry (s, d)
    belongs to row (s // tile_size * T + d // tile_size) * tile_size + s % tile_size; rows are
    binned in entry order and each row's destinations sorted ascending.  Returns (tile_src_ptr with
    T*T*tile_size + 1 offsets, src, dst)."""
    src, dst = _u32(src).astype(np.int64), _u32(dst).astype(np.int64)
    T = int(tiles_per_dim)
    ts = (num_nodes + T - 1) // T
    rows = T * T * ts
    tile_src = (src // ts * T + dst // ts) * ts + src % ts
    ptr = np.zeros(rows + 1, np.int64)
    np.add.at(ptr, tile_src + 1, 1)
    ptr = np.cumsum(ptr)
    order = np.lexsort((dst, tile_src))  # by row, then destination (rows hold one source each)
    return ptr.astype(np.uint32), src[order].astype(np.uint32), dst[order].astype(np.uint32)
