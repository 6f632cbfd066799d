"""ORACLE -- test infrastructure only.  Python driver of the C restatement
in oracle/models.c (see its header for what it restates and how it is
pinned).  Used as the checker; never by the product."""
import ctypes as C
import os

import numpy as np

from . import build as _build

_L = None


def lib():
    global _L
    if _L is None:
        _L = C.CDLL(_build.build())
        u64p, u32p, i64, u8p, i32p, f64p = (C.c_void_p,) * 6
        _L.or_build_inedges.argtypes = [C.c_int64, C.c_int64, C.c_void_p, C.c_void_p,
                                        C.c_void_p, C.c_void_p, C.c_void_p]
        _L.or_sir_step.argtypes = [C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                   C.c_void_p, C.c_void_p, C.c_double, C.c_int32, C.c_uint64,
                                   C.c_uint32, C.c_int]
        _L.or_opinion_step.argtypes = [C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                       C.c_void_p, C.c_double, C.c_double, C.c_double, C.c_int]
        _L.or_life_step.argtypes = [C.c_int64, C.c_int64, C.c_void_p, C.c_void_p, C.c_int]
        _L.or_life_step_p.argtypes = [C.c_int64, C.c_int64, C.c_int, C.c_void_p, C.c_void_p,
                                      C.c_int]
        _L.or_walk_step.argtypes = [C.c_int64, C.c_int64, C.c_int64, C.c_void_p, C.c_void_p,
                                    C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint64, C.c_uint32,
                                    C.c_int]
        _L.or_philox.argtypes = [C.c_uint32] * 4 + [C.c_uint64, C.c_void_p]
        _L.or_gen_chung_lu.argtypes = [C.c_uint64, C.c_uint64, C.c_double, C.c_double,
                                       C.c_double, C.c_uint64, C.c_int, C.c_void_p, C.c_void_p,
                                       C.c_void_p, C.c_int]
        _L.or_gen_uniform_out.argtypes = [C.c_uint64, C.c_uint32, C.c_uint64, C.c_int,
                                          C.c_void_p, C.c_void_p]
    return _L


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def threads():
    return int(os.environ.get("ORACLE_THREADS", os.cpu_count() or 1))


def philox(c0, c1, c2, c3, seed):
    out = np.zeros(4, dtype=np.uint32)
    lib().or_philox(c0, c1, c2, c3, seed, _p(out))
    return out


def gen_chung_lu(n, nedges, mean, gamma, wmax, seed, type_nr=1):
    """Host restatement of the device Chung-Lu generator: (from, to, w)."""
    frm = np.zeros(nedges, dtype=np.uint64)
    to = np.zeros(nedges, dtype=np.uint64)
    w = np.zeros(nedges, dtype=np.float64)
    if lib().or_gen_chung_lu(n, nedges, mean, gamma, wmax, seed, type_nr, _p(frm), _p(to),
                             _p(w), threads()):
        raise MemoryError("oracle generator")
    return frm, to, w


def gen_uniform_out(n, k, seed, type_nr=1):
    frm = np.zeros(n * k, dtype=np.uint64)
    to = np.zeros(n * k, dtype=np.uint64)
    lib().or_gen_uniform_out(n, k, seed, type_nr, _p(frm), _p(to))
    return frm, to


def build_inedges(n, frm, to):
    """Per-target in-edge lists in add_edge! call order: (rowptr, src, rec)."""
    frm = np.ascontiguousarray(frm, dtype=np.uint64)
    to = np.ascontiguousarray(to, dtype=np.uint64)
    E = to.size
    rowptr = np.zeros(n + 1, dtype=np.uint64)
    src = np.zeros(max(E, 1), dtype=np.uint32)
    rec = np.zeros(max(E, 1), dtype=np.uint64)
    rc = lib().or_build_inedges(n, E, _p(frm), _p(to), _p(rowptr), _p(src), _p(rec))
    if rc:
        raise ValueError("edge target outside 1..n")
    return rowptr, src[:E], rec[:E]


def sir_step(g, state, days, beta, recovery, seed, step, nthreads=None):
    rowptr, src, _ = g
    n = state.size
    so = np.empty_like(state)
    do = np.empty_like(days)
    lib().or_sir_step(n, _p(rowptr), _p(src), _p(state), _p(days), _p(so), _p(do), beta,
                      recovery, seed, step, nthreads or threads())
    return so, do


def run_sir(n, frm, to, state, days, beta, recovery, seed, steps, first_step=1):
    g = build_inedges(n, frm, to)
    s, d = np.ascontiguousarray(state, np.uint8), np.ascontiguousarray(days, np.int32)
    for t in range(steps):
        s, d = sir_step(g, s, d, beta, recovery, seed, first_step + t)
    return s, d


def opinion_step(g, w_in_order, x, eps, a=0.5, b=0.5, nthreads=None):
    rowptr, src, _ = g
    xo = np.empty_like(x)
    lib().or_opinion_step(x.size, _p(rowptr), _p(src), _p(w_in_order), _p(x), _p(xo), eps, a, b,
                          nthreads or threads())
    return xo


def run_opinion(n, frm, to, w, x, eps, steps, a=0.5, b=0.5):
    g = build_inedges(n, frm, to)
    w_in_order = np.ascontiguousarray(np.asarray(w, dtype=np.float64)[g[2]])
    x = np.ascontiguousarray(x, dtype=np.float64)
    for _ in range(steps):
        x = opinion_step(g, w_in_order, x, eps, a, b)
    return x


def life_step(alive, W, H, nthreads=None, periodic=True):
    a = np.ascontiguousarray(alive, dtype=np.uint8)
    o = np.empty_like(a)
    lib().or_life_step_p(W, H, int(bool(periodic)), _p(a), _p(o), nthreads or threads())
    return o


def walk_step(x, y, W, H, seed, step, nthreads=None):
    n = x.size
    xo, yo = np.empty_like(x), np.empty_like(y)
    cell = np.empty(n, dtype=np.int64)
    lib().or_walk_step(n, W, H, _p(x), _p(y), _p(xo), _p(yo), _p(cell), seed, step,
                       nthreads or threads())
    return xo, yo, cell


def run_life_walkers(alive, x, y, W, H, seed, steps, first_step=1):
    """One model step = apply!(life) then apply!(random_walk); the walk runs
    at transition number first_step + 2t + 1.  Returns the final cells,
    walker positions and the walker -> cell edge lists of the last step
    (per cell, walker numbers in call order)."""
    a = np.ascontiguousarray(alive, dtype=np.uint8)
    x = np.ascontiguousarray(x, dtype=np.int32)
    y = np.ascontiguousarray(y, dtype=np.int32)
    cell = (x.astype(np.int64) - 1) + (y.astype(np.int64) - 1) * W
    for t in range(steps):
        a = life_step(a, W, H)
        x, y, cell = walk_step(x, y, W, H, seed, first_step + 2 * t + 1)
    n = x.size
    order = np.argsort(cell, kind="stable")  # per-cell lists in walker order
    counts = np.bincount(cell, minlength=W * H)
    rowptr = np.zeros(W * H + 1, dtype=np.uint64)
    rowptr[1:] = np.cumsum(counts)
    return a, x, y, rowptr, (order + 1).astype(np.uint64)
