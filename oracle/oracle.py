"""numpy wrapper of the CPU oracle (liboracle.so).

TEST INFRASTRUCTURE ONLY: the sequential CPU restatement of the reference services used
to check the CUDA path. Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline
and reference legs may use it. Arrays are numpy (SZ, SX, SY) in [z][x][y] order.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")


class _Pore(ctypes.Structure):
    _fields_ = [("id", ctypes.c_uint32), ("seed_x", ctypes.c_int32), ("seed_y", ctypes.c_int32),
                ("seed_z", ctypes.c_int32), ("seed_r2", ctypes.c_uint32),
                ("is_boundary", ctypes.c_int32), ("volume", ctypes.c_uint64)]


class _Throat(ctypes.Structure):
    _fields_ = [("id", ctypes.c_uint32), ("n_pores", ctypes.c_uint32),
                ("volume", ctypes.c_uint64), ("pool_offset", ctypes.c_uint64)]


class _Cavity(ctypes.Structure):
    _fields_ = [("id", ctypes.c_uint32), ("seed_x", ctypes.c_int32), ("seed_y", ctypes.c_int32),
                ("seed_z", ctypes.c_int32), ("distance_to_center", ctypes.c_float),
                ("reached_walls", ctypes.c_int32), ("void_count", ctypes.c_uint64),
                ("reaches_all_walls", ctypes.c_int32), ("pad_", ctypes.c_int32)]


_lib = None
P = ctypes.c_void_p


def build():
    """Compiles liboracle.so with the Makefile in this folder."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        l = ctypes.CDLL(LIB_PATH)
        l.orc_edt.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_int, P, P, P, ctypes.c_size_t, P]
        l.orc_containing_balls.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                           ctypes.c_uint32, P, P, P, P]
        l.orc_max_ball_mask.argtypes = [P, P, P, ctypes.c_int, ctypes.c_int, ctypes.c_int, P, P]
        l.orc_pores.argtypes = [P, P, P, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, P]
        l.orc_pores.restype = P
        l.orc_sorted_balls.argtypes = [P, P, ctypes.c_int, ctypes.c_int, ctypes.c_int, P, ctypes.c_size_t]
        l.orc_sorted_balls.restype = ctypes.c_size_t
        l.orc_remove_empty_pores.argtypes = [P, P, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        l.orc_watershed.argtypes = [P, P, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                    ctypes.c_uint32, P]
        l.orc_watershed.restype = P
        for name, res in (("npores", ctypes.c_size_t), ("nthroats", ctypes.c_size_t),
                          ("pool_size", ctypes.c_size_t)):
            f = getattr(l, "orc_table_" + name)
            f.argtypes = [P]
            f.restype = res
        l.orc_table_pores.argtypes = [P]
        l.orc_table_pores.restype = ctypes.POINTER(_Pore)
        l.orc_table_throats.argtypes = [P]
        l.orc_table_throats.restype = ctypes.POINTER(_Throat)
        l.orc_table_pool.argtypes = [P]
        l.orc_table_pool.restype = ctypes.POINTER(ctypes.c_uint32)
        l.orc_table_free.argtypes = [P]
        l.orc_table_free.restype = None
        l.orc_table_from_pores.argtypes = [P, ctypes.c_size_t]
        l.orc_table_from_pores.restype = P
        for fn in (l.orc_geodesic_f32, l.orc_geodesic_f64):
            fn.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, P, P, P,
                           ctypes.c_int]
        _lib = l
    return _lib


def _p(a):
    return ctypes.c_void_p(a.ctypes.data)


def _dims(a):
    sz, sx, sy = a.shape
    return sx, sy, sz


def edt(solid):
    """(edt2 uint32, max_edt2, histogram uint64 of length max_edt2+1)."""
    solid = np.ascontiguousarray(solid, dtype=np.uint8)
    out = np.empty(solid.shape, dtype=np.uint32)
    mx = ctypes.c_uint32()
    ln = ctypes.c_size_t()
    sx, sy, sz = _dims(solid)
    cap = 1 << 22
    hist = np.zeros(cap, dtype=np.uint64)
    rc = lib().orc_edt(_p(solid), sx, sy, sz, _p(out), ctypes.byref(mx), _p(hist), cap, ctypes.byref(ln))
    assert rc == 0
    return out, mx.value, hist[:min(ln.value, cap)].copy()


def containing_balls(edt2, max_edt2):
    """(crad2, cx, cy, cz) uint32 arrays."""
    edt2 = np.ascontiguousarray(edt2, dtype=np.uint32)
    sx, sy, sz = _dims(edt2)
    outs = [np.empty(edt2.shape, dtype=np.uint32) for _ in range(4)]
    rc = lib().orc_containing_balls(_p(edt2), sx, sy, sz, max_edt2, *[_p(o) for o in outs])
    assert rc == 0
    return tuple(outs)


def max_ball_mask(cx, cy, cz):
    sx, sy, sz = _dims(cx)
    mask = np.empty(cx.shape, dtype=np.uint8)
    cnt = ctypes.c_uint64()
    rc = lib().orc_max_ball_mask(_p(cx), _p(cy), _p(cz), sx, sy, sz, _p(mask), ctypes.byref(cnt))
    assert rc == 0
    return mask, cnt.value


def _table(h):
    l = lib()
    n = l.orc_table_npores(h)
    pp = l.orc_table_pores(h)
    pores = [(pp[i].id, pp[i].seed_x, pp[i].seed_y, pp[i].seed_z, pp[i].seed_r2,
              pp[i].is_boundary, pp[i].volume) for i in range(n)]
    m = l.orc_table_nthroats(h)
    tp = l.orc_table_throats(h)
    pool = l.orc_table_pool(h)
    throats = [(tp[i].id, tp[i].volume,
                tuple(pool[tp[i].pool_offset + j] for j in range(tp[i].n_pores))) for i in range(m)]
    return pores, throats


def sorted_balls(mask, edt2):
    """Linear indices of the maximum balls in the reference's std::sort order."""
    mask = np.ascontiguousarray(mask, dtype=np.uint8)
    edt2 = np.ascontiguousarray(edt2, dtype=np.uint32)
    sx, sy, sz = _dims(edt2)
    out = np.empty(int((mask == 255).sum()), dtype=np.uint32)
    n = lib().orc_sorted_balls(_p(mask), _p(edt2), sx, sy, sz, _p(out), out.size)
    assert n == out.size
    return out


class PoreResult:
    """Labels and tables of the initial propagation, the removal and the watershed."""


def pores_and_watershed(mask, edt2, crad2, max_edt2, d3q7=False):
    """Runs a8-a12. Returns a PoreResult with labels_initial (before removal), labels
    (after removal), labels_ws, and the tables pores0/throats0 (initial), pores/throats
    (after removal), pores_ws/throats_ws."""
    l = lib()
    sx, sy, sz = _dims(edt2)
    mask = np.ascontiguousarray(mask, dtype=np.uint8)
    edt2 = np.ascontiguousarray(edt2, dtype=np.uint32)
    crad2 = np.ascontiguousarray(crad2, dtype=np.uint32)
    labels = np.zeros(edt2.shape, dtype=np.uint32)
    r = PoreResult()
    h = l.orc_pores(_p(mask), _p(edt2), _p(crad2), sx, sy, sz, int(d3q7), _p(labels))
    r.labels_initial = labels.copy()
    r.pores0, r.throats0 = _table(h)
    assert l.orc_remove_empty_pores(h, _p(labels), sx, sy, sz) == 0
    r.labels = labels
    r.pores, r.throats = _table(h)
    ws = np.zeros(edt2.shape, dtype=np.uint32)
    h2 = l.orc_watershed(h, _p(crad2), sx, sy, sz, int(d3q7), max_edt2, _p(ws))
    r.labels_ws = ws
    r.pores_ws, r.throats_ws = _table(h2)
    l.orc_table_free(h)
    l.orc_table_free(h2)
    return r


def watershed(pore_rows, crad2, max_edt2, d3q7=False):
    """a12 alone: the watershed from pores given as rows (id, x, y, z, r2, boundary, volume).
    Returns (labels_ws, pores_ws, throats_ws)."""
    l = lib()
    crad2 = np.ascontiguousarray(crad2, dtype=np.uint32)
    sx, sy, sz = _dims(crad2)
    arr = (_Pore * max(1, len(pore_rows)))(*[_Pore(*p) for p in pore_rows])
    h = l.orc_table_from_pores(arr, len(pore_rows))
    ws = np.zeros(crad2.shape, dtype=np.uint32)
    h2 = l.orc_watershed(h, _p(crad2), sx, sy, sz, int(d3q7), max_edt2, _p(ws))
    pores, throats = _table(h2)
    l.orc_table_free(h)
    l.orc_table_free(h2)
    return ws, pores, throats


def geodesic(solid, d3q7=False, fp64=False):
    """(dist float32/float64, cavity uint32, cavity rows)."""
    solid = np.ascontiguousarray(solid, dtype=np.uint8)
    sx, sy, sz = _dims(solid)
    dist = np.empty(solid.shape, dtype=np.float64 if fp64 else np.float32)
    cav = np.empty(solid.shape, dtype=np.uint32)
    fn = lib().orc_geodesic_f64 if fp64 else lib().orc_geodesic_f32
    cap = 64
    while True:  # the call returns the number of cavities; rerun with room for all of them
        rows = (_Cavity * cap)()
        n = fn(_p(solid), sx, sy, sz, int(d3q7), _p(dist), _p(cav), rows, cap)
        assert n >= 0
        if n <= cap:
            break
        cap = n
    out = [(c.id, c.seed_x, c.seed_y, c.seed_z, c.distance_to_center, c.void_count,
            c.reached_walls, c.reaches_all_walls) for c in rows[:n]]
    return dist, cav, out


def full(solid, d3q7=False, geodesic_too=True):
    """Every stage on one volume; returns a dict of arrays and tables."""
    e, mx, hist = edt(solid)
    crad2, cx, cy, cz = containing_balls(e, mx)
    mask, nballs = max_ball_mask(cx, cy, cz)
    r = pores_and_watershed(mask, e, crad2, mx, d3q7)
    out = dict(edt2=e, max_edt2=mx, hist=hist, crad2=crad2, cx=cx, cy=cy, cz=cz, mask=mask,
               maximum_balls_count=nballs, pores=r)
    if geodesic_too:
        out["dist"], out["cavity"], out["cavities"] = geodesic(solid, d3q7)
    return out
