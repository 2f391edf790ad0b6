"""GB300-native pore-throat and shortest-path pipeline (PorousMediaAnalysis drop-in).

The compute path is libpma.so: hand-written CUDA kernels for sm_103a behind the C ABI of
include/pma.h. This module wraps that ABI for torch CUDA tensors; torch only provides the
device memory and the stream. Volumes are (SZ, SX, SY) tensors, the reference's [z][x][y]
memory order; uint32 fields are carried in int32 tensors with the same bits.

Stage functions mirror the reference services:
    compute_euclidean_distances   EuclideanDistanceComputer::ComputeEuclideanDistances
    set_containing_balls          ContainingBallsAssigner::SetContainingBalls
    assign_pore_and_throat_ids    PoreAndThroatComputer::AssignPoreAndThroatIds
    remove_empty_pores            EmptyPoresRemover::RemoveEmptyPores
    assign_watershed_ids          WatershedComputer::AssignPoreAndThroatIds
    compute_shortest_path_distances ShortestPathComputer::ComputeShortestPathDistances
    run_folder                    the -all/-edt/-rib/-apt/-spd command-line modes
"""
import ctypes

from . import capi
from .capi import D3Q7, D3Q27, MODE_ALL, MODE_APT, MODE_EDT, MODE_RIB, MODE_SPD, PmaError

__all__ = ["Context", "Table", "compute_euclidean_distances", "set_containing_balls",
           "assign_pore_and_throat_ids", "remove_empty_pores", "assign_watershed_ids",
           "compute_shortest_path_distances", "run_folder", "pipeline_host", "pipeline_batch",
           "Server", "D3Q7", "D3Q27",
           "MODE_ALL", "MODE_EDT", "MODE_RIB", "MODE_APT", "MODE_SPD", "PmaError"]


class Context:
    """One pma_ctx: a device, a stream (torch's current stream) and cached scratch."""

    def __init__(self, device=0, stream=None):
        import torch
        self.device = device
        h = ctypes.c_void_p()
        capi.check(capi.lib().pma_ctx_create(device, ctypes.byref(h)))
        self.handle = h
        if stream is None:
            stream = torch.cuda.current_stream(device)
        self.stream = stream
        handle = stream.cuda_stream
        if handle == 0:  # torch's default stream is CUDA's legacy default stream
            handle = capi.CUDA_STREAM_LEGACY
        capi.check(capi.lib().pma_ctx_set_stream(h, ctypes.c_void_p(handle)))

    def close(self):
        if self.handle:
            capi.lib().pma_ctx_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def launch_count(self):
        return capi.lib().pma_ctx_launch_count(self.handle)

    @property
    def scratch_bytes(self):
        return capi.lib().pma_ctx_scratch_bytes(self.handle)

    def trim(self):
        """Give the scratch cache (this context's and its batch lanes') back to the device."""
        capi.check(capi.lib().pma_ctx_trim(self.handle))

    def set_timing(self, enable=True):
        capi.check(capi.lib().pma_ctx_set_timing(self.handle, int(enable)))

    @property
    def limits(self):
        """Bounds of the device loops: dict of spin_limit, union_limit,
        watershed_generations and geodesic_buckets (pma_limits)."""
        lim = capi.Limits()
        capi.check(capi.lib().pma_ctx_get_limits(self.handle, ctypes.byref(lim)))
        return {name: getattr(lim, name) for name, _ in capi.Limits._fields_}

    def set_limits(self, **kw):
        """Changes some of the loop bounds (others keep their values)."""
        cur = self.limits
        cur.update(kw)
        lim = capi.Limits(**cur)
        capi.check(capi.lib().pma_ctx_set_limits(self.handle, ctypes.byref(lim)))

    def set_throat_numbering(self, reference=True):
        """Shared-type ids of the initial propagation: the reference's creation order (a host
        replay), or the default cheaper order equal to it up to a renaming
        (pma_ctx_set_throat_numbering)."""
        capi.check(capi.lib().pma_ctx_set_throat_numbering(self.handle, int(bool(reference))))

    def selftest_bounded_wait(self):
        """True when a device wait on a flag nothing sets gave up after spin_limit polls and
        reported it (pma_selftest_bounded_wait)."""
        t = ctypes.c_int()
        capi.check(capi.lib().pma_selftest_bounded_wait(self.handle, ctypes.byref(t)))
        return bool(t.value)

    def timing_report(self):
        """{kernel: (total_ms, launches)} of timed kernels since the previous report."""
        import json
        buf = ctypes.create_string_buffer(1 << 16)  # one call: the report is consumed
        capi.lib().pma_ctx_timing_report(self.handle, buf, len(buf))
        return {k: tuple(v) for k, v in json.loads(buf.value.decode()).items()}


class Table:
    """Owning wrapper of a pma_table (pores + throats)."""

    def __init__(self, handle):
        self.handle = handle

    @classmethod
    def from_rows(cls, pores, throats=()):
        pa = (capi.Pore * max(1, len(pores)))()
        for i, p in enumerate(pores):
            pa[i] = capi.Pore(*p)
        pool = []
        ta = (capi.Throat * max(1, len(throats)))()
        for i, (tid, vol, plist) in enumerate(throats):
            ta[i] = capi.Throat(tid, len(plist), vol, len(pool))
            pool.extend(plist)
        pl = (ctypes.c_uint32 * max(1, len(pool)))(*pool)
        h = ctypes.c_void_p()
        capi.check(capi.lib().pma_table_create(pa, len(pores), ta, len(throats), pl, len(pool),
                                               ctypes.byref(h)))
        return cls(h)

    def rows(self):
        return capi.table_to_python(self.handle)

    def counts(self):
        """(number of pores, number of shared types) without converting the rows."""
        return (capi.lib().pma_table_npores(self.handle), capi.lib().pma_table_nthroats(self.handle))

    def __del__(self):
        if getattr(self, "handle", None):
            capi.lib().pma_table_free(self.handle)
            self.handle = None


def _dims(t):
    sz, sx, sy = t.shape
    return capi.Dims(sx, sy, sz)


def _ptr(t):
    assert t.is_cuda and t.is_contiguous()
    return ctypes.c_void_p(t.data_ptr())


def compute_euclidean_distances(ctx, solid, hist_cap=0):
    """Squared EDT of a (SZ, SX, SY) uint8 CUDA tensor (non-zero = solid).
    Returns (edt2 int32 tensor, max_edt2, histogram list)."""
    import torch
    edt2 = torch.empty(solid.shape, dtype=torch.int32, device=solid.device)
    st = capi.EdtStats()
    hist = (ctypes.c_uint64 * max(1, hist_cap))()
    capi.check(capi.lib().pma_edt(ctx.handle, _ptr(solid), _dims(solid), _ptr(edt2),
                                  ctypes.byref(st), hist if hist_cap else None, hist_cap))
    n = min(hist_cap, st.max_edt2 + 1)
    return edt2, st.max_edt2, [hist[i] for i in range(n)]


def set_containing_balls(ctx, edt2, max_edt2):
    """Returns (crad2, cx, cy, cz, maxball_mask, maximum_balls_count)."""
    import torch
    dev = edt2.device
    crad2 = torch.empty(edt2.shape, dtype=torch.int32, device=dev)
    cx = torch.empty_like(crad2)
    cy = torch.empty_like(crad2)
    cz = torch.empty_like(crad2)
    mask = torch.empty(edt2.shape, dtype=torch.uint8, device=dev)
    count = ctypes.c_uint64()
    capi.check(capi.lib().pma_containing_balls(ctx.handle, _ptr(edt2), _dims(edt2), max_edt2,
                                               _ptr(crad2), _ptr(cx), _ptr(cy), _ptr(cz),
                                               _ptr(mask), ctypes.byref(count)))
    return crad2, cx, cy, cz, mask, count.value


def assign_pore_and_throat_ids(ctx, mask, edt2, crad2, stencil=D3Q27):
    """Returns (labels int32 tensor, Table)."""
    import torch
    labels = torch.empty(edt2.shape, dtype=torch.int32, device=edt2.device)
    h = ctypes.c_void_p()
    capi.check(capi.lib().pma_pores(ctx.handle, _ptr(mask), _ptr(edt2), _ptr(crad2), _dims(edt2),
                                    stencil, _ptr(labels), ctypes.byref(h)))
    return labels, Table(h)


def remove_empty_pores(ctx, table, labels):
    capi.check(capi.lib().pma_remove_empty_pores(ctx.handle, table.handle, _ptr(labels),
                                                 _dims(labels)))


def assign_watershed_ids(ctx, table, crad2, max_edt2, stencil=D3Q27):
    """Returns (watershed labels int32 tensor, Table)."""
    import torch
    labels = torch.empty(crad2.shape, dtype=torch.int32, device=crad2.device)
    h = ctypes.c_void_p()
    capi.check(capi.lib().pma_watershed(ctx.handle, table.handle, _ptr(crad2), _dims(crad2),
                                        stencil, max_edt2, _ptr(labels), ctypes.byref(h)))
    return labels, Table(h)


def compute_shortest_path_distances(ctx, solid, stencil=D3Q27, fp64=False, cavity_cap=None):
    """Returns (dist float32/float64 tensor, cavity int32 tensor, cavity rows). Every cavity's
    row is returned; with cavity_cap given, at most that many rows are kept (the rest are
    counted: see shortest_path_with_count)."""
    if cavity_cap is not None:
        return _shortest_path(ctx, solid, stencil, fp64, cavity_cap)[:3]
    dist, cav, out, n = _shortest_path(ctx, solid, stencil, fp64, 64)
    if n > 64:  # more cavities than the first buffer held: run again with room for all
        dist, cav, out, n = _shortest_path(ctx, solid, stencil, fp64, n)
    return dist, cav, out


def shortest_path_with_count(ctx, solid, stencil=D3Q27, fp64=False, cavity_cap=64):
    """(dist, cavity, the first cavity_cap rows, the number of cavities)."""
    return _shortest_path(ctx, solid, stencil, fp64, cavity_cap)


def _shortest_path(ctx, solid, stencil, fp64, cavity_cap):
    import torch
    dist = torch.empty(solid.shape, dtype=torch.float64 if fp64 else torch.float32,
                       device=solid.device)
    cav = torch.empty(solid.shape, dtype=torch.int32, device=solid.device)
    cap = cavity_cap
    rows = (capi.Cavity * cap)()
    n = ctypes.c_int()
    fn = capi.lib().pma_geodesic_f64 if fp64 else capi.lib().pma_geodesic_f32
    capi.check(fn(ctx.handle, _ptr(solid), _dims(solid), stencil, _ptr(dist), _ptr(cav), rows, cap,
                  ctypes.byref(n)))
    out = [(r.id, r.seed_x, r.seed_y, r.seed_z, r.distance_to_center, r.void_count,
            r.reached_walls, r.reaches_all_walls) for r in rows[:min(cap, n.value)]]
    return dist, cav, out, n.value


def run_folder(ctx, base_folder, mode=MODE_ALL):
    capi.check(capi.lib().pma_run_folder(ctx.handle, str(base_folder).encode(), mode))


CAVITY_ROWS = 4096  # cavity rows kept per volume by the pipeline calls

_KINDS = {"edt2": "uint32", "crad2": "uint32", "cx": "uint32", "cy": "uint32", "cz": "uint32",
          "maxball_mask": "uint8", "pore_labels": "uint32", "watershed_labels": "uint32",
          "dist_f32": "float32", "dist_f64": "float64", "cavity": "uint32"}


def _bind_outputs(out, shape, fields, given, device=None):
    """Points the Outputs fields at numpy arrays (device None) or torch CUDA tensors."""
    import numpy as np
    res = dict(given or {})
    for name in fields:
        arr = res.get(name)
        if arr is None:
            if device is None:
                arr = np.empty(shape, dtype=_KINDS[name])
            else:
                import torch
                dt = {"uint32": torch.int32, "uint8": torch.uint8, "float32": torch.float32,
                      "float64": torch.float64}[_KINDS[name]]
                arr = torch.empty(shape, dtype=dt, device=device)
            res[name] = arr
        addr = arr.ctypes.data if device is None else arr.data_ptr()
        setattr(out, name, ctypes.cast(addr, type(getattr(out, name))))
    # room for every cavity row (the call reports how many there are in n_cavities)
    rows = (capi.Cavity * CAVITY_ROWS)()
    res["_cavity_rows"] = rows
    out.cavity_rows = ctypes.cast(rows, ctypes.POINTER(capi.Cavity))
    out.cavity_rows_cap = CAVITY_ROWS
    return res


def _collect(out, res):
    res["max_edt2"] = out.edt_stats.max_edt2
    res["maximum_balls_count"] = out.maximum_balls_count
    res["pores"] = Table(out.pores) if out.pores else None
    res["watershed"] = Table(out.watershed) if out.watershed else None
    rows = res.pop("_cavity_rows")
    if out.n_cavities > CAVITY_ROWS:
        raise PmaError(5, "%d cavities, more rows than the %d kept" % (out.n_cavities, CAVITY_ROWS))
    res["cavities"] = [(c.id, c.seed_x, c.seed_y, c.seed_z, c.distance_to_center, c.void_count,
                        c.reached_walls, c.reaches_all_walls)
                       for c in rows[:out.n_cavities]]
    return res


def pipeline_host(ctx, solid_np, stencil=D3Q27, run_pores=True, run_geodesic=True, fp64=False,
                  fields=("watershed_labels", "dist_f32"), out_arrays=None):
    """Whole pipeline on a host (SZ, SX, SY) uint8 array through pma_pipeline_host (the
    host<->device copies happen inside the call). Returns a dict of numpy outputs for
    `fields` (geodesics in float64 with fp64=True: field "dist_f64"), plus tables and
    statistics. out_arrays may supply preallocated (e.g. pinned) numpy outputs."""
    import numpy as np
    solid_np = np.ascontiguousarray(solid_np, dtype=np.uint8)
    out = capi.Outputs()
    res = _bind_outputs(out, solid_np.shape, fields, out_arrays)
    opts = capi.Options(stencil, int(run_pores), int(run_geodesic), int(fp64))
    capi.check(capi.lib().pma_pipeline_host(ctx.handle, solid_np.ctypes.data, capi.Dims(
        solid_np.shape[1], solid_np.shape[2], solid_np.shape[0]), ctypes.byref(opts),
        ctypes.byref(out)))
    return _collect(out, res)


def pipeline_batch(ctx, volumes, stencil=D3Q27, run_pores=True, run_geodesic=True, fp64=False,
                   fields=("watershed_labels", "dist_f32"), resident=False, lanes=0, out_arrays=None):
    """Whole pipeline on many independent (SZ, SX, SY) volumes through pma_pipeline_batch.
    Host numpy volumes give numpy outputs; with resident=True the volumes are uint8 CUDA
    tensors and the outputs CUDA tensors (uint32 fields in int32 tensors). Returns one dict
    per volume, as pipeline_host does. out_arrays may supply one dict of outputs per volume."""
    import numpy as np
    n = len(volumes)
    items = (capi.BatchItem * max(n, 1))()
    outs = [capi.Outputs() for _ in range(n)]
    results, keep = [], []
    for i, v in enumerate(volumes):
        if resident:
            assert v.is_cuda and v.is_contiguous() and v.dtype.itemsize == 1
            addr, shape, dev = v.data_ptr(), tuple(v.shape), v.device
        else:
            v = np.ascontiguousarray(v, dtype=np.uint8)
            addr, shape, dev = v.ctypes.data, v.shape, None
        keep.append(v)
        given = out_arrays[i] if out_arrays else None
        results.append(_bind_outputs(outs[i], shape, fields, given, dev))
        items[i].solid = addr
        items[i].dims = capi.Dims(shape[1], shape[2], shape[0])
        items[i].out = ctypes.pointer(outs[i])
    opts = capi.Options(stencil, int(run_pores), int(run_geodesic), int(fp64))
    status = capi.lib().pma_pipeline_batch(ctx.handle, items, n, ctypes.byref(opts), int(resident),
                                           int(lanes))
    res = [_collect(outs[i], results[i]) for i in range(n)]
    capi.check(status)
    return res


class Server:
    """Request loop with continuous batching (pma_server_*): volumes are admitted in arrival
    order as lanes and device memory free up, and run concurrently on the device."""

    def __init__(self, ctx, lanes=8, memory_budget=0, stencil=D3Q27, run_pores=True,
                 run_geodesic=True, fp64=False):
        cfg = capi.ServerConfig(lanes, 0, memory_budget,
                                capi.Options(stencil, int(run_pores), int(run_geodesic), int(fp64)))
        h = ctypes.c_void_p()
        capi.check(capi.lib().pma_server_create(ctx.handle, ctypes.byref(cfg), ctypes.byref(h)))
        self.handle = h
        self._pending = {}

    def submit(self, solid_np, fields=("watershed_labels", "dist_f32"), out_arrays=None):
        """Queues a host (SZ, SX, SY) volume; returns its ticket."""
        import numpy as np
        solid_np = np.ascontiguousarray(solid_np, dtype=np.uint8)
        out = capi.Outputs()
        res = _bind_outputs(out, solid_np.shape, fields, out_arrays)
        t = ctypes.c_uint64()
        capi.check(capi.lib().pma_server_submit(self.handle, solid_np.ctypes.data, capi.Dims(
            solid_np.shape[1], solid_np.shape[2], solid_np.shape[0]), ctypes.byref(out), ctypes.byref(t)))
        self._pending[t.value] = (solid_np, out, res)
        return t.value

    def wait(self, ticket, timeout_ms=-1):
        """(result dict as pipeline_host returns, latency in ms); raises PmaError on failure."""
        status = ctypes.c_int()
        lat = ctypes.c_double()
        capi.check(capi.lib().pma_server_wait(self.handle, ticket, timeout_ms, ctypes.byref(status),
                                              ctypes.byref(lat)))
        _, out, res = self._pending.pop(ticket)
        res = _collect(out, res)
        capi.check(status.value)
        return res, lat.value

    def stats(self):
        st = capi.ServerStats()
        capi.check(capi.lib().pma_server_get_stats(self.handle, ctypes.byref(st)))
        return {name: getattr(st, name) for name, _ in capi.ServerStats._fields_ if name != "pad_"}

    def close(self):
        if getattr(self, "handle", None):
            capi.check(capi.lib().pma_server_destroy(self.handle))
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
