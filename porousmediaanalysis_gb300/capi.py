"""ctypes binding of the pma C ABI (include/pma.h).

Loads the in-tree libpma.so built by porousmediaanalysis_gb300/build.py. Loading fails
loudly when the library is missing: there is no CPU fallback.
"""
import ctypes
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libpma.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "pma.h")

c_u8p = ctypes.POINTER(ctypes.c_uint8)
c_u32p = ctypes.POINTER(ctypes.c_uint32)
c_u64p = ctypes.POINTER(ctypes.c_uint64)

PMA_OK = 0
STATUS = {0: "PMA_OK", 1: "PMA_ERR_ARGUMENT", 2: "PMA_ERR_CUDA", 3: "PMA_ERR_IO",
          4: "PMA_ERR_MEMORY", 5: "PMA_ERR_LIMIT", 6: "PMA_ERR_INTERNAL"}
D3Q27, D3Q7 = 0, 1
CUDA_STREAM_LEGACY = 1  # cudaStreamLegacy: the legacy default stream as a stream handle
MODE_ALL, MODE_EDT, MODE_RIB, MODE_APT, MODE_SPD = 1, 2, 3, 4, 5


class Dims(ctypes.Structure):
    _fields_ = [("sx", ctypes.c_int32), ("sy", ctypes.c_int32), ("sz", ctypes.c_int32)]


class EdtStats(ctypes.Structure):
    _fields_ = [("max_edt2", ctypes.c_uint32), ("pad_", ctypes.c_uint32),
                ("hist_len", ctypes.c_uint64)]


class Pore(ctypes.Structure):
    _fields_ = [("id", ctypes.c_uint32), ("seed_x", ctypes.c_int32), ("seed_y", ctypes.c_int32),
                ("seed_z", ctypes.c_int32), ("seed_r2", ctypes.c_uint32),
                ("is_boundary", ctypes.c_int32), ("volume", ctypes.c_uint64)]


class Throat(ctypes.Structure):
    _fields_ = [("id", ctypes.c_uint32), ("n_pores", ctypes.c_uint32),
                ("volume", ctypes.c_uint64), ("pool_offset", ctypes.c_uint64)]


class Cavity(ctypes.Structure):
    _fields_ = [("id", ctypes.c_uint32), ("seed_x", ctypes.c_int32), ("seed_y", ctypes.c_int32),
                ("seed_z", ctypes.c_int32), ("distance_to_center", ctypes.c_float),
                ("reached_walls", ctypes.c_int32), ("void_count", ctypes.c_uint64),
                ("reaches_all_walls", ctypes.c_int32), ("pad_", ctypes.c_int32)]


class Outputs(ctypes.Structure):
    _fields_ = [("edt2", c_u32p), ("crad2", c_u32p), ("cx", c_u32p), ("cy", c_u32p),
                ("cz", c_u32p), ("maxball_mask", c_u8p), ("pore_labels", c_u32p),
                ("watershed_labels", c_u32p), ("dist_f32", ctypes.POINTER(ctypes.c_float)),
                ("dist_f64", ctypes.POINTER(ctypes.c_double)), ("cavity", c_u32p),
                ("edt_stats", EdtStats), ("maximum_balls_count", ctypes.c_uint64),
                ("pores", ctypes.c_void_p), ("watershed", ctypes.c_void_p),
                ("cavities", Cavity * 16), ("n_cavities", ctypes.c_int), ("cavity_rows_cap", ctypes.c_int),
                ("cavity_rows", ctypes.POINTER(Cavity))]


class Limits(ctypes.Structure):
    _fields_ = [("spin_limit", ctypes.c_int32), ("union_limit", ctypes.c_int32),
                ("watershed_generations", ctypes.c_uint64), ("geodesic_buckets", ctypes.c_uint64)]


class Options(ctypes.Structure):
    _fields_ = [("stencil", ctypes.c_int), ("run_pores", ctypes.c_int),
                ("run_geodesic", ctypes.c_int), ("geodesic_fp64", ctypes.c_int)]


class BatchItem(ctypes.Structure):
    _fields_ = [("solid", ctypes.c_void_p), ("dims", Dims), ("status", ctypes.c_int),
                ("out", ctypes.POINTER(Outputs))]


class ServerConfig(ctypes.Structure):
    _fields_ = [("lanes", ctypes.c_int), ("pad_", ctypes.c_int), ("memory_budget", ctypes.c_uint64),
                ("options", Options)]


class ServerStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_uint64), ("completed", ctypes.c_uint64),
                ("failed", ctypes.c_uint64), ("rejected", ctypes.c_uint64), ("queued", ctypes.c_uint64),
                ("peak_reserved_bytes", ctypes.c_uint64), ("resident_bytes", ctypes.c_uint64),
                ("bytes_per_voxel", ctypes.c_double), ("max_in_flight", ctypes.c_uint32),
                ("pad_", ctypes.c_uint32)]


_SIGNATURES = {
    "pma_last_error": (ctypes.c_size_t, [ctypes.c_char_p, ctypes.c_size_t]),
    "pma_abi_version": (ctypes.c_int, []),
    "pma_ctx_create": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]),
    "pma_ctx_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "pma_ctx_set_stream": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "pma_ctx_launch_count": (ctypes.c_uint64, [ctypes.c_void_p]),
    "pma_ctx_scratch_bytes": (ctypes.c_size_t, [ctypes.c_void_p]),
    "pma_ctx_set_timing": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "pma_ctx_timing_report": (ctypes.c_size_t, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_size_t]),
    "pma_ctx_trim": (ctypes.c_int, [ctypes.c_void_p]),
    "pma_ctx_get_limits": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Limits)]),
    "pma_ctx_set_limits": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Limits)]),
    "pma_selftest_bounded_wait": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int)]),
    "pma_ctx_set_throat_numbering": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "pma_edt": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, Dims, ctypes.c_void_p,
                               ctypes.POINTER(EdtStats), ctypes.c_void_p, ctypes.c_size_t]),
    "pma_pipeline_batch": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(BatchItem), ctypes.c_size_t,
                                          ctypes.POINTER(Options), ctypes.c_int, ctypes.c_int]),
    "pma_server_create": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ServerConfig),
                                         ctypes.POINTER(ctypes.c_void_p)]),
    "pma_server_submit": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, Dims, ctypes.POINTER(Outputs),
                                         ctypes.POINTER(ctypes.c_uint64)]),
    "pma_server_wait": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int64,
                                       ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double)]),
    "pma_server_get_stats": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ServerStats)]),
    "pma_server_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "pma_edt_noalloc": (ctypes.c_int, [ctypes.c_void_p, Dims, ctypes.c_void_p, ctypes.POINTER(EdtStats),
                                       ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    "pma_containing_balls": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, Dims, ctypes.c_uint32,
                                            ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                            ctypes.c_void_p, ctypes.c_void_p, c_u64p]),
    "pma_table_create": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p,
                                        ctypes.c_size_t, ctypes.c_void_p, ctypes.c_size_t,
                                        ctypes.POINTER(ctypes.c_void_p)]),
    "pma_table_npores": (ctypes.c_size_t, [ctypes.c_void_p]),
    "pma_table_pores": (ctypes.POINTER(Pore), [ctypes.c_void_p]),
    "pma_table_nthroats": (ctypes.c_size_t, [ctypes.c_void_p]),
    "pma_table_throats": (ctypes.POINTER(Throat), [ctypes.c_void_p]),
    "pma_table_pool_size": (ctypes.c_size_t, [ctypes.c_void_p]),
    "pma_table_pool": (c_u32p, [ctypes.c_void_p]),
    "pma_table_free": (None, [ctypes.c_void_p]),
    "pma_pores": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                 Dims, ctypes.c_int, ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p)]),
    "pma_remove_empty_pores": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, Dims]),
    "pma_watershed": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, Dims,
                                     ctypes.c_int, ctypes.c_uint32, ctypes.c_void_p,
                                     ctypes.POINTER(ctypes.c_void_p)]),
    "pma_geodesic_f32": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, Dims, ctypes.c_int,
                                        ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(Cavity),
                                        ctypes.c_int, ctypes.POINTER(ctypes.c_int)]),
    "pma_geodesic_f64": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, Dims, ctypes.c_int,
                                        ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(Cavity),
                                        ctypes.c_int, ctypes.POINTER(ctypes.c_int)]),
    "pma_pipeline_host": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, Dims,
                                         ctypes.POINTER(Options), ctypes.POINTER(Outputs)]),
    "pma_run_folder": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int]),
    "pma_read_tiff_stack": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_int, ctypes.POINTER(Dims),
                                           ctypes.c_void_p, ctypes.c_size_t]),
    "pma_write_tiff_stack": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_int, Dims, ctypes.c_void_p]),
    "pma_read_config": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_void_p]),
}

_lib = None


class PmaError(RuntimeError):
    def __init__(self, status, message):
        super().__init__("%s: %s" % (STATUS.get(status, status), message))
        self.status = status


def declared_symbols():
    """Function names declared in include/pma.h."""
    text = open(HEADER).read()
    return sorted(set(re.findall(r"\b(pma_[a-z0-9_]+)\s*\(", text)))


def lib():
    """The loaded libpma.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libpma.so is not built; run porousmediaanalysis_gb300/build.py "
                               "(or __graft_entry__.build())")
        l = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in _SIGNATURES.items():
            f = getattr(l, name)
            f.restype = res
            f.argtypes = args
        _lib = l
    return _lib


def last_error():
    buf = ctypes.create_string_buffer(4096)
    lib().pma_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


def check(status):
    if status != PMA_OK:
        raise PmaError(status, last_error())
    return status


def read_tiff_stack(folder, bytes_per_voxel=1):
    """Reads a TIFF-stack folder into a numpy array shaped (SZ, SX, SY)."""
    import numpy as np
    d = Dims()
    check(lib().pma_read_tiff_stack(folder.encode(), bytes_per_voxel, ctypes.byref(d), None, 0))
    dtype = np.uint8 if bytes_per_voxel == 1 else np.uint32
    out = np.empty((d.sz, d.sx, d.sy), dtype=dtype)
    check(lib().pma_read_tiff_stack(folder.encode(), bytes_per_voxel, ctypes.byref(d),
                                    out.ctypes.data, out.nbytes))
    return out


class RunConfig(ctypes.Structure):
    _fields_ = [("resolution", ctypes.c_double * 3), ("max_pore_radius_ratio", ctypes.c_double),
                ("available_memory_mb", ctypes.c_int32), ("use_d3q7", ctypes.c_int32),
                ("threads", ctypes.c_int32), ("pad_", ctypes.c_int32)]


def read_config(path):
    """config.txt of a sample folder as a dict (pma_read_config)."""
    c = RunConfig()
    check(lib().pma_read_config(str(path).encode(), ctypes.byref(c)))
    return {"resolution": tuple(c.resolution), "max_pore_radius_ratio": c.max_pore_radius_ratio,
            "available_memory_mb": c.available_memory_mb, "use_d3q7": c.use_d3q7, "threads": c.threads}


def write_tiff_stack(folder, array):
    """Writes a (SZ, SX, SY) uint8 or 32-bit array as slices 1.tif .. SZ.tif (zero-padded)."""
    import numpy as np
    a = np.ascontiguousarray(array)
    bpv = a.dtype.itemsize
    d = Dims(a.shape[1], a.shape[2], a.shape[0])
    check(lib().pma_write_tiff_stack(folder.encode(), bpv, d, a.ctypes.data))


def table_to_python(handle):
    """(pores, throats) of a pma_table handle as lists of tuples."""
    l = lib()
    n = l.pma_table_npores(handle)
    pp = l.pma_table_pores(handle)
    pores = [(pp[i].id, pp[i].seed_x, pp[i].seed_y, pp[i].seed_z, pp[i].seed_r2,
              pp[i].is_boundary, pp[i].volume) for i in range(n)]
    m = l.pma_table_nthroats(handle)
    tp = l.pma_table_throats(handle)
    pool = l.pma_table_pool(handle)
    throats = []
    for i in range(m):
        t = tp[i]
        throats.append((t.id, t.volume, tuple(pool[t.pool_offset + j] for j in range(t.n_pores))))
    return pores, throats
