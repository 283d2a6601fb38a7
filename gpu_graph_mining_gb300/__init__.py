"""GB300 gSpan frequent-subgraph miner: Python bindings over the C ABI.

The native library (``_lib/libgspan_gb300.so``, built by ``build.py``) does
all the work; this module only marshals arguments through ctypes.  There is
no Python or CPU fallback: if the library is missing, every call raises.

The classes mirror the reference's mining interface
(``gspan_cuda::gspan_cuda`` in src/gspan_cuda/gspan_cuda.hpp:53,284-292):
``GSpanMiner.set_database / set_min_support / set_graph_output / run``, with
the output sink receiving ``(DFS code, support)`` once per frequent pattern
like ``graph_output::output_graph`` (src/globals/graph_output.hpp:12).
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libgspan_gb300.so")
CLI_PATH = os.path.join(_HERE, "_lib", "gspan_gb300")

TXT, BIN, FSG, CUDABIN = 0, 1, 2, 3
LABELS_FULL, LABELS_SEQ = 0, 1

STATUS_NAMES = {
    0: "GS_OK", 1: "GS_ERR_USAGE", 2: "GS_ERR_IO", 3: "GS_ERR_FORMAT", 4: "GS_ERR_CUDA",
    5: "GS_ERR_NOMEM", 6: "GS_ERR_MINSUP_TOO_LARGE", 7: "GS_ERR_MINSUP_TOO_SMALL", 8: "GS_ERR_LIMIT",
    9: "GS_ERR_TIMEOUT", 10: "GS_ERR_CANCELLED", 11: "GS_ERR_BUDGET", 12: "GS_ERR_STATE",
}

# every symbol include/gspan_gb300.h declares
EXPORTS = [
    "gs_last_error", "gs_filetype_from_name", "gs_db_load", "gs_db_from_arrays", "gs_db_from_arrays_device",
    "gs_db_generate", "gs_db_convert",
    "gs_db_write", "gs_db_size", "gs_db_get_info", "gs_db_upload", "gs_db_free", "gs_mine_opts_default",
    "gs_mine", "gs_mine_ex", "gs_mine_collect", "gs_patterns_free", "gs_mine_batch", "gs_support_count",
    "gs_filter_backward", "gs_segmented_scan", "gs_segmented_reduce",
    "gs_support_count_noalloc",
    "gs_dfs_code_is_min", "gs_engine_reset", "gs_engine_set_pool_bytes",
    "gs_server_opts_default", "gs_server_create", "gs_server_add_db", "gs_server_submit", "gs_server_poll",
    "gs_server_cancel", "gs_server_get_stats", "gs_server_destroy", "gs_autotune",
]


class GSpanError(RuntimeError):
    def __init__(self, status, message):
        super().__init__("%s: %s" % (STATUS_NAMES.get(status, status), message))
        self.status = status


class MineOpts(ctypes.Structure):
    _fields_ = [("max_edges", ctypes.c_int32), ("label_style", ctypes.c_int32),
                ("wave_nodes", ctypes.c_int32), ("threads", ctypes.c_int32),
                ("wave_rows", ctypes.c_int64), ("wave_words", ctypes.c_int64),
                ("root_part", ctypes.c_int32), ("root_parts", ctypes.c_int32),
                ("min_check", ctypes.c_int32), ("launch_mode", ctypes.c_int32),
                ("count_grid", ctypes.c_int32), ("extension", ctypes.c_int32),
                ("deep_nodes", ctypes.c_int32), ("serial", ctypes.c_int32), ("schedulers", ctypes.c_int32)]


# extension strategies (gs_mine_opts.extension)
EXTENSION_RMPATH = 0
EXTENSION_LISTS = 1
EXTENSION_AUTO = 2


class ConvertInfo(ctypes.Structure):
    _fields_ = [("graphs", ctypes.c_int64), ("graphs_fixed", ctypes.c_int64), ("graphs_renumbered", ctypes.c_int64),
                ("vertex_labels", ctypes.c_int32), ("edge_labels", ctypes.c_int32)]


class TuneReport(ctypes.Structure):
    _fields_ = [("trials", ctypes.c_int32), ("wave_nodes", ctypes.c_int32), ("wave_rows", ctypes.c_int64),
                ("count_grid", ctypes.c_int32), ("deep_nodes", ctypes.c_int32), ("base_ms", ctypes.c_double),
                ("best_ms", ctypes.c_double), ("schedulers", ctypes.c_int32)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class MineStats(ctypes.Structure):
    _fields_ = [("patterns", ctypes.c_int64), ("waves", ctypes.c_int64), ("launches", ctypes.c_int64),
                ("nodes", ctypes.c_int64), ("rows", ctypes.c_int64), ("extensions", ctypes.c_int64),
                ("candidates", ctypes.c_int64), ("count_bytes", ctypes.c_int64), ("mat_bytes", ctypes.c_int64),
                ("count_ms", ctypes.c_double), ("mat_ms", ctypes.c_double), ("support_ms", ctypes.c_double),
                ("root_ms", ctypes.c_double), ("host_min_ms", ctypes.c_double), ("wall_ms", ctypes.c_double),
                ("peak_pool_bytes", ctypes.c_int64), ("h2d_bytes", ctypes.c_int64), ("d2h_bytes", ctypes.c_int64),
                ("host_build_ms", ctypes.c_double), ("host_wait_ms", ctypes.c_double),
                ("host_select_ms", ctypes.c_double), ("host_emit_ms", ctypes.c_double),
                ("min_host_checks", ctypes.c_int64), ("list_entries", ctypes.c_int64),
                ("join_nodes", ctypes.c_int64), ("sel_bytes", ctypes.c_int64), ("sel_ms", ctypes.c_double),
                ("min_ms", ctypes.c_double)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class DbInfo(ctypes.Structure):
    _fields_ = [("graphs", ctypes.c_int64), ("vertices", ctypes.c_int64),
                ("adjacency_entries", ctypes.c_int64), ("vertex_labels", ctypes.c_int32),
                ("edge_labels", ctypes.c_int32), ("device_bytes", ctypes.c_int64)]


class Patterns(ctypes.Structure):
    _fields_ = [("count", ctypes.c_int64), ("n_tuples", ctypes.c_int64),
                ("offset", ctypes.POINTER(ctypes.c_int64)), ("dfs", ctypes.POINTER(ctypes.c_int32)),
                ("support", ctypes.POINTER(ctypes.c_int64))]


class ServerOpts(ctypes.Structure):
    _fields_ = [("budget_bytes", ctypes.c_int64), ("pool_bytes", ctypes.c_int64),
                ("max_active", ctypes.c_int32), ("wave_nodes", ctypes.c_int32),
                ("threads", ctypes.c_int32), ("label_style", ctypes.c_int32),
                ("extension", ctypes.c_int32), ("reserved", ctypes.c_int32)]


class RequestInfo(ctypes.Structure):
    _fields_ = [("state", ctypes.c_int32), ("status", ctypes.c_int32), ("patterns", ctypes.c_int64),
                ("queue_ms", ctypes.c_double), ("latency_ms", ctypes.c_double), ("peak_bytes", ctypes.c_int64)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class ServerStats(ctypes.Structure):
    _fields_ = [(f, ctypes.c_int64) for f in ("submitted", "completed", "cancelled", "failed", "queued",
                                              "running", "max_running", "patterns")] + \
               [(f, ctypes.c_double) for f in ("p50_ms", "p99_ms", "mean_ms", "wall_ms", "busy_ms")] + \
               [(f, ctypes.c_int64) for f in ("budget_bytes", "reserved_bytes", "pool_used_bytes",
                                              "peak_pool_bytes", "waves", "launches")]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


REQ_QUEUED, REQ_RUNNING, REQ_DONE, REQ_CANCELLED, REQ_FAILED = range(5)

EMIT_FN = ctypes.CFUNCTYPE(None, ctypes.POINTER(ctypes.c_int32), ctypes.c_int32, ctypes.c_int64, ctypes.c_void_p)
BATCH_EMIT_FN = ctypes.CFUNCTYPE(None, ctypes.c_int32, ctypes.POINTER(ctypes.c_int32), ctypes.c_int32,
                                 ctypes.c_int64, ctypes.c_void_p)

_lib = None


def lib():
    """Loads the native library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError("native library missing: %s (run gpu_graph_mining_gb300/build.py)" % LIB_PATH)
    L = ctypes.CDLL(LIB_PATH)
    i32, i64, vp = ctypes.c_int32, ctypes.c_int64, ctypes.c_void_p
    pi32 = ctypes.POINTER(ctypes.c_int32)
    L.gs_last_error.restype = ctypes.c_char_p
    L.gs_filetype_from_name.argtypes = [ctypes.c_char_p]
    L.gs_filetype_from_name.restype = i32
    L.gs_db_load.argtypes = [ctypes.c_char_p, i32, pi32]
    L.gs_db_load.restype = vp
    L.gs_db_from_arrays.argtypes = [i32, i32, i32, i32, pi32, pi32, pi32, pi32, pi32]
    L.gs_db_from_arrays.restype = vp
    L.gs_db_from_arrays_device.argtypes = [i32, i32, i32, i32, pi32, pi32, pi32, pi32, pi32]
    L.gs_db_from_arrays_device.restype = vp
    L.gs_db_generate.argtypes = [i32, ctypes.c_uint64, ctypes.c_double, pi32]
    L.gs_db_generate.restype = vp
    L.gs_db_write.argtypes = [vp, ctypes.c_char_p, i32]
    L.gs_db_write.restype = i32
    L.gs_db_size.argtypes = [vp]
    L.gs_db_size.restype = i32
    L.gs_db_get_info.argtypes = [vp, ctypes.POINTER(DbInfo)]
    L.gs_db_get_info.restype = i32
    L.gs_db_upload.argtypes = [vp]
    L.gs_db_upload.restype = i32
    L.gs_db_free.argtypes = [vp]
    L.gs_db_free.restype = None
    L.gs_mine_opts_default.argtypes = [ctypes.POINTER(MineOpts)]
    L.gs_mine_opts_default.restype = None
    L.gs_mine.argtypes = [vp, i32, i32, EMIT_FN, vp]
    L.gs_mine.restype = i32
    L.gs_mine_ex.argtypes = [vp, i32, ctypes.POINTER(MineOpts), EMIT_FN, vp, ctypes.POINTER(MineStats)]
    L.gs_mine_ex.restype = i32
    L.gs_mine_collect.argtypes = [vp, i32, ctypes.POINTER(MineOpts), ctypes.POINTER(ctypes.POINTER(Patterns)),
                                  ctypes.POINTER(MineStats)]
    L.gs_mine_collect.restype = i32
    L.gs_patterns_free.argtypes = [ctypes.POINTER(Patterns)]
    L.gs_patterns_free.restype = None
    L.gs_mine_batch.argtypes = [ctypes.POINTER(vp), i32, pi32, ctypes.POINTER(MineOpts), BATCH_EMIT_FN, vp,
                                ctypes.POINTER(MineStats)]
    L.gs_mine_batch.restype = i32
    L.gs_support_count.argtypes = [pi32, pi32, i64, i32, i32, pi32]
    L.gs_support_count.restype = i32
    L.gs_filter_backward.argtypes = [pi32, i64, pi32, i64, pi32, pi32, ctypes.POINTER(i64)]
    L.gs_filter_backward.restype = i32
    pu32 = ctypes.POINTER(ctypes.c_uint32)
    L.gs_segmented_scan.argtypes = [pu32, i64, i32, pu32]
    L.gs_segmented_scan.restype = i32
    L.gs_segmented_reduce.argtypes = [pu32, i64, pu32, pu32, i32, i32, pu32, ctypes.POINTER(i64)]
    L.gs_segmented_reduce.restype = i32
    L.gs_support_count_noalloc.argtypes = [vp, vp, i64, i32, i32, vp, vp]
    L.gs_support_count_noalloc.restype = i32
    L.gs_dfs_code_is_min.argtypes = [pi32, i32]
    L.gs_dfs_code_is_min.restype = i32
    L.gs_engine_reset.argtypes = []
    L.gs_engine_reset.restype = None
    L.gs_engine_set_pool_bytes.argtypes = [i64]
    L.gs_engine_set_pool_bytes.restype = None
    L.gs_server_opts_default.argtypes = [ctypes.POINTER(ServerOpts)]
    L.gs_server_opts_default.restype = None
    L.gs_server_create.argtypes = [ctypes.POINTER(ServerOpts), ctypes.POINTER(vp)]
    L.gs_server_create.restype = i32
    L.gs_server_add_db.argtypes = [vp, vp, pi32]
    L.gs_server_add_db.restype = i32
    L.gs_server_submit.argtypes = [vp, i32, i32, i32, ctypes.POINTER(i64)]
    L.gs_server_submit.restype = i32
    L.gs_server_poll.argtypes = [vp, i64, i32, ctypes.POINTER(RequestInfo), ctypes.POINTER(ctypes.POINTER(Patterns))]
    L.gs_server_poll.restype = i32
    L.gs_server_cancel.argtypes = [vp, i64]
    L.gs_server_cancel.restype = i32
    L.gs_server_get_stats.argtypes = [vp, ctypes.POINTER(ServerStats)]
    L.gs_server_get_stats.restype = i32
    L.gs_server_destroy.argtypes = [vp]
    L.gs_server_destroy.restype = None
    L.gs_autotune.argtypes = [ctypes.POINTER(vp), i32, pi32, ctypes.POINTER(MineOpts), ctypes.POINTER(TuneReport)]
    L.gs_autotune.restype = i32
    L.gs_db_convert.argtypes = [ctypes.c_char_p, i32, ctypes.c_char_p, i32, ctypes.POINTER(ConvertInfo)]
    L.gs_db_convert.restype = i32
    _lib = L
    return L


def _check(status):
    if status != 0:
        raise GSpanError(status, lib().gs_last_error().decode(errors="replace"))


def filetype(name):
    if isinstance(name, int):
        return name
    ft = lib().gs_filetype_from_name(name.encode())
    if ft < 0:
        raise ValueError("unknown filetype %r" % name)
    return ft


class Database:
    """A graph database (host copy plus, once mined or uploaded, its HBM copy)."""

    def __init__(self, handle):
        self._h = handle

    @classmethod
    def load(cls, path, ftype="txt"):
        st = ctypes.c_int32(0)
        h = lib().gs_db_load(os.fsencode(path), filetype(ftype), ctypes.byref(st))
        if not h:
            _check(st.value or 2)
        return cls(h)

    @classmethod
    def generate(cls, config, seed=0, scale=1.0):
        st = ctypes.c_int32(0)
        h = lib().gs_db_generate(int(config), int(seed), float(scale), ctypes.byref(st))
        if not h:
            _check(st.value or 1)
        return cls(h)

    @classmethod
    def from_arrays(cls, db_size, max_graph_vertex_count, edges, edges_labels, vertex_labels, vertex_offsets,
                    vertex_count=-1, device=False):
        """The reference's cudabin arrays (graph_database_cuda): int32 numpy arrays
        or sequences.  device=True converts on the GPU (gs_db_from_arrays_device)."""
        import numpy as np
        keep = [np.ascontiguousarray(np.asarray(x, dtype=np.int32))
                for x in (edges, edges_labels, vertex_labels, vertex_offsets)]
        P = ctypes.POINTER(ctypes.c_int32)
        e, el, vl, vo = (x.ctypes.data_as(P) for x in keep)
        st = ctypes.c_int32(0)
        fn = lib().gs_db_from_arrays_device if device else lib().gs_db_from_arrays
        h = fn(int(db_size), int(keep[0].size), int(max_graph_vertex_count), int(vertex_count), e, el, vl, vo,
               ctypes.byref(st))
        if not h:
            _check(st.value or 3)
        return cls(h)

    def write(self, path, ftype="txt"):
        _check(lib().gs_db_write(self._h, os.fsencode(path), filetype(ftype)))

    def __len__(self):
        return lib().gs_db_size(self._h)

    def info(self):
        i = DbInfo()
        _check(lib().gs_db_get_info(self._h, ctypes.byref(i)))
        return {f: getattr(i, f) for f, _ in DbInfo._fields_}

    def upload(self):
        _check(lib().gs_db_upload(self._h))

    def free(self):
        if self._h:
            lib().gs_db_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    @property
    def handle(self):
        if not self._h:
            raise ValueError("database freed")
        return self._h


def code_to_string(code):
    """'(f t fl el tl);...' as DFSCode::to_string(false) (src/globals/dfs_code.cpp:199-216)."""
    return ";".join("(%d %d %d %d %d)" % tuple(d) for d in code)


def _extension(x):
    if x in (EXTENSION_RMPATH, "rmpath", None):
        return EXTENSION_RMPATH
    if x in (EXTENSION_AUTO, "auto"):
        return EXTENSION_AUTO
    if x in (EXTENSION_LISTS, "lists"):
        return EXTENSION_LISTS
    raise ValueError("extension must be 'auto', 'rmpath' or 'lists'")


def _opts(max_edges=0, label_style=LABELS_FULL, wave_nodes=None, threads=0, wave_rows=0, wave_words=0,
          root_part=0, root_parts=1, min_check=0, launch_mode=0, count_grid=0, extension=EXTENSION_RMPATH,
          deep_nodes=0, serial=0, schedulers=0):
    o = MineOpts()
    lib().gs_mine_opts_default(ctypes.byref(o))
    o.max_edges = int(max_edges)
    o.label_style = int(label_style)
    if wave_nodes is not None:
        o.wave_nodes = int(wave_nodes)
    if threads:
        o.threads = int(threads)
    if wave_rows:
        o.wave_rows = int(wave_rows)
    if wave_words:
        o.wave_words = int(wave_words)
    o.root_part = int(root_part)
    o.root_parts = int(root_parts)
    o.min_check = int(min_check)
    o.launch_mode = int(launch_mode)
    o.count_grid = int(count_grid)
    o.extension = _extension(extension)
    if deep_nodes:
        o.deep_nodes = int(deep_nodes)
    o.serial = 1 if serial else 0
    o.schedulers = int(schedulers)
    return o


def mine(db, minsup, max_edges=0, label_style=LABELS_FULL, wave_nodes=None, threads=0, collect=True, sink=None,
         wave_rows=0, wave_words=0, root_part=0, root_parts=1, min_check=0, launch_mode=0, count_grid=0,
         extension=EXTENSION_RMPATH, deep_nodes=0, serial=0, schedulers=0):
    """Mines db at absolute support minsup.

    Returns (patterns, stats): patterns is a list of (code, support) with code a
    tuple of 5-tuples, in the reference's traversal order (empty when
    collect=False); sink(code, support) is called per pattern if given.
    extension: "rmpath" (default), "lists" (the reference's lists (intersection)
    strategy) or "auto" (the lists for the waves whose databases do not stay in L2).
    """
    out = []

    def cb(ptr, n, support, user):
        code = tuple(tuple(ptr[5 * i + j] for j in range(5)) for i in range(n))
        if collect:
            out.append((code, support))
        if sink is not None:
            sink(code, support)

    fn = EMIT_FN(cb) if (collect or sink is not None) else ctypes.cast(None, EMIT_FN)
    o = _opts(max_edges, label_style, wave_nodes, threads, wave_rows, wave_words, root_part, root_parts, min_check,
              launch_mode, count_grid, extension, deep_nodes, serial, schedulers)
    st = MineStats()
    _check(lib().gs_mine_ex(db.handle, int(minsup), ctypes.byref(o), fn, None, ctypes.byref(st)))
    return out, st.as_dict()


def mine_collect(db, minsup, decode=True, **kw):
    """Bulk form (gs_mine_collect): all patterns land in one native host buffer.

    Returns (patterns, stats); with decode=False the buffer is freed without
    converting it to Python objects and patterns is its pattern count.
    """
    o = _opts(**kw)
    st = MineStats()
    p = ctypes.POINTER(Patterns)()
    _check(lib().gs_mine_collect(db.handle, int(minsup), ctypes.byref(o), ctypes.byref(p), ctypes.byref(st)))
    return _take_patterns(p, decode), st.as_dict()


def _take_patterns(p, decode=True):
    """Converts a native gs_patterns buffer to [(code, support)] and frees it."""
    try:
        P = p.contents
        if not decode:
            return P.count
        import numpy as np
        off = np.ctypeslib.as_array(P.offset, shape=(P.count + 1,)).copy() if P.count else np.zeros(1, np.int64)
        dfs = (np.ctypeslib.as_array(P.dfs, shape=(5 * P.n_tuples,)).reshape(-1, 5).copy()
               if P.n_tuples else np.zeros((0, 5), np.int32))
        sup = np.ctypeslib.as_array(P.support, shape=(P.count,)).copy() if P.count else np.zeros(0, np.int64)
        return [(tuple(tuple(int(x) for x in row) for row in dfs[off[i]:off[i + 1]]), int(sup[i]))
                for i in range(P.count)]
    finally:
        lib().gs_patterns_free(p)


def convert_database(in_path, in_type, out_path, out_type):
    """The reference's convertdb (gs_db_convert): read, apply the fix_database
    repairs, write.  Returns the counts of graphs written, repaired and
    renumbered, and of labels."""
    info = ConvertInfo()
    _check(lib().gs_db_convert(os.fsencode(in_path), filetype(in_type), os.fsencode(out_path), filetype(out_type),
                               ctypes.byref(info)))
    return {f: getattr(info, f) for f, _ in info._fields_}


def autotune(dbs, minsups, **kw):
    """Picks wave options for mining these databases together (gs_autotune).
    Returns (options for mine / mine_batch / mine_collect, report)."""
    o = _opts(**kw)
    hs = (ctypes.c_void_p * len(dbs))(*[d.handle for d in dbs])
    ms = (ctypes.c_int32 * len(dbs))(*[int(m) for m in minsups])
    r = TuneReport()
    _check(lib().gs_autotune(hs, len(dbs), ms, ctypes.byref(o), ctypes.byref(r)))
    return ({"wave_nodes": o.wave_nodes, "wave_rows": o.wave_rows, "count_grid": o.count_grid,
             "deep_nodes": o.deep_nodes, "schedulers": o.schedulers}, r.as_dict())


def mine_batch(dbs, minsups, max_edges=0, label_style=LABELS_FULL, wave_nodes=None, threads=0, collect=True,
               **kw):
    """Mines several databases in shared launches; returns ([patterns per db], stats)."""
    out = [[] for _ in dbs]

    def cb(idx, ptr, n, support, user):
        code = tuple(tuple(ptr[5 * i + j] for j in range(5)) for i in range(n))
        out[idx].append((code, support))

    fn = BATCH_EMIT_FN(cb) if collect else ctypes.cast(None, BATCH_EMIT_FN)
    hs = (ctypes.c_void_p * len(dbs))(*[d.handle for d in dbs])
    ms = (ctypes.c_int32 * len(dbs))(*[int(m) for m in minsups])
    o = _opts(max_edges, label_style, wave_nodes, threads, **kw)
    st = MineStats()
    _check(lib().gs_mine_batch(hs, len(dbs), ms, ctypes.byref(o), fn, None, ctypes.byref(st)))
    return out, st.as_dict()


def support_count(keys, graph_ids, n_keys, n_graphs):
    """support[k] = distinct graph ids among records with key k (GPU)."""
    n = len(keys)
    k = (ctypes.c_int32 * max(1, n))(*[int(x) for x in keys])
    g = (ctypes.c_int32 * max(1, n))(*[int(x) for x in graph_ids])
    out = (ctypes.c_int32 * max(1, n_keys))()
    _check(lib().gs_support_count(k, g, n, int(n_keys), int(n_graphs), out))
    return list(out)[:n_keys]


def filter_backward(column, records, dfs):
    """Backward child column (GPU): the (vertex, back_link) elements of
    column at the rows named by the extension records (8-tuples {from, to,
    fromlabel, elabel, tolabel, from_grph, to_grph, row}) equal to the
    backward edge dfs, in row order (the reference's
    filter_backward_embeddings)."""
    n = len(column)
    col = (ctypes.c_int32 * max(2, 2 * n))(*[int(x) for e in column for x in e])
    flat = [int(x) for r in records for x in r]
    if any(len(r) != 8 for r in records):
        raise ValueError("a record has 8 fields")
    rec = (ctypes.c_int32 * max(8, len(flat)))(*flat)
    if len(dfs) != 5:
        raise ValueError("a DFS edge has 5 fields")
    d = (ctypes.c_int32 * 5)(*[int(x) for x in dfs])
    out = (ctypes.c_int32 * max(2, 2 * n))()
    n_out = ctypes.c_int64(0)
    _check(lib().gs_filter_backward(col, n, rec, len(records), d, out, ctypes.byref(n_out)))
    return [(out[2 * i], out[2 * i + 1]) for i in range(n_out.value)]


def segmented_scan(data, exclusive=False):
    """The reference's packed segmented scan on the GPU: bit 31 of a value
    starts a segment; returns the unpacked running sums (uint32)."""
    n = len(data)
    arr = (ctypes.c_uint32 * max(1, n))(*[int(x) & 0xffffffff for x in data])
    out = (ctypes.c_uint32 * max(1, n))()
    _check(lib().gs_segmented_scan(arr, n, 1 if exclusive else 0, out))
    return list(out)[:n]


def segmented_reduce(data, segment_count, segment_sizes, exclusive=False):
    """The reference's segmented reduction: the segmented scan at the last
    element of each segment, segments given as runs of equal sizes."""
    n = len(data)
    arr = (ctypes.c_uint32 * max(1, n))(*[int(x) & 0xffffffff for x in data])
    g = len(segment_count)
    if len(segment_sizes) != g:
        raise ValueError("segment_count and segment_sizes differ in length")
    cnt = (ctypes.c_uint32 * max(1, g))(*segment_count)
    siz = (ctypes.c_uint32 * max(1, g))(*segment_sizes)
    m = sum(int(c) for c in segment_count)
    res = (ctypes.c_uint32 * max(1, m))()
    nr = ctypes.c_int64(0)
    _check(lib().gs_segmented_reduce(arr, n, cnt, siz, g, 1 if exclusive else 0, res, ctypes.byref(nr)))
    return list(res)[:nr.value]


def dfs_code_is_min(code):
    """Canonicality of a DFS code given as a sequence of 5-tuples (host only)."""
    flat = [int(x) for d in code for x in d]
    arr = (ctypes.c_int32 * max(1, len(flat)))(*flat)
    r = lib().gs_dfs_code_is_min(arr, len(code))
    if r < 0:
        raise ValueError("invalid DFS code")
    return bool(r)


def parse_code(s):
    """'(0 1 2 0 3);(1 2 -1 0 4)' -> tuple of 5-tuples (DFSCode::read_from_str)."""
    out = []
    for part in s.strip().split(";"):
        part = part.strip()
        if not part:
            continue
        out.append(tuple(int(x) for x in part.strip("()").split()))
    return tuple(out)


class GSpanMiner:
    """The reference's miner interface (gspan_cuda::gspan_cuda) over the GB300 engine."""

    def __init__(self, wave_nodes=None, label_style=LABELS_FULL, max_edges=0):
        self._db = None
        self._minsup = -1
        self._out = None
        self.wave_nodes = wave_nodes
        self.label_style = label_style
        self.max_edges = max_edges
        self.stats = None

    def set_database(self, db):
        self._db = db

    def set_min_support(self, minsup):
        self._minsup = int(minsup)

    def set_graph_output(self, sink):
        """sink(code, support), called once per frequent pattern."""
        self._out = sink

    def run(self):
        if self._db is None:
            raise GSpanError(1, "no database set")
        _, self.stats = mine(self._db, self._minsup, self.max_edges, self.label_style, self.wave_nodes,
                             collect=False, sink=self._out)

    def delete_database_from_device(self):
        lib().gs_engine_reset()


class Server:
    """Serving loop (gs_server_*): requests on resident databases, mined with
    continuous batching by a native server thread."""

    def __init__(self, budget_bytes=0, pool_bytes=0, max_active=0, wave_nodes=0, threads=0,
                 label_style=LABELS_FULL, extension=EXTENSION_RMPATH):
        o = ServerOpts()
        lib().gs_server_opts_default(ctypes.byref(o))
        o.budget_bytes, o.pool_bytes = int(budget_bytes), int(pool_bytes)
        if max_active:
            o.max_active = int(max_active)
        o.wave_nodes, o.threads, o.label_style = int(wave_nodes), int(threads), int(label_style)
        o.extension = _extension(extension)
        h = ctypes.c_void_p()
        _check(lib().gs_server_create(ctypes.byref(o), ctypes.byref(h)))
        self._h = h
        self._dbs = []   # the server borrows the databases: keep them alive

    def add_db(self, db):
        i = ctypes.c_int32()
        _check(lib().gs_server_add_db(self._h, db.handle, ctypes.byref(i)))
        self._dbs.append(db)
        return i.value

    def submit(self, db_id, minsup, max_edges=0):
        rid = ctypes.c_int64()
        _check(lib().gs_server_submit(self._h, int(db_id), int(minsup), int(max_edges), ctypes.byref(rid)))
        return rid.value

    def status(self, request_id, wait_ms=0):
        """Request info without taking the result; None while it is still running."""
        info = RequestInfo()
        st = lib().gs_server_poll(self._h, int(request_id), int(wait_ms), ctypes.byref(info), None)
        if st == 9:
            return None
        _check(st)
        return info.as_dict()

    def result(self, request_id, timeout_ms=-1, decode=True):
        """Waits for the request; returns (patterns or None, info) and forgets it."""
        info = RequestInfo()
        p = ctypes.POINTER(Patterns)()
        _check(lib().gs_server_poll(self._h, int(request_id), int(timeout_ms), ctypes.byref(info), ctypes.byref(p)))
        pats = _take_patterns(p, decode) if p else None
        return pats, info.as_dict()

    def cancel(self, request_id):
        _check(lib().gs_server_cancel(self._h, int(request_id)))

    def stats(self):
        s = ServerStats()
        _check(lib().gs_server_get_stats(self._h, ctypes.byref(s)))
        return s.as_dict()

    def close(self):
        if self._h:
            lib().gs_server_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def engine_reset():
    lib().gs_engine_reset()


def set_pool_bytes(n):
    lib().gs_engine_set_pool_bytes(int(n))
