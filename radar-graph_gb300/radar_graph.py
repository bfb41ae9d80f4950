"""Python mirror of the librg.so C ABI (include/radar_graph.h).

This is the host-side face of the GB300 frontier engine for Python callers:
it mirrors the reference's per-app Compute(graph, P) interface
(PageRank.C:120, BFS.C:122, BC-manyiter-v2.C:205, Radii.C:140) and the
Ligra command-line options (-s, -r, -maxiters, -preprocess, -b) through
`run_app`.  Arrays are numpy; every call checks the returned rg_status and
raises RgError with the library's message.  There is no CPU fallback: if
librg.so is missing or no GPU is present, calls raise.
"""

import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "librg.so")

VARIANTS = {"push": 0, "push-pull": 1, "degree-sorting": 2, "hubdup": 3, "radar": 4}
# variants whose reference binaries degree-sort the graph before Compute by
# default (-preprocess 1, ligra.h:566 in RADAR and degree-sorting)
SORTED_VARIANTS = ("degree-sorting", "radar")

OPS = {"pagerank": 0, "bfs": 1, "bc_fwd": 2, "bc_bwd": 3, "radii": 4}
VOPS = {"pr_damp": 0, "bc_visit": 1, "bc_back": 2, "radii_sync": 3}
NO_OUTPUT = 1
DENSE_FORWARD = 8

STATUS = {0: "RG_OK", 1: "RG_EINVAL", 2: "RG_ENOMEM", 3: "RG_ECUDA", 4: "RG_EIO",
          5: "RG_EFORMAT", 6: "RG_EUNSUPPORTED", 7: "RG_ETIMEOUT", 8: "RG_ENODEV", 9: "RG_ECANCELED"}


class RgError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


class Timing(C.Structure):
    _fields_ = [("total_ms", C.c_double), ("edge_ms", C.c_double), ("edges_traversed", C.c_int64),
                ("algorithmic_bytes", C.c_int64), ("edge_launches", C.c_int64),
                ("kernel_launches", C.c_int64)]


class LevelTrace(C.Structure):
    _fields_ = [("mode", C.c_int32), ("hub_mode", C.c_int32), ("frontier", C.c_int64), ("degsum", C.c_int64),
                ("threshold", C.c_int64)]


class OpArgs(C.Structure):
    _fields_ = [("p_curr", C.c_void_p), ("p_next", C.c_void_p), ("parents", C.c_void_p),
                ("num_paths", C.c_void_p), ("deps", C.c_void_p), ("visited_bits", C.c_void_p),
                ("visited", C.c_void_p), ("next_visited", C.c_void_p), ("radii", C.c_void_p),
                ("round", C.c_int32)]


_lib = None

_P = C.POINTER
_u32p = _P(C.c_uint32)
_i32p = _P(C.c_int32)
_i64p = _P(C.c_int64)
_f64p = _P(C.c_double)
_u8p = _P(C.c_uint8)

# name -> argtypes (restype is always c_int = rg_status unless listed in _RESTYPE)
_SIGS = {
    "rg_last_error": [], "rg_status_str": [C.c_int], "rg_version": [], "rg_set_stream": [C.c_void_p],
    "rg_generate_edges": [C.c_int, C.c_int, C.c_uint64, C.c_int, _u32p, _u32p],
    "rg_csr_from_edges": [C.c_int64, C.c_int64, _u32p, _u32p, _P(_u32p), _P(_u32p), _i64p],
    "rg_write_adjacency": [C.c_char_p, C.c_int64, C.c_int64, _u32p, _u32p],
    "rg_read_graph": [C.c_char_p, C.c_int, C.c_int, _i64p, _i64p, _P(_u32p), _P(_u32p)],
    "rg_host_free": [C.c_void_p],
    "rg_graph_create": [C.c_int64, C.c_int64, _u32p, _u32p, C.c_void_p],
    "rg_graph_create_device": [C.c_int64, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p],
    "rg_graph_degree_sort": [C.c_void_p, C.c_void_p, _u32p],
    "rg_graph_info": [C.c_void_p, _i64p, _i64p, _i32p],
    "rg_graph_download": [C.c_void_p, _u32p, _u32p, _u32p],
    "rg_graph_free": [C.c_void_p],
    "rg_pagerank": [C.c_void_p, C.c_int, C.c_int64, _f64p, _i64p, _f64p],
    "rg_bfs": [C.c_void_p, C.c_int, C.c_uint32, _u32p, _i32p, _i64p, _i64p],
    "rg_bc": [C.c_void_p, C.c_int, C.c_int, _f64p, _i64p],
    "rg_bc_sources": [C.c_void_p, C.c_int, _u32p, C.c_int, _f64p, _i64p],
    "rg_bc_pick_sources": [C.c_void_p, C.c_int, _u32p],
    "rg_pick_roots": [C.c_void_p, C.c_int, _u32p],
    "rg_radii": [C.c_void_p, C.c_int, _i32p, _i64p],
    "rg_radii_seeds": [C.c_void_p, C.c_int, _u32p, C.c_int, _i32p, _i64p],
    "rg_frontier_create": [C.c_void_p, C.c_void_p],
    "rg_frontier_free": [C.c_void_p],
    "rg_frontier_set": [C.c_void_p, _u32p, C.c_int64],
    "rg_frontier_set_all": [C.c_void_p],
    "rg_frontier_count": [C.c_void_p, _i64p],
    "rg_frontier_get": [C.c_void_p, _u8p],
    "rg_edgemap": [C.c_void_p, C.c_void_p, C.c_int, _P(OpArgs), C.c_void_p, C.c_uint32, C.c_int64,
                   C.c_void_p],
    "rg_vertexmap": [C.c_void_p, C.c_void_p, C.c_int, _P(OpArgs), C.c_void_p],
    "rg_device_alloc": [C.c_size_t, _P(C.c_void_p)],
    "rg_device_free": [C.c_void_p],
    "rg_copy_to_device": [C.c_void_p, C.c_void_p, C.c_size_t],
    "rg_copy_to_host": [C.c_void_p, C.c_void_p, C.c_size_t],
    "rg_synchronize": [],
    "rg_last_timing": [_P(Timing)],
    "rg_set_kernel_timing": [C.c_int],
    "rg_set_trace": [C.c_int],
    "rg_trace_take": [_P(LevelTrace), C.c_int64, _i64p],
    "rg_device_info": [C.c_char_p, C.c_int, _i32p, _f64p],
    "rg_bfs_depth_noalloc": [C.c_void_p, C.c_void_p, C.c_int64, C.c_int64, C.c_uint32, C.c_void_p, C.c_void_p,
                             _i64p],
    "rg_set_option": [C.c_int, C.c_int64],
    "rg_get_option": [C.c_int, _i64p],
    "rg_bfs_multi": [C.c_void_p, _u32p, C.c_int, _i32p, _i64p],
    "rg_bc_multi": [C.c_void_p, _u32p, C.c_int, _f64p, _i64p],
    "rg_radii_multi": [C.c_void_p, _u32p, C.c_int, C.c_int, _i32p, _i64p],
    "rg_batch_create": [C.c_int, _i64p, _i64p, _P(_u32p), _P(_u32p), C.c_void_p],
    "rg_batch_run": [C.c_void_p, _u32p, C.c_int, C.c_int64, _i32p, _f64p, _i32p, _f64p],
    "rg_batch_free": [C.c_void_p],
    "rg_server_create": [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_double, C.c_void_p],
    "rg_server_submit": [C.c_void_p, C.c_int, C.c_int, C.c_uint32, _P(C.c_uint64)],
    "rg_server_wait": [C.c_void_p, C.c_uint64, C.c_void_p, C.c_size_t, _f64p],
    "rg_server_wait_for": [C.c_void_p, C.c_uint64, C.c_void_p, C.c_size_t, _f64p, C.c_double],
    "rg_server_cancel": [C.c_void_p, C.c_uint64],
    "rg_server_pause": [C.c_void_p, C.c_int],
    "rg_server_get_stats": [C.c_void_p, C.c_void_p],
    "rg_server_reset_stats": [C.c_void_p],
    "rg_server_free": [C.c_void_p],
    "rg_autotune": [C.c_void_p, C.c_int, _f64p],
    "rg_graph_tuned_option": [C.c_void_p, C.c_int, C.c_int, _i64p],
    "rg_graph_clear_tuning": [C.c_void_p],
    "rg_graph_set_tuned_option": [C.c_void_p, C.c_int, C.c_int, C.c_int64],
    "rg_pinned_alloc": [C.c_size_t, _P(C.c_void_p)],
    "rg_graph_create_directed": [C.c_int64, C.c_int64, _u32p, _u32p, _P(C.c_void_p)],
    "rg_graph_is_directed": [C.c_void_p, _P(C.c_int)],
    "rg_graph_degree_sort_by": [C.c_void_p, C.c_int, _P(C.c_void_p), _u32p],
    "rg_triangle_count": [C.c_void_p, _P(C.c_uint64), _P(C.c_uint64)],
    "rg_read_sg": [C.c_char_p, _i64p, _i64p, _P(_u32p), _P(_u32p), _P(C.c_int)],
    "rg_read_edges": [C.c_char_p, _i64p, _i64p, _P(_u32p), _P(_u32p)],
    "rg_graph_create_sorted": [C.c_int64, C.c_int64, C.c_void_p, C.c_void_p, _P(C.c_void_p), C.c_void_p],
    "rg_graph_create_from_edges": [C.c_int64, C.c_int64, C.c_void_p, C.c_void_p, C.c_int, _P(C.c_void_p)],
    "rg_graph_create_directed_from_edges": [C.c_int64, C.c_int64, C.c_void_p, C.c_void_p, C.c_int, _P(C.c_void_p)],
    "rg_pagerank_delta": [C.c_void_p, C.c_int, C.c_int64, _P(C.c_double), _i64p, _P(C.c_double)],
    "rg_pinned_free": [C.c_void_p],
}


class _Pinned:
    """Owner of one page-locked host allocation backing a numpy array."""

    def __init__(self, nbytes):
        self.p = C.c_void_p()
        _check(lib().rg_pinned_alloc(max(int(nbytes), 1), C.byref(self.p)))

    def __del__(self):
        try:
            if self.p and self.p.value:
                lib().rg_pinned_free(self.p)
        except Exception:
            pass


class PinnedArray(np.ndarray):
    """ndarray whose memory is page-locked; it keeps its allocation alive."""


def pinned_empty(shape, dtype):
    """A numpy array in page-locked host memory (fast device->host copies)."""
    dtype = np.dtype(dtype)
    count = int(np.prod(shape))
    owner = _Pinned(count * dtype.itemsize)
    buf = (C.c_char * max(count * dtype.itemsize, 1)).from_address(owner.p.value)
    arr = np.frombuffer(buf, dtype=dtype, count=count).reshape(shape).view(PinnedArray)
    arr._owner = owner
    return arr

QUERY_KINDS = {"bfs": 0, "bc": 1, "radii": 2}


class ServerStats(C.Structure):
    _fields_ = [("completed", C.c_int64), ("launches", C.c_int64), ("batched", C.c_int64),
                ("p50_ms", C.c_double), ("p99_ms", C.c_double), ("qps", C.c_double),
                ("admission_waits", C.c_int64), ("cancelled", C.c_int64), ("peak_running", C.c_int32)]

# RG_OPT_*: the scheduling options a graph's tuning holds, and the thread's
# result-copy mode (RG_OPT_ASYNC_RESULTS)
SCHEDULE_OPTIONS = {"direction": 0, "hub_slots": 1, "hub_smem_kb": 2, "dense_div": 3, "sweep_shape": 4,
                    "bc_fwd_hubs": 5}
OPTIONS = dict(SCHEDULE_OPTIONS, async_results=6)
_RESTYPE = {"rg_last_error": C.c_char_p, "rg_status_str": C.c_char_p, "rg_version": C.c_char_p,
            "rg_host_free": None}


def exported_symbols():
    """Names the C ABI exports (every function declared in include/*.h)."""
    return sorted(_SIGS)


def lib():
    """Loads librg.so (raises if it is missing: there is no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RgError(8, f"{LIB_PATH} is missing; build it with radar-graph_gb300/build.py")
        L = C.CDLL(LIB_PATH)
        for name, args in _SIGS.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = _RESTYPE.get(name, C.c_int)
        _lib = L
    return _lib


def _check(status):
    if status != 0:
        msg = lib().rg_last_error()
        raise RgError(status, msg.decode() if msg else "")


def _ptr(a, t):
    return a.ctypes.data_as(_P(t))


def version():
    return lib().rg_version().decode()


def last_timing():
    t = Timing()
    _check(lib().rg_last_timing(C.byref(t)))
    return {k: getattr(t, k) for k, _ in Timing._fields_}


def set_option(name, value):
    """Engine scheduling option (RG_OPT_*); results never depend on them."""
    _check(lib().rg_set_option(OPTIONS[name], int(value)))


def get_option(name):
    v = C.c_int64()
    _check(lib().rg_get_option(OPTIONS[name], C.byref(v)))
    return v.value


def synchronize():
    """rg_synchronize: waits for the device, including result copies left in
    flight by the async_results option."""
    _check(lib().rg_synchronize())


TRACE_MODES = {0: "sparse-push", 1: "dense-push", 2: "pull"}


def set_trace(on):
    """Record one entry per edgeMap of this thread (rg_set_trace)."""
    _check(lib().rg_set_trace(1 if on else 0))


def take_trace(cap=4096):
    """The recorded edgeMaps, oldest first, as dicts; clears the record."""
    buf = (LevelTrace * cap)()
    k = C.c_int64()
    _check(lib().rg_trace_take(buf, cap, C.byref(k)))
    return [{"mode": TRACE_MODES[buf[i].mode], "hub_mode": buf[i].hub_mode, "frontier": buf[i].frontier,
             "degsum": buf[i].degsum, "threshold": buf[i].threshold} for i in range(k.value)]


def device_info():
    """(name, SM count, nominal HBM GB/s) of the current device."""
    name = C.create_string_buffer(256)
    sms, gbs = C.c_int32(), C.c_double()
    _check(lib().rg_device_info(name, 256, C.byref(sms), C.byref(gbs)))
    return name.value.decode(), sms.value, gbs.value


def set_kernel_timing(on):
    """Bracket every edge-kernel launch with CUDA events (see last_timing()['edge_ms'])."""
    _check(lib().rg_set_kernel_timing(1 if on else 0))


# ---------------------------------------------------------------------------
# input formats (host side)
# ---------------------------------------------------------------------------

def generate_edges(scale, edge_factor, seed=1, uniform=False):
    """Seeded R-MAT / Erdos-Renyi edge list (GAP generator algorithm)."""
    ne = edge_factor << scale
    src = np.empty(ne, np.uint32)
    dst = np.empty(ne, np.uint32)
    _check(lib().rg_generate_edges(scale, edge_factor, seed, 1 if uniform else 0, _ptr(src, C.c_uint32),
                                   _ptr(dst, C.c_uint32)))
    return src, dst


def _take_host_csr(n, m, po, pa):
    off = np.ctypeslib.as_array(po, shape=(n + 1,)).copy()
    adj = np.ctypeslib.as_array(pa, shape=(max(m, 1),))[:m].copy()
    lib().rg_host_free(C.cast(po, C.c_void_p))
    lib().rg_host_free(C.cast(pa, C.c_void_p))
    return off, adj


def csr_from_edges(n, src, dst):
    """Symmetric CSR (both directions, sorted, deduplicated, no self-loops)."""
    src = np.ascontiguousarray(src, np.uint32)
    dst = np.ascontiguousarray(dst, np.uint32)
    po, pa, m = _u32p(), _u32p(), C.c_int64()
    _check(lib().rg_csr_from_edges(n, len(src), _ptr(src, C.c_uint32), _ptr(dst, C.c_uint32), C.byref(po),
                                   C.byref(pa), C.byref(m)))
    return _take_host_csr(n, m.value, po, pa)


def rmat_csr(scale, edge_factor, seed=1, uniform=False):
    src, dst = generate_edges(scale, edge_factor, seed, uniform)
    return csr_from_edges(1 << scale, src, dst)


def write_adjacency(path, off, adj):
    off = np.ascontiguousarray(off, np.uint32)
    adj = np.ascontiguousarray(adj, np.uint32)
    _check(lib().rg_write_adjacency(str(path).encode(), len(off) - 1, len(adj), _ptr(off, C.c_uint32),
                                    _ptr(adj, C.c_uint32)))


def read_sg(path, allow_directed=False):
    """GAP serialized graph (.sg) -> CSR (off, adj); with allow_directed,
    (off, adj, directed) and a directed file gives its out-lists."""
    n, m, po, pa, dr = C.c_int64(), C.c_int64(), _u32p(), _u32p(), C.c_int()
    _check(lib().rg_read_sg(str(path).encode(), C.byref(n), C.byref(m), C.byref(po), C.byref(pa),
                            C.byref(dr) if allow_directed else None))
    off, adj = _take_host_csr(n.value, m.value, po, pa)
    return (off, adj, bool(dr.value)) if allow_directed else (off, adj)


def read_edges(path):
    """GAP text edge list (.el .wel .gr .graph .mtx) -> (n, src, dst), edges as read."""
    n, ne, ps, pd = C.c_int64(), C.c_int64(), _u32p(), _u32p()
    _check(lib().rg_read_edges(str(path).encode(), C.byref(n), C.byref(ne), C.byref(ps), C.byref(pd)))
    k = ne.value
    src = np.ctypeslib.as_array(ps, shape=(max(k, 1),))[:k].copy()
    dst = np.ctypeslib.as_array(pd, shape=(max(k, 1),))[:k].copy()
    lib().rg_host_free(ps)
    lib().rg_host_free(pd)
    return n.value, src, dst


def read_graph(path, symmetric=True, binary=False):
    """Ligra text (or binary) graph -> cleaned symmetric CSR (off, adj)."""
    n, m, po, pa = C.c_int64(), C.c_int64(), _u32p(), _u32p()
    _check(lib().rg_read_graph(str(path).encode(), 1 if symmetric else 0, 1 if binary else 0, C.byref(n),
                               C.byref(m), C.byref(po), C.byref(pa)))
    return _take_host_csr(n.value, m.value, po, pa)


# ---------------------------------------------------------------------------
# device graph and apps
# ---------------------------------------------------------------------------

def _variant(v):
    if isinstance(v, str):
        if v not in VARIANTS:
            raise ValueError(f"unknown variant {v!r}; one of {list(VARIANTS)}")
        return VARIANTS[v]
    return int(v)


class Graph:
    """A device-resident CSR image (rg_graph)."""

    def __init__(self, handle):
        self._h = C.c_void_p(handle) if not isinstance(handle, C.c_void_p) else handle
        n, m, s = C.c_int64(), C.c_int64(), C.c_int32()
        _check(lib().rg_graph_info(self._h, C.byref(n), C.byref(m), C.byref(s)))
        self.n, self.m, self.sorted = n.value, m.value, bool(s.value)

    @classmethod
    def from_csr(cls, off, adj):
        off = np.ascontiguousarray(off, np.uint32)
        adj = np.ascontiguousarray(adj, np.uint32)
        h = C.c_void_p()
        _check(lib().rg_graph_create(len(off) - 1, len(adj), _ptr(off, C.c_uint32), _ptr(adj, C.c_uint32),
                                     C.byref(h)))
        return cls(h)

    @classmethod
    def from_csr_directed(cls, off, adj):
        """A directed graph from its cleaned out-lists; in-lists built on the device."""
        off = np.ascontiguousarray(off, np.uint32)
        adj = np.ascontiguousarray(adj, np.uint32)
        h = C.c_void_p()
        _check(lib().rg_graph_create_directed(len(off) - 1, len(adj), _ptr(off, C.c_uint32),
                                              _ptr(adj, C.c_uint32), C.byref(h)))
        return cls(h)

    @property
    def directed(self):
        d = C.c_int()
        _check(lib().rg_graph_is_directed(self._h, C.byref(d)))
        return bool(d.value)

    def degree_sort_by(self, by_out_degree):
        """Degree sort with the key chosen (out-degree, or in-degree for a directed graph)."""
        h = C.c_void_p()
        _check(lib().rg_graph_degree_sort_by(self._h, 1 if by_out_degree else 0, C.byref(h), None))
        return Graph(h)

    @classmethod
    def from_edges(cls, n, src, dst, directed=False):
        """CSR built on the device from an edge list with the loader's
        clean-up: symmetric (both directions, sorted, no repeats or self
        loops), or directed (src -> dst out-lists cleaned the same way, plus
        the in-lists)."""
        src = np.ascontiguousarray(src, np.uint32)
        dst = np.ascontiguousarray(dst, np.uint32)
        if len(src) != len(dst):
            raise ValueError("src and dst differ in length")
        h = C.c_void_p()
        fn = lib().rg_graph_create_directed_from_edges if directed else lib().rg_graph_create_from_edges
        _check(fn(n, len(src), src.ctypes.data if len(src) else None, dst.ctypes.data if len(dst) else None, 0,
                  C.byref(h)))
        return cls(h)

    @classmethod
    def from_csr_sorted(cls, off, adj):
        """Upload and degree-sort a symmetric CSR in one call (the same graph as
        from_csr(off, adj).degree_sort()); page-locked adj (pinned_empty) is
        read in place by the relabel."""
        off = np.ascontiguousarray(off, np.uint32)
        adj = np.ascontiguousarray(adj, np.uint32)
        h = C.c_void_p()
        _check(lib().rg_graph_create_sorted(len(off) - 1, len(adj), off.ctypes.data,
                                            adj.ctypes.data if len(adj) else None, C.byref(h), None))
        return cls(h)

    def degree_sort(self):
        """New graph relabelled by degree (preprocessGraph); its permutation
        is `.new_ids` (copied from the device on first access)."""
        h = C.c_void_p()
        _check(lib().rg_graph_degree_sort(self._h, C.byref(h), None))
        return Graph(h)

    @property
    def new_ids(self):
        """new_ids[original id] = internal id (identity when not sorted)."""
        if getattr(self, "_new_ids", None) is None:
            ids = np.empty(self.n, np.uint32)
            _check(lib().rg_graph_download(self._h, None, None, _ptr(ids, C.c_uint32)))
            self._new_ids = ids
        return self._new_ids

    def download(self):
        off = np.empty(self.n + 1, np.uint32)
        adj = np.empty(max(self.m, 1), np.uint32)
        ids = np.empty(self.n, np.uint32)
        _check(lib().rg_graph_download(self._h, _ptr(off, C.c_uint32), _ptr(adj, C.c_uint32),
                                       _ptr(ids, C.c_uint32)))
        return off, adj[:self.m], ids

    def free(self):
        if self._h is not None and self._h.value:
            lib().rg_graph_free(self._h)
        self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.free()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    # -- apps ---------------------------------------------------------------
    def pagerank(self, variant="push", max_iters=100, out=None):
        """(ranks, iterations, L1); out: optional float64[n] buffer (e.g. pinned)."""
        ranks = np.empty(self.n, np.float64) if out is None else out
        it, l1 = C.c_int64(), C.c_double()
        _check(lib().rg_pagerank(self._h, _variant(variant), max_iters, _ptr(ranks, C.c_double), C.byref(it),
                                 C.byref(l1)))
        return ranks, it.value, l1.value

    def triangles(self):
        """(per-vertex triangle counts by original id, total)."""
        counts = np.empty(self.n, np.uint64)
        total = C.c_uint64()
        _check(lib().rg_triangle_count(self._h, _ptr(counts, C.c_uint64), C.byref(total)))
        return counts, total.value

    def pagerank_delta(self, variant="push", max_iters=100):
        """PageRankDelta: (ranks, printed round count, final L1)."""
        ranks = np.empty(self.n, np.float64)
        it, l1 = C.c_int64(), C.c_double()
        _check(lib().rg_pagerank_delta(self._h, _variant(variant), max_iters, _ptr(ranks, C.c_double),
                                       C.byref(it), C.byref(l1)))
        return ranks, it.value, l1.value

    def bfs(self, variant="push", root=0, depth_out=None, parents=True):
        """(parents, depth, rounds, reached); depth_out: optional int32[n]
        buffer (e.g. pinned); parents: True, False (skip the parent array) or
        a uint32[n] buffer to fill."""
        if isinstance(parents, np.ndarray):
            par = parents
        else:
            par = np.empty(self.n, np.uint32) if parents else None
        depth = np.empty(self.n, np.int32) if depth_out is None else depth_out
        rounds, reached = C.c_int64(), C.c_int64()
        _check(lib().rg_bfs(self._h, _variant(variant), root, _ptr(par, C.c_uint32) if par is not None else None,
                            _ptr(depth, C.c_int32), C.byref(rounds), C.byref(reached)))
        return par, depth, rounds.value, reached.value

    def bc(self, variant="push", max_iters=16):
        deps = np.empty(self.n, np.float64)
        lv = C.c_int64()
        _check(lib().rg_bc(self._h, _variant(variant), max_iters, _ptr(deps, C.c_double), C.byref(lv)))
        return deps, lv.value

    def bc_sources(self, sources, variant="push", out=None):
        s = np.ascontiguousarray(sources, np.uint32)
        deps = np.empty(self.n, np.float64) if out is None else out
        lv = C.c_int64()
        _check(lib().rg_bc_sources(self._h, _variant(variant), _ptr(s, C.c_uint32), len(s),
                                   _ptr(deps, C.c_double), C.byref(lv)))
        return deps, lv.value

    def bc_multi(self, sources):
        """k <= 64 independent single-source BCs in one traversal: (k, n)
        array, row q = bc_sources([sources[q]]), and the level count."""
        s = np.ascontiguousarray(sources, np.uint32)
        deps = np.empty((len(s), self.n), np.float64)
        lv = C.c_int64()
        _check(lib().rg_bc_multi(self._h, _ptr(s, C.c_uint32), len(s), _ptr(deps, C.c_double), C.byref(lv)))
        return deps, lv.value

    def radii_multi(self, seeds):
        """nq <= 16 Radii queries in one traversal; seeds: (nq, k) array of
        sample vertices.  Returns (nq, n) radii (row q = radii_seeds(seeds[q]))
        and the round count."""
        s = np.ascontiguousarray(seeds, np.uint32)
        if s.ndim != 2:
            raise ValueError("seeds must be (queries, samples)")
        r = np.empty((s.shape[0], self.n), np.int32)
        rounds = C.c_int64()
        _check(lib().rg_radii_multi(self._h, _ptr(s, C.c_uint32), s.shape[1], s.shape[0], _ptr(r, C.c_int32),
                                    C.byref(rounds)))
        return r, rounds.value

    def bc_pick_sources(self, k):
        out = np.empty(k, np.uint32)
        _check(lib().rg_bc_pick_sources(self._h, k, _ptr(out, C.c_uint32)))
        return out

    def pick_roots(self, k):
        """k search roots (original ids) by GAP's SourcePicker rule."""
        out = np.empty(k, np.uint32)
        _check(lib().rg_pick_roots(self._h, k, _ptr(out, C.c_uint32)))
        return out

    def radii(self, variant="push", out=None):
        r = np.empty(self.n, np.int32) if out is None else out
        rounds = C.c_int64()
        _check(lib().rg_radii(self._h, _variant(variant), _ptr(r, C.c_int32), C.byref(rounds)))
        return r, rounds.value

    def radii_seeds(self, seeds, variant="push", out=None):
        s = np.ascontiguousarray(seeds, np.uint32)
        r = np.empty(self.n, np.int32) if out is None else out
        rounds = C.c_int64()
        _check(lib().rg_radii_seeds(self._h, _variant(variant), _ptr(s, C.c_uint32), len(s), _ptr(r, C.c_int32),
                                    C.byref(rounds)))
        return r, rounds.value


def _graph_bfs_multi(self, sources):
    """BFS from up to 64 sources in one traversal; returns (depths[k, n], rounds)."""
    s = np.ascontiguousarray(sources, np.uint32)
    d = np.empty((len(s), self.n), np.int32)
    rounds = C.c_int64()
    _check(lib().rg_bfs_multi(self._h, _ptr(s, C.c_uint32), len(s), _ptr(d, C.c_int32), C.byref(rounds)))
    return d, rounds.value


Graph.bfs_multi = _graph_bfs_multi


def _graph_autotune(self, variant="radar"):
    """Times candidate schedules per app on this graph and keeps the fastest;
    returns {app: (best ms, {option: value})}."""
    best = (C.c_double * 4)()
    _check(lib().rg_autotune(self._h, _variant(variant), best))
    out = {}
    for a, name in enumerate(("pagerank", "bfs", "bc", "radii")):
        opts = {}
        for o, code in SCHEDULE_OPTIONS.items():
            v = C.c_int64()
            _check(lib().rg_graph_tuned_option(self._h, a, code, C.byref(v)))
            opts[o] = v.value
        out[name] = (best[a], opts)
    return out


Graph.autotune = _graph_autotune


def _graph_set_tuning(self, tuning):
    """Applies a tuning returned by autotune() (e.g. to a copy of the graph)."""
    for a, name in enumerate(("pagerank", "bfs", "bc", "radii")):
        for o, v in tuning[name][1].items():
            if v >= 0:
                _check(lib().rg_graph_set_tuned_option(self._h, a, SCHEDULE_OPTIONS[o], int(v)))


Graph.set_tuning = _graph_set_tuning


def _graph_clear_tuning(self):
    """Forgets the autotuner's choices: later calls use the thread's options."""
    _check(lib().rg_graph_clear_tuning(self._h))


Graph.clear_tuning = _graph_clear_tuning


class Batch:
    """Many graphs resident on the device, run by one persistent launch."""

    def __init__(self, csrs):
        self.csrs = [(np.ascontiguousarray(o, np.uint32), np.ascontiguousarray(a, np.uint32)) for o, a in csrs]
        g = len(self.csrs)
        self.ns = np.array([len(o) - 1 for o, _ in self.csrs], np.int64)
        self.ms = np.array([len(a) for _, a in self.csrs], np.int64)
        offs = (_u32p * g)(*[_ptr(o, C.c_uint32) for o, _ in self.csrs])
        adjs = (_u32p * g)(*[_ptr(a, C.c_uint32) for _, a in self.csrs])
        self._h = C.c_void_p()
        _check(lib().rg_batch_create(g, _ptr(self.ns, C.c_int64), _ptr(self.ms, C.c_int64), offs, adjs,
                                     C.byref(self._h)))

    def run(self, sources, pr_iters=10):
        """sources: [ngraphs, k] graph-local ids.  Returns (depths per graph
        [k, n_i], ranks per graph, PageRank iterations, device ms)."""
        src = np.ascontiguousarray(sources, np.uint32)
        g, k = src.shape
        depths = np.empty(int(k * self.ns.sum()), np.int32)
        ranks = np.empty(int(self.ns.sum()), np.float64)
        iters = np.empty(g, np.int32)
        ms = C.c_double()
        _check(lib().rg_batch_run(self._h, _ptr(src, C.c_uint32), k, pr_iters, _ptr(depths, C.c_int32),
                                  _ptr(ranks, C.c_double), _ptr(iters, C.c_int32), C.byref(ms)))
        out_d, out_r, o, r = [], [], 0, 0
        for n in self.ns:
            out_d.append(depths[o:o + k * n].reshape(k, n))
            out_r.append(ranks[r:r + n])
            o += k * n
            r += n
        return out_d, out_r, iters, ms.value

    def free(self):
        if self._h is not None and self._h.value:
            lib().rg_batch_free(self._h)
        self._h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class Server:
    """Request loop over resident graphs (rg_server_*): submit queries from any
    thread, wait for their results; BFS queries are coalesced into 64-wide
    multi-source traversals."""

    def __init__(self, graphs, workers=4, max_batch=64, hbm_fraction=0.8):
        self.graphs = list(graphs)
        arr = (C.c_void_p * len(self.graphs))(*[g.handle.value for g in self.graphs])
        self._h = C.c_void_p()
        _check(lib().rg_server_create(arr, len(self.graphs), workers, max_batch, hbm_fraction, C.byref(self._h)))

    def submit(self, graph, kind, source):
        t = C.c_uint64()
        _check(lib().rg_server_submit(self._h, graph, QUERY_KINDS[kind], int(source), C.byref(t)))
        return t.value

    def wait(self, ticket, graph, kind, out=None, timeout_ms=None):
        """Result of `ticket` (into `out` if given, e.g. a pinned_empty array).
        With timeout_ms, raises RgError RG_ETIMEOUT if it is not done in time
        (the ticket stays valid); a cancelled ticket raises RG_ECANCELED."""
        n = self.graphs[graph].n
        if out is None:
            out = np.empty(n, np.float64 if kind == "bc" else np.int32)
        lat = C.c_double()
        _check(lib().rg_server_wait_for(self._h, ticket, out.ctypes.data, out.nbytes, C.byref(lat),
                                        -1.0 if timeout_ms is None else float(timeout_ms)))
        return out, lat.value

    def cancel(self, ticket):
        _check(lib().rg_server_cancel(self._h, ticket))

    def pause(self, paused=True):
        """Workers take no new queries while paused (running batches finish)."""
        _check(lib().rg_server_pause(self._h, 1 if paused else 0))

    def stats(self):
        s = ServerStats()
        _check(lib().rg_server_get_stats(self._h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in ServerStats._fields_}

    def reset_stats(self):
        _check(lib().rg_server_reset_stats(self._h))

    def free(self):
        if self._h is not None and self._h.value:
            lib().rg_server_free(self._h)
        self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.free()


def radii_query_seeds(seed, n):
    """Sample vertices of a served Radii query: hashInt(64*seed + i) % n, i < 64."""
    M = (1 << 64) - 1
    out = []
    for i in range(min(n, 64)):
        a = (64 * seed + i) & M
        a = ((a + 0x7ed55d166bef7a1d) + (a << 12)) & M
        a = ((a ^ 0xc761c23c510fa2dd) ^ (a >> 9)) & M
        a = ((a + 0x165667b183a9c0e1) + (a << 59)) & M
        a = ((a + 0xd3a2646cab3487e3) ^ (a << 49)) & M
        a = ((a + 0xfd7046c5ef9ab54c) + (a << 3)) & M
        a = ((a ^ 0xb55a4f090dd4a67b) ^ (a >> 32)) & M
        out.append(a % n)
    return np.array(out, np.uint32)


def radii_seeds_orig(n):
    """Radii sample vertices hashInt(i) % n for i < min(n, 64) (Radii.C:162-169)."""
    M = (1 << 64) - 1
    out = []
    for i in range(min(n, 64)):
        a = i
        a = ((a + 0x7ed55d166bef7a1d) + (a << 12)) & M
        a = ((a ^ 0xc761c23c510fa2dd) ^ (a >> 9)) & M
        a = ((a + 0x165667b183a9c0e1) + (a << 59)) & M
        a = ((a + 0xd3a2646cab3487e3) ^ (a << 49)) & M
        a = ((a + 0xfd7046c5ef9ab54c) + (a << 3)) & M
        a = ((a ^ 0xb55a4f090dd4a67b) ^ (a >> 32)) & M
        out.append(a % n)
    return np.array(out, np.uint32)


def run_app(app, off, adj, variant="push", maxiters=None, root=0, preprocess=None):
    """parallel_main + Compute of one reference app (ligra.h:556-651).

    app: "PageRank" | "BFS" | "BC" | "Radii".  preprocess: None = the variant's
    default (degree sort for degree-sorting and RADAR), 1/0 = sort, -1 = none.
    Returns the app's per-vertex output in ORIGINAL id order.
    """
    if preprocess is None:
        preprocess = 1 if variant in SORTED_VARIANTS else -1
    with Graph.from_csr(off, adj) as g0:
        g = g0.degree_sort() if preprocess in (0, 1) else g0
        try:
            if app == "PageRank":
                return g.pagerank(variant, 100 if maxiters is None else maxiters)
            if app == "BFS":
                return g.bfs(variant, root)
            if app == "BC":
                return g.bc(variant, 16 if maxiters is None else maxiters)
            if app == "Radii":
                return g.radii(variant)
            raise ValueError(f"unknown app {app}")
        finally:
            if g is not g0:
                g.free()
