"""Python binding of librbcgb.so (the engine's C ABI, include/rbc_gb300.h).

A thin ctypes layer for tests, the benchmark and scripting.  Device buffers
are torch CUDA tensors (torch is used only to own device memory and streams);
every computation happens in the engine's CUDA kernels.  If the library is
missing the import of a function fails loudly -- there is no Python or CPU
fallback for any engine operation.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "librbcgb.so")

OK, ERR_INVALID, ERR_CUDA, ERR_NOMEM, ERR_ITER_LIMIT, ERR_UNSUPPORTED, ERR_IO = range(7)
L2, L1 = 0, 1
KMAX = 32
K_LIMIT = 128  # largest k of query / brute_knn (KMAX for batches and the no-alloc call)
BUILD_PARTITION, BUILD_ONESHOT, BUILD_BF16, BUILD_F64 = 1, 2, 4, 8
QUERY_EXACT, QUERY_ONESHOT, QUERY_EXACT_TC = 0, 1, 2
TC_BF16, TC_FP16_SPLIT = 0, 1
TC_ROUTER_ONLY = 0xFF  # tensor-form probes: the router's picks alone (routed calls)
TC_PREFIX_NONE = 0xFFFFFFFFFFFFFFFF  # tensor-form probe rows: no FP32 prefix, the tensor cores take whole lists
QUERY_ROUTED = 0x1000
SYNTH_UNIFORM, SYNTH_MIXTURE, SYNTH_GEOMETRIC = 0, 1, 2
DUMMY = 0xFFFFFFFF
FLT_MAX = float(np.finfo(np.float32).max)


class RBCError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"rbc error {code}: {msg}")
        self.code = code


class BuildParams(C.Structure):
    _fields_ = [("num_reps", C.c_uint32), ("s", C.c_uint32), ("metric", C.c_int), ("flags", C.c_uint32),
                ("seed", C.c_uint64), ("rep_ids", C.POINTER(C.c_uint32))]


class IndexInfo(C.Structure):
    _fields_ = [("n", C.c_uint64), ("d", C.c_uint32), ("ld", C.c_uint32), ("num_reps", C.c_uint32),
                ("s", C.c_uint32), ("metric", C.c_int), ("flags", C.c_uint32), ("min_list", C.c_uint64),
                ("max_list", C.c_uint64), ("device_bytes", C.c_uint64), ("tc_format", C.c_uint32),
                ("tc_plain", C.c_uint32), ("router_picks", C.c_uint32),
                ("tc_unrouted", C.c_uint32), ("tc_probe_cap", C.c_uint64)]


class QueryStats(C.Structure):
    _fields_ = [("queries", C.c_uint64), ("rep_pairs", C.c_uint64), ("lists_probed", C.c_uint64),
                ("point_pairs", C.c_uint64), ("fallback_queries", C.c_uint64)]


class Profile(C.Structure):
    _fields_ = [("search_launches", C.c_uint64), ("search_ms", C.c_double), ("pruned_launches", C.c_uint64),
                ("pruned_ms", C.c_double), ("pruned_pairs", C.c_uint64)]


# Every symbol of include/rbc_gb300.h with its ctypes signature.
_VP, _U32, _U64, _INT, _F = C.c_void_p, C.c_uint32, C.c_uint64, C.c_int, C.c_float
SIGNATURES = {
    "rbc_status_string": ([_INT], C.c_char_p),
    "rbc_last_error": ([], C.c_char_p),
    "rbc_version": ([], _INT),
    "rbc_build": ([_VP, _U64, _U32, _U32, C.POINTER(BuildParams), _VP, C.POINTER(_VP)], _INT),
    "rbc_build_host": ([_VP, _U64, _U32, _U32, C.POINTER(BuildParams), C.POINTER(_VP)], _INT),
    "rbc_destroy": ([_VP], _INT),
    "rbc_get_info": ([_VP, C.POINTER(IndexInfo)], _INT),
    "rbc_save": ([_VP, C.c_char_p], _INT),
    "rbc_load": ([C.c_char_p, C.POINTER(_VP)], _INT),
    "rbc_get_reps": ([_VP, _VP], _INT),
    "rbc_get_partition": ([_VP, _VP, _VP, _VP], _INT),
    "rbc_get_oneshot": ([_VP, _VP, _VP], _INT),
    "rbc_query": ([_VP, _VP, _U64, _U32, _U32, _U32, _VP, _VP, _U32, _VP], _INT),
    "rbc_query_host": ([_VP, _VP, _U64, _U32, _U32, _U32, _VP, _VP, _U32], _INT),
    "rbc_get_query_stats": ([_VP, C.POINTER(QueryStats)], _INT),
    "rbc_get_fallback_queries": ([_VP, _VP, _U64, C.POINTER(_U64)], _INT),
    "rbc_batch_create": ([C.POINTER(_VP)], _INT),
    "rbc_batch_add": ([_VP, _VP, _VP, _U64, _U32, _U32, _VP, _VP, _U32], _INT),
    "rbc_batch_add_mode": ([_VP, _VP, _VP, _U64, _U32, _U32, _U32, _VP, _VP, _U32], _INT),
    "rbc_batch_run": ([_VP, _VP], _INT),
    "rbc_batch_destroy": ([_VP], _INT),
    "rbc_set_tuning": ([_VP, _INT, _U32], _INT),
    "rbc_autotune": ([_VP, _VP, _U64, _U32, _U32, C.c_char_p, _VP], _INT),
    "rbc_set_tc_tuning": ([_VP, _U32, _U64], _INT),
    "rbc_autotune_tc": ([_VP, _VP, _U64, _U32, _U32, _U32, _VP], _INT),
    "rbc_get_tc_tuning": ([_VP, C.POINTER(_U32), C.POINTER(_U64)], _INT),
    "rbc_set_tc_probe_cap": ([_VP, _U64], _INT),
    "rbc_router_create": ([_U32, _U32, _U32, _U64, C.POINTER(_VP)], _INT),
    "rbc_router_destroy": ([_VP], _INT),
    "rbc_router_num_params": ([_VP, C.POINTER(_U64)], _INT),
    "rbc_router_get_params": ([_VP, _VP], _INT),
    "rbc_router_set_params": ([_VP, _VP], _INT),
    "rbc_router_gradients": ([_VP, _VP, _U32, _U32, _VP, C.POINTER(_F), _VP, _VP], _INT),
    "rbc_router_train": ([_VP, _VP, _U64, _U32, _VP, _U32, _U32, _F, _U64, C.POINTER(_F), _VP], _INT),
    "rbc_router_logits": ([_VP, _VP, _U64, _U32, _VP, _VP], _INT),
    "rbc_owner_labels": ([_VP, _VP, _U64, _U32, _VP, _VP], _INT),
    "rbc_router_create_with_distance": ([_U32, _U32, _U32, _U64, C.POINTER(_VP)], _INT),
    "rbc_router_labels": ([_VP, _VP, _U64, _U32, _U32, _VP, _VP, _VP, _VP], _INT),
    "rbc_router_train_with_distance": ([_VP, _VP, _U64, _U32, _VP, _VP, _VP, _U32, _U32, _F, _U64, C.POINTER(_F),
                                        _VP], _INT),
    "rbc_router_gradients_with_distance": ([_VP, _VP, _U32, _U32, _VP, _VP, C.POINTER(_F), _VP, _VP], _INT),
    "rbc_router_predict_distance": ([_VP, _VP, _U64, _U32, _VP, _VP, _VP], _INT),
    "rbc_router_top_lists": ([_VP, _VP, _U64, _U32, _U32, _VP, _VP], _INT),
    "rbc_router_distance_params": ([_VP, C.POINTER(_F), C.POINTER(_F), C.POINTER(_F)], _INT),
    "rbc_router_set_distance_margin": ([_VP, _F], _INT),
    "rbc_set_router": ([_VP, _VP, _U32], _INT),
    "rbc_set_profiling": ([_VP, _INT], _INT),
    "rbc_get_profile": ([_VP, C.POINTER(Profile)], _INT),
    "rbc_kernel_launches": ([], _U64),
    "rbc_selftest_bounded_wait": ([C.POINTER(_U32), C.POINTER(_U32), _VP], _INT),
    "rbc_brute_knn": ([_VP, _U64, _U32, _VP, _U64, _U32, _U32, _U32, _INT, _VP, _VP, _U32, _VP], _INT),
    "rbc_brute_knn_noalloc": ([_VP, _U64, _U32, _VP, _U64, _U32, _U32, _U32, _INT, _VP, _VP, _U32, _VP], _INT),
    "rbc_brute_range_count": ([_VP, _U64, _U32, _VP, _U64, _U32, _U32, _INT, _VP, _VP, _VP], _INT),
    "rbc_build_f64": ([_VP, _U64, _U32, _U32, C.POINTER(BuildParams), _VP, C.POINTER(_VP)], _INT),
    "rbc_query_f64": ([_VP, _VP, _U64, _U32, _U32, _U32, _VP, _VP, _U32, _VP], _INT),
    "rbc_brute_knn_f64": ([_VP, _U64, _U32, _VP, _U64, _U32, _U32, _U32, _INT, _VP, _VP, _U32, C.POINTER(_U64), _VP],
                          _INT),
    "rbc_brute_range_count_f64": ([_VP, _U64, _U32, _VP, _U64, _U32, _U32, _INT, _VP, _VP, _VP], _INT),
    "rbc_synth": ([_INT, _U64, _U64, _U64, _U64, _U32, _U32, _VP, _U32, _F, _F, _VP], _INT),
    "rbc_read_matrix_bin": ([C.c_char_p, _VP, _U64, _U32, _U32], _INT),
    "rbc_read_matrix_text": ([C.c_char_p, _VP, _U64, _U32, _U32], _INT),
    "rbc_write_matrix_bin": ([C.c_char_p, _VP, _U64, _U32, _U32], _INT),
    "rbc_write_neighbors_bin": ([C.c_char_p, _VP, _VP, _U64, _U32, _U32], _INT),
    "rbc_write_neighbors_text": ([C.c_char_p, _VP, _VP, _U64, _U32, _U32], _INT),
    "rbc_read_matrix_bin_f64": ([C.c_char_p, _VP, _U64, _U32, _U32], _INT),
    "rbc_read_matrix_text_f64": ([C.c_char_p, _VP, _U64, _U32, _U32], _INT),
    "rbc_write_matrix_bin_f64": ([C.c_char_p, _VP, _U64, _U32, _U32], _INT),
    "rbc_write_neighbors_bin_f64": ([C.c_char_p, _VP, _VP, _U64, _U32, _U32], _INT),
    "rbc_write_neighbors_text_f64": ([C.c_char_p, _VP, _VP, _U64, _U32, _U32], _INT),
}

_lib = None


def lib():
    """Load the engine library (build it first with build_ext.build())."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RBCError(ERR_CUDA, f"engine library not built: {LIB_PATH}")
        L = C.CDLL(LIB_PATH)
        for name, (args, res) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _lib = L
    return _lib


def check(rc):
    if rc != OK:
        raise RBCError(rc, lib().rbc_last_error().decode())


def _ptr(t):
    if t is None:
        return None
    if isinstance(t, np.ndarray):
        return t.ctypes.data
    return t.data_ptr()


def _stream(stream):
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return s.cuda_stream


def _is_f64(a):
    import torch
    return (isinstance(a, np.ndarray) and a.dtype == np.float64) or \
        (isinstance(a, torch.Tensor) and a.dtype == torch.float64)


def _dev(a, dtype=None):
    import torch
    if isinstance(a, np.ndarray):
        a = torch.from_numpy(np.ascontiguousarray(a))
    if dtype is not None:
        a = a.to(dtype)
    return a.cuda().contiguous()


class Index:
    """An RBC index over the rows of X (n x d, CUDA tensor or numpy).  float64
    data builds the double-precision variant (rbc_build_f64): its queries take
    and return doubles."""

    def __init__(self, X, num_reps, s=0, metric=L2, flags=0, seed=0, rep_ids=None, stream=None):
        import torch
        self.f64 = _is_f64(X)
        X = _dev(X, torch.float64 if self.f64 else torch.float32)
        n, d = X.shape
        p = BuildParams(num_reps, s, metric, flags, seed, None)
        self._rep_buf = None
        if rep_ids is not None:
            self._rep_buf = np.ascontiguousarray(rep_ids, dtype=np.uint32)
            p.rep_ids = self._rep_buf.ctypes.data_as(C.POINTER(C.c_uint32))
        h = C.c_void_p()
        build = lib().rbc_build_f64 if self.f64 else lib().rbc_build
        check(build(X.data_ptr(), n, d, X.stride(0), C.byref(p), _stream(stream), C.byref(h)))
        self.h = h
        self.n, self.d, self.metric = n, d, metric

    @classmethod
    def load(cls, path):
        """An index read from a file written by save()."""
        self = cls.__new__(cls)
        h = C.c_void_p()
        check(lib().rbc_load(path.encode(), C.byref(h)))
        self.h = h
        self._rep_buf = None
        inf = self.info()
        self.n, self.d, self.metric = inf["n"], inf["d"], inf["metric"]
        self.f64 = bool(inf["flags"] & BUILD_F64)
        return self

    def save(self, path):
        check(lib().rbc_save(self.h, path.encode()))

    def close(self):
        if getattr(self, "h", None):
            lib().rbc_destroy(self.h)
            self.h = None

    __del__ = close

    def query(self, Q, k, mode=QUERY_EXACT, stream=None, out=None):
        """Returns (ids uint32-as-int32 tensor [m,k], dists float32 [m,k]) on the device
        (float64 dists on a double-precision index)."""
        import torch
        dt = torch.float64 if self.f64 else torch.float32
        Q = _dev(Q, dt)
        m = Q.shape[0]
        if out is None:
            ids = torch.empty((m, k), dtype=torch.int32, device=Q.device)
            dists = torch.empty((m, k), dtype=dt, device=Q.device)
        else:
            ids, dists = out
        fn = lib().rbc_query_f64 if self.f64 else lib().rbc_query
        check(fn(self.h, Q.data_ptr(), m, Q.stride(0), k, mode, ids.data_ptr(), dists.data_ptr(), ids.stride(0),
                 _stream(stream)))
        return ids, dists

    def query_host(self, Q, k, mode=QUERY_EXACT, out=None):
        """Host in, host out (the copies are part of the call)."""
        Q = np.ascontiguousarray(Q, dtype=np.float32)
        m = Q.shape[0]
        if out is None:
            ids = np.empty((m, k), np.uint32)
            dists = np.empty((m, k), np.float32)
        else:
            ids, dists = out
        check(lib().rbc_query_host(self.h, _ptr(Q), m, Q.shape[1], k, mode, _ptr(ids), _ptr(dists), ids.shape[1]))
        return ids, dists

    def info(self):
        i = IndexInfo()
        check(lib().rbc_get_info(self.h, C.byref(i)))
        return {f: getattr(i, f) for f, _ in IndexInfo._fields_}

    def reps(self):
        nr = self.info()["num_reps"]
        out = np.empty(nr, np.uint32)
        check(lib().rbc_get_reps(self.h, out.ctypes.data))
        return out

    def partition(self):
        inf = self.info()
        off = np.empty(inf["num_reps"] + 1, np.uint64)
        mem = np.empty(inf["n"], np.uint32)
        rad = np.empty(inf["num_reps"], np.float32)
        check(lib().rbc_get_partition(self.h, off.ctypes.data, mem.ctypes.data, rad.ctypes.data))
        return off, mem, rad

    def oneshot(self):
        inf = self.info()
        lists = np.empty((inf["num_reps"], inf["s"]), np.uint32)
        counts = np.empty(inf["num_reps"], np.uint32)
        check(lib().rbc_get_oneshot(self.h, lists.ctypes.data, counts.ctypes.data))
        return lists, counts

    def stats(self):
        st = QueryStats()
        check(lib().rbc_get_query_stats(self.h, C.byref(st)))
        return {f: getattr(st, f) for f, _ in QueryStats._fields_}

    def fallback_queries(self):
        """Indices of the queries the last tensor-form call recomputed on the FP32 path."""
        n = C.c_uint64()
        check(lib().rbc_get_fallback_queries(self.h, None, 0, C.byref(n)))
        out = np.empty(n.value, np.uint32)
        if n.value:
            check(lib().rbc_get_fallback_queries(self.h, out.ctypes.data, n.value, C.byref(n)))
        return out

    def set_profiling(self, enable=True):
        check(lib().rbc_set_profiling(self.h, int(enable)))

    def owner_labels(self, Q, stream=None):
        """The list owning each query's exact nearest neighbour (router training labels)."""
        import torch
        Q = _dev(Q, torch.float32)
        lab = torch.empty(Q.shape[0], dtype=torch.int32, device=Q.device)
        check(lib().rbc_owner_labels(self.h, Q.data_ptr(), Q.shape[0], Q.stride(0), lab.data_ptr(), _stream(stream)))
        return lab

    def router_labels(self, Q, k, stream=None):
        """Labels for both router heads: the list owning each query's exact
        nearest neighbour, the query's exact k-th distance and its nearest
        representative's distance."""
        import torch
        Q = _dev(Q, torch.float32)
        lab = torch.empty(Q.shape[0], dtype=torch.int32, device=Q.device)
        dist = torch.empty(Q.shape[0], dtype=torch.float32, device=Q.device)
        near = torch.empty(Q.shape[0], dtype=torch.float32, device=Q.device)
        check(lib().rbc_router_labels(self.h, Q.data_ptr(), Q.shape[0], Q.stride(0), k, lab.data_ptr(),
                                      dist.data_ptr(), near.data_ptr(), _stream(stream)))
        return lab, dist, near

    def set_tuning(self, tq=0, item_rows=0):
        check(lib().rbc_set_tuning(self.h, tq, item_rows))

    def autotune(self, Q, k, cache_path=None, stream=None):
        import torch
        Q = _dev(Q, torch.float32)
        check(lib().rbc_autotune(self.h, Q.data_ptr(), Q.shape[0], Q.stride(0), k,
                                 cache_path.encode() if cache_path else None, _stream(stream)))

    def set_tc_tuning(self, probes=0, probe_rows=0):
        check(lib().rbc_set_tc_tuning(self.h, probes, probe_rows))

    def set_tc_probe_cap(self, rows):
        """Rows of each probed list the tensor probe round takes (0: all)."""
        check(lib().rbc_set_tc_probe_cap(self.h, rows))

    def tc_tuning(self):
        """(probes, probe_rows) of the tensor form; 0 means the default."""
        p, r = C.c_uint32(), C.c_uint64()
        check(lib().rbc_get_tc_tuning(self.h, C.byref(p), C.byref(r)))
        return p.value, r.value

    def autotune_tc(self, Q, k, mode=QUERY_EXACT_TC, stream=None):
        """Tensor-form knobs (probed lists, FP32/tensor split) timed on sample queries."""
        import torch
        Q = _dev(Q, torch.float32)
        check(lib().rbc_autotune_tc(self.h, Q.data_ptr(), Q.shape[0], Q.stride(0), k, mode, _stream(stream)))

    def set_router(self, router, probes=1):
        self._router = router
        check(lib().rbc_set_router(self.h, router.h if router is not None else None, probes))

    def profile(self):
        p = Profile()
        check(lib().rbc_get_profile(self.h, C.byref(p)))
        return {"search_launches": p.search_launches, "search_ms": p.search_ms, "pruned_launches": p.pruned_launches,
                "pruned_ms": p.pruned_ms, "pruned_pairs": p.pruned_pairs}


def kernel_launches():
    return int(lib().rbc_kernel_launches())


class Batch:
    """Many (index, queries) instances answered by one CUDA graph per run."""

    def __init__(self):
        h = C.c_void_p()
        check(lib().rbc_batch_create(C.byref(h)))
        self.h = h
        self.keep = []

    def add(self, index, Q, k, mode=QUERY_EXACT):
        """Queries Q (CUDA tensor, kept alive by the batch); returns (ids, dists)
        filled by run().  mode QUERY_EXACT_TC answers the instance with the
        tensor form (BF16 index, k <= 32)."""
        import torch
        m = Q.shape[0]
        ids = torch.empty((m, k), dtype=torch.int32, device=Q.device)
        dists = torch.empty((m, k), dtype=torch.float32, device=Q.device)
        check(lib().rbc_batch_add_mode(self.h, index.h, Q.data_ptr(), m, Q.stride(0), k, mode, ids.data_ptr(),
                                       dists.data_ptr(), k))
        self.keep.append((index, Q, ids, dists))
        return ids, dists

    def run(self, stream=None):
        check(lib().rbc_batch_run(self.h, _stream(stream)))

    def close(self):
        if getattr(self, "h", None):
            lib().rbc_batch_destroy(self.h)
            self.h = None

    __del__ = close


class Router:
    """The learned list router (MLP d -> hidden -> hidden -> lists, GELU)."""

    def __init__(self, d, hidden, num_lists, seed=0, distance_head=False):
        h = C.c_void_p()
        create = lib().rbc_router_create_with_distance if distance_head else lib().rbc_router_create
        check(create(d, hidden, num_lists, seed, C.byref(h)))
        self.h = h
        self.d, self.hidden, self.num_lists = d, hidden, num_lists
        self.distance_head = distance_head

    def close(self):
        if getattr(self, "h", None):
            lib().rbc_router_destroy(self.h)
            self.h = None

    __del__ = close

    def num_params(self):
        n = C.c_uint64()
        check(lib().rbc_router_num_params(self.h, C.byref(n)))
        return n.value

    def get_params(self):
        p = np.empty(self.num_params(), np.float32)
        check(lib().rbc_router_get_params(self.h, p.ctypes.data))
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        check(lib().rbc_router_set_params(self.h, p.ctypes.data))

    def gradients(self, Q, labels, stream=None):
        import torch
        Q = _dev(Q, torch.float32)
        lab = _dev(np.asarray(labels, np.int32) if isinstance(labels, np.ndarray) else labels, torch.int32)
        g = np.empty(self.num_params(), np.float32)
        loss = C.c_float()
        check(lib().rbc_router_gradients(self.h, Q.data_ptr(), Q.shape[0], Q.stride(0), lab.data_ptr(),
                                         C.byref(loss), g.ctypes.data, _stream(stream)))
        return loss.value, g

    def train(self, Q, labels, epochs=1, batch=1024, lr=1e-3, seed=0, stream=None):
        import torch
        Q = _dev(Q, torch.float32)
        lab = _dev(labels, torch.int32)
        loss = C.c_float()
        check(lib().rbc_router_train(self.h, Q.data_ptr(), Q.shape[0], Q.stride(0), lab.data_ptr(), epochs, batch,
                                     lr, seed, C.byref(loss), _stream(stream)))
        return loss.value

    def logits(self, Q, stream=None):
        import torch
        Q = _dev(Q, torch.float32)
        out = torch.empty((Q.shape[0], self.num_lists), dtype=torch.float32, device=Q.device)
        check(lib().rbc_router_logits(self.h, Q.data_ptr(), Q.shape[0], Q.stride(0), out.data_ptr(),
                                      _stream(stream)))
        return out

    def top_lists(self, Q, P, stream=None):
        """The P most likely lists per query (largest logit first, ties to the lower list)."""
        import torch
        Q = _dev(Q, torch.float32)
        out = torch.empty((Q.shape[0], P), dtype=torch.int32, device=Q.device)
        check(lib().rbc_router_top_lists(self.h, Q.data_ptr(), Q.shape[0], Q.stride(0), P, out.data_ptr(),
                                         _stream(stream)))
        return out

    def gradients_with_distance(self, Q, labels, targets, stream=None):
        """Loss and gradients of one batch with both heads (targets in the
        distance head's normalised units, NaN for none)."""
        import torch
        Q = _dev(Q, torch.float32)
        lab = _dev(np.asarray(labels, np.int32) if isinstance(labels, np.ndarray) else labels, torch.int32)
        tg = _dev(np.asarray(targets, np.float32) if isinstance(targets, np.ndarray) else targets, torch.float32)
        g = np.empty(self.num_params(), np.float32)
        loss = C.c_float()
        check(lib().rbc_router_gradients_with_distance(self.h, Q.data_ptr(), Q.shape[0], Q.stride(0), lab.data_ptr(),
                                                       tg.data_ptr(), C.byref(loss), g.ctypes.data, _stream(stream)))
        return loss.value, g

    def train_with_distance(self, Q, labels, dist, near, epochs=1, batch=1024, lr=1e-3, seed=0, stream=None):
        import torch
        Q = _dev(Q, torch.float32)
        lab = _dev(labels, torch.int32)
        dd = _dev(dist, torch.float32)
        nn = _dev(near, torch.float32)
        loss = C.c_float()
        check(lib().rbc_router_train_with_distance(self.h, Q.data_ptr(), Q.shape[0], Q.stride(0), lab.data_ptr(),
                                                   dd.data_ptr(), nn.data_ptr(), epochs, batch, lr, seed,
                                                   C.byref(loss), _stream(stream)))
        return loss.value

    def predict_distance(self, Q, near, stream=None):
        import torch
        Q = _dev(Q, torch.float32)
        nn = _dev(near, torch.float32)
        out = torch.empty(Q.shape[0], dtype=torch.float32, device=Q.device)
        check(lib().rbc_router_predict_distance(self.h, Q.data_ptr(), Q.shape[0], Q.stride(0), nn.data_ptr(),
                                                out.data_ptr(), _stream(stream)))
        return out

    def distance_params(self):
        """(mu, sigma, margin): log(distance / nearest representative's) = mu + sigma (head output + margin)."""
        mu, sg, mg = C.c_float(), C.c_float(), C.c_float()
        check(lib().rbc_router_distance_params(self.h, C.byref(mu), C.byref(sg), C.byref(mg)))
        return mu.value, sg.value, mg.value

    def set_distance_margin(self, margin):
        check(lib().rbc_router_set_distance_margin(self.h, float(margin)))


def brute_knn_f64(X, Q, k, metric=L2, stream=None):
    """Double-precision brute force: (ids, float64 dists, queries searched in double)."""
    import torch
    X = _dev(X, torch.float64)
    Q = _dev(Q, torch.float64)
    m = Q.shape[0]
    ids = torch.empty((m, k), dtype=torch.int32, device=Q.device)
    dists = torch.empty((m, k), dtype=torch.float64, device=Q.device)
    nopen = C.c_uint64()
    check(lib().rbc_brute_knn_f64(X.data_ptr(), X.shape[0], X.stride(0), Q.data_ptr(), m, Q.stride(0), Q.shape[1],
                                  k, metric, ids.data_ptr(), dists.data_ptr(), k, C.byref(nopen), _stream(stream)))
    return ids, dists, nopen.value


def brute_knn(X, Q, k, metric=L2, stream=None):
    """Brute-force exact k-NN; float64 inputs take the double-precision variant."""
    import torch
    if _is_f64(X):
        return brute_knn_f64(X, Q, k, metric, stream)[:2]
    X = _dev(X, torch.float32)
    Q = _dev(Q, torch.float32)
    m = Q.shape[0]
    ids = torch.empty((m, k), dtype=torch.int32, device=Q.device)
    dists = torch.empty((m, k), dtype=torch.float32, device=Q.device)
    check(lib().rbc_brute_knn(X.data_ptr(), X.shape[0], X.stride(0), Q.data_ptr(), m, Q.stride(0), Q.shape[1], k,
                              metric, ids.data_ptr(), dists.data_ptr(), k, _stream(stream)))
    return ids, dists


def range_count(X, Q, ranges, metric=L2, stream=None):
    import torch
    if _is_f64(X):
        X = _dev(X, torch.float64)
        Q = _dev(Q, torch.float64)
        r = _dev(ranges, torch.float64)
        cnt = torch.empty(Q.shape[0], dtype=torch.int32, device=Q.device)
        check(lib().rbc_brute_range_count_f64(X.data_ptr(), X.shape[0], X.stride(0), Q.data_ptr(), Q.shape[0],
                                              Q.stride(0), Q.shape[1], metric, r.data_ptr(), cnt.data_ptr(),
                                              _stream(stream)))
        return cnt
    X = _dev(X, torch.float32)
    Q = _dev(Q, torch.float32)
    r = _dev(ranges, torch.float32)
    cnt = torch.empty(Q.shape[0], dtype=torch.int32, device=Q.device)
    check(lib().rbc_brute_range_count(X.data_ptr(), X.shape[0], X.stride(0), Q.data_ptr(), Q.shape[0], Q.stride(0),
                                      Q.shape[1], metric, r.data_ptr(), cnt.data_ptr(), _stream(stream)))
    return cnt


def synth(kind, seed, stream_id, rows, d, r0=0, ncomp=1, sigma_lo=0.0, sigma_hi=0.0, out=None, stream=None):
    """Counter-based synthetic rows on the device (same bits as the CPU recipe)."""
    import torch
    if out is None:
        out = torch.empty((rows, d), dtype=torch.float32, device="cuda")
    check(lib().rbc_synth(kind, seed, stream_id, r0, rows, d, out.stride(0), out.data_ptr(), ncomp, sigma_lo,
                          sigma_hi, _stream(stream)))
    return out


def u32(t):
    """uint32 view of an int32 id tensor as numpy."""
    a = t.cpu().numpy() if hasattr(t, "cpu") else np.asarray(t)
    return a.view(np.uint32)


# ---------------------------------------------------------------- file I/O
def read_matrix_bin(path, rows, cols, ld=None):
    ld = ld or cols
    out = np.zeros((rows, ld), np.float32)
    check(lib().rbc_read_matrix_bin(path.encode(), out.ctypes.data, rows, cols, ld))
    return out


def read_matrix_text(path, rows, cols, ld=None):
    ld = ld or cols
    out = np.zeros((rows, ld), np.float32)
    check(lib().rbc_read_matrix_text(path.encode(), out.ctypes.data, rows, cols, ld))
    return out


def write_matrix_bin(path, A):
    A = np.ascontiguousarray(A, np.float32)
    check(lib().rbc_write_matrix_bin(path.encode(), A.ctypes.data, A.shape[0], A.shape[1], A.shape[1]))


def write_neighbors_bin(path, ids, dists):
    ids = np.ascontiguousarray(ids, np.uint32)
    dists = np.ascontiguousarray(dists, np.float32)
    check(lib().rbc_write_neighbors_bin(path.encode(), ids.ctypes.data, dists.ctypes.data, ids.shape[0],
                                        ids.shape[1], ids.shape[1]))


def write_neighbors_text(path, ids, dists):
    ids = np.ascontiguousarray(ids, np.uint32)
    dists = np.ascontiguousarray(dists, np.float32)
    check(lib().rbc_write_neighbors_text(path.encode(), ids.ctypes.data, dists.ctypes.data, ids.shape[0],
                                         ids.shape[1], ids.shape[1]))
