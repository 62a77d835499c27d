"""ctypes binding of the CPU oracle (oracle/rbc_oracle.c) and of the reference
build in oracle/_ref.

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() as
the checker, and by bench.py's CPU-baseline leg.  The product library never
imports this module.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "librbc_oracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libref.so")
REF64_PATH = os.path.join(HERE, "_ref", "libref_f64.so")  # the reference built with real = double
# where the reference's sources are: this environment variable, else the tree
# the last `make ref` compiled (recorded beside its outputs)
REF_ENV = "RBC_REFERENCE_DIR"
REF_RECORD = os.path.join(HERE, "_ref", "SOURCE_DIR")

L2, L1 = 0, 1
DUMMY = 0xFFFFFFFF
FLT_MAX = np.finfo(np.float32).max

_lib = None
_ref = None
_ref64 = None

F32P = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
U32P = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
U64P = np.ctypeslib.ndpointer(np.uint64, flags="C_CONTIGUOUS")
F64P = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")


def ref_dir():
    """The reference's source tree: $RBC_REFERENCE_DIR, else the one the last
    reference build recorded; None when neither is present on this machine."""
    cands = [os.environ.get(REF_ENV)]
    if os.path.exists(REF_RECORD):
        cands.append(open(REF_RECORD).read().strip())
    for c in cands:
        if c and os.path.isdir(c):
            return c
    return None


def build(with_ref=None, source=None):
    """Compile the oracle (always) and the reference build (when its sources
    are present: `source`, else ref_dir())."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    src = source or ref_dir()
    if with_ref is None:
        with_ref = src is not None
    if with_ref and src:
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF_DIR={src}"], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build(with_ref=False)
        L = C.CDLL(LIB_PATH)
        L.orc_knn.argtypes = [F32P, C.c_uint64, C.c_uint32, F32P, C.c_uint64, C.c_uint32,
                              C.c_uint32, C.c_uint32, C.c_int, U32P, F32P, C.c_uint32, C.c_int]
        L.orc_knn.restype = C.c_int
        L.orc_brute_1nn.argtypes = [F32P, C.c_uint64, C.c_uint32, F32P, C.c_uint64, C.c_uint32,
                                    C.c_uint32, C.c_int, U32P]
        L.orc_range_count.argtypes = [F32P, C.c_uint64, C.c_uint32, F32P, C.c_uint64, C.c_uint32,
                                      C.c_uint32, C.c_int, F32P, U32P]
        L.orc_nearest_rep.argtypes = [F32P, C.c_uint64, C.c_uint32, F32P, C.c_uint32, C.c_uint32,
                                      C.c_uint32, C.c_int, U32P, F32P]
        L.orc_partition.argtypes = [F32P, C.c_uint64, C.c_uint32, U32P, C.c_uint32, C.c_uint32,
                                    C.c_int, U32P, F32P, U64P, U32P, F32P]
        L.orc_oneshot_build.argtypes = [F32P, C.c_uint64, C.c_uint32, U32P, C.c_uint32, C.c_uint32,
                                        C.c_int, C.c_uint32, U32P, C.c_uint32, U32P, F32P]
        L.orc_oneshot_query.argtypes = [F32P, C.c_uint32, U32P, C.c_uint32, U32P, C.c_uint32, U32P,
                                        F32P, C.c_uint64, C.c_uint32, C.c_uint32, C.c_int, C.c_uint32,
                                        U32P, F32P, C.c_uint32]
        L.orc_distance.argtypes = [F32P, F32P, C.c_uint32, C.c_int]
        L.orc_distance.restype = C.c_float
        L.orc_distance_f64.argtypes = [F32P, F32P, C.c_uint32, C.c_int]
        L.orc_distance_f64.restype = C.c_double
        L.orc_knn_f64.argtypes = [F64P, C.c_uint64, C.c_uint32, F64P, C.c_uint64, C.c_uint32,
                                  C.c_uint32, C.c_uint32, C.c_int, U32P, F64P, C.c_uint32, C.c_int]
        L.orc_knn_f64.restype = C.c_int
        L.orc_brute_1nn_f64.argtypes = [F64P, C.c_uint64, C.c_uint32, F64P, C.c_uint64, C.c_uint32,
                                        C.c_uint32, C.c_int, U32P]
        L.orc_range_count_f64.argtypes = [F64P, C.c_uint64, C.c_uint32, F64P, C.c_uint64, C.c_uint32,
                                          C.c_uint32, C.c_int, F64P, U32P]
        L.orc_distance64.argtypes = [F64P, F64P, C.c_uint32, C.c_int]
        L.orc_distance64.restype = C.c_double
        L.orc_geometric_table.argtypes = [C.c_uint32, C.c_uint32, U32P]
        L.orc_synth.argtypes = [C.c_int, C.c_uint64, C.c_uint64, C.c_uint64, C.c_uint64, C.c_uint32,
                                C.c_uint32, F32P, C.c_uint32, C.c_float, C.c_float, U32P]
        _lib = L
    return _lib


# ---------------------------------------------------------------- reference
class RefMatrix(C.Structure):
    """The reference's `matrix` (defs.h:56-63), passed by value."""
    _fields_ = [("mat", C.c_void_p), ("r", C.c_uint32), ("c", C.c_uint32), ("pr", C.c_uint32),
                ("pc", C.c_uint32), ("ld", C.c_uint32)]


def ref_available():
    return os.path.exists(REF_PATH)


def ref_lib():
    """The reference's own code compiled from its sources (oracle/Makefile `ref`)."""
    global _ref
    if _ref is None:
        R = C.CDLL(REF_PATH)
        fn = getattr(R, "_Z8bruteCPU6matrixS_Pj")   # void bruteCPU(matrix, matrix, unint*)
        fn.argtypes = [RefMatrix, RefMatrix, C.c_void_p]
        fn.restype = None
        dv = getattr(R, "_Z7distVec6matrixS_jj")    # real distVec(matrix, matrix, unint, unint)
        dv.argtypes = [RefMatrix, RefMatrix, C.c_uint32, C.c_uint32]
        dv.restype = C.c_float
        _ref = (R, fn, dv)
    return _ref


def ref64_available():
    return os.path.exists(REF64_PATH)


def ref64_lib():
    """The reference's double-precision build (oracle/Makefile `ref`, real = double)."""
    global _ref64
    if _ref64 is None:
        R = C.CDLL(REF64_PATH)
        fn = getattr(R, "_Z8bruteCPU6matrixS_Pj")   # void bruteCPU(matrix, matrix, unint*)
        fn.argtypes = [RefMatrix, RefMatrix, C.c_void_p]
        fn.restype = None
        dv = getattr(R, "_Z7distVec6matrixS_jj")    # real distVec(matrix, matrix, unint, unint)
        dv.argtypes = [RefMatrix, RefMatrix, C.c_uint32, C.c_uint32]
        dv.restype = C.c_double
        _ref64 = (R, fn, dv)
    return _ref64


def pad16(v):
    return (v + 15) // 16 * 16


def ref_brute_cpu_f64(X, Q):
    """The double build's bruteCPU on logical X (n x d), Q (m x d) float64."""
    _, fn, _ = ref64_lib()
    n, d = X.shape
    m = Q.shape[0]
    pc = pad16(d)
    Xp = np.zeros((pad16(n), pc), np.float64)
    Xp[:n, :d] = X
    Qp = np.zeros((pad16(m), pc), np.float64)
    Qp[:m, :d] = Q
    mx = RefMatrix(Xp.ctypes.data, n, d, Xp.shape[0], pc, pc)
    mq = RefMatrix(Qp.ctypes.data, m, d, Qp.shape[0], pc, pc)
    out = np.zeros(m, np.uint32)
    fn(mx, mq, out.ctypes.data)
    return out


def ref_dist_vec_f64(Q, X, i, j):
    """The double build's distVec(Q, X, i, j) on logical float64 arrays of equal width."""
    _, _, dv = ref64_lib()
    d = X.shape[1]
    Qc = np.ascontiguousarray(Q, np.float64)
    Xc = np.ascontiguousarray(X, np.float64)
    mq = RefMatrix(Qc.ctypes.data, Qc.shape[0], d, Qc.shape[0], d, d)
    mx = RefMatrix(Xc.ctypes.data, Xc.shape[0], d, Xc.shape[0], d, d)
    return dv(mq, mx, i, j)


def ref_brute_cpu(X, Q):
    """Run the reference's bruteCPU (brute.cu:91-112) on logical X (n x d), Q (m x d)."""
    _, fn, _ = ref_lib()
    n, d = X.shape
    m = Q.shape[0]
    pc = pad16(d)
    Xp = np.zeros((pad16(n), pc), np.float32)
    Xp[:n, :d] = X
    Qp = np.zeros((pad16(m), pc), np.float32)
    Qp[:m, :d] = Q
    mx = RefMatrix(Xp.ctypes.data, n, d, Xp.shape[0], pc, pc)
    mq = RefMatrix(Qp.ctypes.data, m, d, Qp.shape[0], pc, pc)
    out = np.zeros(m, np.uint32)
    fn(mx, mq, out.ctypes.data)
    return out


def ref_brute_cpu_raw(Xp, n, d, Qp, m, out):
    """bruteCPU on already padded arrays (used by the timed CPU baseline)."""
    _, fn, _ = ref_lib()
    pc = Xp.shape[1]
    mx = RefMatrix(Xp.ctypes.data, n, d, Xp.shape[0], pc, pc)
    mq = RefMatrix(Qp.ctypes.data, m, d, Qp.shape[0], pc, pc)
    fn(mx, mq, out.ctypes.data)


def ref_dist_vec(Q, X, i, j):
    _, _, dv = ref_lib()
    n, d = X.shape
    m = Q.shape[0]
    pc = pad16(d)
    Xp = np.zeros((pad16(n), pc), np.float32)
    Xp[:n, :d] = X
    Qp = np.zeros((pad16(m), pc), np.float32)
    Qp[:m, :d] = Q
    mx = RefMatrix(Xp.ctypes.data, n, d, Xp.shape[0], pc, pc)
    mq = RefMatrix(Qp.ctypes.data, m, d, Qp.shape[0], pc, pc)
    return dv(mq, mx, i, j)


# ---------------------------------------------------------------- oracle API
def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


def knn(X, Q, k, metric=L2, threads=None):
    """Exact k-NN under (dist, id). Returns (ids[m,k] uint32, dists[m,k] float32)."""
    X = _c(X, np.float32)
    Q = _c(Q, np.float32)
    n, d = X.shape
    m = Q.shape[0]
    ids = np.empty((m, k), np.uint32)
    dists = np.empty((m, k), np.float32)
    if threads is None:
        threads = os.cpu_count() or 1
    rc = lib().orc_knn(X, n, d, Q, m, d, d, k, metric, ids, dists, k, threads)
    assert rc == 0
    return ids, dists


def knn_f64(X, Q, k, metric=L2, threads=None):
    """Exact k-NN of the double build under (dist, id): (ids[m,k] uint32, dists[m,k] float64)."""
    X = _c(X, np.float64)
    Q = _c(Q, np.float64)
    n, d = X.shape
    m = Q.shape[0]
    ids = np.empty((m, k), np.uint32)
    dists = np.empty((m, k), np.float64)
    if threads is None:
        threads = os.cpu_count() or 1
    rc = lib().orc_knn_f64(X, n, d, Q, m, d, d, k, metric, ids, dists, k, threads)
    assert rc == 0
    return ids, dists


def brute_1nn_f64(X, Q, metric=L2):
    X = _c(X, np.float64)
    Q = _c(Q, np.float64)
    out = np.empty(Q.shape[0], np.uint32)
    lib().orc_brute_1nn_f64(X, X.shape[0], X.shape[1], Q, Q.shape[0], Q.shape[1], X.shape[1], metric, out)
    return out


def range_count_f64(X, Q, ranges, metric=L2):
    X = _c(X, np.float64)
    Q = _c(Q, np.float64)
    out = np.empty(Q.shape[0], np.uint32)
    lib().orc_range_count_f64(X, X.shape[0], X.shape[1], Q, Q.shape[0], Q.shape[1], X.shape[1], metric,
                              _c(ranges, np.float64), out)
    return out


def distance64(a, b, metric=L2):
    a = _c(a, np.float64)
    b = _c(b, np.float64)
    return lib().orc_distance64(a, b, a.shape[0], metric)


def brute_1nn(X, Q, metric=L2):
    X = _c(X, np.float32)
    Q = _c(Q, np.float32)
    out = np.empty(Q.shape[0], np.uint32)
    lib().orc_brute_1nn(X, X.shape[0], X.shape[1], Q, Q.shape[0], Q.shape[1], X.shape[1], metric, out)
    return out


def range_count(X, Q, ranges, metric=L2):
    X = _c(X, np.float32)
    Q = _c(Q, np.float32)
    out = np.empty(Q.shape[0], np.uint32)
    lib().orc_range_count(X, X.shape[0], X.shape[1], Q, Q.shape[0], Q.shape[1], X.shape[1], metric,
                          _c(ranges, np.float32), out)
    return out


def nearest_rep(A, R, metric=L2):
    A = _c(A, np.float32)
    R = _c(R, np.float32)
    rep = np.empty(A.shape[0], np.uint32)
    dist = np.empty(A.shape[0], np.float32)
    lib().orc_nearest_rep(A, A.shape[0], A.shape[1], R, R.shape[0], R.shape[1], A.shape[1], metric,
                          rep, dist)
    return rep, dist


def partition(X, rep_ids, metric=L2):
    """Exact-search lists: (owner, owner_dist, offsets[nr+1], members, radius[nr])."""
    X = _c(X, np.float32)
    rep_ids = _c(rep_ids, np.uint32)
    n, d = X.shape
    nr = rep_ids.shape[0]
    owner = np.empty(n, np.uint32)
    odist = np.empty(n, np.float32)
    offsets = np.empty(nr + 1, np.uint64)
    members = np.empty(n, np.uint32)
    radius = np.empty(nr, np.float32)
    lib().orc_partition(X, n, d, rep_ids, nr, d, metric, owner, odist, offsets, members, radius)
    return owner, odist, offsets, members, radius


def oneshot_build(X, rep_ids, s, metric=L2):
    """One-shot lists: (lists[nr, s], counts[nr], rho[nr])."""
    X = _c(X, np.float32)
    rep_ids = _c(rep_ids, np.uint32)
    n, d = X.shape
    nr = rep_ids.shape[0]
    lists = np.full((nr, s), DUMMY, np.uint32)
    counts = np.empty(nr, np.uint32)
    rho = np.empty(nr, np.float32)
    lib().orc_oneshot_build(X, n, d, rep_ids, nr, d, metric, s, lists, s, counts, rho)
    return lists, counts, rho


def oneshot_query(X, rep_ids, lists, counts, Q, k, metric=L2):
    X = _c(X, np.float32)
    Q = _c(Q, np.float32)
    lists = _c(lists, np.uint32)
    m, d = Q.shape
    ids = np.empty((m, k), np.uint32)
    dists = np.empty((m, k), np.float32)
    lib().orc_oneshot_query(X, d, _c(rep_ids, np.uint32), len(rep_ids), lists, lists.shape[1],
                            _c(counts, np.uint32), Q, m, d, d, metric, k, ids, dists, k)
    return ids, dists


def distance(a, b, metric=L2):
    a = _c(a, np.float32)
    b = _c(b, np.float32)
    return lib().orc_distance(a, b, a.shape[0], metric)


def distance_f64(a, b, metric=L2):
    a = _c(a, np.float32)
    b = _c(b, np.float32)
    return lib().orc_distance_f64(a, b, a.shape[0], metric)


# ---------------------------------------------------------------- synthetic data
KIND_UNIFORM, KIND_MIXTURE, KIND_GEOMETRIC = 0, 1, 2


def geometric_table(num=20, den=21):
    T = np.empty(256, np.uint32)
    lib().orc_geometric_table(num, den, T)
    return T


def synth(kind, seed, stream, n, d, ncomp=1, sigma_lo=0.0, sigma_hi=0.0, r0=0, table=None):
    """Rows [r0, r0+n) of the counter-based synthetic generator (same bits as the GPU's)."""
    out = np.empty((n, d), np.float32)
    T = table if table is not None else geometric_table()
    lib().orc_synth(kind, seed, stream, r0, r0 + n, d, d, out, ncomp, sigma_lo, sigma_hi,
                    _c(T, np.uint32))
    return out
