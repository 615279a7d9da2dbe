"""ctypes wrapper of the CPU oracle (oracle/haplo_oracle.cpp).

TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and the
CPU-baseline legs of bench.py as the checker / CPU baseline.  The product
never imports this module.  Parity status: unpinned against reference
outputs (the Julia reference cannot run here); see haplo_oracle.cpp.

Arrays use the reference's Julia shapes in Fortran order: q (K, I),
p (K, 4J), XtX_q (K, K, I), XtX_p (K, K, 4J).
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_lib = None


def load():
    return _load()


def _load():
    global _lib
    if _lib is None:
        import importlib.util
        spec = importlib.util.spec_from_file_location("_haplo_build_oracle", os.path.join(HERE, "build_oracle.py"))
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        path = mod.build()
        lib = C.CDLL(path)
        P, I64, I32, Dd = C.c_void_p, C.c_int64, C.c_int32, C.c_double
        sig = {
            "orc_bed_code": (I32, [P, I64, I64, I64]),
            "orc_census": (None, [P, I64, I64, I64, P]),
            "orc_count_double_missing": (None, [P, I64, I64, I64, P]),
            "orc_pair_terms": (None, [I32, I32, P, P]),
            "orc_loglik": (Dd, [P, I64, I64, I64, I32, P, P, I32, I32]),
            "orc_em_accum": (None, [P, I64, I64, I64, I32, P, P, P, P, I32]),
            "orc_accum_q": (None, [P, I64, I64, I64, I32, P, P, P, P, I32]),
            "orc_accum_p": (None, [P, I64, I64, I64, I32, P, P, P, P, I32]),
            "orc_project_q": (None, [P, I32, I64, Dd]),
            "orc_project_p": (None, [P, I32, I64, Dd]),
            "orc_qp_dense": (I32, [I32, P, P, P, P, I32, P]),
            "orc_qp_q": (I32, [I32, I64, P, P, P, P, I32]),
            "orc_qp_p": (I32, [I32, I64, P, P, P, Dd, P, I32]),
            "orc_qp_p_eq": (I32, [I32, I64, P, P, P, P, I32]),
            "orc_em_step": (None, [P, I64, I64, I64, I32, P, P, P, P, P, I32]),
            "orc_update_q": (I32, [P, I64, I64, I64, I32, P, P, P, P, P, I32]),
            "orc_update_p": (I32, [P, I64, I64, I64, I32, P, P, Dd, P, P, P, I32]),
            "orc_zal": (None, [I64, P, P, P, P, P, I32, I32, P]),
            "orc_fit": (I32, [P, I64, I64, I64, I64, I32, I32, P, I32, Dd, I32, Dd, I32, P, P, P]),
            "orc_fit_ex": (I32, [P, I64, I64, I64, I64, I32, I32, P, I32, Dd, I32, Dd, I32, P, P, P,
                                 I32, I32, I32, I32, I32]),
            "orc_qn": (None, [I64, P, P, P, P, P, I32, I32, I32, P]),
            "orc_synth": (None, [C.c_uint64, I64, I64, I32, P, P, Dd, P, I32]),
        }
        for name, (res, args) in sig.items():
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        _lib = lib
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _F(a, shape=None):
    a = np.asfortranarray(a, dtype=np.float64)
    if shape is not None and a.shape != shape:
        raise ValueError("shape %s != %s" % (a.shape, shape))
    return a


def nthreads():
    return os.cpu_count() or 1


class Bed:
    """BED data matrix (n_snp, bps) uint8 plus its dimensions."""

    def __init__(self, data, I, J, n_snp=None):
        self.data = np.ascontiguousarray(data, dtype=np.uint8)
        self.bps = self.data.shape[1]
        self.I, self.J = I, J
        self.n_snp = self.data.shape[0] if n_snp is None else n_snp

    @property
    def ptr(self):
        return _p(self.data)


def census(b):
    c = np.zeros(16, dtype=np.uint64)
    _load().orc_census(b.ptr, b.bps, b.I, b.J, _p(c))
    return c


def double_missing(b):
    d = np.zeros(b.I, dtype=np.int64)
    _load().orc_count_double_missing(b.ptr, b.bps, b.I, b.n_snp, _p(d))
    return d


def pair_terms(g1, g2, qp):
    qp = np.ascontiguousarray(qp, dtype=np.float64)
    out = np.zeros(6)
    _load().orc_pair_terms(g1, g2, _p(qp), _p(out))
    return out


def loglik(b, K, q, p, formula=2, threads=None):
    q, p = _F(q, (K, b.I)), _F(p, (K, 4 * b.J))
    return _load().orc_loglik(b.ptr, b.bps, b.I, b.J, K, _p(q), _p(p), formula, threads or nthreads())


def em_accum(b, K, q, p, threads=None):
    q, p = _F(q, (K, b.I)), _F(p, (K, 4 * b.J))
    qn = np.empty_like(q, order="F")
    pn = np.empty_like(p, order="F")
    _load().orc_em_accum(b.ptr, b.bps, b.I, b.J, K, _p(q), _p(p), _p(qn), _p(pn), threads or nthreads())
    return qn, pn


def accum_q(b, K, q, p, threads=None):
    q, p = _F(q, (K, b.I)), _F(p, (K, 4 * b.J))
    XtX = np.empty((K, K, b.I), order="F")
    Xtz = np.empty((K, b.I), order="F")
    _load().orc_accum_q(b.ptr, b.bps, b.I, b.J, K, _p(q), _p(p), _p(XtX), _p(Xtz), threads or nthreads())
    return XtX, Xtz


def accum_p(b, K, q, p, threads=None):
    q, p = _F(q, (K, b.I)), _F(p, (K, 4 * b.J))
    XtX = np.empty((K, K, 4 * b.J), order="F")
    Xtz = np.empty((K, 4 * b.J), order="F")
    _load().orc_accum_p(b.ptr, b.bps, b.I, b.J, K, _p(q), _p(p), _p(XtX), _p(Xtz), threads or nthreads())
    return XtX, Xtz


def project_q(q, eps=1e-5):
    q = np.array(q, dtype=np.float64, order="F", copy=True)
    _load().orc_project_q(_p(q), q.shape[0], q.shape[1], eps)
    return q


def project_p(p, eps=1e-5):
    p = np.array(p, dtype=np.float64, order="F", copy=True)
    _load().orc_project_p(_p(p), p.shape[0], p.shape[1] // 4, eps)
    return p


def qp_dense(H, z, lo, hi, eq):
    """eq: False/0 no equality, True/1 sum(d) = 0, G >= 2 the G groups
    sum_{a % G == k} d_a = 0."""
    n = len(z)
    H = _F(H, (n, n))
    z, lo, hi = (np.ascontiguousarray(v, dtype=np.float64) for v in (z, lo, hi))
    d = np.zeros(n)
    it = _load().orc_qp_dense(n, _p(H), _p(z), _p(lo), _p(hi), int(eq), _p(d))
    return d, it


def qp_q(XtX, Xtz, q, threads=None):
    K, n = q.shape
    XtX, Xtz, q = _F(XtX, (K, K, n)), _F(Xtz, (K, n)), _F(q, (K, n))
    d = np.empty((K, n), order="F")
    f = _load().orc_qp_q(K, n, _p(XtX), _p(Xtz), _p(q), _p(d), threads or nthreads())
    return d, f


def qp_p(XtX, Xtz, p, rho=1e7, threads=None):
    K, m = p.shape
    XtX, Xtz, p = _F(XtX, (K, K, m)), _F(Xtz, (K, m)), _F(p, (K, m))
    d = np.empty((K, m), order="F")
    f = _load().orc_qp_p(K, m // 4, _p(XtX), _p(Xtz), _p(p), rho, _p(d), threads or nthreads())
    return d, f


def qp_p_eq(XtX, Xtz, p, threads=None):
    """The P QP in equality form (penalty = false): sum_h d[k, h] = 0 for every k."""
    K, m = p.shape
    XtX, Xtz, p = _F(XtX, (K, K, m)), _F(Xtz, (K, m)), _F(p, (K, m))
    d = np.empty((K, m), order="F")
    f = _load().orc_qp_p_eq(K, m // 4, _p(XtX), _p(Xtz), _p(p), _p(d), threads or nthreads())
    return d, f


def em_step(b, K, q, p, dm=None, threads=None):
    q, p = _F(q, (K, b.I)), _F(p, (K, 4 * b.J))
    dm = double_missing(b) if dm is None else np.ascontiguousarray(dm, dtype=np.int64)
    qn = np.empty_like(q, order="F")
    pn = np.empty_like(p, order="F")
    _load().orc_em_step(b.ptr, b.bps, b.I, b.J, K, _p(dm), _p(q), _p(p), _p(qn), _p(pn), threads or nthreads())
    return qn, pn


def update_q(b, K, q, p, threads=None):
    q, p = _F(q, (K, b.I)), _F(p, (K, 4 * b.J))
    qn = np.empty_like(q, order="F")
    f = _load().orc_update_q(b.ptr, b.bps, b.I, b.J, K, _p(q), _p(p), _p(qn), None, None, threads or nthreads())
    return qn, f


def update_p(b, K, q, p, rho=1e7, threads=None):
    q, p = _F(q, (K, b.I)), _F(p, (K, 4 * b.J))
    pn = np.empty_like(p, order="F")
    f = _load().orc_update_p(b.ptr, b.bps, b.I, b.J, K, _p(q), _p(p), rho, _p(pn), None, None,
                             threads or nthreads())
    return pn, f


def zal(x, x_next, x_next2, U, V, it):
    n = x.size
    x, x_next, x_next2 = (np.ascontiguousarray(np.ravel(a, order="F"), dtype=np.float64) for a in (x, x_next, x_next2))
    U = np.array(U, dtype=np.float64, order="F", copy=True)
    V = np.array(V, dtype=np.float64, order="F", copy=True)
    xt = np.empty(n)
    _load().orc_zal(n, _p(x), _p(x_next), _p(x_next2), _p(U), _p(V), U.shape[1], it, _p(xt))
    return xt, U, V


def qn(x, x_next, x_next2, U, V, it, mode="ZAL"):
    """The quasi-Newton point of admixture_qn!: mode "ZAL" or "LBQN"."""
    n = x.size
    x, x_next, x_next2 = (np.ascontiguousarray(np.ravel(a, order="F"), dtype=np.float64) for a in (x, x_next, x_next2))
    U = np.array(U, dtype=np.float64, order="F", copy=True)
    V = np.array(V, dtype=np.float64, order="F", copy=True)
    xt = np.empty(n)
    _load().orc_qn(n, _p(x), _p(x_next), _p(x_next2), _p(U), _p(V), U.shape[1], it, {"ZAL": 0, "LBQN": 1}[mode],
                   _p(xt))
    return xt, U, V


def fit(b, K, q, p, n_iter=1000, rtol=1e-7, em_iters=5, Qs=3, rho=1e7, threads=None, fix_q=False, fix_p=False,
        guarantee_increase=False, penalty=None, mode="ZAL"):
    """init_em! + admixture_qn! on the CPU; returns (q, p, ll, iters, trace).
    penalty None is the reference default (P penalty form, Q equality form);
    True uses the penalty form for both, False the equality form for both.
    mode: "ZAL" (default) or "LBQN", the quasi-Newton step of admixture_qn!."""
    q, p = _F(q, (K, b.I)), _F(p, (K, 4 * b.J))
    x = np.asfortranarray(np.hstack([q, p]))
    ll = C.c_double()
    iters = C.c_int32()
    trace = np.full(n_iter, np.nan)
    pen = -1 if penalty is None else int(bool(penalty))
    r = _load().orc_fit_ex(b.ptr, b.bps, b.n_snp, b.I, b.J, K, Qs, _p(x), n_iter, rtol, em_iters, rho,
                           threads or nthreads(), C.byref(ll), C.byref(iters), _p(trace), int(fix_q), int(fix_p),
                           int(guarantee_increase), pen, {"ZAL": 0, "LBQN": 1}[mode])
    return (np.asfortranarray(x[:, :b.I]), np.asfortranarray(x[:, b.I:]), ll.value, iters.value,
            trace[:iters.value])


def synth(seed, I, J, cumQ, cumP, miss, threads=None):
    K = cumQ.shape[0]
    cumQ, cumP = _F(cumQ, (K, I)), _F(cumP, (K, 4 * J))
    bps = (I + 3) // 4
    out = np.zeros((2 * J, bps), dtype=np.uint8)
    _load().orc_synth(seed, I, J, K, _p(cumQ), _p(cumP), miss, _p(out), threads or nthreads())
    return out
