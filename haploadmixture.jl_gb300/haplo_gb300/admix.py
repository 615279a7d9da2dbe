"""Host-side mirror of HaploADMIXTURE's Julia interface over the C ABI.

Array conventions follow the reference's Julia arrays: q is K x I, p is K x 4J,
XtX_q is K x K x I, XtX_p is K x K x 4J, all column-major (numpy arrays are
returned in Fortran order with those shapes).

  * GB300Admix           -- the device handle; plays the role of CuAdmixData
                            (src/cuda/structs.jl:1-32) plus the on-device
                            QP/QN state, and carries the runner methods of
                            src/cuda/runners.jl.
  * AdmixData2-style init -- random_init() restates src/structs.jl:155-200.
  * run_admixture         -- src/driver.jl:38-79 / 133-201 (no SKFR branch).
"""
import ctypes as C
import time

import numpy as np

from . import _lib
from ._lib import check, ptr
from . import bed as bedio


def _fortran(a, shape):
    a = np.asarray(a, dtype=np.float64)
    if a.shape != shape:
        raise ValueError("expected shape %s, got %s" % (shape, a.shape))
    return np.asfortranarray(a)


class GB300Admix:
    """One fit on one GPU.

    bed: uint8 array of the PLINK .bed data matrix (bytes after the magic),
         SNP-major, shape (n_snp, bytes_per_snp) or flat; or, with
         bed_on_device=True, an integer device address.
    """

    def __init__(self, bed, I, J, K, *, bytes_per_snp=None, n_snp=None, precision="fp64", Q=3, device=0,
                 rho=1e7, pseudocount=1e-5, verbose=False, bed_on_device=False, path="auto"):
        lib = _lib.load()
        self.I, self.J, self.K = int(I), int(J), int(K)
        opts = _lib.HxOpts()
        lib.hx_opts_default(C.byref(opts))
        opts.precision = {"fp64": _lib.HX_PREC_FP64, "mixed": _lib.HX_PREC_MIXED}[precision]
        opts.device = device
        opts.Qsec = Q
        opts.verbose = 1 if verbose else 0
        opts.rho = rho
        opts.pseudocount = pseudocount
        opts.path = {"auto": _lib.HX_PATH_AUTO, "cuda_cores": _lib.HX_PATH_CUDA_CORES}[path]
        self.precision = precision
        self.Q = Q
        h = C.c_void_p()
        if bed_on_device:
            if bytes_per_snp is None or n_snp is None:
                raise ValueError("bytes_per_snp and n_snp are required with bed_on_device")
            st = lib.hx_create_device(C.c_void_p(int(bed)), bytes_per_snp, n_snp, self.I, self.J, self.K,
                                      C.byref(opts), C.byref(h))
        else:
            b = np.ascontiguousarray(bed, dtype=np.uint8)
            if bytes_per_snp is None:
                bytes_per_snp = b.shape[1] if b.ndim == 2 else (self.I + 3) // 4
            if n_snp is None:
                n_snp = b.size // bytes_per_snp
            if b.size < bytes_per_snp * n_snp:
                raise ValueError("BED buffer smaller than bytes_per_snp * n_snp")
            st = lib.hx_create(ptr(b), bytes_per_snp, n_snp, self.I, self.J, self.K, C.byref(opts), C.byref(h))
        self._h = h
        if st != _lib.HX_OK:
            msg = lib.hx_last_error(h).decode() if h.value else ""
            if h.value:
                lib.hx_destroy(h)
            self._h = None
            raise _lib.HxError(st, msg)
        self.bytes_per_snp, self.n_snp = bytes_per_snp, n_snp

    @classmethod
    def shared(cls, parent, K, *, precision=None, Q=3, rho=1e7, pseudocount=1e-5, path="auto"):
        """A context for K ancestries on the parent's decoded genotypes
        (hx_create_shared); it keeps the parent alive."""
        lib = _lib.load()
        self = cls.__new__(cls)
        self.I, self.J, self.K = parent.I, parent.J, int(K)
        self.precision = precision or parent.precision
        self.Q = Q
        opts = _lib.HxOpts()
        lib.hx_opts_default(C.byref(opts))
        opts.precision = {"fp64": _lib.HX_PREC_FP64, "mixed": _lib.HX_PREC_MIXED}[self.precision]
        opts.Qsec = Q
        opts.rho = rho
        opts.pseudocount = pseudocount
        opts.path = {"auto": _lib.HX_PATH_AUTO, "cuda_cores": _lib.HX_PATH_CUDA_CORES}[path]
        h = C.c_void_p()
        st = lib.hx_create_shared(parent._h, self.K, C.byref(opts), C.byref(h))
        self._h = h
        self._parent = parent
        if st != _lib.HX_OK:
            msg = lib.hx_last_error(h).decode() if h.value else ""
            if h.value:
                lib.hx_destroy(h)
            self._h = None
            raise _lib.HxError(st, msg)
        self.bytes_per_snp, self.n_snp = parent.bytes_per_snp, parent.n_snp
        return self

    # -- lifetime
    def close(self):
        if getattr(self, "_h", None):
            _lib.load().hx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _ck(self, st):
        check(st, self._h)

    @property
    def lib(self):
        return _lib.load()

    # -- state
    def set_qp(self, q=None, p=None):
        qa = None if q is None else _fortran(q, (self.K, self.I))
        pa = None if p is None else _fortran(p, (self.K, 4 * self.J))
        self._ck(self.lib.hx_set_qp(self._h, ptr(qa), ptr(pa)))

    def set_qp_device(self, q_addr, p_addr):
        self._ck(self.lib.hx_set_qp_device(self._h, C.c_void_p(q_addr), C.c_void_p(p_addr)))

    def get_qp(self, which="x"):
        w = {"x": 0, "x_next": 1, "x_next2": 2, "x_tmp": 3}[which]
        q = np.empty((self.K, self.I), order="F")
        p = np.empty((self.K, 4 * self.J), order="F")
        self._ck(self.lib.hx_get_qp(self._h, w, ptr(q), ptr(p)))
        return q, p

    @property
    def q(self):
        return self.get_qp()[0]

    @property
    def p(self):
        return self.get_qp()[1]

    @property
    def ll_new(self):
        v = C.c_double()
        self._ck(self.lib.hx_get_ll(self._h, C.byref(v)))
        return v.value

    def census(self):
        c = np.zeros(16, dtype=np.uint64)
        self._ck(self.lib.hx_census(self._h, ptr(c)))
        return c

    def double_missing(self):
        d = np.zeros(self.I, dtype=np.int64)
        self._ck(self.lib.hx_double_missing(self._h, ptr(d)))
        return d

    # -- launch accounting
    KINDS = ("accum_q", "accum_p", "loglik", "qp_q", "qp_p", "qn", "other", "em_q", "em_p")

    def set_loop_opts(self, fix_q=False, fix_p=False, guarantee_increase=False, penalty=None, mode="ZAL"):
        """admixture_qn!/init_em! keyword options (src/algorithms_outer.jl:1-3, 38-41);
        penalty None is the reference default (P penalty form, Q equality form),
        True the penalty form for both steps, False the equality form for both;
        mode "ZAL" (default) or "LBQN" selects admixture_qn!'s quasi-Newton step."""
        o = _lib.HxLoopOpts()
        self._ck(self.lib.hx_loop_opts_default(C.byref(o)))
        o.fix_q, o.fix_p, o.guarantee_increase = int(fix_q), int(fix_p), int(guarantee_increase)
        o.penalty = -1 if penalty is None else int(bool(penalty))
        o.mode = {"ZAL": 0, "LBQN": 1}[mode]
        self._ck(self.lib.hx_set_loop_opts(self._h, C.byref(o)))

    def set_profiling(self, on=True):
        self._ck(self.lib.hx_set_profiling(self._h, 1 if on else 0))

    def reset_stats(self):
        self._ck(self.lib.hx_reset_stats(self._h))

    def kernel_stats(self):
        out = {}
        for k, name in enumerate(self.KINDS):
            n = C.c_int64()
            ms = C.c_double()
            self._ck(self.lib.hx_kernel_stats(self._h, k, C.byref(n), C.byref(ms)))
            out[name] = (n.value, ms.value)
        return out

    # -- runners of src/cuda/runners.jl
    def loglikelihood(self, q=None, p=None):
        v = C.c_double()
        if q is None and p is None:
            self._ck(self.lib.hx_loglikelihood(self._h, None, None, C.byref(v)))
        else:
            qa, pa = _fortran(q, (self.K, self.I)), _fortran(p, (self.K, 4 * self.J))
            self._ck(self.lib.hx_loglikelihood(self._h, ptr(qa), ptr(pa), C.byref(v)))
        return v.value

    def em_accum(self, q, p):
        qa, pa = _fortran(q, (self.K, self.I)), _fortran(p, (self.K, 4 * self.J))
        qn = np.empty_like(qa, order="F")
        pn = np.empty_like(pa, order="F")
        self._ck(self.lib.hx_em_accum(self._h, ptr(qa), ptr(pa), ptr(qn), ptr(pn)))
        return qn, pn

    def em_p_accum(self, q, p):
        """em_p! (src/cuda/runners.jl:51-55): the P numerators p .* Xtz_p only."""
        qa, pa = _fortran(q, (self.K, self.I)), _fortran(p, (self.K, 4 * self.J))
        pn = np.empty_like(pa, order="F")
        self._ck(self.lib.hx_em_p_accum(self._h, ptr(qa), ptr(pa), ptr(pn)))
        return pn

    def set_wait_budget(self, cycles=0):
        """Bound (SM clock cycles) on each pipeline wait of the tensor-core
        passes; 0 restores the default.  A wait that runs out raises HxError
        with status HX_ETIMEOUT and leaves the handle usable."""
        self._ck(self.lib.hx_set_wait_budget(self._h, int(cycles)))

    def autotune(self):
        """hx_autotune: picks the fastest grid splits of the mixed method's
        pass kernels at the current Q/P; returns the chunk counts (Q pass, P
        pass, log-likelihood)."""
        ch = np.zeros(3, dtype=np.int32)
        self._ck(self.lib.hx_autotune(self._h, ptr(ch)))
        return tuple(int(x) for x in ch)

    def update_q_accum(self, q, p):
        qa, pa = _fortran(q, (self.K, self.I)), _fortran(p, (self.K, 4 * self.J))
        XtX = np.empty((self.K, self.K, self.I), order="F")
        Xtz = np.empty((self.K, self.I), order="F")
        self._ck(self.lib.hx_update_q_accum(self._h, ptr(qa), ptr(pa), ptr(XtX), ptr(Xtz)))
        return XtX, Xtz

    def update_p_accum(self, q, p):
        qa, pa = _fortran(q, (self.K, self.I)), _fortran(p, (self.K, 4 * self.J))
        XtX = np.empty((self.K, self.K, 4 * self.J), order="F")
        Xtz = np.empty((self.K, 4 * self.J), order="F")
        self._ck(self.lib.hx_update_p_accum(self._h, ptr(qa), ptr(pa), ptr(XtX), ptr(Xtz)))
        return XtX, Xtz

    # -- batched QP / projection / QN on host arrays
    def qp_q(self, XtX, Xtz, q):
        n = q.shape[1]
        XtX = _fortran(XtX, (self.K, self.K, n))
        Xtz = _fortran(Xtz, (self.K, n))
        q = _fortran(q, (self.K, n))
        d = np.empty((self.K, n), order="F")
        self._ck(self.lib.hx_qp_q(self._h, n, ptr(XtX), ptr(Xtz), ptr(q), ptr(d)))
        return d

    def qp_p(self, XtX, Xtz, p):
        n = p.shape[1] // 4
        XtX = _fortran(XtX, (self.K, self.K, 4 * n))
        Xtz = _fortran(Xtz, (self.K, 4 * n))
        p = _fortran(p, (self.K, 4 * n))
        d = np.empty((self.K, 4 * n), order="F")
        self._ck(self.lib.hx_qp_p(self._h, n, ptr(XtX), ptr(Xtz), ptr(p), ptr(d)))
        return d

    def project_q(self, q):
        q = np.array(_fortran(q, (self.K, q.shape[1])), order="F", copy=True)
        self._ck(self.lib.hx_project_q(self._h, q.shape[1], ptr(q)))
        return q

    def project_p(self, p):
        p = np.array(_fortran(p, (self.K, p.shape[1])), order="F", copy=True)
        self._ck(self.lib.hx_project_p(self._h, p.shape[1] // 4, ptr(p)))
        return p

    def zal(self, x, x_next, x_next2, U, V, it):
        n = self.K * (self.I + 4 * self.J)
        x, x_next, x_next2 = (np.ascontiguousarray(np.ravel(a, order="F"), dtype=np.float64)
                              for a in (x, x_next, x_next2))
        assert x.size == n
        U = np.asfortranarray(U, dtype=np.float64)
        V = np.asfortranarray(V, dtype=np.float64)
        xt = np.empty(n)
        self._ck(self.lib.hx_zal(self._h, ptr(x), ptr(x_next), ptr(x_next2), ptr(U), ptr(V), it, ptr(xt)))
        return xt, U, V

    # -- device-resident algorithm (algorithms_inner.jl / algorithms_outer.jl)
    def em_step(self):
        self._ck(self.lib.hx_em_step(self._h))

    def init_em(self, iters=5):
        self._ck(self.lib.hx_init_em(self._h, iters))

    def update_q(self, update2=False):
        self._ck(self.lib.hx_update_q(self._h, 1 if update2 else 0))

    def update_p(self, update2=False):
        self._ck(self.lib.hx_update_p(self._h, 1 if update2 else 0))

    def qn_iteration(self):
        info = _lib.HxIterInfo()
        self._ck(self.lib.hx_qn_iteration(self._h, C.byref(info)))
        return {f: getattr(info, f) for f, _ in info._fields_}

    def admixture_qn(self, n_iter=1000, rtol=1e-7, iter_count_offset=0):
        info = _lib.HxFitInfo()
        self._ck(self.lib.hx_admixture_qn(self._h, n_iter, rtol, iter_count_offset, C.byref(info)))
        return {f: getattr(info, f) for f, _ in info._fields_ if f != "pad_"}

    def fit(self, n_iter=1000, rtol=1e-7, em_iters=5):
        info = _lib.HxFitInfo()
        self._ck(self.lib.hx_fit(self._h, n_iter, rtol, em_iters, C.byref(info)))
        return {f: getattr(info, f) for f, _ in info._fields_ if f != "pad_"}


def random_init(I, J, K, rng):
    """AdmixData2's random start (src/structs.jl:155-200): x = rand(K, I+4J),
    q normalised per column, p normalised per (k, block) quartet."""
    x = rng.random((K, I + 4 * J))
    q = x[:, :I]
    q = q / q.sum(axis=0, keepdims=True)
    p = x[:, I:].reshape(K, J, 4)
    p = (p / p.sum(axis=2, keepdims=True)).reshape(K, 4 * J)
    return np.asfortranarray(q), np.asfortranarray(p)


class AdmixResult:
    def __init__(self, d, info):
        self.q, self.p = d.get_qp()
        self.ll_new = info["ll"]
        self.info = info
        self.I, self.J, self.K = d.I, d.J, d.K


def run_admixture(filename, I, J, K, *, rng=None, sparsity=None, prefix=None, skfr_tries=1, skfr_max_inner_iter=50,
                  skfr_seed=0,
                  admix_n_iter=1000, admix_rtol=1e-7, admix_n_em_iters=5, precision="fp64", Q=3, init_q=None,
                  init_p=None, fix_q=False, fix_p=False, device=0, verbose=False, return_handle=False):
    """src/driver.jl:38-79 with the _admixture_base sequence (133-201) on the
    GPU: load the .bed (first I individuals, first 2J SNPs), random start,
    init_em! unless both init_q and init_p are given, then admixture_qn!
    (mode :ZAL).  Returns (d, clusters, aims) like the reference.

    With `sparsity` (the reference's SKFR branch, :60-73 and 84-105), the
    AIMs are selected first (haplo_gb300.skfr: sparse k-means with feature
    ranking on blocks of 2 SNPs, `skfr_max_inner_iter` iterations, start from
    `skfr_seed`, the best of `skfr_tries` starts), the file is filtered to them as
    <prefix>_<K>_<2*sparsity>aims.bed, and the fit reads that file; clusters
    and aims are returned.  Without it they are None.

    fix_q / fix_p hold that factor during admixture_qn! (not during
    init_em!, as _admixture_base passes them, src/driver.jl:181-197)."""
    if not str(filename).endswith(".bed"):
        raise ValueError("filename should end with .bed")
    rng = np.random.default_rng(rng) if not isinstance(rng, np.random.Generator) else rng
    clusters = aims = None
    if sparsity is not None:
        from . import skfr
        data, n_ind, n_snp = bedio.read_bed(filename)
        clusters, aims, _ = skfr.select_aims(data, n_ind, K, sparsity, seed=skfr_seed,
                                             max_iter=skfr_max_inner_iter, device=device, tries=skfr_tries)
        filename = skfr.write_filtered(prefix or str(filename)[:-4], data, n_ind, K, aims)
    data, n_ind, n_snp = bedio.read_bed(filename)
    if I > n_ind or 2 * J > n_snp:
        raise ValueError("file has %d individuals and %d SNPs; asked for I=%d, 2J=%d" % (n_ind, n_snp, I, 2 * J))
    d = GB300Admix(data, I, J, K, bytes_per_snp=data.shape[1], n_snp=n_snp, precision=precision, Q=Q,
                   device=device, verbose=verbose)
    q0, p0 = random_init(I, J, K, rng)
    d.set_qp(q0, p0)
    t0 = time.time()
    if init_q is None or init_p is None:
        d.init_em(admix_n_em_iters)
    if init_q is not None or init_p is not None:
        d.set_qp(init_q, init_p)
    if fix_q or fix_p:
        d.set_loop_opts(fix_q=fix_q, fix_p=fix_p)
    info = d.admixture_qn(admix_n_iter, admix_rtol)
    info["seconds"] = time.time() - t0
    res = AdmixResult(d, info)
    if return_handle:
        return res, d
    d.close()
    return res, clusters, aims
