"""CPU oracle for the EnKF-C analysis hot path -- TEST INFRASTRUCTURE ONLY.

This package is the checker the GPU library is compared against (and the CPU
baseline timed beside it).  Only tests, the smoke check and the CPU-baseline
leg of the benchmark import it; the product never does.

  liboracle.so       C restatement of the reference loops (enkf_oracle.c),
                     built by oracle/Makefile on whichever machine runs it.
  _ref/libenkf_ref.so the reference's own calc/calcs.c + common/kdtree.c,
                     compiled unmodified by oracle/ref/Makefile where the
                     reference sources exist; used to pin the restatement.
  _ref/libenkf_ref_update.so  the reference's update/update.c (field update,
                     background update) and common/dasystem.c (hybrid
                     ensemble), compiled unmodified the same way.

The reference tree is ENKFG_REFERENCE_DIR when set, else the default of
oracle/ref/Makefile.
"""
from __future__ import annotations

import ctypes as C
import glob
import os
import subprocess
import threading
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
REFLIB = os.path.join(HERE, "_ref", "libenkf_ref.so")
MAXLOCRAD = 8

_lock = threading.Lock()
_lib = None
_ref = None


def blas_path() -> str:
    """The OpenBLAS shipped inside the scipy (or numpy) wheel."""
    import scipy
    cands = []
    for pkg in (scipy,):
        d = os.path.join(os.path.dirname(pkg.__file__), "..", "scipy.libs")
        cands += sorted(glob.glob(os.path.join(d, "libscipy_openblas*.so*")))
    try:
        import numpy
        d = os.path.join(os.path.dirname(numpy.__file__), "..", "numpy.libs")
        cands += sorted(glob.glob(os.path.join(d, "libscipy_openblas*.so*")))
    except Exception:
        pass
    if not cands:
        raise RuntimeError("no OpenBLAS found inside the scipy/numpy wheels")
    return os.path.realpath(cands[0])


def refdir() -> str:
    """The reference tree: ENKFG_REFERENCE_DIR, else the reference build
    recipe's default (oracle/ref/Makefile)."""
    d = os.environ.get("ENKFG_REFERENCE_DIR")
    if d:
        return d
    r = subprocess.run(["make", "-s", "--no-print-directory", "print-refdir"], cwd=os.path.join(HERE, "ref"),
                       capture_output=True, text=True)
    return r.stdout.strip()


def build(force: bool = False) -> str:
    """Compile liboracle.so in place (and _ref when the reference is present)."""
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < max(
            os.path.getmtime(os.path.join(HERE, f)) for f in ("enkf_oracle.c", "or_blas.c", "enkf_oracle.h")):
        subprocess.run(["make", "-s", "-B" if force else "all"], cwd=HERE, check=True)
    rd = refdir()
    if rd and os.path.isdir(rd):
        subprocess.run(["make", "-s", "REFDIR=" + rd], cwd=os.path.join(HERE, "ref"), check=True)
    return LIB


def _p(a, t):
    return a.ctypes.data_as(C.POINTER(t)) if a is not None else None


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = C.CDLL(LIB)
            rc = L.or_blas_load(blas_path().encode())
            if rc != 0:
                raise RuntimeError(f"or_blas_load failed ({rc})")
            L.or_obs_create.restype = C.c_void_p
            L.or_findlocal.restype = C.c_int
            L.or_taper_gc.restype = C.c_double
            L.or_taper_gc.argtypes = [C.c_double]
            L.or_calclcoeff.restype = C.c_double
            L.or_calctransforms.restype = C.c_int
            _lib = L
    return _lib


def reflib():
    """The reference's own compiled numerics + kd-tree, or None if not built."""
    global _ref
    with _lock:
        if _ref is None and os.path.exists(REFLIB):
            L = C.CDLL(REFLIB)
            if L.or_blas_load(blas_path().encode()) != 0:
                return None
            L.ref_kd_build.restype = C.c_void_p
            L.ref_kd_build.argtypes = [C.c_int, C.c_int, C.c_void_p]
            L.ref_kd_free.argtypes = [C.c_void_p]
            L.ref_kd_range.argtypes = [C.c_void_p, C.c_void_p, C.c_double, C.c_int, C.c_void_p, C.c_void_p, C.c_int]
            _ref = L
    return _ref


class CalcParams(C.Structure):
    _fields_ = [("mode", C.c_int), ("scheme", C.c_int), ("nmem", C.c_int), ("nmem_dynamic", C.c_int),
                ("alpha", C.c_double), ("stride", C.c_int), ("mni", C.c_int), ("mnj", C.c_int),
                ("x", C.POINTER(C.c_double)), ("y", C.POINTER(C.c_double)),
                ("x2d", C.POINTER(C.c_double)), ("y2d", C.POINTER(C.c_double)), ("ii0", C.c_int),
                ("ii1", C.c_int)]


class UpdateParams(C.Structure):
    _fields_ = [("mode", C.c_int), ("nmem", C.c_int), ("nmem_dynamic", C.c_int), ("stride", C.c_int),
                ("periodic_i", C.c_int), ("mni", C.c_int), ("mnj", C.c_int), ("ni", C.c_int), ("nj", C.c_int),
                ("j1", C.c_int), ("j2", C.c_int), ("level", C.c_int), ("surfk", C.c_int),
                ("issurfacevar", C.c_int), ("inflation0", C.c_float), ("inf_ratio", C.c_double),
                ("output_increment", C.c_int), ("applylog", C.c_int)]


def locrad_table(ntypes: int, locrad, locweight=None):
    """[ntypes][MAXLOCRAD] radius / weight tables.  `locrad` is a scalar (one
    radius for every type) or a per-type list of radius lists."""
    nl = np.zeros(ntypes, np.int32)
    lr = np.zeros((ntypes, MAXLOCRAD), np.float64)
    lw = np.zeros((ntypes, MAXLOCRAD), np.float64)
    for t in range(ntypes):
        r = np.atleast_1d(np.asarray(locrad if np.isscalar(locrad) else locrad[t], np.float64))
        wt = np.ones_like(r) if locweight is None else np.atleast_1d(np.asarray(locweight[t], np.float64))
        nl[t] = r.size
        lr[t, :r.size] = r
        lw[t, :r.size] = wt
    return nl, lr, lw


class ObsSet:
    """Observation set with per-type kd-trees (or_obs_create)."""

    def __init__(self, lon, lat, otype, status, ntypes, nlocrad, locrad, locweight, nlobsmax=None,
                 geographic=False):
        L = lib()
        self.lon = np.ascontiguousarray(lon, np.float32)
        self.lat = np.ascontiguousarray(lat, np.float32)
        self.otype = np.ascontiguousarray(otype, np.int16)
        self.status = np.ascontiguousarray(status, np.int16)
        self.ntypes = int(ntypes)
        self.nlocrad = np.ascontiguousarray(nlocrad, np.int32)
        self.locrad = np.ascontiguousarray(locrad, np.float64)
        self.locweight = np.ascontiguousarray(locweight, np.float64)
        nlm = None if nlobsmax is None else np.ascontiguousarray(nlobsmax, np.int32)
        self.h = L.or_obs_create(C.c_int(self.lon.size), _p(self.lon, C.c_float), _p(self.lat, C.c_float),
                                 _p(self.otype, C.c_short), _p(self.status, C.c_short), C.c_int(self.ntypes),
                                 _p(self.nlocrad, C.c_int), _p(self.locrad, C.c_double),
                                 _p(self.locweight, C.c_double), _p(nlm, C.c_int), C.c_int(int(geographic)))
        self.nobs = self.lon.size
        self.geographic = bool(geographic)
        self.nlobsmax = nlm

    def __del__(self):
        try:
            lib().or_obs_destroy(C.c_void_p(self.h))
        except Exception:
            pass

    def findlocal(self, x: float, y: float):
        cap = max(self.nobs, 1)
        ids = np.empty(cap, np.int32)
        lc = np.empty(cap, np.float64)
        n = lib().or_findlocal(C.c_void_p(self.h), C.c_double(x), C.c_double(y), _p(ids, C.c_int),
                               _p(lc, C.c_double), C.c_int(cap))
        assert n >= 0
        return ids[:n].copy(), lc[:n].copy()


def taper_gc(x: float) -> float:
    return lib().or_taper_gc(float(x))


def calc_wT(mode, scheme, m, mout, s, S):
    """Per-point numerics; S is [m][p].  Returns (w, T [m][m], G [p][m])."""
    S = np.ascontiguousarray(S, np.float64).copy()
    s = np.ascontiguousarray(s, np.float64)
    p = S.shape[1]
    w = np.zeros(m)
    T = np.zeros((m, m))
    G = np.zeros((p, m))
    rc = lib().or_calc_wT(C.c_int(mode), C.c_int(scheme), C.c_int(m), C.c_int(mout), C.c_int(p),
                          _p(s, C.c_double), _p(S, C.c_double), _p(w, C.c_double), _p(T, C.c_double),
                          _p(G, C.c_double))
    if rc != 0:
        raise RuntimeError(f"LAPACK info {rc}")
    return w, T, G


def ref_calc_wT(mode, scheme, m, mout, s, S):
    """The same through the reference's own calcs.c (needs oracle/_ref)."""
    L = reflib()
    if L is None:
        raise RuntimeError("reference library not built")
    S = np.ascontiguousarray(S, np.float64).copy()
    s = np.ascontiguousarray(s, np.float64).copy()
    p = S.shape[1]
    w = np.zeros(m)
    T = np.zeros((m, m))
    G = np.zeros((p, m))
    L.ref_calc_wT(C.c_int(mode), C.c_int(scheme), C.c_int(m), C.c_int(mout), C.c_int(p), _p(s, C.c_double),
                  _p(S, C.c_double), _p(w, C.c_double), _p(T, C.c_double), _p(G, C.c_double))
    return w, T, G


class RefKdTree:
    """A reference kd-tree (common/kdtree.c) built as obs_createkdtrees does."""

    def __init__(self, coords: np.ndarray):
        L = reflib()
        self.coords = np.ascontiguousarray(coords, np.float64)
        self.ndim = self.coords.shape[1]
        self.n = self.coords.shape[0]
        self.h = L.ref_kd_build(self.ndim, self.n, self.coords.ctypes.data)

    def __del__(self):
        try:
            reflib().ref_kd_free(self.h)
        except Exception:
            pass

    def range(self, q, r, ordered=False):
        q = np.ascontiguousarray(q, np.float64)
        cap = max(self.n, 1)
        data = np.empty(cap, np.int32)
        d2 = np.empty(cap, np.float64)
        n = reflib().ref_kd_range(self.h, q.ctypes.data, float(r), int(ordered), data.ctypes.data,
                                  d2.ctypes.data, cap)
        assert n >= 0
        return data[:n].copy(), d2[:n].copy()


def calcinnandspread(HE, value, status):
    S = np.ascontiguousarray(HE, np.float32).copy()
    m, n = S.shape
    s_f = np.zeros(n)
    std_f = np.zeros(n)
    lib().or_calcinnandspread(C.c_int(m), C.c_int(n), _p(S, C.c_float), _p(np.ascontiguousarray(value, np.float32), C.c_float),
                              _p(np.ascontiguousarray(status, np.int16), C.c_short), _p(s_f, C.c_double),
                              _p(std_f, C.c_double))
    return S, s_f, std_f


def standardise(S, s_f, estd, otype, rfactor):
    S = np.ascontiguousarray(S, np.float32).copy()
    s_f = np.ascontiguousarray(s_f, np.float64).copy()
    m, n = S.shape
    lib().or_standardise(C.c_int(m), C.c_int(n), _p(S, C.c_float), _p(s_f, C.c_double),
                         _p(np.ascontiguousarray(estd, np.float32), C.c_float),
                         _p(np.ascontiguousarray(otype, np.int16), C.c_short),
                         _p(np.ascontiguousarray(rfactor, np.float64), C.c_double))
    return S, s_f


def calctransforms(obs: ObsSet, *, mode, scheme, nmem, nmem_dynamic, alpha, stride, x, y, S, s,
                   rows=None, threads: int = 1, want64=False, want_diag=True, x2d=None, y2d=None, units=None):
    """das_calctransforms over strided rows `rows` (default all; a (first,
    last+1) tuple or a list of rows), run on `threads` host threads
    (contiguous row blocks, as distribute_iterations assigns them); or, with
    `units`, over a list of (row, first column, end column) pieces taken
    from a shared queue by the threads as they come free.  Returns a dict of
    full-size outputs (points not computed stay zero)."""
    x = np.ascontiguousarray(x, np.float64)
    y = np.ascontiguousarray(y, np.float64)
    mni = x.size if x2d is None else x2d.shape[1]
    mnj = y.size if y2d is None else y2d.shape[0]
    nj = (mnj - 1) // stride + 1
    ni = (mni - 1) // stride + 1
    m, md = nmem, nmem_dynamic
    enkf = mode in (0, 2)
    S = np.ascontiguousarray(S, np.float32)
    s = np.ascontiguousarray(s, np.float64)
    T = np.zeros((nj, ni, md, m), np.float32) if enkf else None
    w = np.zeros((nj, ni, m), np.float32)
    T64 = np.zeros((nj, ni, md, m)) if (want64 and enkf) else None
    w64 = np.zeros((nj, ni, m)) if want64 else None
    nt = obs.ntypes
    nlobs = np.zeros((nj, ni), np.int32) if want_diag else None
    dfs = np.zeros((nj, ni), np.float32) if want_diag else None
    srf = np.zeros((nj, ni), np.float32) if want_diag else None
    pn = np.zeros((nt, nj, ni), np.int32) if want_diag else None
    pd = np.zeros((nt, nj, ni), np.float32) if want_diag else None
    ps = np.zeros((nt, nj, ni), np.float32) if want_diag else None
    x2 = None if x2d is None else np.ascontiguousarray(x2d, np.float64)
    y2 = None if y2d is None else np.ascontiguousarray(y2d, np.float64)
    P = CalcParams(mode, scheme, m, md, float(alpha), stride, mni, mnj, _p(x, C.c_double), _p(y, C.c_double),
                   _p(x2, C.c_double), _p(y2, C.c_double), 0, 0)
    if units is not None:
        # a work queue of (strided row, first column, end column) units taken
        # by the threads as they come free (the dynamic schedule of the
        # reference's mpiqueue, common/mpiqueue.c:124-248)
        units = [tuple(int(v) for v in u) for u in units]
        nxt = [0]
        qlock = threading.Lock()
        L = lib()
        rcs = []

        def worker():
            while True:
                with qlock:
                    k = nxt[0]
                    nxt[0] += 1
                if k >= len(units):
                    return
                jj, i0, i1 = units[k]
                Pk = CalcParams(mode, scheme, m, md, float(alpha), stride, mni, mnj, _p(x, C.c_double),
                                _p(y, C.c_double), _p(x2, C.c_double), _p(y2, C.c_double), i0, i1)
                rcs.append(L.or_calctransforms(C.c_void_p(obs.h), C.byref(Pk), _p(S, C.c_float), _p(s, C.c_double),
                                               _p(obs.otype, C.c_short), C.c_int(jj), C.c_int(jj + 1),
                                               _p(T, C.c_float), _p(w, C.c_float), _p(T64, C.c_double),
                                               _p(w64, C.c_double), _p(nlobs, C.c_int), _p(dfs, C.c_float),
                                               _p(srf, C.c_float), _p(pn, C.c_int), _p(pd, C.c_float),
                                               _p(ps, C.c_float)))

        ts = [threading.Thread(target=worker) for _ in range(max(1, threads))]
        for t in ts:
            t.start()
        for t in ts:
            t.join()
        if any(rcs):
            raise RuntimeError(f"LAPACK failure {[r for r in rcs if r]}")
        return dict(T=T, w=w, T64=T64, w64=w64, nlobs=nlobs, dfs=dfs, srf=srf, pnlobs=pn, pdfs=pd, psrf=ps)
    if rows is None:
        rowlist = list(range(nj))
    elif isinstance(rows, tuple) and len(rows) == 2:
        rowlist = list(range(int(rows[0]), int(rows[1])))
    else:
        rowlist = [int(r) for r in rows]
    L = lib()
    rcs = []

    def run(a, b):
        rc = L.or_calctransforms(C.c_void_p(obs.h), C.byref(P), _p(S, C.c_float), _p(s, C.c_double),
                                 _p(obs.otype, C.c_short), C.c_int(a), C.c_int(b), _p(T, C.c_float),
                                 _p(w, C.c_float), _p(T64, C.c_double), _p(w64, C.c_double), _p(nlobs, C.c_int),
                                 _p(dfs, C.c_float), _p(srf, C.c_float), _p(pn, C.c_int), _p(pd, C.c_float),
                                 _p(ps, C.c_float))
        rcs.append(rc)

    def run_list(lst):
        # contiguous runs of rows in one call each
        k = 0
        while k < len(lst):
            e = k
            while e + 1 < len(lst) and lst[e + 1] == lst[e] + 1:
                e += 1
            run(lst[k], lst[e] + 1)
            k = e + 1

    threads = max(1, min(threads, len(rowlist)))
    if threads == 1:
        run_list(rowlist)
    else:
        # contiguous blocks of rows per thread, as distribute_iterations assigns them
        bounds = np.linspace(0, len(rowlist), threads + 1).astype(int)
        ts = [threading.Thread(target=run_list, args=(rowlist[bounds[k]:bounds[k + 1]],)) for k in range(threads)]
        for t in ts:
            t.start()
        for t in ts:
            t.join()
    if any(rcs):
        raise RuntimeError(f"LAPACK failure {rcs}")
    return dict(T=T, w=w, T64=T64, w64=w64, nlobs=nlobs, dfs=dfs, srf=srf, pnlobs=pn, pdfs=pd, psrf=ps)


def updatefields(v, T, w, numlevels, *, mode, nmem, nmem_dynamic, stride, periodic_i=0, level=0, surfk=0,
                 issurfacevar=0, inflation=1.0, inf_ratio=float("nan"), output_increment=0, applylog=0,
                 j1=0, j2=None, want_infl=False):
    """das_updatefields for one field-layer. v is [nmem][jsize][mni] (copied)."""
    v = np.ascontiguousarray(v, np.float32).copy()
    nl = np.ascontiguousarray(numlevels, np.int32)
    mnj, mni = nl.shape
    nj, ni = w.shape[:2]
    if j2 is None:
        j2 = mnj - 1
    infl = np.zeros((j2 - j1 + 1, mni), np.float32) if want_infl else None
    P = UpdateParams(mode, nmem, nmem_dynamic, stride, periodic_i, mni, mnj, ni, nj, j1, j2, level, surfk,
                     issurfacevar, C.c_float(inflation), float(inf_ratio), output_increment, applylog)
    Tc = np.ascontiguousarray(T, np.float32)
    wc = np.ascontiguousarray(w, np.float32)
    lib().or_updatefields(C.byref(P), _p(Tc, C.c_float), _p(wc, C.c_float), _p(nl, C.c_int), _p(v, C.c_float),
                          _p(infl, C.c_float))
    return (v, infl) if want_infl else v


def updatebg(v, w, numlevels, *, nmem, stride, periodic_i=0, level=0, surfk=0, issurfacevar=0, j1=0, j2=None):
    """das_updatebg for one field-layer. v is [nmem + 1][jsize][mni] (copied)."""
    v = np.ascontiguousarray(v, np.float32).copy()
    nl = np.ascontiguousarray(numlevels, np.int32)
    mnj, mni = nl.shape
    nj, ni = w.shape[:2]
    if j2 is None:
        j2 = mnj - 1
    P = UpdateParams(1, nmem, nmem, stride, periodic_i, mni, mnj, ni, nj, j1, j2, level, surfk, issurfacevar,
                     C.c_float(1.0), float("nan"), 0, 0)
    wc = np.ascontiguousarray(w, np.float32)
    lib().or_updatebg(C.byref(P), _p(wc, C.c_float), _p(nl, C.c_int), _p(v, C.c_float))
    return v


def prepare(HE, value, status, estd, otype, rfactor):
    """das_calcinnandspread then das_standardise: standardised (S, s)."""
    S, s_f, _ = calcinnandspread(HE, value, status)
    return standardise(S, s_f, estd, otype, rfactor)


def sethybridensemble(v, nmem_d, gamma):
    """das_sethybridensemble. v is [nmem][nij] (copied). Returns (v, vmean)."""
    v = np.ascontiguousarray(v, np.float32).copy()
    m, nij = v.shape
    vmean = np.zeros(nij)
    lib().or_sethybridensemble(C.c_int(m), C.c_int(nmem_d), C.c_int(m - nmem_d), C.c_double(gamma),
                               C.c_int(nij), _p(v, C.c_float), _p(vmean, C.c_double))
    return v, vmean


def addnoise(v, deflation, sigma, random):
    """addnoise (update/update.c:46-87) on v [nmem][...] (copied): returns
    the randomised field.  random: at least nmem standard normals."""
    v = np.ascontiguousarray(v, np.float32).copy()
    m = v.shape[0]
    r = np.ascontiguousarray(random, np.float64)
    lib().or_addnoise(C.c_int(m), C.c_long(v.size // m), C.c_double(deflation), C.c_double(sigma), _p(r, C.c_double),
                      _p(v, C.c_float))
    return v


# ---------------------------------------------------------------------------
# forward operator (calc/model2obs.c) and the end of das_getHE (calc/ensobs.c)
# ---------------------------------------------------------------------------

REFLIB_UTILS = os.path.join(HERE, "_ref", "libenkf_ref_utils.so")
_refu = None


def reflib_utils():
    """The reference's own common/utils.c (interpolation, taper), or None."""
    global _refu
    with _lock:
        if _refu is None and os.path.exists(REFLIB_UTILS):
            L = C.CDLL(REFLIB_UTILS)
            L.interpolate2d_structured.restype = C.c_float
            L.interpolate2d_structured.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_int]
            L.interpolate3d_structured.restype = C.c_float
            L.interpolate3d_structured.argtypes = [C.c_void_p, C.c_double, C.c_int, C.c_int, C.c_int, C.c_int,
                                                   C.c_void_p, C.c_void_p, C.c_int]
            L.taper_gc.restype = C.c_double
            L.taper_gc.argtypes = [C.c_double]
            L.ll2xyz.argtypes = [C.c_void_p, C.c_void_p]
            _refu = L
    return _refu


def _rows(a: np.ndarray, t):
    """Row-pointer array (the reference's alloc2d/alloc3d view) over a
    contiguous array's leading dimensions."""
    lead = int(np.prod(a.shape[:-1]))
    flat = a.reshape(lead, a.shape[-1])
    base = flat.ctypes.data
    rows = (C.c_void_p * lead)(*[base + r * flat.strides[0] for r in range(lead)])
    return rows


def ref_interp2d(fi, fj, v, mask, periodic_i=0):
    """interpolate2d_structured from the reference build, one position."""
    L = reflib_utils()
    v = np.ascontiguousarray(v, np.float32)
    mask = np.ascontiguousarray(mask, np.int32)
    nj, ni = v.shape
    vr, mr = _rows(v, C.c_float), _rows(mask, C.c_int)
    fij = (C.c_double * 3)(float(fi), float(fj), float("nan"))
    return np.float32(L.interpolate2d_structured(fij, ni, nj, vr, mr, int(periodic_i)))


def ref_interp3d(fi, fj, fk, v, nlevels, ktop, periodic_i=0):
    """interpolate3d_structured from the reference build, one position;
    v is [nk][nj][ni]."""
    L = reflib_utils()
    v = np.ascontiguousarray(v, np.float32)
    nl = np.ascontiguousarray(nlevels, np.int32)
    nk, nj, ni = v.shape
    # alloc3d view: k -> row-pointer block, row -> data
    rows = _rows(v, C.c_float)
    planes = (C.c_void_p * nk)(*[C.addressof(rows) + k * nj * C.sizeof(C.c_void_p) for k in range(nk)])
    fij = (C.c_double * 3)(float(fi), float(fj), float("nan"))
    # the reference passes observation.fk (a float) as a double
    fk = float(np.float32(fk))
    return np.float32(L.interpolate3d_structured(fij, fk, ni, nj, nk, int(ktop), planes, _rows(nl, C.c_int),
                                                 int(periodic_i)))


def ref_taper_gc(x: float) -> float:
    return reflib_utils().taper_gc(float(x))


def interp2d(fi, fj, v, mask, periodic_i=0):
    """or_interp2d, one position: (value, badpos)."""
    v = np.ascontiguousarray(v, np.float32)
    mask = np.ascontiguousarray(mask, np.int32)
    nj, ni = v.shape
    bad = C.c_int(0)
    L = lib()
    L.or_interp2d.restype = C.c_float
    r = L.or_interp2d(C.c_double(fi), C.c_double(fj), C.c_int(ni), C.c_int(nj), _p(v, C.c_float),
                      _p(mask, C.c_int), C.c_int(int(periodic_i)), C.byref(bad))
    return np.float32(r), bool(bad.value)


def interp3d(fi, fj, fk, v, nlevels, ktop, periodic_i=0):
    """or_interp3d, one position (fk rounded to float as observation.fk)."""
    v = np.ascontiguousarray(v, np.float32)
    nl = np.ascontiguousarray(nlevels, np.int32)
    nk, nj, ni = v.shape
    bad = C.c_int(0)
    L = lib()
    L.or_interp3d.restype = C.c_float
    r = L.or_interp3d(C.c_double(fi), C.c_double(fj), C.c_double(float(np.float32(fk))), C.c_int(ni), C.c_int(nj),
                      C.c_int(nk), C.c_int(int(ktop)), _p(v, C.c_float), _p(nl, C.c_int),
                      C.c_int(int(periodic_i)), C.byref(bad))
    return np.float32(r), bool(bad.value)


def map_obs(HE, row, field, numlevels, ids, fi, fj, fk=None, *, three_d=False, ktop=0, periodic_i=0,
            offset=None, offset_kind=0, skip_bad=False):
    """or_map_obs for one member: HE[row][ids] filled in place (HE float32
    [rows][nobs]).  Returns the oracle's code (0, 1 + id of a bad forecast,
    -(1 + id) of a position off the grid)."""
    field = np.ascontiguousarray(field, np.float32)
    if three_d:
        nk, nj, ni = field.shape
    else:
        (nj, ni), nk = field.shape, 1
    ids = np.ascontiguousarray(ids, np.int32)
    fi = np.ascontiguousarray(fi, np.float64)
    fj = np.ascontiguousarray(fj, np.float64)
    fk = np.ascontiguousarray(fk if fk is not None else np.zeros(fi.size), np.float32)
    off = np.ascontiguousarray(offset, np.float32) if offset is not None else None
    dst = HE[row]
    assert dst.flags.c_contiguous and dst.dtype == np.float32
    return lib().or_map_obs(C.c_int(int(three_d)), C.c_int(ni), C.c_int(nj), C.c_int(nk), C.c_int(int(ktop)),
                            C.c_int(int(periodic_i)), _p(np.ascontiguousarray(numlevels, np.int32), C.c_int),
                            _p(off, C.c_float), C.c_int(int(offset_kind) if off is not None else 0),
                            _p(field, C.c_float), C.c_int(ids.size), _p(ids, C.c_int), _p(fi, C.c_double),
                            _p(fj, C.c_double), _p(fk, C.c_float), C.c_int(int(skip_bad)), _p(dst, C.c_float))


def finish_HE(HE, status, *, mode, nmem_dynamic, gamma=0.0, Hx=None, skip_bad=False):
    """or_finish_HE on copies: returns (HE, status, nbad)."""
    S = np.ascontiguousarray(HE, np.float32).copy()
    st = np.ascontiguousarray(status, np.int16).copy()
    m, n = S.shape
    hx = np.ascontiguousarray(Hx, np.float32) if Hx is not None else None
    nbad = lib().or_finish_HE(C.c_int(mode), C.c_int(m), C.c_int(nmem_dynamic), C.c_double(gamma), C.c_int(n),
                              _p(S, C.c_float), _p(hx, C.c_float), C.c_int(int(skip_bad)), _p(st, C.c_short))
    return S, st, nbad


# ---------------------------------------------------------------------------
# the reference's own field update (update/update.c) and hybrid ensemble
# (common/dasystem.c), compiled unmodified (oracle/ref/ref_update.c)
# ---------------------------------------------------------------------------

REFLIB_ENSOBS = os.path.join(HERE, "_ref", "libenkf_ref_ensobs.so")
_refeo = None


def reflib_ensobs():
    """libenkf_ref_ensobs.so (the reference's calc/ensobs.c), or None where
    it is not built."""
    global _refeo
    with _lock:
        if _refeo is None and os.path.exists(REFLIB_ENSOBS):
            L = C.CDLL(REFLIB_ENSOBS)
            L.ref_calcinnandspread.argtypes = [C.c_int, C.c_int] + [C.c_void_p] * 5
            L.ref_standardise.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                                          C.c_void_p]
            _refeo = L
    return _refeo


def ref_calcinnandspread(HE, value, status):
    """das_calcinnandspread of the reference itself: (S = HA, s_f, std_f)."""
    L = reflib_ensobs()
    if L is None:
        raise RuntimeError("reference ensobs library not built")
    S = np.ascontiguousarray(HE, np.float32).copy()
    m, n = S.shape
    v = np.ascontiguousarray(value, np.float32)
    st = np.ascontiguousarray(status, np.int16)
    s_f = np.zeros(n)
    std_f = np.zeros(n)
    L.ref_calcinnandspread(m, n, S.ctypes.data, v.ctypes.data, st.ctypes.data, s_f.ctypes.data, std_f.ctypes.data)
    return S, s_f, std_f


def ref_standardise(S, s_f, estd, otype, rfactor):
    """das_standardise of the reference itself: (S, s) standardised."""
    L = reflib_ensobs()
    if L is None:
        raise RuntimeError("reference ensobs library not built")
    S = np.ascontiguousarray(S, np.float32).copy()
    s = np.ascontiguousarray(s_f, np.float64).copy()
    m, n = S.shape
    e = np.ascontiguousarray(estd, np.float32)
    t = np.ascontiguousarray(otype, np.int16)
    rf = np.ascontiguousarray(rfactor, np.float64)
    L.ref_standardise(m, n, S.ctypes.data, s.ctypes.data, e.ctypes.data, t.ctypes.data, rf.size, rf.ctypes.data)
    return S, s


REFLIB_OBS = os.path.join(HERE, "_ref", "libenkf_ref_obs.so")
_refob = None


def reflib_obs():
    """libenkf_ref_obs.so (the reference's obs_findlocal), or None where it
    is not built."""
    global _refob
    with _lock:
        if _refob is None and os.path.exists(REFLIB_OBS):
            L = C.CDLL(REFLIB_OBS)
            L.ref_findlocal.restype = C.c_longlong
            L.ref_findlocal.argtypes = [C.c_int] + [C.c_void_p] * 4 + [C.c_int, C.c_int] + [C.c_void_p] * 5 + \
                [C.c_int, C.c_int] + [C.c_void_p] * 5 + [C.c_longlong]
            _refob = L
    return _refob


def ref_findlocal(lon, lat, otype, status, ntypes, nlocrad, locrad, locweight, qlon, qlat, nlobsmax=None,
                  visible=None, geographic=False):
    """obs_findlocal of the reference itself at each query (NaN: a point
    without coordinates): a list of (ids, taper coefficients) in the
    reference's order.  locrad, locweight: [ntypes][MAXLOCRAD]."""
    L = reflib_obs()
    if L is None:
        raise RuntimeError("reference observations library not built")
    lon = np.ascontiguousarray(lon, np.float32)
    lat = np.ascontiguousarray(lat, np.float32)
    ot = np.ascontiguousarray(otype, np.int16)
    st = np.ascontiguousarray(status, np.int16)
    nl = np.ascontiguousarray(nlocrad, np.int32)
    lr = np.ascontiguousarray(locrad, np.float64).reshape(ntypes, -1)
    lw = np.ascontiguousarray(locweight, np.float64).reshape(ntypes, -1)
    nm = None if nlobsmax is None else np.ascontiguousarray(nlobsmax, np.int32)
    vis = None if visible is None else np.ascontiguousarray(visible, np.int32)
    qx = np.ascontiguousarray(qlon, np.float64)
    qy = np.ascontiguousarray(qlat, np.float64)
    nq = qx.size
    cap = max(1, lon.size) * nq
    counts = np.zeros(nq, np.int32)
    ids = np.zeros(cap, np.int32)
    lc = np.zeros(cap)
    tot = L.ref_findlocal(lon.size, lon.ctypes.data, lat.ctypes.data, ot.ctypes.data, st.ctypes.data, ntypes,
                          lr.shape[1], nl.ctypes.data, lr.ctypes.data, lw.ctypes.data,
                          None if nm is None else nm.ctypes.data, None if vis is None else vis.ctypes.data,
                          int(geographic), nq, qx.ctypes.data, qy.ctypes.data, counts.ctypes.data, ids.ctypes.data,
                          lc.ctypes.data, cap)
    assert tot >= 0
    out, k0 = [], 0
    for c in counts:
        out.append((ids[k0:k0 + c].copy(), lc[k0:k0 + c].copy()))
        k0 += c
    return out


REFLIB_TRANSFORMS = os.path.join(HERE, "_ref", "libenkf_ref_transforms.so")
_reftr = None


def reflib_transforms():
    """libenkf_ref_transforms.so (the reference's das_calctransforms), or
    None where it is not built."""
    global _reftr
    with _lock:
        if _reftr is None and os.path.exists(REFLIB_TRANSFORMS):
            L = C.CDLL(REFLIB_TRANSFORMS)
            if L.or_blas_load(blas_path().encode()) != 0:
                return None
            L.ref_calcpointlogtransforms.argtypes = [C.c_int, C.c_int, C.c_double, C.c_int, C.c_int, C.c_int] + \
                [C.c_void_p] * 6 + [C.c_int, C.c_int] + [C.c_void_p] * 4 + [C.c_int, C.c_int] + [C.c_void_p] * 4
            L.ref_calctransforms.argtypes = [C.c_int, C.c_int, C.c_double, C.c_int, C.c_int, C.c_int] + \
                [C.c_void_p] * 6 + [C.c_int, C.c_int] + [C.c_void_p] * 5 + [C.c_int, C.c_int, C.c_int] + \
                [C.c_void_p] * 2 + [C.c_int] + [C.c_void_p] * 8
            _reftr = L
    return _reftr


def ref_calctransforms(obs, *, mode, scheme, nmem, nmem_dynamic, alpha, stride, x, y, S, s, nlobsmax=None,
                       visible=None):
    """das_calctransforms of the reference itself on the rectangular grid
    (x, y) for the observation set `obs` (an ObsSet: positions, types,
    statuses, radii, weights, geographic flag), with S and s standardised.
    Returns the float outputs as the reference writes them: T (ENKF and
    HYBRID), w, nlobs, dfs, srf, pnlobs, pdfs, psrf."""
    L = reflib_transforms()
    if L is None:
        raise RuntimeError("reference transforms library not built")
    x = np.ascontiguousarray(x, np.float64)
    y = np.ascontiguousarray(y, np.float64)
    mni, mnj = x.size, y.size
    nj, ni = (mnj - 1) // stride + 1, (mni - 1) // stride + 1
    m, md, nt = nmem, nmem_dynamic, obs.ntypes
    S = np.ascontiguousarray(S, np.float32).copy()
    s = np.ascontiguousarray(s, np.float64).copy()
    T = np.zeros((nj, ni, md, m), np.float32)
    w = np.zeros((nj, ni, m), np.float32)
    nlobs = np.zeros((nj, ni), np.int32)
    dfs = np.zeros((nj, ni), np.float32)
    srf = np.zeros((nj, ni), np.float32)
    pn = np.zeros((nt, nj, ni), np.int32)
    pd = np.zeros((nt, nj, ni), np.float32)
    ps = np.zeros((nt, nj, ni), np.float32)
    lr = np.ascontiguousarray(obs.locrad, np.float64).reshape(nt, -1)
    lw = np.ascontiguousarray(obs.locweight, np.float64).reshape(nt, -1)
    if nlobsmax is None:
        nlobsmax = obs.nlobsmax
    nm = None if nlobsmax is None else np.ascontiguousarray(nlobsmax, np.int32)
    vis = None if visible is None else np.ascontiguousarray(visible, np.int32)
    # this library's mode codes (0 ENKF, 1 ENOI, 2 HYBRID) and scheme codes
    # (0 DEnKF, 1 ETKF) -> the reference's (common/global.h:64-72)
    L.ref_calctransforms(int(mode) + 1, int(scheme) + 1, float(alpha), m, md, obs.nobs, obs.lon.ctypes.data,
                         obs.lat.ctypes.data, obs.otype.ctypes.data, obs.status.ctypes.data, S.ctypes.data,
                         s.ctypes.data, nt, lr.shape[1], obs.nlocrad.ctypes.data, lr.ctypes.data, lw.ctypes.data,
                         None if nm is None else nm.ctypes.data, None if vis is None else vis.ctypes.data,
                         int(obs.geographic), mni, mnj, x.ctypes.data, y.ctypes.data, int(stride), T.ctypes.data,
                         w.ctypes.data, nlobs.ctypes.data, dfs.ctypes.data, srf.ctypes.data, pn.ctypes.data,
                         pd.ctypes.data, ps.ctypes.data)
    return dict(T=T if mode != 1 else None, w=w, nlobs=nlobs, dfs=dfs, srf=srf, pnlobs=pn, pdfs=pd, psrf=ps)


REFLIB_MODEL2OBS = os.path.join(HERE, "_ref", "libenkf_ref_model2obs.so")
_refmo = None


def reflib_model2obs():
    """libenkf_ref_model2obs.so (the reference's H_surf_standard and
    H_subsurf_standard), or None where it is not built."""
    global _refmo
    with _lock:
        if _refmo is None and os.path.exists(REFLIB_MODEL2OBS):
            L = C.CDLL(REFLIB_MODEL2OBS)
            L.ref_H.argtypes = [C.c_int] * 6 + [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_int] + \
                [C.c_void_p] * 4 + [C.c_int, C.c_void_p]
            _refmo = L
    return _refmo


def ref_H(field3, numlevels, ids, fi, fj, fk=None, *, three_d, ksurf, periodic_i=0, offset=None, offset_kind=0,
          skip_bad=True):
    """H_surf_standard (three_d False: layer ksurf of field3) or
    H_subsurf_standard of the reference itself for one member; field3 is
    [nk][nj][ni].  Returns dst [nobs] (NaN where not computed)."""
    L = reflib_model2obs()
    if L is None:
        raise RuntimeError("reference model2obs library not built")
    f = np.ascontiguousarray(field3, np.float32)
    nk, nj, ni = f.shape
    nl = np.ascontiguousarray(numlevels, np.int32).copy()
    ids = np.ascontiguousarray(ids, np.int32)
    fi = np.ascontiguousarray(fi, np.float64)
    fj = np.ascontiguousarray(fj, np.float64)
    fkk = np.ascontiguousarray(fk if fk is not None else np.zeros(fi.size), np.float32)
    off = None if offset is None else np.ascontiguousarray(offset, np.float32)
    dst = np.zeros(fi.size, np.float32)
    L.ref_H(int(three_d), ni, nj, nk, int(ksurf), int(periodic_i), nl.ctypes.data,
            None if off is None else off.ctypes.data, int(offset_kind) if off is not None else 0, f.ctypes.data,
            fi.size, ids.size, ids.ctypes.data, fi.ctypes.data, fj.ctypes.data, fkk.ctypes.data, int(skip_bad),
            dst.ctypes.data)
    return dst


REFLIB_GETHE = os.path.join(HERE, "_ref", "libenkf_ref_gethe.so")
_refge = None


def reflib_gethe():
    """libenkf_ref_gethe.so (the reference's das_getHE), or None where it is
    not built."""
    global _refge
    with _lock:
        if _refge is None and os.path.exists(REFLIB_GETHE):
            L = C.CDLL(REFLIB_GETHE)
            L.ref_getHE.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_int] + [C.c_int] * 5 + \
                [C.c_void_p, C.c_void_p, C.c_int] + [C.c_void_p] * 5 + [C.c_int, C.c_void_p, C.c_void_p]
            _refge = L
    return _refge


def ref_getHE(members, numlevels, otype, status, fi, fj, fk, issurface, *, mode, nmem_dynamic, gamma=0.0, ksurf=0,
              periodic_i=0, skip_bad=True):
    """das_getHE of the reference itself: members [nmem (+1: the EnOI
    background)][nk][nj][ni] of one variable; observation types with
    issurface[t] (H_surf_standard, else H_subsurf_standard).  mode: this
    library's codes (0 ENKF, 1 ENOI, 2 HYBRID).  Returns (HE [rows][nobs],
    statuses)."""
    L = reflib_gethe()
    if L is None:
        raise RuntimeError("reference das_getHE library not built")
    f = np.ascontiguousarray(members, np.float32)
    rows, nk, nj, ni = f.shape
    nmem = rows - 1 if mode == 1 else rows
    nl = np.ascontiguousarray(numlevels, np.int32).copy()
    ot = np.ascontiguousarray(otype, np.int16)
    st = np.ascontiguousarray(status, np.int16).copy()
    fi = np.ascontiguousarray(fi, np.float64)
    fj = np.ascontiguousarray(fj, np.float64)
    fk = np.ascontiguousarray(fk, np.float32)
    iss = np.ascontiguousarray(issurface, np.int32)
    HE = np.zeros((rows, ot.size), np.float32)
    L.ref_getHE(int(mode) + 1, nmem, int(nmem_dynamic), float(gamma), int(skip_bad), ni, nj, nk, int(ksurf),
                int(periodic_i), nl.ctypes.data, f.ctypes.data, ot.size, ot.ctypes.data, st.ctypes.data,
                fi.ctypes.data, fj.ctypes.data, fk.ctypes.data, iss.size, iss.ctypes.data, HE.ctypes.data)
    return HE, st


def ref_calcpointlogtransforms(obs, *, mode, scheme, nmem, nmem_dynamic, alpha, plon, plat, S, s):
    """das_calcpointlogtransforms of the reference itself at the log points
    (plon, plat): the double T [npl][nmem][nmem] (ENKF, HYBRID; None for
    EnOI) and w [npl][nmem] it hands to the point-log writer."""
    L = reflib_transforms()
    if L is None:
        raise RuntimeError("reference transforms library not built")
    m, nt = nmem, obs.ntypes
    px = np.ascontiguousarray(plon, np.float64)
    py = np.ascontiguousarray(plat, np.float64)
    S = np.ascontiguousarray(S, np.float32).copy()
    s = np.ascontiguousarray(s, np.float64).copy()
    T = np.zeros((px.size, m, m)) if mode != 1 else None
    w = np.zeros((px.size, m))
    lr = np.ascontiguousarray(obs.locrad, np.float64).reshape(nt, -1)
    lw = np.ascontiguousarray(obs.locweight, np.float64).reshape(nt, -1)
    nm = obs.nlobsmax
    L.ref_calcpointlogtransforms(int(mode) + 1, int(scheme) + 1, float(alpha), m, int(nmem_dynamic), obs.nobs,
                                 obs.lon.ctypes.data, obs.lat.ctypes.data, obs.otype.ctypes.data,
                                 obs.status.ctypes.data, S.ctypes.data, s.ctypes.data, nt, lr.shape[1],
                                 obs.nlocrad.ctypes.data, lr.ctypes.data, lw.ctypes.data,
                                 None if nm is None else nm.ctypes.data, int(obs.geographic), px.size,
                                 px.ctypes.data, py.ctypes.data, None if T is None else T.ctypes.data, w.ctypes.data)
    return T, w


REFLIB_UPDATE = os.path.join(HERE, "_ref", "libenkf_ref_update.so")
_refup = None


def reflib_update():
    """libenkf_ref_update.so, or None where it is not built."""
    global _refup
    with _lock:
        if _refup is None and os.path.exists(REFLIB_UPDATE):
            L = C.CDLL(REFLIB_UPDATE)
            if L.or_blas_load(blas_path().encode()) != 0:
                return None
            L.ref_update_layer.argtypes = [C.c_int] * 12 + [C.c_float, C.c_double, C.c_int, C.c_int] + \
                [C.c_void_p] * 4
            L.ref_sethybridensemble.argtypes = [C.c_int, C.c_int, C.c_double, C.c_int, C.c_void_p]
            L.ref_set_noise.argtypes = [C.c_double, C.c_double]
            L.ref_srand48.argtypes = [C.c_long]
            L.ref_normalpair.argtypes = [C.c_void_p]
            _refup = L
    return _refup


def ref_update_layer(v, T, w, numlevels, *, mode, nmem, nmem_dynamic, stride, periodic_i=0, level=0, surfk=0,
                     issurfacevar=0, inflation=1.0, inf_ratio=float("nan"), output_increment=0, applylog=0,
                     j1=0, j2=None):
    """das_updatefields (ENKF/HYBRID) or das_updatebg (ENOI) of the
    reference itself on one field-layer, model rows j1..j2.  v is [nmem][jsize]
    [mni] (ENOI: [nmem + 1][jsize][mni], the background last); returns the
    updated copy."""
    L = reflib_update()
    if L is None:
        raise RuntimeError("reference update library not built")
    v = np.ascontiguousarray(v, np.float32).copy()
    nl = np.ascontiguousarray(numlevels, np.int32).copy()
    mnj, mni = nl.shape
    if j2 is None:
        j2 = mnj - 1
    Tc = None if T is None else np.ascontiguousarray(T, np.float32)
    wc = np.ascontiguousarray(w, np.float32)
    # this library's mode codes (0 ENKF, 1 ENOI, 2 HYBRID) -> the
    # reference's MODE_ENKF 1, MODE_ENOI 2, MODE_HYBRID 3 (common/global.h:64-67)
    L.ref_update_layer(int(mode) + 1, int(nmem), int(nmem_dynamic), int(stride), int(periodic_i), int(mni), int(mnj),
                       int(j1), int(j2), int(level), int(surfk), int(issurfacevar), float(inflation),
                       float(inf_ratio), int(output_increment), int(applylog),
                       None if Tc is None else Tc.ctypes.data, wc.ctypes.data, nl.ctypes.data, v.ctypes.data)
    return v


def ref_update_layer_noise(v, T, w, numlevels, *, deflation, sigma, seed, **kw):
    """ref_update_layer with RANDOMISE: the reference's das_updatefields ends
    with its addnoise, whose normals come from drand48 seeded with `seed`.
    Returns (updated field, the normals addnoise drew: (nmem + 1) // 2 pairs
    flattened)."""
    L = reflib_update()
    if L is None:
        raise RuntimeError("reference update library not built")
    nmem = int(kw["nmem"])
    L.ref_set_noise(float(deflation), float(sigma))
    try:
        L.ref_srand48(int(seed))
        out = ref_update_layer(v, T, w, numlevels, **kw)
    finally:
        L.ref_set_noise(float("nan"), float("nan"))
    L.ref_srand48(int(seed))
    r = np.zeros((nmem + 1) // 2 * 2)
    for e in range((nmem + 1) // 2):
        pair = np.zeros(2)
        L.ref_normalpair(pair.ctypes.data)
        r[2 * e:2 * e + 2] = pair
    return out, r


def ref_sethybridensemble(v, nmem_d, gamma):
    """das_sethybridensemble of the reference itself; v is [nmem][nij]
    (copied).  Returns (v, vmean)."""
    L = reflib_update()
    if L is None:
        raise RuntimeError("reference update library not built")
    v = np.ascontiguousarray(v, np.float32)
    m, nij = v.shape
    buf = np.zeros((m + 2, nij), np.float32)
    buf[:m] = v
    L.ref_sethybridensemble(int(m), int(nmem_d), float(gamma), int(nij), buf.ctypes.data)
    vmean = buf[m:].reshape(-1).view(np.float64)[:nij].copy()
    return buf[:m].copy(), vmean
