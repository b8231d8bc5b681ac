"""Python binding of libenkfg (the C ABI in include/enkfg.h).

The class `Enkfg` exposes the device path under the names of the EnKF-C
routines it replaces (reference enkf/ tree):

  set_obstypes / set_obs        obstypes.c:170-560, observations.c:452 (obs_read)
  set_HE                        das->S in S_MODE_HE_f (dasystem.h:95)
  calcinnandspread              das_calcinnandspread (calc/ensobs.c:541)
  standardise                   das_standardise (calc/ensobs.c:849)
  findlocal                     obs_findlocal (common/observations.c:1837), all points
  calctransforms                das_calctransforms (calc/transforms.c:991)
  updatefields / updatebg       das_updatefields / das_updatebg (update/update.c:92, 568)
  sethybridensemble             das_sethybridensemble (common/dasystem.c:775)

The reference stops the program on any error (enkf_quit); here every failing
call raises `EnkfgError` carrying the status code and the library's message.
There is no CPU fallback: if libenkfg.so cannot be loaded, or no GPU is
present, construction fails.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIBPATH = os.path.join(_HERE, "_lib", "libenkfg.so")

MODE_ENKF, MODE_ENOI, MODE_HYBRID = 0, 1, 2
SCHEME_DENKF, SCHEME_ETKF = 0, 1
PATH_PLAIN, PATH_BATCHED = 0, 1
PREC_FP64, PREC_MIXED = 0, 1
MAXLOCRAD = 8

STATUS = {0: "OK", 1: "EINVAL", 2: "ECUDA", 3: "ENOMEM", 4: "ETIMEOUT", 5: "ENUMERIC", 6: "ECAPACITY",
          7: "ESTATE", 8: "EUNSUPPORTED"}

# every symbol include/enkfg.h declares
EXPORTS = ["enkfg_create", "enkfg_destroy", "enkfg_set_wait_limit", "enkfg_set_wait_drill", "enkfg_set_field_buffer_size", "enkfg_set_field_block_rows", "enkfg_set_solve_batch", "enkfg_last_error", "enkfg_status_string", "enkfg_version",
           "enkfg_set_obstypes", "enkfg_set_obstype_nlobsmax", "enkfg_set_obstype_visible", "enkfg_set_obs", "enkfg_set_HE", "enkfg_calc_innovations", "enkfg_standardise",
           "enkfg_set_S", "enkfg_get_S", "enkfg_set_grid", "enkfg_transform_dims", "enkfg_local_obs",
           "enkfg_calc_transforms", "enkfg_calc_transforms_dev", "enkfg_transforms_dev_ptr",
           "enkfg_set_transforms", "enkfg_update_fields", "enkfg_update_fields_dev", "enkfg_set_field_noise", "enkfg_set_hybrid_ensemble",
           "enkfg_set_hybrid_ensemble_dev", "enkfg_kernel_launches", "enkfg_stage_times", "enkfg_kernel_times", "enkfg_set_stream",
           "enkfg_set_HE_dev", "enkfg_rebuild_index", "enkfg_local_offsets_noalloc", "enkfg_autotune_table",
           "enkfg_autotune_reset", "enkfg_adjoint_transforms", "enkfg_adjoint_mean", "enkfg_set_obs_positions",
           "enkfg_begin_HE", "enkfg_map_obs", "enkfg_map_obs_dev", "enkfg_finish_HE", "enkfg_nc_last_error",
           "enkfg_nc_write_transforms", "enkfg_nc_create_transforms", "enkfg_nc_write_transforms_row",
           "enkfg_nc_write_diag", "enkfg_nc_inq_var", "enkfg_nc_get_vara_float",
           "enkfg_nc_read_layer", "enkfg_nc_read_field3d", "enkfg_nc_write_layer"]


class EnkfgError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


class HopParams(C.Structure):
    """enkfg_hop_params: one forward-operator call (H_surf_standard /
    H_subsurf_standard, model2obs.c:127-348)."""
    _fields_ = [("ni", C.c_int), ("nj", C.c_int), ("nk", C.c_int), ("three_d", C.c_int), ("ksurf", C.c_int),
                ("periodic_i", C.c_int), ("offset_kind", C.c_int), ("skip_bad", C.c_int)]


class Grid(C.Structure):
    _fields_ = [("mni", C.c_int), ("mnj", C.c_int), ("x", C.POINTER(C.c_double)), ("y", C.POINTER(C.c_double)),
                ("x2d", C.POINTER(C.c_double)), ("y2d", C.POINTER(C.c_double)), ("stride", C.c_int),
                ("periodic_i", C.c_int)]


class CalcParams(C.Structure):
    _fields_ = [("mode", C.c_int), ("scheme", C.c_int), ("alpha", C.c_double), ("path", C.c_int),
                ("precision", C.c_int), ("want_diag", C.c_int), ("tune", C.c_int)]


class Diag(C.Structure):
    _fields_ = [("nlobs", C.POINTER(C.c_int)), ("dfs", C.POINTER(C.c_float)), ("srf", C.POINTER(C.c_float)),
                ("pnlobs", C.POINTER(C.c_int)), ("pdfs", C.POINTER(C.c_float)), ("psrf", C.POINTER(C.c_float))]


class UpdateParams(C.Structure):
    _fields_ = [("mode", C.c_int), ("nmem", C.c_int), ("nmem_dynamic", C.c_int), ("surfk", C.c_int),
                ("issurfacevar", C.c_int), ("inflation", C.c_float), ("inf_ratio", C.c_double),
                ("output_increment", C.c_int), ("applylog", C.c_int), ("j1", C.c_int), ("j2", C.c_int),
                ("precision", C.c_int)]


_lib = None


def load(path: str = LIBPATH):
    """Load libenkfg.so (raises if it is missing: there is no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(path):
            raise FileNotFoundError(f"{path} is missing; build it with enkf-c_gb300/build.py")
        L = C.CDLL(path)
        L.enkfg_last_error.restype = C.c_char_p
        L.enkfg_status_string.restype = C.c_char_p
        L.enkfg_kernel_launches.restype = C.c_longlong
        L.enkfg_create.argtypes = [C.c_int, C.POINTER(C.c_void_p)]
        L.enkfg_destroy.argtypes = [C.c_void_p]
        L.enkfg_last_error.argtypes = [C.c_void_p]
        L.enkfg_kernel_launches.argtypes = [C.c_void_p]
        _lib = L
    return _lib


def _p(a, t):
    return None if a is None else a.ctypes.data_as(C.POINTER(t))


class Enkfg:
    """One device context (one GPU, one host thread)."""

    def __init__(self, device: int = 0):
        L = load()
        h = C.c_void_p()
        st = L.enkfg_create(device, C.byref(h))
        if st != 0:
            raise EnkfgError(st, "enkfg_create failed (no CUDA device?)")
        self.h = h
        self.L = L
        self.nobs = 0
        self.nmem = self.nmem_dynamic = 0
        self.ntypes = 0
        self.grid = None
        self.nj = self.ni = 0

    def close(self):
        if getattr(self, "h", None):
            self.L.enkfg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ck(self, st):
        if st != 0:
            raise EnkfgError(st, self.L.enkfg_last_error(self.h).decode())

    @property
    def launches(self) -> int:
        return int(self.L.enkfg_kernel_launches(self.h))

    def set_wait_limit(self, ns: int = 0):
        """Bound on each device wait in ns (0: the library default, 2 s)."""
        self._ck(self.L.enkfg_set_wait_limit(self.h, C.c_ulonglong(int(ns))))

    def set_field_buffer_size(self, nfield: int = 0):
        """Field-layers per group of the host-buffer update (0: about 3 GB)."""
        self._ck(self.L.enkfg_set_field_buffer_size(self.h, C.c_int(int(nfield))))

    def set_solve_batch(self, points: int = 0):
        """Local analyses per batch of the batched solves (0: automatic)."""
        self._ck(self.L.enkfg_set_solve_batch(self.h, C.c_int(int(points))))

    def set_field_block_rows(self, rows: int = 0):
        """Model rows per block of the host-buffer update (0: about 512 MB)."""
        self._ck(self.L.enkfg_set_field_block_rows(self.h, C.c_int(int(rows))))

    def set_wait_drill(self, on: bool):
        """The timeout drill of the mixed kernel (a bounded wait that expires)."""
        self._ck(self.L.enkfg_set_wait_drill(self.h, C.c_int(int(bool(on)))))

    def stage_times(self):
        ms = (C.c_float * 4)()
        self._ck(self.L.enkfg_stage_times(self.h, ms))
        return list(ms)

    def kernel_times(self):
        """[transform kernel ms, rest of the transform stage ms]"""
        ms = (C.c_float * 2)()
        self._ck(self.L.enkfg_kernel_times(self.h, ms))
        return list(ms)

    # ---- inputs ----------------------------------------------------------
    def set_obstypes(self, nlocrad, locrad, locweight=None, rfactor=None, geographic=False):
        nlocrad = np.ascontiguousarray(nlocrad, np.int32)
        self.ntypes = nlocrad.size
        lr = np.ascontiguousarray(locrad, np.float64).reshape(self.ntypes, MAXLOCRAD)
        lw = None if locweight is None else np.ascontiguousarray(locweight, np.float64).reshape(self.ntypes, MAXLOCRAD)
        rf = None if rfactor is None else np.ascontiguousarray(rfactor, np.float64)
        self._keep_types = (nlocrad, lr, lw, rf)
        self._ck(self.L.enkfg_set_obstypes(self.h, C.c_int(self.ntypes), _p(nlocrad, C.c_int), _p(lr, C.c_double),
                                           _p(lw, C.c_double), _p(rf, C.c_double), C.c_int(int(geographic))))

    def set_obstype_nlobsmax(self, nlobsmax=None):
        """NLOBSMAX per type (<= 0: no limit); None clears every limit."""
        nl = None if nlobsmax is None else np.ascontiguousarray(nlobsmax, np.int32)
        self._ck(self.L.enkfg_set_obstype_nlobsmax(self.h, C.c_int(self.ntypes), _p(nl, C.c_int)))

    def set_obstype_visible(self, visible=None):
        """Per type, 0 hides it from the local search (obs-type domains);
        None shows every type."""
        v = None if visible is None else np.ascontiguousarray(visible, np.int32)
        self._ck(self.L.enkfg_set_obstype_visible(self.h, C.c_int(self.ntypes), _p(v, C.c_int)))

    def set_obs(self, lon, lat, otype, status, estd=None, value=None):
        lon = np.ascontiguousarray(lon, np.float32)
        lat = np.ascontiguousarray(lat, np.float32)
        otype = np.ascontiguousarray(otype, np.int16)
        status = np.ascontiguousarray(status, np.int16)
        estd = None if estd is None else np.ascontiguousarray(estd, np.float32)
        value = None if value is None else np.ascontiguousarray(value, np.float32)
        self.nobs = lon.size
        self._ck(self.L.enkfg_set_obs(self.h, C.c_int(self.nobs), _p(lon, C.c_float), _p(lat, C.c_float),
                                      _p(otype, C.c_short), _p(status, C.c_short), _p(estd, C.c_float),
                                      _p(value, C.c_float)))

    def set_HE(self, HE, nmem_dynamic=None):
        HE = np.ascontiguousarray(HE, np.float32)
        m = HE.shape[0]
        md = m if nmem_dynamic is None else int(nmem_dynamic)
        self.nmem, self.nmem_dynamic = m, md
        self._ck(self.L.enkfg_set_HE(self.h, C.c_int(m), C.c_int(md), _p(HE, C.c_float)))

    # ---- forward operator on the device (das_getHE, ensobs.c:46-490) -----
    def set_obs_positions(self, fi, fj, fk=None):
        """observation.fij[0..1] (double) and observation.fk (float, or None)."""
        fi = np.ascontiguousarray(fi, np.float64)
        fj = np.ascontiguousarray(fj, np.float64)
        fk = None if fk is None else np.ascontiguousarray(fk, np.float32)
        self._ck(self.L.enkfg_set_obs_positions(self.h, _p(fi, C.c_double), _p(fj, C.c_double), _p(fk, C.c_float)))

    def begin_HE(self, nmem, nmem_dynamic=None, with_background=False):
        md = nmem if nmem_dynamic is None else int(nmem_dynamic)
        self.nmem, self.nmem_dynamic = int(nmem), md
        self._ck(self.L.enkfg_begin_HE(self.h, C.c_int(int(nmem)), C.c_int(md), C.c_int(int(with_background))))

    def map_obs(self, obstype, fields, numlevels, *, mem0=0, ids=None, three_d=False, ksurf=0, periodic_i=False,
                offset=None, offset_kind=0, skip_bad=False):
        """H for one observation type over members mem0.. (mem0 = -1: the EnOI
        background).  fields [nfield][nk][nj][ni] (three_d) or [nfield][nj][ni]."""
        fields = np.ascontiguousarray(fields, np.float32)
        if three_d:
            nfield, nk, nj, ni = fields.shape
        else:
            (nfield, nj, ni), nk = fields.shape, 1
        prm = HopParams(ni, nj, nk, int(three_d), int(ksurf), int(bool(periodic_i)),
                        int(offset_kind) if offset is not None else 0, int(bool(skip_bad)))
        nl = np.ascontiguousarray(numlevels, np.int32)
        off = None if offset is None else np.ascontiguousarray(offset, np.float32)
        idv = None if ids is None else np.ascontiguousarray(ids, np.int32)
        nids = self.nobs if idv is None else idv.size
        self._ck(self.L.enkfg_map_obs(self.h, C.byref(prm), C.c_int(int(obstype)), C.c_int(nids), _p(idv, C.c_int),
                                      C.c_int(int(mem0)), C.c_int(nfield), _p(fields, C.c_float), _p(nl, C.c_int),
                                      _p(off, C.c_float)))

    def map_obs_dev(self, obstype, fields_ptr, nfield, ni, nj, numlevels_ptr, *, nk=1, mem0=0, ids_ptr=None,
                    nids=None, three_d=False, ksurf=0, periodic_i=False, offset_ptr=None, offset_kind=0,
                    skip_bad=False, stream=None):
        """Device-pointer form of map_obs (int addresses, e.g. tensor.data_ptr())."""
        prm = HopParams(int(ni), int(nj), int(nk), int(three_d), int(ksurf), int(bool(periodic_i)),
                        int(offset_kind) if offset_ptr else 0, int(bool(skip_bad)))
        n = self.nobs if nids is None else int(nids)
        self._ck(self.L.enkfg_map_obs_dev(self.h, C.byref(prm), C.c_int(int(obstype)), C.c_int(n),
                                          C.c_void_p(ids_ptr) if ids_ptr else None, C.c_int(int(mem0)),
                                          C.c_int(int(nfield)), C.c_void_p(fields_ptr), C.c_void_p(numlevels_ptr),
                                          C.c_void_p(offset_ptr) if offset_ptr else None,
                                          C.c_void_p(stream) if stream else None))

    def finish_HE(self, mode=0, gamma=0.0, skip_bad=False):
        """Returns (number of bad-forecast observations, statuses [nobs])."""
        nbad = C.c_int(0)
        status = np.zeros(self.nobs, np.int16)
        self._ck(self.L.enkfg_finish_HE(self.h, C.c_int(int(mode)), C.c_double(gamma), C.c_int(int(skip_bad)),
                                        C.byref(nbad), _p(status, C.c_short)))
        return nbad.value, status

    def set_stream(self, stream):
        """Bind a cudaStream_t (int address, e.g. torch.cuda.Stream().cuda_stream)."""
        self._ck(self.L.enkfg_set_stream(self.h, C.c_void_p(stream)))

    def set_HE_dev(self, HE_ptr, nmem, nmem_dynamic=None):
        md = nmem if nmem_dynamic is None else int(nmem_dynamic)
        self.nmem, self.nmem_dynamic = nmem, md
        self._ck(self.L.enkfg_set_HE_dev(self.h, C.c_int(nmem), C.c_int(md), C.c_void_p(HE_ptr)))

    def rebuild_index(self):
        self._ck(self.L.enkfg_rebuild_index(self.h))

    def calcinnandspread(self, want=True):
        if not want:
            self._ck(self.L.enkfg_calc_innovations(self.h, None, None))
            return None

        s_f = np.zeros(self.nobs)
        std_f = np.zeros(self.nobs)
        self._ck(self.L.enkfg_calc_innovations(self.h, _p(s_f, C.c_double), _p(std_f, C.c_double)))
        return s_f, std_f

    def standardise(self):
        self._ck(self.L.enkfg_standardise(self.h))

    def set_S(self, S, s, nmem_dynamic=None):
        S = np.ascontiguousarray(S, np.float32)
        s = np.ascontiguousarray(s, np.float64)
        m = S.shape[0]
        md = m if nmem_dynamic is None else int(nmem_dynamic)
        self.nmem, self.nmem_dynamic = m, md
        self._ck(self.L.enkfg_set_S(self.h, C.c_int(m), C.c_int(md), _p(S, C.c_float), _p(s, C.c_double)))

    def get_S(self):
        S = np.zeros((self.nmem, self.nobs), np.float32)
        s = np.zeros(self.nobs)
        self._ck(self.L.enkfg_get_S(self.h, _p(S, C.c_float), _p(s, C.c_double)))
        return S, s

    def set_grid(self, x=None, y=None, stride=1, periodic_i=False, x2d=None, y2d=None):
        if x2d is not None:
            x2d = np.ascontiguousarray(x2d, np.float64)
            y2d = np.ascontiguousarray(y2d, np.float64)
            mnj, mni = x2d.shape
            g = Grid(mni, mnj, None, None, _p(x2d, C.c_double), _p(y2d, C.c_double), stride, int(periodic_i))
            keep = (x2d, y2d)
        else:
            x = np.ascontiguousarray(x, np.float64)
            y = np.ascontiguousarray(y, np.float64)
            mni, mnj = x.size, y.size
            g = Grid(mni, mnj, _p(x, C.c_double), _p(y, C.c_double), None, None, stride, int(periodic_i))
            keep = (x, y)
        self._ck(self.L.enkfg_set_grid(self.h, C.byref(g)))
        self._keep_grid = keep
        self.mni, self.mnj, self.stride = mni, mnj, stride
        nj, ni = C.c_int(), C.c_int()
        self._ck(self.L.enkfg_transform_dims(self.h, C.byref(nj), C.byref(ni)))
        self.nj, self.ni = nj.value, ni.value

    # ---- calc ------------------------------------------------------------
    def findlocal(self, lists: bool = True, capacity: Optional[int] = None):
        """Local obs of every strided point: counts [nj][ni] and, if lists,
        (offsets [nj*ni+1], ids, coeffs) with each row sorted by obs id."""
        npts = self.nj * self.ni
        counts = np.zeros(npts, np.int32)
        if not lists:
            self._ck(self.L.enkfg_local_obs(self.h, _p(counts, C.c_int), None, None, None, C.c_longlong(0)))
            return counts.reshape(self.nj, self.ni)
        self._ck(self.L.enkfg_local_obs(self.h, _p(counts, C.c_int), None, None, None, C.c_longlong(0)))
        total = int(counts.astype(np.int64).sum()) if capacity is None else int(capacity)
        offsets = np.zeros(npts + 1, np.int64)
        ids = np.zeros(max(total, 1), np.int32)
        coeffs = np.zeros(max(total, 1), np.float64)
        self._ck(self.L.enkfg_local_obs(self.h, _p(counts, C.c_int), _p(offsets, C.c_longlong), _p(ids, C.c_int),
                                        _p(coeffs, C.c_double), C.c_longlong(total)))
        return counts.reshape(self.nj, self.ni), offsets, ids[:total], coeffs[:total]

    def autotune_table(self):
        t = (C.c_int * 16)()
        st = self.L.enkfg_autotune_table(self.h, t)
        return None if st != 0 else list(t)

    def autotune_reset(self):
        self._ck(self.L.enkfg_autotune_reset(self.h))

    def calctransforms(self, mode=MODE_ENKF, scheme=SCHEME_ETKF, alpha=1.0, path=PATH_PLAIN, precision=PREC_FP64,
                       want64=False, want_diag=True, tune=False, T_out=None, w_out=None):
        """T_out / w_out: caller-owned float32 arrays of the output shapes
        (e.g. in pinned memory) to write T and w into; allocated if None."""
        npts = self.nj * self.ni
        m, md = self.nmem, self.nmem_dynamic
        enkf = mode != MODE_ENOI

        def out_array(a, shape):
            if a is None:
                return np.zeros(shape, np.float32)
            if a.dtype != np.float32 or a.shape != shape or not a.flags.c_contiguous:
                raise ValueError(f"output array must be C-contiguous float32 {shape}")
            return a
        T = out_array(T_out, (self.nj, self.ni, md, m)) if enkf else None
        w = out_array(w_out, (self.nj, self.ni, m))
        T64 = np.zeros((self.nj, self.ni, md, m)) if (want64 and enkf) else None
        w64 = np.zeros((self.nj, self.ni, m)) if want64 else None
        out = dict(T=T, w=w, T64=T64, w64=w64)
        dg = None
        if want_diag:
            nt = self.ntypes
            out.update(nlobs=np.zeros((self.nj, self.ni), np.int32), dfs=np.zeros((self.nj, self.ni), np.float32),
                       srf=np.zeros((self.nj, self.ni), np.float32),
                       pnlobs=np.zeros((nt, self.nj, self.ni), np.int32),
                       pdfs=np.zeros((nt, self.nj, self.ni), np.float32),
                       psrf=np.zeros((nt, self.nj, self.ni), np.float32))
            dg = Diag(_p(out["nlobs"], C.c_int), _p(out["dfs"], C.c_float), _p(out["srf"], C.c_float),
                      _p(out["pnlobs"], C.c_int), _p(out["pdfs"], C.c_float), _p(out["psrf"], C.c_float))
        prm = CalcParams(mode, scheme, float(alpha), path, precision, int(want_diag), int(tune))
        self._ck(self.L.enkfg_calc_transforms(self.h, C.byref(prm), _p(T, C.c_float), _p(w, C.c_float),
                                              _p(T64, C.c_double), _p(w64, C.c_double),
                                              C.byref(dg) if dg is not None else None))
        return out

    def calctransforms_dev(self, mode=MODE_ENKF, scheme=SCHEME_ETKF, alpha=1.0, path=PATH_PLAIN,
                           precision=PREC_FP64, want_diag=False, stream=None, tune=False):
        prm = CalcParams(mode, scheme, float(alpha), path, precision, int(want_diag), int(tune))
        self._ck(self.L.enkfg_calc_transforms_dev(self.h, C.byref(prm), C.c_void_p(stream)))

    def set_transforms(self, T, w, mode=MODE_ENKF, nmem=None, nmem_dynamic=None):
        w = np.ascontiguousarray(w, np.float32)
        m = w.shape[-1] if nmem is None else nmem
        md = (T.shape[-2] if T is not None else m) if nmem_dynamic is None else nmem_dynamic
        T = None if T is None else np.ascontiguousarray(T, np.float32)
        self._ck(self.L.enkfg_set_transforms(self.h, C.c_int(mode), C.c_int(m), C.c_int(md), _p(T, C.c_float),
                                             _p(w, C.c_float)))

    # ---- adjoint (observation impact) -----------------------------------
    def adjoint_transforms(self, wbar, Tbar=None, mode=MODE_ENKF, scheme=SCHEME_ETKF, alpha=1.0,
                           precision=PREC_FP64):
        """dJ/d(innovation) [nobs], dJ/d(estd^2) [nobs], dJ/d(radius scale);
        precision PREC_MIXED runs the FP32 (production) form."""
        wbar = np.ascontiguousarray(wbar, np.float64)
        Tbar = None if Tbar is None else np.ascontiguousarray(Tbar, np.float64)
        dinn = np.zeros(self.nobs)
        dvar = np.zeros(self.nobs)
        drad = np.zeros(1)
        prm = CalcParams(mode, scheme, float(alpha), PATH_PLAIN, precision, 0, 0)
        self._ck(self.L.enkfg_adjoint_transforms(self.h, C.byref(prm), _p(wbar, C.c_double), _p(Tbar, C.c_double),
                                                 _p(dinn, C.c_double), _p(dvar, C.c_double), _p(drad, C.c_double)))
        return dinn, dvar, float(drad[0])

    def adjoint_mean(self, field, dJ_dmean, nmem=None, nmem_dynamic=None):
        """wbar [nj][ni][m] from the forecast field [m][mnj][mni] and dJ/dmean [mnj][mni]."""
        field = np.ascontiguousarray(field, np.float32)
        g = np.ascontiguousarray(dJ_dmean, np.float64)
        m = field.shape[0] if nmem is None else nmem
        md = m if nmem_dynamic is None else nmem_dynamic
        wbar = np.zeros((self.nj, self.ni, m))
        self._ck(self.L.enkfg_adjoint_mean(self.h, C.c_int(m), C.c_int(md), _p(field, C.c_float), _p(g, C.c_double),
                                           _p(wbar, C.c_double)))
        return wbar

    # ---- update ----------------------------------------------------------
    def updatefields(self, fields, numlevels, levels, *, mode=MODE_ENKF, nmem=None, nmem_dynamic=None, surfk=0,
                     issurfacevar=0, inflation=1.0, inf_ratio=float("nan"), output_increment=0, applylog=0, j1=0,
                     j2=-1, precision=PREC_FP64, want_infl=False, inplace=False):
        """fields [nfield][nmem(+1 for EnOI)][jsize][mni] float32, updated
        and returned (a copy, or `fields` itself when inplace -- which then
        must be C-contiguous float32); levels [nfield]."""
        if inplace:
            if fields.dtype != np.float32 or not fields.flags.c_contiguous:
                raise ValueError("inplace update needs a C-contiguous float32 array")
            f = fields
        else:
            f = np.ascontiguousarray(fields, np.float32).copy()
        nl = np.ascontiguousarray(numlevels, np.int32)
        lv = np.ascontiguousarray(levels, np.int32)
        nfield = f.shape[0]
        m = self.nmem if nmem is None else nmem
        md = self.nmem_dynamic if nmem_dynamic is None else nmem_dynamic
        infl = np.zeros((nfield,) + f.shape[2:], np.float32) if want_infl else None
        prm = UpdateParams(mode, m, md, surfk, issurfacevar, C.c_float(inflation), float(inf_ratio),
                           int(output_increment), int(applylog), j1, j2, precision)
        self._ck(self.L.enkfg_update_fields(self.h, C.byref(prm), _p(nl, C.c_int), C.c_int(nfield), _p(lv, C.c_int),
                                            _p(f, C.c_float), _p(infl, C.c_float)))
        return (f, infl) if want_infl else f

    def set_field_noise(self, deflation=None, sigma=None, random=None):
        """RANDOMISE for the next update call: deflation, sigma [nfield]
        (NaN deflation: no noise for that field-layer), random [nfield][nmem]
        standard normals.  No arguments: none."""
        if deflation is None:
            self._ck(self.L.enkfg_set_field_noise(self.h, C.c_int(0), C.c_int(0), None, None, None))
            return
        d = np.ascontiguousarray(deflation, np.float64)
        sg = np.ascontiguousarray(sigma, np.float64)
        r = np.ascontiguousarray(random, np.float64)
        nfield, nmem = r.shape
        self._ck(self.L.enkfg_set_field_noise(self.h, C.c_int(nfield), C.c_int(nmem), _p(d, C.c_double),
                                              _p(sg, C.c_double), _p(r, C.c_double)))

    def updatebg(self, fields, numlevels, levels, **kw):
        kw["mode"] = MODE_ENOI
        return self.updatefields(fields, numlevels, levels, **kw)

    def updatefields_dev(self, fields_ptr, numlevels_ptr, nfield, levels, *, mode=MODE_ENKF, nmem=None,
                         nmem_dynamic=None, surfk=0, issurfacevar=0, inflation=1.0, inf_ratio=float("nan"),
                         output_increment=0, applylog=0, j1=0, j2=-1, precision=PREC_FP64, infl_ptr=None,
                         stream=None):
        lv = np.ascontiguousarray(levels, np.int32)
        m = self.nmem if nmem is None else nmem
        md = self.nmem_dynamic if nmem_dynamic is None else nmem_dynamic
        prm = UpdateParams(mode, m, md, surfk, issurfacevar, C.c_float(inflation), float(inf_ratio),
                           int(output_increment), int(applylog), j1, j2, precision)
        self._ck(self.L.enkfg_update_fields_dev(self.h, C.byref(prm), C.c_void_p(numlevels_ptr), C.c_int(nfield),
                                                _p(lv, C.c_int), C.c_void_p(fields_ptr), C.c_void_p(infl_ptr),
                                                C.c_void_p(stream)))

    def sethybridensemble(self, v, nmem_dynamic, gamma):
        v = np.ascontiguousarray(v, np.float32).copy()
        m, nij = v.shape[0], int(np.prod(v.shape[1:]))
        self._ck(self.L.enkfg_set_hybrid_ensemble(self.h, C.c_int(m), C.c_int(nmem_dynamic), C.c_double(gamma),
                                                  C.c_int(nij), _p(v, C.c_float)))
        return v


# ---------------------------------------------------------------------------
# NetCDF classic files (host only; no context, no GPU)
# ---------------------------------------------------------------------------

NC_MAXDIMS = 8


def _nc_ck(st):
    if st != 0:
        L = load()
        L.enkfg_nc_last_error.restype = C.c_char_p
        raise EnkfgError(st, L.enkfg_nc_last_error().decode())


def nc_write_transforms(path, T, w, stride=1, grid_name=""):
    """transforms.nc (calc/transforms.c:54-131); T [nj][ni][m_dyn][m] or None
    (EnOI), w [nj][ni][m]."""
    w = np.ascontiguousarray(w, np.float32)
    nj, ni, m = w.shape
    Tc = None if T is None else np.ascontiguousarray(T, np.float32)
    md = 0 if Tc is None else Tc.shape[2]
    _nc_ck(load().enkfg_nc_write_transforms(os.fsencode(path), C.c_int(nj), C.c_int(ni), C.c_int(md), C.c_int(m),
                                            _p(Tc, C.c_float), _p(w, C.c_float), C.c_int(int(stride)),
                                            grid_name.encode()))


def nc_create_transforms(path, nj, ni, nmem_dynamic, nmem, with_T=True, stride=1, grid_name=""):
    """nc_createtransforms (calc/transforms.c:54-94): the file, rows to follow."""
    _nc_ck(load().enkfg_nc_create_transforms(os.fsencode(path), C.c_int(nj), C.c_int(ni), C.c_int(nmem_dynamic),
                                             C.c_int(nmem), C.c_int(int(with_T)), C.c_int(int(stride)),
                                             grid_name.encode()))


def nc_write_transforms_row(path, j, Tj, wj):
    """nc_writetransforms (calc/transforms.c:98-131): strided row j."""
    wj = np.ascontiguousarray(wj, np.float32)
    Tj = None if Tj is None else np.ascontiguousarray(Tj, np.float32)
    _nc_ck(load().enkfg_nc_write_transforms_row(os.fsencode(path), C.c_int(int(j)), _p(Tj, C.c_float),
                                                _p(wj, C.c_float)))


def nc_write_diag(path, type_names, nlobs, dfs, srf, pnlobs, pdfs, psrf, stride=1):
    """enkf_diag.nc (calc/transforms.c:380-470)."""
    nlobs = np.ascontiguousarray(nlobs, np.int32)
    nj, ni = nlobs.shape
    nt = len(type_names)
    names = (C.c_char_p * nt)(*[n.encode() for n in type_names])
    arrs = [np.ascontiguousarray(a, t) for a, t in ((dfs, np.float32), (srf, np.float32), (pnlobs, np.int32),
                                                    (pdfs, np.float32), (psrf, np.float32))]
    _nc_ck(load().enkfg_nc_write_diag(os.fsencode(path), C.c_int(nj), C.c_int(ni), C.c_int(nt), names,
                                      C.c_int(int(stride)), _p(nlobs, C.c_int), _p(arrs[0], C.c_float),
                                      _p(arrs[1], C.c_float), _p(arrs[2], C.c_int), _p(arrs[3], C.c_float),
                                      _p(arrs[4], C.c_float)))


def nc_inq_var(path, var):
    """(dims tuple, NetCDF type code, has record dimension)."""
    nd = C.c_int(0)
    dims = (C.c_longlong * NC_MAXDIMS)()
    t = C.c_int(0)
    rec = C.c_int(0)
    _nc_ck(load().enkfg_nc_inq_var(os.fsencode(path), var.encode(), C.byref(nd), dims, C.byref(t), C.byref(rec)))
    return tuple(dims[k] for k in range(nd.value)), t.value, bool(rec.value)


def nc_get_vara_float(path, var, start=None, count=None):
    dims, _, _ = nc_inq_var(path, var)
    start = [0] * len(dims) if start is None else list(start)
    count = [d - s for d, s in zip(dims, start)] if count is None else list(count)
    out = np.empty([int(c) for c in count], np.float32)
    st = (C.c_longlong * max(1, len(dims)))(*start)
    ct = (C.c_longlong * max(1, len(dims)))(*count)
    _nc_ck(load().enkfg_nc_get_vara_float(os.fsencode(path), var.encode(), st, ct, _p(out, C.c_float)))
    return out


def nc_read_layer(path, var, ni, nj, nk=1, k=0, r=-1):
    """ncu_readfield (common/ncutils.c:102-530): layer k of record r."""
    v = np.empty((nj, ni), np.float32)
    _nc_ck(load().enkfg_nc_read_layer(os.fsencode(path), var.encode(), C.c_int(r), C.c_int(k), C.c_int(ni),
                                      C.c_int(nj), C.c_int(nk), _p(v, C.c_float)))
    return v


def nc_read_field3d(path, var, ni, nj, nk, r=-1):
    """ncu_read3dfield (common/ncutils.c:923-1245): the [nk][nj][ni] field."""
    v = np.empty((nk, nj, ni), np.float32)
    _nc_ck(load().enkfg_nc_read_field3d(os.fsencode(path), var.encode(), C.c_int(r), C.c_int(ni), C.c_int(nj),
                                        C.c_int(nk), _p(v, C.c_float)))
    return v


def nc_write_layer(path, var, v, nk=1, k=0):
    """ncu_writefield (common/ncutils.c:537-700), into an existing file."""
    v = np.ascontiguousarray(v, np.float32)
    nj, ni = v.shape
    _nc_ck(load().enkfg_nc_write_layer(os.fsencode(path), var.encode(), C.c_int(int(k)), C.c_int(ni), C.c_int(nj),
                                       C.c_int(int(nk)), _p(v, C.c_float)))
