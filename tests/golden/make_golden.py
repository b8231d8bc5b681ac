"""Generate the golden fixtures under tests/golden/ from the REFERENCE itself.

Run in a container that holds the reference sources (it builds
oracle/_ref/libenkf_ref.so from the reference's calc/calcs.c and
common/kdtree.c, unmodified).  The fixtures pin the oracle restatement and the
GPU library without needing the reference at test time:

  numerics.npz    calc_wT_etkf / calc_wT_denkf / calc_G+calc_w (calcs.c) on
                  seeded S, s for p < m and p >= m: outputs w, T, G.
  kdtree.npz      kd_findnodeswithinrange (kdtree.c) results, in the tree's
                  own order, for trees built as obs_createkdtrees does
                  (sequential insertion by obs index), several query points,
                  two observation types.
  nlobsmax.npz    kd_findnodeswithinrange with ordered = 1 (the distance
                  sort obs_findlocal asks for when NLOBSMAX is set), in the
                  order the reference returns, for two observation types
                  whose observations come partly in groups at one position
                  (profiles: equal distances), at grid and off-grid queries;
                  in 2-D and on the sphere (3-D trees of the reference's
                  ll2xyz coordinates).
  transforms.npz  das_calctransforms on a sample of workload-1 points: local
                  obs from the reference kd-tree, taper and gather as
                  transforms.c:1250-1258 (restated here), numerics from the
                  reference's calcs.c: double T and w before the float cast.
                  The inputs (obs, S, s) are stored alongside.
  transforms_multitype.npz
                  the same for a two-type workload with rejected
                  observations (ENKF DEnKF and ETKF, EnOI; alpha 0.7), with
                  the diagnostics dfs, srf and per-type pdfs, psrf through
                  the reference's traceprod.
  calctransforms.npz
                  das_calctransforms itself (calc/transforms.c and the
                  files it calls, compiled unmodified, the grid and the
                  output files in memory): the float T, w and diagnostics of
                  a two-type workload at stride 3, ETKF (alpha 0.7) and DEnKF.
  model2obs.npz   interpolate2d_structured / interpolate3d_structured
                  (common/utils.c, from oracle/_ref/libenkf_ref_utils.so) on
                  seeded fields, wet-level counts, OFFSET data and positions
                  (integer positions, all edges, periodic and not, both
                  surface-layer conventions): the HE that H_surf_standard /
                  H_subsurf_standard (calc/model2obs.c) give with footprint 0.
  update.npz      das_updatefields / das_updatebg (update/update.c) and
                  das_sethybridensemble (common/dasystem.c), from
                  oracle/_ref/libenkf_ref_update.so (both files compiled
                  unmodified), on seeded transforms, fields and wet-level
                  counts: strides 1, 2 and 3, periodic i, field tiles
                  (j1..j2), land and level masks with surfk 0 and > 0,
                  missing values in dynamic and static members, spread-capped
                  inflation, increments, log10 fields, hybrid and EnOI.
  addnoise.npz    das_updatefields with RANDOMISE (deflation and sigma of the
                  variable set, so update.c ends with its addnoise), the
                  normals drawn by the reference's get_normalpair from a
                  seeded drand48 stored as inputs: ENKF and hybrid, odd and
                  even ensembles, strides 1-3, increments, log10 fields.

Usage:  python tests/golden/make_golden.py [fixture ...]   (default: all)
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "enkf-c_gb300"))

import oracle  # noqa: E402
import synth  # noqa: E402


def numerics():
    rng = np.random.default_rng(20240)
    cases = []
    for (m, mout, p) in [(24, 24, 60), (24, 24, 7), (24, 16, 40), (48, 48, 48), (48, 48, 300), (96, 96, 150),
                         (96, 64, 20)]:
        S = rng.standard_normal((m, p)) * (0.5 / np.sqrt(m - 1)) * rng.uniform(0.2, 3.0)
        S -= S.mean(axis=0, keepdims=True)   # anomalies: columns of HA sum to zero
        s = rng.standard_normal(p)
        for mode, scheme in [(0, 1), (0, 0), (1, 0)]:
            w, T, G = oracle.ref_calc_wT(mode, scheme, m, mout, s, S)
            cases.append(dict(m=m, mout=mout, p=p, mode=mode, scheme=scheme, S=S, s=s, w=w, T=T[:mout] if mode != 1 else T[:0], G=G))
    out = {}
    for k, c in enumerate(cases):
        for key, v in c.items():
            out[f"c{k}_{key}"] = np.asarray(v)
    out["ncases"] = np.array(len(cases))
    np.savez_compressed(os.path.join(HERE, "numerics.npz"), **out)
    print("numerics:", len(cases), "cases")


def kdtree():
    w = synth.make(2, scale=0.12, with_fields=False)
    coords = np.stack([w.lon.astype(np.float64), w.lat.astype(np.float64)], 1)
    rng = np.random.default_rng(7)
    qs = np.stack([rng.uniform(0, w.ni - 1, 40), rng.uniform(0, w.nj - 1, 40)], 1)
    qs[:8] = np.floor(qs[:8])           # grid points (integer coordinates)
    out = dict(lon=w.lon, lat=w.lat, otype=w.otype, q=qs, r=np.array([6.0, 9.0]))
    for t in range(w.ntypes):
        ids = np.nonzero(w.otype == t)[0]
        tree = oracle.RefKdTree(coords[ids])
        for k, q in enumerate(qs):
            d, d2 = tree.range(q, out["r"][t])
            out[f"t{t}_q{k}_ids"] = ids[d].astype(np.int32)
            out[f"t{t}_q{k}_d2"] = d2
    np.savez_compressed(os.path.join(HERE, "kdtree.npz"), **out)
    print("kdtree:", w.nobs, "obs,", len(qs), "queries")


def nlobsmax_obs(seed=5):
    """Observations of two types on a 60 x 40 domain; a third of each type in
    groups of 2-6 at one position (equal distances to any query)."""
    rng = np.random.default_rng(seed)
    lon, lat, ot = [], [], []
    for t, n in ((0, 900), (1, 500)):
        k = 0
        while k < n:
            x, y = rng.uniform(0, 60), rng.uniform(0, 40)
            g = int(rng.integers(2, 7)) if rng.uniform() < 0.33 else 1
            g = min(g, n - k)
            lon += [x] * g
            lat += [y] * g
            ot += [t] * g
            k += g
    perm = rng.permutation(len(lon))     # types and groups interleaved in id order
    lon = np.asarray(lon, np.float32)[perm]
    lat = np.asarray(lat, np.float32)[perm]
    ot = np.asarray(ot, np.int16)[perm]
    qs = np.stack([rng.uniform(0, 59, 30), rng.uniform(0, 39, 30)], 1)
    qs[:10] = np.floor(qs[:10])
    return lon, lat, ot, qs


def ref_xyz(lon, lat):
    """ll2xyz of the reference's own utils.c for each (lon, lat)."""
    import ctypes as C
    R = oracle.reflib_utils()
    out = np.zeros((len(lon), 3))
    for i, (x, y) in enumerate(zip(lon, lat)):
        ll = (C.c_double * 2)(float(x), float(y))
        v = (C.c_double * 3)()
        R.ll2xyz(ll, v)
        out[i] = list(v)
    return out


def nlobsmax():
    lon, lat, ot, qs = nlobsmax_obs()
    coords = np.stack([lon.astype(np.float64), lat.astype(np.float64)], 1)
    r = np.array([8.0, 11.0])
    out = dict(lon=lon, lat=lat, otype=ot, q=qs, r=r)
    for t in range(2):
        ids = np.nonzero(ot == t)[0]
        tree = oracle.RefKdTree(coords[ids])
        for k, q in enumerate(qs):
            d, d2 = tree.range(q, r[t], ordered=True)
            out[f"t{t}_q{k}_ids"] = ids[d].astype(np.int32)
            out[f"t{t}_q{k}_d2"] = d2
    # the same layout as degrees on the sphere (GEOGRAPHIC 1): 3-D trees of
    # the reference's ll2xyz coordinates, radii in km
    glon = (150.0 + 0.5 * lon).astype(np.float32)
    glat = (-10.0 + 0.5 * lat).astype(np.float32)
    gq = np.stack([150.0 + 0.5 * qs[:, 0], -10.0 + 0.5 * qs[:, 1]], 1)
    gr = np.array([450.0, 600.0])
    out.update(g_lon=glon, g_lat=glat, g_q=gq, g_r=gr)
    gxyz = ref_xyz(glon.astype(np.float64), glat.astype(np.float64))
    qxyz = ref_xyz(gq[:, 0], gq[:, 1])
    for t in range(2):
        ids = np.nonzero(ot == t)[0]
        tree = oracle.RefKdTree(gxyz[ids])
        for k in range(len(gq)):
            d, d2 = tree.range(qxyz[k], gr[t], ordered=True)
            out[f"g_t{t}_q{k}_ids"] = ids[d].astype(np.int32)
            out[f"g_t{t}_q{k}_d2"] = d2
    np.savez_compressed(os.path.join(HERE, "nlobsmax.npz"), **out)
    print("nlobsmax:", lon.size, "obs,", len(qs), "queries (2-D and on the sphere)")


def transforms():
    w = synth.make(1, with_fields=False)
    S, s_f, _ = oracle.calcinnandspread(w.HE, w.value, w.status)
    S, s = oracle.standardise(S, s_f, w.estd, w.otype, np.ones(w.ntypes))
    m = w.nmem
    coords = np.stack([w.lon.astype(np.float64), w.lat.astype(np.float64)], 1)
    tree = oracle.RefKdTree(coords)      # one type, all status OK
    rng = np.random.default_rng(11)
    npts = w.nanalyses
    pts = np.sort(rng.choice(npts, 160, replace=False))
    T64 = np.zeros((pts.size, m, m))
    w64 = np.zeros((pts.size, m))
    nl = np.zeros(pts.size, np.int32)
    for k, pt in enumerate(pts):
        jj, ii = divmod(int(pt), w.ni_s)
        q = np.array([w.x[ii * w.stride], w.y[jj * w.stride]])
        d, d2 = tree.range(q, w.locrad)
        lobs = d
        lc = np.array([oracle.taper_gc(np.sqrt(v) / w.locrad) for v in d2])
        nl[k] = lobs.size
        if lobs.size == 0:
            T64[k] = np.eye(m)
            continue
        Sloc = S[:, lobs].astype(np.float64) * lc[None, :]
        sloc = s[lobs] * lc
        ww, T, G = oracle.ref_calc_wT(w.mode, w.scheme, m, m, sloc, Sloc)
        # relaxation to prior with alpha = 1 (transforms.c:1276-1286)
        for e1 in range(m):
            T[e1, e1] -= 1.0
            T[e1, :] *= w.alpha
            T[e1, e1] += 1.0
        T64[k] = T
        w64[k] = ww
    np.savez_compressed(os.path.join(HERE, "transforms.npz"), lon=w.lon, lat=w.lat, otype=w.otype,
                        status=w.status, S=S, s=s, x=w.x, y=w.y, locrad=np.array(w.locrad), pts=pts, T64=T64,
                        w64=w64, nlobs=nl, mode=np.array(w.mode), scheme=np.array(w.scheme),
                        stride=np.array(w.stride))
    print("transforms:", pts.size, "points, mean p", nl.mean())


def ref_traceprod(ta, tb, m, n, A, B, compact=True):
    """traceprod of the reference's calcs.c; A and B row-major blocks, or
    (compact False) lists of row addresses."""
    import ctypes as C
    R = oracle.reflib()
    R.traceprod.restype = C.c_double
    R.traceprod.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_int]
    ra = oracle._rows(A, C.c_double) if compact else A
    rb = oracle._rows(B, C.c_double) if compact else B
    return R.traceprod(ta, tb, m, n, ra, rb, 1 if compact else 0)


def transforms_multitype():
    """das_calctransforms on a sample of points of a two-type workload with
    rejected observations, with the diagnostics of transforms.c:1298-1345:
    local obs from the reference kd-trees (type by type, tree order), the
    reference's taper_gc, calcs.c for w, T and G, relaxation alpha = 0.7,
    then dfs/srf and per-type pdfs/psrf through the reference's traceprod
    (the per-type ones in its row-pointer form), with the float stores of
    the reference's diagnostic arrays."""
    import ctypes as C
    w = synth.make(2, scale=0.1, nobs=6000, with_fields=False, nmem=20)
    st = w.status.copy()
    st[::17] = 1
    S, s_f, _ = oracle.calcinnandspread(w.HE, w.value, st)
    S, s = oracle.standardise(S, s_f, w.estd, w.otype, np.ones(w.ntypes))
    m, alpha = w.nmem, 0.7
    radius = np.array([6.0, 9.0])
    coords = np.stack([w.lon.astype(np.float64), w.lat.astype(np.float64)], 1)
    trees, tids = [], []
    for t in range(w.ntypes):
        ids = np.nonzero((w.otype == t) & (st == 0))[0]
        tids.append(ids)
        trees.append(oracle.RefKdTree(coords[ids]))
    rng = np.random.default_rng(13)
    npts = w.nanalyses
    pts = np.sort(rng.choice(npts, 120, replace=False))
    out = dict(lon=w.lon, lat=w.lat, otype=w.otype, status=st, S=S, s=s, x=w.x, y=w.y, radius=radius,
               stride=np.array(w.stride), pts=pts, alpha=np.array(alpha))
    for mode, scheme, name in ((0, 0, "denkf"), (0, 1, "etkf"), (1, 0, "enoi")):
        T64 = np.zeros((pts.size, m, m))
        w64 = np.zeros((pts.size, m))
        diag = np.zeros((pts.size, 3))              # nlobs, dfs, srf (the stored floats)
        pdiag = np.zeros((pts.size, w.ntypes, 3))   # pnlobs, pdfs, psrf
        for k, pt in enumerate(pts):
            jj, ii = divmod(int(pt), w.ni_s)
            q = np.array([w.x[ii * w.stride], w.y[jj * w.stride]])
            lobs, lc, lt = [], [], []
            for t in range(w.ntypes):
                d, d2 = trees[t].range(q, radius[t])
                lobs += list(tids[t][d])
                lc += [oracle.ref_taper_gc(np.sqrt(v) / radius[t]) for v in d2]
                lt += [t] * d.size
            p = len(lobs)
            if p == 0:
                T64[k] = np.eye(m)
                continue
            lobs, lc = np.array(lobs), np.array(lc)
            Sloc = np.ascontiguousarray(S[:, lobs].astype(np.float64) * lc[None, :])
            sloc = s[lobs] * lc
            ww, T, G = oracle.ref_calc_wT(mode, scheme, m, m, sloc, Sloc)
            if mode != 1:
                for e1 in range(m):
                    T[e1, e1] -= 1.0
                    T[e1, :] *= alpha
                    T[e1, e1] += 1.0
                T64[k] = T
            w64[k] = ww
            G = np.ascontiguousarray(G)
            dfs = np.float32(ref_traceprod(0, 0, p, m, G, Sloc))
            srf = np.float32(np.sqrt(ref_traceprod(0, 1, m, p, Sloc, Sloc) / float(dfs)) - 1.0)
            diag[k] = [p, dfs, srf]
            lt = np.array(lt)
            for t in range(w.ntypes):
                sel = np.nonzero(lt == t)[0]
                if sel.size == 0:
                    continue
                o0, pq = int(sel[0]), sel.size
                gr = (C.c_void_p * pq)(*[G.ctypes.data + (o0 + i) * G.strides[0] for i in range(pq)])
                sr = (C.c_void_p * m)(*[Sloc.ctypes.data + e * Sloc.strides[0] + o0 * 8 for e in range(m)])
                pdfs = np.float32(ref_traceprod(0, 0, pq, m, gr, sr, compact=False))
                psrf = np.float32(np.sqrt(ref_traceprod(0, 1, m, pq, sr, sr, compact=False) / float(pdfs)) - 1.0) \
                    if float(pdfs) > 1.0e-6 else np.float32(0.0)
                pdiag[k, t] = [pq, pdfs, psrf]
        out[f"{name}_T64"] = T64
        out[f"{name}_w64"] = w64
        out[f"{name}_diag"] = diag
        out[f"{name}_pdiag"] = pdiag
    np.savez_compressed(os.path.join(HERE, "transforms_multitype.npz"), **out)
    print("transforms_multitype:", pts.size, "points")


def calctransforms():
    """das_calctransforms of the reference itself (calc/transforms.c with
    calcs.c, observations.c, obstypes.c, kdtree.c, compiled unmodified; grid
    and output files in memory) on a two-type workload with rejected
    observations at stride 3: the float T, w and diagnostics it writes, for
    ETKF with alpha 0.7 and for DEnKF.  S and s are stored standardised."""
    w = synth.make(2, scale=0.1, nobs=6000, with_fields=False, nmem=20)
    st = w.status.copy()
    st[::23] = 1
    S, s_f, _ = oracle.calcinnandspread(w.HE, w.value, st)
    S, s = oracle.standardise(S, s_f, w.estd, w.otype, np.ones(w.ntypes))
    nl, lr, lw = oracle.locrad_table(w.ntypes, 12.0)
    obs = oracle.ObsSet(w.lon, w.lat, w.otype, st, w.ntypes, nl, lr, lw)
    out = dict(lon=w.lon, lat=w.lat, otype=w.otype, status=st, S=S, s=s, x=w.x, y=w.y, locrad=np.array(12.0),
               stride=np.array(w.stride), nmem=np.array(w.nmem))
    for mode, scheme, alpha, name in ((0, 1, 0.7, "etkf"), (0, 0, 1.0, "denkf")):
        r = oracle.ref_calctransforms(obs, mode=mode, scheme=scheme, nmem=w.nmem, nmem_dynamic=w.nmem, alpha=alpha,
                                      stride=w.stride, x=w.x, y=w.y, S=S, s=s)
        out[f"{name}_alpha"] = np.array(alpha)
        for k in ("T", "w", "nlobs", "dfs", "srf", "pnlobs", "pdfs", "psrf"):
            out[f"{name}_{k}"] = r[k]
    np.savez_compressed(os.path.join(HERE, "calctransforms.npz"), **out)
    print("calctransforms:", w.nj_s * w.ni_s, "points")


def model2obs():
    rng = np.random.default_rng(20250)
    ni, nj, nk, m, n = 23, 17, 5, 3, 600
    nl = rng.integers(0, nk + 1, (nj, ni)).astype(np.int32)
    f2 = rng.normal(10.0, 2.0, (m, nj, ni)).astype(np.float32)
    f3 = rng.normal(10.0, 2.0, (m, nk, nj, ni)).astype(np.float32)
    off2 = rng.normal(0.0, 0.5, (nj, ni)).astype(np.float32)
    off1 = rng.normal(0.0, 0.5, nk).astype(np.float32)
    fi = rng.uniform(-0.99, ni + 0.5, n)
    fj = rng.uniform(-0.99, nj + 0.5, n)
    fi[:80] = np.maximum(np.floor(fi[:80]), 0.0)   # on grid lines (-1 fails the reference's assert)
    fj[40:120] = np.maximum(np.floor(fj[40:120]), 0.0)
    fi[120:140] = rng.uniform(-0.99, 0.0, 20)      # below the first column
    fi[140:160] = rng.uniform(ni - 1.0, ni, 20)    # past the last column
    fj[160:180] = rng.uniform(nj - 1.0, nj + 0.5, 20)
    fi[fi == ni] = ni - 0.25                       # the 3-D rule asserts on fi == ni (utils.c:1265)
    fk = rng.uniform(-0.6, nk - 0.4, n).astype(np.float32)
    fk[::7] = np.round(fk[::7])
    out = dict(ni=np.array(ni), nj=np.array(nj), nk=np.array(nk), numlevels=nl, f2=f2, f3=f3, off2=off2, off1=off1,
               fi=fi, fj=fj, fk=fk)
    for per in (0, 1):
        he2 = np.empty((m, n), np.float32)
        for e in range(m):
            v = f2[e] - off2
            for o in range(n):
                he2[e, o] = oracle.ref_interp2d(fi[o], fj[o], v, nl, per)
        out[f"he2_p{per}"] = he2
        for ktop in (0, nk - 1):
            he3 = np.empty((m, n), np.float32)
            for e in range(m):
                v = f3[e] - off1[:, None, None]
                for o in range(n):
                    he3[e, o] = oracle.ref_interp3d(fi[o], fj[o], fk[o], v, nl, ktop, per)
            out[f"he3_p{per}_k{ktop}"] = he3
    np.savez_compressed(os.path.join(HERE, "model2obs.npz"), **out)
    print("model2obs:", n, "positions,", int(np.isnan(out["he2_p0"]).sum()), "all-dry 2-D cases")


# the update cases: (name, mode (0 ENKF, 1 ENOI, 2 HYBRID), nj, ni, m, m_dyn,
# stride, periodic_i, j1, j2 (-1: last row), level, surfk, issurfacevar,
# inflation, inf_ratio, output_increment, applylog)
UPDATE_CASES = [
    ("enkf_s1_infl", 0, 24, 31, 12, 12, 1, 0, 0, -1, 0, 0, 0, 1.05, float("nan"), 0, 0),
    ("enkf_s3_mask_ratio", 0, 37, 44, 16, 16, 3, 0, 0, -1, 1, 0, 0, 1.1, 0.5, 0, 0),
    ("enkf_s2_periodic_tile", 0, 30, 25, 12, 12, 2, 1, 6, 19, 0, 0, 0, 1.0, float("nan"), 0, 0),
    ("enkf_s3_surfk", 0, 28, 34, 12, 12, 3, 0, 3, 20, 2, 4, 0, 1.02, 0.3, 0, 0),
    ("enkf_s3_surfk_surfacevar", 0, 28, 34, 12, 12, 3, 1, 0, -1, 0, 4, 1, 1.0, float("nan"), 0, 0),
    ("enkf_s2_increment", 0, 26, 29, 12, 12, 2, 0, 0, -1, 0, 0, 0, 1.0, float("nan"), 1, 0),
    ("enkf_s2_increment_log", 0, 26, 29, 12, 12, 2, 0, 0, -1, 0, 0, 0, 1.0, float("nan"), 1, 1),
    ("hybrid_s3", 2, 31, 40, 18, 12, 3, 0, 0, -1, 0, 0, 0, 1.04, 0.4, 0, 0),
    ("hybrid_s1_missing_static", 2, 20, 22, 16, 10, 1, 0, 0, -1, 0, 0, 0, 1.0, float("nan"), 0, 0),
    ("enoi_s3", 1, 31, 40, 14, 14, 3, 0, 0, -1, 0, 0, 0, 1.0, float("nan"), 0, 0),
    ("enoi_s2_tile_surfk", 1, 30, 27, 10, 10, 2, 1, 4, 21, 1, 3, 0, 1.0, float("nan"), 0, 0),
    # ensembles above 64 members (the device's warp-per-cell kernel)
    ("enkf_m80_s3_mask_ratio", 0, 13, 13, 80, 80, 3, 0, 0, -1, 1, 0, 0, 1.1, 0.5, 0, 0),
    ("hybrid_m72_s2_periodic_tile", 2, 11, 13, 72, 48, 2, 1, 2, 9, 0, 0, 0, 1.03, 0.3, 0, 0),
    ("enkf_m96_s1_increment_log", 0, 6, 7, 96, 96, 1, 0, 0, -1, 0, 2, 0, 1.0, float("nan"), 1, 1),
]


def update():
    rng = np.random.default_rng(20260)
    out = {"names": np.array([c[0] for c in UPDATE_CASES])}
    for k, (name, mode, mnj, mni, m, md, stride, per, j1, j2, level, surfk, issv, infl, ratio, inc,
            alog) in enumerate(UPDATE_CASES):
        nj = (mnj - 1) // stride + 1
        ni = (mni - 1) // stride + 1
        j2 = mnj - 1 if j2 < 0 else j2
        jsize = j2 - j1 + 1
        # transforms near the identity (ETKF-like) and small mean weights
        T = (np.eye(m, dtype=np.float64)[None, None, :md, :] +
             0.15 * rng.standard_normal((nj, ni, md, m))).astype(np.float32)
        w = (0.08 * rng.standard_normal((nj, ni, m))).astype(np.float32)
        nk = 5
        numlevels = rng.integers(0, nk + 1, (mnj, mni)).astype(np.int32)
        numlevels[rng.random((mnj, mni)) < 0.55] = nk
        base = 15.0 + 2.0 * np.sin(np.arange(mni)[None, :] / 5.0) * np.cos(np.arange(mnj)[:, None] / 7.0)
        rows = m + 1 if mode == 1 else m
        v = (base[None, j1:j2 + 1, :] + rng.standard_normal((rows, jsize, mni))).astype(np.float32)
        if alog:
            v = np.log10(np.abs(v) + 1.0).astype(np.float32)
        if mode == 2:
            # the hybrid ensemble as das_update builds it before the update
            flat = v.reshape(m, -1)
            hv, vmean = oracle.ref_sethybridensemble(flat, md, 0.5)
            out[f"u{k}_hyb_in"] = flat.copy()
            out[f"u{k}_hyb_out"] = hv.copy()
            out[f"u{k}_hyb_mean"] = vmean
            v = hv.reshape(m, jsize, mni).copy()
        # missing values: a dynamic member's NaN, a value above MAXOBSVAL,
        # a static member's missing value (hybrid), a missing background
        cells = rng.integers(0, [jsize, mni], (4, 2))
        v[0, cells[0, 0], cells[0, 1]] = np.nan
        v[min(1, rows - 1), cells[1, 0], cells[1, 1]] = 2.0e6
        if mode == 2:
            v[m - 1, cells[2, 0], cells[2, 1]] = -3.0e6
        if mode == 1:
            v[m, cells[3, 0], cells[3, 1]] = 5.0e6
        res = oracle.ref_update_layer(v, None if mode == 1 else T, w, numlevels, mode=mode, nmem=m, nmem_dynamic=md,
                                      stride=stride, periodic_i=per, level=level, surfk=surfk, issurfacevar=issv,
                                      inflation=infl, inf_ratio=ratio, output_increment=inc, applylog=alog, j1=j1,
                                      j2=j2)
        out[f"u{k}_prm"] = np.array([mode, mnj, mni, m, md, stride, per, j1, j2, level, surfk, issv, inc, alog],
                                    np.int32)
        out[f"u{k}_infl"] = np.array([infl, ratio])
        out[f"u{k}_T"] = T
        out[f"u{k}_w"] = w
        out[f"u{k}_numlevels"] = numlevels
        out[f"u{k}_v"] = v
        out[f"u{k}_out"] = res
    np.savez_compressed(os.path.join(HERE, "update.npz"), **out)
    print("update:", len(UPDATE_CASES), "cases")


# (name, mode, mnj, mni, m, md, stride, periodic, inc, alog, deflation, sigma, seed)
NOISE_CASES = [
    ("enkf_m10_s1", 0, 14, 17, 10, 10, 1, 0, 0, 0, 0.9, 0.4, 11),
    ("enkf_m11_s2_periodic", 0, 15, 16, 11, 11, 2, 1, 0, 0, 0.6, 1.5, 12),
    ("hybrid_m12_s3", 2, 16, 19, 12, 8, 3, 0, 0, 0, 0.95, 0.2, 13),
    ("enkf_m10_increment", 0, 12, 13, 10, 10, 2, 0, 1, 0, 0.8, 0.3, 14),
    ("enkf_m24_log", 0, 13, 15, 24, 24, 1, 0, 0, 1, 0.7, 0.1, 15),
]


def addnoise():
    rng = np.random.default_rng(20261)
    out = {"names": np.array([c[0] for c in NOISE_CASES])}
    for k, (name, mode, mnj, mni, m, md, stride, per, inc, alog, defl, sigma, seed) in enumerate(NOISE_CASES):
        nj = (mnj - 1) // stride + 1
        ni = (mni - 1) // stride + 1
        T = (np.eye(m, dtype=np.float64)[None, None, :md, :] +
             0.15 * rng.standard_normal((nj, ni, md, m))).astype(np.float32)
        w = (0.08 * rng.standard_normal((nj, ni, m))).astype(np.float32)
        numlevels = np.full((mnj, mni), 4, np.int32)
        numlevels[rng.random((mnj, mni)) < 0.2] = 0
        v = (15.0 + rng.standard_normal((m, mnj, mni))).astype(np.float32)
        if alog:
            v = np.log10(np.abs(v) + 1.0).astype(np.float32)
        if mode == 2:
            v = oracle.ref_sethybridensemble(v.reshape(m, -1), md, 0.5)[0].reshape(m, mnj, mni).copy()
        res, r = oracle.ref_update_layer_noise(v, T, w, numlevels, deflation=defl, sigma=sigma, seed=seed, mode=mode,
                                               nmem=m, nmem_dynamic=md, stride=stride, periodic_i=per,
                                               output_increment=inc, applylog=alog)
        plain = oracle.ref_update_layer(v, T, w, numlevels, mode=mode, nmem=m, nmem_dynamic=md, stride=stride,
                                        periodic_i=per, output_increment=inc, applylog=alog)
        out[f"n{k}_prm"] = np.array([mode, mnj, mni, m, md, stride, per, inc, alog], np.int32)
        out[f"n{k}_noise"] = np.array([defl, sigma])
        out[f"n{k}_random"] = r
        out[f"n{k}_T"] = T
        out[f"n{k}_w"] = w
        out[f"n{k}_numlevels"] = numlevels
        out[f"n{k}_v"] = v
        out[f"n{k}_plain"] = plain
        out[f"n{k}_out"] = res
    np.savez_compressed(os.path.join(HERE, "addnoise.npz"), **out)
    print("addnoise:", len(NOISE_CASES), "cases")


if __name__ == "__main__":
    oracle.build()
    if (oracle.reflib() is None or oracle.reflib_utils() is None or oracle.reflib_update() is None
            or oracle.reflib_transforms() is None):
        sys.exit("the reference libraries under oracle/_ref could not be built")
    which = sys.argv[1:] or ["numerics", "kdtree", "nlobsmax", "transforms", "transforms_multitype", "calctransforms",
                             "model2obs", "update", "addnoise"]
    for name in which:
        {"numerics": numerics, "kdtree": kdtree, "nlobsmax": nlobsmax, "transforms": transforms,
         "transforms_multitype": transforms_multitype, "calctransforms": calctransforms, "model2obs": model2obs,
         "update": update, "addnoise": addnoise}[name]()
