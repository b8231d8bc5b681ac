"""Parity of the plain FP64 transform path at every register-block size the
kernels instantiate, on the workload shapes the path runs, with local
observation counts in the thousands; and the geographic (lon/lat, 3-D search
on the sphere) form of the search and the transforms.

Tolerances (the plain FP64 contract): double T and w within 1e-10 relative
per point (max |a - b| / max |b|) of the FP64 oracle; local-observation counts
bit-exact; dfs within 1e-6.

The FP64 kernels are templated on R, the register block of the S'S tile: R =
ceil(m / 16), so m = 48, 64, 96 and 144 run R = 3, 4, 6 and 9.  Each case runs
the plain path (one CTA per point, with per-type diagnostics, so the solve
stays in the transform kernel) and the batched path (persistent kernel over
the size-sorted queue, no diagnostics, so the batched eigensolver / inverse
finishes the points).
"""
import numpy as np
import pytest

import oracle
import synth
from helpers import gpu_setup, obsset, prepare, rel

pytestmark = pytest.mark.gpu


def per_point_rel(a, b):
    a = a.reshape(a.shape[0] * a.shape[1], -1)
    b = b.reshape(b.shape[0] * b.shape[1], -1)
    den = np.maximum(np.abs(b).max(axis=1), 1e-300)
    return float((np.abs(a - b).max(axis=1) / den).max())


# (name, workload, scale, m, m_dyn, mode (0 ENKF, 1 ENOI, 2 HYBRID), scheme (0 DEnKF, 1 ETKF), rows compared)
CASES = [
    ("R3_m48_denkf_swaths", 2, 0.2, 48, 48, 0, 0, None),
    ("R3_m48_etkf_swaths", 2, 0.2, 48, 48, 0, 1, None),
    ("R3_m48_enoi_swaths", 2, 0.2, 48, 48, 1, 0, None),
    ("R4_m64_denkf_swaths", 2, 0.2, 64, 64, 0, 0, None),
    ("R4_m64_etkf_swaths", 2, 0.2, 64, 64, 0, 1, None),
    ("R6_m96_etkf_dense", 3, 0.1, 96, 96, 0, 1, 10),
    ("R6_m96_denkf_dense", 3, 0.1, 96, 96, 0, 0, 10),
    ("R6_m96_enoi_dense", 3, 0.1, 96, 96, 1, 0, 10),
    ("R9_m144_etkf_hybrid", 3, 0.1, 144, 96, 2, 1, 6),
    ("R9_m144_denkf", 3, 0.1, 144, 144, 0, 0, 6),
]


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_fp64_register_blocks_large_p(ctx, case):
    name, cfg, scale, m, md, mode, scheme, nrows = case
    w = synth.make(cfg, scale=scale, nmem=m, with_fields=False)
    w.nmem_dynamic = md
    S, s = prepare(w)
    obs, tabs = obsset(w)
    rows = None if nrows is None else [int(r) for r in np.linspace(0, w.nj_s - 1, nrows).astype(int)]
    ref = oracle.calctransforms(obs, mode=mode, scheme=scheme, nmem=m, nmem_dynamic=md, alpha=1.0,
                                stride=w.stride, x=w.x, y=w.y, S=S, s=s, rows=rows, threads=16, want64=True)
    sel = slice(None) if rows is None else rows
    nl = ref["nlobs"][sel]
    assert nl.max() >= 2500, f"{name}: local counts reach only {nl.max()}"
    gpu_setup(ctx, w, S, s, tabs)
    for path, diag in ((0, True), (1, False)):
        out = ctx.calctransforms(mode=mode, scheme=scheme, alpha=1.0, path=path, want64=True, want_diag=diag)
        if diag:
            assert np.array_equal(out["nlobs"][sel], nl), name
            assert rel(out["dfs"][sel], ref["dfs"][sel]) < 1e-6, name
        if mode != 1:
            e = per_point_rel(out["T64"][sel], ref["T64"][sel])
            assert e < 1e-10, (name, path, "T", e)
        e = per_point_rel(out["w64"][sel], ref["w64"][sel])
        assert e < 1e-10, (name, path, "w", e)


def geographic_workload(nobs, lon0, lon1, lat0, lat1, step, seed):
    """Observations uniform in lon/lat (degrees) over a box and a regular
    lon/lat grid of the given step; the reference's GEOGRAPHIC 1 form
    (grid/gridprm.c:95): distances on the sphere through ll2xyz."""
    rng = np.random.default_rng(seed)
    lon = rng.uniform(lon0, lon1, nobs).astype(np.float32)
    lat = rng.uniform(lat0, lat1, nobs).astype(np.float32)
    x = np.arange(lon0, lon1 + 1e-9, step)
    y = np.arange(lat0, lat1 + 1e-9, step)
    return lon, lat, x, y


@pytest.mark.parametrize("scheme", [1, 0])
def test_geographic_lists_and_transforms(ctx, scheme):
    """GEOGRAPHIC 1: observations and grid in degrees, a box that crosses
    the 180th meridian, radius in km; two observation types with different
    radii.  Lists bit-exact (ids and taper coefficients) against the
    oracle's 3-D kd-tree search, T and w within 1e-10."""
    m = 24
    lon, lat, x, y = geographic_workload(6000, 160.0, 200.0, -30.0, 5.0, 1.0, 77)
    n = lon.size
    otype = (np.arange(n) >= n // 2).astype(np.int16)
    rng = np.random.default_rng(5)
    HE = (15.0 + rng.standard_normal((m, n))).astype(np.float32)
    value = (15.0 + rng.standard_normal(n)).astype(np.float32)
    status = np.zeros(n, np.int16)
    status[::29] = 1
    estd = rng.uniform(0.3, 0.8, n).astype(np.float32)
    S, s_f, _ = oracle.calcinnandspread(HE, value, status)
    S, s = oracle.standardise(S, s_f, estd, otype, np.ones(2))
    nl, lr, lw = oracle.locrad_table(2, [[400.0], [250.0, 600.0]], [[1.0], [0.7, 0.3]])
    obs = oracle.ObsSet(lon, lat, otype, status, 2, nl, lr, lw, geographic=True)
    ref = oracle.calctransforms(obs, mode=0, scheme=scheme, nmem=m, nmem_dynamic=m, alpha=1.0, stride=2, x=x, y=y,
                                S=S, s=s, threads=16, want64=True)
    ctx.set_obstypes(nl, lr, lw, np.ones(2), geographic=True)
    ctx.set_obs(lon, lat, otype, status, estd, value)
    ctx.set_S(S, s, m)
    ctx.set_grid(x, y, stride=2)
    counts, offsets, ids, coeffs = ctx.findlocal(lists=True)
    nj_s, ni_s = (y.size - 1) // 2 + 1, (x.size - 1) // 2 + 1
    assert counts.max() > 100
    for pt in range(nj_s * ni_s):
        jj, ii = divmod(pt, ni_s)
        rid, rlc = obs.findlocal(x[ii * 2], y[jj * 2])
        order = np.argsort(rid, kind="stable")
        a, b = offsets[pt], offsets[pt + 1]
        assert np.array_equal(ids[a:b], rid[order]), pt
        assert np.array_equal(coeffs[a:b], rlc[order]), pt
    for path in (0, 1):
        out = ctx.calctransforms(mode=0, scheme=scheme, alpha=1.0, path=path, want64=True)
        assert np.array_equal(out["nlobs"], ref["nlobs"])
        assert per_point_rel(out["T64"], ref["T64"]) < 1e-10
        assert per_point_rel(out["w64"], ref["w64"]) < 1e-10
        assert rel(out["dfs"], ref["dfs"]) < 1e-6
