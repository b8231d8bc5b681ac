"""The CPU oracle, pinned against the reference.

Golden fixtures (tests/golden/*.npz) were produced by the reference's own
calc/calcs.c and common/kdtree.c (see tests/golden/make_golden.py).  Where the
reference library is built in this checkout (oracle/_ref), the oracle is also
compared with it directly on fresh random cases.
"""
import os

import numpy as np
import pytest

import oracle

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)) if b.size else 0.0


def test_taper_known_values():
    # Gaspari & Cohn (1999) eq. 4.10 with support 2c, here c = 1/2 of the radius
    assert oracle.taper_gc(0.0) == 1.0
    assert abs(oracle.taper_gc(0.5) - 5.0 / 24.0) < 1e-15
    assert oracle.taper_gc(1.0) == 0.0
    assert oracle.taper_gc(1.5) == 0.0
    xs = np.linspace(0, 1, 1001)
    v = np.array([oracle.taper_gc(x) for x in xs])
    assert np.all(np.diff(v) <= 1e-15) and np.all(v >= 0)
    # continuity across the two pieces
    assert abs(oracle.taper_gc(0.5 - 1e-12) - oracle.taper_gc(0.5 + 1e-12)) < 1e-10


def test_numerics_against_reference_golden():
    g = np.load(os.path.join(GOLD, "numerics.npz"))
    for k in range(int(g["ncases"])):
        c = {key[len(f"c{k}_"):]: g[key] for key in g.files if key.startswith(f"c{k}_")}
        m, mout, mode, scheme = int(c["m"]), int(c["mout"]), int(c["mode"]), int(c["scheme"])
        w, T, G = oracle.calc_wT(mode, scheme, m, mout, c["s"], c["S"])
        assert rel(w, c["w"]) < 1e-12, (k, rel(w, c["w"]))
        if mode != 1:
            assert rel(T[:mout], c["T"]) < 1e-12, (k, rel(T[:mout], c["T"]))
        assert rel(G, c["G"]) < 1e-12


def test_kdtree_against_reference_golden():
    g = np.load(os.path.join(GOLD, "kdtree.npz"))
    ntypes = int(g["otype"].max()) + 1
    nl, lr, lw = oracle.locrad_table(ntypes, [[float(r)] for r in g["r"]])
    obs = oracle.ObsSet(g["lon"], g["lat"], g["otype"], np.zeros(g["lon"].size, np.int16), ntypes, nl, lr, lw)
    for k, q in enumerate(g["q"]):
        ids, lc = obs.findlocal(q[0], q[1])
        ref_ids = np.concatenate([g[f"t{t}_q{k}_ids"] for t in range(ntypes)])
        ref_d2 = np.concatenate([g[f"t{t}_q{k}_d2"] for t in range(ntypes)])
        # same set, same (type, depth-first) order
        assert np.array_equal(ids, ref_ids), k
        rr = np.concatenate([np.full(g[f"t{t}_q{k}_ids"].size, g["r"][t]) for t in range(ntypes)])
        ref_lc = np.array([oracle.taper_gc(np.sqrt(d) / r) for d, r in zip(ref_d2, rr)])
        assert np.array_equal(lc, ref_lc)


@pytest.mark.parametrize("nmax", [(1, 1), (7, 3), (25, 40), (60, 1000)])
def test_nlobsmax_against_reference_golden(nmax):
    """NLOBSMAX: per type, the first nlobsmax of the reference's distance-sorted
    range results (kd_findnodeswithinrange, ordered = 1), in that order."""
    g = np.load(os.path.join(GOLD, "nlobsmax.npz"))
    nl, lr, lw = oracle.locrad_table(2, [[float(r)] for r in g["r"]])
    n = g["lon"].size
    obs = oracle.ObsSet(g["lon"], g["lat"], g["otype"], np.zeros(n, np.int16), 2, nl, lr, lw, nlobsmax=np.array(nmax))
    cut = 0
    for k, q in enumerate(g["q"]):
        ids, _ = obs.findlocal(q[0], q[1])
        ref = [g[f"t{t}_q{k}_ids"][:nmax[t]] for t in range(2)]
        assert np.array_equal(ids, np.concatenate(ref)), k
        cut += sum(g[f"t{t}_q{k}_ids"].size > nmax[t] for t in range(2))
    if nmax[1] < 1000:
        assert cut > 0


@pytest.mark.parametrize("nmax", [(1, 1), (7, 3), (25, 40)])
def test_nlobsmax_on_the_sphere_against_reference_golden(nmax):
    """NLOBSMAX with GEOGRAPHIC 1: the oracle's 3-D search against the
    reference's distance-sorted kd search on the reference's own ll2xyz
    coordinates (radii in km)."""
    g = np.load(os.path.join(GOLD, "nlobsmax.npz"))
    nl, lr, lw = oracle.locrad_table(2, [[float(r)] for r in g["g_r"]])
    n = g["g_lon"].size
    obs = oracle.ObsSet(g["g_lon"], g["g_lat"], g["otype"], np.zeros(n, np.int16), 2, nl, lr, lw,
                        nlobsmax=np.array(nmax), geographic=True)
    for k, q in enumerate(g["g_q"]):
        ids, _ = obs.findlocal(q[0], q[1])
        ref = [g[f"g_t{t}_q{k}_ids"][:nmax[t]] for t in range(2)]
        assert np.array_equal(ids, np.concatenate(ref)), k


@pytest.mark.parametrize("case", [(0, 0, "denkf"), (0, 1, "etkf"), (1, 0, "enoi")])
def test_transforms_multitype_against_reference_golden(case):
    """Two observation types, rejected observations, alpha 0.7: T and w
    within 1e-12 of the reference's own search, taper and calcs.c, and the
    stored diagnostics (nlobs, dfs, srf and per type pnlobs, pdfs, psrf)
    equal to the reference's float values within one float ulp
    (tests/golden/transforms_multitype.npz)."""
    mode, scheme, name = case
    g = np.load(os.path.join(GOLD, "transforms_multitype.npz"))
    nl, lr, lw = oracle.locrad_table(2, [[float(r)] for r in g["radius"]])
    obs = oracle.ObsSet(g["lon"], g["lat"], g["otype"], g["status"], 2, nl, lr, lw)
    m = g["S"].shape[0]
    out = oracle.calctransforms(obs, mode=mode, scheme=scheme, nmem=m, nmem_dynamic=m, alpha=float(g["alpha"]),
                                stride=int(g["stride"]), x=g["x"], y=g["y"], S=g["S"], s=g["s"], want64=True,
                                threads=8)
    ni = out["w"].shape[1]
    T64, w64 = g[f"{name}_T64"], g[f"{name}_w64"]
    diag, pdiag = g[f"{name}_diag"], g[f"{name}_pdiag"]

    def ulps(a, b):
        a, b = np.float32(a), np.float32(b)
        return abs(float(a) - float(b)) / float(np.spacing(max(abs(a), abs(b), np.float32(1e-30))))

    for k, pt in enumerate(g["pts"]):
        jj, ii = divmod(int(pt), ni)
        if mode != 1:
            assert rel(out["T64"][jj, ii], T64[k]) < 1e-12, (name, k)
        if np.abs(w64[k]).max() > 0:
            assert rel(out["w64"][jj, ii], w64[k]) < 1e-12, (name, k)
        assert out["nlobs"][jj, ii] == diag[k, 0], (name, k)
        if diag[k, 0] > 0:
            assert ulps(out["dfs"][jj, ii], diag[k, 1]) <= 1, (name, k)
            assert ulps(out["srf"][jj, ii], diag[k, 2]) <= 1, (name, k)
        for t in range(2):
            assert out["pnlobs"][t, jj, ii] == pdiag[k, t, 0], (name, k, t)
            if pdiag[k, t, 0] > 0:
                assert ulps(out["pdfs"][t, jj, ii], pdiag[k, t, 1]) <= 1, (name, k, t)
                assert ulps(out["psrf"][t, jj, ii], pdiag[k, t, 2]) <= 1, (name, k, t)


def test_addnoise_against_reference_golden():
    """RANDOMISE: the oracle's addnoise of the reference's plain update equals
    the reference's randomised update bit for bit (tests/golden/addnoise.npz,
    from update.c with DEFLATION and SIGMA set)."""
    g = np.load(os.path.join(GOLD, "addnoise.npz"))
    for k, name in enumerate(g["names"]):
        m = int(g[f"n{k}_prm"][3])
        defl, sigma = [float(x) for x in g[f"n{k}_noise"]]
        got = oracle.addnoise(g[f"n{k}_plain"], defl, sigma, g[f"n{k}_random"][:m])
        assert np.array_equal(got, g[f"n{k}_out"], equal_nan=True), name
        assert not np.array_equal(got, g[f"n{k}_plain"]), name


def test_transforms_against_reference_golden():
    g = np.load(os.path.join(GOLD, "transforms.npz"))
    nl, lr, lw = oracle.locrad_table(1, float(g["locrad"]))
    obs = oracle.ObsSet(g["lon"], g["lat"], g["otype"], g["status"], 1, nl, lr, lw)
    m = g["S"].shape[0]
    out = oracle.calctransforms(obs, mode=int(g["mode"]), scheme=int(g["scheme"]), nmem=m, nmem_dynamic=m, alpha=1.0,
                                stride=int(g["stride"]), x=g["x"], y=g["y"], S=g["S"], s=g["s"], want64=True)
    ni = out["w"].shape[1]
    for k, pt in enumerate(g["pts"]):
        jj, ii = divmod(int(pt), ni)
        assert out["nlobs"][jj, ii] == g["nlobs"][k]
        assert rel(out["T64"][jj, ii], g["T64"][k]) < 1e-12
        assert rel(out["w64"][jj, ii], g["w64"][k]) < 1e-12 or np.abs(g["w64"][k]).max() == 0.0


@pytest.mark.skipif(oracle.reflib() is None, reason="reference library not built here")
def test_oracle_equals_reference_build():
    rng = np.random.default_rng(5)
    for (m, mout, p) in [(24, 24, 200), (24, 24, 3), (64, 48, 64), (96, 96, 500)]:
        S = rng.standard_normal((m, p)) * 0.2
        s = rng.standard_normal(p)
        for mode, scheme in [(0, 1), (0, 0), (1, 0)]:
            a = oracle.calc_wT(mode, scheme, m, mout, s, S)
            b = oracle.ref_calc_wT(mode, scheme, m, mout, s, S)
            for x, y in zip(a, b):
                assert np.array_equal(x, y)


@pytest.mark.skipif(oracle.reflib() is None, reason="reference library not built here")
def test_kdtree_equals_reference_build_random():
    rng = np.random.default_rng(9)
    lon = rng.uniform(0, 100, 4000).astype(np.float32)
    lat = rng.uniform(0, 60, 4000).astype(np.float32)
    nl, lr, lw = oracle.locrad_table(1, [[7.5, 3.0]], [[0.7, 0.3]])
    obs = oracle.ObsSet(lon, lat, np.zeros(4000, np.int16), np.zeros(4000, np.int16), 1, nl, lr, lw)
    tree = oracle.RefKdTree(np.stack([lon.astype(np.float64), lat.astype(np.float64)], 1))
    for q in rng.uniform(0, 100, (30, 2)):
        ids, _ = obs.findlocal(q[0], q[1])
        d, _ = tree.range(q, 7.5)
        assert np.array_equal(ids, d)


def test_innovations_and_standardise_semantics():
    rng = np.random.default_rng(3)
    m, n = 10, 50
    HE = (rng.standard_normal((m, n)) + 5).astype(np.float32)
    value = rng.standard_normal(n).astype(np.float32) + 5
    status = np.zeros(n, np.int16)
    status[3] = 1
    S, s_f, std_f = oracle.calcinnandspread(HE, value, status)
    mean = HE.astype(np.float64).sum(0) / m
    assert np.allclose(S, HE - mean.astype(np.float32)[None], atol=0)
    ok = status == 0
    assert np.allclose(s_f[ok], value[ok] - mean[ok])
    assert s_f[3] == mean[3]            # non-OK obs keep the mean (ensobs.c:605)
    estd = np.full(n, 0.5, np.float32)
    S2, s2 = oracle.standardise(S, s_f, estd, np.zeros(n, np.int16), np.array([4.0]))
    den = 0.5 * 2.0 * np.sqrt(m - 1.0)
    assert np.array_equal(S2, (S.astype(np.float64) / den).astype(np.float32))
    assert np.array_equal(s2, s_f / den)


def test_update_identity_transform_keeps_fields():
    rng = np.random.default_rng(1)
    m, mnj, mni, stride = 8, 7, 9, 2
    nj, ni = (mnj - 1) // stride + 1, (mni - 1) // stride + 1
    T = np.broadcast_to(np.eye(m, dtype=np.float32), (nj, ni, m, m)).copy()
    w = np.zeros((nj, ni, m), np.float32)
    v = (rng.standard_normal((m, mnj, mni)) + 3).astype(np.float32)
    nl = np.ones((mnj, mni), np.int32)
    out = oracle.updatefields(v, T, w, nl, mode=0, nmem=m, nmem_dynamic=m, stride=stride)
    assert np.allclose(out, v, atol=2e-6)
    nl[2, 3] = 0
    out = oracle.updatefields(v, T, w, nl, mode=0, nmem=m, nmem_dynamic=m, stride=stride)
    assert np.all(out[:, 2, 3] == 0.0)


def test_hybrid_semantics():
    rng = np.random.default_rng(2)
    v = rng.standard_normal((10, 30)).astype(np.float32)
    out, mean = oracle.sethybridensemble(v, 6, 0.5)
    assert np.allclose(mean, v[:6].astype(np.float64).mean(0))
    k_d = np.sqrt(9.0 / 5.0)
    assert np.allclose(out[:6], (v[:6] - mean) * k_d + mean, atol=1e-5)


# ---------------------------------------------------------------------------
# forward operator (calc/model2obs.c; common/utils.c interpolation)
# ---------------------------------------------------------------------------

def same_bits(a, b):
    """float32 arrays equal bit for bit, any NaN matching any NaN."""
    a = np.asarray(a, np.float32)
    b = np.asarray(b, np.float32)
    na, nb = np.isnan(a), np.isnan(b)
    return bool(np.array_equal(na, nb) and np.array_equal(a[~na].view(np.uint32), b[~nb].view(np.uint32)))


def test_model2obs_against_reference_golden():
    g = np.load(os.path.join(GOLD, "model2obs.npz"))
    nk = int(g["nk"])
    m, n = g["he2_p0"].shape
    ids = np.arange(n, dtype=np.int32)
    for per in (0, 1):
        HE = np.full((m, n), np.nan, np.float32)
        for e in range(m):
            assert oracle.map_obs(HE, e, g["f2"][e], g["numlevels"], ids, g["fi"], g["fj"], periodic_i=per,
                                  offset=g["off2"], offset_kind=2, skip_bad=True) == 0
        assert same_bits(HE, g[f"he2_p{per}"]), f"2-D periodic={per}"
        for ktop in (0, nk - 1):
            HE = np.full((m, n), np.nan, np.float32)
            for e in range(m):
                assert oracle.map_obs(HE, e, g["f3"][e], g["numlevels"], ids, g["fi"], g["fj"], g["fk"],
                                      three_d=True, ktop=ktop, periodic_i=per, offset=g["off1"], offset_kind=1,
                                      skip_bad=True) == 0
            assert same_bits(HE, g[f"he3_p{per}_k{ktop}"]), f"3-D periodic={per} ktop={ktop}"


@pytest.mark.skipif(oracle.reflib_utils() is None, reason="reference library not built here")
def test_interpolation_equals_reference_build_random():
    rng = np.random.default_rng(7)
    nj, ni, nk = 9, 11, 5
    v = rng.standard_normal((nk, nj, ni)).astype(np.float32)
    nl = rng.integers(0, nk + 1, (nj, ni)).astype(np.int32)
    for t in range(1500):
        fi = rng.uniform(-0.999, ni + 0.5)
        fj = rng.uniform(-0.999, nj + 0.5)
        if t % 7 == 0:
            fi = float(rng.integers(0, ni))
        if t % 11 == 0:
            fj = float(rng.integers(0, nj))
        fk = rng.uniform(-0.5, nk - 0.5) if t % 5 else float(rng.integers(0, nk))
        for per in (0, 1):
            a = oracle.ref_interp2d(fi, fj, v[0], nl, per)
            b, bad = oracle.interp2d(fi, fj, v[0], nl, per)
            assert not bad and same_bits(a, b), (fi, fj, per)
            if fi == ni:
                continue
            for ktop in (0, nk - 1):
                a = oracle.ref_interp3d(fi, fj, fk, v, nl, ktop, per)
                b, bad = oracle.interp3d(fi, fj, fk, v, nl, ktop, per)
                assert not bad and same_bits(a, b), (fi, fj, fk, ktop, per)


@pytest.mark.skipif(oracle.reflib_utils() is None, reason="reference library not built here")
def test_taper_equals_reference_build():
    # the reference asserts 0 <= x <= 1 + 1e-8 (utils.c:1428)
    for x in np.concatenate([np.linspace(0.0, 1.0, 2001), np.random.default_rng(3).uniform(0, 1, 500)]):
        assert oracle.taper_gc(x) == oracle.ref_taper_gc(x)


def test_map_obs_positions_off_grid_and_bad_forecasts():
    nj, ni = 6, 7
    f = np.full((nj, ni), 5.0, np.float32)
    nl = np.ones((nj, ni), np.int32)
    fi = np.array([1.5, -1.0, 2.0, np.nan])
    fj = np.array([1.5, 2.0, -1.5, 1.0])
    HE = np.full((1, 4), np.nan, np.float32)
    # positions at or below -1 and NaN are off the grid: -(1 + id) of the first
    assert oracle.map_obs(HE, 0, f, nl, np.array([0, 1]), fi, fj) == -2
    assert oracle.map_obs(HE, 0, f, nl, np.array([2]), fi, fj) == -3
    assert oracle.map_obs(HE, 0, f, nl, np.array([3]), fi, fj) == -4
    # a huge value: 1 + id, or NaN with skip_bad
    f[1, 1] = 5e6
    HE[:] = np.nan
    assert oracle.map_obs(HE, 0, f, nl, np.array([0]), fi, fj) == 1
    assert oracle.map_obs(HE, 0, f, nl, np.array([0]), fi, fj, skip_bad=True) == 0 and np.isnan(HE[0, 0])
    # all corners dry: 0/0 is not finite, a bad forecast
    f[1, 1] = 5.0
    nl[1:3, 1:3] = 0
    assert oracle.map_obs(HE, 0, f, nl, np.array([0]), fi, fj) == 1


def test_finish_HE_semantics():
    rng = np.random.default_rng(11)
    m, md, n = 10, 6, 200
    HE = rng.normal(3.0, 1.0, (m, n)).astype(np.float32)
    Hx = rng.normal(3.0, 1.0, n).astype(np.float32)
    st = np.zeros(n, np.int16)
    # EnOI: members recentred on the background, anomalies kept
    S, st2, nbad = oracle.finish_HE(HE, st, mode=1, nmem_dynamic=m, Hx=Hx)
    assert nbad == 0
    assert np.allclose(S.mean(0), Hx, atol=1e-5)
    assert np.allclose(S - S.mean(0), HE - HE.mean(0), atol=1e-5)
    # hybrid: dynamic anomalies x k_d, static anomalies x k_s, all about the dynamic mean
    g = 0.5
    S, _, _ = oracle.finish_HE(HE, st, mode=2, nmem_dynamic=md, gamma=g)
    md_mean = HE[:md].astype(np.float64).mean(0)
    kd = np.sqrt((m - 1) / (md - 1))
    ks = np.sqrt(g * (m - 1) / (m - md - 1))
    assert np.allclose(S[:md], (HE[:md] - md_mean) * kd + md_mean, atol=1e-5)
    assert np.allclose(S[md:], (HE[md:] - HE[md:].astype(np.float64).mean(0)) * ks + md_mean, atol=1e-5)
    # bad forecasts: a NaN in any member (or in Hx for EnOI) marks STATUS_BADFC (10)
    HE[3, 5] = np.nan
    Hx[7] = np.nan
    st[9] = 2
    S, st2, nbad = oracle.finish_HE(HE, st, mode=1, nmem_dynamic=m, Hx=Hx, skip_bad=True)
    assert nbad == 2 and st2[5] == 10 and st2[7] == 10 and st2[9] == 2
    S, st2, nbad = oracle.finish_HE(HE, st, mode=0, nmem_dynamic=m, skip_bad=False)
    assert nbad == 0 and st2[5] == 0


@pytest.mark.skipif(oracle.reflib() is None, reason="reference library not built here")
def test_traceprod_equals_reference_build():
    """The diagnostics' traceprod (calc/calcs.c:41-97): the oracle's, on
    contiguous blocks, equals the reference's compiled one bit for bit in the
    compact form (dfs, srf) and in the row-pointer form the per-type pdfs and
    psrf use (transforms.c:1330-1335), for the operand orders those use."""
    import ctypes as C
    L, R = oracle.lib(), oracle.reflib()
    L.or_traceprod.restype = C.c_double
    L.or_traceprod.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p]
    R.traceprod.restype = C.c_double
    R.traceprod.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_int]
    rng = np.random.default_rng(12)
    for (p, m) in [(7, 24), (60, 24), (300, 48), (5, 96)]:
        G = rng.standard_normal((p, m))        # G[o][e]
        S = rng.standard_normal((m, p))        # S[e][o]
        # dfs = traceprod(0, 0, p, m, G, S), srf: traceprod(0, 1, m, p, S, S)
        for ta, tb, mm, nn, A, B in ((0, 0, p, m, G, S), (0, 1, m, p, S, S)):
            want = L.or_traceprod(ta, tb, mm, nn, A.ctypes.data, B.ctypes.data)
            ra, rb = oracle._rows(A, C.c_double), oracle._rows(B, C.c_double)
            assert R.traceprod(ta, tb, mm, nn, ra, rb, 1) == want
        # a type's sub-block in the row-pointer form: rows of G from o0,
        # member rows of S from column o0 (a wider matrix underneath)
        o0, q = p // 3, max(1, p // 2)
        Gw, Sw = rng.standard_normal((p + 4, m)), rng.standard_normal((m, p + 9))
        pG = Gw[o0:o0 + q]
        pS = Sw[:, o0:o0 + q]
        gr = (C.c_void_p * q)(*[Gw.ctypes.data + (o0 + i) * Gw.strides[0] for i in range(q)])
        sr = (C.c_void_p * m)(*[Sw.ctypes.data + e * Sw.strides[0] + o0 * 8 for e in range(m)])
        cG, cS = np.ascontiguousarray(pG), np.ascontiguousarray(pS)
        assert R.traceprod(0, 0, q, m, gr, sr, 0) == L.or_traceprod(0, 0, q, m, cG.ctypes.data, cS.ctypes.data)
        assert R.traceprod(0, 1, m, q, sr, sr, 0) == L.or_traceprod(0, 1, m, q, cS.ctypes.data, cS.ctypes.data)


@pytest.mark.parametrize("name,mode,scheme", [("etkf", 0, 1), ("denkf", 0, 0)])
def test_calctransforms_against_reference_golden(name, mode, scheme):
    """The oracle's transform stage against the float outputs of the
    reference's own das_calctransforms (tests/golden/calctransforms.npz),
    bit for bit."""
    g = np.load(os.path.join(GOLD, "calctransforms.npz"))
    nt = int(g["otype"].max()) + 1
    nl, lr, lw = oracle.locrad_table(nt, float(g["locrad"]))
    obs = oracle.ObsSet(g["lon"], g["lat"], g["otype"], g["status"], nt, nl, lr, lw)
    m = int(g["nmem"])
    out = oracle.calctransforms(obs, mode=mode, scheme=scheme, nmem=m, nmem_dynamic=m, alpha=float(g[f"{name}_alpha"]),
                                stride=int(g["stride"]), x=g["x"], y=g["y"], S=g["S"], s=g["s"], threads=8)
    for k in ("T", "w", "nlobs", "dfs", "srf", "pnlobs", "pdfs", "psrf"):
        assert np.array_equal(out[k], g[f"{name}_{k}"]), (name, k)


# (name, workload, scale, nmem, nmem_dynamic, mode, scheme, alpha, options)
TRANSFORM_CASES = [
    ("w1_etkf", 1, 1.0, 24, 24, 0, 1, 1.0, {}),
    ("w1_denkf_alpha", 1, 0.5, 24, 24, 0, 0, 0.7, {}),
    ("w2_denkf_stride3", 2, 0.1, 20, 20, 0, 0, 1.0, {}),
    ("w2_etkf_alpha", 2, 0.1, 20, 20, 0, 1, 0.7, {}),
    ("w2_enoi", 2, 0.1, 20, 20, 1, 0, 1.0, {}),
    ("w2_hybrid_etkf", 2, 0.1, 24, 16, 2, 1, 0.8, {}),
    ("w2_etkf_nlobsmax_hidden", 2, 0.1, 20, 20, 0, 1, 1.0, dict(nlobsmax=(25, 10), visible=(1, 0))),
    ("w2_denkf_geographic", 2, 0.1, 20, 20, 0, 0, 1.0, dict(geographic=True)),
]


@pytest.mark.skipif(oracle.reflib_transforms() is None, reason="reference library not built here")
@pytest.mark.parametrize("case", TRANSFORM_CASES, ids=[c[0] for c in TRANSFORM_CASES])
def test_calctransforms_equals_reference_build(case):
    """das_calctransforms (calc/transforms.c:991-1637, compiled unmodified
    with calcs.c, observations.c, obstypes.c and kdtree.c; the model grid and
    the output files in memory): the oracle's T, w and diagnostics -- nlobs,
    dfs, srf and per type pnlobs, pdfs, psrf, as the reference writes them in
    float -- equal the reference's bit for bit over the whole strided grid:
    ETKF, DEnKF, EnOI and hybrid, relaxation, one and two observation types
    with rejected observations and points without local observations,
    NLOBSMAX with a type hidden by its domains, and GEOGRAPHIC 1."""
    import synth
    from helpers import prepare
    name, cfg, scale, m, md, mode, scheme, alpha, opt = case
    kw = dict(nobs=6000) if cfg == 2 else {}
    w = synth.make(cfg, scale=scale, nmem=m, with_fields=False, **kw)
    w.nmem_dynamic = md
    st = w.status.copy()
    st[::23] = 1
    w.status = st
    x, y, radius = w.x, w.y, (12.0 if cfg == 2 else w.locrad)
    geo = opt.get("geographic", False)
    if geo:
        sx, sy = 60.0 / (w.x.size - 1), 60.0 / (w.y.size - 1)
        w.lon = (100.0 + w.lon * sx).astype(np.float32)
        w.lat = (-30.0 + w.lat * sy).astype(np.float32)
        x, y, radius = 100.0 + w.x * sx, -30.0 + w.y * sy, 400.0
    S, s = prepare(w)
    nl, lr, lw = oracle.locrad_table(w.ntypes, radius)
    vis = opt.get("visible")
    st_o = st.copy()
    if vis is not None:
        for t, v in enumerate(vis):
            if not v:
                st_o[w.otype == t] = 1
    nm = opt.get("nlobsmax")
    obs_o = oracle.ObsSet(w.lon, w.lat, w.otype, st_o, w.ntypes, nl, lr, lw,
                          nlobsmax=None if nm is None else np.array(nm), geographic=geo)
    obs_r = oracle.ObsSet(w.lon, w.lat, w.otype, st, w.ntypes, nl, lr, lw,
                          nlobsmax=None if nm is None else np.array(nm), geographic=geo)
    out = oracle.calctransforms(obs_o, mode=mode, scheme=scheme, nmem=m, nmem_dynamic=md, alpha=alpha,
                                stride=w.stride, x=x, y=y, S=S, s=s, threads=8)
    ref = oracle.ref_calctransforms(obs_r, mode=mode, scheme=scheme, nmem=m, nmem_dynamic=md, alpha=alpha,
                                    stride=w.stride, x=x, y=y, S=S, s=s, visible=vis)
    assert (ref["nlobs"] == 0).any() or cfg == 1
    for k in ("T", "w", "nlobs", "dfs", "srf", "pnlobs", "pdfs", "psrf"):
        if ref[k] is None:
            continue
        assert np.array_equal(out[k], ref[k]), (name, k)


@pytest.mark.skipif(oracle.reflib_transforms() is None, reason="reference library not built here")
@pytest.mark.parametrize("mode,scheme", [(0, 1), (0, 0), (1, 0)])
def test_pointlog_transforms_equal_reference_build(mode, scheme):
    """das_calcpointlogtransforms (calc/transforms.c:1646-1773, compiled
    unmodified; the point-log writer's arrays captured): the oracle at the
    log points, taken as a 1 x n curvilinear grid -- the recipe the library
    documents for point logs -- gives the reference's double T and w bit for
    bit, including a log point with no local observation."""
    import synth
    from helpers import prepare, obsset
    w = synth.make(1, scale=0.5, with_fields=False)
    S, s = prepare(w)
    obs, _ = obsset(w)
    rng = np.random.default_rng(11)
    n = 37
    px = rng.uniform(w.x.min(), w.x.max(), n)
    py = rng.uniform(w.y.min(), w.y.max(), n)
    px[5], py[5] = w.x.max() + 10 * w.locrad, w.y.max() + 10 * w.locrad
    Tr, wr = oracle.ref_calcpointlogtransforms(obs, mode=mode, scheme=scheme, nmem=w.nmem, nmem_dynamic=w.nmem,
                                               alpha=0.7, plon=px, plat=py, S=S, s=s)
    out = oracle.calctransforms(obs, mode=mode, scheme=scheme, nmem=w.nmem, nmem_dynamic=w.nmem, alpha=0.7, stride=1,
                                x=px, y=py, S=S, s=s, want64=True, x2d=px[None, :], y2d=py[None, :])
    assert np.array_equal(out["w64"][0], wr)
    if mode != 1:
        assert np.array_equal(out["T64"][0], Tr)
    assert np.all(wr[5] == 0.0)


@pytest.mark.skipif(oracle.reflib_obs() is None, reason="reference library not built here")
@pytest.mark.parametrize("geographic", [False, True])
@pytest.mark.parametrize("nlobsmax", [None, (9, 4, 30)])
@pytest.mark.parametrize("hidden", [None, 1])
def test_findlocal_equals_reference_build(geographic, nlobsmax, hidden):
    """obs_findlocal (common/observations.c:1837-1927 with obstypes.c and
    kdtree.c, compiled unmodified): ids and taper coefficients, in the
    reference's order, equal the oracle's at every query -- three types, one
    with two radii and weights, rejected observations, a quarter of the
    observations in groups at one position, NLOBSMAX, a type hidden by its
    domains (the oracle: its observations rejected) and queries without
    coordinates (obs_getglobal)."""
    rng = np.random.default_rng(31 + 2 * int(geographic) + (4 if nlobsmax else 0) + (8 if hidden else 0))
    n = 2500
    lon = rng.uniform(0, 50, n)
    lat = rng.uniform(0, 40, n)
    for i in rng.choice(np.arange(1, n), n // 4, replace=False):
        j = rng.integers(0, i)
        lon[i], lat[i] = lon[j], lat[j]
    otype = rng.integers(0, 3, n).astype(np.int16)
    status = np.zeros(n, np.int16)
    status[::11] = 1
    radii = [[4.0, 2.0], [6.0], [3.0]]
    if geographic:
        lon, lat = 140.0 + 0.4 * lon, -20.0 + 0.4 * lat
        radii = [[180.0, 90.0], [260.0], [130.0]]
    lon, lat = lon.astype(np.float32), lat.astype(np.float32)
    nl, lr, lw = oracle.locrad_table(3, radii, [[0.7, 0.3], [1.0], [1.0]])
    qx = rng.uniform(float(lon.min()), float(lon.max()), 40)
    qy = rng.uniform(float(lat.min()), float(lat.max()), 40)
    qx[:6] = np.floor(qx[:6])
    qx[7], qy[19] = np.nan, np.nan
    visible = None if hidden is None else np.array([1 if t != hidden else 0 for t in range(3)])
    ref = oracle.ref_findlocal(lon, lat, otype, status, 3, nl, lr, lw, qx, qy, nlobsmax=nlobsmax, visible=visible,
                               geographic=geographic)
    st = status.copy()
    if hidden is not None:
        st[otype == hidden] = 1
    obs = oracle.ObsSet(lon, lat, otype, st, 3, nl, lr, lw, nlobsmax=None if nlobsmax is None else np.array(nlobsmax),
                        geographic=geographic)
    for k in range(qx.size):
        ids, lc = obs.findlocal(qx[k], qy[k])
        assert np.array_equal(ids, ref[k][0]), k
        assert np.array_equal(lc, ref[k][1]), k
    assert ref[7][0].size == (st == 0).sum() and np.all(ref[7][1] == 1.0)


@pytest.mark.skipif(oracle.reflib_model2obs() is None, reason="reference library not built here")
@pytest.mark.parametrize("three_d", [False, True])
def test_forward_operators_equal_reference_build(three_d):
    """H_surf_standard and H_subsurf_standard (calc/model2obs.c, compiled
    unmodified; the model variable, grid and observations in memory): the
    oracle's HE equals the reference's bit for bit -- both surface-layer
    conventions, periodic i, OFFSET data of every shape the function takes,
    positions on grid lines, and bad forecasts (NaN under
    --skip-bad-forecast-obs)."""
    rng = np.random.default_rng(5 + int(three_d))
    ni, nj, nk = 23, 17, 5
    nl = rng.integers(0, nk + 1, (nj, ni)).astype(np.int32)
    nl[rng.random((nj, ni)) < 0.5] = nk
    f3 = rng.normal(10.0, 2.0, (nk, nj, ni)).astype(np.float32)
    f3[0, 3, 4] = np.nan
    f3[nk - 1, 5, 6] = 2.0e6
    n = 400
    fi = rng.uniform(0, ni - 1, n)
    fj = rng.uniform(0, nj - 1, n)
    fk = rng.uniform(0, nk - 1, n).astype(np.float32)
    fi[:20] = np.floor(fi[:20])
    fj[20:40] = np.floor(fj[20:40])
    fi[40:44], fj[40:44] = [3.5, 4.0, 6.2, 5.5], [2.5, 3.0, 4.7, 5.0]
    ids = np.arange(n, dtype=np.int32)
    kinds = [0, 1, 2, 3] if three_d else [0, 2]
    for ksurf in (0, nk - 1):
        for per in (0, 1):
            for ok in kinds:
                off = None
                if ok:
                    shape = {1: (nk,), 2: (nj, ni), 3: (nk, nj, ni)}[ok]
                    off = rng.normal(0.0, 1.0, shape).astype(np.float32)
                ref = oracle.ref_H(f3, nl, ids, fi, fj, fk, three_d=three_d, ksurf=ksurf, periodic_i=per, offset=off,
                                   offset_kind=ok)
                HE = np.full((1, n), np.nan, np.float32)
                rc = oracle.map_obs(HE, 0, f3 if three_d else f3[ksurf], nl, ids, fi, fj, fk, three_d=three_d,
                                    ktop=ksurf, periodic_i=per, offset=off, offset_kind=ok, skip_bad=True)
                assert rc == 0
                assert np.array_equal(HE[0], ref, equal_nan=True), (ksurf, per, ok)


@pytest.mark.skipif(oracle.reflib_gethe() is None, reason="reference library not built here")
@pytest.mark.parametrize("mode,m,md,gamma", [(0, 6, 6, 0.0), (1, 6, 6, 0.0), (2, 8, 5, 0.5)])
def test_he_stage_equals_reference_build(mode, m, md, gamma):
    """das_getHE (calc/ensobs.c:46-490 with calc/model2obs.c, calc/allhs.c and
    the observation module, compiled unmodified; members, grid and
    observations in memory): the oracle's per-type forward operators for
    every member (and the EnOI background) followed by its restatement of
    the end of das_getHE give the reference's HE and statuses bit for bit --
    ENKF, EnOI and hybrid, a surface and a subsurface type, both
    surface-layer conventions, rejected observations and a bad forecast
    under --skip-bad-forecast-obs."""
    rng = np.random.default_rng(17 + mode)
    ni, nj, nk = 23, 17, 5
    nl = rng.integers(0, nk + 1, (nj, ni)).astype(np.int32)
    nl[rng.random((nj, ni)) < 0.5] = nk
    n = 300
    fi = rng.uniform(0, ni - 1, n)
    fj = rng.uniform(0, nj - 1, n)
    fk = rng.uniform(0, nk - 1, n).astype(np.float32)
    otype = rng.integers(0, 2, n).astype(np.int16)
    status = np.zeros(n, np.int16)
    status[::13] = 1
    issurface = np.array([1, 0])
    rows = m + 1 if mode == 1 else m
    mem = rng.normal(10.0, 2.0, (rows, nk, nj, ni)).astype(np.float32)
    mem[2, 0, 4, 5] = np.nan
    for ksurf in (0, nk - 1):
        HEr, st_r = oracle.ref_getHE(mem, nl, otype, status, fi, fj, fk, issurface, mode=mode, nmem_dynamic=md,
                                     gamma=gamma, ksurf=ksurf)
        HE = np.full((rows, n), np.nan, np.float32)
        for e in range(rows):
            for t in range(2):
                ids = np.nonzero((otype == t) & (status == 0))[0].astype(np.int32)
                three = not issurface[t]
                assert oracle.map_obs(HE, e, mem[e] if three else mem[e][ksurf], nl, ids, fi, fj, fk, three_d=three,
                                      ktop=ksurf, skip_bad=True) == 0
        S, st, nbad = oracle.finish_HE(HE[:m], status, mode=mode, nmem_dynamic=md, gamma=gamma,
                                       Hx=HE[m] if mode == 1 else None, skip_bad=True)
        assert np.array_equal(S, HEr[:m], equal_nan=True), ksurf
        assert np.array_equal(st, st_r), ksurf
        assert nbad == (st_r == 10).sum() > 0


@pytest.mark.skipif(oracle.reflib_ensobs() is None, reason="reference library not built here")
@pytest.mark.parametrize("m,n", [(24, 3000), (96, 5000), (7, 40)])
def test_innovations_and_standardise_equal_reference_build(m, n):
    """das_calcinnandspread and das_standardise (calc/ensobs.c:541-690,
    849-898, compiled unmodified): the oracle's S, s_f, std_f and the
    standardised S and s equal the reference's bit for bit, with rejected
    observations (their s_f and std_f stay the ensemble mean and the sum of
    squares, as the reference leaves them) and three types of different
    rfactor."""
    rng = np.random.default_rng(m + n)
    HE = (15.0 + rng.standard_normal((m, n)) * rng.uniform(0.1, 3.0, n)).astype(np.float32)
    value = (15.0 + rng.standard_normal(n)).astype(np.float32)
    status = np.zeros(n, np.int16)
    status[rng.uniform(size=n) < 0.1] = 1
    status[rng.uniform(size=n) < 0.02] = 2
    S0, s0, d0 = oracle.calcinnandspread(HE, value, status)
    S1, s1, d1 = oracle.ref_calcinnandspread(HE, value, status)
    assert np.array_equal(S0, S1)
    assert np.array_equal(s0, s1)
    assert np.array_equal(d0, d1)
    estd = rng.uniform(0.2, 0.9, n).astype(np.float32)
    otype = rng.integers(0, 3, n).astype(np.int16)
    rfactor = np.array([1.0, 2.5, 0.7])
    Sa, sa = oracle.standardise(S0, s0, estd, otype, rfactor)
    Sb, sb = oracle.ref_standardise(S1, s1, estd, otype, rfactor)
    assert np.array_equal(Sa, Sb)
    assert np.array_equal(sa, sb)


@pytest.mark.skipif(oracle.reflib_utils() is None, reason="reference library not built here")
def test_ll2xyz_equals_reference_build():
    import ctypes as C
    rng = np.random.default_rng(8)
    L, R = oracle.lib(), oracle.reflib_utils()
    for _ in range(2000):
        ll = (C.c_double * 2)(rng.uniform(-360, 360), rng.uniform(-90, 90))
        a, b = (C.c_double * 3)(), (C.c_double * 3)()
        L.or_ll2xyz(ll, a)
        R.ll2xyz(ll, b)
        assert list(a) == list(b)


# ---------------------------------------------------------------------------
# known answers of the per-point numerics (calc/calcs.c), for the oracle and,
# where it is built here, the reference itself
# ---------------------------------------------------------------------------

def _impls():
    out = [("oracle", oracle.calc_wT)]
    if oracle.reflib() is not None:
        out.append(("reference", oracle.ref_calc_wT))
    return out


@pytest.mark.parametrize("name,calc", _impls())
def test_single_observation_closed_form(name, calc):
    rng = np.random.default_rng(31)
    m = 9
    S = rng.normal(0, 0.7, (m, 1))                   # one observation: S [m][p = 1]
    d = np.array([0.8])
    a = float((S[:, 0] ** 2).sum())
    ss = np.outer(S[:, 0], S[:, 0])
    w_exact = S[:, 0] * d[0] / (1.0 + a)
    # ETKF: T = (I + s s')^(-1/2) = I + (1/sqrt(1 + a) - 1) s s' / a
    w, T, _ = calc(0, 1, m, m, d, S)
    assert np.abs(w - w_exact).max() < 1e-13, name
    assert np.abs(T - (np.eye(m) + (1.0 / np.sqrt(1.0 + a) - 1.0) * ss / a)).max() < 1e-13, name
    # DEnKF: T = (I + M^-1) / 2 = I - s s' / (2 (1 + a))
    w, T, _ = calc(0, 0, m, m, d, S)
    assert np.abs(w - w_exact).max() < 1e-13, name
    assert np.abs(T - (np.eye(m) - ss / (2.0 * (1.0 + a)))).max() < 1e-13, name
    # EnOI: w only
    w, _, _ = calc(1, 0, m, m, d, S)
    assert np.abs(w - w_exact).max() < 1e-13, name


@pytest.mark.parametrize("name,calc", _impls())
@pytest.mark.parametrize("p", [5, 40])              # p < m and p >= m: the two branches of calcs.c
def test_transform_identities(name, calc, p):
    rng = np.random.default_rng(32 + p)
    m = 16
    S = rng.normal(0, 0.5, (m, p))
    S -= S.mean(axis=0)                              # member-mean-free anomalies, as after das_calcinnandspread
    d = rng.normal(0, 1, p)
    M = np.eye(m) + S @ S.T
    lam, U = np.linalg.eigh(M)                       # an independent path: numpy's symmetric eigensolver
    T_etkf = (U / np.sqrt(lam)) @ U.T
    Minv = (U / lam) @ U.T
    w_exact = Minv @ (S @ d)
    w_e, T_e, _ = calc(0, 1, m, m, d, S)
    w_d, T_d, _ = calc(0, 0, m, m, d, S)
    assert np.abs(T_e - T_e.T).max() < 1e-12, name                     # ETKF transform is symmetric
    assert np.abs(T_e - T_etkf).max() < 1e-11, name
    assert np.abs(T_d - 0.5 * (np.eye(m) + Minv)).max() < 1e-11, name
    assert np.abs(w_e - w_exact).max() < 1e-11 and np.abs(w_d - w_exact).max() < 1e-11, name
    assert np.abs(w_e - w_d).max() < 1e-12, name                        # the schemes agree on w
    ones = np.ones(m)
    assert np.abs(T_e @ ones - ones).max() < 1e-12, name                # the mean is kept
    assert np.abs(T_d @ ones - ones).max() < 1e-12, name


def _golden_update():
    import os
    return np.load(os.path.join(os.path.dirname(__file__), "golden", "update.npz"))


def oracle_update_case(g, k):
    """The oracle's update of golden case k (its inputs as the reference got them)."""
    mode, mnj, mni, m, md, stride, per, j1, j2, level, surfk, issv, inc, alog = [int(x) for x in g[f"u{k}_prm"]]
    infl, ratio = [float(x) for x in g[f"u{k}_infl"]]
    v, T, w, nl = g[f"u{k}_v"], g[f"u{k}_T"], g[f"u{k}_w"], g[f"u{k}_numlevels"]
    if mode == 1:
        return oracle.updatebg(v, w, nl, nmem=m, stride=stride, periodic_i=per, level=level, surfk=surfk,
                               issurfacevar=issv, j1=j1, j2=j2)
    return oracle.updatefields(v, T, w, nl, mode=mode, nmem=m, nmem_dynamic=md, stride=stride, periodic_i=per,
                               level=level, surfk=surfk, issurfacevar=issv, inflation=infl, inf_ratio=ratio,
                               output_increment=inc, applylog=alog, j1=j1, j2=j2)


def test_update_restatement_against_reference_golden():
    """or_updatefields / or_updatebg / or_sethybridensemble against the
    reference's own update/update.c and common/dasystem.c (compiled
    unmodified; tests/golden/update.npz), bit for bit: every case of strides,
    masks, missing values, inflation, increments, log fields, hybrid, EnOI."""
    g = _golden_update()
    for k, name in enumerate(g["names"]):
        got = oracle_update_case(g, k)
        exp = g[f"u{k}_out"]
        # bit for bit; NaNs (a NaN member in EnOI propagates into the
        # background, as in the reference) compare as NaNs, payloads aside
        assert np.array_equal(got, exp, equal_nan=True), name
        if f"u{k}_hyb_in" in g.files:
            md = int(g[f"u{k}_prm"][4])
            hv, vmean = oracle.sethybridensemble(g[f"u{k}_hyb_in"], md, 0.5)
            assert np.array_equal(hv, g[f"u{k}_hyb_out"]), name
            assert np.array_equal(vmean, g[f"u{k}_hyb_mean"]), name


def test_update_reference_build_matches_golden():
    """Where the reference build exists, it reproduces the committed fixture
    (the fixture is its output, not a stale copy)."""
    if oracle.reflib_update() is None:
        pytest.skip("reference update library not built here")
    g = _golden_update()
    for k, name in enumerate(g["names"]):
        mode, mnj, mni, m, md, stride, per, j1, j2, level, surfk, issv, inc, alog = [int(x) for x in g[f"u{k}_prm"]]
        infl, ratio = [float(x) for x in g[f"u{k}_infl"]]
        res = oracle.ref_update_layer(g[f"u{k}_v"], None if mode == 1 else g[f"u{k}_T"], g[f"u{k}_w"],
                                      g[f"u{k}_numlevels"], mode=mode, nmem=m, nmem_dynamic=md, stride=stride,
                                      periodic_i=per, level=level, surfk=surfk, issurfacevar=issv, inflation=infl,
                                      inf_ratio=ratio, output_increment=inc, applylog=alog, j1=j1, j2=j2)
        assert np.array_equal(res, g[f"u{k}_out"], equal_nan=True), name
