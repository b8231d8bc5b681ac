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
