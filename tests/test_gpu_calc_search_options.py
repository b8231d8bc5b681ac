"""The two per-type options of obs_findlocal (common/observations.c:1837-1927)
on the device: NLOBSMAX (the nlobsmax nearest observations of a type, from
the distance-sorted range search, kdtree.c:558-574) and obs-type domains (a
type the grid's domain does not see is skipped).

Tolerances: local lists bit-exact (ids and taper coefficients); double T and
w within 1e-10 per point of the FP64 oracle on the FP64 path, 1e-5 on the
mixed path (the contracts of test_gpu_calc.py and test_gpu_mixed.py).
"""
import os

import numpy as np
import pytest

import oracle
import synth
from helpers import gpu_setup, prepare

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def per_point_rel(a, b):
    a = a.reshape(a.shape[0] * a.shape[1], -1)
    b = b.reshape(b.shape[0] * b.shape[1], -1)
    den = np.maximum(np.abs(b).max(axis=1), 1e-300)
    return float((np.abs(a - b).max(axis=1) / den).max())


@pytest.fixture
def octx(ctx):
    """The session context, with the options cleared again afterwards."""
    yield ctx
    try:
        ctx.set_obstype_nlobsmax(None)
        ctx.set_obstype_visible(None)
    except Exception:
        pass


@pytest.mark.parametrize("nmax", [(1, 1), (7, 3), (25, 40)])
def test_nlobsmax_lists_against_reference_golden(octx, nmax):
    """Lists under NLOBSMAX against the reference's own distance-sorted range
    search; a third of the observations come in groups at one position, so
    the cut often falls inside a group of equal distances."""
    ctx = octx
    g = np.load(os.path.join(GOLD, "nlobsmax.npz"))
    nl, lr, lw = oracle.locrad_table(2, [[float(r)] for r in g["r"]])
    n = g["lon"].size
    ctx.set_obstypes(nl, lr, lw, np.ones(2))
    ctx.set_obs(g["lon"], g["lat"], g["otype"], np.zeros(n, np.int16), np.ones(n, np.float32),
                np.zeros(n, np.float32))
    ctx.set_S(np.zeros((4, n), np.float32), np.zeros(n), 4)
    q = g["q"]
    ctx.set_grid(x2d=q[:, 0][None, :], y2d=q[:, 1][None, :], stride=1)
    ctx.set_obstype_nlobsmax(np.array(nmax))
    obs = oracle.ObsSet(g["lon"], g["lat"], g["otype"], np.zeros(n, np.int16), 2, nl, lr, lw, nlobsmax=np.array(nmax))
    counts, offsets, ids, coeffs = ctx.findlocal(lists=True)
    ties_cut = 0
    for k in range(q.shape[0]):
        ref = np.concatenate([g[f"t{t}_q{k}_ids"][:nmax[t]] for t in range(2)])
        order = np.argsort(ref, kind="stable")
        a, b = offsets[k], offsets[k + 1]
        assert counts[0, k] == ref.size, k
        assert np.array_equal(ids[a:b], ref[order]), k
        rid, rlc = obs.findlocal(q[k, 0], q[k, 1])
        assert np.array_equal(coeffs[a:b], rlc[np.argsort(rid, kind="stable")]), k
        for t in range(2):
            d2 = g[f"t{t}_q{k}_d2"]
            if d2.size > nmax[t] and d2[nmax[t] - 1] == d2[nmax[t]]:
                ties_cut += 1
    if nmax == (7, 3):
        assert ties_cut > 0     # some cut inside a group of equal distances
    # the limit cleared: the full lists again
    ctx.set_obstype_nlobsmax(None)
    full = np.array([sum(g[f"t{t}_q{k}_ids"].size for t in range(2)) for k in range(q.shape[0])])
    assert np.array_equal(ctx.findlocal(lists=False)[0], full)


def with_groups(w, seed=3, frac=0.3):
    """Moves a fraction of the observations onto the position of an earlier
    observation of the same type (groups at one position: equal distances)."""
    rng = np.random.default_rng(seed)
    lon, lat = w.lon.copy(), w.lat.copy()
    for t in range(w.ntypes):
        ids = np.nonzero(w.otype == t)[0]
        mv = rng.choice(ids[1:], int(frac * ids.size), replace=False)
        for i in mv:
            j = ids[rng.integers(0, np.searchsorted(ids, i))]
            lon[i], lat[i] = lon[j], lat[j]
    w.lon, w.lat = lon, lat
    return w


# (name, workload, scale, m, mode, scheme, precision, nlobsmax per type, geographic)
TCASES = [
    ("fp64_etkf_2types", 2, 0.1, 20, 0, 1, 0, (30, 12), False),
    ("fp64_denkf_2types", 2, 0.1, 20, 0, 0, 0, (30, 12), False),
    ("fp64_enoi_2types", 2, 0.1, 20, 1, 0, 0, (5, 50), False),
    ("mixed_etkf_2types", 2, 0.1, 20, 0, 1, 1, (30, 12), False),
    ("mixed_etkf_m96", 3, 0.12, 96, 0, 1, 1, (300,), False),
    ("fp64_etkf_geographic", 2, 0.1, 20, 0, 1, 0, (30, 12), True),
    ("mixed_denkf_geographic", 2, 0.1, 20, 0, 0, 1, (30, 12), True),
]


@pytest.mark.parametrize("case", TCASES, ids=[c[0] for c in TCASES])
def test_transforms_under_nlobsmax(octx, case):
    ctx = octx
    name, cfg, scale, m, mode, scheme, prec, nmax, geo = case
    kw = dict(nobs=6000) if cfg == 2 else {}
    w = with_groups(synth.make(cfg, scale=scale, nmem=m, with_fields=False, **kw))
    if cfg == 2:
        w.locrad = 12.0
    x, y = w.x, w.y
    if geo:
        # the same layout as degrees on the sphere: lon 100..160, lat -30..30
        sx, sy = 60.0 / (w.x.size - 1), 60.0 / (w.y.size - 1)
        w.lon = (100.0 + w.lon * sx).astype(np.float32)
        w.lat = (-30.0 + w.lat * sy).astype(np.float32)
        x, y = 100.0 + w.x * sx, -30.0 + w.y * sy
        w.locrad = 400.0            # km on the sphere
    S, s = prepare(w)
    nl, lr, lw = oracle.locrad_table(w.ntypes, w.locrad)
    obs = oracle.ObsSet(w.lon, w.lat, w.otype, w.status, w.ntypes, nl, lr, lw, nlobsmax=np.array(nmax),
                        geographic=geo)
    ref = oracle.calctransforms(obs, mode=mode, scheme=scheme, nmem=m, nmem_dynamic=m, alpha=1.0, stride=w.stride,
                                x=x, y=y, S=S, s=s, want64=True, threads=16)
    ctx.set_obstypes(nl, lr, lw, np.ones(w.ntypes), geographic=geo)
    ctx.set_obs(w.lon, w.lat, w.otype, w.status, w.estd, w.value)
    ctx.set_S(S, s, m)
    ctx.set_grid(x, y, stride=w.stride)
    ctx.set_obstype_nlobsmax(np.array(nmax))
    tol = 1e-10 if prec == 0 else 1e-5
    paths = (0, 1) if prec == 0 else (1,)
    for path in paths:
        out = ctx.calctransforms(mode=mode, scheme=scheme, alpha=1.0, path=path, precision=prec, want64=True,
                                 want_diag=(path == 0))
        if path == 0:
            assert np.array_equal(out["nlobs"], ref["nlobs"]), name
            assert np.array_equal(out["pnlobs"], ref["pnlobs"]), name
        if mode != 1:
            assert per_point_rel(out["T64"], ref["T64"]) < tol, (name, path)
        assert per_point_rel(out["w64"], ref["w64"]) < tol, (name, path)
    assert np.array_equal(ctx.findlocal(lists=False), ref["nlobs"])
    # the limit shows: without it the counts are larger somewhere
    ctx.set_obstype_nlobsmax(None)
    full = ctx.findlocal(lists=False)
    assert (full > ref["nlobs"]).any() and (full >= ref["nlobs"]).all()


@pytest.mark.parametrize("prec", [0, 1])
def test_obstype_domains_hide_a_type(octx, prec):
    """A type hidden from the grid (its domains exclude the grid's) takes no
    part: the same as the oracle without that type's observations; shown
    again, everything is back."""
    ctx = octx
    w = synth.make(2, scale=0.1, nobs=6000, with_fields=False, nmem=20)
    w.locrad = 12.0
    S, s = prepare(w)
    nl, lr, lw = oracle.locrad_table(w.ntypes, w.locrad)
    st_hidden = w.status.copy()
    st_hidden[w.otype == 1] = 1
    obs_h = oracle.ObsSet(w.lon, w.lat, w.otype, st_hidden, w.ntypes, nl, lr, lw)
    obs_all = oracle.ObsSet(w.lon, w.lat, w.otype, w.status, w.ntypes, nl, lr, lw)
    kw = dict(mode=0, scheme=1, nmem=w.nmem, nmem_dynamic=w.nmem, alpha=1.0, stride=w.stride, x=w.x, y=w.y, S=S,
              s=s, want64=True, threads=16)
    ref_h = oracle.calctransforms(obs_h, **kw)
    ref_all = oracle.calctransforms(obs_all, **kw)
    gpu_setup(ctx, w, S, s, (nl, lr, lw))
    tol = 1e-10 if prec == 0 else 1e-5
    ctx.set_obstype_visible(np.array([1, 0]))
    out = ctx.calctransforms(mode=0, scheme=1, path=1, precision=prec, want64=True, want_diag=False)
    assert per_point_rel(out["T64"], ref_h["T64"]) < tol
    assert per_point_rel(out["w64"], ref_h["w64"]) < tol
    out = ctx.calctransforms(mode=0, scheme=1, path=0, precision=0, want64=True)
    assert np.array_equal(out["nlobs"], ref_h["nlobs"])
    assert np.all(out["pnlobs"][1] == 0)
    ctx.set_obstype_visible(None)
    out = ctx.calctransforms(mode=0, scheme=1, path=1, precision=prec, want64=True, want_diag=False)
    assert per_point_rel(out["T64"], ref_all["T64"]) < tol
    assert per_point_rel(out["w64"], ref_all["w64"]) < tol
