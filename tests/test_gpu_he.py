"""Parity of the device forward operator with the oracle and with the
reference's own interpolation (golden fixture), through the C ABI.

Covers das_getHE (calc/ensobs.c:46-490): H_surf_standard / H_subsurf_standard
(calc/model2obs.c:127-348) with interpolate2d_structured /
interpolate3d_structured (common/utils.c:1140-1366), the bad-forecast rule,
and the EnOI / hybrid post-processing.  The device follows the reference's
operation order in double with round-to-nearest intrinsics, so HE is compared
bit for bit (a NaN matches a NaN).
"""
import os

import numpy as np
import pytest

import oracle
import synth

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def same_bits(a, b):
    a = np.asarray(a, np.float32)
    b = np.asarray(b, np.float32)
    na, nb = np.isnan(a), np.isnan(b)
    return bool(np.array_equal(na, nb) and np.array_equal(a[~na].view(np.uint32), b[~nb].view(np.uint32)))


def setup_obs(ctx, fi, fj, fk=None, otype=None, status=None, ntypes=1):
    n = fi.size
    nl, lr, lw = oracle.locrad_table(ntypes, 5.0)
    ctx.set_obstypes(nl, lr, lw, np.ones(ntypes))
    otype = np.zeros(n, np.int16) if otype is None else otype
    status = np.zeros(n, np.int16) if status is None else status
    lon = np.nan_to_num(fi, nan=0.0).astype(np.float32)
    lat = np.nan_to_num(fj, nan=0.0).astype(np.float32)
    ctx.set_obs(lon, lat, otype, status, np.full(n, 0.5, np.float32), np.zeros(n, np.float32))
    ctx.set_obs_positions(fi, fj, fk)


def test_he_against_reference_golden(ctx):
    g = np.load(os.path.join(GOLD, "model2obs.npz"))
    nk = int(g["nk"])
    m, n = g["he2_p0"].shape
    # each case starts from fresh statuses: finish_HE(skip_bad) marks the
    # all-dry observations STATUS_BADFC, and later calls select status 0 only
    for per in (0, 1):
        setup_obs(ctx, g["fi"], g["fj"], g["fk"])
        ctx.begin_HE(m)
        ctx.map_obs(0, g["f2"], g["numlevels"], periodic_i=per, offset=g["off2"], offset_kind=2, skip_bad=True)
        ctx.finish_HE(skip_bad=True)
        assert same_bits(ctx.get_S()[0], g[f"he2_p{per}"]), f"2-D periodic={per}"
        for ktop in (0, nk - 1):
            setup_obs(ctx, g["fi"], g["fj"], g["fk"])
            ctx.begin_HE(m)
            ctx.map_obs(0, g["f3"], g["numlevels"], three_d=True, ksurf=ktop, periodic_i=per, offset=g["off1"],
                        offset_kind=1, skip_bad=True)
            ctx.finish_HE(skip_bad=True)
            assert same_bits(ctx.get_S()[0], g[f"he3_p{per}_k{ktop}"]), f"3-D periodic={per} ktop={ktop}"


@pytest.mark.parametrize("three_d,offset_kind", [(False, 0), (False, 2), (True, 0), (True, 2), (True, 3)])
def test_he_against_oracle(ctx, three_d, offset_kind):
    rng = np.random.default_rng(100 + 10 * int(three_d) + offset_kind)
    ni, nj, nk, m, n = 61, 43, 6, 7, 5000
    nl = rng.integers(0, nk + 1, (nj, ni)).astype(np.int32)
    nl[rng.random((nj, ni)) < 0.5] = nk                    # mostly wet
    shape = (m, nk, nj, ni) if three_d else (m, nj, ni)
    fields = rng.normal(15.0, 2.0, shape).astype(np.float32)
    offset = None
    if offset_kind == 2:
        offset = rng.normal(0.0, 0.3, (nj, ni)).astype(np.float32)
    elif offset_kind == 3:
        offset = rng.normal(0.0, 0.3, (nk, nj, ni)).astype(np.float32)
    fi = rng.uniform(-0.9, ni - 0.01, n)
    fj = rng.uniform(-0.9, nj + 0.3, n)
    fi[::9] = np.floor(np.maximum(fi[::9], 0.0))
    fk = rng.uniform(-0.5, nk - 0.5, n).astype(np.float32)
    otype = (rng.random(n) < 0.3).astype(np.int16)            # two types
    status = np.where(rng.random(n) < 0.05, 2, 0).astype(np.int16)
    setup_obs(ctx, fi, fj, fk, otype, status, ntypes=2)
    ktop = nk - 1 if three_d else 0
    kw = dict(three_d=three_d, ksurf=ktop, periodic_i=True, offset=offset, offset_kind=offset_kind, skip_bad=True)
    ctx.begin_HE(m)
    # type 0 by selection (status 0 only), in two member blocks
    ctx.map_obs(0, fields[:4], nl, mem0=0, **kw)
    ctx.map_obs(0, fields[4:], nl, mem0=4, **kw)
    # type 1 by an explicit id list (a strided subset)
    ids1 = np.nonzero((otype == 1) & (status == 0))[0][::2].astype(np.int32)
    ctx.map_obs(1, fields, nl, mem0=0, ids=ids1, **kw)
    nbad, st = ctx.finish_HE(skip_bad=True)
    got = ctx.get_S()[0]

    exp = np.full((m, n), np.nan, np.float32)
    ids0 = np.nonzero((otype == 0) & (status == 0))[0].astype(np.int32)
    for e in range(m):
        for ids in (ids0, ids1):
            assert oracle.map_obs(exp, e, fields[e], nl, ids, fi, fj, fk, three_d=three_d, ktop=ktop, periodic_i=1,
                                  offset=offset, offset_kind=offset_kind, skip_bad=True) == 0
    exp, est, enbad = oracle.finish_HE(exp, status, mode=0, nmem_dynamic=m, skip_bad=True)
    assert same_bits(got, exp)
    assert np.array_equal(st, est) and nbad == enbad


def test_he_bad_forecasts_and_positions(ctx):
    rng = np.random.default_rng(5)
    ni, nj, m, n = 30, 20, 4, 400
    nl = np.ones((nj, ni), np.int32)
    fields = rng.normal(15.0, 1.0, (m, nj, ni)).astype(np.float32)
    fi = rng.uniform(0.0, ni - 1.0, n)
    fj = rng.uniform(0.0, nj - 1.0, n)
    fi[17], fj[17] = 4.0, 6.0                                   # exactly on cell (6, 4)
    fields[2, 6, 4] = 5e6                                       # beyond MAXOBSVAL
    fields[1, 6, 4] = np.inf
    exp = np.full((m, n), np.nan, np.float32)
    ids = np.arange(n, dtype=np.int32)
    for e in range(m):
        oracle.map_obs(exp, e, fields[e], nl, ids, fi, fj, skip_bad=True)
    first_bad = int(np.nonzero(np.isnan(exp).any(0))[0].min())   # the device names the lowest id
    setup_obs(ctx, fi, fj)
    ctx.begin_HE(m)
    with pytest.raises(Exception) as ei:
        ctx.map_obs(0, fields, nl)
    assert getattr(ei.value, "status", None) == 5 and f"obs # {first_bad}:" in str(ei.value)
    # with --skip-bad-forecast-obs: NaN, then STATUS_BADFC
    ctx.begin_HE(m)
    ctx.map_obs(0, fields, nl, skip_bad=True)
    nbad, st = ctx.finish_HE(skip_bad=True)
    got = ctx.get_S()[0]
    exp, est, enbad = oracle.finish_HE(exp, np.zeros(n, np.int16), mode=0, nmem_dynamic=m, skip_bad=True)
    assert same_bits(got, exp) and np.array_equal(st, est) and nbad == enbad >= 1 and st[17] == 10
    # a position off the grid is an argument error
    fi2 = fi.copy()
    fi2[3] = -1.5
    setup_obs(ctx, fi2, fj)
    ctx.begin_HE(m)
    with pytest.raises(Exception) as ei:
        ctx.map_obs(0, fields, nl, skip_bad=True)
    assert getattr(ei.value, "status", None) == 1 and "obs # 3:" in str(ei.value)


@pytest.mark.parametrize("mode", [1, 2])
def test_he_enoi_and_hybrid_finish(ctx, mode):
    rng = np.random.default_rng(20 + mode)
    ni, nj, m, md, n, gamma = 40, 30, 9, 6, 3000, 0.5
    nl = np.ones((nj, ni), np.int32)
    fields = rng.normal(15.0, 1.0, (m, nj, ni)).astype(np.float32)
    bg = rng.normal(15.0, 1.0, (1, nj, ni)).astype(np.float32)
    fi = rng.uniform(0.0, ni - 1.0, n)
    fj = rng.uniform(0.0, nj - 1.0, n)
    setup_obs(ctx, fi, fj)
    enoi = mode == 1
    ctx.begin_HE(m, m if enoi else md, with_background=enoi)
    ctx.map_obs(0, fields, nl)
    if enoi:
        ctx.map_obs(0, bg, nl, mem0=-1)
    ctx.finish_HE(mode=mode, gamma=gamma)
    got = ctx.get_S()[0]

    exp = np.full((m, n), np.nan, np.float32)
    hx = np.full((1, n), np.nan, np.float32)
    ids = np.arange(n, dtype=np.int32)
    for e in range(m):
        oracle.map_obs(exp, e, fields[e], nl, ids, fi, fj)
    oracle.map_obs(hx, 0, bg[0], nl, ids, fi, fj)
    exp, _, _ = oracle.finish_HE(exp, np.zeros(n, np.int16), mode=mode, nmem_dynamic=m if enoi else md,
                                 gamma=gamma, Hx=hx[0] if enoi else None)
    assert same_bits(got, exp)


def test_he_cycle_matches_set_HE(ctx, gpu_lib):
    """Device HE -> innovations -> standardisation -> transforms gives the
    transforms that the same HE given through enkfg_set_HE gives."""
    w = synth.make(1, scale=0.5)
    fields = w.fields[0, 0]                      # [m][nj][ni], the observed layer
    fi = w.lon.astype(np.float64)                # cell units: x = i, y = j
    fj = w.lat.astype(np.float64)
    nl, lr, lw = oracle.locrad_table(w.ntypes, w.locrad)
    ctx.set_obstypes(nl, lr, lw, np.ones(w.ntypes))
    ctx.set_obs(w.lon, w.lat, w.otype, w.status, w.estd, w.value)
    ctx.set_obs_positions(fi, fj)
    ctx.begin_HE(w.nmem)
    ctx.map_obs(0, fields, w.numlevels)
    ctx.finish_HE()
    HE_dev = ctx.get_S()[0]
    ctx.calcinnandspread()
    ctx.standardise()
    ctx.set_grid(w.x, w.y, stride=w.stride)
    a = ctx.calctransforms(mode=w.mode, scheme=w.scheme, want64=True, want_diag=False)

    exp = np.full((w.nmem, w.nobs), np.nan, np.float32)
    ids = np.arange(w.nobs, dtype=np.int32)
    for e in range(w.nmem):
        assert oracle.map_obs(exp, e, fields[e], w.numlevels, ids, fi, fj) == 0
    assert same_bits(HE_dev, exp)
    c2 = gpu_lib.Enkfg(0)
    try:
        c2.set_obstypes(nl, lr, lw, np.ones(w.ntypes))
        c2.set_obs(w.lon, w.lat, w.otype, w.status, w.estd, w.value)
        c2.set_HE(exp)
        c2.calcinnandspread()
        c2.standardise()
        c2.set_grid(w.x, w.y, stride=w.stride)
        b = c2.calctransforms(mode=w.mode, scheme=w.scheme, want64=True, want_diag=False)
    finally:
        c2.close()
    assert np.array_equal(a["T64"], b["T64"]) and np.array_equal(a["w64"], b["w64"])


def test_he_device_pointer_form(ctx):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(9)
    ni, nj, nk, m, n = 50, 35, 4, 6, 2000
    nl = rng.integers(1, nk + 1, (nj, ni)).astype(np.int32)
    fields = rng.normal(15.0, 2.0, (m, nk, nj, ni)).astype(np.float32)
    fi = rng.uniform(0.0, ni - 1.0, n)
    fj = rng.uniform(0.0, nj - 1.0, n)
    fk = rng.uniform(0.0, nk - 1.0, n).astype(np.float32)
    setup_obs(ctx, fi, fj, fk)
    # wet-level counts leave some positions with every corner dry: those
    # forecasts are NaN (skip_bad), in both forms alike
    ctx.begin_HE(m)
    ctx.map_obs(0, fields, nl, three_d=True, ksurf=0, skip_bad=True)
    ctx.finish_HE()
    host = ctx.get_S()[0]
    f_d = torch.from_numpy(fields).cuda()
    nl_d = torch.from_numpy(nl).cuda()
    ids_d = torch.arange(n, dtype=torch.int32, device="cuda")
    ctx.begin_HE(m)
    ctx.map_obs_dev(0, f_d.data_ptr(), m, ni, nj, nl_d.data_ptr(), nk=nk, ids_ptr=ids_d.data_ptr(), nids=n,
                    three_d=True, ksurf=0, skip_bad=True)
    ctx.finish_HE()
    assert same_bits(ctx.get_S()[0], host)
