"""Parity of the GPU transform stage with the CPU oracle (through the C ABI).

Tolerances (the contract of the plain FP64 path):
  * local-observation lists, counts, stride/point indexing: bit-exact
    (same obs ids, id-sorted; taper coefficients bit-identical);
  * double T and w before the float cast: relative error <= 1e-10
    (max |a - b| / max |b| per point);
  * float T and w: within 2 float ulps of the oracle's cast;
  * nlobs bit-exact; dfs/srf/pdfs/psrf relative error <= 1e-6.
"""
import numpy as np
import pytest

import oracle
import synth
from helpers import gpu_setup, max_ulps32, obsset, prepare, rel

pytestmark = pytest.mark.gpu


def per_point_rel(a, b):
    a = a.reshape(-1, *a.shape[2:]).reshape(a.shape[0] * a.shape[1], -1)
    b = b.reshape(-1, *b.shape[2:]).reshape(b.shape[0] * b.shape[1], -1)
    den = np.maximum(np.abs(b).max(axis=1), 1e-300)
    return float((np.abs(a - b).max(axis=1) / den).max())


def check_lists(ctx, w, obs):
    counts, offsets, ids, coeffs = ctx.findlocal(lists=True)
    for pt in range(w.nanalyses):
        jj, ii = divmod(pt, w.ni_s)
        rid, rlc = obs.findlocal(w.x[ii * w.stride], w.y[jj * w.stride])
        order = np.argsort(rid, kind="stable")
        a, b = offsets[pt], offsets[pt + 1]
        assert counts[jj, ii] == rid.size, (pt, counts[jj, ii], rid.size)
        assert np.array_equal(ids[a:b], rid[order]), pt
        assert np.array_equal(coeffs[a:b], rlc[order]), pt


def test_local_obs_bitexact_workload1(ctx):
    w = synth.make(1, with_fields=False)
    S, s = prepare(w)
    obs, tabs = obsset(w)
    gpu_setup(ctx, w, S, s, tabs)
    check_lists(ctx, w, obs)


def test_local_obs_bitexact_multitype_multiradius(ctx):
    w = synth.make(2, scale=0.08, with_fields=False)
    S, s = prepare(w)
    radii = [[6.0, 2.5], [4.0]]
    obs, tabs = obsset(w, radii)
    nl, lr, lw = tabs
    lw[0, :2] = [0.6, 0.4]
    obs = oracle.ObsSet(w.lon, w.lat, w.otype, w.status, w.ntypes, nl, lr, lw)
    st = w.status.copy()
    st[::17] = 1                       # some rejected observations
    w.status = st
    obs = oracle.ObsSet(w.lon, w.lat, w.otype, st, w.ntypes, nl, lr, lw)
    gpu_setup(ctx, w, S, s, (nl, lr, lw))
    check_lists(ctx, w, obs)


def test_local_obs_golden_kdtree(ctx):
    """Neighbour sets against the reference kd-tree's own output."""
    import os
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "kdtree.npz"))
    ntypes = int(g["otype"].max()) + 1
    nl, lr, lw = oracle.locrad_table(ntypes, [[float(r)] for r in g["r"]])
    n = g["lon"].size
    ctx.set_obstypes(nl, lr, lw, np.ones(ntypes))
    ctx.set_obs(g["lon"], g["lat"], g["otype"], np.zeros(n, np.int16), np.ones(n, np.float32), np.zeros(n, np.float32))
    q = g["q"]
    # the queries as a curvilinear "grid" of 1 x nq points
    ctx.set_S(np.zeros((4, n), np.float32), np.zeros(n), 4)
    ctx.set_grid(x2d=q[:, 0][None, :], y2d=q[:, 1][None, :], stride=1)
    counts, offsets, ids, coeffs = ctx.findlocal(lists=True)
    for k in range(q.shape[0]):
        ref = np.sort(np.concatenate([g[f"t{t}_q{k}_ids"] for t in range(ntypes)]))
        assert np.array_equal(ids[offsets[k]:offsets[k + 1]], ref), k


@pytest.mark.parametrize("path", [0, 1])
def test_transforms_etkf_workload1(ctx, path):
    w = synth.make(1, with_fields=False)
    S, s = prepare(w)
    obs, tabs = obsset(w)
    ref = oracle.calctransforms(obs, mode=0, scheme=1, nmem=w.nmem, nmem_dynamic=w.nmem, alpha=1.0, stride=1,
                                x=w.x, y=w.y, S=S, s=s, want64=True, threads=4)
    gpu_setup(ctx, w, S, s, tabs)
    out = ctx.calctransforms(mode=0, scheme=1, alpha=1.0, path=path, want64=True)
    assert np.array_equal(out["nlobs"], ref["nlobs"])
    assert per_point_rel(out["T64"], ref["T64"]) < 1e-10
    assert per_point_rel(out["w64"], ref["w64"]) < 1e-10
    assert max_ulps32(out["T"], ref["T"]) <= 2
    assert max_ulps32(out["w"], ref["w"]) <= 2 or rel(out["w"], ref["w"]) < 1e-6
    assert rel(out["dfs"], ref["dfs"]) < 1e-6
    assert rel(out["srf"], ref["srf"]) < 1e-5
    assert np.array_equal(out["pnlobs"], ref["pnlobs"])
    assert rel(out["pdfs"], ref["pdfs"]) < 1e-6


def test_transforms_against_reference_golden(ctx):
    import os
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "transforms.npz"))
    nl, lr, lw = oracle.locrad_table(1, float(g["locrad"]))
    n = g["lon"].size
    ctx.set_obstypes(nl, lr, lw, np.ones(1))
    ctx.set_obs(g["lon"], g["lat"], g["otype"], g["status"], np.ones(n, np.float32), np.zeros(n, np.float32))
    ctx.set_S(g["S"], g["s"])
    ctx.set_grid(g["x"], g["y"], stride=int(g["stride"]))
    out = ctx.calctransforms(mode=int(g["mode"]), scheme=int(g["scheme"]), want64=True)
    T64 = out["T64"].reshape(-1, *out["T64"].shape[2:])
    w64 = out["w64"].reshape(-1, out["w64"].shape[-1])
    for k, pt in enumerate(g["pts"]):
        assert rel(T64[pt], g["T64"][k]) < 1e-10
        if np.abs(g["w64"][k]).max() > 0:
            assert rel(w64[pt], g["w64"][k]) < 1e-10


@pytest.mark.parametrize("mode,scheme", [(0, 0), (1, 0), (0, 1)])
def test_transforms_multitype_stride(ctx, mode, scheme):
    """Workload-2 shapes (2 obs types, land, swaths, stride 3) at reduced size,
    DEnKF / EnOI / ETKF, per-type diagnostics, plain and batched paths."""
    w = synth.make(2, scale=0.1, nobs=6000, with_fields=False, nmem=20)
    w.locrad = 12.0
    S, s = prepare(w)
    obs, tabs = obsset(w)
    ref = oracle.calctransforms(obs, mode=mode, scheme=scheme, nmem=w.nmem, nmem_dynamic=w.nmem, alpha=0.7,
                                stride=w.stride, x=w.x, y=w.y, S=S, s=s, want64=True, threads=4)
    gpu_setup(ctx, w, S, s, tabs)
    for path in (0, 1):
        out = ctx.calctransforms(mode=mode, scheme=scheme, alpha=0.7, path=path, want64=True)
        assert np.array_equal(out["nlobs"], ref["nlobs"])
        assert np.array_equal(out["pnlobs"], ref["pnlobs"])
        if mode != 1:
            assert per_point_rel(out["T64"], ref["T64"]) < 1e-10
        assert per_point_rel(out["w64"], ref["w64"]) < 1e-10
        assert rel(out["dfs"], ref["dfs"]) < 1e-6
        assert rel(out["pdfs"], ref["pdfs"]) < 1e-5
        assert rel(out["psrf"], ref["psrf"]) < 1e-4


@pytest.mark.parametrize("mode,scheme", [(0, 0), (1, 0), (0, 1)])
def test_transforms_batched_solvers(ctx, mode, scheme):
    """Without per-type diagnostics the solve leaves the transform kernel: the
    batched DEnKF/EnOI inverse and the batched ETKF eigensolver, plain and
    batched paths, against the FP64 oracle."""
    w = synth.make(2, scale=0.1, nobs=6000, with_fields=False, nmem=20)
    w.locrad = 12.0
    S, s = prepare(w)
    obs, tabs = obsset(w)
    ref = oracle.calctransforms(obs, mode=mode, scheme=scheme, nmem=w.nmem, nmem_dynamic=w.nmem, alpha=0.7,
                                stride=w.stride, x=w.x, y=w.y, S=S, s=s, want64=True, threads=4)
    gpu_setup(ctx, w, S, s, tabs)
    for path in (0, 1):
        out = ctx.calctransforms(mode=mode, scheme=scheme, alpha=0.7, path=path, want64=True, want_diag=False)
        if mode != 1:
            assert per_point_rel(out["T64"], ref["T64"]) < 1e-10
        assert per_point_rel(out["w64"], ref["w64"]) < 1e-10


def test_transforms_hybrid_dynamic_subset(ctx):
    """m_dyn < m (hybrid): T is the leading m_dyn columns."""
    w = synth.make(1, scale=0.5, with_fields=False)
    w.nmem_dynamic = 16
    S, s = prepare(w)
    obs, tabs = obsset(w)
    ref = oracle.calctransforms(obs, mode=2, scheme=1, nmem=w.nmem, nmem_dynamic=16, alpha=1.0, stride=1, x=w.x,
                                y=w.y, S=S, s=s, want64=True)
    gpu_setup(ctx, w, S, s, tabs)
    out = ctx.calctransforms(mode=2, scheme=1, want64=True)
    assert out["T"].shape[-2:] == (16, w.nmem)
    assert per_point_rel(out["T64"], ref["T64"]) < 1e-10


def test_innovations_and_standardise_bitexact(ctx):
    w = synth.make(1, with_fields=False)
    w.status = w.status.copy()
    w.status[5] = 2
    S_ref, s_f_ref, std_ref = oracle.calcinnandspread(w.HE, w.value, w.status)
    nl, lr, lw = oracle.locrad_table(1, w.locrad)
    ctx.set_obstypes(nl, lr, lw, np.array([2.0]))
    ctx.set_obs(w.lon, w.lat, w.otype, w.status, w.estd, w.value)
    ctx.set_HE(w.HE)
    s_f, std_f = ctx.calcinnandspread()
    assert np.array_equal(s_f, s_f_ref)
    assert np.array_equal(std_f, std_ref)
    S_d, _ = ctx.get_S()
    assert np.array_equal(S_d, S_ref)
    ctx.standardise()
    S2, s2 = oracle.standardise(S_ref, s_f_ref, w.estd, w.otype, np.array([2.0]))
    S_d, s_d = ctx.get_S()
    assert np.array_equal(S_d, S2)
    assert np.array_equal(s_d, s2)


def test_empty_and_edge_points(ctx):
    """Points with no local obs (T = I, w = 0) and a point far outside."""
    w = synth.make(1, scale=0.25, nobs=40, with_fields=False)
    w.locrad = 3.0
    S, s = prepare(w)
    obs, tabs = obsset(w)
    ref = oracle.calctransforms(obs, mode=0, scheme=1, nmem=w.nmem, nmem_dynamic=w.nmem, alpha=1.0, stride=1,
                                x=w.x, y=w.y, S=S, s=s, want64=True)
    gpu_setup(ctx, w, S, s, tabs)
    out = ctx.calctransforms(mode=0, scheme=1, want64=True)
    assert (ref["nlobs"] == 0).any()
    assert np.array_equal(out["nlobs"], ref["nlobs"])
    z = ref["nlobs"] == 0
    assert np.array_equal(out["T"][z], ref["T"][z])
    assert np.all(out["w"][z] == 0)
    assert per_point_rel(out["T64"], ref["T64"]) < 1e-10


@pytest.mark.parametrize("mode,scheme,prec", [(0, 1, 0), (0, 0, 0), (0, 1, 1)])
def test_transforms_at_point_logs(ctx, mode, scheme, prec):
    """Transforms at point-log positions (the recipe of a 1 x n curvilinear
    "grid" of log points, as das_calcpointlogtransforms needs them at
    arbitrary positions), plain and batched paths: local counts bit-exact,
    T and w against the oracle at the same positions.  One log point lies
    outside the observed region (T = I, w = 0)."""
    w = synth.make(1, scale=0.5, with_fields=False)
    S, s = prepare(w)
    obs, tabs = obsset(w)
    rng = np.random.default_rng(11)
    n = 37
    px = rng.uniform(w.x.min(), w.x.max(), n)
    py = rng.uniform(w.y.min(), w.y.max(), n)
    px[5], py[5] = w.x.max() + 10 * w.locrad, w.y.max() + 10 * w.locrad
    x2d, y2d = px[None, :], py[None, :]
    ref = oracle.calctransforms(obs, mode=mode, scheme=scheme, nmem=w.nmem, nmem_dynamic=w.nmem, alpha=1.0,
                                stride=1, x=px, y=py, S=S, s=s, want64=True, x2d=x2d, y2d=y2d)
    gpu_setup(ctx, w, S, s, tabs)
    ctx.set_grid(x2d=x2d, y2d=y2d, stride=1)
    assert (ctx.nj, ctx.ni) == (1, n)
    assert ref["nlobs"][0, 5] == 0 and (ref["nlobs"] > 0).sum() == n - 1
    tol = 1e-10 if prec == 0 else 1e-5     # the FP64 and the mixed-precision contracts
    for path in ((0, 1) if prec == 0 else (1,)):
        out = ctx.calctransforms(mode=mode, scheme=scheme, alpha=1.0, path=path, precision=prec, want64=True)
        assert np.array_equal(out["nlobs"], ref["nlobs"])
        assert per_point_rel(out["T64"], ref["T64"]) < tol, path
        assert per_point_rel(out["w64"], ref["w64"]) < tol, path
        assert np.array_equal(out["T"][0, 5], np.eye(w.nmem, dtype=np.float32))
        assert np.all(out["w"][0, 5] == 0)


def test_errors_are_status_codes(ctx, gpu_lib):
    with pytest.raises(gpu_lib.EnkfgError) as e:
        ctx.set_obstypes(np.array([0], np.int32), np.zeros(8))
    assert e.value.status == 1
    c2 = gpu_lib.Enkfg(0)
    with pytest.raises(gpu_lib.EnkfgError) as e:
        c2.calctransforms()
    assert e.value.status == 7
    # a strided point without coordinates (a grid of type NONE) is refused
    nl, lr, lw = oracle.locrad_table(1, 5.0)
    c2.set_obstypes(nl, lr, lw, np.ones(1))
    with pytest.raises(gpu_lib.EnkfgError) as e:
        c2.set_grid(x2d=np.array([[0.0, np.nan]]), y2d=np.array([[0.0, 1.0]]), stride=1)
    assert e.value.status == 8
    c2.close()


# (precision, mode, scheme, workload, members): the three batched solves --
# the refined mixed ETKF solve, the FP64 eigensolver and the FP64 inverse
SPLIT_CASES = [(1, 0, 1, 3, 96), (0, 0, 1, 3, 48), (0, 0, 0, 2, 48), (1, 0, 0, 2, 48)]


@pytest.mark.parametrize("case", SPLIT_CASES, ids=["mixed_etkf_m96", "fp64_etkf_m48", "fp64_denkf_m48",
                                                   "mixed_denkf_m48"])
def test_transforms_in_several_solve_batches(ctx, case):
    """The batched path in batches of 1,024 and 2,048 points (the queue is
    then sorted within each batch, and the host outputs leave batch by
    batch) gives the same T and w, bit for bit, as one batch."""
    prec, mode, scheme, cfg, m = case
    w = synth.make(cfg, scale=0.15 if cfg == 3 else 0.35, nmem=m, with_fields=False)
    S, s = prepare(w)
    _, tabs = obsset(w)
    gpu_setup(ctx, w, S, s, tabs)
    npts = w.nj_s * w.ni_s
    assert npts > 4096
    one = ctx.calctransforms(mode=mode, scheme=scheme, path=1, precision=prec, want_diag=False)
    for b in (1024, 2048):
        ctx.set_solve_batch(b)
        try:
            got = ctx.calctransforms(mode=mode, scheme=scheme, path=1, precision=prec, want_diag=False)
        finally:
            ctx.set_solve_batch(0)
        assert np.array_equal(got["w"], one["w"]), (case, b)
        assert np.array_equal(got["T"], one["T"]), (case, b)
