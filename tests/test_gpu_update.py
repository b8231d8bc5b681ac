"""Parity of the GPU update stage (das_updatefields / das_updatebg /
das_sethybridensemble) with the CPU oracle, through the C ABI.

Tolerances: the reference applies X5 with a float sgemv whose summation order
is the BLAS's; the device sums in its own order, so analysis fields agree to
float rounding: |a - b| <= 2e-5 * max(1, |b|) (fields here are O(15)).
Masked cells, missing values and the EnOI/hybrid kernels, which follow the
reference's operation order exactly, are compared bit for bit.
"""
import numpy as np
import pytest

import oracle
import synth
from helpers import gpu_setup, obsset, prepare

pytestmark = pytest.mark.gpu


def close(a, b, tol=2e-5):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float((np.abs(a - b) / np.maximum(1.0, np.abs(b))).max())


def transforms(ctx, w, mode=0, scheme=1):
    S, s = prepare(w)
    obs, tabs = obsset(w)
    gpu_setup(ctx, w, S, s, tabs)
    return ctx.calctransforms(mode=mode, scheme=scheme, alpha=1.0, want_diag=False)


def run_both(ctx, w, out, fields, levels, **kw):
    nfield = fields.shape[0]
    got = ctx.updatefields(fields, w.numlevels, levels, **kw)
    ref = np.empty_like(fields)
    okw = dict(kw)
    okw.pop("precision", None)
    mode = okw.pop("mode", 0)
    nmem = okw.pop("nmem", w.nmem)
    nmd = okw.pop("nmem_dynamic", w.nmem_dynamic)
    j2 = okw.pop("j2", -1)
    j1 = okw.get("j1", 0)
    for f in range(nfield):
        ref[f] = oracle.updatefields(fields[f], out["T"], out["w"], w.numlevels, mode=mode, nmem=nmem,
                                     nmem_dynamic=nmd, stride=w.stride, level=int(levels[f]),
                                     j2=None if j2 < 0 else j2, **okw)
    return got, ref


def test_update_stride1_inflation(ctx):
    w = synth.make(1)
    out = transforms(ctx, w)
    fields = w.fields[0]                       # [1 layer][m][nj][ni]
    got, ref = run_both(ctx, w, out, fields, np.array([0]), inflation=1.05)
    assert close(got, ref) < 2e-5
    assert not np.array_equal(got, fields)


@pytest.mark.parametrize("precision", [0, 1])
def test_update_stride3_mask_layers(ctx, precision):
    w = synth.make(2, scale=0.1, nobs=5000, nmem=24)
    w.locrad = 10.0
    out = transforms(ctx, w, mode=0, scheme=0)
    fl = w.fields.reshape(-1, *w.fields.shape[2:])          # [nf*nl][m][nj][ni]
    levels = np.tile(np.arange(w.nlayers), w.nfields)
    nl = w.numlevels.copy()
    nl[nl > 0] = np.random.default_rng(0).integers(1, w.nlayers + 1, (nl > 0).sum())
    w.numlevels = nl
    got, ref = run_both(ctx, w, out, fl, levels, inflation=1.1, inf_ratio=0.5, precision=precision)
    assert close(got, ref) < 2e-5
    masked = nl[None, :, :] <= levels[:, None, None]
    assert np.all(got.transpose(1, 0, 2, 3)[:, masked] == 0.0)


def test_update_missing_values_increment_log_periodic(ctx):
    w = synth.make(1, scale=0.5)
    w.stride = 2
    out = transforms(ctx, w)
    fields = w.fields[0].copy()
    fields[0, 3, 5, 7] = np.nan                 # dynamic member missing -> cell zeroed
    fields[0, 0, 9, 9] = 2.0e6                  # |v| > MAXOBSVAL
    got, ref = run_both(ctx, w, out, fields, np.array([0]), output_increment=1)
    assert close(got, ref) < 2e-5
    assert np.all(got[0, :, 5, 7] == 0) and np.all(got[0, :, 9, 9] == 0)
    lg = np.log10(np.abs(w.fields[0]) + 1).astype(np.float32)
    got, ref = run_both(ctx, w, out, lg, np.array([0]), output_increment=1, applylog=1)
    assert close(got, ref, 1e-4) < 1e-4


def test_update_periodic_and_tile(ctx):
    w = synth.make(1, scale=0.5)
    w.stride = 3
    S, s = prepare(w)
    obs, tabs = obsset(w)
    nl, lr, lw = tabs
    ctx.set_obstypes(nl, lr, lw, np.ones(1))
    ctx.set_obs(w.lon, w.lat, w.otype, w.status, w.estd, w.value)
    ctx.set_S(S, s)
    ctx.set_grid(w.x, w.y, stride=3, periodic_i=True)
    out = ctx.calctransforms(mode=0, scheme=1, want_diag=False)
    fields = w.fields[0]
    got = ctx.updatefields(fields, w.numlevels, [0])
    ref = oracle.updatefields(fields[0], out["T"], out["w"], w.numlevels, mode=0, nmem=w.nmem,
                              nmem_dynamic=w.nmem, stride=3, periodic_i=1)
    assert close(got[0], ref) < 2e-5
    # a field tile (FIELDSPLIT) of rows 6..20
    sub = fields[:, :, 6:21, :]
    got = ctx.updatefields(sub, w.numlevels, [0], j1=6, j2=20)
    ref = oracle.updatefields(sub[0], out["T"], out["w"], w.numlevels, mode=0, nmem=w.nmem, nmem_dynamic=w.nmem,
                              stride=3, periodic_i=1, j1=6, j2=20)
    assert close(got[0], ref) < 2e-5


@pytest.mark.parametrize("precision", [0, 1])
def test_update_hybrid(ctx, precision):
    w = synth.make(1, scale=0.5, nmem=24)
    w.nmem_dynamic = 16
    out = transforms(ctx, w, mode=2)
    v = w.fields[0, 0].reshape(w.nmem, -1)
    hv = ctx.sethybridensemble(v, 16, 0.5)
    rv, _ = oracle.sethybridensemble(v, 16, 0.5)
    assert np.array_equal(hv, rv)
    fields = hv.reshape(1, w.nmem, w.nj, w.ni)
    got, ref = run_both(ctx, w, out, fields, np.array([0]), mode=2, nmem=24, nmem_dynamic=16, inflation=1.02,
                        inf_ratio=0.3, precision=precision)
    assert close(got, ref) < 2e-5


def test_update_large_ensemble_many_layers(ctx):
    """m = 96 (three members per lane) and more field-layers than one register block."""
    w = synth.make(3, scale=0.06, nobs=3000, nmem=96)
    w.nlayers = 10
    out = transforms(ctx, w)
    fl = w.fields.reshape(-1, *w.fields.shape[2:])
    levels = np.tile(np.arange(w.fields.shape[1]), w.fields.shape[0])
    for precision in (0, 1):
        got, ref = run_both(ctx, w, out, fl, levels, inflation=1.03, precision=precision)
        assert close(got, ref) < 2e-5


def test_update_enoi_bg_bitexact(ctx):
    w = synth.make(1, scale=0.5)
    w.stride = 2
    out = transforms(ctx, w, mode=1, scheme=0)
    m = w.nmem
    fields = np.concatenate([w.fields[0, 0], w.fields[0, 0].mean(0, keepdims=True)], 0)[None]
    nl = w.numlevels.copy()
    nl[::5, ::7] = 0
    w.numlevels = nl
    got = ctx.updatebg(fields, nl, [0], nmem=m, nmem_dynamic=m)
    ref = oracle.updatebg(fields[0], out["w"], nl, nmem=m, stride=2)
    assert np.array_equal(got[0], ref)


def _golden_update():
    import os
    return np.load(os.path.join(os.path.dirname(__file__), "golden", "update.npz"))


@pytest.mark.parametrize("precision", [0, 1])
def test_update_against_reference_golden(ctx, precision):
    """The device update against the reference's own update/update.c and
    common/dasystem.c (compiled unmodified; tests/golden/update.npz): every
    case of strides, periodic i, tiles, masks with surfk 0 and > 0, missing
    values, spread-capped inflation, increments, log fields, hybrid (the
    hybrid ensemble bit for bit) and EnOI (bit for bit, NaN payloads aside)."""
    g = _golden_update()
    nl1, lr1, lw1 = oracle.locrad_table(1, 5.0)
    for k, name in enumerate(g["names"]):
        mode, mnj, mni, m, md, stride, per, j1, j2, level, surfk, issv, inc, alog = [int(x) for x in g[f"u{k}_prm"]]
        infl, ratio = [float(x) for x in g[f"u{k}_infl"]]
        ctx.set_obstypes(nl1, lr1, lw1, np.ones(1))
        ctx.set_obs(np.array([1.0], np.float32), np.array([1.0], np.float32), np.zeros(1, np.int16),
                    np.zeros(1, np.int16), np.ones(1, np.float32), np.zeros(1, np.float32))
        ctx.set_grid(np.arange(mni, dtype=np.float64), np.arange(mnj, dtype=np.float64), stride=stride,
                     periodic_i=bool(per))
        ctx.set_transforms(None if mode == 1 else g[f"u{k}_T"], g[f"u{k}_w"], mode=mode, nmem=m,
                           nmem_dynamic=md if mode != 1 else m)
        if f"u{k}_hyb_in" in g.files:
            hv = ctx.sethybridensemble(g[f"u{k}_hyb_in"], md, 0.5)
            assert np.array_equal(hv, g[f"u{k}_hyb_out"]), name
        v = g[f"u{k}_v"][None]
        exp = g[f"u{k}_out"]
        got = ctx.updatefields(v, g[f"u{k}_numlevels"], [level], mode=mode, nmem=m,
                               nmem_dynamic=md if mode != 1 else m, surfk=surfk, issurfacevar=issv, inflation=infl,
                               inf_ratio=ratio, output_increment=inc, applylog=alog, j1=j1, j2=j2,
                               precision=precision)[0]
        if mode == 1:
            assert np.array_equal(got, exp, equal_nan=True), name
            continue
        # masked and missing cells are exact zeros in both
        assert np.array_equal(got == 0.0, exp == 0.0), name
        tol = 1e-4 if alog else 2e-5
        assert close(got, exp) < tol, (name, close(got, exp))


def test_update_streamed_groups_match_one_group(ctx):
    """The host-buffer update in groups of 1 and 3 field-layers (three device
    buffers in turn, copies overlapped on the copy streams), and in blocks of
    model rows, gives the same fields (and inflation) as one group, and as
    the oracle (m = 96 and m = 24 kernels)."""
    for nmem in (96, 24):
        w = synth.make(3, scale=0.06, nobs=3000, nmem=nmem)
        w.nlayers = 10
        out = transforms(ctx, w)
        fl = np.ascontiguousarray(w.fields.reshape(-1, *w.fields.shape[2:]))   # 20 field-layers
        levels = np.tile(np.arange(w.fields.shape[1]), w.fields.shape[0])
        ctx.set_field_buffer_size(0)
        whole = ctx.updatefields(fl, w.numlevels, levels, inflation=1.03, inf_ratio=0.4)
        for g in (1, 3):
            ctx.set_field_buffer_size(g)
            got = ctx.updatefields(fl, w.numlevels, levels, inflation=1.03, inf_ratio=0.4)
            assert np.array_equal(got, whole), (nmem, g)
        ctx.set_field_buffer_size(0)
        # blocks of model rows (a multiple of the stride, the last one
        # shorter), with the inflation output
        whole_f, whole_i = ctx.updatefields(fl, w.numlevels, levels, inflation=1.03, inf_ratio=0.4, want_infl=True)
        for g, rows in ((1, 1), (3, 5), (20, 7)):
            ctx.set_field_buffer_size(g)
            ctx.set_field_block_rows(rows)
            try:
                got_f, got_i = ctx.updatefields(fl, w.numlevels, levels, inflation=1.03, inf_ratio=0.4,
                                                want_infl=True)
            finally:
                ctx.set_field_buffer_size(0)
                ctx.set_field_block_rows(0)
            assert np.array_equal(got_f, whole_f), (nmem, g, rows)
            assert np.array_equal(got_i, whole_i), (nmem, g, rows)
        ref = np.stack([oracle.updatefields(fl[f], out["T"], out["w"], w.numlevels, mode=0, nmem=w.nmem,
                                            nmem_dynamic=w.nmem_dynamic, stride=w.stride, level=int(levels[f]),
                                            inflation=1.03, inf_ratio=0.4) for f in range(fl.shape[0])])
        assert close(whole, ref) < 2e-5


def test_randomise_against_reference_golden(ctx):
    """RANDOMISE (addnoise, update/update.c:46-87) after the update, against
    the reference's own das_updatefields with DEFLATION and SIGMA set
    (tests/golden/addnoise.npz: the normals its get_normalpair drew are
    inputs): the field within the update tolerance of the reference's, and
    the noise itself bit for bit (the randomised device field equals the
    oracle's addnoise of the device's plain update).  Host-buffer and
    device-buffer calls."""
    import os
    import torch
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "addnoise.npz"))
    nl1, lr1, lw1 = oracle.locrad_table(1, 5.0)
    dev = torch.device("cuda", 0)
    for k, name in enumerate(g["names"]):
        mode, mnj, mni, m, md, stride, per, inc, alog = [int(x) for x in g[f"n{k}_prm"]]
        defl, sigma = [float(x) for x in g[f"n{k}_noise"]]
        r = g[f"n{k}_random"][:m]
        ctx.set_obstypes(nl1, lr1, lw1, np.ones(1))
        ctx.set_obs(np.array([1.0], np.float32), np.array([1.0], np.float32), np.zeros(1, np.int16),
                    np.zeros(1, np.int16), np.ones(1, np.float32), np.zeros(1, np.float32))
        ctx.set_grid(np.arange(mni, dtype=np.float64), np.arange(mnj, dtype=np.float64), stride=stride,
                     periodic_i=bool(per))
        ctx.set_transforms(g[f"n{k}_T"], g[f"n{k}_w"], mode=mode, nmem=m, nmem_dynamic=md)
        kw = dict(mode=mode, nmem=m, nmem_dynamic=md, output_increment=inc, applylog=alog)
        v = g[f"n{k}_v"][None]
        plain = ctx.updatefields(v, g[f"n{k}_numlevels"], [0], **kw)[0]
        ctx.set_field_noise([defl], [sigma], r[None])
        got = ctx.updatefields(v, g[f"n{k}_numlevels"], [0], **kw)[0]
        assert np.array_equal(got, oracle.addnoise(plain, defl, sigma, r), equal_nan=True), name
        assert close(got, g[f"n{k}_out"]) < (1e-4 if alog else 2e-5), name
        # device buffers
        fd = torch.from_numpy(np.ascontiguousarray(v)).to(dev)
        nd = torch.from_numpy(g[f"n{k}_numlevels"]).to(dev)
        ctx.set_field_noise([defl], [sigma], r[None])
        ctx.updatefields_dev(fd.data_ptr(), nd.data_ptr(), 1, [0], **kw)
        torch.cuda.synchronize()
        assert np.array_equal(fd.cpu().numpy()[0], got, equal_nan=True), name
        # the noise is used up: the next update has none
        assert np.array_equal(ctx.updatefields(v, g[f"n{k}_numlevels"], [0], **kw)[0], plain, equal_nan=True)


def test_randomise_streamed_layers_and_blocks(ctx, gpu_lib):
    """Several field-layers, one without noise (NaN deflation), through the
    host-buffer pipeline in groups and row blocks: each layer is the oracle's
    addnoise of the plain device update with that layer's normals; a noise
    set for another layer count is refused."""
    w = synth.make(3, scale=0.06, nobs=3000, nmem=24)
    w.nlayers = 3
    transforms(ctx, w)
    fl = np.ascontiguousarray(w.fields.reshape(-1, *w.fields.shape[2:]))[:5]
    levels = [0, 1, 2, 0, 1]
    kw = dict(mode=0, nmem=w.nmem, nmem_dynamic=w.nmem, inflation=1.05)
    plain = ctx.updatefields(fl, w.numlevels, levels, **kw)
    rng = np.random.default_rng(4)
    defl = np.array([0.9, np.nan, 0.5, 0.99, 0.7])
    sigma = np.array([0.3, 0.3, 2.0, 0.05, 1.0])
    r = rng.standard_normal((5, w.nmem))
    want = plain.copy()
    for f in range(5):
        if not np.isnan(defl[f]):
            want[f] = oracle.addnoise(plain[f], defl[f], sigma[f], r[f])
    for g_, rows in ((1, 0), (2, 5), (5, 3)):
        ctx.set_field_buffer_size(g_)
        ctx.set_field_block_rows(rows)
        try:
            ctx.set_field_noise(defl, sigma, r)
            got = ctx.updatefields(fl, w.numlevels, levels, **kw)
        finally:
            ctx.set_field_buffer_size(0)
            ctx.set_field_block_rows(0)
        assert np.array_equal(got, want, equal_nan=True), (g_, rows)
    ctx.set_field_noise(defl[:4], sigma[:4], r[:4])
    with pytest.raises(gpu_lib.EnkfgError) as e:
        ctx.updatefields(fl, w.numlevels, levels, **kw)
    assert e.value.status == 1
