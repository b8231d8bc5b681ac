"""Workload 5's shape at reduced size: 51 levels, T and S fields, 40% land,
96 dynamic + 48 static members (hybrid, gamma 0.5), four observation types
(SST swaths, SSH tracks, T and S profiles), radius 40 cells, stride 3.

  * transforms of the plain FP64 path (nmem 144: the largest register block)
    against the FP64 oracle, 1e-10 relative on T (m_dyn x m) and w, on a
    sample of strided rows;
  * the update with the field-layers streamed through the device from host
    memory in groups (three device buffers, copies overlapped), after the
    hybrid conditioning of every layer, against the oracle (2e-5, float
    rounding of the X5 apply; the hybrid ensemble bit for bit).
"""
import numpy as np
import pytest

import oracle
import synth
from helpers import gpu_setup, obsset, prepare

pytestmark = pytest.mark.gpu


def per_point_rel(a, b):
    a = a.reshape(a.shape[0] * a.shape[1], -1)
    b = b.reshape(b.shape[0] * b.shape[1], -1)
    den = np.maximum(np.abs(b).max(axis=1), 1e-300)
    return float((np.abs(a - b).max(axis=1) / den).max())


def close(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float((np.abs(a - b) / np.maximum(1.0, np.abs(b))).max())


def test_workload5_shape_hybrid_transforms_and_streamed_update(ctx):
    w = synth.make(5, scale=0.03, nobs=3000)
    assert (w.nmem, w.nmem_dynamic, w.ntypes, w.mode) == (144, 96, 4, 2)
    S, s = prepare(w)
    obs, tabs = obsset(w)
    rows = [0, w.nj_s // 2, w.nj_s - 1]
    ref = oracle.calctransforms(obs, mode=w.mode, scheme=w.scheme, nmem=w.nmem, nmem_dynamic=w.nmem_dynamic,
                                alpha=1.0, stride=w.stride, x=w.x, y=w.y, S=S, s=s, rows=rows, threads=16,
                                want64=True)
    gpu_setup(ctx, w, S, s, tabs)
    out = ctx.calctransforms(mode=w.mode, scheme=w.scheme, path=1, precision=0, want64=True, want_diag=False)
    assert out["T"].shape[-2:] == (w.nmem_dynamic, w.nmem)
    assert per_point_rel(out["T64"][rows], ref["T64"][rows]) < 1e-10
    assert per_point_rel(out["w64"][rows], ref["w64"][rows]) < 1e-10

    # the update of every layer of one field (hybrid conditioning first),
    # the field-layers streamed in groups of 8
    f = 0
    layers = np.ascontiguousarray(w.fields[f])                  # [nl][m][nj][ni]
    hyb = np.stack([ctx.sethybridensemble(layers[k].reshape(w.nmem, -1), w.nmem_dynamic, w.gamma)
                    for k in range(w.nlayers)]).reshape(layers.shape)
    for k in (0, w.nlayers - 1):
        rv, _ = oracle.sethybridensemble(layers[k].reshape(w.nmem, -1), w.nmem_dynamic, w.gamma)
        assert np.array_equal(hyb[k].reshape(w.nmem, -1), rv)
    levels = np.arange(w.nlayers, dtype=np.int32)
    nl = np.full_like(w.numlevels, w.nlayers)
    nl[w.numlevels == 0] = 0
    # a sloping bottom: fewer wet levels towards one edge
    nl = np.where(nl > 0, np.minimum(nl, 5 + (np.arange(w.ni)[None, :] * (w.nlayers - 5)) // (w.ni - 1)), 0)
    nl = nl.astype(np.int32)
    ctx.set_field_buffer_size(8)
    try:
        got = ctx.updatefields(hyb, nl, levels, mode=w.mode, nmem=w.nmem, nmem_dynamic=w.nmem_dynamic,
                               inflation=1.02, inf_ratio=0.3)
    finally:
        ctx.set_field_buffer_size(0)
    for k in (0, 7, 8, w.nlayers - 1):
        exp = oracle.updatefields(hyb[k], out["T"], out["w"], nl, mode=w.mode, nmem=w.nmem,
                                  nmem_dynamic=w.nmem_dynamic, stride=w.stride, level=k, inflation=1.02,
                                  inf_ratio=0.3)
        assert close(got[k], exp) < 2e-5, k
