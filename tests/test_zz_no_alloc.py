"""enkfg_local_offsets_noalloc: the CSR offsets of local-observation counts
for callers that cannot allocate device memory (a pool or another framework
owns the device, allocation is forbidden after start-up, or the implicit
synchronisation of cudaMalloc/cudaFree is not acceptable).  It must give the
same offsets as enkfg_local_obs, which allocates its scan scratch, on two
calls in a row (the shared scratch array keeps the previous call's data).
This file is collected last so that a failure here comes after every other
test; it also passes alone in a fresh process."""
import ctypes as C

import numpy as np
import pytest

import oracle
import synth
from helpers import gpu_setup, obsset, prepare

pytestmark = pytest.mark.gpu


def existing_offsets(ctx, cfg, scale, radius):
    w = synth.make(cfg, scale=scale, with_fields=False)
    w.locrad = radius
    S, s = prepare(w)
    _, tabs = obsset(w)
    gpu_setup(ctx, w, S, s, tabs)
    counts, offsets, _, _ = ctx.findlocal(lists=True)
    return counts.reshape(-1).astype(np.int32), offsets


def noalloc_offsets(ctx, counts):
    import torch
    dev = torch.device("cuda", 0)
    c = torch.from_numpy(counts).to(dev)
    out = torch.full((counts.size + 1,), -7, dtype=torch.int64, device=dev)
    torch.cuda.synchronize()
    st = ctx.L.enkfg_local_offsets_noalloc(C.c_void_p(c.data_ptr()), C.c_longlong(counts.size),
                                           C.c_void_p(out.data_ptr()), None)
    torch.cuda.synchronize()
    assert st == 0, st
    return out.cpu().numpy()


def test_noalloc_offsets_match_existing_entry_point(ctx, gpu_lib):
    pytest.importorskip("torch")
    # first call: many points with large counts
    c1, o1 = existing_offsets(ctx, 1, 1.0, 20.0)
    got1 = noalloc_offsets(ctx, c1)
    assert np.array_equal(got1, o1)
    # second call in a row: fewer points, different counts; the scratch
    # still holds the first call's block sums
    c2, o2 = existing_offsets(ctx, 2, 0.1, 9.0)
    assert c2.size != c1.size
    got2 = noalloc_offsets(ctx, c2)
    assert np.array_equal(got2, o2)
    # more counts than one scan block (4096), and n = 0
    big = np.tile(c1, 3)
    ref = np.concatenate([[0], np.cumsum(big.astype(np.int64))])
    assert np.array_equal(noalloc_offsets(ctx, big), ref)
    assert np.array_equal(noalloc_offsets(ctx, np.zeros(0, np.int32)), np.zeros(1, np.int64))


def test_noalloc_rejects_sizes_beyond_the_limit(ctx, gpu_lib):
    st = ctx.L.enkfg_local_offsets_noalloc(C.c_void_p(16), C.c_longlong(134217729), C.c_void_p(16), None)
    assert st == 6          # ENKFG_ECAPACITY, checked before any device work
    st = ctx.L.enkfg_local_offsets_noalloc(None, C.c_longlong(10), None, None)
    assert st == 1          # ENKFG_EINVAL
