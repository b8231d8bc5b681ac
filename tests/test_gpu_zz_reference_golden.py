"""The GPU transform stage against the reference's own das_calctransforms
(tests/golden/calctransforms.npz: calc/transforms.c and the files it calls,
compiled unmodified, on a two-type workload with rejected observations at
stride 3; the float T, w and diagnostics it writes).

Tolerances (the contract of the plain FP64 path, test_gpu_calc.py): local
counts bit-exact; float T and w within 2 float ulps (w: or 1e-6 relative);
dfs within 1e-6, srf 1e-5, per-type pdfs 1e-5 and psrf 1e-4 relative to the
largest value.
"""
import os

import numpy as np
import pytest

import oracle
from helpers import max_ulps32, rel

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name,mode,scheme", [("etkf", 0, 1), ("denkf", 0, 0)])
def test_transforms_against_reference_calctransforms(ctx, name, mode, scheme):
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "calctransforms.npz"))
    nt = int(g["otype"].max()) + 1
    nl, lr, lw = oracle.locrad_table(nt, float(g["locrad"]))
    n = g["lon"].size
    m = int(g["nmem"])
    ctx.set_obstypes(nl, lr, lw, np.ones(nt))
    ctx.set_obs(g["lon"], g["lat"], g["otype"], g["status"], np.ones(n, np.float32), np.zeros(n, np.float32))
    ctx.set_S(g["S"], g["s"], m)
    ctx.set_grid(g["x"], g["y"], stride=int(g["stride"]))
    alpha = float(g[f"{name}_alpha"])
    out = ctx.calctransforms(mode=mode, scheme=scheme, alpha=alpha, path=0, want64=False, want_diag=True)
    assert np.array_equal(out["nlobs"], g[f"{name}_nlobs"])
    assert np.array_equal(out["pnlobs"], g[f"{name}_pnlobs"])
    assert max_ulps32(out["T"], g[f"{name}_T"]) <= 2
    assert max_ulps32(out["w"], g[f"{name}_w"]) <= 2 or rel(out["w"], g[f"{name}_w"]) < 1e-6
    assert rel(out["dfs"], g[f"{name}_dfs"]) < 1e-6
    assert rel(out["srf"], g[f"{name}_srf"]) < 1e-5
    assert rel(out["pdfs"], g[f"{name}_pdfs"]) < 1e-5
    assert rel(out["psrf"], g[f"{name}_psrf"]) < 1e-4
    # the batched path (the solve leaves the transform kernel)
    out = ctx.calctransforms(mode=mode, scheme=scheme, alpha=alpha, path=1, want64=False, want_diag=False)
    assert max_ulps32(out["T"], g[f"{name}_T"]) <= 2
    assert max_ulps32(out["w"], g[f"{name}_w"]) <= 2 or rel(out["w"], g[f"{name}_w"]) < 1e-6
