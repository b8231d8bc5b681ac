"""Shared set-up for the parity tests: one workload, the oracle and the GPU
library fed the same inputs."""
import numpy as np

import oracle
import synth


def prepare(w: "synth.Workload"):
    """Innovations + standardisation on the CPU oracle; returns (S, s)."""
    S, s_f, _ = oracle.calcinnandspread(w.HE, w.value, w.status)
    return oracle.standardise(S, s_f, w.estd, w.otype, np.ones(w.ntypes))


def obsset(w, locrad=None):
    nl, lr, lw = oracle.locrad_table(w.ntypes, w.locrad if locrad is None else locrad)
    return oracle.ObsSet(w.lon, w.lat, w.otype, w.status, w.ntypes, nl, lr, lw), (nl, lr, lw)


def gpu_setup(ctx, w, S=None, s=None, tables=None, from_HE=False):
    nl, lr, lw = tables if tables is not None else oracle.locrad_table(w.ntypes, w.locrad)
    ctx.set_obstypes(nl, lr, lw, np.ones(w.ntypes))
    ctx.set_obs(w.lon, w.lat, w.otype, w.status, w.estd, w.value)
    if from_HE:
        ctx.set_HE(w.HE, w.nmem_dynamic)
        ctx.calcinnandspread()
        ctx.standardise()
    else:
        ctx.set_S(S, s, w.nmem_dynamic)
    ctx.set_grid(w.x, w.y, stride=w.stride)


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    d = np.abs(a - b).max() if b.size else 0.0
    return float(d / max(np.abs(b).max(), 1e-300)) if b.size else 0.0


def max_ulps32(a, b):
    a = np.asarray(a, np.float32)
    b = np.asarray(b, np.float32)
    sp = np.spacing(np.maximum(np.abs(a), np.abs(b)).astype(np.float32))
    sp = np.maximum(sp, np.float32(1e-38))
    return float((np.abs(a.astype(np.float64) - b.astype(np.float64)) / sp).max())
