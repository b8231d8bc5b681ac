"""Seeded synthetic workloads for the EnKF-C analysis hot path.

The reference's example data sets are not available, so every workload is a
seeded synthetic stand-in with the shapes, sizes and value distributions of
the five workload definitions:

  1. 128x128, 1 layer, 1 field, no land, m=24, 3000 uniform obs (sigma 0.5),
     ETKF, radius 20, stride 1, inflation 1.05.
  2. 600x900 with a 30% land mask, 4 layers, 2 fields, m=48, 400k obs (70% on
     50 straight swaths 20 cells wide, 30% uniform over ocean, sigma U[0.3,0.8]),
     DEnKF, radius 30, stride 3.
  3. 1000x1000, 10 layers, 2 fields, m=96, 2M uniform obs (sigma 0.5), ETKF,
     radius 25, stride 2.
  4. grid/obs of workload 2 with m=64 plus an independent verifying field.
  5. 51 levels, 1500x3600, 40% land, T/S (3-D) + SSH (2-D), 96 dynamic + 48
     static members (hybrid, gamma 0.5), 14M obs, radius 40, stride 3.

Coordinates are in cell units with non-geographic distances (x = i, y = j,
radius in cells).  Gaussian random fields are white noise filtered in Fourier
space by a Gaussian kernel of the stated length scale and normalised to the
stated standard deviation.  Member e's forecast observation (HE) is the
bilinear interpolation of member e at the observation position.

Seeds: config_id * 1000 + stream, streams 0 background/ensemble, 1 truth,
2 obs locations, 3 obs noise, 4 land mask, 5 swaths, 6 static members.
"""
from __future__ import annotations

import dataclasses
from typing import Optional

import numpy as np


def _rng(cfg: int, stream: int) -> np.random.Generator:
    return np.random.default_rng(cfg * 1000 + stream)


def _fft_workers() -> int:
    import os
    return max(1, os.cpu_count() or 1)


def grf_filter(noise: np.ndarray, length: float, std: float = 1.0) -> np.ndarray:
    """Gaussian random fields from white noise [count][nj][ni] (float32): the
    noise filtered in Fourier space by a Gaussian kernel of the given length
    scale, each field centred and scaled to `std`."""
    import scipy.fft as sfft
    count, nj, ni = noise.shape
    ky = np.fft.fftfreq(nj)[:, None]
    kx = np.fft.rfftfreq(ni)[None, :]
    # Gaussian covariance exp(-r^2 / (2 L^2)) <-> amplitude filter exp(-pi^2 k^2 L^2)
    filt = np.exp(-(np.pi ** 2) * (kx ** 2 + ky ** 2) * length ** 2).astype(np.float32)
    wk = _fft_workers()
    out = np.empty((count, nj, ni), np.float32)
    step = 16
    for c0 in range(0, count, step):
        spec = sfft.rfft2(noise[c0:c0 + step], workers=wk)
        spec *= filt
        f = sfft.irfft2(spec, s=(nj, ni), workers=wk).astype(np.float32)
        f -= f.mean(axis=(1, 2), keepdims=True)
        sd = np.sqrt(np.einsum("kij,kij->k", f, f, dtype=np.float64) / (nj * ni))
        f *= (std / np.maximum(sd, 1e-30)).astype(np.float32)[:, None, None]
        out[c0:c0 + step] = f
    return out


def grf(rng: np.random.Generator, nj: int, ni: int, length: float, std: float = 1.0,
        count: int = 1) -> np.ndarray:
    """`count` independent Gaussian random fields [count][nj][ni] (float32)."""
    noise = rng.standard_normal((count, nj, ni), dtype=np.float32)
    return grf_filter(noise, length, std)


def _layer_noise(cfg: int, stream: int, f: int, k: int, count: int, nj: int, ni: int, ex=None) -> np.ndarray:
    """White noise of layer k of field f: every member draws from its own
    seeded generator (config * 1000 + stream, field, layer, member), so the
    values do not depend on how the draws are spread over threads."""
    out = np.empty((count, nj, ni), np.float32)

    def draw(e):
        np.random.default_rng([cfg * 1000 + stream, f, k, e]).standard_normal((nj, ni), dtype=np.float32,
                                                                               out=out[e])
    if ex is None:
        for e in range(count):
            draw(e)
    else:
        list(ex.map(draw, range(count)))
    return out


def ensemble_layers(cfg: int, nf: int, nl: int, m: int, md: int, nj: int, ni: int, length: float,
                    bg: float = 15.0):
    """Yield (f, k, layer [m][nj][ni]) of the ensemble in field, layer order.
    Layer k of a field is 0.8 layer k-1 + 0.6 new (inter-layer correlation
    0.8); static members (md..m-1, hybrid) are 0.7 x one field-level draw."""
    import concurrent.futures as cf
    with cf.ThreadPoolExecutor(max_workers=_fft_workers()) as ex:
        for f in range(nf):
            static = None
            if md < m:
                static = grf_filter(_layer_noise(cfg, 6, f, 0, m - md, nj, ni, ex), length) * np.float32(0.7)
            prev = None
            for k in range(nl):
                new = grf_filter(_layer_noise(cfg, 0, f, k, m, nj, ni, ex), length)
                lay = new if prev is None else (np.float32(0.8) * prev + np.float32(0.6) * new)
                prev = lay
                out = lay.copy()
                if static is not None:
                    out[md:] = static
                out += np.float32(bg)
                yield f, k, out


def bilinear(field: np.ndarray, x: np.ndarray, y: np.ndarray) -> np.ndarray:
    """Bilinear interpolation of field[..., nj, ni] at cell coordinates (x, y)."""
    nj, ni = field.shape[-2:]
    x = np.asarray(x, np.float64)
    y = np.asarray(y, np.float64)
    i0 = np.clip(np.floor(x).astype(np.int64), 0, ni - 2)
    j0 = np.clip(np.floor(y).astype(np.int64), 0, nj - 2)
    fx = (x - i0).astype(np.float32)
    fy = (y - j0).astype(np.float32)
    f00 = field[..., j0, i0]
    f01 = field[..., j0, i0 + 1]
    f10 = field[..., j0 + 1, i0]
    f11 = field[..., j0 + 1, i0 + 1]
    return ((f00 * (1 - fx) + f01 * fx) * (1 - fy) + (f10 * (1 - fx) + f11 * fx) * fy).astype(np.float32)


@dataclasses.dataclass
class Workload:
    """Everything one calc + update cycle needs."""
    cfg: int
    mode: int              # 0 ENKF, 1 ENOI, 2 HYBRID
    scheme: int            # 0 DEnKF, 1 ETKF
    ni: int
    nj: int
    nlayers: int
    nfields: int
    nmem: int
    nmem_dynamic: int
    stride: int
    locrad: float
    alpha: float
    inflation: float
    inf_ratio: float
    gamma: float
    # grid
    x: np.ndarray          # [ni] float64
    y: np.ndarray          # [nj] float64
    numlevels: np.ndarray  # [nj][ni] int32
    # observations (grouped by type)
    ntypes: int
    lon: np.ndarray        # float32 [nobs]
    lat: np.ndarray        # float32 [nobs]
    otype: np.ndarray      # int16 [nobs]
    status: np.ndarray     # int16 [nobs]
    estd: np.ndarray       # float32 [nobs]
    value: np.ndarray      # float32 [nobs]
    HE: np.ndarray         # float32 [nmem][nobs]
    # ensemble fields: [nfields][nlayers][nmem][nj][ni] float32 (None if not generated)
    fields: Optional[np.ndarray] = None
    verify: Optional[np.ndarray] = None   # [nj][ni] (workload 4)

    @property
    def nobs(self) -> int:
        return int(self.lon.shape[0])

    @property
    def nj_s(self) -> int:
        return (self.nj - 1) // self.stride + 1

    @property
    def ni_s(self) -> int:
        return (self.ni - 1) // self.stride + 1

    @property
    def nanalyses(self) -> int:
        return self.nj_s * self.ni_s


def _land_mask(rng, nj, ni, frac, length):
    blob = grf(rng, nj, ni, length, 1.0)[0]
    thr = np.quantile(blob, frac)
    return blob < thr   # True on land


def _swaths(rng, n, nswath, width, ni, nj, land):
    """n obs on `nswath` random straight swaths of the given width (cells)."""
    xs, ys = [], []
    need = n
    while need > 0:
        k = rng.integers(nswath)
        # swath k: a line through a random point with a random direction
        # (regenerated deterministically from k)
        lr = np.random.default_rng(10_000 + int(k))
        cx, cy = lr.uniform(0, ni - 1), lr.uniform(0, nj - 1)
        ang = lr.uniform(0, np.pi)
        m = max(need * 2, 1024)
        t = rng.uniform(-np.hypot(ni, nj), np.hypot(ni, nj), m)
        d = rng.uniform(-width / 2, width / 2, m)
        x = cx + t * np.cos(ang) - d * np.sin(ang)
        y = cy + t * np.sin(ang) + d * np.cos(ang)
        ok = (x >= 0) & (x <= ni - 1) & (y >= 0) & (y <= nj - 1)
        x, y = x[ok], y[ok]
        if land is not None and x.size:
            keep = ~land[np.rint(y).astype(int), np.rint(x).astype(int)]
            x, y = x[keep], y[keep]
        take = min(need, x.size, max(1, n // nswath))
        xs.append(x[:take])
        ys.append(y[:take])
        need -= take
    return np.concatenate(xs), np.concatenate(ys)


def _uniform_ocean(rng, n, ni, nj, land):
    xs, ys = [], []
    need = n
    while need > 0:
        m = need * 2 + 16
        x = rng.uniform(0, ni - 1, m)
        y = rng.uniform(0, nj - 1, m)
        if land is not None:
            keep = ~land[np.rint(y).astype(int), np.rint(x).astype(int)]
            x, y = x[keep], y[keep]
        xs.append(x[:need])
        ys.append(y[:need])
        need -= min(need, x.size)
    return np.concatenate(xs), np.concatenate(ys)


def make(cfg: int, *, scale: float = 1.0, nobs: Optional[int] = None, with_fields: bool = True,
         nmem: Optional[int] = None) -> Workload:
    """Build workload `cfg` (1-5).  `scale` < 1 shrinks the grid edge lengths and
    the obs count by scale and scale**2 (for tests); `nobs` overrides the count."""
    if cfg == 1:
        ni = nj = 128; nl = 1; nf = 1; m = 24; md = 24; n = 3000; L = 8.0
        mode, scheme, stride, r = 0, 1, 1, 20.0
        infl, ratio, gamma, landfrac = 1.05, float("nan"), 0.0, 0.0
    elif cfg in (2, 4):
        ni, nj = 600, 900; nl = 4; nf = 2; m = 48 if cfg == 2 else 64; md = m; n = 400_000; L = 10.0
        mode, scheme, stride, r = 0, 0, 3, 30.0
        infl, ratio, gamma, landfrac = 1.0, float("nan"), 0.0, 0.3
    elif cfg == 3:
        ni = nj = 1000; nl = 10; nf = 2; m = 96; md = 96; n = 2_000_000; L = 12.0
        mode, scheme, stride, r = 0, 1, 2, 25.0
        infl, ratio, gamma, landfrac = 1.0, float("nan"), 0.0, 0.0
    elif cfg == 5:
        ni, nj = 3600, 1500; nl = 51; nf = 2; m = 144; md = 96; n = 14_000_000; L = 15.0
        mode, scheme, stride, r = 2, 1, 3, 40.0
        infl, ratio, gamma, landfrac = 1.0, float("nan"), 0.5, 0.4
    else:
        raise ValueError(f"unknown workload {cfg}")
    if nmem is not None:
        m = md = nmem
        if cfg == 5:
            md = max(2, (2 * nmem) // 3)
    if scale != 1.0:
        ni = max(8, int(round(ni * scale)))
        nj = max(8, int(round(nj * scale)))
        n = max(16, int(round(n * scale * scale)))
    if nobs is not None:
        n = int(nobs)

    land = _land_mask(_rng(cfg, 4), nj, ni, landfrac, 3 * L) if landfrac > 0 else None
    numlevels = np.full((nj, ni), nl, np.int32)
    if land is not None:
        numlevels[land] = 0

    # observations; types are contiguous in obs order
    rl = _rng(cfg, 2)
    if cfg in (2, 4):
        n_sw = int(round(0.7 * n))
        xs0, ys0 = _swaths(_rng(cfg, 5), n_sw, 50, 20.0, ni, nj, land)
        xs1, ys1 = _uniform_ocean(rl, n - n_sw, ni, nj, land)
        xs = np.concatenate([xs0, xs1]); ys = np.concatenate([ys0, ys1])
        otype = np.concatenate([np.zeros(xs0.size, np.int16), np.ones(xs1.size, np.int16)])
        ntypes = 2
        estd = rl.uniform(0.3, 0.8, xs.size).astype(np.float32)
    elif cfg == 5:
        n_sst = int(round(0.6 * n)); n_ssh = int(round(0.3 * n)); n_pr = n - n_sst - n_ssh
        xs0, ys0 = _swaths(_rng(cfg, 5), n_sst, 200, 30.0, ni, nj, land)
        xs1, ys1 = _swaths(_rng(cfg, 7), n_ssh, 400, 2.0, ni, nj, land)
        ncol = max(1, min(30_000, n_pr // nl))
        cx, cy = _uniform_ocean(rl, ncol, ni, nj, land)
        reps = int(np.ceil(n_pr / ncol))
        xs2 = np.tile(cx, reps)[:n_pr]; ys2 = np.tile(cy, reps)[:n_pr]
        half = n_pr // 2
        xs = np.concatenate([xs0, xs1, xs2[:half], xs2[half:]])
        ys = np.concatenate([ys0, ys1, ys2[:half], ys2[half:]])
        otype = np.concatenate([np.zeros(xs0.size, np.int16), np.ones(xs1.size, np.int16),
                                np.full(half, 2, np.int16), np.full(n_pr - half, 3, np.int16)])
        ntypes = 4
        estd = np.full(xs.size, 0.5, np.float32)
    else:
        xs, ys = _uniform_ocean(rl, n, ni, nj, land)
        otype = np.zeros(xs.size, np.int16)
        ntypes = 1
        estd = np.full(xs.size, 0.5, np.float32)
    lon = xs.astype(np.float32)
    lat = ys.astype(np.float32)
    status = np.zeros(lon.size, np.int16)

    # ensemble (observed field = field 0, layer 0) and truth
    bg = 15.0
    fields = None
    if with_fields:
        fields = np.empty((nf, nl, m, nj, ni), np.float32)
        for f, k, lay in ensemble_layers(cfg, nf, nl, m, md, nj, ni, L, bg):
            fields[f, k] = lay
        obs_member = fields[0, 0]
    else:
        obs_member = next(ensemble_layers(cfg, 1, 1, m, md, nj, ni, L, bg))[2]
    truth = grf(_rng(cfg, 1), nj, ni, L, 1.0)[0] + bg
    noise = _rng(cfg, 3).standard_normal(lon.size).astype(np.float32)
    value = (bilinear(truth, lon, lat) + estd * noise).astype(np.float32)
    HE = bilinear(obs_member, lon, lat)

    verify = None
    if cfg == 4:
        verify = grf(_rng(cfg, 8), nj, ni, L, 1.0)[0] + bg

    return Workload(cfg=cfg, mode=mode, scheme=scheme, ni=ni, nj=nj, nlayers=nl, nfields=nf, nmem=m,
                    nmem_dynamic=md, stride=stride, locrad=r, alpha=1.0, inflation=infl,
                    inf_ratio=ratio, gamma=gamma,
                    x=np.arange(ni, dtype=np.float64), y=np.arange(nj, dtype=np.float64),
                    numlevels=numlevels, ntypes=ntypes, lon=lon, lat=lat, otype=otype,
                    status=status, estd=estd, value=value, HE=np.ascontiguousarray(HE),
                    fields=fields, verify=verify)
