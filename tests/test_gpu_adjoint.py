"""Observation-impact adjoint (enkfg_adjoint_mean + enkfg_adjoint_transforms).

Objective (workload 4): J = sum over wet cells of (analysis mean - verifying
field)^2 for the observed field-layer, with the analysis mean of the FP64
transforms: x_a = x_f + A w_cell (A the forecast anomalies, w_cell the
stride-interpolated w).  Independent variables: the innovations d_o, the
obs-error variances R_o = estd_o^2 and a common scale rho of the
localisation radius.

The GPU forward and the GPU adjoint are wrapped, for this test only, in a
torch.autograd.Function (ObsImpact).  Checks, all in FP64:
  * central finite differences (step 1e-6) of the GPU forward for 200 random
    innovations and for rho: relative error <= 1e-6 (normwise over the 200);
  * an FP64 reference gradient -- torch autograd through an independent
    pure-torch forward of the same analysis -- for the innovations, the
    variances and rho: relative error <= 1e-6.
The variances are checked against the reference gradient only: S is stored
in float (as in the reference), so a 1e-6 step in R_o is below S's rounding
and finite differences through the GPU forward would measure that rounding.
"""
import numpy as np
import pytest

import oracle
import synth

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def interp_weights(w):
    """Per cell: the strided points and float-rounded weights of the stride
    interpolation (update.c:195-272), as a dense [ncell][npts] matrix."""
    st, ni, nj = w.stride, w.ni_s, w.nj_s
    Wm = np.zeros((w.nj * w.ni, nj * ni))
    for j in range(w.nj):
        jj, sj = divmod(j, st)
        rows = [(jj, 1.0)]
        if st > 1 and sj > 0:
            w2 = np.float32(sj) / np.float32(st)
            w1 = np.float32(1.0) - w2
            rows = [(jj, float(w1)), (jj + 1 if jj < nj - 1 else jj, float(w2))]
        for i in range(w.ni):
            ii, si = divmod(i, st)
            cols = [(ii, 1.0)]
            if st > 1 and si > 0:
                u2 = np.float32(si) / np.float32(st)
                u1 = np.float32(1.0) - u2
                cols = [(ii, float(u1)), (ii + 1 if ii < ni - 1 else ii, float(u2))]
            for (r, a) in rows:
                for (c, b) in cols:
                    Wm[j * w.ni + i, r * ni + c] += a * b
    return Wm


CHECKS = {}


def record(name, summary):
    """Keep the measured errors (adjoint_checks.json in the directory named
    by ENKFG_RESULTS_DIR, when that is set)."""
    import json
    import os
    CHECKS[name] = summary
    out = os.environ.get("ENKFG_RESULTS_DIR")
    if out and os.path.isdir(out):
        with open(os.path.join(out, "adjoint_checks.json"), "w") as f:
            json.dump(CHECKS, f, indent=1)


class Problem:
    def __init__(self, ctx, nmem=64, scale=0.1, nobs=4000):
        w = synth.make(4, scale=scale, nobs=nobs, nmem=nmem)
        w.locrad = 8.0
        self.w = w
        self.ctx = ctx
        m = w.nmem
        HE = w.HE.astype(np.float64)
        self.mean_he = HE.mean(axis=0)
        self.HA = (w.HE - self.mean_he.astype(np.float32)[None]).astype(np.float32)   # float HA
        self.d0 = w.value.astype(np.float64) - self.mean_he
        self.R0 = w.estd.astype(np.float64) ** 2
        self.nl, self.lr, self.lw = oracle.locrad_table(w.ntypes, w.locrad)
        self.field = w.fields[0, 0]                            # forecast [m][nj][ni]
        mean = self.field.astype(np.float64).mean(axis=0)
        self.xf = mean.reshape(-1)
        # the anomalies as the update kernel forms them: (float)(v - mean)
        self.A = (self.field.astype(np.float64) - mean[None]).astype(np.float32).astype(np.float64).reshape(m, -1)
        self.wet = (w.numlevels.reshape(-1) > 0)
        self.verify = w.verify.reshape(-1).astype(np.float64)
        self.Wm = interp_weights(w)

    def standardise(self, d, R):
        m = self.w.nmem
        sig = np.sqrt(R) * np.sqrt(m - 1.0)
        S = (self.HA.astype(np.float64) / sig[None]).astype(np.float32)
        return S, d / sig

    def forward(self, d, R, rho):
        w, ctx = self.w, self.ctx
        ctx.set_obstypes(self.nl, self.lr * rho, self.lw, np.ones(w.ntypes))
        ctx.set_obs(w.lon, w.lat, w.otype, w.status, np.sqrt(R).astype(np.float32), w.value)
        S, s = self.standardise(d, R)
        ctx.set_S(S, s)
        ctx.set_grid(w.x, w.y, stride=w.stride)
        out = ctx.calctransforms(mode=0, scheme=w.scheme, want64=True, want_diag=False)
        w64 = out["w64"].reshape(-1, w.nmem)
        wc = self.Wm @ w64                                      # [ncell][m]
        xa = self.xf + np.einsum("ec,ce->c", self.A, wc)
        r = np.where(self.wet, xa - self.verify, 0.0)
        return float((r * r).sum()), r

    def adjoint(self, r, rho, precision=0):
        w, ctx = self.w, self.ctx
        g = 2.0 * r
        wbar = ctx.adjoint_mean(self.field, g.reshape(w.nj, w.ni))
        dinn, dvar, drho = ctx.adjoint_transforms(wbar, mode=0, scheme=w.scheme, precision=precision)
        return dinn, dvar, drho


class ObsImpact(torch.autograd.Function):
    """J(d, R, rho) with the GPU forward and the GPU adjoint (test harness only)."""

    @staticmethod
    def forward(c, d, R, rho, prob):
        J, r = prob.forward(d.detach().numpy(), R.detach().numpy(), float(rho))
        c.prob = prob
        c.r = r
        c.rho = float(rho)
        return torch.tensor(J, dtype=torch.float64)

    @staticmethod
    def backward(c, gJ):
        dinn, dvar, drho = c.prob.adjoint(c.r, c.rho)
        return (gJ * torch.from_numpy(dinn), gJ * torch.from_numpy(dvar), gJ * torch.tensor(drho, dtype=torch.float64),
                None)


def gc_torch(x):
    """Gaspari-Cohn taper of x = dist / radius (support x < 1), differentiable."""
    z = 2.0 * x
    inner = 1 + z ** 2 * (-z ** 3 / 4 + z ** 2 / 2) + z ** 3 * (5 / 8) - z ** 2 * (5 / 3)
    outer = z ** 2 * (z ** 3 / 12 - z ** 2 / 2) + z ** 3 * (5 / 8) + z ** 2 * (5 / 3) - z * 5 + 4 - (2 / 3) / z
    return torch.where(x < 1, torch.where(z < 1, inner, outer), torch.zeros_like(x)).clamp(min=0)


def local_lists(w, tabs):
    """Local obs (ids, distances) of every strided point from the oracle."""
    nl, lr, lw = tabs
    obs = oracle.ObsSet(w.lon, w.lat, w.otype, w.status, w.ntypes, nl, lr, lw)
    lists = []
    for pt in range(w.nanalyses):
        jj, ii = divmod(pt, w.ni_s)
        qx, qy = w.x[ii * w.stride], w.y[jj * w.stride]
        ids, _ = obs.findlocal(qx, qy)
        dist = np.sqrt((w.lon[ids].astype(np.float64) - qx) ** 2 + (w.lat[ids].astype(np.float64) - qy) ** 2)
        lists.append((ids, dist))
    return lists


def inv_sqrt_db(M, iters=60):
    """M^-1/2 of a batch of SPD matrices by the Denman-Beavers iteration
    (Y -> M^1/2, Z -> M^-1/2), differentiable without eigenvectors, so that
    clustered eigenvalues do not break the reference gradient."""
    Y, Z = M, torch.eye(M.shape[-1], dtype=M.dtype).expand_as(M)
    for _ in range(iters):
        Yi, Zi = torch.linalg.inv(Y), torch.linalg.inv(Z)
        Y, Z = 0.5 * (Y + Zi), 0.5 * (Z + Yi)
    return Z


def torch_transforms(S0, sig0, d, R, rho, r0, lists, m, want_T=False, scheme=1, alpha=1.0):
    """Independent FP64 forward in torch: w (and T) of every point.  S is the
    float S the library holds, rescaled by sig0 / sig so that it equals it at
    R = R0 and varies with R as S does; the taper is re-evaluated in rho."""
    sig = torch.sqrt(R) * np.sqrt(m - 1.0)
    S = torch.from_numpy(S0.astype(np.float64)) * (torch.from_numpy(sig0) / sig)[None]
    s = d / sig
    I = torch.eye(m, dtype=torch.float64)
    Ms, bs = [], []
    for (ids, dist) in lists:
        if ids.size == 0:
            Ms.append(I)
            bs.append(torch.zeros(m, dtype=torch.float64))
            continue
        lc = gc_torch(torch.from_numpy(dist) / (rho * r0))
        Si = S[:, ids].T * lc[:, None]                          # p x m
        si = s[ids] * lc
        Ms.append(I + Si.T @ Si)
        bs.append(Si.T @ si)
    M = torch.stack(Ms)
    W = torch.linalg.solve(M, torch.stack(bs))
    if not want_T:
        return W, None
    fM = inv_sqrt_db(M) if scheme == 1 else 0.5 * (I + torch.linalg.inv(M))
    return W, I + alpha * (fM - I)


def test_adjoint_against_fd_and_reference(ctx):
    prob = Problem(ctx)
    w = prob.w
    m = w.nmem
    d = torch.tensor(prob.d0, dtype=torch.float64, requires_grad=True)
    R = torch.tensor(prob.R0, dtype=torch.float64, requires_grad=True)
    rho = torch.tensor(1.0, dtype=torch.float64, requires_grad=True)
    J = ObsImpact.apply(d, R, rho, prob)
    J.backward()
    gd, gR, grho = d.grad.numpy().copy(), R.grad.numpy().copy(), float(rho.grad)
    assert np.isfinite(gd).all() and np.abs(gd).max() > 0

    # central finite differences (step 1e-6) through the GPU forward
    rng = np.random.default_rng(4)
    infl = np.nonzero(np.abs(gd) > 1e-3 * np.abs(gd).max())[0]
    pick = rng.choice(infl, size=min(200, infl.size), replace=False)
    h = 1e-6
    fd = np.zeros(pick.size)
    for k, o in enumerate(pick):
        dp = prob.d0.copy()
        dp[o] += h
        jp, _ = prob.forward(dp, prob.R0, 1.0)
        dp[o] -= 2 * h
        jm, _ = prob.forward(dp, prob.R0, 1.0)
        fd[k] = (jp - jm) / (2 * h)
    err_fd = float(np.linalg.norm(gd[pick] - fd) / np.linalg.norm(fd))
    jp, _ = prob.forward(prob.d0, prob.R0, 1.0 + h)
    jm, _ = prob.forward(prob.d0, prob.R0, 1.0 - h)
    fd_rho = (jp - jm) / (2 * h)
    err_rho_fd = abs(grho - fd_rho) / abs(fd_rho)

    # FP64 reference gradient (torch autograd on an independent forward)
    lists = local_lists(w, (prob.nl, prob.lr, prob.lw))
    S0, _ = prob.standardise(prob.d0, prob.R0)
    sig0 = np.sqrt(prob.R0) * np.sqrt(m - 1.0)
    d2 = torch.tensor(prob.d0, dtype=torch.float64, requires_grad=True)
    R2 = torch.tensor(prob.R0, dtype=torch.float64, requires_grad=True)
    rho2 = torch.tensor(1.0, dtype=torch.float64, requires_grad=True)
    W, _ = torch_transforms(S0, sig0, d2, R2, rho2, float(prob.lr[0, 0]), lists, m)
    wc = torch.from_numpy(prob.Wm) @ W
    xa = torch.from_numpy(prob.xf) + (torch.from_numpy(prob.A).T * wc).sum(1)
    res = torch.where(torch.from_numpy(prob.wet), xa - torch.from_numpy(prob.verify), torch.zeros_like(xa))
    Jr = (res * res).sum()
    Jr.backward()
    rel = lambda a, b: float(np.linalg.norm(a - b) / np.linalg.norm(b))
    err_ref_d = rel(gd, d2.grad.numpy())
    err_ref_R = rel(gR, R2.grad.numpy())
    err_ref_rho = abs(grho - float(rho2.grad)) / abs(float(rho2.grad))
    jrel = abs(float(J.detach()) - float(Jr.detach())) / abs(float(Jr.detach()))
    summary = dict(J=float(J.detach()), J_ref_rel=jrel, fd_innov=err_fd, fd_rho=err_rho_fd, ref_innov=err_ref_d,
                   ref_var=err_ref_R, ref_rho=err_ref_rho, n_fd=int(pick.size), nobs=int(w.nobs), nmem=m)
    record(f"w_term_workload4_m{m}", summary)
    assert jrel < 1e-9, summary
    assert err_fd < 1e-6, summary
    assert err_rho_fd < 1e-6, summary
    assert err_ref_d < 1e-9 and err_ref_R < 1e-9 and err_ref_rho < 1e-9, summary


def test_adjoint_fp32_production_against_fp64(ctx):
    """The FP32 production adjoint (S'S, eigendecomposition, Daleckii-Krein
    and per-observation passes in FP32, FP64 accumulators) against the FP64
    adjoint on workload 4's shape with m = 64: normwise relative error of
    each gradient (recorded; bound 1e-3)."""
    prob = Problem(ctx)
    J, r = prob.forward(prob.d0, prob.R0, 1.0)
    g64 = prob.adjoint(r, 1.0, precision=0)
    g32 = prob.adjoint(r, 1.0, precision=1)
    rel = lambda a, b: float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))
    summary = dict(innov=rel(g32[0], g64[0]), var=rel(g32[1], g64[1]), rho=abs(g32[2] - g64[2]) / abs(g64[2]),
                   nmem=prob.w.nmem, nobs=int(prob.w.nobs))
    record(f"fp32_vs_fp64_workload4_m{prob.w.nmem}", summary)
    assert summary["innov"] < 1e-3 and summary["var"] < 1e-3 and summary["rho"] < 1e-3, summary


@pytest.mark.parametrize("scheme,nmem", [(1, 24), (0, 24), (1, 80)])
def test_adjoint_T_term_daleckii_krein(ctx, scheme, nmem):
    """J = sum(Tbar * T) + sum(wbar * w): the Daleckii-Krein term against an
    FP64 torch reference (Denman-Beavers M^-1/2, or the inverse for DEnKF) for
    the innovations, variances and rho, and against central
    finite differences of the GPU forward in rho.  ETKF and DEnKF; m = 80
    exercises the batched in-place products past 64 members."""
    w = synth.make(1, scale=0.25, nobs=1500 if nmem <= 24 else 6000, nmem=nmem, with_fields=False)
    w.locrad = 6.0
    alpha = 0.8
    tabs = oracle.locrad_table(1, w.locrad)
    nl, lr, lw = tabs
    S, s_f, _ = oracle.calcinnandspread(w.HE, w.value, w.status)
    S, s = oracle.standardise(S, s_f, w.estd, w.otype, np.ones(1))
    rng = np.random.default_rng(8 + scheme)
    nj, ni, m = w.nj_s, w.ni_s, w.nmem
    Tbar = rng.standard_normal((nj, ni, m, m))
    Tbar = 0.5 * (Tbar + Tbar.transpose(0, 1, 3, 2))
    wbar = rng.standard_normal((nj, ni, m))

    def J_of(rho):
        ctx.set_obstypes(nl, lr * rho, lw, np.ones(1))
        ctx.set_obs(w.lon, w.lat, w.otype, w.status, w.estd, w.value)
        ctx.set_S(S, s)
        ctx.set_grid(w.x, w.y, stride=w.stride)
        out = ctx.calctransforms(mode=0, scheme=scheme, alpha=alpha, want64=True, want_diag=False)
        return float((Tbar * out["T64"]).sum() + (wbar * out["w64"]).sum())

    J0 = J_of(1.0)
    dinn, dvar, drho = ctx.adjoint_transforms(wbar, Tbar=Tbar, mode=0, scheme=scheme, alpha=alpha)
    h = 1e-6
    fd = (J_of(1.0 + h) - J_of(1.0 - h)) / (2 * h)

    # central differences in 50 innovations (J depends on them through w;
    # the variances act through S, which is stored in float, so a 1e-6 step
    # would measure S's rounding: they are checked against the reference)
    def J_of_s(s_new):
        ctx.set_obstypes(nl, lr, lw, np.ones(1))
        ctx.set_obs(w.lon, w.lat, w.otype, w.status, w.estd, w.value)
        ctx.set_S(S, s_new)
        ctx.set_grid(w.x, w.y, stride=w.stride)
        out = ctx.calctransforms(mode=0, scheme=scheme, alpha=alpha, want64=True, want_diag=False)
        return float((Tbar * out["T64"]).sum() + (wbar * out["w64"]).sum())

    R0v = w.estd.astype(np.float64) ** 2
    sig0v = np.sqrt(R0v) * np.sqrt(m - 1.0)
    big = np.nonzero(np.abs(dinn) > 1e-3 * np.abs(dinn).max())[0]
    pick = np.random.default_rng(12).choice(big, size=min(50, big.size), replace=False)
    fd_inn = np.zeros(pick.size)
    for k, o in enumerate(pick):
        sp = s.copy()
        sp[o] += h / sig0v[o]
        jp = J_of_s(sp)
        sp[o] -= 2 * h / sig0v[o]
        jm = J_of_s(sp)
        fd_inn[k] = (jp - jm) / (2 * h)
    err_fd_inn = float(np.linalg.norm(dinn[pick] - fd_inn) / np.linalg.norm(fd_inn))

    R0 = w.estd.astype(np.float64) ** 2
    sig0 = np.sqrt(R0) * np.sqrt(m - 1.0)
    d0 = s * sig0
    lists = local_lists(w, tabs)
    d2 = torch.tensor(d0, dtype=torch.float64, requires_grad=True)
    R2 = torch.tensor(R0, dtype=torch.float64, requires_grad=True)
    rho2 = torch.tensor(1.0, dtype=torch.float64, requires_grad=True)
    W, T = torch_transforms(S, sig0, d2, R2, rho2, float(lr[0, 0]), lists, m, want_T=True, scheme=scheme,
                            alpha=alpha)
    Jr = (torch.from_numpy(Tbar.reshape(-1, m, m)) * T).sum() + (torch.from_numpy(wbar.reshape(-1, m)) * W).sum()
    Jr.backward()
    rel = lambda a, b: float(np.linalg.norm(a - b) / np.linalg.norm(b))
    summary = dict(J_ref_rel=abs(J0 - float(Jr)) / abs(float(Jr)), fd_rho=abs(drho - fd) / abs(fd),
                   fd_innov=err_fd_inn, n_fd=int(pick.size),
                   ref_innov=rel(dinn, d2.grad.numpy()), ref_var=rel(dvar, R2.grad.numpy()),
                   ref_rho=abs(drho - float(rho2.grad)) / abs(float(rho2.grad)), nmem=m, nobs=int(w.nobs))
    record(f"T_term_{'etkf' if scheme == 1 else 'denkf'}_m{m}", summary)
    assert summary["J_ref_rel"] < 1e-9, summary
    assert summary["fd_rho"] < 1e-6, summary
    assert summary["fd_innov"] < 1e-6, summary
    # 1e-8: the Denman-Beavers reference itself is good to ~1e-10 when M's
    # eigenvalues cluster near 1 (m = 80 members over ~a dozen field modes)
    assert summary["ref_innov"] < 1e-8 and summary["ref_var"] < 1e-8 and summary["ref_rho"] < 1e-8, summary
