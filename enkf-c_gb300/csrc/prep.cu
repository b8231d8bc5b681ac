// prep.cu -- inputs of the transform stage: innovations and ensemble spread
// (das_calcinnandspread, reference calc/ensobs.c:541-690), standardisation
// (das_standardise, ensobs.c:849-898), observation and query coordinates.
//
// One thread per observation runs the reference's per-observation sequence
// of float/double operations in the same order (member sums accumulate from
// member 0 upwards), so S, s_f and std_f are bit-identical to the host code.
#include "internal.cuh"

__global__ void k_innovations(int nmem, int nobs, float* __restrict__ S, const float* __restrict__ value,
                              const short* __restrict__ status, double* __restrict__ s_f, double* __restrict__ std_f)
{
    int o = blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= nobs) return;
    double mean = 0.0;
    for (int e = 0; e < nmem; ++e) mean = __dadd_rn(mean, (double)S[(size_t)e * nobs + o]);
    mean = __ddiv_rn(mean, (double)nmem);
    float fm = (float)mean;
    double sd = 0.0;
    for (int e = 0; e < nmem; ++e) {
        float v = __fsub_rn(S[(size_t)e * nobs + o], fm);
        S[(size_t)e * nobs + o] = v;
        sd = __dadd_rn(sd, (double)__fmul_rn(v, v));
    }
    if (status[o] == 0) {
        sd = __dsqrt_rn(__ddiv_rn(sd, (double)(nmem - 1)));
        mean = __dsub_rn((double)value[o], mean);
    }
    s_f[o] = mean;
    std_f[o] = sd;
}

__global__ void k_standardise(int nmem, int nobs, double mult, float* __restrict__ S, double* __restrict__ s_f,
                              const float* __restrict__ estd, const short* __restrict__ type,
                              const double* __restrict__ sqrt_rfac)
{
    int o = blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= nobs) return;
    double den = __dmul_rn(__dmul_rn((double)estd[o], sqrt_rfac[type[o]]), mult);
    for (int e = 0; e < nmem; ++e) {
        float* x = &S[(size_t)e * nobs + o];
        *x = (float)__ddiv_rn((double)*x, den);
    }
    s_f[o] = __ddiv_rn(s_f[o], den);
}

__global__ void k_obs_coords(int nobs, const float* __restrict__ lon, const float* __restrict__ lat,
                             double* __restrict__ ox, double* __restrict__ oy)
{
    int o = blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= nobs) return;
    ox[o] = (double)lon[o];
    oy[o] = (double)lat[o];
}

// coordinates of the strided points (grid_ij2xy -> hgrid_ij2xy,
// hgrid.c:457-472): rectangular x[i], y[j] or curvilinear [j][i]
__global__ void k_query_coords(int nj, int ni, int stride, int mni, const double* __restrict__ x,
                               const double* __restrict__ y, int curvilinear, double* __restrict__ qx,
                               double* __restrict__ qy)
{
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nj * ni) return;
    int jj = p / ni, ii = p - jj * ni;
    int i = ii * stride, j = jj * stride;
    if (curvilinear) {
        qx[p] = x[(size_t)j * mni + i];
        qy[p] = y[(size_t)j * mni + i];
    } else {
        qx[p] = x[i];
        qy[p] = y[j];
    }
}

enkfg_status run_innovations(enkfg_ctx* ctx, cudaStream_t st)
{
    k_innovations<<<div_up(ctx->nobs, 256), 256, 0, st>>>(ctx->nmem, ctx->nobs, ctx->d_S, ctx->d_value,
                                                         ctx->d_status, ctx->d_s, ctx->d_std);
    CKL();
    return ENKFG_OK;
}

enkfg_status run_standardise(enkfg_ctx* ctx, cudaStream_t st)
{
    double mult = sqrt((double)ctx->nmem - 1);
    k_standardise<<<div_up(ctx->nobs, 256), 256, 0, st>>>(ctx->nmem, ctx->nobs, mult, ctx->d_S, ctx->d_s,
                                                         ctx->d_estd, ctx->d_type, ctx->d_rfac_sqrt);
    CKL();
    return ENKFG_OK;
}

enkfg_status upload_obs_coords(enkfg_ctx* ctx, const float* lon, const float* lat, cudaStream_t st)
{
    int n = ctx->nobs;
    if (n <= 0) return ENKFG_OK;
    if (!ctx->geographic) {
        k_obs_coords<<<div_up(n, 256), 256, 0, st>>>(n, ctx->d_lon, ctx->d_lat, ctx->d_ox, ctx->d_oy);
        CKL();
        return ENKFG_OK;
    }
    // On the sphere the reference converts with libm cos/sin (ll2xyz,
    // utils.c:1449-1458); the conversion is done here on the host with the
    // same libm so that coordinates, and therefore neighbour sets, are
    // bit-identical.
    double* h = (double*)malloc((size_t)n * 3 * sizeof(double));
    if (!h) return ENKFG_ENOMEM;
    const double R = 6371.0, D = M_PI / 180.0;
    for (int o = 0; o < n; ++o) {
        double lo = (double)lon[o] * D, la = (double)lat[o] * D, cl = cos(la);
        h[o] = R * cos(lo) * cl;
        h[n + o] = R * sin(lo) * cl;
        h[2 * n + o] = R * sin(la);
    }
    cudaError_t e1 = cudaMemcpy(ctx->d_ox, h, n * sizeof(double), cudaMemcpyHostToDevice);
    cudaError_t e2 = cudaMemcpy(ctx->d_oy, h + n, n * sizeof(double), cudaMemcpyHostToDevice);
    cudaError_t e3 = cudaMemcpy(ctx->d_oz, h + 2 * n, n * sizeof(double), cudaMemcpyHostToDevice);
    free(h);
    if (e1 != cudaSuccess || e2 != cudaSuccess || e3 != cudaSuccess) return cuda_fail(ctx, e1 ? e1 : e2 ? e2 : e3, "obs xyz", __LINE__);
    return ENKFG_OK;
}

enkfg_status upload_query_coords(enkfg_ctx* ctx, const enkfg_grid* g, cudaStream_t st)
{
    int npts = ctx->nj * ctx->ni;
    bool curv = (g->x2d != nullptr);
    if (!ctx->geographic) {
        size_t nx = curv ? (size_t)g->mni * g->mnj : (size_t)g->mni;
        size_t ny = curv ? (size_t)g->mni * g->mnj : (size_t)g->mnj;
        double *dx, *dy;
        CK(cudaMalloc(&dx, nx * sizeof(double)));
        CK(cudaMalloc(&dy, ny * sizeof(double)));
        CK(cudaMemcpy(dx, curv ? g->x2d : g->x, nx * sizeof(double), cudaMemcpyHostToDevice));
        CK(cudaMemcpy(dy, curv ? g->y2d : g->y, ny * sizeof(double), cudaMemcpyHostToDevice));
        k_query_coords<<<div_up(npts, 256), 256, 0, st>>>(ctx->nj, ctx->ni, ctx->stride, g->mni, dx, dy, curv ? 1 : 0,
                                                         ctx->d_qx, ctx->d_qy);
        ctx->launches++;
        cudaError_t e = cudaStreamSynchronize(st);
        cudaFree(dx);
        cudaFree(dy);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "query coords", __LINE__);
        return ENKFG_OK;
    }
    double* h = (double*)malloc((size_t)npts * 3 * sizeof(double));
    if (!h) return ENKFG_ENOMEM;
    const double R = 6371.0, D = M_PI / 180.0;
    for (int p = 0; p < npts; ++p) {
        int jj = p / ctx->ni, ii = p - jj * ctx->ni;
        int i = ii * ctx->stride, j = jj * ctx->stride;
        double lon = curv ? g->x2d[(size_t)j * g->mni + i] : g->x[i];
        double lat = curv ? g->y2d[(size_t)j * g->mni + i] : g->y[j];
        double lo = lon * D, la = lat * D, cl = cos(la);
        h[p] = R * cos(lo) * cl;
        h[npts + p] = R * sin(lo) * cl;
        h[2 * npts + p] = R * sin(la);
    }
    cudaError_t e1 = cudaMemcpy(ctx->d_qx, h, npts * sizeof(double), cudaMemcpyHostToDevice);
    cudaError_t e2 = cudaMemcpy(ctx->d_qy, h + npts, npts * sizeof(double), cudaMemcpyHostToDevice);
    cudaError_t e3 = cudaMemcpy(ctx->d_qz, h + 2 * npts, npts * sizeof(double), cudaMemcpyHostToDevice);
    free(h);
    if (e1 != cudaSuccess || e2 != cudaSuccess || e3 != cudaSuccess) return cuda_fail(ctx, e1 ? e1 : e2 ? e2 : e3, "grid xyz", __LINE__);
    return ENKFG_OK;
}
