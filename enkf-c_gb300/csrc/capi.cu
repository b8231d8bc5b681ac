// capi.cu -- the C ABI of libenkfg (declared in include/enkfg.h).
#include "internal.cuh"
#include <stdarg.h>
#include <stdlib.h>
#include <math.h>

enkfg_status upload_obs_coords(enkfg_ctx* ctx, const float* lon, const float* lat, cudaStream_t st);
enkfg_status run_adjoint(enkfg_ctx* ctx, const enkfg_calc_params* p, const double* d_wbar, const double* d_Tbar,
                         double* d_dinn, double* d_dvar, double* d_drho, cudaStream_t st);
enkfg_status run_adj_mean(enkfg_ctx* ctx, int m, int md, const float* d_field, const double* d_g, double* d_wbar,
                          cudaStream_t st);
enkfg_status upload_query_coords(enkfg_ctx* ctx, const enkfg_grid* g, cudaStream_t st);

void set_err(enkfg_ctx* c, const char* fmt, ...)
{
    if (!c) return;
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(c->err, sizeof(c->err), fmt, ap);
    va_end(ap);
}

enkfg_status cuda_fail(enkfg_ctx* c, cudaError_t e, const char* what, int line)
{
    set_err(c, "CUDA error in %s (line %d): %s", what, line, cudaGetErrorString(e));
    if (e == cudaErrorMemoryAllocation) return ENKFG_ENOMEM;
    return ENKFG_ECUDA;
}


extern "C" {
static enkfg_status check_calc(enkfg_ctx* ctx, const enkfg_calc_params* p);
}

static cudaStream_t pick(enkfg_ctx* ctx, void* stream)
{
    return stream ? (cudaStream_t)stream : ctx->stream;
}

extern "C" {

ENKFG_API int enkfg_version(void)
{
    return ENKFG_VERSION;
}

ENKFG_API const char* enkfg_status_string(enkfg_status st)
{
    switch (st) {
    case ENKFG_OK: return "ok";
    case ENKFG_EINVAL: return "invalid argument";
    case ENKFG_ECUDA: return "CUDA error";
    case ENKFG_ENOMEM: return "out of device memory";
    case ENKFG_ETIMEOUT: return "device wait timed out";
    case ENKFG_ENUMERIC: return "numerical failure";
    case ENKFG_ECAPACITY: return "capacity exceeded";
    case ENKFG_ESTATE: return "required inputs not set";
    case ENKFG_EUNSUPPORTED: return "unsupported option";
    }
    return "unknown status";
}

ENKFG_API const char* enkfg_last_error(const enkfg_ctx* ctx)
{
    return ctx ? ctx->err : "no context";
}

ENKFG_API enkfg_status enkfg_set_wait_limit(enkfg_ctx* ctx, unsigned long long ns)
{
    if (!ctx) return ENKFG_EINVAL;
    ctx->wait_ns = ns ? ns : ENKFG_DEFAULT_WAIT_NS;
    return ENKFG_OK;
}

ENKFG_API enkfg_status enkfg_set_field_buffer_size(enkfg_ctx* ctx, int nfield)
{
    if (!ctx || nfield < 0) return ENKFG_EINVAL;
    ctx->field_buffer = nfield;
    return ENKFG_OK;
}

ENKFG_API enkfg_status enkfg_set_solve_batch(enkfg_ctx* ctx, int points)
{
    if (!ctx || points < 0) return ENKFG_EINVAL;
    ctx->solve_batch = points;
    return ENKFG_OK;
}

ENKFG_API enkfg_status enkfg_set_field_block_rows(enkfg_ctx* ctx, int rows)
{
    if (!ctx || rows < 0) return ENKFG_EINVAL;
    ctx->field_rows = rows;
    return ENKFG_OK;
}

ENKFG_API enkfg_status enkfg_set_wait_drill(enkfg_ctx* ctx, int on)
{
    if (!ctx) return ENKFG_EINVAL;
    ctx->wait_drill = on ? 1 : 0;
    return ENKFG_OK;
}

ENKFG_API enkfg_status enkfg_create(int device, enkfg_ctx** out)
{
    if (!out) return ENKFG_EINVAL;
    *out = nullptr;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || device < 0 || device >= n) {
        cudaGetLastError();
        return e != cudaSuccess ? ENKFG_ECUDA : ENKFG_EINVAL;
    }
    if (cudaSetDevice(device) != cudaSuccess) return ENKFG_ECUDA;
    enkfg_ctx* ctx = (enkfg_ctx*)calloc(1, sizeof(enkfg_ctx));
    if (!ctx) return ENKFG_ENOMEM;
    ctx->device = device;
    ctx->wait_ns = ENKFG_DEFAULT_WAIT_NS;
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
        free(ctx);
        return ENKFG_ECUDA;
    }
    for (int k = 0; k < 10; ++k) cudaEventCreate(&ctx->ev[k]);
    if (cudaMalloc(&ctx->d_qhead, 1024 * sizeof(int)) != cudaSuccess ||
        cudaMalloc(&ctx->d_rfac, ENKFG_MAXTYPES * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&ctx->d_rfac_sqrt, ENKFG_MAXTYPES * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&ctx->d_smax, ENKFG_MAXMEM * sizeof(unsigned int)) != cudaSuccess ||
        cudaMalloc(&ctx->d_qscale, 2 * ENKFG_MAXMEM * sizeof(float)) != cudaSuccess) {
        enkfg_destroy(ctx);
        return ENKFG_ENOMEM;
    }
    *out = ctx;
    return ENKFG_OK;
}

ENKFG_API void enkfg_destroy(enkfg_ctx* ctx)
{
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    void* ptrs[] = { ctx->d_lon, ctx->d_lat, ctx->d_type, ctx->d_status, ctx->d_estd, ctx->d_value, ctx->d_rfac, ctx->d_rfac_sqrt, ctx->d_gtmp, ctx->d_smax, ctx->d_qscale, ctx->d_eq, ctx->d_ed, ctx->d_ee, ctx->d_eb, ctx->d_eaux, ctx->d_eval, ctx->d_erot, ctx->d_ehdr, ctx->d_enh,
                     ctx->d_emq, ctx->d_emmhl, ctx->d_emd, ctx->d_eme, ctx->d_emrot, ctx->d_emhdr, ctx->d_emnh,
                     ctx->d_emz0, ctx->d_emp,
                     ctx->d_S, ctx->d_s, ctx->d_std, ctx->d_types, ctx->d_bstart, ctx->d_bfill, ctx->d_key,
                     ctx->d_sid, ctx->d_sx, ctx->d_sy, ctx->d_sz, ctx->d_sxf, ctx->d_syf, ctx->d_stype, ctx->d_St, ctx->d_ss, ctx->d_ssf, ctx->d_ox,
                     ctx->d_oy, ctx->d_oz, ctx->d_qx, ctx->d_qy, ctx->d_qz, ctx->d_T, ctx->d_w, ctx->d_T64,
                     ctx->d_w64, ctx->d_nlobs, ctx->d_dfs, ctx->d_srf, ctx->d_pnlobs, ctx->d_pdfs, ctx->d_psrf,
                     ctx->d_counts, ctx->d_order, ctx->d_qhead, ctx->d_status_pt, ctx->d_scratch,
                     ctx->d_numlevels, ctx->d_fields, ctx->d_infl, ctx->d_fi, ctx->d_fj, ctx->d_fk, ctx->d_Hx,
                     ctx->d_hflag, ctx->d_hids, ctx->d_hsrc, ctx->d_hlev, ctx->d_hoff, ctx->d_cut, ctx->d_noise };
    for (size_t k = 0; k < sizeof(ptrs) / sizeof(ptrs[0]); ++k)
        if (ptrs[k]) cudaFree(ptrs[k]);
    for (int k = 0; k < 10; ++k)
        if (ctx->ev[k]) cudaEventDestroy(ctx->ev[k]);
    for (int k = 0; k < ctx->nbev; ++k) cudaEventDestroy(ctx->bev[k]);
    for (int k = 0; k < 2; ++k)
        if (ctx->cstream[k]) cudaStreamDestroy(ctx->cstream[k]);
    for (int k = 0; k < 9; ++k)
        if (ctx->uev[k]) cudaEventDestroy(ctx->uev[k]);
    if (ctx->out_ev) cudaEventDestroy(ctx->out_ev);
    if (ctx->own_stream) ctx->stream = ctx->own_stream;
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    free(ctx);
}

ENKFG_API enkfg_status enkfg_set_stream(enkfg_ctx* ctx, void* stream)
{
    if (!ctx) return ENKFG_EINVAL;
    if (ctx->own_stream == nullptr) ctx->own_stream = ctx->stream;
    ctx->stream = stream ? (cudaStream_t)stream : ctx->own_stream;
    return ENKFG_OK;
}

ENKFG_API enkfg_status enkfg_rebuild_index(enkfg_ctx* ctx)
{
    if (!ctx) return ENKFG_EINVAL;
    ctx->index_valid = false;
    ctx->gather_valid = false;
    // build now, on the context's stream: the build reads sizes back to the
    // host, so it must not be left to a later call that a CUDA graph captures
    if (!ctx->obs_set || !ctx->types_set) return ENKFG_OK;
    SETDEV();
    return build_index(ctx, ctx->stream);
}

ENKFG_API enkfg_status enkfg_adjoint_transforms(enkfg_ctx* ctx, const enkfg_calc_params* p, const double* wbar,
                                                const double* Tbar, double* dinn, double* dvar, double* drad)
{
    if (!ctx) return ENKFG_EINVAL;
    enkfg_status s = check_calc(ctx, p);
    if (s) return s;
    NEED(wbar && dinn && dvar && drad, ENKFG_EINVAL, "wbar and the three outputs are required");
    SETDEV();
    cudaStream_t st = ctx->stream;
    const size_t npts = (size_t)ctx->nj * ctx->ni, m = ctx->nmem, md = ctx->nmem_dyn, n = ctx->nobs > 0 ? ctx->nobs : 1;
    double *d_wbar = nullptr, *d_Tbar = nullptr, *d_out = nullptr;
    cudaError_t e = cudaMalloc(&d_wbar, npts * m * sizeof(double));
    if (e == cudaSuccess && Tbar) e = cudaMalloc(&d_Tbar, npts * md * m * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&d_out, (2 * n + 1) * sizeof(double));
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_wbar, wbar, npts * m * sizeof(double), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && Tbar)
        e = cudaMemcpyAsync(d_Tbar, Tbar, npts * md * m * sizeof(double), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_out, 0, (2 * n + 1) * sizeof(double), st);
    if (e == cudaSuccess) {
        s = run_adjoint(ctx, p, d_wbar, d_Tbar, d_out, d_out + n, d_out + 2 * n, st);
        if (!s && ctx->nobs > 0) {
            cudaMemcpyAsync(dinn, d_out, ctx->nobs * sizeof(double), cudaMemcpyDeviceToHost, st);
            cudaMemcpyAsync(dvar, d_out + n, ctx->nobs * sizeof(double), cudaMemcpyDeviceToHost, st);
        }
        if (!s) cudaMemcpyAsync(drad, d_out + 2 * n, sizeof(double), cudaMemcpyDeviceToHost, st);
        e = cudaStreamSynchronize(st);
    } else {
        cudaGetLastError();
        s = ENKFG_ENOMEM;
        set_err(ctx, "adjoint: device allocation failed");
    }
    cudaFree(d_wbar);
    cudaFree(d_Tbar);
    cudaFree(d_out);
    if (s) return s;
    if (e != cudaSuccess) return cuda_fail(ctx, e, "adjoint copy", __LINE__);
    // dJ/dR -> dJ/d(estd^2): R = estd^2 rfactor
    if (ctx->nobs > 0) {
        short* ty = (short*)malloc(ctx->nobs * sizeof(short));
        if (!ty) return ENKFG_ENOMEM;
        CK(cudaMemcpy(ty, ctx->d_type, ctx->nobs * sizeof(short), cudaMemcpyDeviceToHost));
        for (int o = 0; o < ctx->nobs; ++o) dvar[o] *= ctx->rfactor[ty[o]];
        free(ty);
    }
    // per-point failures
    int* h = (int*)malloc(npts * sizeof(int));
    if (!h) return ENKFG_ENOMEM;
    CK(cudaMemcpy(h, ctx->d_status_pt, npts * sizeof(int), cudaMemcpyDeviceToHost));
    for (size_t k = 0; k < npts; ++k)
        if (h[k]) {
            set_err(ctx, "adjoint: eigendecomposition failed at point %zu", k);
            free(h);
            return ENKFG_ENUMERIC;
        }
    free(h);
    return ENKFG_OK;
}

ENKFG_API enkfg_status enkfg_adjoint_mean(enkfg_ctx* ctx, int nmem, int nmem_dynamic, const float* field,
                                          const double* dJ_dmean, double* wbar)
{
    if (!ctx) return ENKFG_EINVAL;
    NEED(ctx->grid_set, ENKFG_ESTATE, "the grid must be set");
    NEED(field && dJ_dmean && wbar && nmem >= 2 && nmem_dynamic >= 1 && nmem_dynamic <= nmem, ENKFG_EINVAL,
         "bad arguments");
    SETDEV();
    cudaStream_t st = ctx->stream;
    const size_t cells = (size_t)ctx->mni * ctx->mnj, npts = (size_t)ctx->nj * ctx->ni;
    float* d_f = nullptr;
    double *d_g = nullptr, *d_w = nullptr;
    cudaError_t e = cudaMalloc(&d_f, (size_t)nmem * cells * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&d_g, cells * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&d_w, npts * nmem * sizeof(double));
    enkfg_status s = ENKFG_OK;
    if (e == cudaSuccess) {
        cudaMemcpyAsync(d_f, field, (size_t)nmem * cells * sizeof(float), cudaMemcpyHostToDevice, st);
        cudaMemcpyAsync(d_g, dJ_dmean, cells * sizeof(double), cudaMemcpyHostToDevice, st);
        cudaMemsetAsync(d_w, 0, npts * nmem * sizeof(double), st);
        s = run_adj_mean(ctx, nmem, nmem_dynamic, d_f, d_g, d_w, st);
        if (!s) cudaMemcpyAsync(wbar, d_w, npts * nmem * sizeof(double), cudaMemcpyDeviceToHost, st);
        e = cudaStreamSynchronize(st);
    } else {
        cudaGetLastError();
        s = ENKFG_ENOMEM;
        set_err(ctx, "adjoint_mean: device allocation failed");
    }
    cudaFree(d_f);
    cudaFree(d_g);
    cudaFree(d_w);
    if (s) return s;
    if (e != cudaSuccess) return cuda_fail(ctx, e, "adjoint_mean", __LINE__);
    return ENKFG_OK;
}

ENKFG_API enkfg_status enkfg_autotune_table(const enkfg_ctx* ctx, int* table)
{
    if (!ctx || !table) return ENKFG_EINVAL;
    if (!ctx->kc_tuned) return ENKFG_ESTATE;
    memcpy(table, ctx->kc_table, sizeof(ctx->kc_table));
    return ENKFG_OK;
}

ENKFG_API enkfg_status enkfg_autotune_reset(enkfg_ctx* ctx)
{
    if (!ctx) return ENKFG_EINVAL;
    ctx->kc_tuned = false;
    ctx->kc_loaded = 0;
    return ENKFG_OK;
}

ENKFG_API long long enkfg_kernel_launches(const enkfg_ctx* ctx)
{
    return ctx ? ctx->launches : 0;
}

ENKFG_API enkfg_status enkfg_stage_times(const enkfg_ctx* ctx, float* ms4)
{
    if (!ctx || !ms4) return ENKFG_EINVAL;
    // from the stage events themselves when they have completed (the _dev
    // entry points return before the work ends), else the last stored values
    static const int pair[4][2] = { { 0, 1 }, { 1, 2 }, { 2, 3 }, { 4, 5 } };
    for (int k = 0; k < 4; ++k) {
        float v = 0.0f;
        if (ctx->ev[pair[k][0]] && ctx->ev[pair[k][1]] &&
            cudaEventElapsedTime(&v, ctx->ev[pair[k][0]], ctx->ev[pair[k][1]]) == cudaSuccess)
            ms4[k] = v;
        else
            ms4[k] = ctx->stage_ms[k];
    }
    cudaGetLastError();
    return ENKFG_OK;
}

ENKFG_API enkfg_status enkfg_kernel_times(const enkfg_ctx* ctx, float* ms2)
{
    if (!ctx || !ms2) return ENKFG_EINVAL;
    ms2[0] = ms2[1] = 0.0f;
    const int nb = ctx->nbatch < ENKFG_TIMED_BATCHES ? ctx->nbatch : ENKFG_TIMED_BATCHES;
    for (int b = 0; b < nb && 3 * b + 2 < ctx->nbev; ++b) {
        float t0 = 0.0f, t1 = 0.0f;
        if (cudaEventElapsedTime(&t0, ctx->bev[3 * b], ctx->bev[3 * b + 1]) == cudaSuccess) ms2[0] += t0;
        if (cudaEventElapsedTime(&t1, ctx->bev[3 * b + 1], ctx->bev[3 * b + 2]) == cudaSuccess) ms2[1] += t1;
    }
    cudaGetLastError();
    return ENKFG_OK;
}

ENKFG_API enkfg_status enkfg_set_obstypes(enkfg_ctx* ctx, int ntypes, const int* nlocrad, const double* locrad,
                                          const double* locweight, const double* rfactor, int geographic)
{
    if (!ctx) return ENKFG_EINVAL;
    NEED(ntypes >= 1 && ntypes <= ENKFG_MAXTYPES, ENKFG_EINVAL, "ntypes = %d out of range 1..%d", ntypes,
         ENKFG_MAXTYPES);
    NEED(nlocrad && locrad, ENKFG_EINVAL, "nlocrad/locrad are required");
    for (int t = 0; t < ntypes; ++t) {
        NEED(nlocrad[t] >= 1 && nlocrad[t] <= ENKFG_MAXLOCRAD, ENKFG_EINVAL, "type %d: nlocrad = %d", t, nlocrad[t]);
        ctx->nlocrad[t] = nlocrad[t];
        for (int k = 0; k < ENKFG_MAXLOCRAD; ++k) {
            double r = locrad[t * ENKFG_MAXLOCRAD + k];
            double w = locweight ? locweight[t * ENKFG_MAXLOCRAD + k] : 1.0;
            if (k < nlocrad[t]) NEED(r > 0.0 && isfinite(r), ENKFG_EINVAL, "type %d: locrad[%d] = %g", t, k, r);
            ctx->locrad[t][k] = k < nlocrad[t] ? r : 0.0;
            ctx->locweight[t][k] = k < nlocrad[t] ? w : 0.0;
        }
        ctx->rfactor[t] = rfactor ? rfactor[t] : 1.0;
    }
    if (ctx->types_set && (ctx->ntypes != ntypes || ctx->geographic != (geographic ? 1 : 0))) ctx->obs_set = false;
    // a new type table: no NLOBSMAX limits, every type visible
    memset(ctx->nlobsmax, 0, sizeof(ctx->nlobsmax));
    memset(ctx->hidden, 0, sizeof(ctx->hidden));
    ctx->ntypes = ntypes;
    ctx->geographic = geographic ? 1 : 0;
    ctx->types_set = true;
    ctx->index_valid = false;
    ctx->gather_valid = false;
    // sqrt(rfactor) per type for the standardisation, uploaded once here so
    // that the per-cycle work has no host-to-device copy
    {
        double sr[ENKFG_MAXTYPES];
        for (int t = 0; t < ntypes; ++t) sr[t] = sqrt(ctx->rfactor[t]);
        SETDEV();
        CK(cudaMemcpy(ctx->d_rfac_sqrt, sr, ntypes * sizeof(double), cudaMemcpyHostToDevice));
    }
    return ENKFG_OK;
}

ENKFG_API enkfg_status enkfg_set_obstype_nlobsmax(enkfg_ctx* ctx, int ntypes, const int* nlobsmax)
{
    if (!ctx) return ENKFG_EINVAL;
    NEED(ctx->types_set, ENKFG_ESTATE, "enkfg_set_obstypes must come first");
    NEED(ntypes == ctx->ntypes, ENKFG_EINVAL, "ntypes = %d, the context has %d types", ntypes, ctx->ntypes);
    for (int t = 0; t < ENKFG_MAXTYPES; ++t)
        ctx->nlobsmax[t] = (nlobsmax != nullptr && t < ntypes && nlobsmax[t] > 0) ? nlobsmax[t] : 0;
    ctx->cut_valid = false;
    if (ctx->index_valid) {
        SETDEV();
        enkfg_status s = upload_types(ctx, ctx->stream);
        if (s) return s;
    }
    return ENKFG_OK;
}

ENKFG_API enkfg_status enkfg_set_obstype_visible(enkfg_ctx* ctx, int ntypes, const int* visible)
{
    if (!ctx) return ENKFG_EINVAL;
    NEED(ctx->types_set, ENKFG_ESTATE, "enkfg_set_obstypes must come first");
    NEED(ntypes == ctx->ntypes, ENKFG_EINVAL, "ntypes = %d, the context has %d types", ntypes, ctx->ntypes);
    for (int t = 0; t < ENKFG_MAXTYPES; ++t) ctx->hidden[t] = (visible != nullptr && t < ntypes && !visible[t]) ? 1 : 0;
    ctx->cut_valid = false;
    if (ctx->index_valid) {
        SETDEV();
        enkfg_status s = upload_types(ctx, ctx->stream);
        if (s) return s;
    }
    return ENKFG_OK;
}

ENKFG_API enkfg_status enkfg_set_obs(enkfg_ctx* ctx, int nobs, const float* lon, const float* lat, const short* type,
                                     const short* status, const float* estd, const float* value)
{
    if (!ctx) return ENKFG_EINVAL;
    NEED(ctx->types_set, ENKFG_ESTATE, "enkfg_set_obstypes must come first");
    NEED(nobs >= 0 && lon && lat && type && status, ENKFG_EINVAL, "bad observation arrays");
    for (int o = 0; o < nobs; ++o)
        NEED(type[o] >= 0 && type[o] < ctx->ntypes, ENKFG_EINVAL, "obs %d: type %d out of range", o, (int)type[o]);
    SETDEV();
    enkfg_status s;
    size_t n = nobs > 0 ? nobs : 1;
    void** bufs[] = { (void**)&ctx->d_lon, (void**)&ctx->d_lat, (void**)&ctx->d_type, (void**)&ctx->d_status,
                      (void**)&ctx->d_estd, (void**)&ctx->d_value, (void**)&ctx->d_ox, (void**)&ctx->d_oy,
                      (void**)&ctx->d_oz, (void**)&ctx->d_fi, (void**)&ctx->d_fj, (void**)&ctx->d_fk,
                      (void**)&ctx->d_Hx };
    for (size_t k = 0; k < sizeof(bufs) / sizeof(bufs[0]); ++k) {
        if (*bufs[k]) cudaFree(*bufs[k]);
        *bufs[k] = nullptr;
    }
    CK(cudaMalloc(&ctx->d_lon, n * sizeof(float)));
    CK(cudaMalloc(&ctx->d_lat, n * sizeof(float)));
    CK(cudaMalloc(&ctx->d_type, n * sizeof(short)));
    CK(cudaMalloc(&ctx->d_status, n * sizeof(short)));
    CK(cudaMalloc(&ctx->d_estd, n * sizeof(float)));
    CK(cudaMalloc(&ctx->d_value, n * sizeof(float)));
    CK(cudaMalloc(&ctx->d_ox, n * sizeof(double)));
    CK(cudaMalloc(&ctx->d_oy, n * sizeof(double)));
    if (ctx->geographic) CK(cudaMalloc(&ctx->d_oz, n * sizeof(double)));
    ctx->nobs = nobs;
    ctx->pos_set = ctx->pos_3d = false;
    ctx->he_nmem = 0;
    if (nobs > 0) {
        CK(cudaMemcpyAsync(ctx->d_lon, lon, nobs * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
        CK(cudaMemcpyAsync(ctx->d_lat, lat, nobs * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
        CK(cudaMemcpyAsync(ctx->d_type, type, nobs * sizeof(short), cudaMemcpyHostToDevice, ctx->stream));
        CK(cudaMemcpyAsync(ctx->d_status, status, nobs * sizeof(short), cudaMemcpyHostToDevice, ctx->stream));
        if (estd) CK(cudaMemcpyAsync(ctx->d_estd, estd, nobs * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
        if (value) CK(cudaMemcpyAsync(ctx->d_value, value, nobs * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
        if ((s = upload_obs_coords(ctx, lon, lat, ctx->stream))) return s;
    }
    CK(cudaStreamSynchronize(ctx->stream));
    ctx->obs_set = true;
    ctx->index_valid = false;
    ctx->gather_valid = false;
    ctx->s_mode = 0;
    return ENKFG_OK;
}

enkfg_status alloc_S(enkfg_ctx* ctx, int nmem, int nmem_dynamic)
{
    if (ctx->d_S) cudaFree(ctx->d_S);
    if (ctx->d_s) cudaFree(ctx->d_s);
    if (ctx->d_std) cudaFree(ctx->d_std);
    ctx->d_S = nullptr;
    ctx->d_s = ctx->d_std = nullptr;
    size_t n = ctx->nobs > 0 ? ctx->nobs : 1;
    CK(cudaMalloc(&ctx->d_S, (size_t)nmem * n * sizeof(float)));
    CK(cudaMalloc(&ctx->d_s, n * sizeof(double)));
    CK(cudaMalloc(&ctx->d_std, n * sizeof(double)));
    CK(cudaMemsetAsync(ctx->d_s, 0, n * sizeof(double), ctx->stream));
    ctx->nmem = nmem;
    ctx->nmem_dyn = nmem_dynamic;
    ctx->gather_valid = false;
    return ENKFG_OK;
}

ENKFG_API enkfg_status enkfg_set_HE(enkfg_ctx* ctx, int nmem, int nmem_dynamic, const float* HE)
{
    if (!ctx) return ENKFG_EINVAL;
    NEED(ctx->obs_set, ENKFG_ESTATE, "enkfg_set_obs must come first");
    NEED(nmem >= 2 && nmem <= 144 && nmem_dynamic >= 1 && nmem_dynamic <= nmem && HE, ENKFG_EINVAL,
         "bad ensemble size %d/%d", nmem, nmem_dynamic);
    SETDEV();
    enkfg_status s = alloc_S(ctx, nmem, nmem_dynamic);
    if (s) return s;
    if (ctx->nobs > 0)
        CK(cudaMemcpyAsync(ctx->d_S, HE, (size_t)nmem * ctx->nobs * sizeof(float), cudaMemcpyHostToDevice,
                           ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    ctx->s_mode = 1;
    return ENKFG_OK;
}

ENKFG_API enkfg_status enkfg_set_HE_dev(enkfg_ctx* ctx, int nmem, int nmem_dynamic, const float* HE_dev)
{
    if (!ctx) return ENKFG_EINVAL;
    NEED(ctx->obs_set, ENKFG_ESTATE, "enkfg_set_obs must come first");
    NEED(nmem >= 2 && nmem <= 144 && nmem_dynamic >= 1 && nmem_dynamic <= nmem && HE_dev, ENKFG_EINVAL,
         "bad ensemble size %d/%d", nmem, nmem_dynamic);
    SETDEV();
    if (ctx->d_S == nullptr || ctx->nmem != nmem) {
        enkfg_status s = alloc_S(ctx, nmem, nmem_dynamic);
        if (s) return s;
    }
    ctx->nmem_dyn = nmem_dynamic;
    if (ctx->nobs > 0)
        CK(cudaMemcpyAsync(ctx->d_S, HE_dev, (size_t)nmem * ctx->nobs * sizeof(float), cudaMemcpyDeviceToDevice,
                           ctx->stream));
    ctx->s_mode = 1;
    ctx->gather_valid = false;
    return ENKFG_OK;
}

ENKFG_API enkfg_status enkfg_calc_innovations(enkfg_ctx* ctx, double* s_f, double* std_f)
{
    if (!ctx) return ENKFG_EINVAL;
    NEED(ctx->s_mode == 1, ENKFG_ESTATE, "innovations need HE (enkfg_set_HE) and are computed once");
    SETDEV();
    enkfg_status s;
    if (ctx->nobs > 0 && (s = run_innovations(ctx, ctx->stream))) return s;
    if (s_f && ctx->nobs > 0)
        CK(cudaMemcpyAsync(s_f, ctx->d_s, ctx->nobs * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    if (std_f && ctx->nobs > 0)
        CK(cudaMemcpyAsync(std_f, ctx->d_std, ctx->nobs * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    // wait only when host outputs were asked for (the device-only call stays
    // asynchronous, and can be captured into a CUDA graph)
    if (s_f || std_f) CK(cudaStreamSynchronize(ctx->stream));
    ctx->s_mode = 2;
    ctx->gather_valid = false;
    return ENKFG_OK;
}

ENKFG_API enkfg_status enkfg_standardise(enkfg_ctx* ctx)
{
    if (!ctx) return ENKFG_EINVAL;
    NEED(ctx->s_mode == 2, ENKFG_ESTATE, "standardisation needs innovations (enkfg_calc_innovations)");
    SETDEV();
    enkfg_status s;
    if (ctx->nobs > 0 && (s = run_standardise(ctx, ctx->stream))) return s;
    ctx->s_mode = 3;
    ctx->gather_valid = false;
    return ENKFG_OK;
}

ENKFG_API enkfg_status enkfg_set_S(enkfg_ctx* ctx, int nmem, int nmem_dynamic, const float* S, const double* sv)
{
    if (!ctx) return ENKFG_EINVAL;
    NEED(ctx->obs_set, ENKFG_ESTATE, "enkfg_set_obs must come first");
    NEED(nmem >= 2 && nmem <= 144 && nmem_dynamic >= 1 && nmem_dynamic <= nmem && S && sv, ENKFG_EINVAL,
         "bad ensemble size %d/%d", nmem, nmem_dynamic);
    SETDEV();
    enkfg_status s = alloc_S(ctx, nmem, nmem_dynamic);
    if (s) return s;
    if (ctx->nobs > 0) {
        CK(cudaMemcpyAsync(ctx->d_S, S, (size_t)nmem * ctx->nobs * sizeof(float), cudaMemcpyHostToDevice,
                           ctx->stream));
        CK(cudaMemcpyAsync(ctx->d_s, sv, ctx->nobs * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    }
    CK(cudaStreamSynchronize(ctx->stream));
    ctx->s_mode = 3;
    return ENKFG_OK;
}

ENKFG_API enkfg_status enkfg_get_S(enkfg_ctx* ctx, float* S, double* sv)
{
    if (!ctx) return ENKFG_EINVAL;
    NEED(ctx->s_mode >= 1, ENKFG_ESTATE, "no ensemble observations set");
    SETDEV();
    if (S && ctx->nobs > 0)
        CK(cudaMemcpyAsync(S, ctx->d_S, (size_t)ctx->nmem * ctx->nobs * sizeof(float), cudaMemcpyDeviceToHost,
                           ctx->stream));
    if (sv && ctx->nobs > 0)
        CK(cudaMemcpyAsync(sv, ctx->d_s, ctx->nobs * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return ENKFG_OK;
}

ENKFG_API enkfg_status enkfg_set_grid(enkfg_ctx* ctx, const enkfg_grid* g)
{
    if (!ctx || !g) return ENKFG_EINVAL;
    NEED(ctx->types_set, ENKFG_ESTATE, "enkfg_set_obstypes must come first (geographic flag)");
    NEED(g->mni >= 1 && g->mnj >= 1 && g->stride >= 1, ENKFG_EINVAL, "bad grid %d x %d stride %d", g->mni, g->mnj,
         g->stride);
    NEED((g->x && g->y) || (g->x2d && g->y2d), ENKFG_EINVAL, "grid coordinates are required");
    // a point without coordinates (a grid of type NONE) takes every
    // observation in the reference (obs_getglobal, observations.c:
    // 1773-1817); the device search does not do that, so such grids are
    // refused rather than given T = I
    {
        const int nj = (g->mnj - 1) / g->stride + 1, ni = (g->mni - 1) / g->stride + 1;
        for (int j = 0; j < nj; ++j)
            for (int i = 0; i < ni; ++i) {
                const size_t jj = (size_t)j * g->stride, ii = (size_t)i * g->stride;
                const double x = g->x2d ? g->x2d[jj * g->mni + ii] : g->x[ii];
                const double y = g->x2d ? g->y2d[jj * g->mni + ii] : g->y[jj];
                NEED(!isnan(x + y), ENKFG_EUNSUPPORTED,
                     "grid point (%zu, %zu) has no coordinates (a grid of type NONE is not supported)", ii, jj);
            }
    }
    SETDEV();
    ctx->mni = g->mni;
    ctx->mnj = g->mnj;
    ctx->stride = g->stride;
    ctx->periodic_i = g->periodic_i ? 1 : 0;
    ctx->nj = (g->mnj - 1) / g->stride + 1;
    ctx->ni = (g->mni - 1) / g->stride + 1;
    int npts = ctx->nj * ctx->ni;
    if (ctx->d_qx) cudaFree(ctx->d_qx);
    if (ctx->d_qy) cudaFree(ctx->d_qy);
    if (ctx->d_qz) cudaFree(ctx->d_qz);
    ctx->d_qx = ctx->d_qy = ctx->d_qz = nullptr;
    CK(cudaMalloc(&ctx->d_qx, npts * sizeof(double)));
    CK(cudaMalloc(&ctx->d_qy, npts * sizeof(double)));
    if (ctx->geographic) CK(cudaMalloc(&ctx->d_qz, npts * sizeof(double)));
    enkfg_status s = upload_query_coords(ctx, g, ctx->stream);
    if (s) return s;
    ctx->grid_set = true;
    ctx->t_valid = false;
    ctx->cut_valid = false;
    return ENKFG_OK;
}

ENKFG_API enkfg_status enkfg_transform_dims(const enkfg_ctx* ctx, int* nj, int* ni)
{
    if (!ctx || !ctx->grid_set) return ENKFG_ESTATE;
    if (nj) *nj = ctx->nj;
    if (ni) *ni = ctx->ni;
    return ENKFG_OK;
}

ENKFG_API enkfg_status enkfg_local_obs(enkfg_ctx* ctx, int* counts, long long* offsets, int* ids, double* coeffs,
                                      long long capacity)
{
    if (!ctx) return ENKFG_EINVAL;
    NEED(ctx->obs_set && ctx->grid_set, ENKFG_ESTATE, "observations and grid must be set");
    NEED(counts, ENKFG_EINVAL, "counts is required");
    NEED(!ids || (offsets && coeffs), ENKFG_EINVAL, "ids needs offsets and coeffs");
    SETDEV();
    enkfg_status s;
    cudaStream_t st = ctx->stream;
    if ((s = prepare_search(ctx, st))) return s;
    int npts = ctx->nj * ctx->ni;
    if ((s = ensure(ctx, &ctx->d_counts, &ctx->counts_cap, (size_t)npts))) return s;
    if ((s = count_local(ctx, ctx->d_counts, nullptr, st))) return s;
    CK(cudaMemcpyAsync(counts, ctx->d_counts, npts * sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (!ids) return ENKFG_OK;
    long long* d_off;
    CK(cudaMalloc(&d_off, (npts + 1) * sizeof(long long)));
    if ((s = scan_counts(ctx, ctx->d_counts, d_off, npts, st))) {
        cudaFree(d_off);
        return s;
    }
    long long total = 0;
    cudaMemcpyAsync(&total, d_off + npts, sizeof(long long), cudaMemcpyDeviceToHost, st);
    cudaStreamSynchronize(st);
    if (total > capacity) {
        cudaFree(d_off);
        set_err(ctx, "%lld local observations exceed the capacity %lld", total, capacity);
        return ENKFG_ECAPACITY;
    }
    int* d_ids = nullptr;
    double* d_c = nullptr;
    cudaError_t e1 = cudaMalloc(&d_ids, (total > 0 ? total : 1) * sizeof(int));
    cudaError_t e2 = cudaMalloc(&d_c, (total > 0 ? total : 1) * sizeof(double));
    if (e1 != cudaSuccess || e2 != cudaSuccess) {
        cudaGetLastError();
        cudaFree(d_off);
        cudaFree(d_ids);
        cudaFree(d_c);
        set_err(ctx, "cannot allocate %lld list entries", total);
        return ENKFG_ENOMEM;
    }
    s = list_local(ctx, d_off, d_ids, d_c, st);
    if (!s) {
        cudaMemcpyAsync(offsets, d_off, (npts + 1) * sizeof(long long), cudaMemcpyDeviceToHost, st);
        cudaMemcpyAsync(ids, d_ids, total * sizeof(int), cudaMemcpyDeviceToHost, st);
        cudaMemcpyAsync(coeffs, d_c, total * sizeof(double), cudaMemcpyDeviceToHost, st);
        cudaError_t e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) s = cuda_fail(ctx, e, "list copy", __LINE__);
    }
    cudaFree(d_off);
    cudaFree(d_ids);
    cudaFree(d_c);
    return s;
}

static enkfg_status check_calc(enkfg_ctx* ctx, const enkfg_calc_params* p)
{
    NEED(p, ENKFG_EINVAL, "params are required");
    NEED(ctx->obs_set && ctx->grid_set, ENKFG_ESTATE, "observations and grid must be set");
    NEED(ctx->s_mode == 3, ENKFG_ESTATE, "S must be standardised (enkfg_standardise or enkfg_set_S)");
    NEED(p->mode == ENKFG_MODE_ENKF || p->mode == ENKFG_MODE_ENOI || p->mode == ENKFG_MODE_HYBRID, ENKFG_EINVAL,
         "bad mode %d", p->mode);
    NEED(p->scheme == ENKFG_SCHEME_DENKF || p->scheme == ENKFG_SCHEME_ETKF, ENKFG_EINVAL, "bad scheme %d", p->scheme);
    NEED(p->path == ENKFG_PATH_PLAIN || p->path == ENKFG_PATH_BATCHED, ENKFG_EINVAL, "bad path %d", p->path);
    NEED(isfinite(p->alpha), ENKFG_EINVAL, "alpha must be finite");
    return ENKFG_OK;
}

static enkfg_status finish_calc(enkfg_ctx* ctx, cudaStream_t st)
{
    int npts = ctx->nj * ctx->ni;
    CK(cudaStreamSynchronize(st));
    // first failing point, if any
    int* h = (int*)malloc(npts * sizeof(int));
    if (!h) return ENKFG_ENOMEM;
    CK(cudaMemcpy(h, ctx->d_status_pt, npts * sizeof(int), cudaMemcpyDeviceToHost));
    for (int k = 0; k < npts; ++k)
        if (h[k] == ENKFG_POINT_TIMEOUT) {
            set_err(ctx, "local analysis (j=%d, i=%d): a device wait exceeded its limit (%llu ns)", k / ctx->ni,
                    k % ctx->ni, ctx->wait_ns);
            free(h);
            return ENKFG_ETIMEOUT;
        }
    for (int k = 0; k < npts; ++k)
        if (h[k]) {
            set_err(ctx, "local analysis (j=%d, i=%d): factorisation failed (code %d)", k / ctx->ni, k % ctx->ni, h[k]);
            free(h);
            return ENKFG_ENUMERIC;
        }
    free(h);
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[1]);
    ctx->stage_ms[0] = ms;
    cudaEventElapsedTime(&ms, ctx->ev[1], ctx->ev[2]);
    ctx->stage_ms[1] = ms;
    cudaEventElapsedTime(&ms, ctx->ev[2], ctx->ev[3]);
    ctx->stage_ms[2] = ms;
    return ENKFG_OK;
}

ENKFG_API enkfg_status enkfg_calc_transforms_dev(enkfg_ctx* ctx, const enkfg_calc_params* p, void* stream)
{
    if (!ctx) return ENKFG_EINVAL;
    enkfg_status s = check_calc(ctx, p);
    if (s) return s;
    SETDEV();
    ctx->want64 = false;
    return run_transforms(ctx, p, pick(ctx, stream));
}

ENKFG_API enkfg_status enkfg_calc_transforms(enkfg_ctx* ctx, const enkfg_calc_params* p, float* T, float* w,
                                             double* T64, double* w64, const enkfg_diag* diag)
{
    if (!ctx) return ENKFG_EINVAL;
    enkfg_status s = check_calc(ctx, p);
    if (s) return s;
    NEED(w, ENKFG_EINVAL, "w is required");
    bool enkf = (p->mode != ENKFG_MODE_ENOI);
    NEED(!enkf || T, ENKFG_EINVAL, "T is required for EnKF/hybrid");
    SETDEV();
    cudaStream_t st = ctx->stream;
    enkfg_calc_params q = *p;
    if (diag && diag->nlobs) q.want_diag = 1;
    ctx->want64 = (T64 != nullptr || w64 != nullptr);
    // T and w leave batch by batch on the output copy stream while the next
    // batch runs, where the batches cover contiguous ranges of points
    if (ctx->cstream[1] == nullptr) CK(cudaStreamCreateWithFlags(&ctx->cstream[1], cudaStreamNonBlocking));
    if (ctx->out_ev == nullptr) CK(cudaEventCreateWithFlags(&ctx->out_ev, cudaEventDisableTiming));
    struct OutGuard {
        enkfg_ctx* c;
        ~OutGuard()
        {
            c->out_T = c->out_w = nullptr;
            c->out_T64 = c->out_w64 = nullptr;
            c->out_seg = 0;
        }
    } guard{ ctx };
    ctx->out_T = enkf ? T : nullptr;
    ctx->out_w = w;
    ctx->out_T64 = enkf ? T64 : nullptr;
    ctx->out_w64 = w64;
    ctx->out_seg = 1;
    s = run_transforms(ctx, &q, st);
    const bool per_batch = ctx->out_seg > 0;
    ctx->out_seg = 0;
    cudaStreamSynchronize(ctx->cstream[1]);   // no copy in flight past this call
    if (s) return s;
    if ((s = finish_calc(ctx, st))) return s;
    size_t npts = (size_t)ctx->nj * ctx->ni, m = ctx->nmem, md = ctx->nmem_dyn;
    if (!per_batch) {
        if (enkf) CK(cudaMemcpyAsync(T, ctx->d_T, npts * md * m * sizeof(float), cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(w, ctx->d_w, npts * m * sizeof(float), cudaMemcpyDeviceToHost, st));
        if (enkf && T64)
            CK(cudaMemcpyAsync(T64, ctx->d_T64, npts * md * m * sizeof(double), cudaMemcpyDeviceToHost, st));
        if (w64) CK(cudaMemcpyAsync(w64, ctx->d_w64, npts * m * sizeof(double), cudaMemcpyDeviceToHost, st));
    }
    if (diag && q.want_diag) {
        size_t pn = npts * ctx->ntypes;
        if (diag->nlobs) CK(cudaMemcpyAsync(diag->nlobs, ctx->d_nlobs, npts * sizeof(int), cudaMemcpyDeviceToHost, st));
        if (diag->dfs) CK(cudaMemcpyAsync(diag->dfs, ctx->d_dfs, npts * sizeof(float), cudaMemcpyDeviceToHost, st));
        if (diag->srf) CK(cudaMemcpyAsync(diag->srf, ctx->d_srf, npts * sizeof(float), cudaMemcpyDeviceToHost, st));
        if (diag->pnlobs) CK(cudaMemcpyAsync(diag->pnlobs, ctx->d_pnlobs, pn * sizeof(int), cudaMemcpyDeviceToHost, st));
        if (diag->pdfs) CK(cudaMemcpyAsync(diag->pdfs, ctx->d_pdfs, pn * sizeof(float), cudaMemcpyDeviceToHost, st));
        if (diag->psrf) CK(cudaMemcpyAsync(diag->psrf, ctx->d_psrf, pn * sizeof(float), cudaMemcpyDeviceToHost, st));
    }
    CK(cudaStreamSynchronize(st));
    return ENKFG_OK;
}

ENKFG_API enkfg_status enkfg_transforms_dev_ptr(enkfg_ctx* ctx, float** T, float** w)
{
    if (!ctx) return ENKFG_EINVAL;
    NEED(ctx->t_valid, ENKFG_ESTATE, "no transforms computed");
    if (T) *T = ctx->d_T;
    if (w) *w = ctx->d_w;
    return ENKFG_OK;
}

ENKFG_API enkfg_status enkfg_set_transforms(enkfg_ctx* ctx, int mode, int nmem, int nmem_dynamic, const float* T,
                                            const float* w)
{
    if (!ctx) return ENKFG_EINVAL;
    NEED(ctx->grid_set, ENKFG_ESTATE, "the grid must be set");
    NEED(w && (mode == ENKFG_MODE_ENOI || T), ENKFG_EINVAL, "T/w are required");
    NEED(nmem >= 2 && nmem_dynamic >= 1 && nmem_dynamic <= nmem, ENKFG_EINVAL, "bad ensemble size");
    SETDEV();
    enkfg_status s;
    size_t npts = (size_t)ctx->nj * ctx->ni;
    size_t nT = mode == ENKFG_MODE_ENOI ? 1 : npts * nmem_dynamic * nmem;
    if ((s = ensure(ctx, &ctx->d_T, &ctx->T_cap, nT))) return s;
    if ((s = ensure(ctx, &ctx->d_w, &ctx->w_cap, npts * nmem))) return s;
    if (mode != ENKFG_MODE_ENOI)
        CK(cudaMemcpyAsync(ctx->d_T, T, nT * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(ctx->d_w, w, npts * nmem * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    ctx->t_mode = mode;
    ctx->t_nmem = nmem;
    ctx->t_ndyn = nmem_dynamic;
    ctx->t_valid = true;
    return ENKFG_OK;
}

static enkfg_status check_update(enkfg_ctx* ctx, const enkfg_update_params* p, int nfield, const int* levels)
{
    NEED(p && levels && nfield >= 1, ENKFG_EINVAL, "params, levels and nfield >= 1 are required");
    NEED(ctx->grid_set, ENKFG_ESTATE, "the grid must be set");
    NEED(p->mode == ENKFG_MODE_ENKF || p->mode == ENKFG_MODE_HYBRID || p->mode == ENKFG_MODE_ENOI, ENKFG_EINVAL,
         "bad mode");
    NEED(p->nmem >= 2 && p->nmem_dynamic >= 0 && p->nmem_dynamic <= p->nmem, ENKFG_EINVAL, "bad ensemble size");
    return ENKFG_OK;
}

// The noise given by enkfg_set_field_noise is for this call: it must match
// its field-layers and ensemble (and is used up by it).
static enkfg_status take_noise(enkfg_ctx* ctx, const enkfg_update_params* p, int nfield, bool* on)
{
    *on = ctx->noise_nfield > 0;
    if (!*on) return ENKFG_OK;
    const int nf = ctx->noise_nfield, nm = ctx->noise_nmem;
    ctx->noise_nfield = 0;
    NEED(p->mode != ENKFG_MODE_ENOI, ENKFG_EINVAL, "RANDOMISE noise is not applied by the EnOI update");
    NEED(nf == nfield && nm == p->nmem, ENKFG_EINVAL, "noise given for %d field-layers of %d members, update of %d of %d",
         nf, nm, nfield, p->nmem);
    return ENKFG_OK;
}

ENKFG_API enkfg_status enkfg_set_field_noise(enkfg_ctx* ctx, int nfield, int nmem, const double* deflation,
                                             const double* sigma, const double* random)
{
    if (!ctx) return ENKFG_EINVAL;
    ctx->noise_nfield = 0;
    if (nfield == 0 || deflation == nullptr) return ENKFG_OK;
    NEED(nfield > 0 && nmem >= 1 && sigma && random, ENKFG_EINVAL, "bad noise arguments");
    // addnoise (update/update.c:46-87): the mean of the member normals is
    // removed; mult = (float)(sqrt(1 - deflation^2) * sigma); each member's
    // term mult * r_e in double
    const size_t n = (size_t)nfield * (nmem + 1);
    double* h = (double*)malloc(n * sizeof(double));
    NEED(h, ENKFG_ENOMEM, "host allocation failed");
    for (int f = 0; f < nfield; ++f) {
        const double d = deflation[f];
        double* term = h + nfield + (size_t)f * nmem;
        h[f] = d;
        if (isnan(d)) {
            for (int e = 0; e < nmem; ++e) term[e] = 0.0;
            continue;
        }
        // the reference's model parameters allow a deflation in [0, 1]
        // (common/model.c:253-256)
        if (!(d >= 0.0 && d <= 1.0) || !isfinite(sigma[f])) {
            free(h);
            set_err(ctx, "field-layer %d: deflation %g (must be in [0, 1]), sigma %g", f, d, sigma[f]);
            return ENKFG_EINVAL;
        }
        const double* r = random + (size_t)f * nmem;
        double sum = 0.0;
        for (int e = 0; e < nmem; ++e) sum += r[e];
        sum /= (double)nmem;
        const double dd = d * d;
        const float mult = (float)(sqrt(1.0 - dd) * sigma[f]);
        for (int e = 0; e < nmem; ++e) term[e] = (double)mult * (r[e] - sum);
    }
    SETDEV();
    enkfg_status s = ensure(ctx, &ctx->d_noise, &ctx->noise_cap, n);
    if (!s) {
        cudaError_t e = cudaMemcpy(ctx->d_noise, h, n * sizeof(double), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) s = cuda_fail(ctx, e, "noise upload", __LINE__);
    }
    free(h);
    if (s) return s;
    ctx->noise_nfield = ctx->noise_nlayer = nfield;
    ctx->noise_nmem = nmem;
    return ENKFG_OK;
}

ENKFG_API enkfg_status enkfg_update_fields_dev(enkfg_ctx* ctx, const enkfg_update_params* p, const int* numlevels_dev,
                                               int nfield, const int* levels, float* fields_dev, float* infl_dev,
                                               void* stream)
{
    if (!ctx) return ENKFG_EINVAL;
    enkfg_status s = check_update(ctx, p, nfield, levels);
    if (s) return s;
    bool noise;
    if ((s = take_noise(ctx, p, nfield, &noise))) return s;
    NEED(numlevels_dev && fields_dev, ENKFG_EINVAL, "device buffers are required");
    SETDEV();
    cudaStream_t st = pick(ctx, stream);
    if ((s = run_update(ctx, p, numlevels_dev, nfield, levels, fields_dev, infl_dev, st))) return s;
    if (noise) {
        const int j2 = p->j2 < 0 ? ctx->mnj - 1 : p->j2;
        s = run_noise(ctx, fields_dev, 0, nfield, p->nmem, (long long)(j2 - p->j1 + 1) * ctx->mni, st);
    }
    return s;
}

// The host-buffer update streams the field-layers through the device in
// units (the reference's FIELDBUFFERSIZE batches, update/update.c:1552-2132):
// a unit is a group of field-layers -- whole multiples of the update
// kernel's ten-layer pass where it can, within about 3 GB -- cut into blocks
// of model rows of about UPD_UNIT_BYTES (a multiple of the stride, so that a
// block starts on a strided row and its rows interpolate X5 exactly as in
// one call).  Three device buffers in turn: the copy of unit u + 1 in and of
// unit u - 1 out run on the context's two copy streams (one 2-D copy each,
// the unit's rows of every member plane) while unit u is updated.  With
// pinned host buffers the copies overlap the update; with pageable ones they
// are staged by the driver and serialise.
#define UPD_GROUP_BYTES ((size_t)3 << 30)
#define UPD_UNIT_BYTES ((size_t)512 << 20)
ENKFG_API enkfg_status enkfg_update_fields(enkfg_ctx* ctx, const enkfg_update_params* p, const int* numlevels,
                                          int nfield, const int* levels, float* fields, float* infl)
{
    if (!ctx) return ENKFG_EINVAL;
    enkfg_status s = check_update(ctx, p, nfield, levels);
    if (s) return s;
    bool noise;
    if ((s = take_noise(ctx, p, nfield, &noise))) return s;
    NEED(numlevels && fields, ENKFG_EINVAL, "numlevels and fields are required");
    SETDEV();
    cudaStream_t st = ctx->stream;
    int j2 = p->j2 < 0 ? ctx->mnj - 1 : p->j2;
    const int jsize = j2 - p->j1 + 1;
    const size_t mni = (size_t)ctx->mni;
    const size_t plane = (size_t)jsize * mni;
    const int mp = p->mode == ENKFG_MODE_ENOI ? p->nmem + 1 : p->nmem;   // member planes a field-layer
    const size_t per = (size_t)mp * plane;                                // floats per field-layer
    int G = (int)(UPD_GROUP_BYTES / (per * sizeof(float)));
    if (G < 1) G = 1;
    if (G >= 10) G -= G % 10;
    if (ctx->field_buffer > 0) G = ctx->field_buffer;
    if (G > nfield) G = nfield;
    const int ngroups = (nfield + G - 1) / G;
    // rows per unit
    const int stp = ctx->stride > 0 ? ctx->stride : 1;
    int R = (int)(UPD_UNIT_BYTES / ((size_t)G * mp * mni * sizeof(float)));
    if (ctx->field_rows > 0) R = (ctx->field_rows + stp - 1) / stp * stp;
    R -= R % stp;
    if (R < stp) R = stp;
    if (R > jsize) R = jsize;
    const int nrb = (jsize + R - 1) / R;
    const int nunits = ngroups * nrb;
    const int nbuf = nunits < 3 ? nunits : 3;
    const size_t ufl = (size_t)G * mp * R * mni, uinf = (size_t)G * R * mni;   // floats a buffer
    if ((s = ensure(ctx, &ctx->d_numlevels, &ctx->numlevels_cap, (size_t)ctx->mnj * ctx->mni))) return s;
    if ((s = ensure(ctx, &ctx->d_fields, &ctx->fields_cap, (size_t)nbuf * ufl))) return s;
    if (infl && (s = ensure(ctx, &ctx->d_infl, &ctx->infl_cap, (size_t)nbuf * uinf))) return s;
    for (int k = 0; k < 2; ++k)
        if (ctx->cstream[k] == nullptr) CK(cudaStreamCreateWithFlags(&ctx->cstream[k], cudaStreamNonBlocking));
    for (int k = 0; k < 9; ++k)
        if (ctx->uev[k] == nullptr) CK(cudaEventCreateWithFlags(&ctx->uev[k], cudaEventDisableTiming));
    cudaStream_t cin = ctx->cstream[0], cout = ctx->cstream[1];
    CK(cudaMemcpyAsync(ctx->d_numlevels, numlevels, (size_t)ctx->mnj * ctx->mni * sizeof(int), cudaMemcpyHostToDevice,
                       st));
    cudaEventRecord(ctx->ev[6], st);
    for (int u = 0; u < nunits; ++u) {
        const int g = u / nrb, rb = u - g * nrb;
        const int b = u % nbuf, f0 = g * G, nf = (nfield - f0 < G) ? nfield - f0 : G;
        const int r0 = rb * R, rr = (jsize - r0 < R) ? jsize - r0 : R;
        const size_t wbytes = (size_t)rr * mni * sizeof(float);            // one member plane's rows
        float* dbuf = ctx->d_fields + (size_t)b * ufl;
        float* dinf = infl ? ctx->d_infl + (size_t)b * uinf : nullptr;
        float* hsrc = fields + (size_t)f0 * per + (size_t)r0 * mni;
        cudaEvent_t in_done = ctx->uev[3 * b], upd_done = ctx->uev[3 * b + 1], out_done = ctx->uev[3 * b + 2];
        // the buffer's previous unit has left the device; the update before
        // this call (stream order of st) has finished with the buffers
        if (u >= nbuf) CK(cudaStreamWaitEvent(cin, out_done, 0));
        else {
            CK(cudaEventRecord(in_done, st));
            CK(cudaStreamWaitEvent(cin, in_done, 0));
        }
        CK(cudaMemcpy2DAsync(dbuf, wbytes, hsrc, plane * sizeof(float), wbytes, (size_t)nf * mp,
                             cudaMemcpyHostToDevice, cin));
        CK(cudaEventRecord(in_done, cin));
        CK(cudaStreamWaitEvent(st, in_done, 0));
        enkfg_update_params pu = *p;
        pu.j1 = p->j1 + r0;
        pu.j2 = pu.j1 + rr - 1;
        if ((s = run_update(ctx, &pu, ctx->d_numlevels, nf, levels + f0, dbuf, dinf, st))) return s;
        if (noise && (s = run_noise(ctx, dbuf, f0, nf, p->nmem, (long long)rr * mni, st))) return s;
        CK(cudaEventRecord(upd_done, st));
        CK(cudaStreamWaitEvent(cout, upd_done, 0));
        CK(cudaMemcpy2DAsync(hsrc, plane * sizeof(float), dbuf, wbytes, wbytes, (size_t)nf * mp,
                             cudaMemcpyDeviceToHost, cout));
        if (infl)
            CK(cudaMemcpy2DAsync(infl + (size_t)f0 * plane + (size_t)r0 * mni, plane * sizeof(float), dinf, wbytes,
                                 wbytes, (size_t)nf, cudaMemcpyDeviceToHost, cout));
        CK(cudaEventRecord(out_done, cout));
    }
    cudaEventRecord(ctx->ev[7], st);
    CK(cudaStreamSynchronize(cout));
    CK(cudaStreamSynchronize(st));
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, ctx->ev[6], ctx->ev[7]);
    ctx->stage_ms[3] = ms;
    return ENKFG_OK;
}

ENKFG_API enkfg_status enkfg_set_hybrid_ensemble_dev(enkfg_ctx* ctx, int nmem, int nmem_dynamic, double gamma, int nij,
                                                     float* v_dev, void* stream)
{
    if (!ctx) return ENKFG_EINVAL;
    NEED(nmem > nmem_dynamic + 1 && nmem_dynamic >= 1 && nij >= 0 && v_dev, ENKFG_EINVAL,
         "hybrid needs at least 2 static members");
    SETDEV();
    return run_hybrid(ctx, nmem, nmem_dynamic, gamma, nij, v_dev, pick(ctx, stream));
}

ENKFG_API enkfg_status enkfg_set_hybrid_ensemble(enkfg_ctx* ctx, int nmem, int nmem_dynamic, double gamma, int nij,
                                                 float* v)
{
    if (!ctx) return ENKFG_EINVAL;
    NEED(nmem > nmem_dynamic + 1 && nmem_dynamic >= 1 && nij >= 0 && v, ENKFG_EINVAL,
         "hybrid needs at least 2 static members");
    SETDEV();
    enkfg_status s;
    size_t n = (size_t)nmem * nij;
    if ((s = ensure(ctx, &ctx->d_fields, &ctx->fields_cap, n))) return s;
    CK(cudaMemcpyAsync(ctx->d_fields, v, n * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
    if ((s = run_hybrid(ctx, nmem, nmem_dynamic, gamma, nij, ctx->d_fields, ctx->stream))) return s;
    CK(cudaMemcpyAsync(v, ctx->d_fields, n * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return ENKFG_OK;
}

}  // extern "C"
