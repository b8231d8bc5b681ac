// update.cu -- application of the ensemble transforms to the model fields
// (das_updatefields, reference update/update.c:92-564; das_updatebg,
// update.c:568-814) and hybrid ensemble conditioning (das_sethybridensemble,
// common/dasystem.c:775-819).
//
// Field layout is the reference's: one field-layer is [nmem][jsize][mni]
// floats (member slabs); nfield field-layers follow each other.
//
// das_updatefields: a CTA owns NK consecutive cells of one model row for all
// field-layers of the call.  The [nfield][nmem][NK] block is staged in shared
// memory with coalesced row loads (NK consecutive floats per member slab).
// For each cell the interpolated transform X5 = (T, w) is built once in
// shared memory -- exactly the reference's float arithmetic: linear in j
// (weights stepj/stride) then in i (stepi/stride), constant past the last
// strided row/column, periodic wrap in i (update.c:195-272) -- and every
// warp applies it to one field-layer: mask, missing-value test, ensemble
// mean (FP64), anomalies, A^a = A^f T (FP32), mean update with w (FP64),
// hybrid rescaling, spread-limited inflation, increment output.
//
// das_updatebg (EnOI) and das_sethybridensemble are per-cell sequential
// loops in the reference; here one thread owns one cell and runs the same
// sequence of float/double operations, so results are bit-identical.
#include "internal.cuh"
#include <math.h>

#define UPD_NT 256
#define MAXOBSVAL_F 999999.0f

struct UpdArgs {
    int mode, m, md, mni, ni, nj, stride, periodic_i, j1, jsize, nfield;
    int surfk, issurfacevar, output_increment, applylog;
    float inflation0;
    double inf_ratio;
    const int* numlevels;
    const int* levels;
    const float* T;
    const float* w;
    float* fields;
    float* infl;
    size_t plane;               // jsize * mni
    int nk;                     // cells per CTA
};

// One element of the interpolated X5 for model cell (jt, i) of the tile
// (update.c:195-272): X is the strided array [nj][ni][nelem].
__device__ __forceinline__ float interp_x5(const float* __restrict__ X, int nelem, int e, int jj, int stepj, int ii,
                                           int stepi, const UpdArgs& a)
{
    const int ni = a.ni, nj = a.nj, stride = a.stride;
    float v1 = __ldg(&X[((size_t)jj * ni + ii) * nelem + e]);
    int ii2 = 0;
    if (stride > 1 && stepi > 0) ii2 = (ii < ni - 1) ? ii + 1 : (a.periodic_i ? (ii + 1) % ni : ii);
    if (stride > 1 && stepj > 0) {
        int jj2 = (jj < nj - 1) ? jj + 1 : jj;
        float w2 = __fdiv_rn((float)stepj, (float)stride);
        float w1 = __fsub_rn(1.0f, w2);
        float b = __ldg(&X[((size_t)jj2 * ni + ii) * nelem + e]);
        v1 = __fadd_rn(__fmul_rn(v1, w1), __fmul_rn(b, w2));
        if (stepi > 0) {
            float c = __ldg(&X[((size_t)jj * ni + ii2) * nelem + e]);
            float d = __ldg(&X[((size_t)jj2 * ni + ii2) * nelem + e]);
            float v2 = __fadd_rn(__fmul_rn(c, w1), __fmul_rn(d, w2));
            float u2 = __fdiv_rn((float)stepi, (float)stride);
            float u1 = __fsub_rn(1.0f, u2);
            return __fadd_rn(__fmul_rn(v1, u1), __fmul_rn(v2, u2));
        }
        return v1;
    }
    if (stride > 1 && stepi > 0) {
        float v2 = __ldg(&X[((size_t)jj * ni + ii2) * nelem + e]);
        float u2 = __fdiv_rn((float)stepi, (float)stride);
        float u1 = __fsub_rn(1.0f, u2);
        return __fadd_rn(__fmul_rn(v1, u1), __fmul_rn(v2, u2));
    }
    return v1;
}

__device__ __forceinline__ double warp_sum_d(double v)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

#define MAXE_PER_LANE 5   // members per lane (nmem <= 160)

__global__ void __launch_bounds__(UPD_NT) k_update_fields(UpdArgs a)
{
    extern __shared__ __align__(16) float usm[];
    const int m = a.m, md = a.md, nk = a.nk, nf = a.nfield;
    const int TLD = m + 1;
    float* Tc = usm;                                   // [md][m+1]
    float* wc = Tc + (size_t)md * TLD;                 // [m]
    float* tile = wc + ((m + 3) & ~3);                 // [nf][m][nk]
    float* Asm = tile + (size_t)nf * m * nk;           // [UPD_NT/32][m]
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int jt = blockIdx.y;
    const int i0 = blockIdx.x * nk;
    const int ncell = min(nk, a.mni - i0);
    const int jj = a.j1 / a.stride + jt / a.stride, stepj = jt % a.stride;
    const int jg = a.j1 + jt;

    // stage the field block
    for (int idx = tid; idx < nf * m * nk; idx += UPD_NT) {
        int c = idx % nk, fe = idx / nk;
        if (c < ncell) {
            int f = fe / m, e = fe - f * m;
            tile[idx] = a.fields[((size_t)f * m + e) * a.plane + (size_t)jt * a.mni + i0 + c];
        }
    }
    float* Aw = Asm + wid * m;

    for (int c = 0; c < ncell; ++c) {
        const int i = i0 + c;
        const int ii = i / a.stride, stepi = i % a.stride;
        __syncthreads();
        for (int idx = tid; idx < md * m; idx += UPD_NT) {
            int e1 = idx / m, e2 = idx - e1 * m;
            Tc[e1 * TLD + e2] = interp_x5(a.T, md * m, idx, jj, stepj, ii, stepi, a);
        }
        for (int idx = tid; idx < m; idx += UPD_NT) wc[idx] = interp_x5(a.w, m, idx, jj, stepj, ii, stepi, a);
        __syncthreads();
        const int nl = a.numlevels[(size_t)jg * a.mni + i];
        for (int f = wid; f < nf; f += UPD_NT / 32) {
            float* v = tile + (size_t)f * m * nk;      // v[e * nk + c]
            const int level = a.levels[f];
            float inflation = a.inflation0;
            bool masked = (a.surfk == 0) ? (nl <= level) : (nl <= (a.issurfacevar ? 0 : a.surfk - level));
            if (masked) {
                for (int e = lane; e < m; e += 32) v[e * nk + c] = 0.0f;
                if (a.infl && lane == 0) a.infl[(size_t)f * a.plane + (size_t)jt * a.mni + i] = 0.0f;
                continue;
            }
            // first member with a missing value (update.c:337-350)
            int first = m;
            for (int e0 = 0; e0 < m && first == m; e0 += 32) {
                int e = e0 + lane;
                bool bad = false;
                if (e < m) {
                    float x = v[e * nk + c];
                    bad = !isfinite(x) || fabsf(x) > MAXOBSVAL_F;
                }
                unsigned bal = __ballot_sync(0xffffffffu, bad);
                if (bal) first = e0 + __ffs(bal) - 1;
            }
            if (first < md) {
                for (int e = lane; e < m; e += 32) v[e * nk + c] = 0.0f;
                if (a.infl && lane == 0) a.infl[(size_t)f * a.plane + (size_t)jt * a.mni + i] = 0.0f;
                continue;
            } else if (first < m) {
                for (int e = md + lane; e < m; e += 32) v[e * nk + c] = 0.0f;
                if (md == 0) continue;
            }
            // ensemble mean of the dynamic members (FP64)
            double s = 0.0;
            for (int e = lane; e < md; e += 32) s += (double)v[e * nk + c];
            const double v1_f = warp_sum_d(s) / (double)md;
            // anomalies of all members
            for (int e = lane; e < m; e += 32) Aw[e] = (float)((double)v[e * nk + c] - v1_f);
            __syncwarp();
            // A^a = A^f T  (T[e1] is column e1 of the reference's m x m_dyn
            // matrix, update.c:399)
            float aa[MAXE_PER_LANE];
#pragma unroll
            for (int k = 0; k < MAXE_PER_LANE; ++k) {
                int e1 = lane + 32 * k;
                float acc = 0.0f;
                if (e1 < md) {
                    const float* Tr = Tc + e1 * TLD;
                    for (int e2 = 0; e2 < m; ++e2) acc = fmaf(Tr[e2], Aw[e2], acc);
                }
                aa[k] = acc;
            }
            // mean increment: sum of float products in FP64 (update.c:405-410)
            s = 0.0;
            for (int e = lane; e < m; e += 32) s += (double)__fmul_rn(Aw[e], wc[e]);
            const double v1_a = warp_sum_d(s) + v1_f;
            float af[MAXE_PER_LANE];
#pragma unroll
            for (int k = 0; k < MAXE_PER_LANE; ++k) {
                int e1 = lane + 32 * k;
                af[k] = (e1 < m) ? Aw[e1] : 0.0f;
            }
            if (a.mode == ENKFG_MODE_HYBRID) {
                double k_d = (md > 1) ? sqrt((double)(m - 1) / (double)(md - 1)) : 1.0;
#pragma unroll
                for (int k = 0; k < MAXE_PER_LANE; ++k)
                    if (lane + 32 * k < md) {
                        aa[k] = (float)((double)aa[k] / k_d);
                        af[k] = (float)((double)af[k] / k_d);
                    }
            }
            if (!isnan(a.inf_ratio)) {
                double s2f = 0.0, s2a = 0.0;
#pragma unroll
                for (int k = 0; k < MAXE_PER_LANE; ++k)
                    if (lane + 32 * k < md) {
                        s2f += (double)__fmul_rn(af[k], af[k]);
                        s2a += (double)__fmul_rn(aa[k], aa[k]);
                    }
                double v2_f = warp_sum_d(s2f), v2_a = warp_sum_d(s2a);
                if (v2_a > 0.0) {
                    inflation = (float)(sqrt(v2_f / v2_a) * a.inf_ratio + 1.0 - a.inf_ratio);
                    if (inflation >= a.inflation0) inflation = a.inflation0;
                }
            }
            const bool inflate = __fsub_rn(inflation, 1.0f) > 1.0e-6f;
            if (!inflate) inflation = 1.0f;
#pragma unroll
            for (int k = 0; k < MAXE_PER_LANE; ++k) {
                int e1 = lane + 32 * k;
                if (e1 < md) {
                    float va = inflate ? __fmul_rn(aa[k], inflation) : aa[k];
                    va = (float)((double)va + v1_a);
                    float vf = (float)((double)af[k] + v1_f);
                    float out;
                    if (!a.output_increment) out = va;
                    else if (!a.applylog) out = __fsub_rn(va, vf);
                    else {
                        // --output-increment of a log10 variable: difference
                        // in physical space, 0 where the forecast is not a
                        // normal number (update.c:484-497)
                        float avf = fabsf(vf);
                        bool normal = (avf >= 1.17549435e-38f) && (avf <= 3.40282347e+38f);
                        double ea = pow(10.0, (double)va), ef = pow(10.0, (double)vf);
                        out = normal ? (float)(ea - ef) : 0.0f;
                    }
                    v[e1 * nk + c] = out;
                }
            }
            if (a.infl && lane == 0) a.infl[(size_t)f * a.plane + (size_t)jt * a.mni + i] = inflation;
            __syncwarp();
        }
    }
    __syncthreads();
    for (int idx = tid; idx < nf * m * nk; idx += UPD_NT) {
        int c = idx % nk, fe = idx / nk;
        if (c < ncell) {
            int f = fe / m, e = fe - f * m;
            a.fields[((size_t)f * m + e) * a.plane + (size_t)jt * a.mni + i0 + c] = tile[idx];
        }
    }
}

// EnOI background update, one thread per cell (update.c:706-745)
__global__ void k_update_bg(UpdArgs a)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int jt = blockIdx.y;
    if (i >= a.mni) return;
    const int m = a.m;
    const int jj = a.j1 / a.stride + jt / a.stride, stepj = jt % a.stride;
    const int ii = i / a.stride, stepi = i % a.stride;
    const int nl = a.numlevels[(size_t)(a.j1 + jt) * a.mni + i];
    const size_t mstride = (size_t)(m + 1) * a.plane;
    for (int f = 0; f < a.nfield; ++f) {
        float* v = a.fields + (size_t)f * mstride + (size_t)jt * a.mni + i;
        float* bg = v + (size_t)m * a.plane;
        const int level = a.levels[f];
        bool masked = (a.surfk == 0) ? (nl <= level) : (nl <= (a.issurfacevar ? 1 : a.surfk - level));
        if (masked || fabsf(*bg) > MAXOBSVAL_F) {
            *bg = 0.0f;
            continue;
        }
        int e;
        for (e = 0; e < m; ++e)
            if (fabsf(v[(size_t)e * a.plane]) > MAXOBSVAL_F) break;
        if (e < m) {
            *bg = 0.0f;
            continue;
        }
        float xmean = 0.0f;
        for (e = 0; e < m; ++e) xmean = __fadd_rn(xmean, v[(size_t)e * a.plane]);
        xmean = __fdiv_rn(xmean, (float)m);
        float b = *bg;
        for (e = 0; e < m; ++e) {
            float we = interp_x5(a.w, m, e, jj, stepj, ii, stepi, a);
            b = __fadd_rn(b, __fmul_rn(__fsub_rn(v[(size_t)e * a.plane], xmean), we));
        }
        *bg = b;
    }
}

// das_sethybridensemble, one thread per cell
__global__ void k_hybrid(int nmem, int nmem_d, double k_d, double k_s, long long nij, float* __restrict__ v)
{
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nij) return;
    double mean = 0.0;
    for (int e = 0; e < nmem_d; ++e) mean = __dadd_rn(mean, (double)v[(size_t)e * nij + i]);
    mean = __ddiv_rn(mean, (double)nmem_d);
    for (int e = 0; e < nmem_d; ++e) {
        float* x = &v[(size_t)e * nij + i];
        *x = (float)__dadd_rn(__dmul_rn(__dsub_rn((double)*x, mean), k_d), mean);
    }
    for (int e = nmem_d; e < nmem; ++e) {
        float* x = &v[(size_t)e * nij + i];
        *x = (float)__dadd_rn(__dmul_rn((double)*x, k_s), mean);
    }
}

enkfg_status run_hybrid(enkfg_ctx* ctx, int nmem, int nmem_d, double gamma, int nij, float* d_v, cudaStream_t st)
{
    double k_d = (nmem_d > 1) ? sqrt((double)(nmem - 1) / (double)(nmem_d - 1)) : 0.0;
    double k_s = sqrt(gamma * (double)(nmem - 1) / (double)(nmem - nmem_d - 1));
    k_hybrid<<<div_up(nij, 256), 256, 0, st>>>(nmem, nmem_d, k_d, k_s, nij, d_v);
    CKL();
    return ENKFG_OK;
}

enkfg_status run_update(enkfg_ctx* ctx, const enkfg_update_params* p, const int* d_numlevels, int nfield,
                        const int* levels, float* d_fields, float* d_infl, cudaStream_t st)
{
    if (!ctx->t_valid) {
        set_err(ctx, "no transforms in the context");
        return ENKFG_ESTATE;
    }
    if (p->nmem != ctx->t_nmem || (p->mode != ENKFG_MODE_ENOI && p->nmem_dynamic != ctx->t_ndyn)) {
        set_err(ctx, "ensemble size %d/%d differs from the transforms' %d/%d", p->nmem, p->nmem_dynamic,
                ctx->t_nmem, ctx->t_ndyn);
        return ENKFG_EINVAL;
    }
    if (p->mode != ENKFG_MODE_ENOI && ctx->t_mode == ENKFG_MODE_ENOI) {
        set_err(ctx, "the resident transforms hold no T (EnOI)");
        return ENKFG_ESTATE;
    }
    if (p->precision != ENKFG_PREC_FP64 && p->precision != ENKFG_PREC_MIXED) {
        set_err(ctx, "bad precision %d", p->precision);
        return ENKFG_EINVAL;
    }
    int j1 = p->j1, j2 = p->j2 < 0 ? ctx->mnj - 1 : p->j2;
    if (j1 < 0 || j2 >= ctx->mnj || j1 > j2 || j1 % ctx->stride != 0) {
        set_err(ctx, "bad field tile rows j1=%d j2=%d (stride %d)", j1, j2, ctx->stride);
        return ENKFG_EINVAL;
    }
    UpdArgs a;
    memset(&a, 0, sizeof(a));
    a.mode = p->mode;
    a.m = p->nmem;
    a.md = p->mode == ENKFG_MODE_ENOI ? p->nmem : p->nmem_dynamic;
    a.mni = ctx->mni;
    a.ni = ctx->ni;
    a.nj = ctx->nj;
    a.stride = ctx->stride;
    a.periodic_i = ctx->periodic_i;
    a.j1 = j1;
    a.jsize = j2 - j1 + 1;
    a.surfk = p->surfk;
    a.issurfacevar = p->issurfacevar;
    a.output_increment = p->output_increment;
    a.applylog = p->applylog;
    a.inflation0 = p->inflation;
    a.inf_ratio = p->inf_ratio;
    a.numlevels = d_numlevels;
    a.T = ctx->d_T;
    a.w = ctx->d_w;
    a.plane = (size_t)a.jsize * a.mni;
    int* d_levels = ctx->d_qhead + 64;       // up to 448 levels per launch group
    cudaEventRecord(ctx->ev[4], st);
    if (p->mode == ENKFG_MODE_ENOI) {
        for (int f0 = 0; f0 < nfield; f0 += 448) {
            int nf = nfield - f0 < 448 ? nfield - f0 : 448;
            CK(cudaMemcpyAsync(d_levels, levels + f0, nf * sizeof(int), cudaMemcpyHostToDevice, st));
            a.levels = d_levels;
            a.nfield = nf;
            a.fields = d_fields + (size_t)f0 * (a.m + 1) * a.plane;
            dim3 g(div_up(a.mni, 128), a.jsize);
            k_update_bg<<<g, 128, 0, st>>>(a);
            CKL();
            CK(cudaStreamSynchronize(st));
        }
        cudaEventRecord(ctx->ev[5], st);
        return ENKFG_OK;
    }
    if (a.m > 32 * MAXE_PER_LANE) {
        set_err(ctx, "nmem = %d too large for the update kernel", a.m);
        return ENKFG_EUNSUPPORTED;
    }
    // choose cells per CTA and field-layers per launch to fit shared memory
    const size_t smem_cap = 200 * 1024;
    size_t fixed = ((size_t)a.md * (a.m + 1) + ((a.m + 3) & ~3) + (UPD_NT / 32) * a.m) * sizeof(float);
    int nk = 32;
    int fg = nfield;
    while (nk > 4 && fixed + (size_t)fg * a.m * nk * 4 > smem_cap) nk >>= 1;
    while (fg > 1 && fixed + (size_t)fg * a.m * nk * 4 > smem_cap) fg = (fg + 1) / 2;
    if (fg > 448) fg = 448;
    size_t smem = fixed + (size_t)fg * a.m * nk * 4;
    if (smem > 227 * 1024) {
        set_err(ctx, "update tile does not fit in shared memory (nmem %d)", a.m);
        return ENKFG_EUNSUPPORTED;
    }
    CK(cudaFuncSetAttribute(k_update_fields, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    a.nk = nk;
    for (int f0 = 0; f0 < nfield; f0 += fg) {
        int nf = nfield - f0 < fg ? nfield - f0 : fg;
        CK(cudaMemcpyAsync(d_levels, levels + f0, nf * sizeof(int), cudaMemcpyHostToDevice, st));
        a.levels = d_levels;
        a.nfield = nf;
        a.fields = d_fields + (size_t)f0 * a.m * a.plane;
        a.infl = d_infl ? d_infl + (size_t)f0 * a.plane : nullptr;
        dim3 g(div_up(a.mni, nk), a.jsize);
        k_update_fields<<<g, UPD_NT, smem, st>>>(a);
        CKL();
        if (f0 + fg < nfield) CK(cudaStreamSynchronize(st));
    }
    cudaEventRecord(ctx->ev[5], st);
    return ENKFG_OK;
}
