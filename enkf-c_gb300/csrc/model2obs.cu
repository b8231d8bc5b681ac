// model2obs.cu -- the forward operator on the device: HE built from the
// ensemble fields (das_getHE, calc/ensobs.c:46-490; H_surf_standard and
// H_subsurf_standard, calc/model2obs.c:127-348; interpolate2d_structured and
// interpolate3d_structured, common/utils.c:1140-1366).
//
// One thread per (observation, block of members): the corner indices and
// weights of the observation are formed once and applied to each member's
// field.  The arithmetic is the reference's, operation by operation in
// double with round-to-nearest intrinsics (no contraction), so HE is
// bit-identical to the reference's on the same positions and fields.  FP64
// bounds the kernel on this part: conversions run on the integer pipe, and
// the division by the kept weights' sum becomes a product by its reciprocal
// wherever the float rounding of the quotient is decided with a margin.
#include "internal.cuh"
#include <math.h>

namespace {

constexpr int MAP_NT = 256;
constexpr int MAP_MG = 16;                 // members per thread
constexpr short STATUS_BADFC = 10;         // common/global.h:62
constexpr double EPS_EDGE = 1.0e-7;        // common/utils.c:51

struct MapArgs {
    const double* fi;
    const double* fj;
    const float* fk;
    const short* type;
    const short* status;
    const int* ids;             // nullptr: every obs of type otype with status 0
    int nids;
    int nobs;
    int otype;
    int ni, nj, nk, ktop, periodic_i;
    const int* numlevels;       // [nj][ni]
    const float* offset;
    int offset_kind;            // 0 none, 1 [nk], 2 [nj][ni], 3 [nk][nj][ni]
    const float* fields;        // [nfield][nk][nj][ni]
    long long fstride;          // floats per member
    int nfield;
    float* dst;                 // row of the first member; rows nobs apart
    long long dstride;
    int skip_bad;
    unsigned long long* flag;   // [0] bad forecast key, [1] position off the grid, [3] id out of range
};

// corner indices and weights, the reference's edge rules (utils.c:1158-1184)
__device__ __forceinline__ bool corners(double fi, double fj, int ni, int nj, int periodic_i, int i[2], int j[2],
                                        double wi[2], double wj[2])
{
    const double fli = floor(fi), cli = ceil(fi), flj = floor(fj), clj = ceil(fj);
    i[0] = (int)fli;
    wi[0] = __dsub_rn(cli, fi);
    i[1] = (int)cli;
    wi[1] = __dsub_rn(fi, fli);
    j[0] = (int)flj;
    wj[0] = __dsub_rn(clj, fj);
    j[1] = (int)clj;
    wj[1] = __dsub_rn(fj, flj);
    if (i[0] == i[1]) wi[0] = 1.0;
    if (j[0] == j[1]) wj[0] = 1.0;
    if (i[0] == -1) i[0] = periodic_i ? ni - 1 : i[1];
    if (i[1] == ni) i[1] = periodic_i ? 0 : i[0];
    if (j[0] == -1) j[0] = j[1];
    if (j[1] == nj) j[1] = j[0];
    return i[0] >= 0 && i[0] < ni && i[1] >= 0 && i[1] < ni && j[0] >= 0 && j[0] < nj && j[1] >= 0 && j[1] < nj;
}

// float -> double (exact) on the integer pipe for normal floats; FP64 is the
// scarce unit on this part, and the conversion instruction runs on it
__device__ __forceinline__ double widen(float v)
{
    const unsigned u = __float_as_uint(v);
    const unsigned ex = (u >> 23) & 0xffu;
    if (ex == 0u || ex == 0xffu) return (double)v;
    return __longlong_as_double((long long)(((unsigned long long)(u & 0x80000000u) << 32) |
                                            ((unsigned long long)(ex + 896u) << 52) |
                                            ((unsigned long long)(u & 0x7fffffu) << 29)));
}

// Round-to-nearest float of a double q on the integer pipe, when that
// rounding is decided with a margin: q a normal double of moderate exponent
// whose low 29 mantissa bits are more than 8 double ulps away from the float
// tie point.  Then any double within 2.5 ulps of q (in particular the
// correctly rounded quotient the reference forms, when q approximates it to
// within 2 ulps) has the same float rounding.  Returns false otherwise.
__device__ __forceinline__ bool narrow_decided(double q, float& r)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(q);
    const int ex = (int)((b >> 52) & 0x7ffu);
    if (ex < 1023 - 100 || ex > 1023 + 100) return false;          // also NaN / inf / 0
    const long long dt = (long long)(b & ((1ull << 29) - 1)) - (1ll << 28);
    if (dt >= -8 && dt <= 8) return false;
    unsigned f = ((unsigned)(b >> 63) << 31) | ((unsigned)(ex - 896) << 23) | (unsigned)((b >> 29) & 0x7fffffu);
    f += dt > 0 ? 1u : 0u;                                         // a carry moves into the exponent
    r = __uint_as_float(f);
    return true;
}

__device__ __forceinline__ float offset_at(const MapArgs& a, long long q, long long nij)
{
    switch (a.offset_kind) {
    case 1: return a.offset[q / nij];
    case 2: return a.offset[q % nij];
    case 3: return a.offset[q];
    default: return 0.0f;
    }
}

template <bool THREE_D>
__global__ void __launch_bounds__(MAP_NT) k_map_obs(MapArgs a)
{
    const int k = blockIdx.x * MAP_NT + threadIdx.x;
    if (k >= a.nids) return;
    int o = k;
    if (a.ids) {
        o = a.ids[k];
        if ((unsigned)o >= (unsigned)a.nobs) {        // a caller's device list is checked here
            atomicMin(&a.flag[3], (unsigned long long)k);
            return;
        }
    } else if (a.type[o] != a.otype || a.status[o] != 0) {
        return;
    }
    const int e0 = blockIdx.y * MAP_MG;
    const int e1 = min(e0 + MAP_MG, a.nfield);

    double fi = a.fi[o], fj = a.fj[o];
    bool ok = fi > -1.0 && fj > -1.0;       // false for NaN as well
    const long long nij = (long long)a.ni * a.nj;
    int i[2], j[2], k2[2] = { 0, 0 }, ktp[2] = { 0, 0 };
    double wi[2], wj[2], wk[2] = { 1.0, 0.0 };
    if (ok) {
        if (THREE_D) {
            if (fi > (double)a.ni) fi = __dsub_rn((double)a.ni, EPS_EDGE);   // strict, utils.c:1265
        } else {
            if (fi >= (double)a.ni) fi = __dsub_rn((double)a.ni, EPS_EDGE);
        }
        if (fj >= (double)a.nj) fj = __dsub_rn((double)a.nj, EPS_EDGE);
        if (THREE_D) {
            double fk = (double)a.fk[o];
            if (fk != fk) {
                ok = false;
            } else {
                if (fk < 0.0) fk = 0.0;
                if (fk > (double)(a.nk - 1)) fk = (double)(a.nk - 1);
                const double flk = floor(fk), clk = ceil(fk);
                k2[0] = (int)flk;
                wk[0] = __dsub_rn(clk, fk);
                k2[1] = (int)clk;
                wk[1] = __dsub_rn(fk, flk);
                if (wk[0] == 0.0 && wk[1] == 0.0) wk[0] = 1.0;
                if (k2[0] == k2[1]) wk[0] = 1.0;
                ktp[0] = abs(a.ktop - k2[0]);
                ktp[1] = abs(a.ktop - k2[1]);
            }
        }
        if (ok) ok = corners(fi, fj, a.ni, a.nj, a.periodic_i, i, j, wi, wj);
    }
    if (!ok) {
        atomicMin(&a.flag[1], (unsigned long long)o);
        for (int e = e0; e < e1; ++e) a.dst[e * a.dstride + o] = __int_as_float(0x7fc00000);
        return;
    }

    // corner cells and weights, in the reference's order
    constexpr int NC = THREE_D ? 8 : 4;
    long long cell[NC];
    double ww[NC];
    bool wet[NC];
#pragma unroll
    for (int c = 0; c < NC; ++c) {
        const int a_ = c & 1, b_ = (c >> 1) & 1, kc = c >> 2;
        const long long q = (long long)j[b_] * a.ni + i[a_];
        const int nl = a.numlevels[q];
        if (THREE_D) {
            wet[c] = nl > ktp[kc];
            ww[c] = __dmul_rn(__dmul_rn(wj[b_], wi[a_]), wk[kc]);
            cell[c] = (long long)k2[kc] * nij + q;
        } else {
            wet[c] = nl != 0;
            ww[c] = __dmul_rn(wj[b_], wi[a_]);
            cell[c] = q;
        }
    }
    // the kept weights' sum is the same for every member; its reciprocal
    // turns the per-member division into a product, checked for a decided
    // float rounding (the exact division where it is not)
    double w = 0.0;
#pragma unroll
    for (int c = 0; c < NC; ++c)
        if (wet[c]) w = __dadd_rn(w, ww[c]);
    const bool wpos = w > 0.0;
    const double rw = wpos ? __drcp_rn(w) : 0.0;
#pragma unroll 2
    for (int e = e0; e < e1; ++e) {
        const float* f = a.fields + e * a.fstride;
        double sum = 0.0;
#pragma unroll
        for (int c = 0; c < NC; ++c) {
            if (!wet[c]) continue;
            float v = __ldg(f + cell[c]);
            if (a.offset_kind) v = __fsub_rn(v, offset_at(a, cell[c], nij));
            sum = __dadd_rn(sum, __dmul_rn(widen(v), ww[c]));
        }
        float r;
        if (!(wpos && narrow_decided(__dmul_rn(sum, rw), r))) r = __double2float_rn(__ddiv_rn(sum, w));
        if (!(fabsf(r) <= 999999.0f)) {                           // not finite, or |r| > MAXOBSVAL
            if (!a.skip_bad)
                atomicMin(&a.flag[0], ((unsigned long long)o << 32) | __float_as_uint(r));
            r = __int_as_float(0x7fc00000);
        }
        a.dst[e * a.dstride + o] = r;
    }
}

// end of das_getHE (ensobs.c:372-490): BADFC statuses, EnOI recentring or
// hybrid rescaling; one thread per observation, members looped in order
__global__ void __launch_bounds__(256) k_he_finish(float* S, const float* Hx, short* status, int nobs, int nmem,
                                                   int nmem_d, int mode, int skip_bad, double k_d, double k_s,
                                                   unsigned long long* count)
{
    const int o = blockIdx.x * blockDim.x + threadIdx.x;
    bool badfc = false;
    if (o < nobs) {
        if (skip_bad) {
            bool nan = false;
            for (int e = 0; e < nmem; ++e) nan |= isnan(S[(size_t)e * nobs + o]);
            if (mode == ENKFG_MODE_ENOI) nan |= isnan(Hx[o]);
            if (nan) status[o] = STATUS_BADFC;
        }
        badfc = status[o] == STATUS_BADFC;
        if (mode == ENKFG_MODE_ENOI) {
            float mean = 0.0f;
            for (int e = 0; e < nmem; ++e) mean = __fadd_rn(mean, S[(size_t)e * nobs + o]);
            mean = __fdiv_rn(mean, (float)nmem);
            const float shift = __fsub_rn(Hx[o], mean);
            for (int e = 0; e < nmem; ++e) {
                float* p = S + (size_t)e * nobs + o;
                *p = __fadd_rn(*p, shift);
            }
        } else if (mode == ENKFG_MODE_HYBRID) {
            double md = 0.0, ms = 0.0;
            for (int e = 0; e < nmem_d; ++e) md = __dadd_rn(md, (double)S[(size_t)e * nobs + o]);
            md = __ddiv_rn(md, (double)nmem_d);
            for (int e = 0; e < nmem_d; ++e) {
                float* p = S + (size_t)e * nobs + o;
                *p = __double2float_rn(__dadd_rn(__dmul_rn(__dsub_rn((double)*p, md), k_d), md));
            }
            for (int e = nmem_d; e < nmem; ++e) ms = __dadd_rn(ms, (double)S[(size_t)e * nobs + o]);
            ms = __ddiv_rn(ms, (double)(nmem - nmem_d));
            for (int e = nmem_d; e < nmem; ++e) {
                float* p = S + (size_t)e * nobs + o;
                *p = __double2float_rn(__dadd_rn(__dmul_rn(__dsub_rn((double)*p, ms), k_s), md));
            }
        }
    }
    const unsigned b = __ballot_sync(0xffffffffu, badfc);
    if ((threadIdx.x & 31) == 0 && b) atomicAdd(count, (unsigned long long)__popc(b));
}

}  // namespace

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------

static enkfg_status check_hop(enkfg_ctx* ctx, const enkfg_hop_params* p, int obstype, int nids, int mem0, int nfield)
{
    NEED(p, ENKFG_EINVAL, "no forward-operator parameters");
    NEED(ctx->he_nmem > 0, ENKFG_ESTATE, "enkfg_begin_HE must come first");
    NEED(ctx->pos_set, ENKFG_ESTATE, "enkfg_set_obs_positions must come first");
    NEED(obstype >= 0 && obstype < ctx->ntypes, ENKFG_EINVAL, "observation type %d out of range", obstype);
    NEED(p->ni >= 1 && p->nj >= 1 && p->nk >= 1, ENKFG_EINVAL, "bad grid %d x %d x %d", p->ni, p->nj, p->nk);
    NEED(p->three_d || p->nk == 1, ENKFG_EINVAL, "a 2-D forward operator takes one layer (nk = 1)");
    NEED(!p->three_d || ctx->pos_3d, ENKFG_ESTATE, "a 3-D forward operator needs fk (enkfg_set_obs_positions)");
    NEED(!p->three_d || p->ksurf == 0 || p->ksurf == p->nk - 1, ENKFG_EINVAL, "ksurf must be 0 or nk - 1");
    NEED(p->offset_kind >= 0 && p->offset_kind <= 3 && (p->three_d || p->offset_kind == 0 || p->offset_kind == 2),
         ENKFG_EINVAL, "offset_kind %d does not fit a %s field", p->offset_kind, p->three_d ? "3-D" : "2-D");
    NEED(nids >= 0 && nids <= ctx->nobs, ENKFG_EINVAL, "bad observation count %d", nids);
    NEED(nfield >= 1, ENKFG_EINVAL, "bad member count %d", nfield);
    if (mem0 == -1)
        NEED(ctx->he_bg && nfield == 1, ENKFG_EINVAL, "mem0 = -1 is the background row (begin_HE with_background, one field)");
    else
        NEED(mem0 >= 0 && mem0 + nfield <= ctx->he_nmem, ENKFG_EINVAL, "members %d..%d outside 0..%d", mem0,
             mem0 + nfield - 1, ctx->he_nmem - 1);
    return ENKFG_OK;
}

static enkfg_status launch_map(enkfg_ctx* ctx, const enkfg_hop_params* p, int obstype, int nids, const int* d_ids,
                               int mem0, int nfield, const float* d_fields, const int* d_numlevels,
                               const float* d_offset, cudaStream_t st)
{
    MapArgs a;
    a.fi = ctx->d_fi;
    a.fj = ctx->d_fj;
    a.fk = ctx->d_fk;
    a.type = ctx->d_type;
    a.status = ctx->d_status;
    a.ids = d_ids;
    a.nids = d_ids ? nids : ctx->nobs;
    a.nobs = ctx->nobs;
    a.otype = obstype;
    a.ni = p->ni;
    a.nj = p->nj;
    a.nk = p->three_d ? p->nk : 1;
    a.ktop = p->three_d ? p->ksurf : 0;
    a.periodic_i = p->periodic_i ? 1 : 0;
    a.numlevels = d_numlevels;
    a.offset = d_offset;
    a.offset_kind = d_offset ? p->offset_kind : 0;
    a.fields = d_fields;
    a.fstride = (long long)a.nk * p->nj * p->ni;
    a.nfield = nfield;
    a.dst = mem0 < 0 ? ctx->d_Hx : ctx->d_S + (size_t)mem0 * ctx->nobs;
    a.dstride = ctx->nobs;
    a.skip_bad = p->skip_bad ? 1 : 0;
    a.flag = ctx->d_hflag;
    if (a.nids == 0) return ENKFG_OK;
    dim3 grid(div_up(a.nids, MAP_NT), div_up(nfield, MAP_MG));
    if (p->three_d)
        k_map_obs<true><<<grid, MAP_NT, 0, st>>>(a);
    else
        k_map_obs<false><<<grid, MAP_NT, 0, st>>>(a);
    CKL();
    return ENKFG_OK;
}

// reads the error flags (synchronises `st`)
static enkfg_status check_flags(enkfg_ctx* ctx, cudaStream_t st, int skip_bad)
{
    unsigned long long f[4];
    CK(cudaMemcpyAsync(f, ctx->d_hflag, sizeof(f), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    NEED(f[3] == ~0ull, ENKFG_EINVAL, "ids[%llu]: observation id out of range", f[3]);
    NEED(f[1] == ~0ull, ENKFG_EINVAL, "obs # %llu: position off the model grid", f[1]);
    if (!skip_bad && f[0] != ~0ull) {
        const unsigned bits = (unsigned)(f[0] & 0xffffffffu);
        float v;
        memcpy(&v, &bits, sizeof(v));
        set_err(ctx, "obs # %llu: forecast = %.3g; not finite or |value| > 999999 (skip_bad turns it into a bad "
                "forecast observation)", f[0] >> 32, (double)v);
        return ENKFG_ENUMERIC;
    }
    return ENKFG_OK;
}

extern "C" {

ENKFG_API enkfg_status enkfg_set_obs_positions(enkfg_ctx* ctx, const double* fi, const double* fj, const float* fk)
{
    if (!ctx) return ENKFG_EINVAL;
    NEED(ctx->obs_set, ENKFG_ESTATE, "enkfg_set_obs must come first");
    NEED((fi && fj) || ctx->nobs == 0, ENKFG_EINVAL, "fi and fj are required");
    SETDEV();
    const size_t n = ctx->nobs > 0 ? ctx->nobs : 1;
    void** bufs[] = { (void**)&ctx->d_fi, (void**)&ctx->d_fj, (void**)&ctx->d_fk };
    for (void** b : bufs) {
        if (*b) cudaFree(*b);
        *b = nullptr;
    }
    CK(cudaMalloc(&ctx->d_fi, n * sizeof(double)));
    CK(cudaMalloc(&ctx->d_fj, n * sizeof(double)));
    if (fk) CK(cudaMalloc(&ctx->d_fk, n * sizeof(float)));
    if (ctx->nobs > 0) {
        CK(cudaMemcpyAsync(ctx->d_fi, fi, ctx->nobs * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
        CK(cudaMemcpyAsync(ctx->d_fj, fj, ctx->nobs * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
        if (fk) CK(cudaMemcpyAsync(ctx->d_fk, fk, ctx->nobs * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
    }
    CK(cudaStreamSynchronize(ctx->stream));
    ctx->pos_set = true;
    ctx->pos_3d = fk != nullptr;
    return ENKFG_OK;
}

ENKFG_API enkfg_status enkfg_begin_HE(enkfg_ctx* ctx, int nmem, int nmem_dynamic, int with_background)
{
    if (!ctx) return ENKFG_EINVAL;
    NEED(ctx->obs_set, ENKFG_ESTATE, "enkfg_set_obs must come first");
    NEED(nmem >= 2 && nmem <= 144 && nmem_dynamic >= 1 && nmem_dynamic <= nmem, ENKFG_EINVAL,
         "bad ensemble size %d/%d", nmem, nmem_dynamic);
    SETDEV();
    enkfg_status s = alloc_S(ctx, nmem, nmem_dynamic);
    if (s) return s;
    const size_t n = ctx->nobs > 0 ? ctx->nobs : 1;
    if (with_background) {
        if (ctx->d_Hx) cudaFree(ctx->d_Hx);
        ctx->d_Hx = nullptr;
        CK(cudaMalloc(&ctx->d_Hx, n * sizeof(float)));
        CK(cudaMemsetAsync(ctx->d_Hx, 0xff, n * sizeof(float), ctx->stream));
    }
    if (!ctx->d_hflag) CK(cudaMalloc(&ctx->d_hflag, 4 * sizeof(unsigned long long)));
    // NaN everywhere (all bits set is a NaN), as the reference's set-up
    CK(cudaMemsetAsync(ctx->d_S, 0xff, (size_t)nmem * n * sizeof(float), ctx->stream));
    CK(cudaMemsetAsync(ctx->d_hflag, 0xff, 4 * sizeof(unsigned long long), ctx->stream));
    CK(cudaMemsetAsync(ctx->d_hflag + 2, 0, sizeof(unsigned long long), ctx->stream));
    ctx->he_nmem = nmem;
    ctx->he_nmem_dyn = nmem_dynamic;
    ctx->he_bg = with_background != 0;
    ctx->s_mode = 0;
    ctx->gather_valid = false;
    return ENKFG_OK;
}

ENKFG_API enkfg_status enkfg_map_obs(enkfg_ctx* ctx, const enkfg_hop_params* p, int obstype, int nids, const int* ids,
                                     int mem0, int nfield, const float* fields, const int* numlevels,
                                     const float* offset)
{
    if (!ctx) return ENKFG_EINVAL;
    enkfg_status s = check_hop(ctx, p, obstype, nids, mem0, nfield);
    if (s) return s;
    NEED(fields && numlevels, ENKFG_EINVAL, "fields and numlevels are required");
    NEED(ids || nids == 0 || nids == ctx->nobs, ENKFG_EINVAL, "ids NULL selects by type (pass nids = nobs or 0)");
    if (ids)
        for (int k = 0; k < nids; ++k)
            NEED(ids[k] >= 0 && ids[k] < ctx->nobs, ENKFG_EINVAL, "ids[%d] = %d out of range", k, ids[k]);
    SETDEV();
    const size_t nk = p->three_d ? p->nk : 1, nij = (size_t)p->ni * p->nj;
    const size_t nv = (size_t)nfield * nk * nij;
    const size_t noff = offset && p->offset_kind ? (p->offset_kind == 1 ? nk : p->offset_kind == 2 ? nij : nk * nij) : 0;
    if ((s = ensure(ctx, &ctx->d_hsrc, &ctx->hsrc_cap, nv))) return s;
    if ((s = ensure(ctx, &ctx->d_hlev, &ctx->hlev_cap, nij))) return s;
    if (noff && (s = ensure(ctx, &ctx->d_hoff, &ctx->hoff_cap, noff))) return s;
    if (ids && (s = ensure(ctx, &ctx->d_hids, &ctx->hids_cap, (size_t)nids))) return s;
    cudaStream_t st = ctx->stream;
    CK(cudaMemcpyAsync(ctx->d_hsrc, fields, nv * sizeof(float), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(ctx->d_hlev, numlevels, nij * sizeof(int), cudaMemcpyHostToDevice, st));
    if (noff) CK(cudaMemcpyAsync(ctx->d_hoff, offset, noff * sizeof(float), cudaMemcpyHostToDevice, st));
    if (ids && nids) CK(cudaMemcpyAsync(ctx->d_hids, ids, nids * sizeof(int), cudaMemcpyHostToDevice, st));
    if ((s = launch_map(ctx, p, obstype, nids, ids ? ctx->d_hids : nullptr, mem0, nfield, ctx->d_hsrc, ctx->d_hlev,
                        noff ? ctx->d_hoff : nullptr, st)))
        return s;
    return check_flags(ctx, st, p->skip_bad);
}

ENKFG_API enkfg_status enkfg_map_obs_dev(enkfg_ctx* ctx, const enkfg_hop_params* p, int obstype, int nids,
                                         const int* ids_dev, int mem0, int nfield, const float* fields_dev,
                                         const int* numlevels_dev, const float* offset_dev, void* stream)
{
    if (!ctx) return ENKFG_EINVAL;
    enkfg_status s = check_hop(ctx, p, obstype, nids, mem0, nfield);
    if (s) return s;
    NEED(fields_dev && numlevels_dev, ENKFG_EINVAL, "fields and numlevels are required");
    NEED(ids_dev || nids == 0 || nids == ctx->nobs, ENKFG_EINVAL, "ids NULL selects by type (pass nids = nobs or 0)");
    SETDEV();
    return launch_map(ctx, p, obstype, nids, ids_dev, mem0, nfield, fields_dev, numlevels_dev, offset_dev,
                      stream ? (cudaStream_t)stream : ctx->stream);
}

ENKFG_API enkfg_status enkfg_finish_HE(enkfg_ctx* ctx, int mode, double gamma, int skip_bad, int* nbad, short* status)
{
    if (!ctx) return ENKFG_EINVAL;
    NEED(ctx->he_nmem > 0, ENKFG_ESTATE, "enkfg_begin_HE must come first");
    NEED(mode == ENKFG_MODE_ENKF || mode == ENKFG_MODE_ENOI || mode == ENKFG_MODE_HYBRID, ENKFG_EINVAL,
         "bad mode %d", mode);
    NEED(mode != ENKFG_MODE_ENOI || ctx->he_bg, ENKFG_ESTATE, "EnOI needs the background row (begin_HE)");
    const int m = ctx->he_nmem, md = ctx->he_nmem_dyn;
    NEED(mode != ENKFG_MODE_HYBRID || (md < m && m - md >= 2), ENKFG_EINVAL,
         "a hybrid ensemble needs at least two static members (%d of %d dynamic)", md, m);
    SETDEV();
    cudaStream_t st = ctx->stream;
    enkfg_status s = check_flags(ctx, st, skip_bad);
    if (s) return s;
    const double k_d = md > 1 ? sqrt((double)(m - 1) / (double)(md - 1)) : 0.0;
    const double k_s = mode == ENKFG_MODE_HYBRID ? sqrt(gamma * (double)(m - 1) / (double)(m - md - 1)) : 0.0;
    if (ctx->nobs > 0) {
        k_he_finish<<<div_up(ctx->nobs, 256), 256, 0, st>>>(ctx->d_S, ctx->d_Hx, ctx->d_status, ctx->nobs, m, md,
                                                            mode, skip_bad ? 1 : 0, k_d, k_s, ctx->d_hflag + 2);
        CKL();
    }
    unsigned long long cnt = 0;
    CK(cudaMemcpyAsync(&cnt, ctx->d_hflag + 2, sizeof(cnt), cudaMemcpyDeviceToHost, st));
    if (status && ctx->nobs > 0)
        CK(cudaMemcpyAsync(status, ctx->d_status, ctx->nobs * sizeof(short), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (nbad) *nbad = (int)cnt;
    // statuses may have changed: the index holds only status-0 observations
    if (skip_bad && cnt > 0) ctx->index_valid = false;
    ctx->he_nmem = 0;
    ctx->s_mode = 1;
    ctx->gather_valid = false;
    return ENKFG_OK;
}

}  // extern "C"
