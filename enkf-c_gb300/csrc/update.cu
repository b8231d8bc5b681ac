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
    int nk;                     // cells per CTA (tile cell stride)
    int G;                      // strided columns per CTA (version 2 kernel)
    int fc;                     // field-layers per warp task (version 2 kernel)
    float inv_kd;               // 1 / k_d (hybrid rescaling, FP32 variant)
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
#define UPD_FC 8          // field-layers per register block

// double or double-float (FP32 pair) accumulation of the per-row sums the
// reference keeps in double (update.c:381-383, 405-410, 437-441)
template <bool F64>
struct Acc;
template <>
struct Acc<true> {
    double v;
    __device__ __forceinline__ Acc() : v(0.0) {}
    __device__ __forceinline__ void add(float x) { v += (double)x; }
    __device__ __forceinline__ void add_prod(float a, float b) { v += (double)__fmul_rn(a, b); }
    __device__ __forceinline__ void reduce()
    {
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    }
    __device__ __forceinline__ double value() const { return v; }
};
template <>
struct Acc<false> {
    float hi, lo;
    __device__ __forceinline__ Acc() : hi(0.0f), lo(0.0f) {}
    __device__ __forceinline__ void add(float x)
    {
        float s = hi + x, bp = s - hi;
        lo += (hi - (s - bp)) + (x - bp);
        hi = s;
    }
    __device__ __forceinline__ void add_prod(float a, float b) { add(__fmul_rn(a, b)); }
    __device__ __forceinline__ void reduce()
    {
        for (int o = 16; o > 0; o >>= 1) {
            float oh = __shfl_xor_sync(0xffffffffu, hi, o), ol = __shfl_xor_sync(0xffffffffu, lo, o);
            add(oh);
            lo += ol;
        }
    }
    __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
};

// The ensemble mean and the updated mean: double (F64, the reference's
// arithmetic) or a double-float hi + lo (FP32 pipe only; GB300 issues FP64 at
// 1/64 of the FP32 rate, and the conversions float <-> double run on the
// FP64 pipe as well).
template <bool F64>
struct Mean;
template <>
struct Mean<true> {
    double v;
    __device__ __forceinline__ void set(const Acc<true>& s, int n) { v = s.value() / (double)n; }
    __device__ __forceinline__ void zero() { v = 0.0; }
    // (float)(x - mean)
    __device__ __forceinline__ float sub(float x) const { return (float)((double)x - v); }
    // (float)(x + mean)
    __device__ __forceinline__ float add(float x) const { return (float)((double)x + v); }
    // mean + s (the updated mean, update.c:405-410)
    __device__ __forceinline__ Mean plus(const Acc<true>& s) const { Mean r; r.v = s.value() + v; return r; }
};
template <>
struct Mean<false> {
    float h, l;
    __device__ __forceinline__ void set(const Acc<false>& s, int n)
    {
        const float fn = (float)n;
        h = __fdiv_rn(s.hi, fn);
        l = __fdiv_rn(fmaf(-h, fn, s.hi) + s.lo, fn);
    }
    __device__ __forceinline__ void zero() { h = l = 0.0f; }
    __device__ __forceinline__ float sub(float x) const { return __fsub_rn(__fsub_rn(x, h), l); }
    __device__ __forceinline__ float add(float x) const { return __fadd_rn(__fadd_rn(x, h), l); }
    __device__ __forceinline__ Mean plus(const Acc<false>& s) const
    {
        Mean r;
        const float sm = s.hi + h, bp = sm - s.hi;
        r.l = ((s.hi - (sm - bp)) + (h - bp)) + (s.lo + l);
        r.h = sm;
        return r;
    }
};

// das_updatefields, version 2.  A CTA owns one model row j and G strided
// columns (cells i in [ii0*stride, (ii0+G)*stride)).  It builds, once, the
// j-interpolated transforms Tjj/wjj of the G strided columns plus the i-
// neighbour of the last one (the reference's Tjj, update.c:224-241), stages
// the [nfield][nmem][cells] field block, and then every warp takes one cell:
// lanes own output members, the i-interpolated X5 element (update.c:255-265,
// same float operations) is formed in registers and applied to UPD_FC
// field-layers at a time, and the per-row statistics use warp shuffles.
template <bool F64>
__global__ void __launch_bounds__(UPD_NT) k_update_v2(UpdArgs a)
{
    extern __shared__ __align__(16) float usm[];
    const int m = a.m, md = a.md, G = a.G, st = a.stride, nf = a.nfield;
    const int TLD = m + 1, M4 = (m + 3) & ~3;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int jt = blockIdx.y, jg = a.j1 + jt;
    const int jj = a.j1 / st + jt / st, stepj = jt % st;
    const int jj2 = (jj < a.nj - 1) ? jj + 1 : jj;
    const int ii0 = blockIdx.x * G;
    const int gv = min(G, a.ni - ii0);                       // strided columns of this CTA
    const int i0 = ii0 * st;
    const int ncell = min(gv * st, a.mni - i0);
    const int CP = a.nk;                                     // cell stride of the tile
    // carve (every region starts on a 16-byte boundary: Abuf is read as float4)
    float* Tjj = usm;                                                    // [(G+1)][md][TLD]
    float* Wjj = Tjj + (((size_t)(G + 1) * md * TLD + 3) & ~(size_t)3); // [(G+1)][M4]
    float* tile = Wjj + (size_t)(G + 1) * M4;                            // [nf][m][CP]
    float* Abuf = tile + (((size_t)nf * m * CP + 3) & ~(size_t)3);       // [8 warps][fcap][M4]
    const int fcap = a.fc;                                               // rows per task (<= UPD_FC)

    // 1. Tjj / wjj for slots 0..gv (slot gv = i-neighbour of the last column)
    {
        const int last = ii0 + gv - 1;
        const int nb = (last < a.ni - 1) ? last + 1 : (a.periodic_i ? (last + 1) % a.ni : last);
        const float w2 = __fdiv_rn((float)stepj, (float)st), w1 = __fsub_rn(1.0f, w2);
        const bool jint = (st > 1 && stepj > 0);
        const int ntot = (gv + 1) * md * m;
        for (int idx = tid; idx < ntot; idx += UPD_NT) {
            int k = idx / (md * m), e = idx - k * (md * m);
            int col = (k < gv) ? ii0 + k : nb;
            float v = __ldg(&a.T[((size_t)jj * a.ni + col) * md * m + e]);
            if (jint) {
                float b = __ldg(&a.T[((size_t)jj2 * a.ni + col) * md * m + e]);
                v = __fadd_rn(__fmul_rn(v, w1), __fmul_rn(b, w2));
            }
            int e1 = e / m, e2 = e - e1 * m;
            Tjj[((size_t)k * md + e1) * TLD + e2] = v;
        }
        for (int idx = tid; idx < (gv + 1) * m; idx += UPD_NT) {
            int k = idx / m, e = idx - k * m;
            int col = (k < gv) ? ii0 + k : nb;
            float v = __ldg(&a.w[((size_t)jj * a.ni + col) * m + e]);
            if (jint) {
                float b = __ldg(&a.w[((size_t)jj2 * a.ni + col) * m + e]);
                v = __fadd_rn(__fmul_rn(v, w1), __fmul_rn(b, w2));
            }
            Wjj[k * M4 + e] = v;
        }
    }
    // 2. stage the field block (NK consecutive floats per member row)
    for (int idx = tid; idx < nf * m * CP; idx += UPD_NT) {
        int c = idx % CP, fe = idx / CP;
        if (c < ncell) {
            int f = fe / m, e = fe - f * m;
            tile[idx] = a.fields[((size_t)f * m + e) * a.plane + (size_t)jt * a.mni + i0 + c];
        }
    }
    __syncthreads();

    float* Aw = Abuf + (size_t)wid * fcap * M4;
    const int EPL = (md + 31) >> 5;                          // output members per lane
    // tasks = (cell, block of fcap field-layers), spread over the warps
    const int nchunk = (nf + fcap - 1) / fcap;
    for (int task = wid; task < ncell * nchunk; task += UPD_NT / 32) {
        const int c = task % ncell;
        const int f0 = (task / ncell) * fcap;
        const int i = i0 + c;
        const int slot = i / st - ii0, stepi = i % st;
        const bool iint = (st > 1 && stepi > 0);
        const float u2 = __fdiv_rn((float)stepi, (float)st), u1 = __fsub_rn(1.0f, u2);
        const float* Ta = Tjj + (size_t)slot * md * TLD;
        const float* Tb = Tjj + (size_t)(slot + 1) * md * TLD;
        const int nl = a.numlevels[(size_t)jg * a.mni + i];
        const size_t ioff = (size_t)jt * a.mni + i;
        {
            const int fc = min(fcap, nf - f0);
            unsigned active = 0;                              // rows to update
            Mean<F64> mean[UPD_FC];
            // per row: mask, missing values, mean, anomalies (update.c:296-392)
            for (int q = 0; q < fc; ++q) {
                const int f = f0 + q;
                float* v = tile + (size_t)f * m * CP;
                const int level = a.levels[f];
                mean[q].zero();
                bool masked = (a.surfk == 0) ? (nl <= level) : (nl <= (a.issurfacevar ? 0 : a.surfk - level));
                if (masked) {
                    for (int e = lane; e < m; e += 32) v[e * CP + c] = 0.0f;
                    if (a.infl && lane == 0) a.infl[(size_t)f * a.plane + ioff] = 0.0f;
                    continue;
                }
                int first = m;
                for (int e0 = 0; e0 < m && first == m; e0 += 32) {
                    int e = e0 + lane;
                    bool bad = false;
                    if (e < m) {
                        float x = v[e * CP + c];
                        bad = !isfinite(x) || fabsf(x) > MAXOBSVAL_F;
                    }
                    unsigned bal = __ballot_sync(0xffffffffu, bad);
                    if (bal) first = e0 + __ffs(bal) - 1;
                }
                if (a.infl && lane == 0) a.infl[(size_t)f * a.plane + ioff] = 0.0f;
                if (first < md) {
                    for (int e = lane; e < m; e += 32) v[e * CP + c] = 0.0f;
                    continue;
                } else if (first < m) {
                    for (int e = md + lane; e < m; e += 32) v[e * CP + c] = 0.0f;
                    if (md == 0) continue;
                }
                Acc<F64> sm;
                for (int e = lane; e < md; e += 32) sm.add(v[e * CP + c]);
                sm.reduce();
                mean[q].set(sm, md);
                for (int e = lane; e < M4; e += 32) Aw[q * M4 + e] = (e < m) ? mean[q].sub(v[e * CP + c]) : 0.0f;
                active |= 1u << q;
            }
            __syncwarp();
            if (active == 0) {
                __syncwarp();
                continue;
            }
            // A^a = A^f T on the active rows: acc[q][k] for member lane+32k
            float acc[UPD_FC][MAXE_PER_LANE];
#pragma unroll
            for (int q = 0; q < UPD_FC; ++q)
#pragma unroll
                for (int k = 0; k < MAXE_PER_LANE; ++k) acc[q][k] = 0.0f;
            for (int e2 = 0; e2 < m; e2 += 4) {
                float4 av[UPD_FC];
#pragma unroll
                for (int q = 0; q < UPD_FC; ++q)
                    av[q] = (q < fc) ? *reinterpret_cast<const float4*>(&Aw[q * M4 + e2]) : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
                for (int k = 0; k < MAXE_PER_LANE; ++k) {
                    if (k >= EPL) break;
                    const int e1 = lane + 32 * k;
                    if (e1 < md) {
                        float t4[4];
#pragma unroll
                        for (int u = 0; u < 4; ++u) {
                            const int e = e2 + u;
                            float t = 0.0f;
                            if (e < m) {
                                t = Ta[e1 * TLD + e];
                                if (iint) t = __fadd_rn(__fmul_rn(t, u1), __fmul_rn(Tb[e1 * TLD + e], u2));
                            }
                            t4[u] = t;
                        }
#pragma unroll
                        for (int q = 0; q < UPD_FC; ++q) {
                            acc[q][k] = fmaf(t4[0], av[q].x, acc[q][k]);
                            acc[q][k] = fmaf(t4[1], av[q].y, acc[q][k]);
                            acc[q][k] = fmaf(t4[2], av[q].z, acc[q][k]);
                            acc[q][k] = fmaf(t4[3], av[q].w, acc[q][k]);
                        }
                    }
                }
            }
            // interpolated w for the mean increment
            float wl[MAXE_PER_LANE];
#pragma unroll
            for (int k = 0; k < MAXE_PER_LANE; ++k) {
                const int e = lane + 32 * k;
                float t = 0.0f;
                if (e < m) {
                    t = Wjj[slot * M4 + e];
                    if (iint) t = __fadd_rn(__fmul_rn(t, u1), __fmul_rn(Wjj[(slot + 1) * M4 + e], u2));
                }
                wl[k] = t;
            }
            // per row: mean update, hybrid rescaling, inflation, output
#pragma unroll
            for (int q = 0; q < UPD_FC; ++q) {
                if (!((active >> q) & 1u)) continue;
                const int f = f0 + q;
                float* v = tile + (size_t)f * m * CP;
                float inflation = a.inflation0;
                Acc<F64> sa;
#pragma unroll
                for (int k = 0; k < MAXE_PER_LANE; ++k) {
                    const int e = lane + 32 * k;
                    if (e < m) sa.add_prod(Aw[q * M4 + e], wl[k]);
                }
                sa.reduce();
                const Mean<F64> v1_a = mean[q].plus(sa);
                float af[MAXE_PER_LANE], aa[MAXE_PER_LANE];
#pragma unroll
                for (int k = 0; k < MAXE_PER_LANE; ++k) {
                    const int e = lane + 32 * k;
                    af[k] = (e < m) ? Aw[q * M4 + e] : 0.0f;
                    aa[k] = acc[q][k];
                }
                if (a.mode == ENKFG_MODE_HYBRID) {
                    if constexpr (F64) {
                        const double k_d = (md > 1) ? sqrt((double)(m - 1) / (double)(md - 1)) : 1.0;
#pragma unroll
                        for (int k = 0; k < MAXE_PER_LANE; ++k)
                            if (lane + 32 * k < md) {
                                aa[k] = (float)((double)aa[k] / k_d);
                                af[k] = (float)((double)af[k] / k_d);
                            }
                    } else {
                        const float rk = a.inv_kd;
#pragma unroll
                        for (int k = 0; k < MAXE_PER_LANE; ++k)
                            if (lane + 32 * k < md) {
                                aa[k] = __fmul_rn(aa[k], rk);
                                af[k] = __fmul_rn(af[k], rk);
                            }
                    }
                }
                if (!isnan(a.inf_ratio)) {
                    Acc<F64> s2f, s2a;
#pragma unroll
                    for (int k = 0; k < MAXE_PER_LANE; ++k)
                        if (lane + 32 * k < md) {
                            s2f.add_prod(af[k], af[k]);
                            s2a.add_prod(aa[k], aa[k]);
                        }
                    s2f.reduce();
                    s2a.reduce();
                    if constexpr (F64) {
                        const double v2_f = s2f.value(), v2_a = s2a.value();
                        if (v2_a > 0.0) {
                            inflation = (float)(sqrt(v2_f / v2_a) * a.inf_ratio + 1.0 - a.inf_ratio);
                            if (inflation >= a.inflation0) inflation = a.inflation0;
                        }
                    } else {
                        const float v2_f = s2f.hi + s2f.lo, v2_a = s2a.hi + s2a.lo;
                        if (v2_a > 0.0f) {
                            const float r = (float)a.inf_ratio;
                            inflation = fmaf(sqrtf(__fdiv_rn(v2_f, v2_a)), r, 1.0f - r);
                            if (inflation >= a.inflation0) inflation = a.inflation0;
                        }
                    }
                }
                const bool inflate = __fsub_rn(inflation, 1.0f) > 1.0e-6f;
                if (!inflate) inflation = 1.0f;
#pragma unroll
                for (int k = 0; k < MAXE_PER_LANE; ++k) {
                    const int e1 = lane + 32 * k;
                    if (e1 < md) {
                        float va = inflate ? __fmul_rn(aa[k], inflation) : aa[k];
                        va = v1_a.add(va);
                        float vf = mean[q].add(af[k]);
                        float out;
                        if (!a.output_increment) out = va;
                        else if (!a.applylog) out = __fsub_rn(va, vf);
                        else {
                            float avf = fabsf(vf);
                            bool normal = (avf >= 1.17549435e-38f) && (avf <= 3.40282347e+38f);
                            double ea = pow(10.0, (double)va), ef = pow(10.0, (double)vf);
                            out = normal ? (float)(ea - ef) : 0.0f;
                        }
                        v[e1 * CP + c] = out;
                    }
                }
                if (a.infl && lane == 0) a.infl[(size_t)f * a.plane + ioff] = inflation;
            }
            __syncwarp();
        }
    }
    __syncthreads();
    for (int idx = tid; idx < nf * m * CP; idx += UPD_NT) {
        int c = idx % CP, fe = idx / CP;
        if (c < ncell) {
            int f = fe / m, e = fe - f * m;
            a.fields[((size_t)f * m + e) * a.plane + (size_t)jt * a.mni + i0 + c] = tile[idx];
        }
    }
}

// das_updatefields, version 3 (nmem > 64).  A CTA of 8 warps owns U3_NC = 8
// consecutive cells of one model row (warp w: cell i0 + w) and up to U3_FG
// field-layers.  The [nf][nmem][8] field block is staged with 32-byte row
// pieces; each warp forms its cell's mask, missing-value test, mean and
// anomalies (update.c:296-392).  The j-interpolated transforms of the
// strided columns the 8 cells touch (Tjj, update.c:224-241) are streamed
// through shared memory U3_KE members of the reduction at a time and shared
// by all cells and field-layers: lane l of a warp owns output members l,
// l + 32, ... (EPL of them), forms the i-interpolated X5 elements with the
// reference's float operations (update.c:255-265) once per chunk, and
// applies them to every field-layer's anomalies (register accumulators, 16-
// byte broadcast loads of the anomalies).  The epilogue is version 2's: mean
// update, hybrid rescaling, spread-capped inflation, increments, outputs back
// into the staged block, then 32-byte row pieces out.
#define U3_NC 8
#define U3_KE 16
#define U3_FG 10
#define U3_TLD (U3_KE + 4)      // padded chunk row: 16-byte loads of 8 lanes hit distinct banks

static inline size_t upd_v3_smem(int m, int md, int stride, int nf)
{
    const int M4 = (m + 3) & ~3, M16 = (m + 15) & ~15;
    const int nsc = (U3_NC - 1 + stride - 1) / stride + 2;
    return ((size_t)nf * m * U3_NC + (size_t)nf * U3_NC * M16 + (size_t)nsc * md * U3_TLD + (size_t)nsc * M4) *
           sizeof(float);
}

template <bool F64, int EPL>
__global__ void __launch_bounds__(UPD_NT) k_update_v3(UpdArgs a)
{
    static_assert(U3_KE == 16 && U3_NC == 8, "the staging loops index by shifts");
    extern __shared__ __align__(16) float usm[];
    const int m = a.m, md = a.md, st = a.stride, nf = a.nfield;   // nf <= U3_FG
    const int tid = threadIdx.x, lane = tid & 31, c = tid >> 5;
    const int M4 = (m + 3) & ~3, M16 = (m + 15) & ~15;
    const int jt = blockIdx.y, jg = a.j1 + jt;
    const int jj = a.j1 / st + jt / st, stepj = jt % st;
    const int jj2 = (jj < a.nj - 1) ? jj + 1 : jj;
    const int i0 = blockIdx.x * U3_NC;
    const int ncell = min(U3_NC, a.mni - i0);
    const int iia = i0 / st, iib = (i0 + ncell - 1) / st;
    const int nsc = iib - iia + 2;                 // strided columns, the last the i-neighbour
    const int nb = (iib < a.ni - 1) ? iib + 1 : (a.periodic_i ? (iib + 1) % a.ni : iib);
    const int nscap = (U3_NC - 1 + st - 1) / st + 2;   // strided columns of 8 cells, at most
    float* raw = usm;                                          // [nf][m][U3_NC]
    float* Am = raw + (size_t)nf * m * U3_NC;                  // [nf][U3_NC][M16] (zero past m)
    float* Tc = Am + (size_t)nf * U3_NC * M16;                 // [nscap][md][U3_TLD]
    float* Wc = Tc + (size_t)nscap * md * U3_TLD;              // [nscap][M4]
    const float w2j = __fdiv_rn((float)stepj, (float)st), w1j = __fsub_rn(1.0f, w2j);
    const bool jint = (st > 1 && stepj > 0);

    // 1. the field block (member rows of 8 cells: 32-byte pieces) and the
    //    j-interpolated w of the strided columns
    for (int q = 0; q < nf; ++q) {
        const float* src = a.fields + (size_t)q * m * a.plane + (size_t)jt * a.mni + i0;
        float* dst = raw + (size_t)q * m * U3_NC;
        for (int idx = tid; idx < m * U3_NC; idx += UPD_NT) {
            const int e = idx >> 3, cc = idx & 7;
            if (cc < ncell) dst[idx] = src[(size_t)e * a.plane + cc];
        }
    }
    for (int idx = tid; idx < nsc * m; idx += UPD_NT) {
        const int k = idx / m, e = idx - k * m;
        const int col = (k < nsc - 1) ? iia + k : nb;
        float v = __ldg(&a.w[((size_t)jj * a.ni + col) * m + e]);
        if (jint) v = __fadd_rn(__fmul_rn(v, w1j), __fmul_rn(__ldg(&a.w[((size_t)jj2 * a.ni + col) * m + e]), w2j));
        Wc[k * M4 + e] = v;
    }
    __syncthreads();

    // 2. per warp (its cell): masks, missing values, mean, anomalies
    const int i = i0 + c;
    const bool live = c < ncell;
    const int slot = live ? i / st - iia : 0, stepi = live ? i % st : 0;
    const bool iint = (st > 1 && stepi > 0);
    const float u2 = __fdiv_rn((float)stepi, (float)st), u1 = __fsub_rn(1.0f, u2);
    const size_t ioff = (size_t)jt * a.mni + i;
    unsigned active = 0;
    Mean<F64> mean[U3_FG];
    if (live) {
        const int nl = a.numlevels[(size_t)jg * a.mni + i];
        // (q unrolled: the means stay in registers)
#pragma unroll
        for (int q = 0; q < U3_FG; ++q) {
            if (q >= nf) break;
            float* v = raw + (size_t)q * m * U3_NC;
            float* Aq = Am + ((size_t)q * U3_NC + c) * M16;
            const int level = a.levels[q];
            mean[q].zero();
            const bool masked = (a.surfk == 0) ? (nl <= level) : (nl <= (a.issurfacevar ? 0 : a.surfk - level));
            if (masked) {
                for (int e = lane; e < m; e += 32) v[e * U3_NC + c] = 0.0f;
                if (a.infl && lane == 0) a.infl[(size_t)q * a.plane + ioff] = 0.0f;
                continue;
            }
            int first = m;
            for (int e0 = 0; e0 < m && first == m; e0 += 32) {
                const int e = e0 + lane;
                bool bad = false;
                if (e < m) {
                    const float x = v[e * U3_NC + c];
                    bad = !isfinite(x) || fabsf(x) > MAXOBSVAL_F;
                }
                const unsigned bal = __ballot_sync(0xffffffffu, bad);
                if (bal) first = e0 + __ffs(bal) - 1;
            }
            if (a.infl && lane == 0) a.infl[(size_t)q * a.plane + ioff] = 0.0f;
            if (first < md) {
                for (int e = lane; e < m; e += 32) v[e * U3_NC + c] = 0.0f;
                continue;
            } else if (first < m) {
                for (int e = md + lane; e < m; e += 32) v[e * U3_NC + c] = 0.0f;
                if (md == 0) continue;
            }
            Acc<F64> sm;
            for (int e = lane; e < md; e += 32) sm.add(v[e * U3_NC + c]);
            sm.reduce();
            mean[q].set(sm, md);
            for (int e = lane; e < M16; e += 32) Aq[e] = (e < m) ? mean[q].sub(v[e * U3_NC + c]) : 0.0f;
            active |= 1u << q;
        }
    }

    // 3. A^a = A^f X5 over chunks of U3_KE members of the reduction
    float acc[U3_FG][EPL];
#pragma unroll
    for (int q = 0; q < U3_FG; ++q)
#pragma unroll
        for (int k = 0; k < EPL; ++k) acc[q][k] = 0.0f;
    for (int e0 = 0; e0 < m; e0 += U3_KE) {
        const int ke_n = min(U3_KE, m - e0);
        __syncthreads();   // the previous chunk is consumed (and the anomalies are written)
        // rows (slot, e1) of U3_KE members: four lanes per row with 16-byte
        // loads when the rows are 16-byte aligned (nmem a multiple of 4 and
        // the chunk whole), else one lane per element
        const size_t jstep = ((size_t)jj2 - jj) * a.ni * md * m;
        if ((m & 3) == 0 && ke_n == U3_KE) {
            for (int idx = tid; idx < nsc * md * 4; idx += UPD_NT) {
                const int qd = idx & 3, se = idx >> 2;
                const int sl = se / md, e1 = se - sl * md;
                const int col = (sl < nsc - 1) ? iia + sl : nb;
                const size_t o = ((size_t)jj * a.ni + col) * md * m + (size_t)e1 * m + e0 + 4 * qd;
                float4 v = __ldg(reinterpret_cast<const float4*>(a.T + o));
                if (jint) {
                    const float4 b = __ldg(reinterpret_cast<const float4*>(a.T + o + jstep));
                    v.x = __fadd_rn(__fmul_rn(v.x, w1j), __fmul_rn(b.x, w2j));
                    v.y = __fadd_rn(__fmul_rn(v.y, w1j), __fmul_rn(b.y, w2j));
                    v.z = __fadd_rn(__fmul_rn(v.z, w1j), __fmul_rn(b.z, w2j));
                    v.w = __fadd_rn(__fmul_rn(v.w, w1j), __fmul_rn(b.w, w2j));
                }
                *reinterpret_cast<float4*>(&Tc[((size_t)sl * md + e1) * U3_TLD + 4 * qd]) = v;
            }
        } else {
            for (int sl = 0; sl < nsc; ++sl) {
                const int col = (sl < nsc - 1) ? iia + sl : nb;
                for (int idx = tid; idx < md * U3_KE; idx += UPD_NT) {
                    const int e1 = idx >> 4, ke = idx & 15;
                    float v = 0.0f;
                    if (ke < ke_n) {
                        const size_t o = ((size_t)jj * a.ni + col) * md * m + (size_t)e1 * m + e0 + ke;
                        v = __ldg(&a.T[o]);
                        if (jint) v = __fadd_rn(__fmul_rn(v, w1j), __fmul_rn(__ldg(&a.T[o + jstep]), w2j));
                    }
                    Tc[((size_t)sl * md + e1) * U3_TLD + ke] = v;
                }
            }
        }
        __syncthreads();
        if (active) {
#pragma unroll
            for (int ke = 0; ke < U3_KE; ke += 4) {
                float4 t[EPL];
#pragma unroll
                for (int k = 0; k < EPL; ++k) {
                    const int e1 = lane + 32 * k;
                    t[k] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                    if (e1 < md) {
                        t[k] = *reinterpret_cast<const float4*>(&Tc[((size_t)slot * md + e1) * U3_TLD + ke]);
                        if (iint) {
                            const float4 tb =
                                *reinterpret_cast<const float4*>(&Tc[((size_t)(slot + 1) * md + e1) * U3_TLD + ke]);
                            t[k].x = __fadd_rn(__fmul_rn(t[k].x, u1), __fmul_rn(tb.x, u2));
                            t[k].y = __fadd_rn(__fmul_rn(t[k].y, u1), __fmul_rn(tb.y, u2));
                            t[k].z = __fadd_rn(__fmul_rn(t[k].z, u1), __fmul_rn(tb.z, u2));
                            t[k].w = __fadd_rn(__fmul_rn(t[k].w, u1), __fmul_rn(tb.w, u2));
                        }
                    }
                }
#pragma unroll
                for (int q = 0; q < U3_FG; ++q) {
                    if (q < nf) {
                        const float4 av =
                            *reinterpret_cast<const float4*>(&Am[((size_t)q * U3_NC + c) * M16 + e0 + ke]);
#pragma unroll
                        for (int k = 0; k < EPL; ++k) {
                            acc[q][k] = fmaf(t[k].x, av.x, acc[q][k]);
                            acc[q][k] = fmaf(t[k].y, av.y, acc[q][k]);
                            acc[q][k] = fmaf(t[k].z, av.z, acc[q][k]);
                            acc[q][k] = fmaf(t[k].w, av.w, acc[q][k]);
                        }
                    }
                }
            }
        }
    }

    // 4. per warp and field-layer: mean update, hybrid rescaling, inflation,
    //    outputs into the staged block (update.c:393-516)
    if (active) {
        // (q unrolled: the accumulators stay in registers)
#pragma unroll
        for (int q = 0; q < U3_FG; ++q) {
            if (q >= nf) break;
            if (!((active >> q) & 1u)) continue;
            float* v = raw + (size_t)q * m * U3_NC;
            const float* Aq = Am + ((size_t)q * U3_NC + c) * M16;
            float inflation = a.inflation0;
            Acc<F64> sa;
            for (int e = lane; e < m; e += 32) {
                float t = Wc[slot * M4 + e];
                if (iint) t = __fadd_rn(__fmul_rn(t, u1), __fmul_rn(Wc[(slot + 1) * M4 + e], u2));
                sa.add_prod(Aq[e], t);
            }
            sa.reduce();
            const Mean<F64> v1_a = mean[q].plus(sa);
            float af[EPL], aa[EPL];
#pragma unroll
            for (int k = 0; k < EPL; ++k) {
                const int e = lane + 32 * k;
                af[k] = (e < m) ? Aq[e] : 0.0f;
                aa[k] = acc[q][k];
            }
            if (a.mode == ENKFG_MODE_HYBRID) {
                if constexpr (F64) {
                    const double k_d = (md > 1) ? sqrt((double)(m - 1) / (double)(md - 1)) : 1.0;
#pragma unroll
                    for (int k = 0; k < EPL; ++k)
                        if (lane + 32 * k < md) {
                            aa[k] = (float)((double)aa[k] / k_d);
                            af[k] = (float)((double)af[k] / k_d);
                        }
                } else {
                    const float rk = a.inv_kd;
#pragma unroll
                    for (int k = 0; k < EPL; ++k)
                        if (lane + 32 * k < md) {
                            aa[k] = __fmul_rn(aa[k], rk);
                            af[k] = __fmul_rn(af[k], rk);
                        }
                }
            }
            if (!isnan(a.inf_ratio)) {
                Acc<F64> s2f, s2a;
#pragma unroll
                for (int k = 0; k < EPL; ++k)
                    if (lane + 32 * k < md) {
                        s2f.add_prod(af[k], af[k]);
                        s2a.add_prod(aa[k], aa[k]);
                    }
                s2f.reduce();
                s2a.reduce();
                if constexpr (F64) {
                    const double v2_f = s2f.value(), v2_a = s2a.value();
                    if (v2_a > 0.0) {
                        inflation = (float)(sqrt(v2_f / v2_a) * a.inf_ratio + 1.0 - a.inf_ratio);
                        if (inflation >= a.inflation0) inflation = a.inflation0;
                    }
                } else {
                    const float v2_f = s2f.hi + s2f.lo, v2_a = s2a.hi + s2a.lo;
                    if (v2_a > 0.0f) {
                        const float r = (float)a.inf_ratio;
                        inflation = fmaf(sqrtf(__fdiv_rn(v2_f, v2_a)), r, 1.0f - r);
                        if (inflation >= a.inflation0) inflation = a.inflation0;
                    }
                }
            }
            const bool inflate = __fsub_rn(inflation, 1.0f) > 1.0e-6f;
            if (!inflate) inflation = 1.0f;
#pragma unroll
            for (int k = 0; k < EPL; ++k) {
                const int e1 = lane + 32 * k;
                if (e1 < md) {
                    float va = inflate ? __fmul_rn(aa[k], inflation) : aa[k];
                    va = v1_a.add(va);
                    const float vf = mean[q].add(af[k]);
                    float out;
                    if (!a.output_increment) out = va;
                    else if (!a.applylog) out = __fsub_rn(va, vf);
                    else {
                        const float avf = fabsf(vf);
                        const bool normal = (avf >= 1.17549435e-38f) && (avf <= 3.40282347e+38f);
                        const double ea = pow(10.0, (double)va), ef = pow(10.0, (double)vf);
                        out = normal ? (float)(ea - ef) : 0.0f;
                    }
                    v[e1 * U3_NC + c] = out;
                }
            }
            if (a.infl && lane == 0) a.infl[(size_t)q * a.plane + ioff] = inflation;
        }
    }
    __syncthreads();
    // 5. the block back out
    for (int q = 0; q < nf; ++q) {
        float* dst = a.fields + (size_t)q * m * a.plane + (size_t)jt * a.mni + i0;
        const float* src = raw + (size_t)q * m * U3_NC;
        for (int idx = tid; idx < m * U3_NC; idx += UPD_NT) {
            const int e = idx >> 3, cc = idx & 7;
            if (cc < ncell) dst[(size_t)e * a.plane + cc] = src[idx];
        }
    }
}

// das_updatefields, thread-per-cell form for nmem <= 64 (MT = nmem rounded
// up to a multiple of 8).  A CTA of 4 warps owns UPC_NC = 16 consecutive
// cells of one model row: lane l of warp w takes cell i0 + (l & 15) and
// field-layer 2 w + (l >> 4) (then + 8, ...).  The j-interpolated transforms
// of the strided columns those cells touch (Tjj, update.c:224-241) are
// staged once in shared memory, rows padded to a multiple of 4 floats and
// slots spaced 4 words mod 32 apart, so that lanes on different slots read
// different banks with 16-byte loads and lanes on the same slot share a
// broadcast; about 74 KB at nmem 48 and stride 3, three CTAs per SM.  Per
// cell and layer the thread keeps the member values in registers: member
// planes load and store coalesced over the 16 consecutive cells, and the
// mean, the mean increment and the spread sums are sequential sums over
// members in the reference's order -- no cross-lane reductions.  Each row of
// A^a = X5 A is formed and written at once, several rows at a time
// (independent sums, so that the FMA chains overlap); with spread-capped
// inflation (inf_ratio set) the rows are formed twice, first for the spread.
// The FP64 variant forms the i-interpolated X5 element with the reference's
// float operations (update.c:255-265) and sums each row in the reference's
// order; the FP32 variant applies the two strided columns' rows to the
// member values separately and interpolates the two sums (u1 Ta x + u2 Tb x).
#define UPC_NC 16
#define UPC_NT 128
// rows e1b .. e1b+R-1 (those below md) of A^a = X5 A for one cell and layer
// (R = 4 rows at a time in the FP32 variant, 2 in the FP64 one, whose
// per-element interpolation needs more registers)
template <bool F64>
struct X5Rows {
    static constexpr int R = F64 ? 2 : 4;
};

template <bool F64, int MT>
__device__ __forceinline__ void x5_rows(const float* __restrict__ Ta, const float* __restrict__ Tb, int e1b, int m4,
                                        int m, int md, float u1, float u2, const float (&x)[MT],
                                        float (&y)[X5Rows<F64>::R])
{
    constexpr int R = X5Rows<F64>::R;
    float sa[R], sb[R];
#pragma unroll
    for (int r = 0; r < R; ++r) sa[r] = sb[r] = 0.0f;
#pragma unroll
    for (int q = 0; q < MT / 4; ++q) {
        if (4 * q < m) {
#pragma unroll
            for (int r = 0; r < R; ++r) {
                if (e1b + r < md) {
                    const float4 p = reinterpret_cast<const float4*>(Ta + (e1b + r) * m4)[q];
                    const float4 t = reinterpret_cast<const float4*>(Tb + (e1b + r) * m4)[q];
                    if constexpr (F64) {
                        const float t0 = __fadd_rn(__fmul_rn(p.x, u1), __fmul_rn(t.x, u2));
                        const float t1 = __fadd_rn(__fmul_rn(p.y, u1), __fmul_rn(t.y, u2));
                        const float t2 = __fadd_rn(__fmul_rn(p.z, u1), __fmul_rn(t.z, u2));
                        const float t3 = __fadd_rn(__fmul_rn(p.w, u1), __fmul_rn(t.w, u2));
                        sa[r] = fmaf(t0, x[4 * q], sa[r]);
                        sa[r] = fmaf(t1, x[4 * q + 1], sa[r]);
                        sa[r] = fmaf(t2, x[4 * q + 2], sa[r]);
                        sa[r] = fmaf(t3, x[4 * q + 3], sa[r]);
                    } else {
                        sa[r] = fmaf(p.x, x[4 * q], sa[r]);
                        sb[r] = fmaf(t.x, x[4 * q], sb[r]);
                        sa[r] = fmaf(p.y, x[4 * q + 1], sa[r]);
                        sb[r] = fmaf(t.y, x[4 * q + 1], sb[r]);
                        sa[r] = fmaf(p.z, x[4 * q + 2], sa[r]);
                        sb[r] = fmaf(t.z, x[4 * q + 2], sb[r]);
                        sa[r] = fmaf(p.w, x[4 * q + 3], sa[r]);
                        sb[r] = fmaf(t.w, x[4 * q + 3], sb[r]);
                    }
                }
            }
        }
    }
#pragma unroll
    for (int r = 0; r < R; ++r) y[r] = F64 ? sa[r] : fmaf(sa[r], u1, sb[r] * u2);
}

template <bool F64, int MT>
__global__ void __launch_bounds__(UPC_NT) k_update_cells(UpdArgs a, int sstride)
{
    extern __shared__ __align__(16) float usm[];
    const int m = a.m, md = a.md, st = a.stride, nf = a.nfield;
    const int m4 = (m + 3) & ~3;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int jt = blockIdx.y, jg = a.j1 + jt;
    const int jj = a.j1 / st + jt / st, stepj = jt % st;
    const int jj2 = (jj < a.nj - 1) ? jj + 1 : jj;
    const int i0 = blockIdx.x * UPC_NC;
    const int ilast = min(i0 + UPC_NC, a.mni) - 1;
    const int s0 = i0 / st;
    const int ns = ilast / st - s0 + 2;                      // staged slots (the last one: i-neighbour)
    const int nsmax = (UPC_NC - 1) / st + 3;
    float* Tjj = usm;                                        // [nsmax][sstride]: [md][m4] per slot
    float* Wjj = usm + (size_t)nsmax * sstride;              // [nsmax][m4]

    // 1. stage: staged slot k holds strided column g(k) = s0 + k, wrapped
    //    (periodic) or clamped past the last column, j-interpolated; pads 0
    {
        const float w2 = __fdiv_rn((float)stepj, (float)st), w1 = __fsub_rn(1.0f, w2);
        const bool jint = (st > 1 && stepj > 0);
        const int per = md * m4;
        if ((m & 3) == 0 && ((uintptr_t)a.T & 15) == 0) {
            // rows of m = m4 floats, 16-byte aligned: four elements a load
            const int q4 = m4 >> 2, per4 = md * q4;
            for (int k = 0; k < ns; ++k) {
                int g = s0 + k;
                if (g >= a.ni) g = a.periodic_i ? g - a.ni : a.ni - 1;
                const float4* ta = reinterpret_cast<const float4*>(a.T + ((size_t)jj * a.ni + g) * md * m);
                const float4* tb = reinterpret_cast<const float4*>(a.T + ((size_t)jj2 * a.ni + g) * md * m);
                float4* dst = reinterpret_cast<float4*>(Tjj + (size_t)k * sstride);
                for (int i = tid; i < per4; i += UPC_NT) {
                    float4 v = __ldg(ta + i);
                    if (jint) {
                        const float4 u = __ldg(tb + i);
                        v.x = __fadd_rn(__fmul_rn(v.x, w1), __fmul_rn(u.x, w2));
                        v.y = __fadd_rn(__fmul_rn(v.y, w1), __fmul_rn(u.y, w2));
                        v.z = __fadd_rn(__fmul_rn(v.z, w1), __fmul_rn(u.z, w2));
                        v.w = __fadd_rn(__fmul_rn(v.w, w1), __fmul_rn(u.w, w2));
                    }
                    dst[i] = v;   // row e1 = i / q4 at e1 * m4: the same offset, m4 = m
                }
            }
        } else {
            for (int idx = tid; idx < ns * per; idx += UPC_NT) {
                const int k = idx / per, r = idx - k * per;
                const int e1 = r / m4, e = r - e1 * m4;
                int g = s0 + k;
                if (g >= a.ni) g = a.periodic_i ? g - a.ni : a.ni - 1;
                float v = 0.0f;
                if (e < m) {
                    v = __ldg(a.T + (((size_t)jj * a.ni + g) * md + e1) * m + e);
                    if (jint)
                        v = __fadd_rn(__fmul_rn(v, w1),
                                      __fmul_rn(__ldg(a.T + (((size_t)jj2 * a.ni + g) * md + e1) * m + e), w2));
                }
                Tjj[(size_t)k * sstride + r] = v;
            }
        }
        for (int idx = tid; idx < ns * m4; idx += UPC_NT) {
            const int k = idx / m4, e = idx - k * m4;
            int g = s0 + k;
            if (g >= a.ni) g = a.periodic_i ? g - a.ni : a.ni - 1;
            float v = 0.0f;
            if (e < m) {
                v = __ldg(a.w + ((size_t)jj * a.ni + g) * m + e);
                if (jint) v = __fadd_rn(__fmul_rn(v, w1), __fmul_rn(__ldg(a.w + ((size_t)jj2 * a.ni + g) * m + e), w2));
            }
            Wjj[k * m4 + e] = v;
        }
    }
    __syncthreads();

    const int i = i0 + (lane & 15);
    if (i > ilast) return;                                   // no barrier below
    const int ii = i / st, stepi = i % st;
    const bool iint = (st > 1 && stepi > 0);
    const float u2 = iint ? __fdiv_rn((float)stepi, (float)st) : 0.0f;
    const float u1 = iint ? __fsub_rn(1.0f, u2) : 1.0f;
    const float* Ta = Tjj + (size_t)(ii - s0) * sstride;
    const float* Tb = Ta + sstride;
    const float* Wa = Wjj + (ii - s0) * m4;
    const float* Wb = Wa + m4;
    const int nl = a.numlevels[(size_t)jg * a.mni + i];
    const size_t ioff = (size_t)jt * a.mni + i;
    const bool capped = !isnan(a.inf_ratio);

    for (int f = 2 * wid + (lane >> 4); f < nf; f += 2 * (UPC_NT / 32)) {
        float* v = a.fields + (size_t)f * m * a.plane + ioff;   // member e at v[e * plane]
        const int level = a.levels[f];
        const bool masked = (a.surfk == 0) ? (nl <= level) : (nl <= (a.issurfacevar ? 0 : a.surfk - level));
        if (masked) {
            for (int e = 0; e < m; ++e) v[(size_t)e * a.plane] = 0.0f;
            if (a.infl) a.infl[(size_t)f * a.plane + ioff] = 0.0f;
            continue;
        }
        float x[MT];
        int first = m;
#pragma unroll
        for (int e = 0; e < MT; ++e) {
            x[e] = 0.0f;
            if (e < m) x[e] = v[(size_t)e * a.plane];
        }
#pragma unroll
        for (int e = 0; e < MT; ++e)
            if (e < m && first == m && (!isfinite(x[e]) || fabsf(x[e]) > MAXOBSVAL_F)) first = e;
        if (a.infl) a.infl[(size_t)f * a.plane + ioff] = 0.0f;
        if (first < md) {
            for (int e = 0; e < m; ++e) v[(size_t)e * a.plane] = 0.0f;
            continue;
        }
        if (first < m) {
            for (int e = md; e < m; ++e) v[(size_t)e * a.plane] = 0.0f;
#pragma unroll
            for (int e = 0; e < MT; ++e)
                if (e >= md) x[e] = 0.0f;
        }
        // mean over the dynamic members (update.c:381-383)
        Acc<F64> sm;
#pragma unroll
        for (int e = 0; e < MT; ++e)
            if (e < md) sm.add(x[e]);
        Mean<F64> mean;
        mean.set(sm, md);
        // anomalies (float) and the mean increment (update.c:381-410)
        Acc<F64> sa;
#pragma unroll
        for (int e = 0; e < MT; ++e)
            if (e < m) {
                x[e] = mean.sub(x[e]);
                const float wc = __fadd_rn(__fmul_rn(Wa[e], u1), __fmul_rn(Wb[e], u2));
                sa.add_prod(x[e], wc);
            }
        const Mean<F64> v1_a = mean.plus(sa);
        // hybrid rescaling factor (update.c:420-427)
        const bool hyb = (a.mode == ENKFG_MODE_HYBRID);
        const double k_d = (F64 && hyb && md > 1) ? sqrt((double)(m - 1) / (double)(md - 1)) : 1.0;
        auto rescale = [&](float y) -> float {
            if (!hyb) return y;
            if constexpr (F64) return (float)((double)y / k_d);
            else return __fmul_rn(y, a.inv_kd);
        };
        // spread-capped inflation (update.c:432-458): needs every row first
        float inflation = a.inflation0;
        if (capped) {
            Acc<F64> s2f, s2a;
#pragma unroll
            for (int e = 0; e < MT; ++e)
                if (e < md) {
                    const float y = rescale(x[e]);
                    s2f.add_prod(y, y);
                }
            for (int e1b = 0; e1b < md; e1b += X5Rows<F64>::R) {
                float y4[X5Rows<F64>::R];
                x5_rows<F64, MT>(Ta, Tb, e1b, m4, m, md, u1, u2, x, y4);
#pragma unroll
                for (int r = 0; r < X5Rows<F64>::R; ++r)
                    if (e1b + r < md) {
                        const float y = rescale(y4[r]);
                        s2a.add_prod(y, y);
                    }
            }
            if constexpr (F64) {
                const double v2_f = s2f.value(), v2_a = s2a.value();
                if (v2_a > 0.0) {
                    inflation = (float)(sqrt(v2_f / v2_a) * a.inf_ratio + 1.0 - a.inf_ratio);
                    if (inflation >= a.inflation0) inflation = a.inflation0;
                }
            } else {
                const float v2_f = s2f.hi + s2f.lo, v2_a = s2a.hi + s2a.lo;
                if (v2_a > 0.0f) {
                    const float r = (float)a.inf_ratio;
                    inflation = fmaf(sqrtf(__fdiv_rn(v2_f, v2_a)), r, 1.0f - r);
                    if (inflation >= a.inflation0) inflation = a.inflation0;
                }
            }
        }
        const bool inflate = __fsub_rn(inflation, 1.0f) > 1.0e-6f;
        if (!inflate) inflation = 1.0f;
        // A^a = X5 A (update.c:399) and the output (update.c:460-516)
        for (int e1b = 0; e1b < md; e1b += X5Rows<F64>::R) {
          float y4[X5Rows<F64>::R];
          x5_rows<F64, MT>(Ta, Tb, e1b, m4, m, md, u1, u2, x, y4);
#pragma unroll
          for (int r = 0; r < X5Rows<F64>::R; ++r) {
            const int e1 = e1b + r;
            if (e1 >= md) break;
            const float y = rescale(y4[r]);
            float va = inflate ? __fmul_rn(y, inflation) : y;
            va = v1_a.add(va);
            float out;
            if (!a.output_increment) out = va;
            else {
                // forecast member value (its anomaly, hybrid-rescaled, plus the mean)
                float xf = 0.0f;
#pragma unroll
                for (int e = 0; e < MT; ++e)
                    if (e == e1) xf = x[e];
                const float vf = mean.add(rescale(xf));
                if (!a.applylog) out = __fsub_rn(va, vf);
                else {
                    const float avf = fabsf(vf);
                    const bool normal = (avf >= 1.17549435e-38f) && (avf <= 3.40282347e+38f);
                    const double ea = pow(10.0, (double)va), ef = pow(10.0, (double)vf);
                    out = normal ? (float)(ea - ef) : 0.0f;
                }
            }
            v[(size_t)e1 * a.plane] = out;
          }
        }
        if (a.infl) a.infl[(size_t)f * a.plane + ioff] = inflation;
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

// The field-layer levels of one launch group go to the device only when they
// differ from the group last uploaded (no host-to-device copy in a steady
// cycle, which CUDA graphs capture).  Synchronous copy: it is rare.
// The field-layers' levels on the device, copied only when they change: in
// stream order on `st` (after the kernels that read the previous ones), from
// the context's host copy.
static enkfg_status upload_levels(enkfg_ctx* ctx, const int* levels, int nf, int* d_levels, cudaStream_t st)
{
    if (ctx->n_levels == nf && memcmp(ctx->h_levels, levels, nf * sizeof(int)) == 0) return ENKFG_OK;
    memcpy(ctx->h_levels, levels, nf * sizeof(int));
    ctx->n_levels = nf;
    CK(cudaMemcpyAsync(d_levels, ctx->h_levels, nf * sizeof(int), cudaMemcpyHostToDevice, st));
    return ENKFG_OK;
}

enkfg_status run_update(enkfg_ctx* ctx, const enkfg_update_params* p, const int* d_numlevels, int nfield,
                        const int* levels, float* d_fields, float* d_infl, cudaStream_t st)
{
    enkfg_status s;
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
    a.inv_kd = (float)(1.0 / ((a.md > 1) ? sqrt((double)(a.m - 1) / (double)(a.md - 1)) : 1.0));
    int* d_levels = ctx->d_qhead + 64;       // up to 448 levels per launch group
    cudaEventRecord(ctx->ev[4], st);
    if (p->mode == ENKFG_MODE_ENOI) {
        for (int f0 = 0; f0 < nfield; f0 += 448) {
            int nf = nfield - f0 < 448 ? nfield - f0 : 448;
            if ((s = upload_levels(ctx, levels + f0, nf, d_levels, st))) return s;
            a.levels = d_levels;
            a.nfield = nf;
            a.fields = d_fields + (size_t)f0 * (a.m + 1) * a.plane;
            dim3 g(div_up(a.mni, 128), a.jsize);
            k_update_bg<<<g, 128, 0, st>>>(a);
            CKL();
        }
        cudaEventRecord(ctx->ev[5], st);
        return ENKFG_OK;
    }
    // thread-per-cell kernel (nmem <= 64) when its staged slots fit
    if (a.m <= 64) {
        const int MT = a.m <= 24 ? 24 : a.m <= 32 ? 32 : a.m <= 48 ? 48 : 64;
        const int m4 = (a.m + 3) & ~3;
        int sstride = a.md * m4;
        sstride += (4 - sstride % 32 + 32) % 32;             // slot stride = 4 mod 32 words
        const size_t nsmax = (size_t)(UPC_NC - 1) / a.stride + 3;
        const size_t smem = (nsmax * sstride + nsmax * m4) * sizeof(float);
        if (smem <= 200 * 1024) {
            const bool f64 = (p->precision == ENKFG_PREC_FP64);
            auto launch = [&](auto kern) -> enkfg_status {
                CK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
                for (int f0 = 0; f0 < nfield; f0 += 448) {
                    int nf = nfield - f0 < 448 ? nfield - f0 : 448;
                    if ((s = upload_levels(ctx, levels + f0, nf, d_levels, st))) return s;
                    a.levels = d_levels;
                    a.nfield = nf;
                    a.fields = d_fields + (size_t)f0 * a.m * a.plane;
                    a.infl = d_infl ? d_infl + (size_t)f0 * a.plane : nullptr;
                    dim3 g(div_up(a.mni, UPC_NC), a.jsize);
                    kern<<<g, UPC_NT, smem, st>>>(a, sstride);
                    CKL();
                }
                cudaEventRecord(ctx->ev[5], st);
                return ENKFG_OK;
            };
            if (f64) {
                if (MT == 24) return launch(k_update_cells<true, 24>);
                if (MT == 32) return launch(k_update_cells<true, 32>);
                if (MT == 48) return launch(k_update_cells<true, 48>);
                return launch(k_update_cells<true, 64>);
            }
            if (MT == 24) return launch(k_update_cells<false, 24>);
            if (MT == 32) return launch(k_update_cells<false, 32>);
            if (MT == 48) return launch(k_update_cells<false, 48>);
            return launch(k_update_cells<false, 64>);
        }
    }
    if (a.m > 32 * MAXE_PER_LANE || a.md > 32 * MAXE_PER_LANE) {
        set_err(ctx, "nmem = %d too large for the update kernel", a.m);
        return ENKFG_EUNSUPPORTED;
    }
    // version 3: 8 cells per CTA, the transforms streamed once per group of
    // U3_FG field-layers
    {
        const int fg3 = nfield < U3_FG ? nfield : U3_FG;
        const size_t smem3 = upd_v3_smem(a.m, a.md, a.stride, fg3);
        if (smem3 <= 200 * 1024) {
            const bool f64 = (p->precision == ENKFG_PREC_FP64);
            const int epl = (a.md + 31) / 32;
            auto launch3 = [&](auto kern) -> enkfg_status {
                CK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem3));
                for (int g0 = 0; g0 < nfield; g0 += 448) {
                    const int ng = nfield - g0 < 448 ? nfield - g0 : 448;
                    if ((s = upload_levels(ctx, levels + g0, ng, d_levels, st))) return s;
                    for (int f0 = g0; f0 < g0 + ng; f0 += fg3) {
                        const int nf = g0 + ng - f0 < fg3 ? g0 + ng - f0 : fg3;
                        a.levels = d_levels + (f0 - g0);
                        a.nfield = nf;
                        a.fields = d_fields + (size_t)f0 * a.m * a.plane;
                        a.infl = d_infl ? d_infl + (size_t)f0 * a.plane : nullptr;
                        dim3 g(div_up(a.mni, U3_NC), a.jsize);
                        kern<<<g, UPD_NT, smem3, st>>>(a);
                        CKL();
                    }
                }
                cudaEventRecord(ctx->ev[5], st);
                return ENKFG_OK;
            };
            switch (epl) {
            case 1: return f64 ? launch3(k_update_v3<true, 1>) : launch3(k_update_v3<false, 1>);
            case 2: return f64 ? launch3(k_update_v3<true, 2>) : launch3(k_update_v3<false, 2>);
            case 3: return f64 ? launch3(k_update_v3<true, 3>) : launch3(k_update_v3<false, 3>);
            case 4: return f64 ? launch3(k_update_v3<true, 4>) : launch3(k_update_v3<false, 4>);
            default: return f64 ? launch3(k_update_v3<true, 5>) : launch3(k_update_v3<false, 5>);
            }
        }
    }
    // strided columns per CTA, field-layers per warp task and per launch: keep
    // two CTAs per SM (<= ~100 KB of shared memory each) when possible
    const size_t smem_cap = 100 * 1024;
    const int M4 = (a.m + 3) & ~3, TLD = a.m + 1;
    auto need = [&](int G, int nf, int fc) {
        size_t cp = (size_t)G * a.stride;
        return ((((size_t)(G + 1) * a.md * TLD + 3) & ~(size_t)3) + (size_t)(G + 1) * M4 +
                (((size_t)nf * a.m * cp + 3) & ~(size_t)3) + (size_t)(UPD_NT / 32) * fc * M4) * sizeof(float);
    };
    int G = a.stride >= 16 ? 1 : (16 + a.stride - 1) / a.stride;
    int fg = nfield;
    int fc = UPD_FC;
    while (G > 1 && need(G, fg, fc) > smem_cap) --G;
    if (need(G, fg, fc) > smem_cap) fc = 4;
    while (fg > 1 && need(G, fg, fc) > smem_cap) fg = (fg + 1) / 2;
    if (fg > 448) fg = 448;
    // enough warp tasks for the 8 warps of a CTA
    if ((G * a.stride) * ((fg + fc - 1) / fc) < 16) fc = 4;
    size_t smem = need(G, fg, fc);
    if (smem > 227 * 1024) {
        set_err(ctx, "update tile does not fit in shared memory (nmem %d)", a.m);
        return ENKFG_EUNSUPPORTED;
    }
    a.fc = fc;
    const bool f64 = (p->precision == ENKFG_PREC_FP64);
    if (f64) CK(cudaFuncSetAttribute(k_update_v2<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    else CK(cudaFuncSetAttribute(k_update_v2<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    a.G = G;
    a.nk = G * a.stride;
    // the levels of up to 448 field-layers go to the device once; launch
    // groups index into them, so nothing waits between groups (and the
    // steady cycle, with unchanged levels, makes no host copy)
    for (int g0 = 0; g0 < nfield; g0 += 448) {
        const int ng = nfield - g0 < 448 ? nfield - g0 : 448;
        if ((s = upload_levels(ctx, levels + g0, ng, d_levels, st))) return s;
        for (int f0 = g0; f0 < g0 + ng; f0 += fg) {
            const int nf = g0 + ng - f0 < fg ? g0 + ng - f0 : fg;
            a.levels = d_levels + (f0 - g0);
            a.nfield = nf;
            a.fields = d_fields + (size_t)f0 * a.m * a.plane;
            a.infl = d_infl ? d_infl + (size_t)f0 * a.plane : nullptr;
            dim3 g(div_up(a.ni, G), a.jsize);
            if (f64) k_update_v2<true><<<g, UPD_NT, smem, st>>>(a);
            else k_update_v2<false><<<g, UPD_NT, smem, st>>>(a);
            CKL();
        }
    }
    cudaEventRecord(ctx->ev[5], st);
    return ENKFG_OK;
}

// ---------------------------------------------------------------------------
// RANDOMISE (addnoise, update/update.c:46-87, applied after the update of a
// set of fields, :552-563): every cell of member e of a field-layer with a
// finite deflation becomes v * (float)deflation + mult * r_e, where the
// member's term mult * r_e (mult = (float)(sqrt(1 - deflation^2) * sigma), r
// the host's normals less their member mean) is a double formed on the host
// (enkfg_set_field_noise).  The precisions are the reference's: the float
// product, then the double sum rounded to float.  One plane (member of a
// field-layer) per blockIdx.y; planes are [layer][member], ncell floats each.
// ---------------------------------------------------------------------------
__global__ void k_add_noise(float* __restrict__ v, int nplanes, int nmem, long long ncell,
                            const double* __restrict__ defl, const double* __restrict__ term)
{
    for (int pl = blockIdx.y; pl < nplanes; pl += gridDim.y) {
        const double d = defl[pl / nmem];
        if (d != d) continue;   // NaN deflation: the layer takes no noise
        const float fd = (float)d;
        const double t = term[pl];
        float* vp = v + (size_t)pl * ncell;
        for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < ncell;
             c += (long long)gridDim.x * blockDim.x)
            vp[c] = __double2float_rn(__dadd_rn((double)__fmul_rn(vp[c], fd), t));
    }
}

enkfg_status run_noise(enkfg_ctx* ctx, float* d_v, int f0, int nf, int nmem, long long ncell, cudaStream_t st)
{
    if (nf <= 0 || ncell <= 0) return ENKFG_OK;
    const int nplanes = nf * nmem;
    const int gx = ncell >= 256 * 64 ? 64 : div_up(ncell, 256);
    dim3 g(gx, nplanes < 65535 ? nplanes : 65535);
    k_add_noise<<<g, 256, 0, st>>>(d_v, nplanes, nmem, ncell, ctx->d_noise + f0,
                                   ctx->d_noise + ctx->noise_nlayer + (size_t)f0 * nmem);
    CKL();
    return ENKFG_OK;
}
