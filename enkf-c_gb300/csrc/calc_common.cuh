// calc_common.cuh -- pieces shared by the FP64 and the mixed-precision
// local-analysis kernels: arguments, neighbour cells, the enumeration of the
// local observations in chunks, the FP64 solve and the output epilogue.
// Reference: calc/transforms.c:1150-1360, calc/calcs.c, common/observations.c:
// 1837-1927.
#pragma once
#include "internal.cuh"
#include "exact.cuh"
#include "linalg.cuh"

#define CALC_NT 256
#define KC_MAX 64
#define LIST_EXTRA (CALC_NT + KC_MAX)
#define NBINS 16

struct CalcArgs {
    int npts, ntypes, ndim, m, md, mode, scheme, want_diag, persistent, kc;
    int nitems;        // queue length (npts, or a sample while autotuning)
    double alpha;
    unsigned long long wait_ns;   // bound on a device wait (mixed path), ns
    int wait_drill;               // the mixed kernel's timeout drill (enkfg_set_wait_drill)
    const TypeIndex* types;
    const long long* bstart;
    const double* sx;
    const double* sy;
    const double* sz;
    const float* sxf;  // FP32 coordinate copies (2-D; null: FP64 search only)
    const float* syf;
    const float* St;
    const float* qscale;   // [2][ENKFG_MAXMEM] mixed path: per-member quantum q and 1/q
    int mpad;
    const double* ss;
    const float* ssf;      // ss rounded to float (mixed path)
    const double* qx;
    const double* qy;
    const double* qz;
    const int* sid;        // observation id at each sorted position
    const CutKey* cut;     // [ntypes][npts] NLOBSMAX cuts (null: no type has a limit)
    const int* order;
    int* qhead;
    const int* counts;
    const int* kc_table;
    float* T;
    float* w;
    double* T64;
    double* w64;
    int* nlobs;
    float* dfs;
    float* srf;
    int* pnlobs;
    float* pdfs;
    float* psrf;
    int* status;
    // batched ETKF eigensolver: with defer set, the transform kernels stop an
    // ETKF point after the tridiagonalisation and save it in slot idx (the
    // point's position in this launch); item0: first point when order is null
    int defer, item0;
    double* eq;        // [slots][m][m] Q of tred2
    double* ed;        // [slots][m] tridiagonal: diagonal
    double* ee;        // [slots][m] and off-diagonal (QL form)
    double* eb;        // [slots][m] S's
    double* eaux;      // [slots][2] local obs count p, tr(S'S)
    float2* emhl;      // [slots][m][m] refined ETKF solve: M also as a float pair (hi + lo exact), upper triangle
};

__host__ __device__ static inline int count_bin(int p)
{
    int b = 0;
    while (b < NBINS - 1 && (1 << (b + 1)) <= p + 1) ++b;
    return b;
}

__device__ __forceinline__ unsigned int cc_spread2(unsigned int v)
{
    v &= 0x0000ffffu;
    v = (v | (v << 8)) & 0x00ff00ffu;
    v = (v | (v << 4)) & 0x0f0f0f0fu;
    v = (v | (v << 2)) & 0x33333333u;
    v = (v | (v << 1)) & 0x55555555u;
    return v;
}

__device__ __forceinline__ unsigned int cc_spread3(unsigned int v)
{
    v &= 0x000003ffu;
    v = (v | (v << 16)) & 0x030000ffu;
    v = (v | (v << 8)) & 0x0300f00fu;
    v = (v | (v << 4)) & 0x030c30c3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

// Morton-numbered buckets of the 3x3 (3x3x3) cells around a query point
__device__ __forceinline__ int calc_neighbours(const TypeIndex& t, int ndim, double qx, double qy, double qz,
                                               long long* b)
{
    double fx = floor((qx - t.x0) * t.inv_cell), fy = floor((qy - t.y0) * t.inv_cell);
    double fz = ndim == 3 ? floor((qz - t.z0) * t.inv_cell) : 0.0;
    int n = 0;
    if (!(fx >= -1.0 && fx <= (double)t.ncx && fy >= -1.0 && fy <= (double)t.ncy)) return 0;
    if (ndim == 3 && !(fz >= -1.0 && fz <= (double)t.ncz)) return 0;
    int cx = (int)fx, cy = (int)fy, cz = (int)fz;
    int zlo = ndim == 3 ? cz - 1 : 0, zhi = ndim == 3 ? cz + 1 : 0;
    for (int z = zlo; z <= zhi; ++z) {
        if (z < 0 || z >= t.ncz) continue;
        for (int y = cy - 1; y <= cy + 1; ++y) {
            if (y < 0 || y >= t.ncy) continue;
            for (int x = cx - 1; x <= cx + 1; ++x) {
                if (x < 0 || x >= t.ncx) continue;
                unsigned int code = (ndim == 2) ? (cc_spread2(x) | (cc_spread2(y) << 1))
                                                : (cc_spread3(x) | (cc_spread3(y) << 1) | (cc_spread3(z) << 2));
                b[n++] = t.bucket_base + (long long)code;
            }
        }
    }
    return n;
}

// per-CTA shared scratch used while enumerating / solving one point
struct PointScratch {
    int* lid;          // [LIST_EXTRA] sorted positions of accepted obs
    double* llc;       // [LIST_EXTRA] their taper coefficients
    int* ictl;         // control ints: [0] list count, [6] queue item, [8..15] warp sums, [16..19] solver
    int* tcount;       // [MAXTYPES] local obs per type
    double* tss;       // [MAXTYPES] per-type sum of squared tapered S
    double* tpd;       // [MAXTYPES] per-type dfs (second pass)
    double* red;       // [CALC_NT/32]
};

// Enumerate the local observations of a point in (type, bucket, position)
// order and hand them to proc.chunk(nc, t) in chunks of kc entries
// (lid/llc[0..nc)); chunks never straddle a type.  Returns the count of
// local observations; per-type counts go to s.tcount if count_types.
// FAST: taper coefficients in FP32, stored as floats in s.llc (mixed path);
// otherwise exact FP64 coefficients (bit-identical to the reference's).
// The exact FP64 membership test for the few candidates whose FP32 squared
// distance falls inside the undecided band.  Not inlined, so that its FP64
// instructions stay off the common path (an if-converted FP64 block issues
// on the 1/64-rate FP64 pipe even for predicated-off lanes).
static __device__ __noinline__ bool exact_in2(double ox, double oy, double qx, double qy, double r2)
{
    return exact::dist2(ox, oy, qx, qy) <= r2;
}

// The NLOBSMAX cut of a candidate the FP32 pre-test accepted: its exact FP64
// squared distance against the point's cut key *ck (not inlined, as
// exact_in2; the key is loaded here, so that the search loop keeps nothing
// of it live).
static __device__ __noinline__ bool exact_cut2(double ox, double oy, double qx, double qy, int id,
                                               const CutKey* ck)
{
    return cut_keeps(exact::dist2(ox, oy, qx, qy), id, *ck);
}

// The same for a candidate whose exact squared distance d2 is at hand.
static __device__ __noinline__ bool keeps_cut(double d2, int id, const CutKey* ck)
{
    return cut_keeps(d2, id, *ck);
}

// SEARCH: 0 exact FP64 distance and FP64 taper (bit-exact coefficients);
// 1 FP64 distance, FP32 taper; 2 FP32 distance with the exact FP64 test only
// inside the undecided band, FP32 taper from the double-float distance (2-D).
template <int SEARCH, class Proc>
__device__ int enumerate_obs(const CalcArgs& a, int pt, int kc, double qx, double qy, double qz,
                             const PointScratch& s, Proc& proc, bool count_types)
{
    constexpr bool FAST = SEARCH > 0;
    float* llcf = reinterpret_cast<float*>(s.llc);
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    int* wsum = s.ictl + 8;
    int total = 0;
    for (int t = 0; t < a.ntypes; ++t) {
        const TypeIndex& ti = a.types[t];
        int tcnt = 0;
        if (ti.pos_end > ti.pos_begin) {
            // NLOBSMAX: the point's cut for this type applies (a point with
            // no more observations in range than the limit has none)
            bool cut_on = false;
            if (a.cut != nullptr && ti.nlobsmax > 0) cut_on = a.cut[(size_t)t * a.npts + pt].d2 <= ti.rmax2;
            long long bk[27];
            int nb = calc_neighbours(ti, a.ndim, qx, qy, qz, bk);
            // FP32 pre-test (SEARCH 2): the query split into hi + lo floats;
            // candidates inside the band [rmax2_lo, rmax2_hi] take the exact
            // FP64 test, which keeps the neighbour sets bit-exact
            const float qxh = (float)qx, qyh = (float)qy;
            const float qxl = (float)(qx - (double)qxh), qyl = (float)(qy - (double)qyh);
            if (tid == 0) s.ictl[0] = 0;
            __syncthreads();
            for (int k = 0; k < nb; ++k) {
                long long b0 = a.bstart[bk[k]], b1 = a.bstart[bk[k] + 1];
                for (long long base = b0; base < b1; base += CALC_NT) {
                    long long p = base + tid;
                    bool in = false;
                    double d2 = 0.0;
                    float d2f = 0.0f, d2l = 0.0f;
                    if constexpr (SEARCH == 2) {
                        bool band = false;
                        if (p < b1) {
                            exact::dist2_df(a.sxf[p], a.syf[p], qxh, qxl, qyh, qyl, d2f, d2l);
                            in = d2f <= ti.rmax2_lo;
                            band = !in && d2f <= ti.rmax2_hi;
                        }
                        if (__any_sync(0xffffffffu, band))
                            if (band) in = exact_in2(a.sx[p], a.sy[p], qx, qy, ti.rmax2);
                        if (cut_on && in)
                            in = exact_cut2(a.sx[p], a.sy[p], qx, qy, a.sid[p], a.cut + (size_t)t * a.npts + pt);
                    } else {
                        if (p < b1) {
                            d2 = a.ndim == 2 ? exact::dist2(a.sx[p], a.sy[p], qx, qy)
                                             : exact::dist3(a.sx[p], a.sy[p], a.sz[p], qx, qy, qz);
                            in = d2 <= ti.rmax2;
                            if (cut_on && in) in = keeps_cut(d2, a.sid[p], a.cut + (size_t)t * a.npts + pt);
                        }
                    }
                    unsigned bal = __ballot_sync(0xffffffffu, in);
                    if (lane == 0) wsum[wid] = __popc(bal);
                    __syncthreads();
                    int before = 0, tot = 0;
#pragma unroll
                    for (int w = 0; w < CALC_NT / 32; ++w) {
                        int c = wsum[w];
                        before += (w < wid) ? c : 0;
                        tot += c;
                    }
                    int n0 = s.ictl[0];
                    if (in) {
                        int pos = n0 + before + __popc(bal & ((1u << lane) - 1));
                        s.lid[pos] = (int)p;
                        if constexpr (SEARCH == 2)
                            llcf[pos] = exact::calclcoeff_df(ti, d2f, d2l);
                        else if constexpr (SEARCH == 1)
                            llcf[pos] = exact::calclcoeff_f(ti.nlocrad, ti.locrad, ti.locweight, d2);
                        else
                            s.llc[pos] = exact::calclcoeff(ti.nlocrad, ti.locrad, ti.locweight, __dsqrt_rn(d2));
                    }
                    __syncthreads();
                    int n = n0 + tot;
                    tcnt += tot;
                    while (n >= kc) {
                        proc.chunk(kc, t);
                        int rest = n - kc;
                        int id = 0;
                        double lc = 0.0;
                        float lcf = 0.0f;
                        if (tid < rest) {
                            id = s.lid[kc + tid];
                            if constexpr (FAST) lcf = llcf[kc + tid];
                            else lc = s.llc[kc + tid];
                        }
                        __syncthreads();
                        if (tid < rest) {
                            s.lid[tid] = id;
                            if constexpr (FAST) llcf[tid] = lcf;
                            else s.llc[tid] = lc;
                        }
                        __syncthreads();
                        n = rest;
                    }
                    if (tid == 0) s.ictl[0] = n;
                    __syncthreads();
                }
            }
            int n = s.ictl[0];
            if (n > 0) proc.chunk(n, t);
            __syncthreads();
        }
        proc.type_end(t);
        if (count_types && tid == 0) s.tcount[t] = tcnt;
        total += tcnt;
        __syncthreads();
    }
    return total;
}

// Second pass for the per-type degrees of freedom (ntypes > 1): for every
// local obs o of type t, s_o' M^-1 s_o, with M^-1 = Q diag(g) Q' (ETKF,
// g != null) or M^-1 = Q (DEnKF/EnOI), accumulated per type.
struct QuadProc {
    const CalcArgs& a;
    const PointScratch& s;
    double* tile;      // [KC_MAX][tld] doubles
    int tld;
    const double* Q;
    const double* g;
    int lda;
    double pd;
    __device__ QuadProc(const CalcArgs& a_, const PointScratch& s_, double* tile_, int tld_, const double* Q_,
                        const double* g_, int lda_)
        : a(a_), s(s_), tile(tile_), tld(tld_), Q(Q_), g(g_), lda(lda_), pd(0.0) {}
    __device__ void chunk(int nc, int t)
    {
        const int tid = threadIdx.x, m = a.m;
        for (int i = tid; i < nc * tld; i += CALC_NT) {
            int o = i / tld, e = i - o * tld;
            tile[i] = (e < m) ? __dmul_rn((double)a.St[(size_t)s.lid[o] * a.mpad + e], s.llc[o]) : 0.0;
        }
        __syncthreads();
        if (tid < m) {
            for (int o = 0; o < nc; ++o) {
                double u = 0.0;
                for (int e = 0; e < m; ++e) u = fma(Q[(size_t)e * lda + tid], tile[o * tld + e], u);
                pd += (g != nullptr) ? u * u * g[tid] : u * tile[o * tld + tid];
            }
        }
        __syncthreads();
    }
    __device__ void type_end(int t)
    {
        double v = la::block_sum<CALC_NT>(pd, s.red);
        if (threadIdx.x == 0) s.tpd[t] = v;
        pd = 0.0;
    }
};

// Output of a point with no local observations (transforms.c:1219-1236)
__device__ inline void store_empty(const CalcArgs& a, int pt)
{
    const int tid = threadIdx.x, m = a.m, md = a.md;
    const size_t tbase = (size_t)pt * md * m;
    if (a.T != nullptr)
        for (int i = tid; i < md * m; i += CALC_NT) {
            int e1 = i / m, e2 = i - e1 * m;
            a.T[tbase + i] = (e1 == e2) ? 1.0f : 0.0f;
            if (a.T64) a.T64[tbase + i] = (e1 == e2) ? 1.0 : 0.0;
        }
    for (int i = tid; i < m; i += CALC_NT) {
        a.w[(size_t)pt * m + i] = 0.0f;
        if (a.w64) a.w64[(size_t)pt * m + i] = 0.0;
    }
    if (a.want_diag && tid == 0) {
        a.nlobs[pt] = 0;
        a.dfs[pt] = 0.0f;
        a.srf[pt] = 0.0f;
        for (int t = 0; t < a.ntypes; ++t) {
            a.pnlobs[(size_t)t * a.npts + pt] = 0;
            a.pdfs[(size_t)t * a.npts + pt] = 0.0f;
            a.psrf[(size_t)t * a.npts + pt] = 0.0f;
        }
    }
}

// ETKF outputs from the eigendecomposition M = Z diag(d) Z' (Z in the columns
// of A): w = Z diag(1/d) Z' b, T = Z diag(d^-1/2) Z' relaxed by alpha and
// cast (calcs.c:300-412, transforms.c:1270-1296).  cs, sn, v: scratch of m
// doubles (cs = d^-1/2 and sn = 1/d on return).  Returns dfs = m - tr(M^-1).
__device__ inline double etkf_outputs(const CalcArgs& a, int pt, const double* A, int lda, const double* d,
                                      const double* b, double* cs, double* sn, double* v, double* red)
{
    const int tid = threadIdx.x, m = a.m, md = a.md;
    const size_t tbase = (size_t)pt * md * m;
    if (tid < m) {
        double lam = d[tid];
        cs[tid] = 1.0 / sqrt(lam);
        sn[tid] = 1.0 / lam;
        double c = 0.0;
        for (int q = 0; q < m; ++q) c = fma(A[q * lda + tid], b[q], c);
        v[tid] = c * sn[tid];
    }
    __syncthreads();
    if (tid < m) {
        double wv = 0.0;
        for (int k = 0; k < m; ++k) wv = fma(A[tid * lda + k], v[k], wv);
        a.w[(size_t)pt * m + tid] = (float)wv;
        if (a.w64) a.w64[(size_t)pt * m + tid] = wv;
    }
    const double dfs = la::block_sum<CALC_NT>(tid < m ? 1.0 - sn[tid] : 0.0, red);
    if (a.mode != ENKFG_MODE_ENOI && a.T != nullptr) {
        for (int i = tid; i < md * m; i += CALC_NT) {
            int e1 = i / m, e2 = i - e1 * m;
            double t = 0.0;
            const double* z1 = A + e1 * lda;
            const double* z2 = A + e2 * lda;
            for (int k = 0; k < m; ++k) t = fma(z1[k] * cs[k], z2[k], t);
            if (e1 == e2) t = (t - 1.0) * a.alpha + 1.0;   // transforms.c:1276-1286
            else t = t * a.alpha;
            a.T[tbase + i] = (float)t;
            if (a.T64) a.T64[tbase + i] = t;
        }
    }
    return dfs;
}

// Diagnostics of a point when there is one observation type
// (transforms.c:1298-1345): nlobs, dfs, srf and their per-type copies.
__device__ inline void diag_single(const CalcArgs& a, int pt, int p, double dfs, double trss)
{
    float dfs_f = (float)dfs;
    if (threadIdx.x == 0) {
        a.nlobs[pt] = p;
        a.dfs[pt] = dfs_f;
        a.srf[pt] = (float)(sqrt(trss / (double)dfs_f) - 1.0);
        a.pnlobs[pt] = p;
        a.pdfs[pt] = dfs_f;
        a.psrf[pt] = (dfs_f > 1.0e-6f) ? (float)(sqrt(trss / (double)dfs_f) - 1.0) : 0.0f;
    }
}

// DEnKF / EnOI outputs from M^-1 in A (calcs.c:279-284): w = M^-1 S's, the
// degrees of freedom m - tr(M^-1), and (DEnKF) T = (I + M^-1) / 2 with the
// relaxation; returns dfs.  Threads of a block of NT.
template <int NT>
__device__ inline double denkf_outputs(const CalcArgs& a, int pt, const double* A, int lda, const double* b,
                                       double* red)
{
    const int tid = threadIdx.x, m = a.m, md = a.md;
    const size_t tbase = (size_t)pt * md * m;
    double dpart = 0.0;
    for (int r = tid; r < m; r += NT) {
        double wv = 0.0;
        for (int k = 0; k < m; ++k) wv = fma(A[r * lda + k], b[k], wv);
        a.w[(size_t)pt * m + r] = (float)wv;
        if (a.w64) a.w64[(size_t)pt * m + r] = wv;
        dpart += 1.0 - A[r * lda + r];
    }
    const double dfs = la::block_sum<NT>(dpart, red);
    if (a.mode != ENKFG_MODE_ENOI && a.T != nullptr && a.T64 == nullptr && a.alpha == 1.0) {
        // no relaxation, float output only: off the diagonal (float)(a / 2)
        // is (float)a / 2 (halving commutes with rounding), so only the
        // diagonal needs FP64 arithmetic
        for (int i = tid; i < md * m; i += NT) {
            int e1 = i / m, e2 = i - e1 * m;
            a.T[tbase + i] = (e1 == e2) ? (float)(0.5 * A[e1 * lda + e2] + 0.5)
                                        : 0.5f * (float)A[e1 * lda + e2];
        }
    } else if (a.mode != ENKFG_MODE_ENOI && a.T != nullptr) {
        for (int i = tid; i < md * m; i += NT) {
            int e1 = i / m, e2 = i - e1 * m;
            double t = 0.5 * A[e1 * lda + e2];
            if (e1 == e2) t += 0.5;
            if (e1 == e2) t = (t - 1.0) * a.alpha + 1.0;
            else t = t * a.alpha;
            a.T[tbase + i] = (float)t;
            if (a.T64) a.T64[tbase + i] = t;
        }
    }
    return dfs;
}

// FP64 solve of one point from M = I + S'S in A (n = m, stride lda) and b =
// S's, then relaxation, float cast and diagnostics.  A is overwritten (by the
// eigenvectors, or by M^-1); tile/tld: FP64 chunk buffer for the per-type
// pass.
__device__ inline void solve_point(const CalcArgs& a, int pt, int slot, int p, int kc, double qx, double qy,
                                   double qz, double* A, int lda, double* b, double trss, double* d, double* e,
                                   double* cs, double* sn, double* v, const PointScratch& s, double* tile, int tld)
{
    const int tid = threadIdx.x, m = a.m;
    const bool need_inv = (a.mode == ENKFG_MODE_ENOI || a.scheme == ENKFG_SCHEME_DENKF);
    int rc = 0;
    double dfs = 0.0;
    const double* Q;
    const double* gq;
    if (a.defer) {
        // batched solve: save the upper triangle of M, S's and the point's
        // count and tr(S'S); the batched inverse (k_inv_finish) or the
        // batched eigensolver (k_tred_batch, k_ql_batch, k_eig_finish) does
        // the rest
        const size_t q0 = (size_t)slot * m * m;
        for (int i = tid; i < m * m; i += CALC_NT) {
            const int r = i / m, c = i - r * m;
            if (c >= r) {
                const double x = A[r * lda + c];
                a.eq[q0 + i] = x;
                if (a.emhl) {
                    const float hi = (float)x;
                    a.emhl[q0 + i] = make_float2(hi, (float)(x - (double)hi));
                }
            }
        }
        if (tid < m) a.eb[(size_t)slot * m + tid] = b[tid];
        if (tid == 0) {
            a.eaux[2 * (size_t)slot] = (double)p;
            a.eaux[2 * (size_t)slot + 1] = trss;
        }
        __syncthreads();
        return;
    }
    if (!need_inv) {
        // ETKF (calcs.c:300-412): T = M^-1/2, w = M^-1 S's
        rc = la::eig_sym<CALC_NT>(A, m, lda, d, e, cs, sn, s.ictl + 16, s.red);
        dfs = etkf_outputs(a, pt, A, lda, d, b, cs, sn, v, s.red);
        Q = A;
        gq = sn;
    } else {
        // DEnKF (calcs.c:279-284) / EnOI: M^-1 in place (symmetric sweep)
        rc = la::spd_inverse<CALC_NT>(A, m, lda, cs, sn, d, s.ictl + 16);
        dfs = denkf_outputs<CALC_NT>(a, pt, A, lda, b, s.red);
        Q = A;
        gq = nullptr;
    }
    if (rc != 0 && tid == 0) a.status[pt] = rc;
    if (a.want_diag) {
        float dfs_f = (float)dfs;
        if (tid == 0) {
            a.nlobs[pt] = p;
            a.dfs[pt] = dfs_f;
            a.srf[pt] = (float)(sqrt(trss / (double)dfs_f) - 1.0);
        }
        if (a.ntypes == 1) {
            diag_single(a, pt, p, dfs, trss);
        } else {
            __syncthreads();
            QuadProc qp(a, s, tile, tld, Q, gq, lda);
            enumerate_obs<0>(a, pt, kc, qx, qy, qz, s, qp, false);
            if (tid < a.ntypes) {
                int t = tid;
                size_t k = (size_t)t * a.npts + pt;
                a.pnlobs[k] = s.tcount[t];
                if (s.tcount[t] == 0) {
                    a.pdfs[k] = 0.0f;
                    a.psrf[k] = 0.0f;
                } else {
                    float pf = (float)s.tpd[t];
                    a.pdfs[k] = pf;
                    a.psrf[k] = ((double)pf > 1.0e-6) ? (float)(sqrt(s.tss[t] / (double)pf) - 1.0) : 0.0f;
                }
            }
        }
    }
    __syncthreads();
}

// next queue item for this CTA (persistent) or the CTA's own point; -1 at end
__device__ __forceinline__ int next_item(const CalcArgs& a, int it, int* ictl)
{
    int idx;
    if (a.persistent) {
        if (threadIdx.x == 0) ictl[6] = atomicAdd(a.qhead, 1);
        __syncthreads();
        idx = ictl[6];
        __syncthreads();
    } else {
        idx = (it == 0) ? (int)blockIdx.x : a.nitems;
    }
    return idx < a.nitems ? idx : -1;
}
