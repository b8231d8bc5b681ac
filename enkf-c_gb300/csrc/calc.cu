// calc.cu -- local-analysis transforms (das_calctransforms, reference
// calc/transforms.c:991-1637, numerics calc/calcs.c).
//
// One CTA computes one local analysis at a time:
//   1. enumerate the observations within range from the spatial index
//      (same membership and taper as obs_findlocal, observations.c:1837),
//      in chunks of kc observations;
//   2. gather each chunk's rows of the standardised S (member-contiguous,
//      sorted by bucket) and innovations, taper them in FP64
//      (transforms.c:1250-1258), and accumulate S'S and S's in FP64
//      registers (upper-triangular register blocks, 16x16 threads);
//   3. solve in FP64 in shared memory with M = I + S'S:
//        ETKF  (calcs.c:300-412): M = Z diag(l) Z'; T = Z diag(l^-1/2) Z',
//              w = Z diag(1/l) Z' S's
//        DEnKF (calcs.c:279-284): M^-1 by Cholesky; T = (I + M^-1) / 2,
//              w = M^-1 S's
//        EnOI  (transforms.c:1260-1262): w only
//      (closed forms of the reference's G/T products, identical in exact
//      arithmetic: G S = I - M^-1, (M + M^1/2)^-1 S'S = I - M^-1/2);
//   4. relaxation to prior T = I + alpha (T - I) and float cast
//      (transforms.c:1270-1296), diagnostics dfs = tr(GS) = m - tr(M^-1),
//      srf, and per obs type pdfs/psrf (transforms.c:1298-1345).
//
// The plain path launches one CTA per point in grid order.  The batched path
// runs a persistent grid that pulls points from a queue sorted by descending
// local-obs count, with the chunk size per count bucket taken from a table
// filled by the autotuner.
#include "internal.cuh"
#include "exact.cuh"
#include "linalg.cuh"

#define CALC_NT 256
#define KC_MAX 64
#define LIST_EXTRA (CALC_NT + KC_MAX)
#define NBINS 16

struct CalcArgs {
    int npts, ntypes, ndim, m, md, mode, scheme, want_diag, persistent, kc;
    double alpha;
    const TypeIndex* types;
    const long long* bstart;
    const double* sx;
    const double* sy;
    const double* sz;
    const float* St;
    int mpad;
    const double* ss;
    const double* qx;
    const double* qy;
    const double* qz;
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
};

__host__ __device__ static inline int count_bin(int p)
{
    int b = 0;
    while (b < NBINS - 1 && (1 << (b + 1)) <= p + 1) ++b;
    return b;
}

__device__ __forceinline__ unsigned int d_spread2(unsigned int v)
{
    v &= 0x0000ffffu;
    v = (v | (v << 8)) & 0x00ff00ffu;
    v = (v | (v << 4)) & 0x0f0f0f0fu;
    v = (v | (v << 2)) & 0x33333333u;
    v = (v | (v << 1)) & 0x55555555u;
    return v;
}

__device__ __forceinline__ unsigned int d_spread3(unsigned int v)
{
    v &= 0x000003ffu;
    v = (v | (v << 16)) & 0x030000ffu;
    v = (v | (v << 8)) & 0x0300f00fu;
    v = (v | (v << 4)) & 0x030c30c3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

__device__ int calc_neighbours(const TypeIndex& t, int ndim, double qx, double qy, double qz, long long* b)
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
                unsigned int code = (ndim == 2) ? (d_spread2(x) | (d_spread2(y) << 1))
                                                : (d_spread3(x) | (d_spread3(y) << 1) | (d_spread3(z) << 2));
                b[n++] = t.bucket_base + (long long)code;
            }
        }
    }
    return n;
}

// shared-memory layout of one CTA
template <int R>
struct CalcSmem {
    static constexpr int MP = 16 * R;       // padded member count
    static constexpr int TLD = MP;          // tile row stride (doubles)
    static constexpr int LDA = MP + 1;      // matrix row stride (doubles)
    static size_t bytes(int need_x)
    {
        size_t s = 0;
        s += (size_t)KC_MAX * TLD * 8;                 // tile
        s += (size_t)LIST_EXTRA * 8;                   // list taper
        s += (size_t)KC_MAX * 8;                       // sloc
        s += (size_t)MP * LDA * 8;                     // A
        if (need_x) s += (size_t)MP * LDA * 8;         // X (Cholesky inverse)
        s += (size_t)6 * MP * 8;                       // b d e cs sn v
        s += (size_t)ENKFG_MAXTYPES * 8 * 2;           // per-type ss, pdfs
        s += (size_t)(CALC_NT / 32) * 8;               // red
        s += (size_t)LIST_EXTRA * 4;                   // list ids
        s += (size_t)ENKFG_MAXTYPES * 4;               // per-type counts
        s += 256;                                      // ints (list count, warp sums, solver control)
        return s;
    }
};

template <int R>
__device__ void process_chunk(const CalcArgs& a, int nc, int t, const int* lid, const double* llc, double* tile,
                              double* sloc, double (&acc)[R][R], double& bacc, double* tss, double* red,
                              bool second_pass, const double* Q, const double* g, double* pd, int lda)
{
    constexpr int MP = 16 * R, TLD = MP;
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    const int m = a.m;
    double ssq = 0.0;
    for (int i = tid; i < nc * MP; i += CALC_NT) {
        int o = i / MP, e = i - o * MP;
        double v = 0.0;
        if (e < m) v = __dmul_rn((double)a.St[(size_t)lid[o] * a.mpad + e], llc[o]);
        tile[o * TLD + e] = v;
        if (a.want_diag && a.ntypes > 1) ssq += v * v;
    }
    if (tid < nc) sloc[tid] = __dmul_rn(a.ss[lid[tid]], llc[tid]);
    __syncthreads();
    if (!second_pass) {
        if (tx >= ty) {
            for (int o = 0; o < nc; ++o) {
                double av[R], bv[R];
#pragma unroll
                for (int i = 0; i < R; ++i) av[i] = tile[o * TLD + ty * R + i];
#pragma unroll
                for (int j = 0; j < R; ++j) bv[j] = tile[o * TLD + tx * R + j];
#pragma unroll
                for (int i = 0; i < R; ++i)
#pragma unroll
                    for (int j = 0; j < R; ++j) acc[i][j] = fma(av[i], bv[j], acc[i][j]);
            }
        }
        if (tid < m)
            for (int o = 0; o < nc; ++o) bacc = fma(tile[o * TLD + tid], sloc[o], bacc);
        if (a.want_diag && a.ntypes > 1) {
            double s = la::block_sum<CALC_NT>(ssq, red);
            if (tid == 0) tss[t] += s;
        }
    } else {
        // quadratic forms s_o' M^-1 s_o for the per-type dfs: thread k
        // accumulates sum_o v_k(o)
        if (tid < m) {
            for (int o = 0; o < nc; ++o) {
                double u = 0.0;
                for (int e = 0; e < m; ++e) u = fma(Q[(size_t)e * lda + tid], tile[o * TLD + e], u);
                *pd += (g != nullptr) ? u * u * g[tid] : u * tile[o * TLD + tid];
            }
        }
    }
    __syncthreads();
}

// Enumerate the local observations of point (qx,qy,qz) and feed them to
// process_chunk in chunks of kc, flushing at each type boundary.  Returns
// the number of local observations; per-type counts go to tcount.
template <int R>
__device__ int enumerate_point(const CalcArgs& a, int kc, double qx, double qy, double qz, int* lid, double* llc,
                               int* ictl, double* tile, double* sloc, double (&acc)[R][R], double& bacc, int* tcount,
                               double* tss, double* red, bool second_pass, const double* Q, const double* g,
                               double* tpd, int lda)
{
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    int* wsum = ictl + 8;   // CALC_NT/32 ints
    int total = 0;
    for (int t = 0; t < a.ntypes; ++t) {
        const TypeIndex& ti = a.types[t];
        int tcnt = 0;
        double pd = 0.0;
        if (ti.pos_end > ti.pos_begin) {
            long long bk[27];
            int nb = calc_neighbours(ti, a.ndim, qx, qy, qz, bk);
            if (tid == 0) ictl[0] = 0;
            __syncthreads();
            for (int k = 0; k < nb; ++k) {
                long long b0 = a.bstart[bk[k]], b1 = a.bstart[bk[k] + 1];
                for (long long base = b0; base < b1; base += CALC_NT) {
                    long long p = base + tid;
                    bool in = false;
                    double d2 = 0.0;
                    if (p < b1) {
                        d2 = a.ndim == 2 ? exact::dist2(a.sx[p], a.sy[p], qx, qy)
                                         : exact::dist3(a.sx[p], a.sy[p], a.sz[p], qx, qy, qz);
                        in = d2 <= ti.rmax2;
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
                    int n0 = ictl[0];
                    if (in) {
                        int pos = n0 + before + __popc(bal & ((1u << lane) - 1));
                        lid[pos] = (int)p;
                        llc[pos] = exact::calclcoeff(ti.nlocrad, ti.locrad, ti.locweight, __dsqrt_rn(d2));
                    }
                    __syncthreads();
                    int n = n0 + tot;
                    tcnt += tot;
                    while (n >= kc) {
                        process_chunk<R>(a, kc, t, lid, llc, tile, sloc, acc, bacc, tss, red, second_pass, Q, g,
                                         &pd, lda);
                        int rest = n - kc;
                        int id = 0;
                        double lc = 0.0;
                        if (tid < rest) {
                            id = lid[kc + tid];
                            lc = llc[kc + tid];
                        }
                        __syncthreads();
                        if (tid < rest) {
                            lid[tid] = id;
                            llc[tid] = lc;
                        }
                        __syncthreads();
                        n = rest;
                    }
                    if (tid == 0) ictl[0] = n;
                    __syncthreads();
                }
            }
            int n = ictl[0];
            if (n > 0)
                process_chunk<R>(a, n, t, lid, llc, tile, sloc, acc, bacc, tss, red, second_pass, Q, g, &pd, lda);
            __syncthreads();
        }
        if (second_pass) {
            double s = la::block_sum<CALC_NT>(pd, red);
            if (tid == 0) tpd[t] = s;
        } else if (tid == 0)
            tcount[t] = tcnt;
        total += tcnt;
        __syncthreads();
    }
    return total;
}

template <int R>
__global__ void __launch_bounds__(CALC_NT) k_transforms(CalcArgs a)
{
    constexpr int MP = 16 * R, TLD = MP, LDA = MP + 1;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    const bool need_x = (a.mode == ENKFG_MODE_ENOI || a.scheme == ENKFG_SCHEME_DENKF);
    // carve shared memory (see CalcSmem::bytes)
    unsigned char* sp = smem_raw;
    double* tile = (double*)sp;       sp += (size_t)KC_MAX * TLD * 8;
    double* llc = (double*)sp;        sp += (size_t)LIST_EXTRA * 8;
    double* sloc = (double*)sp;       sp += (size_t)KC_MAX * 8;
    double* A = (double*)sp;          sp += (size_t)MP * LDA * 8;
    double* X = nullptr;
    if (need_x) { X = (double*)sp;    sp += (size_t)MP * LDA * 8; }
    double* b = (double*)sp;          sp += MP * 8;
    double* d = (double*)sp;          sp += MP * 8;
    double* e = (double*)sp;          sp += MP * 8;
    double* cs = (double*)sp;         sp += MP * 8;
    double* sn = (double*)sp;         sp += MP * 8;
    double* v = (double*)sp;          sp += MP * 8;
    double* tss = (double*)sp;        sp += ENKFG_MAXTYPES * 8;
    double* tpd = (double*)sp;        sp += ENKFG_MAXTYPES * 8;
    double* red = (double*)sp;        sp += (CALC_NT / 32) * 8;
    int* lid = (int*)sp;              sp += LIST_EXTRA * 4;
    int* tcount = (int*)sp;           sp += ENKFG_MAXTYPES * 4;
    int* ictl = (int*)sp;

    const int m = a.m, md = a.md;
    for (int it = 0;; ++it) {
        int idx;
        if (a.persistent) {
            if (tid == 0) ictl[6] = atomicAdd(a.qhead, 1);
            __syncthreads();
            idx = ictl[6];
            __syncthreads();
        } else {
            idx = blockIdx.x;
            if (it > 0) break;
        }
        if (idx >= a.npts) break;
        const int pt = a.order ? a.order[idx] : idx;
        int kc = a.kc;
        if (a.kc_table != nullptr && a.counts != nullptr) kc = a.kc_table[count_bin(a.counts[pt])];
        const double qx = a.qx[pt], qy = a.qy[pt], qz = a.ndim == 3 ? a.qz[pt] : 0.0;

        if (tid < ENKFG_MAXTYPES) {
            tss[tid] = 0.0;
            tpd[tid] = 0.0;
            tcount[tid] = 0;
        }
        __syncthreads();
        double acc[R][R];
#pragma unroll
        for (int i = 0; i < R; ++i)
#pragma unroll
            for (int j = 0; j < R; ++j) acc[i][j] = 0.0;
        double bacc = 0.0;
        int p = enumerate_point<R>(a, kc, qx, qy, qz, lid, llc, ictl, tile, sloc, acc, bacc, tcount, tss, red, false,
                                   nullptr, nullptr, tpd, LDA);

        const size_t tbase = (size_t)pt * md * m;
        if (p == 0) {
            // transforms.c:1219-1236
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
            __syncthreads();
            continue;
        }

        // M = I + S'S
        if (tx >= ty) {
#pragma unroll
            for (int i = 0; i < R; ++i)
#pragma unroll
                for (int j = 0; j < R; ++j) {
                    int r = ty * R + i, c = tx * R + j;
                    if (r < m && c < m) {
                        A[r * LDA + c] = acc[i][j];
                        A[c * LDA + r] = acc[i][j];
                    }
                }
        }
        if (tid < m) b[tid] = bacc;
        __syncthreads();
        double trss = la::block_sum<CALC_NT>(tid < m ? A[tid * LDA + tid] : 0.0, red);
        if (tid < m) A[tid * LDA + tid] += 1.0;
        __syncthreads();

        int rc = 0;
        double dfs = 0.0;
        const double* Q;     // for the per-type pass
        const double* gq;
        if (!need_x) {
            // ---- ETKF ----
            rc = la::eig_sym<CALC_NT>(A, m, LDA, d, e, cs, sn, ictl + 16, red);
            if (tid < m) {
                double lam = d[tid];
                cs[tid] = 1.0 / sqrt(lam);    // T weights
                sn[tid] = 1.0 / lam;          // M^-1 weights
                double c = 0.0;
                for (int q = 0; q < m; ++q) c = fma(A[q * LDA + tid], b[q], c);
                v[tid] = c * sn[tid];
            }
            __syncthreads();
            if (tid < m) {
                double wv = 0.0;
                for (int k = 0; k < m; ++k) wv = fma(A[tid * LDA + k], v[k], wv);
                a.w[(size_t)pt * m + tid] = (float)wv;
                if (a.w64) a.w64[(size_t)pt * m + tid] = wv;
            }
            dfs = la::block_sum<CALC_NT>(tid < m ? 1.0 - sn[tid] : 0.0, red);
            if (a.mode != ENKFG_MODE_ENOI && a.T != nullptr) {
                for (int i = tid; i < md * m; i += CALC_NT) {
                    int e1 = i / m, e2 = i - e1 * m;
                    double t = 0.0;
                    const double* z1 = A + e1 * LDA;
                    const double* z2 = A + e2 * LDA;
                    for (int k = 0; k < m; ++k) t = fma(z1[k] * cs[k], z2[k], t);
                    // relaxation to prior (transforms.c:1276-1286)
                    if (e1 == e2) t = (t - 1.0) * a.alpha + 1.0;
                    else t = t * a.alpha;
                    a.T[tbase + i] = (float)t;
                    if (a.T64) a.T64[tbase + i] = t;
                }
            }
            Q = A;
            gq = sn;
        } else {
            // ---- DEnKF / EnOI ----
            rc = la::chol_inverse<CALC_NT>(A, X, m, LDA, ictl + 16);
            if (tid < m) {
                double wv = 0.0;
                for (int k = 0; k < m; ++k) wv = fma(X[tid * LDA + k], b[k], wv);
                a.w[(size_t)pt * m + tid] = (float)wv;
                if (a.w64) a.w64[(size_t)pt * m + tid] = wv;
            }
            dfs = la::block_sum<CALC_NT>(tid < m ? 1.0 - X[tid * LDA + tid] : 0.0, red);
            if (a.mode != ENKFG_MODE_ENOI && a.T != nullptr) {
                for (int i = tid; i < md * m; i += CALC_NT) {
                    int e1 = i / m, e2 = i - e1 * m;
                    double t = 0.5 * X[e1 * LDA + e2];
                    if (e1 == e2) t += 0.5;
                    if (e1 == e2) t = (t - 1.0) * a.alpha + 1.0;
                    else t = t * a.alpha;
                    a.T[tbase + i] = (float)t;
                    if (a.T64) a.T64[tbase + i] = t;
                }
            }
            Q = X;
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
                if (tid == 0) {
                    a.pnlobs[pt] = p;
                    a.pdfs[pt] = dfs_f;
                    a.psrf[pt] = (dfs_f > 1.0e-6f) ? (float)(sqrt(trss / (double)dfs_f) - 1.0) : 0.0f;
                }
            } else {
                enumerate_point<R>(a, kc, qx, qy, qz, lid, llc, ictl, tile, sloc, acc, bacc, tcount, tss, red, true,
                                   Q, gq, tpd, LDA);
                if (tid < a.ntypes) {
                    int t = tid;
                    size_t k = (size_t)t * a.npts + pt;
                    a.pnlobs[k] = tcount[t];
                    if (tcount[t] == 0) {
                        a.pdfs[k] = 0.0f;
                        a.psrf[k] = 0.0f;
                    } else {
                        float pf = (float)tpd[t];
                        a.pdfs[k] = pf;
                        a.psrf[k] = ((double)pf > 1.0e-6) ? (float)(sqrt(tss[t] / (double)pf) - 1.0) : 0.0f;
                    }
                }
            }
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// size-sorted work queue: counting sort of points by descending count bin
// ---------------------------------------------------------------------------
__global__ void k_bin_hist(int n, const int* __restrict__ counts, int* __restrict__ hist)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) atomicAdd(&hist[NBINS - 1 - count_bin(counts[i])], 1);
}

__global__ void k_bin_scan(int* hist)
{
    if (threadIdx.x == 0) {
        int acc = 0;
        for (int b = 0; b < NBINS; ++b) {
            int v = hist[b];
            hist[b] = acc;
            acc += v;
        }
    }
}

__global__ void k_bin_scatter(int n, const int* __restrict__ counts, int* __restrict__ hist, int* __restrict__ order)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) order[atomicAdd(&hist[NBINS - 1 - count_bin(counts[i])], 1)] = i;
}

template <int R>
static enkfg_status launch_R(enkfg_ctx* ctx, CalcArgs& a, cudaStream_t st)
{
    bool need_x = (a.mode == ENKFG_MODE_ENOI || a.scheme == ENKFG_SCHEME_DENKF);
    size_t smem = CalcSmem<R>::bytes(need_x);
    if (smem > 227 * 1024) {
        set_err(ctx, "nmem = %d needs %zu bytes of shared memory for this scheme", a.m, smem);
        return ENKFG_EUNSUPPORTED;
    }
    CK(cudaFuncSetAttribute(k_transforms<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int grid = a.npts;
    if (a.persistent) {
        int per_sm = 0, nsm = 0;
        CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_transforms<R>, CALC_NT, smem));
        CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, ctx->device));
        if (per_sm < 1) per_sm = 1;
        grid = per_sm * nsm;
        if (grid > a.npts) grid = a.npts;
    }
    if (grid < 1) return ENKFG_OK;
    k_transforms<R><<<grid, CALC_NT, smem, st>>>(a);
    CKL();
    return ENKFG_OK;
}

enkfg_status run_transforms(enkfg_ctx* ctx, const enkfg_calc_params* p, cudaStream_t st)
{
    enkfg_status s;
    int npts = ctx->nj * ctx->ni;
    int m = ctx->nmem, md = ctx->nmem_dyn;
    bool enkf = (p->mode == ENKFG_MODE_ENKF || p->mode == ENKFG_MODE_HYBRID);
    if (p->precision != ENKFG_PREC_FP64) {
        set_err(ctx, "mixed-precision transforms are not available in this build");
        return ENKFG_EUNSUPPORTED;
    }
    if (m > 144) {
        set_err(ctx, "nmem = %d above the supported maximum 144", m);
        return ENKFG_EUNSUPPORTED;
    }
    cudaEventRecord(ctx->ev[0], st);
    if (!ctx->index_valid && (s = build_index(ctx, st))) return s;
    if (!ctx->gather_valid && (s = build_gather(ctx, st))) return s;
    cudaEventRecord(ctx->ev[1], st);

    // outputs
    size_t nT = enkf ? (size_t)npts * md * m : 1;
    if ((s = ensure(ctx, &ctx->d_T, &ctx->T_cap, nT))) return s;
    if ((s = ensure(ctx, &ctx->d_w, &ctx->w_cap, (size_t)npts * m))) return s;
    if ((s = ensure(ctx, &ctx->d_T64, &ctx->T64_cap, nT))) return s;
    if ((s = ensure(ctx, &ctx->d_w64, &ctx->w64_cap, (size_t)npts * m))) return s;
    if ((s = ensure(ctx, &ctx->d_nlobs, &ctx->nlobs_cap, (size_t)npts))) return s;
    if ((s = ensure(ctx, &ctx->d_dfs, &ctx->dfs_cap, (size_t)npts))) return s;
    if ((s = ensure(ctx, &ctx->d_srf, &ctx->srf_cap, (size_t)npts))) return s;
    size_t pn = (size_t)npts * ctx->ntypes;
    if ((s = ensure(ctx, &ctx->d_pnlobs, &ctx->pnlobs_cap, pn))) return s;
    if ((s = ensure(ctx, &ctx->d_pdfs, &ctx->pdfs_cap, pn))) return s;
    if ((s = ensure(ctx, &ctx->d_psrf, &ctx->psrf_cap, pn))) return s;
    if ((s = ensure(ctx, &ctx->d_counts, &ctx->counts_cap, (size_t)npts))) return s;
    if ((s = ensure(ctx, &ctx->d_order, &ctx->order_cap, (size_t)npts))) return s;
    if ((s = ensure(ctx, &ctx->d_status_pt, &ctx->status_cap, (size_t)npts))) return s;
    CK(cudaMemsetAsync(ctx->d_status_pt, 0, (size_t)npts * sizeof(int), st));

    CalcArgs a;
    memset(&a, 0, sizeof(a));
    a.npts = npts;
    a.ntypes = ctx->ntypes;
    a.ndim = ctx->geographic ? 3 : 2;
    a.m = m;
    a.md = md;
    a.mode = p->mode;
    a.scheme = p->scheme;
    a.want_diag = p->want_diag ? 1 : 0;
    a.alpha = p->alpha;
    a.kc = 32;
    a.types = ctx->d_types;
    a.bstart = ctx->d_bstart;
    a.sx = ctx->d_sx;
    a.sy = ctx->d_sy;
    a.sz = ctx->d_sz;
    a.St = ctx->d_St;
    a.mpad = ctx->mpad;
    a.ss = ctx->d_ss;
    a.qx = ctx->d_qx;
    a.qy = ctx->d_qy;
    a.qz = ctx->d_qz;
    a.T = enkf ? ctx->d_T : nullptr;
    a.w = ctx->d_w;
    a.T64 = enkf ? ctx->d_T64 : nullptr;
    a.w64 = ctx->d_w64;
    a.nlobs = ctx->d_nlobs;
    a.dfs = ctx->d_dfs;
    a.srf = ctx->d_srf;
    a.pnlobs = ctx->d_pnlobs;
    a.pdfs = ctx->d_pdfs;
    a.psrf = ctx->d_psrf;
    a.status = ctx->d_status_pt;

    if (p->path == ENKFG_PATH_BATCHED) {
        // size-sorted queue
        if ((s = count_local(ctx, ctx->d_counts, nullptr, st))) return s;
        int* hist = ctx->d_qhead + 2;
        CK(cudaMemsetAsync(ctx->d_qhead, 0, (2 + NBINS) * sizeof(int), st));
        k_bin_hist<<<div_up(npts, 256), 256, 0, st>>>(npts, ctx->d_counts, hist);
        CKL();
        k_bin_scan<<<1, 32, 0, st>>>(hist);
        CKL();
        k_bin_scatter<<<div_up(npts, 256), 256, 0, st>>>(npts, ctx->d_counts, hist, ctx->d_order);
        CKL();
        a.persistent = 1;
        a.order = ctx->d_order;
        a.qhead = ctx->d_qhead;
        a.counts = ctx->d_counts;
        a.kc_table = ctx->d_qhead + 2 + NBINS;   // filled by the tuner (defaults below)
        static const int kc_default[NBINS] = { 8, 8, 8, 8, 16, 16, 32, 32, 32, 64, 64, 64, 64, 64, 64, 64 };
        CK(cudaMemcpyAsync(ctx->d_qhead + 2 + NBINS, kc_default, sizeof(kc_default), cudaMemcpyHostToDevice, st));
        CK(cudaMemsetAsync(ctx->d_qhead, 0, sizeof(int), st));
    }
    cudaEventRecord(ctx->ev[2], st);
    if (m <= 32) s = launch_R<2>(ctx, a, st);
    else if (m <= 48) s = launch_R<3>(ctx, a, st);
    else if (m <= 64) s = launch_R<4>(ctx, a, st);
    else if (m <= 96) s = launch_R<6>(ctx, a, st);
    else s = launch_R<9>(ctx, a, st);
    if (s) return s;
    cudaEventRecord(ctx->ev[3], st);
    ctx->t_mode = p->mode;
    ctx->t_nmem = m;
    ctx->t_ndyn = md;
    ctx->t_valid = true;
    return ENKFG_OK;
}
