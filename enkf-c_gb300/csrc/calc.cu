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
// calc_mixed.cu holds the mixed-precision variant of step 2 (S'S on the
// tensor cores).  The plain path launches one CTA per point in grid order.  The batched path
// runs a persistent grid that pulls points from a queue sorted by descending
// local-obs count, with the chunk size per count bucket taken from a table
// filled by the autotuner.
#include "calc_common.cuh"

// shared-memory layout of the FP64 kernel
template <int R>
struct CalcSmem {
    static constexpr int MP = 16 * R;       // padded member count
    static constexpr int TLD = MP;          // tile row stride (doubles)
    static constexpr int LDA = MP + 1;      // matrix row stride (doubles)
    // observations per chunk at most: KC_MAX, but 32 for the largest
    // ensembles, whose FP64 M (144 x 145 doubles) leaves no room for more
    static constexpr int KC = (R >= 9) ? 32 : KC_MAX;
    static size_t bytes()
    {
        size_t s = 0;
        s += (size_t)KC * TLD * 8;                     // tile
        s += (size_t)LIST_EXTRA * 8;                   // list taper
        s += (size_t)KC * 8;                           // sloc
        s += (size_t)MP * LDA * 8;                     // A
        s += (size_t)6 * MP * 8;                       // b d e cs sn v
        s += (size_t)ENKFG_MAXTYPES * 8 * 2;           // per-type ss, pdfs
        s += (size_t)(CALC_NT / 32) * 8;               // red
        s += (size_t)LIST_EXTRA * 4;                   // list ids
        s += (size_t)ENKFG_MAXTYPES * 4;               // per-type counts
        s += 256;                                      // control ints
        return s;
    }
};

// FP64 accumulation of S'S (upper-triangular R x R register blocks on a
// 16 x 16 thread grid) and S's over the chunks of one point
template <int R>
struct GramProc64 {
    const CalcArgs& a;
    const PointScratch& s;
    double* tile;
    double* sloc;
    double acc[R][R];
    double bacc;
    __device__ __forceinline__ GramProc64(const CalcArgs& a_, const PointScratch& s_, double* tile_, double* sloc_)
        : a(a_), s(s_), tile(tile_), sloc(sloc_), bacc(0.0)
    {
#pragma unroll
        for (int i = 0; i < R; ++i)
#pragma unroll
            for (int j = 0; j < R; ++j) acc[i][j] = 0.0;
    }
    __device__ __forceinline__ void chunk(int nc, int t)
    {
        constexpr int MP = 16 * R, TLD = MP;
        const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
        const int m = a.m;
        const bool tsum = a.want_diag && a.ntypes > 1;
        double ssq = 0.0;
        for (int i = tid; i < nc * MP; i += CALC_NT) {
            int o = i / MP, e = i - o * MP;
            double v = 0.0;
            if (e < m) v = __dmul_rn((double)a.St[(size_t)s.lid[o] * a.mpad + e], s.llc[o]);   // transforms.c:1250-1254
            tile[o * TLD + e] = v;
            if (tsum) ssq += v * v;
        }
        if (tid < nc) sloc[tid] = __dmul_rn(a.ss[s.lid[tid]], s.llc[tid]);                  // transforms.c:1255-1256
        __syncthreads();
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
        if (tsum) {
            double v = la::block_sum<CALC_NT>(ssq, s.red);
            if (tid == 0) s.tss[t] += v;
        }
        __syncthreads();
    }
    __device__ __forceinline__ void type_end(int) {}
};

template <int R>
__global__ void __launch_bounds__(CALC_NT) k_transforms(CalcArgs a)
{
    constexpr int MP = 16 * R, TLD = MP, LDA = MP + 1, KC = CalcSmem<R>::KC;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    unsigned char* sp = smem_raw;
    double* tile = (double*)sp;       sp += (size_t)KC * TLD * 8;
    double* llc = (double*)sp;        sp += (size_t)LIST_EXTRA * 8;
    double* sloc = (double*)sp;       sp += (size_t)KC * 8;
    double* A = (double*)sp;          sp += (size_t)MP * LDA * 8;
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
    const PointScratch s{ lid, llc, ictl, tcount, tss, tpd, red };
    const int m = a.m;

    for (int it = 0;; ++it) {
        const int idx = next_item(a, it, ictl);
        if (idx < 0) break;
        const int pt = a.order ? a.order[idx] : a.item0 + idx;
        int kc = a.kc;
        if (a.kc_table != nullptr && a.counts != nullptr) kc = a.kc_table[count_bin(a.counts[pt])];
        if (kc > KC) kc = KC;
        const double qx = a.qx[pt], qy = a.qy[pt], qz = a.ndim == 3 ? a.qz[pt] : 0.0;
        if (tid < ENKFG_MAXTYPES) {
            tss[tid] = 0.0;
            tpd[tid] = 0.0;
            tcount[tid] = 0;
        }
        __syncthreads();
        GramProc64<R> proc(a, s, tile, sloc);
        const int p = enumerate_obs<0>(a, pt, kc, qx, qy, qz, s, proc, true);
        if (p == 0) {
            store_empty(a, pt);
            if (a.defer && tid == 0) a.eaux[2 * (size_t)idx] = 0.0;
            __syncthreads();
            continue;
        }
        // M = I + S'S (calcs.c:315-329)
        if (tx >= ty) {
#pragma unroll
            for (int i = 0; i < R; ++i)
#pragma unroll
                for (int j = 0; j < R; ++j) {
                    int r = ty * R + i, c = tx * R + j;
                    if (r < m && c < m) {
                        A[r * LDA + c] = proc.acc[i][j];
                        A[c * LDA + r] = proc.acc[i][j];
                    }
                }
        }
        if (tid < m) b[tid] = proc.bacc;
        __syncthreads();
        const double trss = la::block_sum<CALC_NT>(tid < m ? A[tid * LDA + tid] : 0.0, red);
        if (tid < m) A[tid * LDA + tid] += 1.0;
        __syncthreads();
        solve_point(a, pt, idx, p, kc, qx, qy, qz, A, LDA, b, trss, d, e, cs, sn, v, s, tile, TLD);
    }
}

// ---------------------------------------------------------------------------
// size-sorted work queue: a stable counting sort of the points by descending
// local-obs count bin.  Within a bin the grid order is kept, so consecutive
// queue items stay spatially close and share their observations in L2.
// ---------------------------------------------------------------------------
#define QS_T 1024

__global__ void k_queue_rank(int n, const int* __restrict__ counts, int* __restrict__ rank,
                             int* __restrict__ blkcnt)
{
    __shared__ int wcnt[QS_T / 32][NBINS];
    const int i = blockIdx.x * QS_T + threadIdx.x, lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int b = (i < n) ? NBINS - 1 - count_bin(counts[i]) : NBINS;   // descending count
    for (int k = threadIdx.x; k < (QS_T / 32) * NBINS; k += QS_T) (&wcnt[0][0])[k] = 0;
    __syncthreads();
    const unsigned same = __match_any_sync(0xffffffffu, b);
    const int r_in_warp = __popc(same & ((1u << lane) - 1));
    if (b < NBINS && r_in_warp == 0) wcnt[wid][b] = __popc(same);
    __syncthreads();
    if (b < NBINS) {
        int before = 0;
        for (int w = 0; w < wid; ++w) before += wcnt[w][b];
        rank[i] = before + r_in_warp;
    }
    if (threadIdx.x < NBINS) {
        int t = 0;
        for (int w = 0; w < QS_T / 32; ++w) t += wcnt[w][threadIdx.x];
        blkcnt[blockIdx.x * NBINS + threadIdx.x] = t;
    }
}

// blkcnt [nblk][NBINS] -> exclusive offsets of (block, bin): segments of
// bps blocks in turn, bin-major within a segment, so that the queue holds
// each segment's points (sorted by bin) in the segment's own range
__global__ void k_queue_offsets(int nblk, int bps, int* blkcnt)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    int acc = 0;
    for (int k0 = 0; k0 < nblk; k0 += bps) {
        const int k1 = (k0 + bps < nblk) ? k0 + bps : nblk;
        for (int b = 0; b < NBINS; ++b)
            for (int k = k0; k < k1; ++k) {
                int v = blkcnt[k * NBINS + b];
                blkcnt[k * NBINS + b] = acc;
                acc += v;
            }
    }
}

__global__ void k_queue_scatter(int n, const int* __restrict__ counts, const int* __restrict__ rank,
                                const int* __restrict__ blkoff, int* __restrict__ order)
{
    const int i = blockIdx.x * QS_T + threadIdx.x;
    if (i >= n) return;
    const int b = NBINS - 1 - count_bin(counts[i]);
    order[blkoff[blockIdx.x * NBINS + b] + rank[i]] = i;
}

// seg: points per segment (a multiple of QS_T; 0: one segment)
enkfg_status build_queue(enkfg_ctx* ctx, int npts, int seg, cudaStream_t st)
{
    enkfg_status s;
    const int nblk = div_up(npts, QS_T);
    size_t need = (size_t)npts + (size_t)nblk * NBINS;
    // the scratch capacity is kept in bytes (scan_counts shares the buffer)
    if ((s = ensure(ctx, (char**)&ctx->d_scratch, &ctx->scratch_cap, need * sizeof(int)))) return s;
    int* rank = (int*)ctx->d_scratch;
    int* blk = rank + npts;
    k_queue_rank<<<nblk, QS_T, 0, st>>>(npts, ctx->d_counts, rank, blk);
    CKL();
    k_queue_offsets<<<1, 32, 0, st>>>(nblk, seg > 0 ? seg / QS_T : nblk, blk);
    CKL();
    k_queue_scatter<<<nblk, QS_T, 0, st>>>(npts, ctx->d_counts, rank, blk, ctx->d_order);
    CKL();
    return ENKFG_OK;
}

enkfg_status resident_ctas(enkfg_ctx* ctx, const void* fn, int nt, size_t dsmem, int* per_sm, int* carveout)
{
    cudaFuncAttributes fa;
    int smem_sm = 0, reserved = 0, regs_sm = 0, thr_sm = 0, blk_sm = 0;
    CK(cudaFuncGetAttributes(&fa, fn));
    CK(cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, ctx->device));
    CK(cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, ctx->device));
    CK(cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, ctx->device));
    CK(cudaDeviceGetAttribute(&thr_sm, cudaDevAttrMaxThreadsPerMultiProcessor, ctx->device));
    CK(cudaDeviceGetAttribute(&blk_sm, cudaDevAttrMaxBlocksPerMultiprocessor, ctx->device));
    const size_t per_blk = dsmem + fa.sharedSizeBytes + (size_t)reserved;
    int n = per_blk > 0 ? (int)((size_t)smem_sm / per_blk) : blk_sm;
    const int warps = (nt + 31) / 32;
    const int warp_regs = ((fa.numRegs * 32 + 255) / 256) * 256;   // allocation unit: 256 registers a warp
    if (warp_regs > 0 && regs_sm / (warp_regs * warps) < n) n = regs_sm / (warp_regs * warps);
    if (thr_sm / (warps * 32) < n) n = thr_sm / (warps * 32);
    if (blk_sm < n) n = blk_sm;
    *per_sm = n < 1 ? 1 : n;
    const size_t need = (size_t)*per_sm * per_blk;
    int pct = smem_sm > 0 ? (int)((need * 100 + (size_t)smem_sm - 1) / (size_t)smem_sm) : 100;
    *carveout = pct > 100 ? 100 : pct;
    return ENKFG_OK;
}

template <int R>
static enkfg_status launch_R(enkfg_ctx* ctx, CalcArgs& a, cudaStream_t st)
{
    size_t smem = CalcSmem<R>::bytes();
    if (smem > 227 * 1024) {
        set_err(ctx, "nmem = %d needs %zu bytes of shared memory for this scheme", a.m, smem);
        return ENKFG_EUNSUPPORTED;
    }
    CK(cudaFuncSetAttribute(k_transforms<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    // the residency count is computed rather than taken from the occupancy
    // query, which reports one CTA per SM for these kernels where two run;
    // the carveout asks for just the shared memory those CTAs need
    int per_sm = 0, carve = 100;
    enkfg_status s = resident_ctas(ctx, (const void*)k_transforms<R>, CALC_NT, smem, &per_sm, &carve);
    if (s) return s;
    CK(cudaFuncSetAttribute(k_transforms<R>, cudaFuncAttributePreferredSharedMemoryCarveout, carve));
    int grid = a.nitems;
    if (a.persistent) {
        int nsm = 0;
        CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, ctx->device));
        grid = per_sm * nsm;
        if (grid > a.nitems) grid = a.nitems;
    }
    if (grid < 1) return ENKFG_OK;
    k_transforms<R><<<grid, CALC_NT, smem, st>>>(a);
    CKL();
    return ENKFG_OK;
}

static enkfg_status dispatch(enkfg_ctx* ctx, CalcArgs& a, int precision, cudaStream_t st)
{
    const int m = a.m;
    if (precision == ENKFG_PREC_MIXED) return launch_mixed(ctx, a, st);
    if (m <= 32) return launch_R<2>(ctx, a, st);
    if (m <= 48) return launch_R<3>(ctx, a, st);
    if (m <= 64) return launch_R<4>(ctx, a, st);
    if (m <= 96) return launch_R<6>(ctx, a, st);
    return launch_R<9>(ctx, a, st);
}

// Autotuner: for every local-obs count bin that holds points, time the
// persistent kernel on (up to) TUNE_SAMPLE of that bin's points -- taken from
// the middle of the bin's stretch of the queue, so spatially contiguous --
// with each candidate chunk size, and keep the fastest.  The table lives in
// the context and is reused by later batched calls (enkfg_autotune_reset
// drops it).
#define TUNE_SAMPLE 1536
static enkfg_status autotune(enkfg_ctx* ctx, CalcArgs a, int precision, cudaStream_t st)
{
    const int npts = a.npts;
    int* order = (int*)malloc((size_t)npts * sizeof(int));
    int* counts = (int*)malloc((size_t)npts * sizeof(int));
    if (!order || !counts) {
        free(order);
        free(counts);
        return ENKFG_ENOMEM;
    }
    cudaMemcpyAsync(order, ctx->d_order, (size_t)npts * sizeof(int), cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(counts, ctx->d_counts, (size_t)npts * sizeof(int), cudaMemcpyDeviceToHost, st);
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        free(order);
        free(counts);
        return cuda_fail(ctx, e, "autotune copy", __LINE__);
    }
    // the mixed kernel's rounds are powers of two (8, 16 or 32 observations)
    static const int cand64[4] = { 8, 16, 32, 64 };
    static const int candmx[3] = { 8, 16, 32 };
    const int* cand = precision == ENKFG_PREC_MIXED ? candmx : cand64;
    const int ncand = precision == ENKFG_PREC_MIXED ? 3 : 4;
    int table[NBINS];
    for (int b = 0; b < NBINS; ++b) table[b] = precision == ENKFG_PREC_MIXED ? 32 : (b < 4 ? 8 : b < 6 ? 16 : b < 9 ? 32 : 64);
    int* kct = ctx->d_qhead + 2 + NBINS;
    enkfg_status s = ENKFG_OK;
    bool done[NBINS] = {};   // the queue repeats the bins once per segment: tune each once
    int pos = 0;
    while (pos < npts && s == ENKFG_OK) {
        const int bin = count_bin(counts[order[pos]]);
        int end = pos;
        while (end < npts && count_bin(counts[order[end]]) == bin) ++end;
        const int len = end - pos;
        const int take = len < TUNE_SAMPLE ? len : TUNE_SAMPLE;
        const int first = pos + (len - take) / 2;
        if (take >= 64 && bin >= 2 && !done[bin]) {
            done[bin] = true;
            float best = 1e30f;
            for (int k = 0; k < ncand; ++k) {
                int tab[NBINS];
                for (int q = 0; q < NBINS; ++q) tab[q] = cand[k];
                cudaMemcpyAsync(kct, tab, sizeof(tab), cudaMemcpyHostToDevice, st);
                CalcArgs t = a;
                t.order = ctx->d_order + first;
                t.nitems = take;
                float ms = 0.0f;
                for (int rep = 0; rep < 2; ++rep) {       // first repetition warms the caches
                    cudaMemsetAsync(ctx->d_qhead, 0, sizeof(int), st);
                    cudaEventRecord(ctx->ev[6], st);
                    if ((s = dispatch(ctx, t, precision, st))) break;
                    cudaEventRecord(ctx->ev[7], st);
                    cudaEventSynchronize(ctx->ev[7]);
                    cudaEventElapsedTime(&ms, ctx->ev[6], ctx->ev[7]);
                }
                if (s) break;
                if (ms < best) {
                    best = ms;
                    table[bin] = cand[k];
                }
            }
        }
        pos = end;
    }
    free(order);
    free(counts);
    if (s) return s;
    CK(cudaMemcpyAsync(kct, table, sizeof(table), cudaMemcpyHostToDevice, st));
    CK(cudaStreamSynchronize(st));
    memcpy(ctx->kc_table, table, sizeof(table));
    ctx->kc_tuned = true;
    ctx->kc_loaded = 3;
    ctx->kc_tuned_prec = precision;
    return ENKFG_OK;
}

// ---------------------------------------------------------------------------
// batched ETKF eigensolver.  The QL iteration of tql2 is a chain of dependent
// FP64 operations on the tridiagonal alone; run inside the point's CTA it
// leaves the SM idle (GB300 issues FP64 at 1/64 of the FP32 rate, so every
// link costs tens of cycles).  Here the transform kernels stop an ETKF point
// after tred2 (saving Q, the tridiagonal and S's), k_ql_batch runs the QL
// chains with one thread per point, logging the rotations, and k_eig_finish
// replays the rotations onto Q (rows in parallel) and forms T, w and the
// diagnostics.  A point whose log would overflow, or whose QL does not
// converge in the chain, takes tql2 in k_eig_finish instead.
// ---------------------------------------------------------------------------
#define QLB_T 32

__global__ void __launch_bounds__(QLB_T) k_ql_batch(int nslots, int m, const double* __restrict__ eaux,
                                                    const double* __restrict__ ed, const double* __restrict__ ee,
                                                    double* __restrict__ eval, double2* __restrict__ rot, int rcap,
                                                    int2* __restrict__ hdr, int hcap, int* __restrict__ nh)
{
    extern __shared__ double qsm[];   // [2][m][QLB_T]: one column of d and of e per thread
    const int lane = threadIdx.x;
    const int slot = blockIdx.x * QLB_T + lane;
    if (slot >= nslots || !(eaux[2 * (size_t)slot] > 0.0)) return;   // no barrier below
    double* dcol = qsm + lane;
    double* ecol = qsm + (size_t)m * QLB_T + lane;
    for (int i = 0; i < m; ++i) {
        dcol[i * QLB_T] = ed[(size_t)slot * m + i];
        ecol[i * QLB_T] = ee[(size_t)slot * m + i];
    }
    int n = 0;
    const int stt = la::ql_chain(dcol, ecol, m, QLB_T, rot + (size_t)slot * rcap, rcap, hdr + (size_t)slot * hcap,
                                 hcap, &n);
    nh[slot] = stt == 0 ? n : -stt;
    for (int i = 0; i < m; ++i) eval[(size_t)slot * m + i] = dcol[i * QLB_T];
}

__global__ void __launch_bounds__(CALC_NT) k_eig_finish(CalcArgs a, const double* __restrict__ eval,
                                                        const double2* __restrict__ rot, int rcap,
                                                        const int2* __restrict__ hdr, int hcap,
                                                        const int* __restrict__ nh)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int m = a.m, lda = (m % 2 == 0) ? m + 1 : m + 2;
    const int tid = threadIdx.x, slot = blockIdx.x;
    double* A = (double*)smem_raw;
    double* d = A + (size_t)m * lda;
    double* e = d + m;
    double* b = e + m;
    double* cs = b + m;
    double* sn = cs + m;
    double* v = sn + m;
    double* red = v + m;
    int* ctl = (int*)(red + CALC_NT / 32);
    const double pd = a.eaux[2 * (size_t)slot];
    if (!(pd > 0.0)) return;   // empty point: written by the transform kernel
    const int pt = a.order ? a.order[slot] : a.item0 + slot;
    const double trss = a.eaux[2 * (size_t)slot + 1];
    const int stt = nh[slot];
    for (int i = tid; i < m * m; i += CALC_NT) {
        const int r = i / m, c = i - r * m;
        A[r * lda + c] = a.eq[(size_t)slot * m * m + i];
    }
    for (int i = tid; i < m; i += CALC_NT) {
        b[i] = a.eb[(size_t)slot * m + i];
        d[i] = stt >= 0 ? eval[(size_t)slot * m + i] : a.ed[(size_t)slot * m + i];
        e[i] = a.ee[(size_t)slot * m + i];
    }
    __syncthreads();
    int rc = 0;
    if (stt >= 0) la::ql_replay<CALC_NT>(A, m, lda, rot + (size_t)slot * rcap, hdr + (size_t)slot * hcap, stt);
    else rc = la::tql2<CALC_NT>(A, m, lda, d, e, cs, sn, ctl);
    const double dfs = etkf_outputs(a, pt, A, lda, d, b, cs, sn, v, red);
    if (rc != 0 && tid == 0) a.status[pt] = rc;
    if (a.want_diag) diag_single(a, pt, (int)pd, dfs, trss);
}

// Batched DEnKF / EnOI solve: the transform kernels save M (upper triangle)
// and S's per slot; one CTA of INV_NT threads per point inverts M with the
// symmetric sweep and forms w, dfs and T.  Inside the transform kernel the
// sweep leaves the FP64 units idle between pivots (barriers, the pivot's
// reciprocal); here a dozen points per SM keep them busy.
#define INV_NT 128

__global__ void __launch_bounds__(INV_NT) k_inv_finish(CalcArgs a)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int m = a.m, lda = (m % 2 == 0) ? m + 1 : m + 2;
    const int tid = threadIdx.x, slot = blockIdx.x;
    double* A = (double*)smem_raw;
    double* b = A + (size_t)m * lda;
    double* U = b + m;
    double* V = U + m;
    double* piv = V + m;
    double* red = piv + 2;
    int* ctl = (int*)(red + INV_NT / 32);
    const double pd = a.eaux[2 * (size_t)slot];
    if (!(pd > 0.0)) return;   // empty point: written by the transform kernel
    const int pt = a.order ? a.order[slot] : a.item0 + slot;
    const double trss = a.eaux[2 * (size_t)slot + 1];
    const size_t q0 = (size_t)slot * m * m;
    for (int i = tid; i < m * m; i += INV_NT) {
        const int r = i / m, c = i - r * m;
        if (c >= r) A[r * lda + c] = a.eq[q0 + i];
    }
    for (int i = tid; i < m; i += INV_NT) b[i] = a.eb[(size_t)slot * m + i];
    __syncthreads();
    const int rc = la::spd_inverse<INV_NT>(A, m, lda, U, V, piv, ctl);
    const double dfs = denkf_outputs<INV_NT>(a, pt, A, lda, b, red);
    if (rc != 0 && tid == 0) a.status[pt] = rc;
    if (a.want_diag) diag_single(a, pt, (int)pd, dfs, trss);
}

// Per-batch timing: events before and after each batch's transform kernel
// and after its solve kernels, summed by enkfg_kernel_times.  Events are
// created on first use (outside stream capture); batches past
// ENKFG_TIMED_BATCHES, or marked while no event could be created, are not
// timed.
void batch_mark(enkfg_ctx* ctx, int k, cudaStream_t st)
{
    if (k == 0) ++ctx->nbatch;
    const int b = ctx->nbatch - 1;
    if (b < 0 || b >= ENKFG_TIMED_BATCHES) return;
    const int idx = 3 * b + k;
    while (ctx->nbev <= idx) {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        if (cudaStreamIsCapturing(st, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone ||
            cudaEventCreate(&ctx->bev[ctx->nbev]) != cudaSuccess) {
            cudaGetLastError();
            return;
        }
        ++ctx->nbev;
    }
    cudaEventRecord(ctx->bev[idx], st);
}

size_t batch_points(const enkfg_ctx* ctx, size_t per_slot, size_t budget, int nitems)
{
    size_t B = ctx->solve_batch > 0 ? (size_t)ctx->solve_batch : budget / per_slot;
    if (B < 256) B = 256;
    if (B >= 1024) B -= B % 1024;
    if (B > (size_t)nitems) B = (size_t)nitems;
    return B;
}

// slot bytes of the batched FP64 inverse and eigensolver
static size_t inv_slot_bytes(int m) { return (size_t)m * m * 8 + (size_t)m * 8 + 16; }
static size_t etkf_slot_bytes(int m)
{
    const size_t rcap = (size_t)m * m + 64 * (size_t)m, hcap = 8 * (size_t)m;
    return (size_t)m * m * 8 + (size_t)5 * m * 8 + 16 + rcap * 16 + hcap * 8 + 4;
}

void batch_out(enkfg_ctx* ctx, int i0, int nb, cudaStream_t st)
{
    if (ctx->out_seg <= 0) return;
    cudaStream_t cout = ctx->cstream[1];
    const size_t m = ctx->nmem, md = ctx->nmem_dyn;
    cudaEventRecord(ctx->out_ev, st);
    cudaStreamWaitEvent(cout, ctx->out_ev, 0);
    if (ctx->out_T)
        cudaMemcpyAsync(ctx->out_T + (size_t)i0 * md * m, ctx->d_T + (size_t)i0 * md * m, (size_t)nb * md * m * 4,
                        cudaMemcpyDeviceToHost, cout);
    if (ctx->out_w)
        cudaMemcpyAsync(ctx->out_w + (size_t)i0 * m, ctx->d_w + (size_t)i0 * m, (size_t)nb * m * 4,
                        cudaMemcpyDeviceToHost, cout);
    if (ctx->out_T64)
        cudaMemcpyAsync(ctx->out_T64 + (size_t)i0 * md * m, ctx->d_T64 + (size_t)i0 * md * m,
                        (size_t)nb * md * m * 8, cudaMemcpyDeviceToHost, cout);
    if (ctx->out_w64)
        cudaMemcpyAsync(ctx->out_w64 + (size_t)i0 * m, ctx->d_w64 + (size_t)i0 * m, (size_t)nb * m * 8,
                        cudaMemcpyDeviceToHost, cout);
}

static enkfg_status run_inv_batched(enkfg_ctx* ctx, const CalcArgs& a0, int precision, cudaStream_t st)
{
    enkfg_status s;
    const int m = a0.m, nitems = a0.nitems;
    const size_t B = batch_points(ctx, inv_slot_bytes(m), (size_t)2 << 30, nitems);   // about 2 GB a batch
    if ((s = ensure(ctx, &ctx->d_eq, &ctx->eq_cap, B * m * m))) return s;
    if ((s = ensure(ctx, &ctx->d_eb, &ctx->eb_cap, B * m))) return s;
    if ((s = ensure(ctx, &ctx->d_eaux, &ctx->eaux_cap, B * 2))) return s;
    const int lda = (m % 2 == 0) ? m + 1 : m + 2;
    const size_t ismem = ((size_t)m * lda + 3 * (size_t)m + 2 + INV_NT / 32) * 8 + 16;
    if (ismem > 227 * 1024) {
        set_err(ctx, "batched inverse: nmem = %d needs %zu bytes of shared memory", m, ismem);
        return ENKFG_EUNSUPPORTED;
    }
    CK(cudaFuncSetAttribute(k_inv_finish, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ismem));
    for (int i0 = 0; i0 < nitems; i0 += (int)B) {
        const int nb = (nitems - i0 < (int)B) ? nitems - i0 : (int)B;
        CalcArgs b = a0;
        b.defer = 1;
        b.nitems = nb;
        if (a0.order) {
            b.order = a0.order + i0;
            b.item0 = 0;
        } else {
            b.item0 = a0.item0 + i0;
        }
        b.eq = ctx->d_eq;
        b.eb = ctx->d_eb;
        b.eaux = ctx->d_eaux;
        if (b.persistent) CK(cudaMemsetAsync(ctx->d_qhead, 0, sizeof(int), st));
        batch_mark(ctx, 0, st);
        if ((s = dispatch(ctx, b, precision, st))) return s;
        batch_mark(ctx, 1, st);
        k_inv_finish<<<nb, INV_NT, ismem, st>>>(b);
        CKL();
        batch_mark(ctx, 2, st);
        batch_out(ctx, i0, nb, st);
    }
    return ENKFG_OK;
}

// Batched Householder tridiagonalisation for the ETKF eigensolver: one small
// CTA per point (dozens per SM at small nmem), from the upper triangle of M
// the transform kernel saved; Q, the diagonal and the off-diagonal go back
// to the slot for k_ql_batch and k_eig_finish.  In the transform kernel the
// reduction's FP64 divisions and dependent FMA chains left the SM idle.
template <int NT>
__global__ void __launch_bounds__(NT) k_tred_batch(CalcArgs a)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int m = a.m, lda = (m % 2 == 0) ? m + 1 : m + 2;
    const int tid = threadIdx.x, slot = blockIdx.x;
    double* A = (double*)smem_raw;
    double* d = A + (size_t)m * lda;
    double* e = d + m;
    double* red = e + m;
    if (!(a.eaux[2 * (size_t)slot] > 0.0)) return;   // empty point
    const size_t q0 = (size_t)slot * m * m;
    for (int i = tid; i < m * m; i += NT) {
        const int r = i / m, c = i - r * m;
        if (c >= r) {
            const double v = a.eq[q0 + i];
            A[r * lda + c] = v;
            A[c * lda + r] = v;
        }
    }
    __syncthreads();
    la::tred2<NT>(A, m, lda, d, e, red);
    for (int i = tid; i < m * m; i += NT) {
        const int r = i / m, c = i - r * m;
        a.eq[q0 + i] = A[r * lda + c];
    }
    for (int i = tid; i < m; i += NT) {
        a.ed[(size_t)slot * m + i] = d[i];
        a.ee[(size_t)slot * m + i] = e[i];
    }
}

static enkfg_status run_etkf_batched(enkfg_ctx* ctx, const CalcArgs& a0, int precision, cudaStream_t st)
{
    enkfg_status s;
    const int m = a0.m, nitems = a0.nitems;
    const int rcap = m * m + 64 * m;         // QL typically needs about 0.75 m^2 rotations
    const int hcap = 8 * m;
    const size_t B = batch_points(ctx, etkf_slot_bytes(m), (size_t)2 << 30, nitems);   // about 2 GB a batch
    if ((s = ensure(ctx, &ctx->d_eq, &ctx->eq_cap, B * m * m))) return s;
    if ((s = ensure(ctx, &ctx->d_ed, &ctx->ed_cap, B * m))) return s;
    if ((s = ensure(ctx, &ctx->d_ee, &ctx->ee_cap, B * m))) return s;
    if ((s = ensure(ctx, &ctx->d_eb, &ctx->eb_cap, B * m))) return s;
    if ((s = ensure(ctx, &ctx->d_eaux, &ctx->eaux_cap, B * 2))) return s;
    if ((s = ensure(ctx, &ctx->d_eval, &ctx->eval_cap, B * m))) return s;
    if ((s = ensure(ctx, &ctx->d_erot, &ctx->erot_cap, B * rcap))) return s;
    if ((s = ensure(ctx, &ctx->d_ehdr, &ctx->ehdr_cap, B * hcap))) return s;
    if ((s = ensure(ctx, &ctx->d_enh, &ctx->enh_cap, B))) return s;
    const size_t qsmem = (size_t)2 * m * QLB_T * 8;
    const int lda = (m % 2 == 0) ? m + 1 : m + 2;
    const size_t fsmem = ((size_t)m * lda + 6 * (size_t)m + CALC_NT / 32) * 8 + 16;
    const size_t tsmem = ((size_t)m * lda + 2 * (size_t)m + 4) * 8 + 16;
    const bool tr64 = m <= 64;   // 64 threads up to nmem 64, else 128
    if (tr64) CK(cudaFuncSetAttribute(k_tred_batch<64>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tsmem));
    else CK(cudaFuncSetAttribute(k_tred_batch<128>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tsmem));
    CK(cudaFuncSetAttribute(k_ql_batch, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)qsmem));
    CK(cudaFuncSetAttribute(k_eig_finish, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fsmem));
    for (int i0 = 0; i0 < nitems; i0 += (int)B) {
        const int nb = (nitems - i0 < (int)B) ? nitems - i0 : (int)B;
        CalcArgs b = a0;
        b.defer = 1;
        b.nitems = nb;
        if (a0.order) {
            b.order = a0.order + i0;
            b.item0 = 0;
        } else {
            b.item0 = a0.item0 + i0;
        }
        b.eq = ctx->d_eq;
        b.ed = ctx->d_ed;
        b.ee = ctx->d_ee;
        b.eb = ctx->d_eb;
        b.eaux = ctx->d_eaux;
        if (b.persistent) CK(cudaMemsetAsync(ctx->d_qhead, 0, sizeof(int), st));
        batch_mark(ctx, 0, st);
        if ((s = dispatch(ctx, b, precision, st))) return s;
        batch_mark(ctx, 1, st);
        if (tr64) k_tred_batch<64><<<nb, 64, tsmem, st>>>(b);
        else k_tred_batch<128><<<nb, 128, tsmem, st>>>(b);
        CKL();
        k_ql_batch<<<div_up(nb, QLB_T), QLB_T, qsmem, st>>>(nb, m, ctx->d_eaux, ctx->d_ed, ctx->d_ee, ctx->d_eval,
                                                           ctx->d_erot, rcap, ctx->d_ehdr, hcap, ctx->d_enh);
        CKL();
        k_eig_finish<<<nb, CALC_NT, fsmem, st>>>(b, ctx->d_eval, ctx->d_erot, rcap, ctx->d_ehdr, hcap, ctx->d_enh);
        CKL();
        batch_mark(ctx, 2, st);
        batch_out(ctx, i0, nb, st);
    }
    return ENKFG_OK;
}

enkfg_status run_transforms(enkfg_ctx* ctx, const enkfg_calc_params* p, cudaStream_t st)
{
    enkfg_status s;
    int npts = ctx->nj * ctx->ni;
    int m = ctx->nmem, md = ctx->nmem_dyn;
    bool enkf = (p->mode == ENKFG_MODE_ENKF || p->mode == ENKFG_MODE_HYBRID);
    if (p->precision == ENKFG_PREC_MIXED && m > 127) {
        set_err(ctx, "the mixed-precision path supports nmem <= 127 (got %d)", m);
        return ENKFG_EUNSUPPORTED;
    }
    if (m > 144) {
        set_err(ctx, "nmem = %d above the supported maximum 144", m);
        return ENKFG_EUNSUPPORTED;
    }
    cudaEventRecord(ctx->ev[0], st);
    if ((s = prepare_search(ctx, st))) return s;
    if (!ctx->gather_valid && (s = build_gather(ctx, st))) return s;
    cudaEventRecord(ctx->ev[1], st);

    // outputs
    size_t nT = enkf ? (size_t)npts * md * m : 1;
    if ((s = ensure(ctx, &ctx->d_T, &ctx->T_cap, nT))) return s;
    if ((s = ensure(ctx, &ctx->d_w, &ctx->w_cap, (size_t)npts * m))) return s;
    const bool w64 = ctx->want64;
    if (w64 && (s = ensure(ctx, &ctx->d_T64, &ctx->T64_cap, nT))) return s;
    if (w64 && (s = ensure(ctx, &ctx->d_w64, &ctx->w64_cap, (size_t)npts * m))) return s;
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
    a.nitems = npts;
    a.ntypes = ctx->ntypes;
    a.ndim = ctx->geographic ? 3 : 2;
    a.m = m;
    a.md = md;
    a.mode = p->mode;
    a.scheme = p->scheme;
    a.want_diag = p->want_diag ? 1 : 0;
    a.alpha = p->alpha;
    a.wait_ns = ctx->wait_ns;
    a.wait_drill = ctx->wait_drill;
    a.kc = 32;
    a.types = ctx->d_types;
    a.bstart = ctx->d_bstart;
    a.sx = ctx->d_sx;
    a.sxf = ctx->d_sxf;
    a.syf = ctx->d_syf;
    a.sy = ctx->d_sy;
    a.sz = ctx->d_sz;
    a.St = ctx->d_St;
    a.qscale = ctx->d_qscale;
    a.mpad = ctx->mpad;
    a.ss = ctx->d_ss;
    a.ssf = ctx->d_ssf;
    a.qx = ctx->d_qx;
    a.qy = ctx->d_qy;
    a.qz = ctx->d_qz;
    a.sid = ctx->d_sid;
    a.cut = any_nlobsmax(ctx) ? ctx->d_cut : nullptr;
    a.T = enkf ? ctx->d_T : nullptr;
    a.w = ctx->d_w;
    a.T64 = (enkf && w64) ? ctx->d_T64 : nullptr;
    a.w64 = w64 ? ctx->d_w64 : nullptr;
    a.nlobs = ctx->d_nlobs;
    a.dfs = ctx->d_dfs;
    a.srf = ctx->d_srf;
    a.pnlobs = ctx->d_pnlobs;
    a.pdfs = ctx->d_pdfs;
    a.psrf = ctx->d_psrf;
    a.status = ctx->d_status_pt;

    if (p->path == ENKFG_PATH_BATCHED) {
        // size-sorted queue (by candidate count)
        if ((s = count_candidates(ctx, ctx->d_counts, st))) return s;
        // the queue sorted within segments of one solve batch, so that a
        // batch covers a contiguous range of points and its outputs can
        // leave while the next batch runs
        int seg = 0;
        {
            const bool etkf_ = (p->mode != ENKFG_MODE_ENOI && p->scheme == ENKFG_SCHEME_ETKF);
            const bool defer_ = !(p->want_diag && ctx->ntypes > 1);
            if (defer_) {
                size_t B;
                if (etkf_ && p->precision == ENKFG_PREC_MIXED && etkf_mixed_supported(m))
                    B = batch_points(ctx, etkf_mixed_slot_bytes(m), (size_t)8 << 30, npts);
                else if (etkf_)
                    B = batch_points(ctx, etkf_slot_bytes(m), (size_t)2 << 30, npts);
                else
                    B = batch_points(ctx, inv_slot_bytes(m), (size_t)2 << 30, npts);
                if (B % QS_T == 0 && B < (size_t)npts) seg = (int)B;
                else if (B >= (size_t)npts) seg = npts;   // one batch
            }
        }
        if ((s = build_queue(ctx, npts, seg % QS_T == 0 ? seg : 0, st))) return s;
        if (ctx->out_seg && seg == 0) ctx->out_seg = 0;   // batches mix regions: copy at the end
        a.persistent = 1;
        a.order = ctx->d_order;
        a.qhead = ctx->d_qhead;
        a.counts = ctx->d_counts;
        a.kc_table = ctx->d_qhead + 2 + NBINS;   // chunk size per count bin (autotuned)
        // the chunk-size table goes to the device only when it changes (no
        // host-to-device copy in a steady cycle, which CUDA graphs capture)
        const int want = (ctx->kc_tuned && ctx->kc_tuned_prec == p->precision) ? 3
                         : (p->precision == ENKFG_PREC_MIXED ? 2 : 1);
        if (ctx->kc_loaded != want) {
            static const int kc_default[NBINS] = { 8, 8, 8, 8, 16, 16, 32, 32, 32, 64, 64, 64, 64, 64, 64, 64 };
            static const int kc_mixed[NBINS] = { 8, 8, 8, 8, 16, 16, 24, 32, 32, 32, 32, 32, 32, 32, 32, 32 };
            const int* tab = want == 3 ? ctx->kc_table : (want == 2 ? kc_mixed : kc_default);
            CK(cudaMemcpy(ctx->d_qhead + 2 + NBINS, tab, sizeof(kc_default), cudaMemcpyHostToDevice));
            ctx->kc_loaded = want;
        }
        CK(cudaMemsetAsync(ctx->d_qhead, 0, sizeof(int), st));
    }
    cudaEventRecord(ctx->ev[2], st);
    if (p->path == ENKFG_PATH_BATCHED && p->tune && !(ctx->kc_tuned && ctx->kc_tuned_prec == p->precision)) {
        if ((s = autotune(ctx, a, p->precision, st))) return s;
        CK(cudaMemsetAsync(ctx->d_status_pt, 0, (size_t)npts * sizeof(int), st));
        CK(cudaMemsetAsync(ctx->d_qhead, 0, sizeof(int), st));
        cudaEventRecord(ctx->ev[2], st);
    }
    // ETKF: the batched eigensolver; DEnKF / EnOI: the batched inverse (the
    // per-type diagnostics need the point's own solve for their second
    // pass, so they keep the in-kernel one)
    const bool etkf = (p->mode != ENKFG_MODE_ENOI && p->scheme == ENKFG_SCHEME_ETKF);
    const bool defer = !(a.want_diag && a.ntypes > 1);
    if (!defer) ctx->out_seg = 0;   // one launch: the host call copies at the end
    ctx->nbatch = 0;
    if (defer && etkf && p->precision == ENKFG_PREC_MIXED && etkf_mixed_supported(m)) {
        if ((s = run_etkf_mixed(ctx, a, st))) return s;
    } else if (defer && etkf) {
        if ((s = run_etkf_batched(ctx, a, p->precision, st))) return s;
    } else if (defer) {
        if ((s = run_inv_batched(ctx, a, p->precision, st))) return s;
    } else {
        batch_mark(ctx, 0, st);
        if ((s = dispatch(ctx, a, p->precision, st))) return s;
        batch_mark(ctx, 1, st);
        batch_mark(ctx, 2, st);
    }
    cudaEventRecord(ctx->ev[3], st);
    ctx->t_mode = p->mode;
    ctx->t_nmem = m;
    ctx->t_ndyn = md;
    ctx->t_valid = true;
    return ENKFG_OK;
}
