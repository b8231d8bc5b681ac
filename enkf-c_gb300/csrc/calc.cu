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
    static size_t bytes()
    {
        size_t s = 0;
        s += (size_t)KC_MAX * TLD * 8;                 // tile
        s += (size_t)LIST_EXTRA * 8;                   // list taper
        s += (size_t)KC_MAX * 8;                       // sloc
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
    constexpr int MP = 16 * R, TLD = MP, LDA = MP + 1;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    unsigned char* sp = smem_raw;
    double* tile = (double*)sp;       sp += (size_t)KC_MAX * TLD * 8;
    double* llc = (double*)sp;        sp += (size_t)LIST_EXTRA * 8;
    double* sloc = (double*)sp;       sp += (size_t)KC_MAX * 8;
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
        GramProc64<R> proc(a, s, tile, sloc);
        const int p = enumerate_obs<0>(a, kc, qx, qy, qz, s, proc, true);
        if (p == 0) {
            store_empty(a, pt);
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
        solve_point(a, pt, p, kc, qx, qy, qz, A, LDA, b, trss, d, e, cs, sn, v, s, tile, TLD);
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

// blkcnt [nblk][NBINS] -> exclusive offsets of (block, bin) in bin-major order
__global__ void k_queue_offsets(int nblk, int* blkcnt)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    int acc = 0;
    for (int b = 0; b < NBINS; ++b)
        for (int k = 0; k < nblk; ++k) {
            int v = blkcnt[k * NBINS + b];
            blkcnt[k * NBINS + b] = acc;
            acc += v;
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

enkfg_status build_queue(enkfg_ctx* ctx, int npts, cudaStream_t st)
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
    k_queue_offsets<<<1, 32, 0, st>>>(nblk, blk);
    CKL();
    k_queue_scatter<<<nblk, QS_T, 0, st>>>(npts, ctx->d_counts, rank, blk, ctx->d_order);
    CKL();
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
    int grid = a.nitems;
    if (a.persistent) {
        int per_sm = 0, nsm = 0;
        CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_transforms<R>, CALC_NT, smem));
        CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, ctx->device));
        if (per_sm < 1) per_sm = 1;
        grid = per_sm * nsm;
        if (grid > a.nitems) grid = a.nitems;
    }
    if (grid < 1) return ENKFG_OK;
    k_transforms<R><<<grid, CALC_NT, smem, st>>>(a);
    CKL();
    return ENKFG_OK;
}

enkfg_status launch_mixed(enkfg_ctx* ctx, CalcArgs& a, cudaStream_t st);

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
    static const int cand64[4] = { 8, 16, 32, 64 };
    static const int candmx[4] = { 8, 16, 24, 32 };
    const int* cand = precision == ENKFG_PREC_MIXED ? candmx : cand64;
    int table[NBINS];
    for (int b = 0; b < NBINS; ++b) table[b] = precision == ENKFG_PREC_MIXED ? 32 : (b < 4 ? 8 : b < 6 ? 16 : b < 9 ? 32 : 64);
    int* kct = ctx->d_qhead + 2 + NBINS;
    enkfg_status s = ENKFG_OK;
    int pos = 0;
    while (pos < npts && s == ENKFG_OK) {
        const int bin = count_bin(counts[order[pos]]);
        int end = pos;
        while (end < npts && count_bin(counts[order[end]]) == bin) ++end;
        const int len = end - pos;
        const int take = len < TUNE_SAMPLE ? len : TUNE_SAMPLE;
        const int first = pos + (len - take) / 2;
        if (take >= 64 && bin >= 2) {
            float best = 1e30f;
            for (int k = 0; k < 4; ++k) {
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
    if (!ctx->index_valid && (s = build_index(ctx, st))) return s;
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
    a.qx = ctx->d_qx;
    a.qy = ctx->d_qy;
    a.qz = ctx->d_qz;
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
        // size-sorted queue
        if ((s = count_local(ctx, ctx->d_counts, nullptr, st))) return s;
        if ((s = build_queue(ctx, npts, st))) return s;
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
    if ((s = dispatch(ctx, a, p->precision, st))) return s;
    cudaEventRecord(ctx->ev[3], st);
    ctx->t_mode = p->mode;
    ctx->t_nmem = m;
    ctx->t_ndyn = md;
    ctx->t_valid = true;
    return ENKFG_OK;
}
