// calc_mixed.cu -- mixed-precision local-analysis transforms: S'S and S's on
// the 5th-generation tensor cores (tcgen05, TF32 inputs, FP32 accumulation in
// tensor memory), everything else in FP64 as in calc.cu.
//
// Per round of kc = 8*NA local observations:
//   * the tapered rows of S (m members, rows m..127 zero) are written to
//     shared memory as a K-major operand tile (rows = members, K =
//     observations), split into TF32 hi = rn(v) and lo = rn(v - hi);
//   * one thread issues, for each group q of 8 observations, three MMAs
//     D_q = hi*hi' + hi*lo' + lo*hi' of shape M=128 x N x 8 into its own TMEM
//     accumulator q (N = m rounded up to 16).  A and B are the same tile, so
//     D_q is that group's contribution to S'S;
//   * the MMAs' completion is signalled by tcgen05.commit on an mbarrier;
//     the CTA then reads the NA accumulators out of TMEM (tcgen05.ld) and adds
//     them, with error-free TwoSum steps, to a double-float (hi + lo FP32)
//     accumulator in shared memory.  Only 8 observations are ever summed in
//     FP32 inside the tensor core, so rounding stays near the split's own
//     (about 2^-22 relative per product) whatever the local obs count;
//   * S's is accumulated on the CUDA cores, one member per thread, with
//     TwoProduct/TwoSum compensated FP32 (double-float) arithmetic.
//
// The accumulators are then converted to FP64 and go through the same FP64
// solve as the plain path (Householder + QL for ETKF, Cholesky for
// DEnKF/EnOI).
//
// Shared-memory operand layout (canonical K-major, no swizzle): core matrices
// of 8 rows x 16 bytes (4 TF32) stored as 128 contiguous bytes; core matrix
// (row group g, K group q) at (g * kc/4 + q) * 128 bytes.  Descriptor:
// leading (K) byte offset 128, stride (row-group) byte offset kc*32.
//
// Every wait on the MMA mbarrier is bounded; on expiry the CTA records an
// error status for the point, stops, releases its TMEM and returns.
#include "calc_common.cuh"

#define MX_ROWS 128
#define MX_WAIT_NS 2000000000ull   // 2 s bound on any wait for the tensor cores
#define MX_TIMEOUT_CODE 99

namespace tc {

__device__ __forceinline__ uint32_t smem_u32(const void* p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ uint64_t desc_kmajor_noswizzle(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;     // descriptor version for tcgen05
    // base offset 0, absolute LBO mode 0, layout type 0 (no swizzle)
    return d;
}

// instruction descriptor: kind::tf32, D = F32, A = B = TF32, K-major, M x N
__host__ __device__ __forceinline__ uint32_t idesc_tf32(int M, int N)
{
    return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_tf32(uint32_t dtmem, uint64_t da, uint64_t db, uint32_t idesc, uint32_t acc)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(dtmem),
        "l"(da), "l"(db), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void commit(uint64_t* mbar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(mbar))
                 : "memory");
}

__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void mbar_init(uint64_t* mbar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(mbar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* mbar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred P;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 P, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, P;\n\t}\n"
        : "=r"(ok)
        : "r"(smem_u32(mbar)), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ uint64_t now_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}

// wait for phase `parity` of the mbarrier, at most MX_WAIT_NS; true if it completed
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* mbar, uint32_t parity)
{
    const uint64_t t0 = now_ns();
    for (;;) {
        if (mbar_try_wait(mbar, parity)) return true;
        if (now_ns() - t0 > MX_WAIT_NS) return false;
    }
}

__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float (&v)[8])
{
    uint32_t r[8];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int k = 0; k < 8; ++k) v[k] = __uint_as_float(r[k]);
}

__device__ __forceinline__ void tmem_ld8_nowait(uint32_t taddr, uint32_t (&r)[8])
{
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr));
}

__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

__device__ __forceinline__ float to_tf32(float x)
{
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}

}  // namespace tc

#define MX_NA 4            // TMEM accumulators (groups of 8 obs) per round

struct MixedShared {
    float* tileH;      // [MX_ROWS x kc] core-matrix layout
    float* tileL;
    float2* Macc;      // [m x lda] double-float accumulator of S'S (later reused as FP64)
    int lda;
    float* sl;         // [kc] tapered innovations of the round
    uint64_t* mbar;
    uint32_t taddr;
    int N;             // MMA N (m rounded up to 16)
    int kc;            // observations per round (8 * MX_NA)
    int* err;          // shared error flag
};

__device__ __forceinline__ int core_offset(int r, int k, int kc)
{
    // float index of element (row r, K index k) in the K-major no-swizzle tile
    return (((r >> 3) * (kc >> 2) + (k >> 2)) << 5) + ((r & 7) << 2) + (k & 3);
}

// error-free (TwoSum) accumulation of x into the double-float (a.x + a.y)
__device__ __forceinline__ void df_add(float2& a, float x)
{
    float s = a.x + x;
    float bp = s - a.x;
    float e = (a.x - (s - bp)) + (x - bp);
    a.x = s;
    a.y += e;
}

// HB: 8-column blocks of S'S each thread accumulates (half of the N columns
// of its TMEM lane), held as double-floats in registers for the whole point.
template <int HB>
struct GramProcTC {
    const CalcArgs& a;
    const PointScratch& s;
    MixedShared& ms;
    uint32_t& phase;
    float bhi, blo;    // S's for member threadIdx.x (double-float)
    float2 acc[HB][8]; // S'S row 32*(warp%4)+lane, columns (warp/4)*half + [0, 8*HB)
    __device__ __forceinline__ GramProcTC(const CalcArgs& a_, const PointScratch& s_, MixedShared& ms_, uint32_t& ph)
        : a(a_), s(s_), ms(ms_), phase(ph), bhi(0.0f), blo(0.0f)
    {
#pragma unroll
        for (int b = 0; b < HB; ++b)
#pragma unroll
            for (int j = 0; j < 8; ++j) acc[b][j] = make_float2(0.0f, 0.0f);
    }

    // write the accumulated S'S into the shared double-float matrix
    __device__ __forceinline__ void store()
    {
        const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, m = a.m;
        const int r = 32 * (wid & 3) + lane;
        const int half = ms.N >> 1, c0 = (wid >> 2) * half;
        if (r >= m) return;
#pragma unroll
        for (int b = 0; b < HB; ++b)
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const int c = c0 + 8 * b + j;
                if (8 * b < half && c < m) ms.Macc[r * ms.lda + c] = acc[b][j];
            }
    }

    __device__ void chunk(int nc, int t)
    {
        const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
        const int m = a.m, kc = ms.kc;
        const bool tsum = a.want_diag && a.ntypes > 1;
        double ssq = 0.0;
        if (*ms.err) return;
        // 1. tapered S rows of the round, split into TF32 hi + lo; the
        //    tapered innovations for S's
        const float* lcf = reinterpret_cast<const float*>(s.llc);   // FP32 taper (enumerate_obs<true>)
        if (tid < kc) ms.sl[tid] = (tid < nc) ? (float)a.ss[s.lid[tid]] * lcf[tid] : 0.0f;
        for (int i = tid; i < kc * m; i += CALC_NT) {
            int k = i / m, r = i - k * m;
            float v = 0.0f;
            if (k < nc) {
                v = __fmul_rn(a.St[(size_t)s.lid[k] * a.mpad + r], lcf[k]);
                if (tsum) ssq += (double)v * (double)v;
            }
            float hi = tc::to_tf32(v);
            int off = core_offset(r, k, kc);
            ms.tileH[off] = hi;
            ms.tileL[off] = tc::to_tf32(v - hi);
        }
        tc::fence_async_smem();
        __syncthreads();
        // 2. one thread issues the MMAs: group q -> accumulator q
        if (tid == 0) {
            tc::fence_after();
            const uint32_t h0 = tc::smem_u32(ms.tileH), l0 = tc::smem_u32(ms.tileL);
            const uint32_t sbo = (uint32_t)kc * 32u, idesc = tc::idesc_tf32(MX_ROWS, ms.N);
            for (int q = 0; q < kc / 8; ++q) {
                const uint32_t off = (uint32_t)q * 256u;    // two 128-byte core matrices per group of 8
                const uint32_t dq = ms.taddr + (uint32_t)(q * ms.N);
                uint64_t dh = tc::desc_kmajor_noswizzle(h0 + off, 128u, sbo);
                uint64_t dl = tc::desc_kmajor_noswizzle(l0 + off, 128u, sbo);
                tc::mma_tf32(dq, dh, dh, idesc, 0u);
                tc::mma_tf32(dq, dh, dl, idesc, 1u);
                tc::mma_tf32(dq, dl, dh, idesc, 1u);
            }
            tc::commit(ms.mbar);
        }
        // S's on the CUDA cores while the tensor cores run (compensated FP32)
        if (tid < m) {
            for (int k = 0; k < nc; ++k) {
                float v = __fmul_rn(a.St[(size_t)s.lid[k] * a.mpad + tid], lcf[k]);
                float x = ms.sl[k];
                float p = v * x, pe = fmaf(v, x, -p);
                float sm = bhi + p, bp = sm - bhi;
                blo += ((bhi - (sm - bp)) + (p - bp)) + pe;
                bhi = sm;
            }
        }
        // 3. bounded wait for the MMAs; on expiry record the error and wait
        // once more (bounded) so that nothing is in flight when TMEM is freed
        bool done = tc::mbar_wait_bounded(ms.mbar, phase);
        if (!done) {
            atomicExch(ms.err, 1);
            tc::mbar_wait_bounded(ms.mbar, phase);
        }
        phase ^= 1u;
        tc::fence_after();
        __syncthreads();
        if (*ms.err) return;
        // 4. accumulators (FP32, TMEM) -> double-float registers.  Warps w and
        // w+4 share the TMEM lanes 32*(w%4).., each reading half of the N
        // columns; the loads of all groups are issued before one wait.
        {
            const int half = ms.N >> 1;
            const int c0 = (wid >> 2) * half;
            const uint32_t lane_addr = ms.taddr + ((uint32_t)(32 * (wid & 3)) << 16);
            const int ngroups = (nc + 7) / 8;
#pragma unroll
            for (int b = 0; b < HB; ++b) {
                if (8 * b < half) {
                    uint32_t v[MX_NA][8];
#pragma unroll
                    for (int q = 0; q < MX_NA; ++q)
                        tc::tmem_ld8_nowait(lane_addr + (uint32_t)(q * ms.N + c0 + 8 * b), v[q]);
                    tc::tmem_wait_ld();
#pragma unroll
                    for (int q = 0; q < MX_NA; ++q)
                        if (q < ngroups) {
#pragma unroll
                            for (int j = 0; j < 8; ++j) df_add(acc[b][j], __uint_as_float(v[q][j]));
                        }
                }
            }
        }
        tc::fence_before();
        if (tsum) {
            double v = la::block_sum<CALC_NT>(ssq, s.red);
            if (tid == 0) s.tss[t] += v;
        }
        __syncthreads();
    }
    __device__ __forceinline__ void type_end(int) {}
};

static size_t mixed_smem_bytes(int m, int kc, bool need_x)
{
    int lda = (m % 2 == 0) ? m + 1 : m + 2;
    size_t s = 0;
    s += 2 * (size_t)MX_ROWS * kc * 4;                     // tiles hi, lo
    s += (size_t)m * lda * 8;                              // Macc (also A)
    s += (size_t)kc * 4;                                   // tapered innovations
    if (need_x) s += (size_t)m * lda * 8;                  // X
    s += (size_t)6 * (m + 1) * 8;                          // b d e cs sn v
    s += (size_t)ENKFG_MAXTYPES * 8 * 2;
    s += (size_t)(CALC_NT / 32) * 8;
    s += (size_t)LIST_EXTRA * 8;                           // llc
    s += (size_t)LIST_EXTRA * 4;                           // lid
    s += (size_t)ENKFG_MAXTYPES * 4;
    s += 256;                                              // control ints
    s += 64;                                               // mbarrier, tmem slot, flags
    return s;
}

template <int HB>
__global__ void __launch_bounds__(CALC_NT) k_transforms_mixed(CalcArgs a, int kcm, int N, uint32_t tcols)
{
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const int tid = threadIdx.x, wid = tid >> 5;
    const int m = a.m, lda = (m % 2 == 0) ? m + 1 : m + 2;   // odd stride: fewer bank conflicts
    const bool need_x = (a.mode == ENKFG_MODE_ENOI || a.scheme == ENKFG_SCHEME_DENKF);
    unsigned char* sp = smem_raw;
    float* tileH = (float*)sp;        sp += (size_t)MX_ROWS * kcm * 4;
    float* tileL = (float*)sp;        sp += (size_t)MX_ROWS * kcm * 4;
    double* Macc = (double*)sp;       sp += (size_t)m * lda * 8;
    float* sl = (float*)sp;           sp += (size_t)((kcm + 3) & ~3) * 4;
    double* X = nullptr;
    if (need_x) { X = (double*)sp;    sp += (size_t)m * lda * 8; }
    double* b = (double*)sp;          sp += (m + 1) * 8;
    double* d = (double*)sp;          sp += (m + 1) * 8;
    double* e = (double*)sp;          sp += (m + 1) * 8;
    double* cs = (double*)sp;         sp += (m + 1) * 8;
    double* sn = (double*)sp;         sp += (m + 1) * 8;
    double* v = (double*)sp;          sp += (m + 1) * 8;
    double* tss = (double*)sp;        sp += ENKFG_MAXTYPES * 8;
    double* tpd = (double*)sp;        sp += ENKFG_MAXTYPES * 8;
    double* red = (double*)sp;        sp += (CALC_NT / 32) * 8;
    double* llc = (double*)sp;        sp += (size_t)LIST_EXTRA * 8;
    int* lid = (int*)sp;              sp += LIST_EXTRA * 4;
    int* tcount = (int*)sp;           sp += ENKFG_MAXTYPES * 4;
    int* ictl = (int*)sp;             sp += 256;
    uint64_t* mbar = (uint64_t*)sp;   sp += 8;
    uint32_t* tslot = (uint32_t*)sp;  sp += 8;
    int* err = (int*)sp;
    const PointScratch s{ lid, llc, ictl, tcount, tss, tpd, red };

    // set-up: TMEM columns, mbarrier, zeroed operand tiles
    if (wid == 0) tc::tmem_alloc(tslot, tcols);
    if (tid == 0) {
        tc::mbar_init(mbar, 1);
        *err = 0;
    }
    for (int i = tid; i < 2 * MX_ROWS * kcm; i += CALC_NT) tileH[i] = 0.0f;   // tileL follows tileH
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    MixedShared ms{ tileH, tileL, (float2*)Macc, lda, sl, mbar, *tslot, N, kcm, err };
    uint32_t phase = 0;

    for (int it = 0;; ++it) {
        const int idx = next_item(a, it, ictl);
        if (idx < 0 || *err) break;
        const int pt = a.order ? a.order[idx] : idx;
        const double qx = a.qx[pt], qy = a.qy[pt], qz = a.ndim == 3 ? a.qz[pt] : 0.0;
        // observations per round: 8 x (accumulators used), per count bin when tuned
        ms.kc = kcm;
        if (a.kc_table != nullptr && a.counts != nullptr) {
            int k = a.kc_table[count_bin(a.counts[pt])];
            ms.kc = (k >= 8 && k <= kcm) ? (k & ~7) : kcm;
        }
        if (tid < ENKFG_MAXTYPES) {
            tss[tid] = 0.0;
            tpd[tid] = 0.0;
            tcount[tid] = 0;
        }
        for (int i = tid; i < m * lda; i += CALC_NT) Macc[i] = 0.0;   // also zero as float2
        __syncthreads();
        GramProcTC<HB> proc(a, s, ms, phase);
        const int p = enumerate_obs<true>(a, ms.kc, qx, qy, qz, s, proc, true);
        proc.store();
        __syncthreads();
        if (*err) {
            if (tid == 0) a.status[pt] = MX_TIMEOUT_CODE;
            break;
        }
        if (p == 0) {
            store_empty(a, pt);
            __syncthreads();
            continue;
        }
        // double-float -> FP64 in place; b = S's from the member threads
        for (int i = tid; i < m * lda; i += CALC_NT) {
            float2 v2 = ((float2*)Macc)[i];
            Macc[i] = (double)v2.x + (double)v2.y;
        }
        if (tid < m) b[tid] = (double)proc.bhi + (double)proc.blo;
        __syncthreads();
        const double trss = la::block_sum<CALC_NT>(tid < m ? Macc[tid * lda + tid] : 0.0, red);
        if (tid < m) Macc[tid * lda + tid] += 1.0;
        __syncthreads();
        // the per-type pass reuses the operand tiles as its FP64 chunk buffer
        solve_point(a, pt, p, ms.kc, qx, qy, qz, Macc, X, lda, b, trss, d, e, cs, sn, v, s, (double*)tileH, m);
        if (a.want_diag && a.ntypes > 1) {
            for (int i = tid; i < 2 * MX_ROWS * kcm; i += CALC_NT) tileH[i] = 0.0f;
            __syncthreads();
        }
    }
    __syncthreads();
    if (wid == 0) tc::tmem_dealloc(*tslot, tcols);
}

template <int HB>
static enkfg_status launch_mixed_hb(enkfg_ctx* ctx, CalcArgs& a, int kcm, int N, uint32_t tcols, size_t smem,
                                    cudaStream_t st)
{
    CK(cudaFuncSetAttribute(k_transforms_mixed<HB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int grid = a.nitems;
    if (a.persistent) {
        int per_sm = 0, nsm = 0;
        CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_transforms_mixed<HB>, CALC_NT, smem));
        CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, ctx->device));
        if (per_sm < 1) per_sm = 1;
        // TMEM: at most 512 columns per SM across resident CTAs
        while (per_sm > 1 && (uint32_t)per_sm * tcols > 512) --per_sm;
        grid = per_sm * nsm;
        if (grid > a.nitems) grid = a.nitems;
    }
    if (grid < 1) return ENKFG_OK;
    k_transforms_mixed<HB><<<grid, CALC_NT, smem, st>>>(a, kcm, N, tcols);
    CKL();
    return ENKFG_OK;
}

enkfg_status launch_mixed(enkfg_ctx* ctx, CalcArgs& a, cudaStream_t st)
{
    const int m = a.m;
    const bool need_x = (a.mode == ENKFG_MODE_ENOI || a.scheme == ENKFG_SCHEME_DENKF);
    const int N = (m + 15) / 16 * 16;
    uint32_t tcols = 32;
    while ((int)tcols < MX_NA * N) tcols <<= 1;
    const int kcm = 8 * MX_NA;
    size_t smem = mixed_smem_bytes(m, kcm, need_x);
    if (smem > 227 * 1024) {
        set_err(ctx, "mixed path: nmem = %d needs %zu bytes of shared memory", m, smem);
        return ENKFG_EUNSUPPORTED;
    }
    // the per-type pass's FP64 chunk buffer (kcm x m doubles) lives in the tiles
    if (tcols > 512 || (size_t)kcm * m * 8 > 2 * (size_t)MX_ROWS * kcm * 4) {
        set_err(ctx, "mixed path: tile too small for the per-type pass");
        return ENKFG_EUNSUPPORTED;
    }
    const int hb = ((N >> 1) + 7) / 8;
    if (hb <= 2) return launch_mixed_hb<2>(ctx, a, kcm, N, tcols, smem, st);
    if (hb <= 3) return launch_mixed_hb<3>(ctx, a, kcm, N, tcols, smem, st);
    if (hb <= 4) return launch_mixed_hb<4>(ctx, a, kcm, N, tcols, smem, st);
    if (hb <= 6) return launch_mixed_hb<6>(ctx, a, kcm, N, tcols, smem, st);
    return launch_mixed_hb<8>(ctx, a, kcm, N, tcols, smem, st);
}
