// calc_mixed.cu -- mixed-precision local-analysis transforms: S'S and S's on
// the 5th-generation tensor cores (tcgen05, TF32 inputs, FP32 accumulation in
// tensor memory), everything else in FP64 as in calc.cu.
//
// Per round (chunk) of kc = 32 local observations:
//   * the tapered rows of S (m members) are written to shared memory as a
//     K-major operand tile (rows = members, K = observations), split into
//     TF32 hi = rn(v) and lo = rn(v - hi), and kept as FP32 for S's;
//   * one thread issues, for each group of 8 observations, three MMAs of
//     shape M=128 x N x 8 (N = m rounded up to 16): hi*hi' into the group's
//     TMEM accumulator, hi*lo' + lo*hi' into the round's cross-term one.  A
//     and B are the same tile, so together they are the round's S'S;
//   * the MMAs' completion is signalled by tcgen05.commit on the round's
//     mbarrier.  Operand tiles are double buffered: while the tensor cores
//     work on round c the CTA stages round c+1, then reads round c's
//     accumulators out of TMEM (tcgen05.ld) and adds them, with error-free
//     TwoSum steps, to double-float (hi + lo FP32) register accumulators.
//     Each group of 8 observations has its own hi*hi' accumulator (nhh = 4
//     per round, 2 when N > 96), so hi*hi' products are not summed inside
//     the tensor core, whose FP32 accumulation truncates; the error stays at
//     the level of the split itself (about 2^-22 relative per product);
//   * S's is accumulated on the CUDA cores from the staged FP32 values, one
//     member per thread, with TwoProduct/TwoSum compensated FP32
//     (double-float) arithmetic.
//
// The accumulators are then converted to FP64 and go through the same FP64
// solve as the plain path (Householder + QL for ETKF, the symmetric sweep
// inverse for DEnKF/EnOI).
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

#define MX_KC 32            // observations per round
#define MX_WIN 256          // observations per exact hi*hi' window (|k| <= 256: sums < 2^24 quanta)

// Operand pieces per round: tapered value v = hi + mid + lo with hi = k q_r
// (k integer, |k| <= 256, q_r the member's power-of-two quantum), mid =
// tf32(v - hi), lo = tf32(v - hi - mid).
#define MX_PIECES 3

struct MixedShared {
    float* tile[2][MX_PIECES]; // [buffer][piece]: N rows x kc, core-matrix layout
    float* tileV;          // [kc][ldv] tapered S of the round being staged (FP32)
    int ldv;               // row stride of tileV: >= m, = 8 mod 32 (conflict-free staging)
    const float* qs;       // [2][m]: quantum q_r and 1/q_r
    float2* Macc;          // [m x lda] double-float S'S (later reused as FP64)
    int lda;
    float* sl;             // [kc] tapered innovations of the round
    uint64_t* mbar;        // [2] one per operand buffer
    uint32_t taddr;
    int N;                 // MMA N (m rounded up to 16)
    int kc;                // observations per round
    int* err;              // shared error flag
};

// error-free (TwoSum) accumulation of x into the double-float (a.x + a.y)
__device__ __forceinline__ void df_add(float2& a, float x)
{
    float s = a.x + x;
    float bp = s - a.x;
    float e = (a.x - (s - bp)) + (x - bp);
    a.x = s;
    a.y += e;
}

// mbarrier bookkeeping of the two operand buffers, kept across points:
// parity of the next completion to wait for, and whether a commit is
// outstanding
struct MixedSync {
    uint32_t phase[2];
    bool outstanding[2];
};

// HB: 8-column blocks of S'S each thread drains (half of the N columns of its
// TMEM lane).  The double-float S'S lives in shared memory (Macc, m x lda
// float2): a thread adds its own (row, column) entries at each drain, so no
// registers are held across the point.
//
// TMEM: two accumulator sets (windows alternate), each [hi*hi' | rest] of N
// columns: set s at columns 2 s N (hi*hi') and (2 s + 1) N (the other five
// products).  A window collects up to MX_WIN observations; its hi*hi' sum is
// exact in FP32 (every product is a multiple of q_r q_s below 2^16 of them),
// the rest is 2^-8 of it or less.  A closed window is drained (tcgen05.ld,
// TwoSum into Macc) one round later, while the next window runs.
template <int HB>
struct GramProcTC {
    const CalcArgs& a;
    const PointScratch& s;
    MixedShared& ms;
    MixedSync& sy;
    uint32_t& rnd;     // rounds issued by this CTA (all points): operand buffer = rnd & 1
    int win;           // current window's accumulator set
    int win_obs;       // observations in the current window
    int drain_set;     // closed window awaiting its drain (-1: none)
    int drain_buf;     // operand buffer whose commit closes it
    float bh[4], bl[4]; // S's for member threadIdx.x: four double-float partial sums
    __device__ __forceinline__ GramProcTC(const CalcArgs& a_, const PointScratch& s_, MixedShared& ms_, MixedSync& sy_,
                                          uint32_t& rnd_)
        : a(a_), s(s_), ms(ms_), sy(sy_), rnd(rnd_), win(0), win_obs(0), drain_set(-1), drain_buf(0)
    {
        for (int j = 0; j < 4; ++j) bh[j] = bl[j] = 0.0f;
    }

    // bounded wait for the outstanding commit of operand buffer `buf`; on
    // expiry record the error and wait once more (bounded), so that nothing
    // is in flight when TMEM is released.  Ends with a barrier, so every
    // thread sees the same error flag.
    __device__ __forceinline__ void wait_buf(int buf)
    {
        if (sy.outstanding[buf]) {
            bool done = tc::mbar_wait_bounded(ms.mbar + buf, sy.phase[buf]);
            if (!done) {
                atomicExch(ms.err, 1);
                tc::mbar_wait_bounded(ms.mbar + buf, sy.phase[buf]);
            }
            sy.phase[buf] ^= 1u;
            sy.outstanding[buf] = false;
        }
        tc::fence_after();
        __syncthreads();
    }

    // add accumulator set `set` to the shared double-float S'S (its MMAs
    // have completed); thread (warp w, lane l) owns row 32 (w % 4) + l and
    // columns (w / 4) N/2 + [0, N/2)
    __device__ __forceinline__ void read_set(int set)
    {
        const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
        if (*ms.err) return;
        const int r = 32 * (wid & 3) + lane;
        if (32 * (wid & 3) < a.m) {
            const int half = ms.N >> 1;
            const int c0 = (wid >> 2) * half;
            const uint32_t base = ms.taddr + ((uint32_t)(32 * (wid & 3)) << 16) + (uint32_t)(2 * set * ms.N + c0);
            float2* row = ms.Macc + (size_t)(r < a.m ? r : 0) * ms.lda;
#pragma unroll
            for (int b = 0; b < HB; ++b)
                if (8 * b < half) {
                    uint32_t vh[8], vr[8];
                    tc::tmem_ld8_nowait(base + (uint32_t)(8 * b), vh);
                    tc::tmem_ld8_nowait(base + (uint32_t)(ms.N + 8 * b), vr);
                    tc::tmem_wait_ld();
                    if (r < a.m) {
#pragma unroll
                        for (int j = 0; j < 8; ++j) {
                            const int c = c0 + 8 * b + j;
                            if (c < a.m) {
                                float2 acc = row[c];
                                df_add(acc, __uint_as_float(vh[j]));
                                acc.y += __uint_as_float(vr[j]);   // <= 2^-8 of hi*hi'
                                row[c] = acc;
                            }
                        }
                    }
                }
        }
        tc::fence_before();
    }

    __device__ void chunk(int nc, int t)
    {
        const int tid = threadIdx.x;
        const int m = a.m, kc = ms.kc;
        const bool tsum = a.want_diag && a.ntypes > 1;
        double ssq = 0.0;
        if (*ms.err) return;
        const int buf = (int)(rnd & 1u);
        // 0. this operand buffer's previous MMAs were waited for at the end of
        //    the last round (this only acts on the first round after an error)
        if (sy.outstanding[buf]) {
            wait_buf(buf);
            if (*ms.err) return;
        }
        float* tH = ms.tile[buf][0];
        float* tM = ms.tile[buf][1];
        float* tL = ms.tile[buf][2];
        // 1. tapered S rows of the round: hi / mid / lo pieces into this
        //    round's operand tiles, FP32 copy for S's; tapered innovations
        const float* lcf = reinterpret_cast<const float*>(s.llc);   // FP32 taper (enumerate_obs<1 or 2>)
        const float* q = ms.qs;
        const float* iq = ms.qs + m;
        if (tid < kc) ms.sl[tid] = (tid < nc) ? (float)a.ss[s.lid[tid]] * lcf[tid] : 0.0f;
        // one warp per core matrix (8 rows x 4 observations = 128 bytes):
        // lane -> row r&7 = lane>>2, observation k&3 = lane&3, so the three
        // piece stores are conflict-free; rows >= m stay zero.  (Two copies of
        // the loop: an FP64 sum under a runtime flag inside the common loop
        // would issue on the FP64 pipe even when off.)
        {
            const int lane = tid & 31, wid = tid >> 5;
            const int nrg = (m + 7) >> 3, nkg = kc >> 2, ncm = nrg * nkg;
            const int ldv = ms.ldv;
            if (tsum) {
                for (int c = wid; c < ncm; c += CALC_NT / 32) {
                    const int rg = c / nkg, kg = c - rg * nkg;
                    const int r = (rg << 3) + (lane >> 2), k = (kg << 2) + (lane & 3);
                    if (r < m) {
                        float v = 0.0f;
                        if (k < nc) {
                            v = __fmul_rn(__ldg(a.St + (size_t)s.lid[k] * a.mpad + r), lcf[k]);
                            ssq += (double)v * (double)v;
                        }
                        const float hi = __fmul_rn(rintf(__fmul_rn(v, iq[r])), q[r]);
                        const float r1 = __fsub_rn(v, hi);
                        const float md = tc::to_tf32(r1);
                        const int off = (c << 5) + lane;
                        tH[off] = hi;
                        tM[off] = md;
                        tL[off] = tc::to_tf32(__fsub_rn(r1, md));
                        ms.tileV[k * ldv + r] = v;
                    }
                }
            } else {
                for (int c = wid; c < ncm; c += CALC_NT / 32) {
                    const int rg = c / nkg, kg = c - rg * nkg;
                    const int r = (rg << 3) + (lane >> 2), k = (kg << 2) + (lane & 3);
                    if (r < m) {
                        float v = 0.0f;
                        if (k < nc) v = __fmul_rn(__ldg(a.St + (size_t)s.lid[k] * a.mpad + r), lcf[k]);
                        const float hi = __fmul_rn(rintf(__fmul_rn(v, iq[r])), q[r]);
                        const float r1 = __fsub_rn(v, hi);
                        const float md = tc::to_tf32(r1);
                        const int off = (c << 5) + lane;
                        tH[off] = hi;
                        tM[off] = md;
                        tL[off] = tc::to_tf32(__fsub_rn(r1, md));
                        ms.tileV[k * ldv + r] = v;
                    }
                }
            }
        }
        tc::fence_async_smem();
        __syncthreads();
        // 2. one thread issues the round's MMAs into the current window's
        //    set: hi*hi' into the exact accumulator, the five other products
        //    (hi*mid', mid*hi', hi*lo', lo*hi', mid*mid') into the rest.  A
        //    and B are the same tiles; A has 128 rows, of which rows >= N
        //    read the padding behind the tiles and land in accumulator rows
        //    that are never read.
        const int ngroups = (nc + 7) / 8;
        // the issuing thread is in the last warp, so that S's (threads < m)
        // runs at the same time
        if (tid == CALC_NT - 32) {
            tc::fence_after();
            const uint32_t sbo = (uint32_t)kc * 32u, idesc = tc::idesc_tf32(MX_ROWS, ms.N);
            const uint32_t dhh = ms.taddr + (uint32_t)(2 * win * ms.N), dr = dhh + (uint32_t)ms.N;
            const uint32_t h0 = tc::smem_u32(tH), m0 = tc::smem_u32(tM), l0 = tc::smem_u32(tL);
            for (int g = 0; g < ngroups; ++g) {
                const uint32_t off = (uint32_t)g * 256u;    // two 128-byte core matrices per group of 8
                const uint64_t dh = tc::desc_kmajor_noswizzle(h0 + off, 128u, sbo);
                const uint64_t dm = tc::desc_kmajor_noswizzle(m0 + off, 128u, sbo);
                const uint64_t dl = tc::desc_kmajor_noswizzle(l0 + off, 128u, sbo);
                const uint32_t fresh = (win_obs == 0 && g == 0) ? 0u : 1u;
                tc::mma_tf32(dhh, dh, dh, idesc, fresh);
                tc::mma_tf32(dr, dh, dm, idesc, fresh);
                tc::mma_tf32(dr, dm, dh, idesc, 1u);
                tc::mma_tf32(dr, dh, dl, idesc, 1u);
                tc::mma_tf32(dr, dl, dh, idesc, 1u);
                tc::mma_tf32(dr, dm, dm, idesc, 1u);
            }
            tc::commit(ms.mbar + buf);
        }
        sy.outstanding[buf] = true;
        ++rnd;
        // 3. S's from the staged FP32 values (compensated FP32, four
        //    independent double-float partial sums for ILP)
        if (tid < m) {
            // unrolled by 4 (static partial-sum index; tileV and sl are zero
            // past nc, so the padded tail adds nothing)
            const int nc4 = (nc + 3) & ~3;
            for (int k0 = 0; k0 < nc4; k0 += 4) {
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const int k = k0 + j;
                    const float v = ms.tileV[k * ms.ldv + tid];
                    const float x = ms.sl[k];
                    const float p = v * x, pe = fmaf(v, x, -p);
                    const float sm = bh[j] + p, bp = sm - bh[j];
                    bl[j] += ((bh[j] - (sm - bp)) + (p - bp)) + pe;
                    bh[j] = sm;
                }
            }
        }
        // 4. the window closed one round ago: its last commit is on the other
        //    buffer; drain it while this round's MMAs run
        if (drain_set >= 0) {
            wait_buf(drain_buf);
            read_set(drain_set);
            drain_set = -1;
        }
        // 5. close the current window when the next round might overflow it
        win_obs += nc;
        if (win_obs + kc > MX_WIN) {
            drain_set = win;
            drain_buf = buf;
            win ^= 1;
            win_obs = 0;
        }
        if (tsum) {
            double v = la::block_sum<CALC_NT>(ssq, s.red);
            if (tid == 0) s.tss[t] += v;
        }
        // 6. the previous round's MMAs (the other operand buffer, which the
        //    next round stages into) ran during this round: wait for them
        //    here, under the round's closing barrier
        if (sy.outstanding[buf ^ 1]) {
            bool done = tc::mbar_wait_bounded(ms.mbar + (buf ^ 1), sy.phase[buf ^ 1]);
            if (!done) {
                atomicExch(ms.err, 1);
                tc::mbar_wait_bounded(ms.mbar + (buf ^ 1), sy.phase[buf ^ 1]);
            }
            sy.phase[buf ^ 1] ^= 1u;
            sy.outstanding[buf ^ 1] = false;
            tc::fence_after();
        }
        __syncthreads();
    }
    // drain what is left (after the enumeration; also after an error, so that
    // no MMA is in flight when TMEM is released)
    __device__ __forceinline__ void finish()
    {
        wait_buf(0);
        wait_buf(1);
        if (drain_set >= 0) read_set(drain_set);
        if (win_obs > 0) read_set(win);
        drain_set = -1;
        win_obs = 0;
        __syncthreads();
    }
    __device__ __forceinline__ void type_end(int) {}
};

// operand tiles: 2 buffers x 3 pieces x N rows x kc, then the padding that
// the 128-row A operand reads past the last tile (rows >= N, never used)
static __host__ __device__ size_t mixed_tile_floats(int m, int kc)
{
    const int N = (m + 15) / 16 * 16;
    return (size_t)2 * MX_PIECES * N * kc + (size_t)(MX_ROWS - N) * kc;
}

static size_t mixed_smem_bytes(int m, int kc)
{
    int lda = (m % 2 == 0) ? m + 1 : m + 2;
    size_t s = 0;
    s += mixed_tile_floats(m, kc) * 4;                     // operand tiles + padding
    s += (size_t)kc * (m + ((8 - m % 32) % 32 + 32) % 32) * 4;   // FP32 staged values (row stride = 8 mod 32)
    s += (size_t)2 * m * 4;                                // quantum q, 1/q
    s += (size_t)m * lda * 8;                              // Macc (also A)
    s += (size_t)kc * 4;                                   // tapered innovations
    s += (size_t)6 * (m + 1) * 8;                          // b d e cs sn v
    s += (size_t)ENKFG_MAXTYPES * 8 * 2;
    s += (size_t)(CALC_NT / 32) * 8;
    s += (size_t)LIST_EXTRA * 8;                           // llc
    s += (size_t)LIST_EXTRA * 4;                           // lid
    s += (size_t)ENKFG_MAXTYPES * 4;
    s += 256;                                              // control ints
    s += 64;                                               // mbarriers, tmem slot, flags
    return s;
}

template <int HB>
__global__ void __launch_bounds__(CALC_NT) k_transforms_mixed(CalcArgs a, int kcm, int N, uint32_t tcols)
{
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const int tid = threadIdx.x, wid = tid >> 5;
    const int m = a.m, lda = (m % 2 == 0) ? m + 1 : m + 2;   // odd stride: fewer bank conflicts
    const size_t ntile = mixed_tile_floats(m, kcm);         // [2][3][N x kc] + padding for A's rows >= N
    unsigned char* sp = smem_raw;
    float* tiles = (float*)sp;        sp += ntile * 4;
    const int ldv = m + ((8 - m % 32) % 32 + 32) % 32;        // >= m, = 8 mod 32
    float* tileV = (float*)sp;        sp += (size_t)kcm * ldv * 4;
    float* qs = (float*)sp;           sp += (size_t)2 * m * 4;
    sp = (unsigned char*)(((uintptr_t)sp + 15) & ~(uintptr_t)15);
    double* Macc = (double*)sp;       sp += (size_t)m * lda * 8;
    float* sl = (float*)sp;           sp += (size_t)((kcm + 3) & ~3) * 4;
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
    uint64_t* mbar = (uint64_t*)sp;   sp += 8 * 2;
    uint32_t* tslot = (uint32_t*)sp;  sp += 8;
    int* err = (int*)sp;
    const PointScratch s{ lid, llc, ictl, tcount, tss, tpd, red };
    const size_t piece = (size_t)N * kcm;

    // set-up: TMEM columns, mbarriers, zeroed operand tiles, the quantum
    if (wid == 0) tc::tmem_alloc(tslot, tcols);
    if (tid == 0) {
        for (int i = 0; i < 2; ++i) tc::mbar_init(mbar + i, 1);
        *err = 0;
    }
    for (size_t i = tid; i < ntile; i += CALC_NT) tiles[i] = 0.0f;
    for (int r = tid; r < m; r += CALC_NT) {
        qs[r] = a.qscale[r];
        qs[m + r] = a.qscale[ENKFG_MAXMEM + r];
    }
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    MixedShared ms{ { { tiles, tiles + piece, tiles + 2 * piece }, { tiles + 3 * piece, tiles + 4 * piece, tiles + 5 * piece } },
                    tileV, ldv, qs, (float2*)Macc, lda, sl, mbar, *tslot, N, kcm, err };
    MixedSync sy{ { 0u, 0u }, { false, false } };
    uint32_t rnd = 0;

    for (int it = 0;; ++it) {
        const int idx = next_item(a, it, ictl);
        if (idx < 0 || *err) break;
        const int pt = a.order ? a.order[idx] : a.item0 + idx;
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
        GramProcTC<HB> proc(a, s, ms, sy, rnd);
        const int p = (a.sxf != nullptr && a.ndim == 2) ? enumerate_obs<2>(a, ms.kc, qx, qy, qz, s, proc, true)
                                                        : enumerate_obs<1>(a, ms.kc, qx, qy, qz, s, proc, true);
        proc.finish();
        __syncthreads();
        if (*err) {
            if (tid == 0) a.status[pt] = MX_TIMEOUT_CODE;
            break;
        }
        if (p == 0) {
            store_empty(a, pt);
            if (a.defer && tid == 0) a.eaux[2 * (size_t)idx] = 0.0;
            __syncthreads();
            continue;
        }
        // double-float -> FP64 in place; b = S's from the member threads
        for (int i = tid; i < m * lda; i += CALC_NT) {
            float2 v2 = ((float2*)Macc)[i];
            Macc[i] = (double)v2.x + (double)v2.y;
        }
        if (tid < m)
            b[tid] = (((double)proc.bh[0] + (double)proc.bh[1]) + ((double)proc.bh[2] + (double)proc.bh[3])) +
                     (((double)proc.bl[0] + (double)proc.bl[1]) + ((double)proc.bl[2] + (double)proc.bl[3]));
        __syncthreads();
        const double trss = la::block_sum<CALC_NT>(tid < m ? Macc[tid * lda + tid] : 0.0, red);
        if (tid < m) Macc[tid * lda + tid] += 1.0;
        __syncthreads();
        // the per-type pass reuses the operand tiles as its FP64 chunk buffer
        solve_point(a, pt, idx, p, ms.kc, qx, qy, qz, Macc, lda, b, trss, d, e, cs, sn, v, s, (double*)tiles, m);
        if (a.want_diag && a.ntypes > 1) {
            for (size_t i = tid; i < ntile; i += CALC_NT) tiles[i] = 0.0f;
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
    CK(cudaFuncSetAttribute(k_transforms_mixed<HB>, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared));
    int grid = a.nitems;
    if (a.persistent) {
        // computed residency (the occupancy query reports one CTA per SM here)
        int per_sm = 0, nsm = 0;
        enkfg_status s = resident_ctas(ctx, (const void*)k_transforms_mixed<HB>, CALC_NT, smem, &per_sm);
        if (s) return s;
        CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, ctx->device));
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
    const int N = (m + 15) / 16 * 16;
    uint32_t tcols = 32;
    while ((int)tcols < 4 * N) tcols <<= 1;              // two windows x (hi*hi' | rest)
    const int kcm = MX_KC;
    size_t smem = mixed_smem_bytes(m, kcm);
    if (smem > 227 * 1024) {
        set_err(ctx, "mixed path: nmem = %d needs %zu bytes of shared memory", m, smem);
        return ENKFG_EUNSUPPORTED;
    }
    // the per-type pass's FP64 chunk buffer (kcm x m doubles) lives in the tiles
    if (tcols > 512 || (size_t)kcm * m * 8 > mixed_tile_floats(m, kcm) * 4) {
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
