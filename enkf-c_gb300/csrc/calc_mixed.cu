// calc_mixed.cu -- mixed-precision local-analysis transforms: S'S on the
// 5th-generation tensor cores (tcgen05, TF32 inputs, FP32 accumulation in
// tensor memory), S's in compensated FP32 on the CUDA cores, everything else
// in FP64 as in calc.cu.
//
// Per local analysis (one CTA, persistent over a work queue):
//   * the search appends accepted observations (position, FP32 taper) to a
//     list segment of up to ~1000 entries; each full segment is consumed in
//     rounds of kc = 32 observations before the search goes on;
//   * the S rows of round j + 1 (mpad floats per observation) and their
//     innovations are copied into shared memory with cp.async while round j
//     is split and multiplied, so no round waits for its L2 gathers;
//   * a round's tapered values v are split into hi = rint(v / q_r) q_r (q_r
//     a power-of-two quantum per member, |hi / q_r| <= 256), mid = tf32(v -
//     hi) and lo = tf32(v - hi - mid), written as K-major operand tiles;
//   * one thread issues, per group of 8 observations, six MMAs of shape
//     M=128 x N x 8 (N = m rounded up to 16): hi*hi' into an exact
//     accumulator and hi*mid' + mid*hi' + hi*lo' + lo*hi' + mid*mid' into a
//     second one.  Windows of up to 256 observations keep the hi*hi' sum
//     exact in FP32 (every term is a multiple of q_r q_s, below 2^24 of
//     them in total);
//   * two TMEM accumulator sets alternate between windows; a closed window
//     is read out (tcgen05.ld) one round later, while the next window's
//     MMAs run, and added with TwoSum steps to a double-float (hi + lo FP32)
//     S'S in shared memory;
//   * operand tiles are double buffered: the MMAs of round j run while round
//     j + 1 is staged; completion is signalled by tcgen05.commit on the
//     buffer's mbarrier.
//
// The double-float S'S is then converted to FP64 and goes through the same
// FP64 solve as the plain path (Householder + QL for ETKF, the symmetric
// sweep inverse for DEnKF/EnOI), or, deferred, is handed to the batched
// solves through a slot in global memory.
//
// The compact deferred form (DF, 64 < m <= 96) differs so that two CTAs fit
// on an SM: rounds of 16 observations; one TMEM accumulator set, a window
// drained at the end of the round that closes it; the S'S upper triangle in
// rectangular packing; each round's MMAs issued at the start of the next
// round, while that round is split; S's fused into the split (split_vec).
//
// Shared-memory operand layout (canonical K-major, no swizzle): core matrices
// of 8 rows x 16 bytes (4 TF32) stored as 128 contiguous bytes; core matrix
// (row group g, K group q) at (g * kc/4 + q) * 128 bytes.  Descriptor:
// leading (K) byte offset 128, stride (row-group) byte offset kc*32.  DF:
// 64-byte swizzled rows of the round's 16 observations (tc.cuh).
//
// Every wait on an MMA mbarrier is bounded; on expiry the CTA records an
// error status for the point, stops, releases its TMEM and returns.
#include "calc_common.cuh"
#include "tc.cuh"

#define MX_ROWS 128
// Bound on a wait for the tensor cores: the context's limit (a.wait_ns,
// enkfg_set_wait_limit, 2 s by default) for the first wait; after it expires
// the drain before TMEM is released waits at most MX_WAIT_NS, whatever the
// limit, so that no MMA is in flight when its TMEM is freed.
#define MX_WAIT_NS ENKFG_DEFAULT_WAIT_NS
#define MX_TIMEOUT_CODE ENKFG_POINT_TIMEOUT


#define MX_KC 32            // observations per round
#define MX_WIN 256          // observations per exact hi*hi' window (|k| <= 256: sums < 2^24 quanta)

// Operand pieces per round: tapered value v = hi + mid + lo with hi = k q_r
// (k integer, |k| <= 256, q_r the member's power-of-two quantum), mid =
// tf32(v - hi), lo = tf32(v - hi - mid).
#define MX_PIECES 3

// (Base pointers and strides rather than arrays of pointers: an array indexed
// by the buffer number would live in local memory.)
struct MixedShared {
    float* tiles;          // [buffer][piece][N x kc], core-matrix layout
    int piece;             // floats per piece tile
    float* raw;            // [buffer][kcm][ldv] untapered S rows of a round (cp.async)
    int rawsz;             // floats per raw buffer
    float* sraw;           // [buffer][kcm] innovations of those observations, float (cp.async)
    int kcm;
    int ldv;               // row stride of raw: >= mpad, = 8 mod 32 (conflict-free reads)
    const float* qs;       // [2][m]: quantum q_r and the rounding constant 1.5 2^23 q_r
    float2* Macc;          // [m x lda] double-float S'S (later reused as FP64)
    float* Mrest;          // [m x lda] stacked form: the remainder products from the offset lanes
    int lda;
    int stacked;           // tile order [hi mid lo Z] [lo hi mid] (else [hi mid lo] x 2)
    uint64_t* mbar;        // [2] one per operand buffer
    uint32_t taddr;
    int N;                 // MMA N (m rounded up to 16)
    int kc;                // observations per round
    int* err;              // shared error flag
    __device__ __forceinline__ float* tile(int buf, int pc) const
    {
        const int idx = stacked ? (buf == 0 ? pc : (pc == 2 ? 4 : 5 + pc)) : buf * MX_PIECES + pc;
        return tiles + idx * piece;
    }
    __device__ __forceinline__ float* zblock() const { return tiles + 3 * piece; }   // stacked: N zero rows
    __device__ __forceinline__ float* rawb(int rb) const { return raw + rb * rawsz; }
    __device__ __forceinline__ float* srawb(int rb) const { return sraw + rb * kcm; }
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

// mbarrier bookkeeping of the two operand buffers, kept across points: bit
// b of `phase` is the parity of buffer b's next completion, bit b of `out`
// says whether a commit on it is outstanding
struct MixedSync {
    uint32_t phase;
    uint32_t out;
    __device__ __forceinline__ bool outstanding(int b) const { return (out >> b) & 1u; }
    __device__ __forceinline__ uint32_t parity(int b) const { return (phase >> b) & 1u; }
    __device__ __forceinline__ void completed(int b)
    {
        phase ^= 1u << b;
        out &= ~(1u << b);
    }
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
// ST: stacked products (N <= 64) -- A = [hi; mid] takes two pieces in one
// MMA: per group of 8 observations hi*[hi; mid]' into the first accumulator
// (rows < N: hi*hi', exact; rows N..2N-1: mid*hi'), mid and lo times [hi;
// mid]' and lo*hi' (A = [lo; Z] or [Z; lo]) into the second: four MMAs
// instead of six, and row r's remainder is acc1[N+r] + acc2[r] + acc2[N+r]
// (mid*lo' included).
// FS: S's fused into the split -- each thread multiplies its observation's
// tapered innovation into every row it splits and keeps a double-float sum
// per row (2 HB rows at most) in registers for the whole point; otherwise
// S's is a separate pass over the staged rows by thread groups.
// DF: compact form of the deferred solve -- one TMEM accumulator set (2N
// columns) and the upper triangle of the double-float S'S packed in shared
// memory, so that two CTAs fit on an SM; a window is drained at the end of
// the round that closes it, after that round's MMAs, before the next round's
// MMAs overwrite the set.
template <int HB, bool FS, bool ST, bool DF>
struct GramProcTC {
    const CalcArgs& a;
    const PointScratch& s;
    MixedShared& ms;
    MixedSync& sy;
    uint32_t& rnd;     // rounds of this point so far: operand buffer = rnd & 1
    int win;           // current window's accumulator set
    int win_obs;       // observations in the current window
    int drain_set;     // closed window awaiting its drain (-1: none)
    int drain_buf;     // operand buffer whose commit closes it
    int sgroups;       // S's observation groups (warps 0 .. 6; the last warp issues the MMAs)
    int s_g, s_q;      // this thread's group and quad of members (4 s_q .. 4 s_q + 3)
    float bh[4], bl[4]; // S's of those four members over group s_g: double-float sums
    // S's fused into the vectorised split: one double-float sum per (member,
    // K group) pair the thread splits (the pairs stay the thread's for the
    // whole point)
    static constexpr int NSLOT = FS ? 1 : (8 * 16 * HB + CALC_NT - 1) / CALC_NT;
    float vh[NSLOT], vl[NSLOT];
    // DF: the batch staged last round, whose MMAs are issued at the start of
    // the next round (while that round is split), and whether the window
    // closes with it
    bool pend, drain_after;
    int pend_buf, pend_nc;
    float fh[FS ? 2 * HB : 1], fl[FS ? 2 * HB : 1];   // fused S's: per row slot
    __device__ __forceinline__ GramProcTC(const CalcArgs& a_, const PointScratch& s_, MixedShared& ms_, MixedSync& sy_,
                                          uint32_t& rnd_)
        : a(a_), s(s_), ms(ms_), sy(sy_), rnd(rnd_), win(0), win_obs(0), drain_set(-1), drain_buf(0), pend(false),
          drain_after(false), pend_buf(0), pend_nc(0)
    {
        const int nq = (a.m + 3) >> 2;
        sgroups = (CALC_NT - 32) / nq;
        s_g = (int)threadIdx.x / nq;
        s_q = (int)threadIdx.x - s_g * nq;
#pragma unroll
        for (int i = 0; i < (FS ? 2 * HB : 1); ++i) fh[i] = fl[i] = 0.0f;
        for (int j = 0; j < 4; ++j) bh[j] = bl[j] = 0.0f;
#pragma unroll
        for (int j = 0; j < NSLOT; ++j) vh[j] = vl[j] = 0.0f;
    }

    // bounded wait for the outstanding commit of operand buffer `buf`; on
    // expiry record the error and wait once more (bounded), so that nothing
    // is in flight when TMEM is released.  With `sync` it ends with a
    // barrier, so every thread sees the same error flag (without, the
    // caller's next barrier does that).
    __device__ __forceinline__ void wait_buf(int buf, bool sync = true)
    {
        if (sy.outstanding(buf)) {
            bool done = tc::mbar_wait_bounded(ms.mbar + buf, sy.parity(buf), a.wait_ns);
            if (!done) {
                atomicExch(ms.err, 1);
                tc::mbar_wait_bounded(ms.mbar + buf, sy.parity(buf), MX_WAIT_NS);
            }
            sy.completed(buf);
        }
        tc::fence_after();
        if (sync) __syncthreads();
    }

    // element (r, c >= r) of the upper triangle (DF) is at e0 + es c:
    // rectangular packing in ceil(m/2) lines of L = m + 1 rounded up to
    // even, line t holding row t and, reversed, row m - 1 - t.  A warp's
    // 32 rows at one column then step by L - 1 (odd) float2 elements, so
    // the drain's accesses do not share banks.
    __device__ __forceinline__ void tri(int r, int& e0, int& es) const
    {
        const int m = a.m, L1 = ((m + 2) & ~1) - 1;
        if (2 * r < m) {
            e0 = r * L1;
            es = 1;
        } else {
            e0 = (m - 1 - r) * L1 + 2 * m - 1;
            es = -1;
        }
    }

    // add accumulator set `set` to the shared double-float S'S (its MMAs
    // have completed); thread (warp w, lane l) owns row 32 (w % 4) + l and
    // columns (w / 4) N/2 + [0, N/2).  The TMEM loads of two 8-column
    // blocks (both accumulators) are issued before one wait.  DF: only c >=
    // r, and blocks wholly below the diagonal are not loaded.
    __device__ __forceinline__ void read_set(int set)
    {
        const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
        if (*ms.err) return;
        const int rq = 32 * (wid & 3), r = rq + lane;
        // stacked: lanes N..N+m-1 hold remainder products of row r - N
        const int lanes = ST ? ms.N + a.m : a.m;
        const int half = ms.N >> 1;
        const int c0 = (wid >> 2) * half;
        if (rq < lanes && !(DF && rq >= c0 + half)) {
            const uint32_t base = ms.taddr + ((uint32_t)rq << 16) + (uint32_t)(2 * set * ms.N + c0);
            const bool direct = r < a.m;
            const bool offset = ST && r >= ms.N && r < ms.N + a.m;
            int e0 = 0, es = 1;
            if (DF) tri(direct ? r : 0, e0, es);
            else e0 = direct ? r * ms.lda : 0;
            float* rrow = ST ? ms.Mrest + (size_t)(offset ? r - ms.N : 0) * ms.lda : nullptr;
            constexpr int BB = 1;
#pragma unroll
            for (int b0 = 0; b0 < HB; b0 += BB) {
                if (8 * b0 >= half || (DF && c0 + 8 * (b0 + BB) <= rq)) continue;
                uint32_t vh[BB][8], vr[BB][8];
#pragma unroll
                for (int u = 0; u < BB; ++u)
                    if (b0 + u < HB && 8 * (b0 + u) < half) {
                        tc::tmem_ld8_nowait(base + (uint32_t)(8 * (b0 + u)), vh[u]);
                        tc::tmem_ld8_nowait(base + (uint32_t)(ms.N + 8 * (b0 + u)), vr[u]);
                    }
                tc::tmem_wait_ld();
#pragma unroll
                for (int u = 0; u < BB; ++u)
                    if (b0 + u < HB && 8 * (b0 + u) < half) {
                        if (direct) {
#pragma unroll
                            for (int j = 0; j < 8; ++j) {
                                const int c = c0 + 8 * (b0 + u) + j;
                                if (c < a.m && (!DF || c >= r)) {
                                    float2* el = ms.Macc + (e0 + es * c);
                                    float2 acc = *el;
                                    df_add(acc, __uint_as_float(vh[u][j]));
                                    acc.y += __uint_as_float(vr[u][j]);   // <= 2^-8 of hi*hi'
                                    *el = acc;
                                }
                            }
                        } else if (offset) {
#pragma unroll
                            for (int j = 0; j < 8; ++j) {
                                const int c = c0 + 8 * (b0 + u) + j;
                                if (c < a.m) rrow[c] += __uint_as_float(vh[u][j]) + __uint_as_float(vr[u][j]);
                            }
                        }
                    }
            }
        }
        tc::fence_before();
    }

    // issue the asynchronous copies of a round's S rows (mpad floats each,
    // 16-byte pieces) and innovations into raw buffer rb; rows past nc are
    // zeroed with plain stores
    __device__ __forceinline__ void stage_rows(const int* lid, int base, int nc, int rb)
    {
        const int tid = threadIdx.x, kc = ms.kc, m4 = a.mpad >> 2;
        float* dst = ms.rawb(rb);
        // (row k, piece c) of element i = tid + j CALC_NT, stepped without a
        // division per element
        const int dk = CALC_NT / m4, dc = CALC_NT - dk * m4;
        int k = tid / m4, c = tid - k * m4;
        for (int i = tid; i < kc * m4; i += CALC_NT) {
            float* d = dst + k * ms.ldv + 4 * c;
            if (k < nc) tc::cp_async16(d, a.St + (size_t)lid[base + k] * a.mpad + 4 * c);
            else *reinterpret_cast<float4*>(d) = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            k += dk;
            c += dc;
            if (c >= m4) {
                c -= m4;
                ++k;
            }
        }
        if (tid < kc) {
            float* d = ms.srawb(rb) + tid;
            if (tid < nc) tc::cp_async4(d, a.ssf + lid[base + tid]);
            else *d = 0.0f;
        }
        tc::cp_async_commit();
    }

    // the hi / mid / lo pieces of this thread's values in one round (and,
    // with FS, their products with the observation's tapered innovation xk
    // into the row sums); returns the sum of squares when TS
    template <bool TS>
    __device__ __forceinline__ double split_rows(float* tH, float* tM, float* tL, const float* rp, float ck, float xk,
                                                 int nrg, int nkg, int kg, int rg0, int rstep, int lane)
    {
        const int m = a.m;
        const float* cq = ms.qs + m;   // 1.5 2^23 q_r: (v + c) - c rounds v to a multiple of q_r
        double ssq = 0.0;
        // the raw values are all loaded before any piece is stored (the
        // tiles and the raw rows share shared memory, so a store would
        // otherwise keep the next load behind it), then split
        auto split = [&](int rg, int r, float raw_v) -> float {
            const float v = __fmul_rn(raw_v, ck);
            if (TS) ssq += (double)v * (double)v;
            // hi = q rint(v / q): |v| <= 256 q < 2^22 q keeps v + c in the
            // binade of c, whose spacing is q (ties to even, as rint)
            const float hi = __fsub_rn(__fadd_rn(v, cq[r]), cq[r]);
            const float r1 = __fsub_rn(v, hi);
            // mid = r1 and lo = r1 - mid rounded to TF32, to nearest with
            // ties away from zero (half a TF32 unit added to the magnitude
            // bits, then the 13 low bits cleared); cut toward zero instead,
            // both would lean the same way and their error would add up
            const float md = tc::tf32_rna(r1);
            const int off = ((rg * nkg + kg) << 5) + lane;
            tH[off] = hi;
            tM[off] = md;
            tL[off] = tc::tf32_rna(__fsub_rn(r1, md));
            return v;
        };
        if constexpr (FS) {
            float rv[2 * HB];
#pragma unroll
            for (int i = 0; i < 2 * HB; ++i) {
                const int rg = rg0 + i * rstep;
                const int r = (rg << 3) + (lane >> 2);
                rv[i] = (rg < nrg && r < m) ? rp[rg << 3] : 0.0f;
            }
#pragma unroll
            for (int i = 0; i < 2 * HB; ++i) {
                const int rg = rg0 + i * rstep;
                const int r = (rg << 3) + (lane >> 2);
                if (rg < nrg && r < m) {
                    const float v = split(rg, r, rv[i]);
                    const float p = v * xk, pe = fmaf(v, xk, -p);
                    const float sm = fh[i] + p, bp = sm - fh[i];
                    fl[i] += ((fh[i] - (sm - bp)) + (p - bp)) + pe;
                    fh[i] = sm;
                }
            }
        } else {
            int rg = rg0;
            for (; rg + 3 * rstep < nrg; rg += 4 * rstep) {
                float rv[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int r = ((rg + u * rstep) << 3) + (lane >> 2);
                    rv[u] = r < m ? rp[(rg + u * rstep) << 3] : 0.0f;
                }
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int r = ((rg + u * rstep) << 3) + (lane >> 2);
                    if (r < m) split(rg + u * rstep, r, rv[u]);
                }
            }
            for (; rg < nrg; rg += rstep) {
                const int r = (rg << 3) + (lane >> 2);
                if (r < m) split(rg, r, rp[rg << 3]);
            }
        }
        return ssq;
    }

    // S's from the staged rows of raw buffer rb (compensated FP32, not
    // fused): thread (group g, quad q) takes members 4q .. 4q + 3 (one
    // 16-byte load a row) and observations g, g + G, ... < nc, with the
    // taper and the tapered innovation formed as the fused split forms them
    __device__ __forceinline__ void ss_pass(const float* lcf, int base, int nc, int rb)
    {
        if (FS || s_g >= sgroups) return;
        const float* raw = ms.rawb(rb) + 4 * s_q;
        const float* sr = ms.srawb(rb);
        for (int k = s_g; k < nc; k += sgroups) {
            const float4 rv = *reinterpret_cast<const float4*>(raw + k * ms.ldv);
            const float c = lcf[base + k];
            const float x = __fmul_rn(sr[k], c);
            const float v[4] = { __fmul_rn(rv.x, c), __fmul_rn(rv.y, c), __fmul_rn(rv.z, c), __fmul_rn(rv.w, c) };
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const float p = v[u] * x, pe = fmaf(v[u], x, -p);
                const float sm = bh[u] + p, bp = sm - bh[u];
                bl[u] += ((bh[u] - (sm - bp)) + (p - bp)) + pe;
                bh[u] = sm;
            }
        }
    }

    // the MMAs of one staged batch (ng groups of 8 observations in operand
    // buffer buf) into the current window's set, issued by one elected lane
    // of the last warp: hi*hi' into the exact accumulator, the five other
    // products (hi*mid', mid*hi', hi*lo', lo*hi', mid*mid') into the rest
    // (stacked: four MMAs, see above).  A and B are the same tiles; A has
    // 128 rows, of which rows >= N read the padding behind the tiles and land
    // in accumulator rows that are never read.
    __device__ __forceinline__ void issue_mmas(int buf, int ngroups)
    {
        if ((threadIdx.x >> 5) != CALC_NT / 32 - 1) return;
        tc::fence_after();
        float* tH = ms.tile(buf, 0);
        float* tM = ms.tile(buf, 1);
        float* tL = ms.tile(buf, 2);
        const uint32_t sbo = (uint32_t)ms.kc * 32u, idesc = tc::idesc_tf32(MX_ROWS, ms.N);
        const uint32_t dhh = ms.taddr + (uint32_t)(2 * win * ms.N), dr = dhh + (uint32_t)ms.N;
        // a group of 8 observations is two 128-byte core matrices further
        // on: 256 bytes, 16 in the descriptor's address field (addresses
        // below 256 KB do not carry out of the field); DF: 64-byte swizzled
        // rows of 16 observations, a group of 8 is 32 bytes (2) along the row
        uint64_t dh, dm, dl;
        uint32_t kstep;
        if constexpr (DF) {
            dh = tc::desc_kmajor_sw64(tc::smem_u32(tH), 512u);
            dm = tc::desc_kmajor_sw64(tc::smem_u32(tM), 512u);
            dl = tc::desc_kmajor_sw64(tc::smem_u32(tL), 512u);
            kstep = 2u;
        } else {
            dh = tc::desc_kmajor_noswizzle(tc::smem_u32(tH), 128u, sbo);
            dm = tc::desc_kmajor_noswizzle(tc::smem_u32(tM), 128u, sbo);
            dl = tc::desc_kmajor_noswizzle(tc::smem_u32(tL), 128u, sbo);
            kstep = 16u;
        }
        const uint32_t lead = tc::elect_lane();
        if constexpr (ST) {
            // A = [lo; Z] (buffer 0) or [Z; lo] (buffer 1) for lo*hi'
            uint64_t dz = tc::desc_kmajor_noswizzle(tc::smem_u32(buf == 0 ? tL : ms.zblock()), 128u, sbo);
            for (int g = 0; g < ngroups; ++g, dh += 16u, dm += 16u, dl += 16u, dz += 16u) {
                const uint32_t fresh = (win_obs == 0 && g == 0) ? 0u : 1u;
                tc::mma_tf32_lead(dhh, dh, dh, idesc, fresh, lead);   // [hi; mid] hi'
                tc::mma_tf32_lead(dr, dh, dm, idesc, fresh, lead);    // [hi; mid] mid'
                tc::mma_tf32_lead(dr, dh, dl, idesc, 1u, lead);       // [hi; mid] lo'
                tc::mma_tf32_lead(dr, dz, dh, idesc, 1u, lead);       // lo hi'
            }
        } else {
            for (int g = 0; g < ngroups; ++g, dh += kstep, dm += kstep, dl += kstep) {
                const uint32_t fresh = (win_obs == 0 && g == 0) ? 0u : 1u;
                tc::mma_tf32_lead(dhh, dh, dh, idesc, fresh, lead);
                tc::mma_tf32_lead(dr, dh, dm, idesc, fresh, lead);
                tc::mma_tf32_lead(dr, dm, dh, idesc, 1u, lead);
                tc::mma_tf32_lead(dr, dh, dl, idesc, 1u, lead);
                tc::mma_tf32_lead(dr, dl, dh, idesc, 1u, lead);
                tc::mma_tf32_lead(dr, dm, dm, idesc, 1u, lead);
            }
        }
        tc::commit_lead(ms.mbar + buf, lead);
    }

    // DF: issue the pending batch (every thread keeps the bookkeeping)
    __device__ __forceinline__ void issue_pending()
    {
        issue_mmas(pend_buf, (pend_nc + 7) / 8);
        sy.out |= 1u << pend_buf;
        win_obs += pend_nc;
        drain_after = win_obs + ms.kc > MX_WIN;
        pend = false;
    }

    // DF round: the MMAs of the previous batch are issued first, so that
    // they run while this batch is split and its S's formed; this batch's
    // operand buffer is free once the MMAs of two batches ago are done.  A
    // window closed by the batch just issued is drained at the end of the
    // round (its MMAs have had the round to finish), before the next issue.
    __device__ void round_df(const float* lcf, int base, int nc, int rb)
    {
        const int buf = (int)(rnd & 1u);
        if (pend) issue_pending();
        if (sy.outstanding(buf)) wait_buf(buf, false);
        split_vec(buf, rb, lcf, base, nc);
        ++rnd;
        pend = true;
        pend_buf = buf;
        pend_nc = nc;
        if (drain_after) {
            wait_buf(buf ^ 1, false);
            read_set(0);
            win_obs = 0;
            drain_after = false;
        }
        tc::fence_async_smem();
        tc::cp_async_wait_all();
        __syncthreads();
    }

    // the hi / mid / lo pieces of a round without the fused S's: a thread
    // takes (member r, K group kg) pairs -- four observations of one member
    // -- and stores each piece as one 16-byte row of a core matrix, so that
    // eight lanes fill one core matrix (128 contiguous bytes) and a warp's
    // raw reads are consecutive members of one observation.  Rows >= m are
    // not written (they only reach accumulator rows and columns that are
    // never read); observations past nc have zero rows and zero taper.
    // Each pair's products with the observations' tapered innovations go
    // into the pair's double-float S's sum (vh, vl).
    __device__ __forceinline__ void split_vec(int buf, int rb, const float* lcf, int base, int nc)
    {
        const int m = a.m, nkg = ms.kc >> 2, rows = ((m + 7) >> 3) << 3;
        const int npair = nkg * rows;
        float* tH = ms.tile(buf, 0);
        float* tM = ms.tile(buf, 1);
        float* tL = ms.tile(buf, 2);
        const float* raw = ms.rawb(rb);
        const float* sr = ms.srawb(rb);
        const float* cq = ms.qs + m;
        const int dk = CALC_NT / rows, dr = CALC_NT - dk * rows;
        int kg = (int)threadIdx.x / rows, r = (int)threadIdx.x - kg * rows;
#pragma unroll
        for (int sl = 0; sl < NSLOT; ++sl) {
            if ((int)threadIdx.x + sl * CALC_NT >= npair) break;
            if (r < m) {
                const int k0 = kg << 2;
                float v[4], c[4];
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    v[j] = raw[(k0 + j) * ms.ldv + r];
                    c[j] = k0 + j < nc ? lcf[base + k0 + j] : 0.0f;
                }
                const float cr = cq[r];
                float h[4], md[4], lo[4];
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    // as split_rows: hi = q rint(v / q) through the rounding
                    // constant, mid and lo rounded to TF32 (to nearest, ties
                    // away from zero)
                    const float vv = __fmul_rn(v[j], c[j]);
                    h[j] = __fsub_rn(__fadd_rn(vv, cr), cr);
                    const float r1 = __fsub_rn(vv, h[j]);
                    md[j] = tc::tf32_rna(r1);
                    lo[j] = tc::tf32_rna(__fsub_rn(r1, md[j]));
                    {
                        // TwoProd and TwoSum into the pair's sum
                        const float x = __fmul_rn(sr[k0 + j], c[j]);
                        const float pp = vv * x, pe = fmaf(vv, x, -pp);
                        const float sm = vh[sl] + pp, bp = sm - vh[sl];
                        vl[sl] += ((vh[sl] - (sm - bp)) + (pp - bp)) + pe;
                        vh[sl] = sm;
                    }
                }
                // DF: 64-byte rows (kc = 16), chunk kg at kg ^ ((r >> 1) & 3)
                const int off = DF ? (((r >> 3) << 7) + ((r & 7) << 4) + ((kg ^ ((r >> 1) & 3)) << 2))
                                   : ((((r >> 3) * nkg + kg) << 5)) + ((r & 7) << 2);
                *reinterpret_cast<float4*>(tH + off) = make_float4(h[0], h[1], h[2], h[3]);
                *reinterpret_cast<float4*>(tM + off) = make_float4(md[0], md[1], md[2], md[3]);
                *reinterpret_cast<float4*>(tL + off) = make_float4(lo[0], lo[1], lo[2], lo[3]);
            }
            kg += dk;
            r += dr;
            if (r >= rows) {
                r -= rows;
                ++kg;
            }
        }
    }

    // one round: nc (<= kc) observations at list positions [base, base + nc)
    // whose rows are in raw buffer rb
    __device__ void round(const float* lcf, int base, int nc, int t, int rb)
    {
        const int tid = threadIdx.x;
        const int m = a.m, kc = ms.kc;
        const bool tsum = a.want_diag && a.ntypes > 1;
        double ssq = 0.0;
        const int buf = (int)(rnd & 1u);
        // 0. this operand buffer's previous MMAs were waited for at the end of
        //    the last round (this only acts on the first round after an error)
        if (sy.outstanding(buf)) {
            wait_buf(buf);
            if (*ms.err) return;
        }
        float* tH = ms.tile(buf, 0);
        float* tM = ms.tile(buf, 1);
        float* tL = ms.tile(buf, 2);
        const float* raw = ms.rawb(rb);
        // 1. tapered S: hi / mid / lo pieces into this round's operand tiles.
        // One warp per core matrix (8 rows x 4 observations = 128 bytes):
        // lane -> row r&7 = lane>>2, observation k&3 = lane&3, so the piece
        // stores and the raw reads (row stride = 8 mod 32) are conflict-free;
        // rows >= m stay zero.  kc is a power of two, so warp w keeps one
        // K group (observations 4 kg .. 4 kg + 3, one taper per thread) and
        // walks the row groups.  Rows of raw past nc are zero.  (Two copies
        // of the loop: an FP64 sum under a runtime flag inside the common
        // loop would issue on the FP64 pipe even when off.)
        {
            const int lane = tid & 31, wid = tid >> 5;
            const int nrg = (m + 7) >> 3, nkg = kc >> 2;
            const int kg = wid & (nkg - 1), rg0 = wid / nkg, rstep = (CALC_NT / 32) / nkg;
            const int k = (kg << 2) + (lane & 3);
            const float ck = k < nc ? lcf[base + k] : 0.0f;
            const float xk = (FS && k < nc) ? __fmul_rn(ms.srawb(rb)[k], ck) : 0.0f;
            const float* rp = raw + k * ms.ldv + (lane >> 2);
            if (tsum) ssq = split_rows<true>(tH, tM, tL, rp, ck, xk, nrg, nkg, kg, rg0, rstep, lane);
            else if (FS) split_rows<false>(tH, tM, tL, rp, ck, xk, nrg, nkg, kg, rg0, rstep, lane);
            else split_vec(buf, rb, lcf, base, nc);
        }
        tc::fence_async_smem();
        __syncthreads();
        // 2. the round's MMAs (the last warp, so that the S's of the first
        //    warps runs at the same time)
        issue_mmas(buf, (nc + 7) / 8);
        sy.out |= 1u << buf;
        ++rnd;
        // 3. S's from the staged rows (fused into the split otherwise)
        if (tsum) ss_pass(lcf, base, nc, rb);
        // 4. the window closed one round ago: its last commit is on the other
        //    buffer; drain it while this round's MMAs run
        if (drain_set >= 0) {
            wait_buf(drain_buf, false);
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
        //    here, and for this thread's copies of the next round's rows,
        //    under the round's closing barrier
        if (sy.outstanding(buf ^ 1)) {
            bool done = tc::mbar_wait_bounded(ms.mbar + (buf ^ 1), sy.parity(buf ^ 1), a.wait_ns);
            if (!done) {
                atomicExch(ms.err, 1);
                tc::mbar_wait_bounded(ms.mbar + (buf ^ 1), sy.parity(buf ^ 1), MX_WAIT_NS);
            }
            sy.completed(buf ^ 1);
            tc::fence_after();
        }
        tc::cp_async_wait_all();
        __syncthreads();
    }

    // the rounds of a list segment of n entries of type t: all of them when
    // `final`, else the whole rounds (the rest stays for the next segment).
    // The rows of round j + 1 are copied in while round j is split and
    // multiplied.  Returns the entries consumed.
    __device__ int segment(const int* lid, const float* lcf, int n, int t, bool final)
    {
        const int kc = ms.kc;
        const int nr = final ? (n + kc - 1) / kc : n / kc;
        const int used = final ? n : nr * kc;
        if (nr == 0 || *ms.err) return used;
        stage_rows(lid, 0, n < kc ? n : kc, 0);
        tc::cp_async_wait_all();
        __syncthreads();
        for (int j = 0; j < nr; ++j) {
            const int base = j * kc, rb = j & 1;
            const int nc = (n - base < kc) ? n - base : kc;
            if (j + 1 < nr) {
                const int nn = n - base - kc;
                stage_rows(lid, base + kc, nn < kc ? nn : kc, rb ^ 1);
            }
            if constexpr (DF) round_df(lcf, base, nc, rb);
            else round(lcf, base, nc, t, rb);
            if (*ms.err) break;
        }
        tc::cp_async_wait_all();   // nothing in flight after an early exit
        __syncthreads();
        return used;
    }

    // drain what is left (after the enumeration; also after an error, so that
    // no MMA is in flight when TMEM is released)
    __device__ __forceinline__ void finish()
    {
        if (DF && pend && !*ms.err) issue_pending();
        pend = false;
        drain_after = false;
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

// Warp 0: the neighbour cells of the query (up to 9 in 2-D, 27 in 3-D), in
// the order calc_neighbours visits them (z, then y, then x ascending), one
// lane each: sb0[j] = first sorted position of the j-th existing cell's
// bucket, scum[j] = sizes of the buckets before it, scum[nb] = their total,
// scum[28] = nb.
__device__ __forceinline__ void neighbour_ranges(const CalcArgs& a, const TypeIndex& t, double qx, double qy,
                                                 double qz, long long* sb0, int* scum)
{
    const int lane = threadIdx.x & 31, ndim = a.ndim;
    const double fx = floor((qx - t.x0) * t.inv_cell), fy = floor((qy - t.y0) * t.inv_cell);
    const double fz = ndim == 3 ? floor((qz - t.z0) * t.inv_cell) : 0.0;
    bool inside = fx >= -1.0 && fx <= (double)t.ncx && fy >= -1.0 && fy <= (double)t.ncy;
    if (ndim == 3) inside = inside && fz >= -1.0 && fz <= (double)t.ncz;
    bool valid = false;
    long long b0 = 0;
    int sz = 0;
    if (inside && lane < (ndim == 3 ? 27 : 9)) {
        const int cx = (int)fx, cy = (int)fy, cz = (int)fz;
        const int r9 = ndim == 3 ? lane % 9 : lane;
        const int z = ndim == 3 ? cz + lane / 9 - 1 : 0, y = cy + r9 / 3 - 1, x = cx + r9 % 3 - 1;
        valid = z >= 0 && z < t.ncz && y >= 0 && y < t.ncy && x >= 0 && x < t.ncx;
        if (valid) {
            const unsigned int code = (ndim == 2) ? (cc_spread2(x) | (cc_spread2(y) << 1))
                                                  : (cc_spread3(x) | (cc_spread3(y) << 1) | (cc_spread3(z) << 2));
            const long long bk = t.bucket_base + (long long)code;
            b0 = a.bstart[bk];
            sz = (int)(a.bstart[bk + 1] - b0);
        }
    }
    const unsigned bal = __ballot_sync(0xffffffffu, valid);
    int incl = sz;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
    }
    if (valid) {
        const int pos = __popc(bal & ((1u << lane) - 1));
        sb0[pos] = b0;
        scum[pos] = incl - sz;
    }
    if (lane == 31) {
        const int nb = __popc(bal);
        scum[nb] = incl;
        scum[28] = nb;
    }
}

// Local-observation enumeration for the mixed path (the search of
// obs_findlocal in common/observations.c, with the acceptance tests of
// enumerate_obs): the candidates are the concatenated position ranges of the
// neighbour buckets, taken 256 at a time across bucket boundaries (the order
// is still bucket, then position), with each thread's coordinates for the
// next block loaded while the current block is tested.  Accepted
// observations are appended to a list of lseg + CALC_NT entries (position,
// FP32 taper); whenever it holds lseg or more, the processor consumes its
// whole rounds (proc.segment) and the rest moves to the front.  A type's
// tail is consumed before the next type starts.  SEARCH 2: FP32 pre-test
// with an exact FP64 test in the band (2-D); SEARCH 1: exact FP64 distances.
// Returns the number of local observations.
template <int SEARCH, class Proc>
__device__ int enumerate_obs_seg(const CalcArgs& a, int pt, int lseg, double qx, double qy, double qz, int* lid,
                                 float* lcf, int* wsum, long long* sb0, int* scum, int* tcount, Proc& proc)
{
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    int total = 0;
    for (int t = 0; t < a.ntypes; ++t) {
        const TypeIndex& ti = a.types[t];
        int n = 0;   // list entries (the same in every thread)
        int tcnt = 0;
        if (ti.pos_end > ti.pos_begin) {
            // NLOBSMAX: the point's cut for this type applies (a point with
            // no more observations in range than the limit has none)
            bool cut_on = false;
            if (a.cut != nullptr && ti.nlobsmax > 0) cut_on = a.cut[(size_t)t * a.npts + pt].d2 <= ti.rmax2;
            if (wid == 0) neighbour_ranges(a, ti, qx, qy, qz, sb0, scum);
            __syncthreads();
            const int nb = scum[28], ncand = scum[nb];
            const float qxh = (float)qx, qyh = (float)qy;
            const float qxl = (float)(qx - (double)qxh), qyl = (float)(qy - (double)qyh);
            // candidate c -> sorted position; j only moves forward
            int j = 0;
            auto position = [&](int c) -> long long {
                while (j + 1 < nb && scum[j + 1] <= c) ++j;
                return sb0[j] + (long long)(c - scum[j]);
            };
            long long pn = -1;
            float nxf = 0.0f, nyf = 0.0f;
            double nx = 0.0, ny = 0.0, nz = 0.0;
            if (tid < ncand) {
                pn = position(tid);
                if constexpr (SEARCH == 2) {
                    nxf = a.sxf[pn];
                    nyf = a.syf[pn];
                } else {
                    nx = a.sx[pn];
                    ny = a.sy[pn];
                    if (a.ndim == 3) nz = a.sz[pn];
                }
            }
            for (int base = 0; base < ncand; base += CALC_NT) {
                const long long p = pn;
                const float xf = nxf, yf = nyf;
                const double x = nx, y = ny, z = nz;
                pn = -1;
                if (base + CALC_NT + tid < ncand) {
                    pn = position(base + CALC_NT + tid);
                    if constexpr (SEARCH == 2) {
                        nxf = a.sxf[pn];
                        nyf = a.syf[pn];
                    } else {
                        nx = a.sx[pn];
                        ny = a.sy[pn];
                        if (a.ndim == 3) nz = a.sz[pn];
                    }
                }
                bool in = false;
                float d2f = 0.0f, d2l = 0.0f;
                double d2 = 0.0;
                if constexpr (SEARCH == 2) {
                    bool band = false;
                    if (p >= 0) {
                        exact::dist2_df(xf, yf, qxh, qxl, qyh, qyl, d2f, d2l);
                        in = d2f <= ti.rmax2_lo;
                        band = !in && d2f <= ti.rmax2_hi;
                    }
                    if (__any_sync(0xffffffffu, band))
                        if (band) in = exact_in2(a.sx[p], a.sy[p], qx, qy, ti.rmax2);
                    if (cut_on && in)
                        in = exact_cut2(a.sx[p], a.sy[p], qx, qy, a.sid[p], a.cut + (size_t)t * a.npts + pt);
                } else {
                    if (p >= 0) {
                        d2 = a.ndim == 2 ? exact::dist2(x, y, qx, qy) : exact::dist3(x, y, z, qx, qy, qz);
                        in = d2 <= ti.rmax2;
                        if (cut_on && in) in = keeps_cut(d2, a.sid[p], a.cut + (size_t)t * a.npts + pt);
                    }
                }
                const unsigned bal = __ballot_sync(0xffffffffu, in);
                if (lane == 0) wsum[wid] = __popc(bal);
                __syncthreads();
                int before = 0, tot = 0;
#pragma unroll
                for (int w = 0; w < CALC_NT / 32; ++w) {
                    const int c = wsum[w];
                    before += (w < wid) ? c : 0;
                    tot += c;
                }
                if (in) {
                    const int pos = n + before + __popc(bal & ((1u << lane) - 1));
                    lid[pos] = (int)p;
                    if constexpr (SEARCH == 2)
                        lcf[pos] = exact::calclcoeff_df(ti, d2f, d2l);
                    else
                        lcf[pos] = exact::calclcoeff_f(ti.nlocrad, ti.locrad, ti.locweight, d2);
                }
                n += tot;
                tcnt += tot;
                __syncthreads();   // list entries visible; wsum free
                if (n >= lseg) {
                    const int used = proc.segment(lid, lcf, n, t, false);
                    const int rest = n - used;   // < kc <= CALC_NT
                    int id = 0;
                    float c = 0.0f;
                    if (tid < rest) {
                        id = lid[used + tid];
                        c = lcf[used + tid];
                    }
                    __syncthreads();
                    if (tid < rest) {
                        lid[tid] = id;
                        lcf[tid] = c;
                    }
                    __syncthreads();
                    n = rest;
                }
            }
            if (n > 0) proc.segment(lid, lcf, n, t, true);
        }
        if (tid == 0) tcount[t] = tcnt;
        total += tcnt;
        __syncthreads();
    }
    return total;
}

// operand tiles: 2 buffers x 3 pieces x N rows x kc, then the padding that
// the 128-row A operand reads past the last tile (rows >= N, never used);
// stacked (N <= 64): [hi mid lo] [Z] [lo hi mid] and the 128 - 2N rows that
// A = [hi; mid; ...] of buffer 1 reads past its mid piece
static __host__ __device__ size_t mixed_tile_floats(int m, int kc, int st)
{
    const int N = (m + 15) / 16 * 16;
    if (st) return (size_t)7 * N * kc + (size_t)(MX_ROWS - 2 * N) * kc;   // 6 pieces + Z + A's reach past b1.mid
    return (size_t)2 * MX_PIECES * N * kc + (size_t)(MX_ROWS - N) * kc;
}

// row stride of the raw S rows: >= mpad (a multiple of 4: 16-byte copies)
// and = 8 mod 32, so that the 8 rows x 4 observations a warp reads per core
// matrix fall in distinct banks
static __host__ __device__ int mixed_ldv(int m)
{
    return m + ((8 - m % 32) % 32 + 32) % 32;
}

// local-observation list: lseg + CALC_NT entries of (position, FP32 taper);
// the FP64 per-type pass reuses it as LIST_EXTRA (position, FP64 taper)
static __host__ __device__ size_t mixed_list_bytes(int lseg)
{
    const size_t a = (size_t)(lseg + CALC_NT) * 8, b = (size_t)LIST_EXTRA * 12 + 8;
    return a > b ? a : b;
}

// df: the compact deferred form (packed upper triangle, b only)
static size_t mixed_smem_bytes(int m, int kc, int lseg, int st, int df)
{
    int lda = (m % 2 == 0) ? m + 1 : m + 2;
    size_t s = 0;
    s += mixed_tile_floats(m, kc, st) * 4;                 // operand tiles + padding
    if (df) s += 1024;                                     // the swizzled tiles on a 1 KB boundary
    if (st) s += (size_t)m * lda * 4;                      // Mrest
    s += (size_t)2 * kc * mixed_ldv(m) * 4;                // raw S rows, two buffers
    s += (size_t)2 * kc * 4;                               // raw innovations, two buffers
    s += (size_t)2 * m * 4;                                // quantum q, rounding constant
    s += 16;                                               // alignment
    s += df ? (size_t)((m + 1) / 2) * ((m + 2) & ~1) * 8 : (size_t)m * lda * 8;   // Macc (also A)
    s += (size_t)(df ? 1 : 6) * (m + 1) * 8;               // b d e cs sn v
    s += (size_t)ENKFG_MAXTYPES * 8 * 2;
    s += (size_t)(CALC_NT / 32) * 8;
    s += mixed_list_bytes(lseg);
    s += (size_t)ENKFG_MAXTYPES * 4;
    s += 256;                                              // control ints
    s += 28 * 8 + 29 * 4 + 8;                              // neighbour bucket ranges
    s += 64;                                               // mbarriers, tmem slot, flags
    return s;
}

template <int HB, bool FS, bool ST, bool DF>
__global__ void __launch_bounds__(CALC_NT, 2) k_transforms_mixed(CalcArgs a, int kcm, int N, uint32_t tcols, int lseg)
{
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const int tid = threadIdx.x, wid = tid >> 5;
    const int m = a.m, lda = (m % 2 == 0) ? m + 1 : m + 2;   // odd stride: fewer bank conflicts
    const size_t ntile = mixed_tile_floats(m, kcm, ST);     // operand pieces + padding for A's rows
    // DF: the swizzled tiles start on a 1 KB boundary of the shared window
    unsigned char* sp = smem_raw + (DF ? (1024u - (tc::smem_u32(smem_raw) & 1023u)) & 1023u : 0u);
    float* tiles = (float*)sp;        sp += ntile * 4;
    const int ldv = mixed_ldv(m);
    float* raw0 = (float*)sp;         sp += (size_t)2 * kcm * ldv * 4;   // two buffers
    float* sraw0 = (float*)sp;        sp += (size_t)2 * kcm * 4;
    float* qs = (float*)sp;           sp += (size_t)2 * m * 4;
    sp = (unsigned char*)(((uintptr_t)sp + 15) & ~(uintptr_t)15);
    const int nmacc = DF ? ((m + 1) / 2) * ((m + 2) & ~1) : m * lda;   // DF: packed upper triangle
    double* Macc = (double*)sp;       sp += (size_t)nmacc * 8;
    float* Mrest = (float*)sp;        sp += ST ? (size_t)m * lda * 4 : 0;
    double* b = (double*)sp;          sp += (m + 1) * 8;
    // the in-kernel solve's vectors (not in the compact deferred form)
    double* d = (double*)sp;          sp += DF ? 0 : (m + 1) * 8;
    double* e = (double*)sp;          sp += DF ? 0 : (m + 1) * 8;
    double* cs = (double*)sp;         sp += DF ? 0 : (m + 1) * 8;
    double* sn = (double*)sp;         sp += DF ? 0 : (m + 1) * 8;
    double* v = (double*)sp;          sp += DF ? 0 : (m + 1) * 8;
    double* tss = (double*)sp;        sp += ENKFG_MAXTYPES * 8;
    double* tpd = (double*)sp;        sp += ENKFG_MAXTYPES * 8;
    double* red = (double*)sp;        sp += (CALC_NT / 32) * 8;
    unsigned char* list = sp;         sp += mixed_list_bytes(lseg);
    int* tcount = (int*)sp;           sp += ENKFG_MAXTYPES * 4;
    int* ictl = (int*)sp;             sp += 256;
    long long* nb0 = (long long*)sp;  sp += 28 * 8;
    int* ncum = (int*)sp;             sp += 29 * 4 + 4;
    uint64_t* mbar = (uint64_t*)sp;   sp += 8 * 2;
    uint32_t* tslot = (uint32_t*)sp;  sp += 8;
    int* err = (int*)sp;
    // the search list (lseg + CALC_NT positions, then their FP32 tapers);
    // the FP64 per-type pass views the same bytes as LIST_EXTRA positions
    // and FP64 tapers
    int* slid = (int*)list;
    float* slcf = (float*)(list + (size_t)(lseg + CALC_NT) * 4);
    double* llc = (double*)(list + (size_t)LIST_EXTRA * 4 + 8 - ((size_t)LIST_EXTRA * 4) % 8);
    const PointScratch s{ slid, llc, ictl, tcount, tss, tpd, red };
    const size_t piece = (size_t)N * kcm;

    // set-up: TMEM columns, mbarriers, zeroed operand tiles, the quantum
    // drill_bar: an mbarrier nothing arrives at (the timeout drill's wait)
    __shared__ uint64_t drill_bar;
    if (wid == 0) tc::tmem_alloc(tslot, tcols);
    if (tid == 0) {
        for (int i = 0; i < 2; ++i) tc::mbar_init(mbar + i, 1);
        tc::mbar_init(&drill_bar, 1);
        *err = 0;
    }
    for (size_t i = tid; i < ntile; i += CALC_NT) tiles[i] = 0.0f;
    for (int r = tid; r < m; r += CALC_NT) {
        qs[r] = a.qscale[r];
        qs[m + r] = 12582912.0f * a.qscale[r];   // 1.5 2^23 q_r
    }
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    MixedShared ms{ tiles, (int)piece, raw0, kcm * ldv, sraw0, kcm, ldv, qs, (float2*)Macc, Mrest, lda, ST ? 1 : 0,
                    mbar, *tslot, N, kcm, err };
    MixedSync sy{ 0u, 0u };
    uint32_t rnd = 0;

    for (int it = 0;; ++it) {
        const int idx = next_item(a, it, ictl);
        if (idx < 0 || *err) break;
        const int pt = a.order ? a.order[idx] : a.item0 + idx;
        if (a.wait_drill && it == 0) {
            // the timeout drill: a bounded wait that nothing completes, so
            // that it expires (enkfg_set_wait_drill)
            if (tid == 0 && !tc::mbar_wait_bounded(&drill_bar, 0, a.wait_ns)) atomicExch(err, 1);
            __syncthreads();
            if (*err) {
                if (tid == 0) a.status[pt] = MX_TIMEOUT_CODE;
                break;
            }
        }
        const double qx = a.qx[pt], qy = a.qy[pt], qz = a.ndim == 3 ? a.qz[pt] : 0.0;
        // observations per round: 8, 16 or 32 (a power of two), per count
        // bin when tuned
        ms.kc = kcm;
        if (!DF && a.kc_table != nullptr && a.counts != nullptr) {   // DF: the swizzled rows are 16 wide
            const int k = a.kc_table[count_bin(a.counts[pt])];
            ms.kc = k >= kcm ? kcm : k >= 16 ? 16 : 8;
        }
        if (tid < ENKFG_MAXTYPES) {
            tss[tid] = 0.0;
            tpd[tid] = 0.0;
            tcount[tid] = 0;
        }
        for (int i = tid; i < nmacc; i += CALC_NT) {
            Macc[i] = 0.0;   // also zero as float2
            if (ST) Mrest[i] = 0.0f;
        }
        // pieces N x kc apart (contiguous, as the stacked A = [hi; mid]
        // needs); the Z block at this spacing is cleared (the previous
        // point's MMAs have completed).  Rows >= m of the other pieces may
        // hold stale values: they only reach accumulator rows and columns
        // that are never read.
        ms.piece = N * ms.kc;
        if (ST)
            for (int i = tid; i < ms.piece; i += CALC_NT) ms.zblock()[i] = 0.0f;
        __syncthreads();
        // every point starts on operand buffer 0 (the previous point's MMAs
        // are all complete: finish() waited for both buffers), so that which
        // buffer a round uses -- and, in the stacked form, which accumulator
        // rows take lo*hi' -- does not depend on the points the CTA did
        // before, and the result of a point does not depend on the queue
        rnd = 0;
        GramProcTC<HB, FS, ST, DF> proc(a, s, ms, sy, rnd);
        const int p = (a.sxf != nullptr && a.ndim == 2)
                          ? enumerate_obs_seg<2>(a, pt, lseg, qx, qy, qz, slid, slcf, ictl + 8, nb0, ncum, tcount,
                                                 proc)
                          : enumerate_obs_seg<1>(a, pt, lseg, qx, qy, qz, slid, slcf, ictl + 8, nb0, ncum, tcount,
                                                 proc);
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
        // S's: partial sums in FP64 into the raw row buffers (idle between
        // points), summed below -- fused: the four lanes of a row group (four
        // observations) combined by shuffles, then one partial per K group
        // (each (K group, row) is written by exactly one warp); separate
        // pass: one partial per thread group
        double* bpart = (double*)raw0;
        int nparts;
        if constexpr (FS) {
            const int lane = tid & 31;
            const int nkg = ms.kc >> 2, nrg = (m + 7) >> 3;
            const int kg = wid & (nkg - 1), rg0 = wid / nkg, rstep = (CALC_NT / 32) / nkg;
#pragma unroll
            for (int i = 0; i < 2 * HB; ++i) {
                double d = (double)proc.fh[i] + (double)proc.fl[i];
                d += __shfl_xor_sync(0xffffffffu, d, 1);
                d += __shfl_xor_sync(0xffffffffu, d, 2);
                const int rg = rg0 + i * rstep, r = (rg << 3) + (lane >> 2);
                if ((lane & 3) == 0 && rg < nrg && r < m) bpart[kg * m + r] = d;
            }
            nparts = nkg;
        } else if (a.want_diag && a.ntypes > 1) {
            if (proc.s_g < proc.sgroups)
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int r = 4 * proc.s_q + u;
                    if (r < m) bpart[proc.s_g * m + r] = (double)proc.bh[u] + (double)proc.bl[u];
                }
            nparts = proc.sgroups;
        } else {
            // one partial per (K group, member): the pairs of split_vec
            const int nkg = ms.kc >> 2, rows = ((m + 7) >> 3) << 3;
            int kg = tid / rows, r = tid - kg * rows;
            const int dk = CALC_NT / rows, dr = CALC_NT - dk * rows;
#pragma unroll
            for (int sl = 0; sl < proc.NSLOT; ++sl) {
                if (tid + sl * CALC_NT < nkg * rows && r < m)
                    bpart[kg * m + r] = (double)proc.vh[sl] + (double)proc.vl[sl];
                kg += dk;
                r += dr;
                if (r >= rows) {
                    r -= rows;
                    ++kg;
                }
            }
            nparts = nkg;
        }
        if constexpr (DF) {
            // the batched solve's inputs straight from the packed S'S: M = I +
            // S'S (upper triangle, FP64) into slot idx, S's, p and tr(S'S)
            __syncthreads();
            const size_t q0 = (size_t)idx * m * m;
            if (tid < m) {
                double acc = 0.0;
                for (int g = 0; g < nparts; ++g) acc += bpart[g * m + tid];
                a.eb[(size_t)idx * m + tid] = acc;
            }
            const float2* Mp = (const float2*)Macc;
            const int lane = tid & 31;
            for (int r = wid; r < m; r += CALC_NT / 32) {
                int e0, es;
                proc.tri(r, e0, es);
                for (int c = r + lane; c < m; c += 32) {
                    const float2 v2 = Mp[e0 + es * c];
                    const double x = (double)v2.x + (double)v2.y;
                    a.eq[q0 + (size_t)r * m + c] = c == r ? x + 1.0 : x;
                    if (a.emhl) {
                        // the same value as a float pair: Fast2Sum (|y| <=
                        // |x|), through FP64 on the diagonal for the 1
                        float2 o;
                        if (c == r) {
                            o.x = (float)(x + 1.0);
                            o.y = (float)((x + 1.0) - (double)o.x);
                        } else {
                            o.x = v2.x + v2.y;
                            o.y = (v2.x - o.x) + v2.y;
                        }
                        a.emhl[q0 + (size_t)r * m + c] = o;
                    }
                }
            }
            double dg = 0.0;
            if (tid < m) {
                int e0, es;
                proc.tri(tid, e0, es);
                const float2 v2 = Mp[e0 + es * tid];
                dg = (double)v2.x + (double)v2.y;
            }
            const double trss = la::block_sum<CALC_NT>(dg, red);
            if (tid == 0) {
                a.eaux[2 * (size_t)idx] = (double)p;
                a.eaux[2 * (size_t)idx + 1] = trss;
            }
            __syncthreads();
        } else {
            // double-float -> FP64 in place
            for (int i = tid; i < m * lda; i += CALC_NT) {
                float2 v2 = ((float2*)Macc)[i];
                Macc[i] = ST ? ((double)v2.x + (double)v2.y) + (double)Mrest[i] : (double)v2.x + (double)v2.y;
            }
            __syncthreads();
            if (tid < m) {
                double acc = 0.0;
                for (int g = 0; g < nparts; ++g) acc += bpart[g * m + tid];
                b[tid] = acc;
            }
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
    }
    __syncthreads();
    if (wid == 0) tc::tmem_dealloc(*tslot, tcols);
}

template <int HB, bool FS, bool ST, bool DF>
static enkfg_status launch_mixed_hb(enkfg_ctx* ctx, CalcArgs& a, int kcm, int N, uint32_t tcols, size_t smem,
                                    int lseg, cudaStream_t st)
{
    CK(cudaFuncSetAttribute(k_transforms_mixed<HB, FS, ST, DF>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    // computed residency (the occupancy query reports one CTA per SM here)
    // and the carveout that holds it, the rest staying L1
    int per_sm = 0, carve = 100;
    enkfg_status s = resident_ctas(ctx, (const void*)k_transforms_mixed<HB, FS, ST, DF>, CALC_NT, smem, &per_sm, &carve);
    if (s) return s;
    CK(cudaFuncSetAttribute(k_transforms_mixed<HB, FS, ST, DF>, cudaFuncAttributePreferredSharedMemoryCarveout, carve));
    int grid = a.nitems;
    if (a.persistent) {
        int nsm = 0;
        CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, ctx->device));
        // TMEM: at most 512 columns per SM across resident CTAs
        while (per_sm > 1 && (uint32_t)per_sm * tcols > 512) --per_sm;
        grid = per_sm * nsm;
        if (grid > a.nitems) grid = a.nitems;
    }
    if (grid < 1) return ENKFG_OK;
    k_transforms_mixed<HB, FS, ST, DF><<<grid, CALC_NT, smem, st>>>(a, kcm, N, tcols, lseg);
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
    // list segment: 1024 entries, fewer where that keeps two CTAs per SM
    // (113 KB each) or the CTA within 227 KB; at least 256
    int lseg = 1024;
    const size_t two = 113 * 1024, one = 227 * 1024;
    const int stk = N <= 64 ? 1 : 0;                     // stacked products
    const int hb = ((N >> 1) + 7) / 8;
    if (a.defer && !stk && hb <= 6) {
        // the compact deferred form: one TMEM set of 2N columns (at most
        // 256) and the packed S'S, 16 observations a round -- two CTAs per
        // SM, where that fits
        int ls = 1024;
        while (ls > 256 && mixed_smem_bytes(m, 16, ls, 0, 1) > two) ls >>= 1;
        const size_t sm = mixed_smem_bytes(m, 16, ls, 0, 1);
        uint32_t tc1 = 32;
        while ((int)tc1 < 2 * N) tc1 <<= 1;
        if (sm <= two && tc1 <= 256) return launch_mixed_hb<6, false, false, true>(ctx, a, 16, N, tc1, sm, ls, st);
    }
    const size_t lim = mixed_smem_bytes(m, kcm, 256, stk, 0) <= two ? two : one;
    while (lseg > 256 && mixed_smem_bytes(m, kcm, lseg, stk, 0) > lim) lseg >>= 1;
    size_t smem = mixed_smem_bytes(m, kcm, lseg, stk, 0);
    if (smem > 227 * 1024) {
        set_err(ctx, "mixed path: nmem = %d needs %zu bytes of shared memory", m, smem);
        return ENKFG_EUNSUPPORTED;
    }
    // the per-type pass's FP64 chunk buffer (kcm x m doubles) lives in the tiles
    if (tcols > 512 || (size_t)kcm * m * 8 > mixed_tile_floats(m, kcm, stk) * 4) {
        set_err(ctx, "mixed path: tile too small for the per-type pass");
        return ENKFG_EUNSUPPORTED;
    }
    // S's fused into the split up to 8 rows per thread (registers)
    // (N <= 64 is hb <= 4: fused S's and stacked products together)
    if (hb <= 2) return launch_mixed_hb<2, true, true, false>(ctx, a, kcm, N, tcols, smem, lseg, st);
    if (hb <= 3) return launch_mixed_hb<3, true, true, false>(ctx, a, kcm, N, tcols, smem, lseg, st);
    if (hb <= 4) return launch_mixed_hb<4, true, true, false>(ctx, a, kcm, N, tcols, smem, lseg, st);
    if (hb <= 6) return launch_mixed_hb<6, false, false, false>(ctx, a, kcm, N, tcols, smem, lseg, st);
    return launch_mixed_hb<8, false, false, false>(ctx, a, kcm, N, tcols, smem, lseg, st);
}
