// etkf_mixed.cu -- the ETKF solve of the mixed-precision batched path.
//
// For every local analysis the transform kernel leaves M = I + S'S (FP64,
// upper triangle), S's, p and tr(S'S) in a batch slot; the reference then
// needs T = M^-1/2 and w = M^-1 S's (calc/calcs.c:300-412).  GB300 issues
// FP64 at 1/64 of its FP32 rate, so an FP64 eigensolver at nmem = 96 costs
// about 10 m^3 FP64 operations a point and dominates the cycle.  Here the
// eigendecomposition only seeds a Newton correction:
//
//   1. M = Q diag(lambda) Q' in FP32 (Householder tridiagonalisation, then
//      the implicit QL chains one thread per point with their rotations
//      logged, then the log replayed onto Q) -- the FP64 pipeline of
//      calc.cu with F = float;
//   2. Z0 = Q diag(lambda^-1/2) Q' (FP32);
//   3. the residual R = I - Z0 M Z0 in double-float arithmetic (every
//      product of a float pair exact through an FMA, every sum a TwoSum), so
//      that R, of order 1e-4, is known to about 1e-12 absolute;
//   4. the correction D solving D (M Z0) + (Z0 M) D = R, in the eigenbasis
//      of step 1: D~ = Q' R Q, D~_ij /= (lambda_i^1/2 + lambda_j^1/2),
//      D = Q D~ Q' (FP32: D is of the size of R);
//   5. T = Z0 + D (summed in FP64), relaxed and cast as the reference does;
//   6. w by iterative refinement: w += Q diag(1/lambda) Q' r with the
//      residual r = S's - M w in FP64, EM_W_STEPS times.
//
// The FP32 decomposition is backward stable with an error of order u32
// lambda_max (about 1e-4 at lambda_max ~ 1e3), which is the error of Z0; one
// Newton step squares it, and the errors of solving the correction in an
// approximate eigenbasis are of the same order.  w converges by a factor of
// about u32 lambda_max per step.  All matrices are zero-padded to MP = 16 R
// rows and columns; the work per point is a handful of m^3 FP32 GEMM-like
// loops on a 16 x 16 thread grid (R x R outputs per thread) and one
// double-float product pair.
#include "calc_common.cuh"

#define EM_QL_T 32
#define EM_NT 256
#define EM_KCH 16      // rows of the global operand staged per step
// iterative-refinement steps of w: each multiplies the relative error by
// about u32 lambda_max(M), so two leave about (6e-8 lambda_max)^2 -- below
// 4e-7 up to lambda_max = 1e4, under the errors of the FP32 taper and S
#define EM_W_STEPS 2

// ---------------------------------------------------------------------------
// per-slot scratch of the refined solve (float unless noted)
// ---------------------------------------------------------------------------
struct EmSlots {
    float* q;          // [slots][m][m]  Q of tred2, then the eigenvectors (columns)
    float2* mhl;       // [slots][m][m]  M as a double-float pair (hi, lo): the upper triangle from the
                       //                transform kernel, the lower one mirrored by k_em_replay
    float* d;          // [slots][m]     tridiagonal diagonal, then the eigenvalues
    float* e;          // [slots][m]     tridiagonal off-diagonal
    float2* rot;       // [slots][rcap]  QL rotation log
    int2* hdr;         // [slots][hcap]
    int* nh;           // [slots]        sweeps logged (< 0: the chain failed)
    float* z0;         // [slots][MP][MP] Z0
    float2* p;         // [slots][MP][MP] P = M Z0 (double-float)
    int rcap, hcap, mp;
};

// ---------------------------------------------------------------------------
// 1a. FP32 Householder tridiagonalisation, one CTA of 256 threads (a 16 x 16
//     grid) per slot, the matrix in registers.  Also splits M into its
//     double-float pair for the residual.
//
//     Reduction: thread (tx, ty) holds A[ty + 16 r][tx + 16 c] (both
//     triangles) in a[r][c].  Step i (i = n-1 .. 1, l = i - 1), with the
//     steps of tred2 (Wilkinson & Reinsch) without the row scaling:
//       - the half-warp that owns row i has written u = A[i][0..l] (with
//         u_l = f - g), h and g to shared memory at the end of step i + 1;
//       - p = A u / h: partial sums over each thread's columns, summed
//         across the half-warp by shuffles; f = p.u from per-half-warp
//         partials;
//       - A -= u q' + q u' (q = p - f / 2h u) on every element j, k <= l,
//         in registers; u / h goes to column i of the shared array;
//     two barriers a step.  Row i lives on in the shared array's lower
//     triangle, u / h in its upper triangle, as tred2 keeps them in A.
//     Accumulation: thread (tx, ty) holds Q[tx + 16 c][ty + 16 r], so that
//     g = u' Q (a sum over rows) stays within a half-warp; no barriers.
// ---------------------------------------------------------------------------
namespace em {

template <int R>
struct TredSmem {
    static constexpr int MP = 16 * R, LD = MP + 1;
    // W [MP][LD]: u_i in row i below the diagonal, u_i / h_i in column i
    // above it; P [MP]: p; hv, ev, dv [MP]: h (0: no reflector), e (tred2
    // form), the diagonal; red [16]: f partials
    static constexpr size_t bytes() { return ((size_t)MP * LD + 4 * MP + 16) * 4; }
};

// the lanes of this thread's half-warp
__device__ __forceinline__ unsigned hw_mask() { return 0xFFFFu << (threadIdx.x & 16); }

// half-warp all-reduce (the lanes of one half-warp hold one row's partials)
__device__ __forceinline__ float hw_sum(float v)
{
    const unsigned hm = hw_mask();
    v += __shfl_xor_sync(hm, v, 1);
    v += __shfl_xor_sync(hm, v, 2);
    v += __shfl_xor_sync(hm, v, 4);
    v += __shfl_xor_sync(hm, v, 8);
    return v;
}

// the owner half-warp of row i (ty == i % 16) publishes u = A[i][0..l], the
// reflector's h and g (or the skip: h = 0, e = A[i][l]) and the final
// diagonal A[i][i]
template <int R>
__device__ __forceinline__ void tred_publish(const float (&a)[R][R], int i, int tx, int ty, float* W, float* hv,
                                             float* ev, float* dv)
{
    constexpr int LD = 16 * R + 1;
    if ((i & 15) != ty) return;
    const int l = i - 1;
    float hp = 0.0f, f = 0.0f, aii = 0.0f;
    // the row's register block (a branch on i / 16, not R predicated copies)
    float rv[R];
    switch (i >> 4) {
#define EM_ROW_CASE(X)                                                          \
    case X:                                                                     \
        _Pragma("unroll") for (int c = 0; c < R; ++c) rv[c] = a[(X) < R ? (X) : 0][c]; \
        break;
        EM_ROW_CASE(0)
        EM_ROW_CASE(1)
        EM_ROW_CASE(2)
        EM_ROW_CASE(3)
        EM_ROW_CASE(4)
        EM_ROW_CASE(5)
#undef EM_ROW_CASE
    default:
#pragma unroll
        for (int c = 0; c < R; ++c) rv[c] = 0.0f;
    }
#pragma unroll
    for (int c = 0; c < R; ++c) {
        const int k = tx + 16 * c;
        const float v = rv[c];
        if (k <= l) {
            W[i * LD + k] = v;
            hp = fmaf(v, v, hp);
        }
        if (k == l) f = v;
        if (k == i) aii = v;
    }
    const float h0 = hw_sum(hp);
    const int lsrc = (threadIdx.x & 16) | (l & 15);   // lane of this half-warp holding column l
    const int isrc = (threadIdx.x & 16) | (i & 15);
    f = __shfl_sync(hw_mask(), f, lsrc);
    aii = __shfl_sync(hw_mask(), aii, isrc);
    if (tx == 0) {
        dv[i] = aii;
        if (l == 0 || h0 == 0.0f) {
            hv[i] = 0.0f;
            ev[i] = f;
        } else {
            const float g = (f >= 0.0f) ? -sqrtf(h0) : sqrtf(h0);
            hv[i] = h0 - f * g;
            ev[i] = g;
            W[i * LD + l] = f - g;
        }
    }
}

// one reduction step on the leading NB x NB blocks of 16 (NB = l / 16 + 1:
// the blocks wholly past l hold no work), with its barrier between p and
// the update
template <int R, int NB>
__device__ __forceinline__ void tred_step(float (&a)[R][R], int i, int l, float h, int tx, int ty, float* W,
                                          float* P, float* red)
{
    constexpr int LD = 16 * R + 1;
    const int tid = threadIdx.x;
    const float ih = 1.0f / h;
    float uk[NB], uj[NB];
#pragma unroll
    for (int c = 0; c < NB; ++c) {
        const int k = tx + 16 * c;
        uk[c] = k <= l ? W[i * LD + k] : 0.0f;
    }
#pragma unroll
    for (int r = 0; r < NB; ++r) {
        const int j = ty + 16 * r;
        uj[r] = j <= l ? W[i * LD + j] : 0.0f;
    }
    // p = A u / h, f = p.u
    float fp = 0.0f;
#pragma unroll
    for (int r = 0; r < NB; ++r) {
        float sm = 0.0f;
#pragma unroll
        for (int c = 0; c < NB; ++c) sm = fmaf(a[r][c], uk[c], sm);
        sm = hw_sum(sm) * ih;
        const int j = ty + 16 * r;
        if (tx == 0 && j <= l) P[j] = sm;
        fp = fmaf(sm, uj[r], fp);
    }
    if (tx == 0) red[ty] = fp;
    // u / h into column i (tred2 keeps it for the accumulation)
    if (tid <= l) W[tid * LD + i] = W[i * LD + tid] * ih;
    __syncthreads();
    // f: the 16 half-warp partials, one a lane, summed across each half-warp
    const float hh = hw_sum(red[tx]) / (h + h);
    float qk[NB];
#pragma unroll
    for (int c = 0; c < NB; ++c) {
        const int k = tx + 16 * c;
        qk[c] = k <= l ? P[k] - hh * uk[c] : 0.0f;
    }
#pragma unroll
    for (int r = 0; r < NB; ++r) {
        const int j = ty + 16 * r;
        const float qj = j <= l ? P[j] - hh * uj[r] : 0.0f;
#pragma unroll
        for (int c = 0; c < NB; ++c) a[r][c] -= uj[r] * qk[c] + qj * uk[c];
    }
}

template <int R, int NB>
__device__ __forceinline__ void tred_step_nb(int nb, float (&a)[R][R], int i, int l, float h, int tx, int ty,
                                             float* W, float* P, float* red)
{
    if constexpr (NB < R) {
        if (nb == NB) tred_step<R, NB>(a, i, l, h, tx, ty, W, P, red);
        else tred_step_nb<R, NB + 1>(nb, a, i, l, h, tx, ty, W, P, red);
    } else {
        tred_step<R, R>(a, i, l, h, tx, ty, W, P, red);
    }
}

// one accumulation step on the leading NB x NB blocks
template <int R, int NB>
__device__ __forceinline__ void acc_step(float (&q)[R][R], int i, int l, int tx, int ty, const float* W)
{
    constexpr int LD = 16 * R + 1;
    float uk[NB], vk[NB];
#pragma unroll
    for (int c = 0; c < NB; ++c) {
        const int k = tx + 16 * c;
        uk[c] = k <= l ? W[i * LD + k] : 0.0f;
        vk[c] = k <= l ? W[k * LD + i] : 0.0f;
    }
#pragma unroll
    for (int r = 0; r < NB; ++r) {
        float g = 0.0f;
#pragma unroll
        for (int c = 0; c < NB; ++c) g = fmaf(uk[c], q[c][r], g);
        g = hw_sum(g);
        const int j = ty + 16 * r;
        if (j <= l)
#pragma unroll
            for (int c = 0; c < NB; ++c) q[c][r] -= g * vk[c];
    }
}

template <int R, int NB>
__device__ __forceinline__ void acc_step_nb(int nb, float (&q)[R][R], int i, int l, int tx, int ty, const float* W)
{
    if constexpr (NB < R) {
        if (nb == NB) acc_step<R, NB>(q, i, l, tx, ty, W);
        else acc_step_nb<R, NB + 1>(nb, q, i, l, tx, ty, W);
    } else {
        acc_step<R, R>(q, i, l, tx, ty, W);
    }
}

}  // namespace em

template <int R>
__global__ void __launch_bounds__(256, 3) k_em_tred(CalcArgs a, EmSlots z)
{
    using TS = em::TredSmem<R>;
    constexpr int MP = TS::MP, LD = TS::LD;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float* W = (float*)smem_raw;
    float* P = W + MP * LD;
    float* hv = P + MP;
    float* ev = hv + MP;
    float* dv = ev + MP;
    float* red = dv + MP;
    const int m = a.m, n = a.m;
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4, slot = blockIdx.x;
    if (!(a.eaux[2 * (size_t)slot] > 0.0)) return;   // empty point
    const size_t q0 = (size_t)slot * m * m;
    if (tid == 0) {
        hv[0] = 0.0f;   // no reflector at index 0
        ev[0] = 0.0f;
    }
    // M as the transform kernel left it (float pairs, upper triangle): the
    // high parts, both triangles, into registers
    float a_[R][R];
#pragma unroll
    for (int r = 0; r < R; ++r)
#pragma unroll
        for (int c = 0; c < R; ++c) {
            const int j = ty + 16 * r, k = tx + 16 * c;
            a_[r][c] = (j < m && k < m) ? z.mhl[q0 + (size_t)(k >= j ? j * m + k : k * m + j)].x : 0.0f;
        }
    em::tred_publish<R>(a_, n - 1, tx, ty, W, hv, ev, dv);
    for (int i = n - 1; i >= 1; --i) {
        const int l = i - 1;
        __syncthreads();   // row i, h, g published; the last step's P and red read
        const float h = hv[i];
        if (h != 0.0f) em::tred_step_nb<R, 1>((l >> 4) + 1, a_, i, l, h, tx, ty, W, P, red);
        if (l >= 1) em::tred_publish<R>(a_, l, tx, ty, W, hv, ev, dv);
        else if (ty == 0 && tx == 0) dv[0] = a_[0][0];
    }
    __syncthreads();
    // accumulation of Q = H_{n-1} ... H_1 (tred2's second loop)
    float q_[R][R];   // q_[c][r] = Q[tx + 16 c][ty + 16 r]
#pragma unroll
    for (int c = 0; c < R; ++c)
#pragma unroll
        for (int r = 0; r < R; ++r) q_[c][r] = 0.0f;
    for (int i = 0; i < n; ++i) {
        const int l = i - 1;
        if (hv[i] != 0.0f) em::acc_step_nb<R, 1>((l >> 4) + 1, q_, i, l, tx, ty, W);
#pragma unroll
        for (int c = 0; c < R; ++c)
#pragma unroll
            for (int r = 0; r < R; ++r)
                if (tx + 16 * c == i && ty + 16 * r == i) q_[c][r] = 1.0f;
    }
    __syncthreads();   // W free
#pragma unroll
    for (int c = 0; c < R; ++c)
#pragma unroll
        for (int r = 0; r < R; ++r) W[(tx + 16 * c) * LD + ty + 16 * r] = q_[c][r];
    __syncthreads();
    for (int i = tid; i < m * m; i += 256) {
        const int r = i / m, c = i - r * m;
        z.q[q0 + i] = W[r * LD + c];
    }
    // d and e in QL form (e[i] couples i and i + 1)
    for (int i = tid; i < m; i += 256) {
        z.d[(size_t)slot * m + i] = dv[i];
        z.e[(size_t)slot * m + i] = i + 1 < m ? ev[i + 1] : 0.0f;
    }
}

// ---------------------------------------------------------------------------
// 1b. FP32 QL chains, one thread per slot, rotations logged.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(EM_QL_T) k_em_ql(int nslots, int m, const double* __restrict__ eaux, EmSlots z)
{
    extern __shared__ float qsf[];   // [2][m][EM_QL_T]
    const int lane = threadIdx.x;
    const int slot = blockIdx.x * EM_QL_T + lane;
    if (slot >= nslots || !(eaux[2 * (size_t)slot] > 0.0)) return;   // no barrier below
    float* dcol = qsf + lane;
    float* ecol = qsf + (size_t)m * EM_QL_T + lane;
    for (int i = 0; i < m; ++i) {
        dcol[i * EM_QL_T] = z.d[(size_t)slot * m + i];
        ecol[i * EM_QL_T] = z.e[(size_t)slot * m + i];
    }
    int n = 0;
    const int stt = la::ql_chain(dcol, ecol, m, EM_QL_T, z.rot + (size_t)slot * z.rcap, z.rcap,
                                 z.hdr + (size_t)slot * z.hcap, z.hcap, &n);
    z.nh[slot] = stt == 0 ? n : -stt;
    if (stt == 0)
        for (int i = 0; i < m; ++i) z.d[(size_t)slot * m + i] = dcol[i * EM_QL_T];
}

// ---------------------------------------------------------------------------
// 1c. The log replayed onto Q (rows in parallel, one thread each); a point
//     whose chain failed (log full, or no convergence within the chain) runs
//     tql2 in the CTA.  The log is staged through shared memory EM_RCH
//     rotations at a time: every row walks the same sequence, so the
//     control flow is uniform and each rotation is read from global memory
//     once per point.
// ---------------------------------------------------------------------------
#define EM_RCH 1024

// NT = m rounded up to 32: a thread per row of Q and no idle warp
template <int NT>
__global__ void __launch_bounds__(NT) k_em_replay(CalcArgs a, EmSlots z)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int m = a.m, lda = m + 1;
    const int tid = threadIdx.x, slot = blockIdx.x;
    float2* rbuf = (float2*)smem_raw;                 // [EM_RCH]
    float* A = (float*)(rbuf + EM_RCH);
    float* d = A + (size_t)m * lda;
    float* e = d + m;
    float* cs = e + m;
    float* sn = cs + m;
    int* ctl = (int*)(sn + m);
    if (!(a.eaux[2 * (size_t)slot] > 0.0)) return;
    const size_t q0 = (size_t)slot * m * m;
    for (int i = tid; i < m * m; i += NT) {
        const int r = i / m, c = i - r * m;
        A[r * lda + c] = z.q[q0 + i];
        // the lower triangle of M's float pairs, for the residual's rows
        if (c < r) z.mhl[q0 + i] = z.mhl[q0 + (size_t)c * m + r];
    }
    const int stt = z.nh[slot];
    for (int i = tid; i < m; i += NT) {
        d[i] = z.d[(size_t)slot * m + i];
        e[i] = z.e[(size_t)slot * m + i];
    }
    __syncthreads();
    int rc = 0;
    if (stt >= 0) {
        const float2* rot = z.rot + (size_t)slot * z.rcap;
        const int2* hdr = z.hdr + (size_t)slot * z.hcap;
        float* Ak = A + (size_t)(tid < m ? tid : 0) * lda;
        int h = 0, i = 0, r = 0;
        bool inside = false;
        float carry = 0.0f;
        for (int c0 = 0; h < stt; c0 += EM_RCH) {
            __syncthreads();
            for (int q = tid; q < EM_RCH && c0 + q < z.rcap; q += NT) rbuf[q] = rot[c0 + q];
            __syncthreads();
            while (h < stt) {
                const int2 hd = hdr[h];
                if (hd.x < hd.y) {       // an empty sweep
                    ++h;
                    continue;
                }
                if (!inside) {
                    i = hd.x;
                    if (tid < m) carry = Ak[i + 1];
                    inside = true;
                }
                // the rotations of this sweep that are in the chunk (i runs
                // down to hd.y), with the bounds taken out of the loop
                const int nit = (i - hd.y + 1 < c0 + EM_RCH - r) ? i - hd.y + 1 : c0 + EM_RCH - r;
                if (tid < m) {
                    const float2* qp = rbuf + (r - c0);
                    float* ap = Ak + i;
#pragma unroll 4
                    for (int t = 0; t < nit; ++t) {
                        const float2 q = qp[t];
                        const float zi = ap[-t];
                        ap[1 - t] = q.y * zi + q.x * carry;
                        carry = q.x * zi - q.y * carry;
                    }
                }
                i -= nit;
                r += nit;
                if (i >= hd.y) break;    // the chunk is used up inside the sweep
                if (tid < m) Ak[hd.y] = carry;
                inside = false;
                ++h;
            }
        }
        __syncthreads();
    } else {
        rc = la::tql2<NT>(A, m, lda, d, e, cs, sn, ctl);
    }
    if (rc != 0 && tid == 0) {
        const int pt = a.order ? a.order[slot] : a.item0 + slot;
        a.status[pt] = rc;
    }
    for (int i = tid; i < m * m; i += NT) {
        const int r = i / m, c = i - r * m;
        z.q[q0 + i] = A[r * lda + c];
    }
    if (stt < 0)
        for (int i = tid; i < m; i += NT) z.d[(size_t)slot * m + i] = d[i];
}

// ---------------------------------------------------------------------------
// 2-6. the refinement, one CTA of 256 threads (a 16 x 16 grid) per slot
// ---------------------------------------------------------------------------
namespace em {

// acc (hi, lo) += (ah + al) b: the product ah b exactly (FMA), summed into
// hi by TwoSum; the errors, and al b, into lo
__device__ __forceinline__ void df_fma(float& sh, float& sl, float ah, float al, float b)
{
    const float p = ah * b;
    const float e = fmaf(ah, b, -p);
    const float s = sh + p;
    const float v = s - sh;
    const float t = (sh - (s - v)) + (p - v);
    sh = s;
    sl += t + e;
    sl = fmaf(al, b, sl);
}

// C = op(X) op(Y) for MP x MP float matrices in shared memory (row stride
// lda): thread (ty, tx) of the 16 x 16 grid owns rows ty + 16 r and columns
// tx + 16 c; k runs over the first n indices (the rest are zero padding).
// SYM: the product is symmetric; only the blocks c >= r are formed and the
// others mirrored.  C may alias X or Y.
template <int R, bool TX, bool TY, bool SYM>
__device__ __forceinline__ void mm(float* C, const float* X, const float* Y, int n, int lda)
{
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    float acc[R][R];
#pragma unroll
    for (int r = 0; r < R; ++r)
#pragma unroll
        for (int c = 0; c < R; ++c) acc[r][c] = 0.0f;
    for (int k = 0; k < n; ++k) {
        float xv[R], yv[R];
#pragma unroll
        for (int r = 0; r < R; ++r) xv[r] = TX ? X[k * lda + ty + 16 * r] : X[(ty + 16 * r) * lda + k];
#pragma unroll
        for (int c = 0; c < R; ++c) yv[c] = TY ? Y[(tx + 16 * c) * lda + k] : Y[k * lda + tx + 16 * c];
#pragma unroll
        for (int r = 0; r < R; ++r)
#pragma unroll
            for (int c = 0; c < R; ++c)
                if (!SYM || c >= r) acc[r][c] = fmaf(xv[r], yv[c], acc[r][c]);
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < R; ++r)
#pragma unroll
        for (int c = 0; c < R; ++c)
            if (!SYM || c >= r) {
                C[(ty + 16 * r) * lda + tx + 16 * c] = acc[r][c];
                if (SYM && c > r) C[(tx + 16 * c) * lda + ty + 16 * r] = acc[r][c];
            }
    __syncthreads();
}

}  // namespace em

template <int R>
__global__ void __launch_bounds__(EM_NT, 2) k_em_refine(CalcArgs a, EmSlots z)
{
    constexpr int MP = 16 * R, LDA = MP + 1;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int m = a.m, md = a.md;
    const int tid = threadIdx.x, slot = blockIdx.x, tx = tid & 15, ty = tid >> 4;
    // two matrices: the products run in place (mm writes its result after
    // every operand read), so that two CTAs fit on an SM
    float* Q = (float*)smem_raw;                     // [MP][LDA] eigenvectors (columns)
    float* B = Q + MP * LDA;                         // [MP][LDA] Z0, then R, D~, D
    float2* S = (float2*)(B + MP * LDA);             // [EM_KCH][MP] staged rows of P
    float* lam = (float*)(S + EM_KCH * MP);          // [MP] eigenvalues
    float* sig = lam + MP;                           // [MP] lambda^1/2
    float* vf = sig + MP;                            // [MP] float vector
    float* vt = vf + MP;                             // [MP] float vector
    double* bv = (double*)(vt + MP);                 // [MP] S's
    double* wv = bv + MP;                            // [MP] w
    double* rv = wv + MP;                            // [MP] residual
    double* red = rv + MP;                           // [EM_NT / 32]
    const double pd = a.eaux[2 * (size_t)slot];
    if (!(pd > 0.0)) return;   // empty point: written by the transform kernel
    const int pt = a.order ? a.order[slot] : a.item0 + slot;
    const double trss = a.eaux[2 * (size_t)slot + 1];
    const size_t q0 = (size_t)slot * m * m, z0 = (size_t)slot * MP * MP;

    // eigenvectors and eigenvalues (zero padding beyond m)
    for (int i = tid; i < MP * MP; i += EM_NT) {
        const int r = i / MP, c = i - r * MP;
        Q[r * LDA + c] = (r < m && c < m) ? z.q[q0 + (size_t)r * m + c] : 0.0f;
    }
    for (int i = tid; i < MP; i += EM_NT) {
        const float l = i < m ? z.d[(size_t)slot * m + i] : 0.0f;
        lam[i] = l;
        sig[i] = i < m ? sqrtf(l) : 0.0f;
        bv[i] = i < m ? a.eb[(size_t)slot * m + i] : 0.0;
    }
    __syncthreads();

    // 2. Z0 = Q diag(lambda^-1/2) Q'  (B = Q diag, then B Q' in place)
    for (int i = tid; i < MP * MP; i += EM_NT) {
        const int r = i / MP, c = i - r * MP;
        B[r * LDA + c] = c < m ? Q[r * LDA + c] * rsqrtf(lam[c]) : 0.0f;
    }
    __syncthreads();
    em::mm<R, false, true, true>(B, B, Q, m, LDA);
    for (int i = tid; i < MP * MP; i += EM_NT) {
        const int r = i / MP, c = i - r * MP;
        z.z0[z0 + i] = B[r * LDA + c];
    }

    // 3a. P = M Z0 (double-float; M as its hi/lo pair, rows from global),
    //     in two halves of the column blocks (register pressure)
    constexpr int RC = (R + 1) / 2;
#pragma unroll
    for (int cb = 0; cb < R; cb += RC) {
        float ph[R][RC], pl[R][RC];
#pragma unroll
        for (int r = 0; r < R; ++r)
#pragma unroll
            for (int c = 0; c < RC; ++c) ph[r][c] = pl[r][c] = 0.0f;
        for (int k = 0; k < m; ++k) {
            float2 mv[R];
            float zv[RC];
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const int i = ty + 16 * r;
                mv[r] = i < m ? z.mhl[q0 + (size_t)i * m + k] : make_float2(0.0f, 0.0f);
            }
#pragma unroll
            for (int c = 0; c < RC; ++c) zv[c] = (cb + c < R) ? B[k * LDA + tx + 16 * (cb + c)] : 0.0f;
#pragma unroll
            for (int r = 0; r < R; ++r)
#pragma unroll
                for (int c = 0; c < RC; ++c)
                    if (cb + c < R) em::df_fma(ph[r][c], pl[r][c], mv[r].x, mv[r].y, zv[c]);
        }
#pragma unroll
        for (int r = 0; r < R; ++r)
#pragma unroll
            for (int c = 0; c < RC; ++c)
                if (cb + c < R)
                    z.p[z0 + (size_t)(ty + 16 * r) * MP + tx + 16 * (cb + c)] = make_float2(ph[r][c], pl[r][c]);
    }
    __syncthreads();   // P complete in global memory for the whole CTA

    // 3b. R = I - Z0 P (double-float), R_hi into B
    {
        float rh[R][R], rl[R][R];
#pragma unroll
        for (int r = 0; r < R; ++r)
#pragma unroll
            for (int c = 0; c < R; ++c) rh[r][c] = rl[r][c] = 0.0f;
        for (int k0 = 0; k0 < m; k0 += EM_KCH) {
            const int kn = (m - k0 < EM_KCH) ? m - k0 : EM_KCH;
            for (int i = tid; i < kn * MP; i += EM_NT) {
                const int kk = i / MP, c = i - kk * MP;
                S[kk * MP + c] = z.p[z0 + (size_t)(k0 + kk) * MP + c];
            }
            __syncthreads();
            for (int kk = 0; kk < kn; ++kk) {
                float zv[R];
                float2 pv[R];
#pragma unroll
                for (int r = 0; r < R; ++r) zv[r] = B[(ty + 16 * r) * LDA + k0 + kk];
#pragma unroll
                for (int c = 0; c < R; ++c) pv[c] = S[kk * MP + tx + 16 * c];
#pragma unroll
                for (int r = 0; r < R; ++r)
#pragma unroll
                    for (int c = 0; c < R; ++c)
                        if (c >= r) em::df_fma(rh[r][c], rl[r][c], pv[c].x, pv[c].y, zv[r]);
            }
            __syncthreads();
        }
        __syncthreads();   // every thread is done reading Z0 from B
        // R is symmetric: blocks c >= r formed, the others mirrored
#pragma unroll
        for (int r = 0; r < R; ++r)
#pragma unroll
            for (int c = 0; c < R; ++c)
                if (c >= r) {
                    const int i = ty + 16 * r, j = tx + 16 * c;
                    // (delta - hi) is exact near 1 (Sterbenz), then the low part
                    const float one = (i == j && i < m) ? 1.0f : 0.0f;
                    const float v = (i < m && j < m) ? (one - rh[r][c]) - rl[r][c] : 0.0f;
                    B[i * LDA + j] = v;
                    if (c > r) B[j * LDA + i] = v;
                }
    }
    __syncthreads();

    // 4. D~ = Q' R Q, D~_ij /= (sigma_i + sigma_j), D = Q D~ Q'
    em::mm<R, true, false, false>(B, Q, B, m, LDA);
    em::mm<R, false, false, true>(B, B, Q, m, LDA);
    for (int i = tid; i < MP * MP; i += EM_NT) {
        const int r = i / MP, c = i - r * MP;
        B[r * LDA + c] = (r < m && c < m) ? B[r * LDA + c] / (sig[r] + sig[c]) : 0.0f;
    }
    __syncthreads();
    em::mm<R, false, false, false>(B, Q, B, m, LDA);
    em::mm<R, false, true, true>(B, B, Q, m, LDA);

    // 5. T = Z0 + D in FP64, relaxed and cast (transforms.c:1270-1296);
    //    tr(M^-1) = |T|_F^2 for the degrees of freedom
    const size_t tbase = (size_t)pt * md * m;
    double tr = 0.0;
    for (int i = tid; i < m * m; i += EM_NT) {
        const int e1 = i / m, e2 = i - e1 * m;
        const double t = (double)z.z0[z0 + (size_t)e1 * MP + e2] + (double)B[e1 * LDA + e2];
        tr = fma(t, t, tr);
        if (e1 < md && a.mode != ENKFG_MODE_ENOI && a.T != nullptr) {
            const double tt = (e1 == e2) ? (t - 1.0) * a.alpha + 1.0 : t * a.alpha;
            a.T[tbase + (size_t)e1 * m + e2] = (float)tt;
            if (a.T64) a.T64[tbase + (size_t)e1 * m + e2] = tt;
        }
    }
    const double trinv = la::block_sum<EM_NT>(tr, red);

    // 6. w = M^-1 S's by iterative refinement: r = S's - M w in FP64 (M from
    //    the slot's FP64 upper triangle), w += Q diag(1/lambda) Q' r in FP32
    for (int i = tid; i < MP; i += EM_NT) {
        wv[i] = 0.0;
        rv[i] = bv[i];
    }
    __syncthreads();
    for (int it = 0; it < EM_W_STEPS; ++it) {
        if (tid < m) {
            float t = 0.0f;
            for (int k = 0; k < m; ++k) t = fmaf(Q[k * LDA + tid], (float)rv[k], t);
            vt[tid] = t / lam[tid];
        }
        __syncthreads();
        if (tid < m) {
            float y = 0.0f;
            for (int k = 0; k < m; ++k) y = fmaf(Q[tid * LDA + k], vt[k], y);
            wv[tid] += (double)y;
        }
        __syncthreads();
        if (tid < m) {
            double r = bv[tid];
            for (int k = 0; k < m; ++k) {
                const double mik = (k >= tid) ? a.eq[q0 + (size_t)tid * m + k] : a.eq[q0 + (size_t)k * m + tid];
                r = fma(-mik, wv[k], r);
            }
            rv[tid] = r;
        }
        __syncthreads();
    }
    if (tid < m) {
        a.w[(size_t)pt * m + tid] = (float)wv[tid];
        if (a.w64) a.w64[(size_t)pt * m + tid] = wv[tid];
    }
    if (a.want_diag) diag_single(a, pt, (int)pd, (double)m - trinv, trss);
}

bool etkf_mixed_supported(int m) { return m >= 2 && m <= 96; }

// bytes of one batch slot of the refined solve
size_t etkf_mixed_slot_bytes(int m)
{
    int R = (m + 15) / 16;
    if (R < 2) R = 2;
    if (R == 5) R = 6;
    const size_t MP = 16 * (size_t)R, rcap = (size_t)m * m + 64 * (size_t)m, hcap = 8 * (size_t)m;
    return (size_t)m * m * 8 + (size_t)3 * m * 8 + 16     // M, S's, aux (FP64 slots)
           + (size_t)m * m * 12 + (size_t)2 * m * 4        // Q, M hi/lo, d, e
           + rcap * 8 + hcap * 8 + 4                       // rotation log
           + MP * MP * 12;                                 // Z0, P
}

template <int R>
static size_t em_refine_smem()
{
    constexpr int MP = 16 * R, LDA = MP + 1;
    return (size_t)2 * MP * LDA * 4 + (size_t)EM_KCH * MP * 8 + (size_t)4 * MP * 4 + (size_t)3 * MP * 8 +
           (EM_NT / 32) * 8;
}

template <int R>
static enkfg_status em_launch_refine(enkfg_ctx* ctx, const CalcArgs& b, const EmSlots& z, int nb, cudaStream_t st)
{
    const size_t smem = em_refine_smem<R>();
    CK(cudaFuncSetAttribute(k_em_refine<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_em_refine<R><<<nb, EM_NT, smem, st>>>(b, z);
    CKL();
    return ENKFG_OK;
}

// The mixed-precision ETKF transform stage in batches of points: the
// transform kernel (S'S and S's on the tensor cores, M saved per slot), then
// the FP32 eigendecomposition and the refined solve of every slot.
enkfg_status run_etkf_mixed(enkfg_ctx* ctx, const CalcArgs& a0, cudaStream_t st)
{
    enkfg_status s;
    const int m = a0.m, nitems = a0.nitems;
    // the register tile of the refinement kernel: R = 2, 3, 4 or 6 (16 R >= m)
    int R = (m + 15) / 16;
    if (R < 2) R = 2;
    if (R == 5) R = 6;
    const int MP = 16 * R;
    const int rcap = m * m + 64 * m;         // QL typically needs about 0.75 m^2 rotations
    const int hcap = 8 * m;
    const size_t B = batch_points(ctx, etkf_mixed_slot_bytes(m), (size_t)8 << 30, nitems);   // about 8 GB a batch
    if ((s = ensure(ctx, &ctx->d_eq, &ctx->eq_cap, B * m * m))) return s;
    if ((s = ensure(ctx, &ctx->d_eb, &ctx->eb_cap, B * m))) return s;
    if ((s = ensure(ctx, &ctx->d_eaux, &ctx->eaux_cap, B * 2))) return s;
    if ((s = ensure(ctx, &ctx->d_emq, &ctx->emq_cap, B * m * m))) return s;
    if ((s = ensure(ctx, &ctx->d_emmhl, &ctx->emmhl_cap, B * m * m))) return s;
    if ((s = ensure(ctx, &ctx->d_emd, &ctx->emd_cap, B * m))) return s;
    if ((s = ensure(ctx, &ctx->d_eme, &ctx->eme_cap, B * m))) return s;
    if ((s = ensure(ctx, &ctx->d_emrot, &ctx->emrot_cap, B * rcap))) return s;
    if ((s = ensure(ctx, &ctx->d_emhdr, &ctx->emhdr_cap, B * hcap))) return s;
    if ((s = ensure(ctx, &ctx->d_emnh, &ctx->emnh_cap, B))) return s;
    if ((s = ensure(ctx, &ctx->d_emz0, &ctx->emz0_cap, B * MP * MP))) return s;
    if ((s = ensure(ctx, &ctx->d_emp, &ctx->emp_cap, B * MP * MP))) return s;
    EmSlots z;
    z.q = ctx->d_emq;
    z.mhl = ctx->d_emmhl;
    z.d = ctx->d_emd;
    z.e = ctx->d_eme;
    z.rot = ctx->d_emrot;
    z.hdr = ctx->d_emhdr;
    z.nh = ctx->d_emnh;
    z.z0 = ctx->d_emz0;
    z.p = ctx->d_emp;
    z.rcap = rcap;
    z.hcap = hcap;
    z.mp = MP;
    const int lda = m + 1;
    const size_t tsmem = R == 2 ? em::TredSmem<2>::bytes() : R == 3 ? em::TredSmem<3>::bytes()
                         : R == 4 ? em::TredSmem<4>::bytes() : em::TredSmem<6>::bytes();
    const size_t qsmem = (size_t)2 * m * EM_QL_T * 4;
    const size_t rsmem = (size_t)EM_RCH * 8 + ((size_t)m * lda + 4 * (size_t)m) * 4 + 16;
    CK(cudaFuncSetAttribute(k_em_ql, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)qsmem));
    const int rnt = (m + 31) / 32 * 32;   // k_em_replay: a thread per row
    switch (rnt) {
    case 32: CK(cudaFuncSetAttribute(k_em_replay<32>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rsmem)); break;
    case 64: CK(cudaFuncSetAttribute(k_em_replay<64>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rsmem)); break;
    default: CK(cudaFuncSetAttribute(k_em_replay<96>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rsmem)); break;
    }
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
        b.emhl = z.mhl;
        if (b.persistent) CK(cudaMemsetAsync(ctx->d_qhead, 0, sizeof(int), st));
        batch_mark(ctx, 0, st);
        if ((s = launch_mixed(ctx, b, st))) return s;
        batch_mark(ctx, 1, st);
        switch (R) {
        case 2: k_em_tred<2><<<nb, 256, tsmem, st>>>(b, z); break;
        case 3: k_em_tred<3><<<nb, 256, tsmem, st>>>(b, z); break;
        case 4: k_em_tred<4><<<nb, 256, tsmem, st>>>(b, z); break;
        default: k_em_tred<6><<<nb, 256, tsmem, st>>>(b, z); break;
        }
        CKL();
        k_em_ql<<<div_up(nb, EM_QL_T), EM_QL_T, qsmem, st>>>(nb, m, ctx->d_eaux, z);
        CKL();
        switch (rnt) {
        case 32: k_em_replay<32><<<nb, 32, rsmem, st>>>(b, z); break;
        case 64: k_em_replay<64><<<nb, 64, rsmem, st>>>(b, z); break;
        default: k_em_replay<96><<<nb, 96, rsmem, st>>>(b, z); break;
        }
        CKL();
        switch (R) {
        case 2: s = em_launch_refine<2>(ctx, b, z, nb, st); break;
        case 3: s = em_launch_refine<3>(ctx, b, z, nb, st); break;
        case 4: s = em_launch_refine<4>(ctx, b, z, nb, st); break;
        case 6: s = em_launch_refine<6>(ctx, b, z, nb, st); break;
        default:
            set_err(ctx, "the refined ETKF solve supports nmem <= 96 (got %d)", m);
            return ENKFG_EUNSUPPORTED;
        }
        if (s) return s;
        batch_mark(ctx, 2, st);
        batch_out(ctx, i0, nb, st);
    }
    return ENKFG_OK;
}
