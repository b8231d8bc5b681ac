// linalg.cuh -- FP64 dense kernels for one local analysis, executed by a
// whole CTA on matrices held in shared memory.
//
//   eig_sym       symmetric eigendecomposition: Householder reduction to
//                 tridiagonal form with accumulation of the transformation
//                 (Wilkinson & Reinsch, Handbook for Automatic Computation
//                 vol. II, "tred2"), then the implicit-shift QL iteration
//                 ("tql2") on the tridiagonal matrix.  The reductions and
//                 rank-2 updates of the Householder step and the rotations
//                 applied to the eigenvector matrix are spread over the CTA;
//                 the QL rotation chain itself is sequential and runs on one
//                 thread while the others wait.
//   spd_inverse   M^-1 of an SPD matrix in place by the symmetric sweep
//                 operator (Gauss-Jordan elimination without pivoting, kept
//                 symmetric, on the upper triangle only).
//
// These replace LAPACK dgesvd (reference calc/calcs.c:338) and dpotrf/dpotri
// (calcs.c:103-132).  For M = I + S'S (eigenvalues >= 1) both are stable, so
// the results agree with LAPACK's to a few units of rounding times the
// condition of M.
//
// The eigensolver routines are templates on the scalar type F: double for
// the FP64 solve, float for the FP32 decomposition that seeds the refined
// inverse square root of the mixed-precision path.
#pragma once

namespace la {

// unit roundoff used by the QL convergence test: 2^-52 (double), 2^-23 (float)
template <typename F> struct Eps;
template <> struct Eps<double> { static constexpr double value = 2.220446049250313e-16; };
template <> struct Eps<float> { static constexpr float value = 1.1920929e-07f; };

// (c, s) pair of a logged rotation
template <typename F> struct Vec2;
template <> struct Vec2<double> { typedef double2 type; };
template <> struct Vec2<float> { typedef float2 type; };

__device__ __forceinline__ double rsq(double x) { return rsqrt(x); }
__device__ __forceinline__ float rsq(float x) { return rsqrtf(x); }

template <int NT, typename F>
__device__ __forceinline__ F block_sum(F v, F* red)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) red[wid] = v;
    __syncthreads();
    F s = F(0);
#pragma unroll
    for (int w = 0; w < NT / 32; ++w) s += red[w];
    return s;
}

// Householder tridiagonalisation of the symmetric A (n x n, row stride lda,
// both triangles valid on entry) with the transformations accumulated: on
// return A holds the orthogonal Q, d the diagonal and e the off-diagonal of
// the tridiagonal matrix in QL form (e[i] couples i and i+1, e[n-1] = 0).
// red: NT/32 doubles.
template <int NT, typename F>
__device__ void tred2(F* A, int n, int lda, F* d, F* e, F* red)
{
    const int tid = threadIdx.x;
    // ---- Householder reduction (rows n-1 .. 1) ----
    for (int i = n - 1; i >= 1; --i) {
        int l = i - 1;
        F* Ai = A + (size_t)i * lda;
        F h = F(0);
        if (l > 0) {
            F part = F(0);
            for (int k = tid; k <= l; k += NT) part += fabs(Ai[k]);
            F scale = block_sum<NT>(part, red);
            if (scale == F(0)) {
                if (tid == 0) e[i] = Ai[l];
                __syncthreads();
            } else {
                // one division a step, multiplications per element (FP64
                // division is a long instruction sequence on GB300)
                const F iscale = F(1) / scale;
                part = F(0);
                for (int k = tid; k <= l; k += NT) {
                    F v = Ai[k] * iscale;
                    Ai[k] = v;
                    part += v * v;
                }
                h = block_sum<NT>(part, red);
                F f = Ai[l];
                F g = (f >= F(0)) ? -sqrt(h) : sqrt(h);
                h -= f * g;
                __syncthreads();
                if (tid == 0) {
                    e[i] = scale * g;
                    Ai[l] = f - g;
                }
                __syncthreads();
                // p = A u / h (into e[0..l]); column i keeps u / h
                const F ih = F(1) / h;
                for (int j = tid; j <= l; j += NT) {
                    F g2 = F(0);
                    const F* Aj = A + (size_t)j * lda;
                    for (int k = 0; k <= j; ++k) g2 += Aj[k] * Ai[k];
                    for (int k = j + 1; k <= l; ++k) g2 += A[(size_t)k * lda + j] * Ai[k];
                    e[j] = g2 * ih;
                }
                __syncthreads();
                for (int j = tid; j <= l; j += NT) A[(size_t)j * lda + i] = Ai[j] * ih;
                part = F(0);
                for (int j = tid; j <= l; j += NT) part += e[j] * Ai[j];
                F ff = block_sum<NT>(part, red);
                F hh = ff / (h + h);
                for (int j = tid; j <= l; j += NT) e[j] = e[j] - hh * Ai[j];
                __syncthreads();
                // rank-2 update of the lower triangle rows 0..l
                int tri = (l + 1) * (l + 2) / 2;
                for (int idx = tid; idx < tri; idx += NT) {
                    int j = (int)((sqrtf(8.0f * (float)idx + 1.0f) - 1.0f) * 0.5f);
                    while ((j + 1) * (j + 2) / 2 <= idx) ++j;
                    while (j * (j + 1) / 2 > idx) --j;
                    int k = idx - j * (j + 1) / 2;
                    A[(size_t)j * lda + k] -= (Ai[j] * e[k] + e[j] * Ai[k]);
                }
                __syncthreads();
            }
        } else {
            if (tid == 0) e[i] = Ai[l];
            __syncthreads();
        }
        if (tid == 0) d[i] = h;
        __syncthreads();
    }
    if (tid == 0) {
        d[0] = F(0);
        e[0] = F(0);
    }
    __syncthreads();
    // ---- accumulate the transformations ----
    for (int i = 0; i < n; ++i) {
        int l = i - 1;
        F* Ai = A + (size_t)i * lda;
        if (d[i] != F(0)) {
            for (int j = tid; j <= l; j += NT) {
                F g = F(0);
                for (int k = 0; k <= l; ++k) g += Ai[k] * A[(size_t)k * lda + j];
                for (int k = 0; k <= l; ++k) A[(size_t)k * lda + j] -= g * A[(size_t)k * lda + i];
            }
        }
        __syncthreads();
        if (tid == 0) d[i] = Ai[i];
        for (int j = tid; j <= l; j += NT) {
            A[(size_t)j * lda + i] = F(0);
            Ai[j] = F(0);
        }
        if (tid == 0) Ai[i] = F(1);
        __syncthreads();
    }
    if (tid == 0) {
        for (int i = 1; i < n; ++i) e[i - 1] = e[i];
        e[n - 1] = F(0);
    }
    __syncthreads();
}

// Implicit QL on the tridiagonal (d, e) of tred2 with the rotations applied to
// the rows of A: on return column k of A is the eigenvector of eigenvalue
// d[k].  cs, sn: scratch of n doubles each; ctl: 4 ints.  Returns 0 or 1 (QL
// did not converge).
template <int NT, typename F>
__device__ int tql2(F* A, int n, int lda, F* d, F* e, F* cs, F* sn, int* ctl)
{
    const int tid = threadIdx.x;
    if (tid == 0) ctl[3] = 0;
    __syncthreads();
    for (int l = 0; l < n; ++l) {
        // the step that ends a sweep leaves the loop below before its
        // closing barrier: every thread must have read that step's control
        // words before thread 0 writes the next sweep's, or a late thread
        // would take the new words for the old sweep and fall out of step
        // with the block's barriers
        __syncthreads();
        int iter = 0;
        for (;;) {
            if (tid == 0) {
                int m;
                for (m = l; m < n - 1; ++m) {
                    F dd = fabs(d[m]) + fabs(d[m + 1]);
                    if (fabs(e[m]) <= Eps<F>::value * dd) break;
                }
                ctl[0] = m;
                if (m != l) {
                    if (iter >= 60) {
                        ctl[0] = l;
                        ctl[3] = 1;
                    } else {
                        F g = (d[l + 1] - d[l]) / (F(2) * e[l]);
                        F r = sqrt(fma(g, g, F(1)));
                        g = d[m] - d[l] + e[l] / (g + copysign(r, g));
                        F s = F(1), c = F(1), p = F(0);
                        int i;
                        bool underflow = false;
                        // This loop is one thread's chain of dependent FP64
                        // operations, and GB300 issues FP64 at 1/64 of the
                        // FP32 rate, so each rotation uses one reciprocal
                        // square root and multiplies (no hypot, no divides).
                        // f and g stay far from overflow for M = I + S'S.
                        for (i = m - 1; i >= l; --i) {
                            F f = s * e[i], b = c * e[i];
                            const F t = fma(f, f, g * g);
                            if (t == F(0)) {
                                e[i + 1] = F(0);
                                d[i + 1] -= p;
                                e[m] = F(0);
                                underflow = true;
                                break;
                            }
                            const F ri = rsq(t);
                            r = t * ri;
                            e[i + 1] = r;
                            s = f * ri;
                            c = g * ri;
                            g = d[i + 1] - p;
                            r = (d[i] - g) * s + F(2) * c * b;
                            p = s * r;
                            d[i + 1] = g + p;
                            g = c * r - b;
                            cs[i] = c;
                            sn[i] = s;
                        }
                        ctl[1] = m - 1;          // first rotation index
                        ctl[2] = underflow ? i + 1 : l;  // last rotation index
                        if (!underflow) {
                            d[l] -= p;
                            e[l] = g;
                            e[m] = F(0);
                        }
                    }
                }
            }
            __syncthreads();
            int m = ctl[0];
            if (m == l) break;
            ++iter;
            int i_hi = ctl[1], i_lo = ctl[2];
            for (int k = tid; k < n; k += NT) {
                F* Ak = A + (size_t)k * lda;
                if (i_hi >= i_lo) {
                    F carry = Ak[i_hi + 1];
                    for (int i = i_hi; i >= i_lo; --i) {
                        F zi = Ak[i];
                        F c = cs[i], s = sn[i];
                        Ak[i + 1] = s * zi + c * carry;
                        carry = c * zi - s * carry;
                    }
                    Ak[i_lo] = carry;
                }
            }
            __syncthreads();
        }
    }
    const int rc = ctl[3];
    __syncthreads();   // every thread has its status before the caller reuses ctl
    return rc;
}

// A: n x n, row stride lda, symmetric (both triangles valid on entry).
// On return: column k of A is the eigenvector of eigenvalue d[k].
// e, cs, sn: scratch of n doubles each; ctl: 4 ints; red: NT/32 doubles.
// Returns 0 or 1 (QL did not converge).
template <int NT, typename F>
__device__ int eig_sym(F* A, int n, int lda, F* d, F* e, F* cs, F* sn, int* ctl, F* red)
{
    tred2<NT>(A, n, lda, d, e, red);
    return tql2<NT>(A, n, lda, d, e, cs, sn, ctl);
}

// The scalar part of tql2 for one point, run by one thread (batched over
// points, one thread each): implicit QL on (d, e) (element i at d[i * ds],
// e[i * ds]) with the same operations as tql2, leaving the eigenvalues in d.
// The rotations are not applied; they are logged for ql_replay: rot[] gets
// (c, s) of every rotation in order, hdr[] one (first, last) index pair per QL
// sweep (rotations i = first down to last; first < last: none).  Returns 0,
// 1 (no convergence) or 2 (the log capacity rcap / hcap was exceeded).
template <typename F>
__device__ inline int ql_chain(F* d, F* e, int n, int ds, typename Vec2<F>::type* rot, int rcap, int2* hdr, int hcap,
                               int* nh_out)
{
    int nr = 0, nh = 0;
    for (int l = 0; l < n; ++l) {
        int iter = 0;
        for (;;) {
            int mm;
            for (mm = l; mm < n - 1; ++mm) {
                const F dd = fabs(d[mm * ds]) + fabs(d[(mm + 1) * ds]);
                if (fabs(e[mm * ds]) <= Eps<F>::value * dd) break;
            }
            if (mm == l) break;
            if (iter >= 60) return 1;
            ++iter;
            if (nh >= hcap || nr + (mm - l) > rcap) return 2;
            F g = (d[(l + 1) * ds] - d[l * ds]) / (F(2) * e[l * ds]);
            F r = sqrt(fma(g, g, F(1)));
            g = d[mm * ds] - d[l * ds] + e[l * ds] / (g + copysign(r, g));
            F sv = F(1), c = F(1), p = F(0);
            int i;
            bool underflow = false;
            for (i = mm - 1; i >= l; --i) {
                const F f = sv * e[i * ds], b = c * e[i * ds];
                const F t = fma(f, f, g * g);
                if (t == F(0)) {
                    e[(i + 1) * ds] = F(0);
                    d[(i + 1) * ds] -= p;
                    e[mm * ds] = F(0);
                    underflow = true;
                    break;
                }
                const F ri = rsq(t);
                r = t * ri;
                e[(i + 1) * ds] = r;
                sv = f * ri;
                c = g * ri;
                g = d[(i + 1) * ds] - p;
                r = (d[i * ds] - g) * sv + F(2) * c * b;
                p = sv * r;
                d[(i + 1) * ds] = g + p;
                g = c * r - b;
                rot[nr].x = c;
                rot[nr].y = sv;
                ++nr;
            }
            hdr[nh++] = make_int2(mm - 1, underflow ? i + 1 : l);
            if (!underflow) {
                d[l * ds] -= p;
                e[l * ds] = g;
                e[mm * ds] = F(0);
            }
        }
    }
    *nh_out = nh;
    return 0;
}

// Apply a ql_chain log to the rows of A (n x n, row stride lda; Q of tred2),
// giving the eigenvectors in the columns as tql2 does.  Rows are
// independent, one thread each; the log is read through the read-only cache
// (every thread reads the same rotation: a broadcast).
template <int NT, typename F>
__device__ void ql_replay(F* A, int n, int lda, const typename Vec2<F>::type* __restrict__ rot,
                          const int2* __restrict__ hdr, int nh)
{
    for (int k = threadIdx.x; k < n; k += NT) {
        F* Ak = A + (size_t)k * lda;
        int r = 0;
        for (int h = 0; h < nh; ++h) {
            const int2 hl = __ldg(hdr + h);
            if (hl.x >= hl.y) {
                F carry = Ak[hl.x + 1];
                for (int i = hl.x; i >= hl.y; --i) {
                    const typename Vec2<F>::type q = __ldg(rot + r);
                    ++r;
                    const F zi = Ak[i];
                    Ak[i + 1] = q.y * zi + q.x * carry;
                    carry = q.x * zi - q.y * carry;
                }
                Ak[hl.y] = carry;
            }
        }
    }
    __syncthreads();
}

// In-place inverse of the SPD matrix A (n x n, row stride lda; the upper
// triangle is read) by the symmetric sweep operator.  Sweeping pivot k with
// D = a_kk and u = column k of the current (symmetric) matrix:
//     a_ij <- a_ij - u_i u_j / D   (i, j != k),
//     a_ik <- u_i / D              (i != k),
//     a_kk <- -1 / D,
// and after all n pivots the matrix holds -A^-1.  Every step updates the
// whole upper triangle in parallel (one FMA per element): the rows, paired
// as (i, n-1-i) so that each pair holds n+1 elements, are laid end to end
// and dealt to the threads one element each, so all threads stay busy
// instead of the serial chains of triangular solves (and every warp
// instruction of the FP64 update but the last is full).
// Without pivoting this is stable for M = I + S'S (pivots >= 1).  On return A
// holds the full symmetric A^-1.  U, V: n doubles each; piv: 2 doubles.
// Returns 0, or 1 if a pivot was not positive.
template <int NT>
__device__ int spd_inverse(double* A, int n, int lda, double* U, double* V, double* piv, int* ctl)
{
    const int tid = threadIdx.x;
    if (tid == 0) {
        ctl[3] = 0;
        double p0 = A[0];
        if (!(p0 > 0.0)) {
            ctl[3] = 1;
            p0 = 1.0;
        }
        piv[0] = 1.0 / p0;
    }
    __syncthreads();
    for (int k = 0; k < n; ++k) {
        const double inv = piv[k & 1];
        for (int i = tid; i < n; i += NT) {
            const double u = (i <= k) ? A[(size_t)i * lda + k] : A[(size_t)k * lda + i];
            U[i] = u;
            V[i] = u * inv;
        }
        __syncthreads();
        // the upper triangle as row pairs (i, n-1-i) of n+1 elements, laid
        // end to end and dealt to the threads one element each: every warp
        // instruction but the last updates 32 elements
        const int ntri = n * (n + 1) / 2, np1 = n + 1;
        for (int el = tid; el < ntri; el += NT) {
            {
                const int pr = el / np1, c = el - pr * np1;
                const int i0 = pr, i1 = n - 1 - pr;
                const int len0 = n - i0;
                int i, j;
                if (c < len0) {
                    i = i0;
                    j = i0 + c;
                } else {
                    i = i1;
                    j = i1 + (c - len0);
                }
                double* aij = A + (size_t)i * lda + j;
                double v;
                if (i == k) v = (j == k) ? -inv : V[j];
                else if (j == k) v = V[i];
                else v = fma(-U[i], V[j], *aij);
                *aij = v;
                if (i == k + 1 && j == k + 1) {
                    if (!(v > 0.0)) {
                        ctl[3] = 1;
                        v = 1.0;
                    }
                    piv[(k + 1) & 1] = 1.0 / v;
                }
            }
        }
        __syncthreads();
    }
    // -A^-1 (upper) -> A^-1 (both triangles); the negation is a sign flip
    for (int idx = tid; idx < n * n; idx += NT) {
        const int i = idx / n, j = idx - i * n;
        if (j < i) continue;
        const double v =
            __longlong_as_double(__double_as_longlong(A[(size_t)i * lda + j]) ^ (long long)0x8000000000000000ull);
        A[(size_t)i * lda + j] = v;
        if (j != i) A[(size_t)j * lda + i] = v;
    }
    __syncthreads();
    return ctl[3];
}

}  // namespace la
