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
//   chol_inverse  M^-1 of an SPD matrix by Cholesky factorisation and two
//                 triangular solves against the identity.
//
// These replace LAPACK dgesvd (reference calc/calcs.c:338) and dpotrf/dpotri
// (calcs.c:103-132).  Both are backward stable, so the results agree with
// LAPACK's to a few units of rounding times the condition of M = I + S'S.
#pragma once

namespace la {

template <int NT>
__device__ __forceinline__ double block_sum(double v, double* red)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) red[wid] = v;
    __syncthreads();
    double s = 0.0;
#pragma unroll
    for (int w = 0; w < NT / 32; ++w) s += red[w];
    return s;
}

// A: n x n, row stride lda, symmetric (both triangles valid on entry).
// On return: column k of A is the eigenvector of eigenvalue d[k].
// e, cs, sn: scratch of n doubles each; ctl: 4 ints; red: NT/32 doubles.
// Returns 0 or 1 (QL did not converge).
template <int NT>
__device__ int eig_sym(double* A, int n, int lda, double* d, double* e, double* cs, double* sn, int* ctl,
                       double* red)
{
    const int tid = threadIdx.x;
    // ---- Householder reduction (rows n-1 .. 1) ----
    for (int i = n - 1; i >= 1; --i) {
        int l = i - 1;
        double* Ai = A + (size_t)i * lda;
        double h = 0.0;
        if (l > 0) {
            double part = 0.0;
            for (int k = tid; k <= l; k += NT) part += fabs(Ai[k]);
            double scale = block_sum<NT>(part, red);
            if (scale == 0.0) {
                if (tid == 0) e[i] = Ai[l];
                __syncthreads();
            } else {
                part = 0.0;
                for (int k = tid; k <= l; k += NT) {
                    double v = Ai[k] / scale;
                    Ai[k] = v;
                    part += v * v;
                }
                h = block_sum<NT>(part, red);
                double f = Ai[l];
                double g = (f >= 0.0) ? -sqrt(h) : sqrt(h);
                h -= f * g;
                __syncthreads();
                if (tid == 0) {
                    e[i] = scale * g;
                    Ai[l] = f - g;
                }
                __syncthreads();
                // p = A u / h (into e[0..l]); column i keeps u / h
                for (int j = tid; j <= l; j += NT) {
                    double g2 = 0.0;
                    const double* Aj = A + (size_t)j * lda;
                    for (int k = 0; k <= j; ++k) g2 += Aj[k] * Ai[k];
                    for (int k = j + 1; k <= l; ++k) g2 += A[(size_t)k * lda + j] * Ai[k];
                    e[j] = g2 / h;
                }
                __syncthreads();
                for (int j = tid; j <= l; j += NT) A[(size_t)j * lda + i] = Ai[j] / h;
                part = 0.0;
                for (int j = tid; j <= l; j += NT) part += e[j] * Ai[j];
                double ff = block_sum<NT>(part, red);
                double hh = ff / (h + h);
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
        d[0] = 0.0;
        e[0] = 0.0;
    }
    __syncthreads();
    // ---- accumulate the transformations ----
    for (int i = 0; i < n; ++i) {
        int l = i - 1;
        double* Ai = A + (size_t)i * lda;
        if (d[i] != 0.0) {
            for (int j = tid; j <= l; j += NT) {
                double g = 0.0;
                for (int k = 0; k <= l; ++k) g += Ai[k] * A[(size_t)k * lda + j];
                for (int k = 0; k <= l; ++k) A[(size_t)k * lda + j] -= g * A[(size_t)k * lda + i];
            }
        }
        __syncthreads();
        if (tid == 0) d[i] = Ai[i];
        for (int j = tid; j <= l; j += NT) {
            A[(size_t)j * lda + i] = 0.0;
            Ai[j] = 0.0;
        }
        if (tid == 0) Ai[i] = 1.0;
        __syncthreads();
    }
    // ---- implicit QL on (d, e) with rotations applied to the rows of A ----
    if (tid == 0) {
        for (int i = 1; i < n; ++i) e[i - 1] = e[i];
        e[n - 1] = 0.0;
        ctl[3] = 0;
    }
    __syncthreads();
    for (int l = 0; l < n; ++l) {
        int iter = 0;
        for (;;) {
            if (tid == 0) {
                int m;
                for (m = l; m < n - 1; ++m) {
                    double dd = fabs(d[m]) + fabs(d[m + 1]);
                    if (fabs(e[m]) <= 2.220446049250313e-16 * dd) break;
                }
                ctl[0] = m;
                if (m != l) {
                    if (iter >= 60) {
                        ctl[0] = l;
                        ctl[3] = 1;
                    } else {
                        double g = (d[l + 1] - d[l]) / (2.0 * e[l]);
                        double r = hypot(g, 1.0);
                        g = d[m] - d[l] + e[l] / (g + copysign(r, g));
                        double s = 1.0, c = 1.0, p = 0.0;
                        int i;
                        bool underflow = false;
                        for (i = m - 1; i >= l; --i) {
                            double f = s * e[i], b = c * e[i];
                            r = hypot(f, g);
                            e[i + 1] = r;
                            if (r == 0.0) {
                                d[i + 1] -= p;
                                e[m] = 0.0;
                                underflow = true;
                                break;
                            }
                            s = f / r;
                            c = g / r;
                            g = d[i + 1] - p;
                            r = (d[i] - g) * s + 2.0 * c * b;
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
                            e[m] = 0.0;
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
                double* Ak = A + (size_t)k * lda;
                if (i_hi >= i_lo) {
                    double carry = Ak[i_hi + 1];
                    for (int i = i_hi; i >= i_lo; --i) {
                        double zi = Ak[i];
                        double c = cs[i], s = sn[i];
                        Ak[i + 1] = s * zi + c * carry;
                        carry = c * zi - s * carry;
                    }
                    Ak[i_lo] = carry;
                }
            }
            __syncthreads();
        }
    }
    return ctl[3];
}

// M^-1 of the SPD matrix A (n x n, stride lda) into X (same shape); A is
// overwritten by its Cholesky factor.  Returns 0, or 1 if a pivot is not
// positive.
template <int NT>
__device__ int chol_inverse(double* A, double* X, int n, int lda, int* ctl)
{
    const int tid = threadIdx.x;
    if (tid == 0) ctl[3] = 0;
    for (int k = 0; k < n; ++k) {
        if (tid == 0) {
            double a = A[(size_t)k * lda + k];
            if (!(a > 0.0)) {
                ctl[3] = 1;
                a = 1.0;
            }
            A[(size_t)k * lda + k] = sqrt(a);
        }
        __syncthreads();
        double dk = A[(size_t)k * lda + k];
        for (int i = k + 1 + tid; i < n; i += NT) A[(size_t)i * lda + k] /= dk;
        __syncthreads();
        int w = n - k - 1;
        int tri = w * (w + 1) / 2;
        for (int idx = tid; idx < tri; idx += NT) {
            int a = (int)((sqrtf(8.0f * (float)idx + 1.0f) - 1.0f) * 0.5f);
            while ((a + 1) * (a + 2) / 2 <= idx) ++a;
            while (a * (a + 1) / 2 > idx) --a;
            int b = idx - a * (a + 1) / 2;
            int i = k + 1 + a, j = k + 1 + b;
            A[(size_t)i * lda + j] -= A[(size_t)i * lda + k] * A[(size_t)j * lda + k];
        }
        __syncthreads();
    }
    // forward: L Y = I (column-parallel), Y in X
    for (int i = 0; i < n; ++i) {
        const double* Li = A + (size_t)i * lda;
        double inv = 1.0 / Li[i];
        for (int j = tid; j < n; j += NT) {
            double s = (i == j) ? 1.0 : 0.0;
            for (int k = j; k < i; ++k) s -= Li[k] * X[(size_t)k * lda + j];
            X[(size_t)i * lda + j] = (j <= i) ? s * inv : 0.0;
        }
        __syncthreads();
    }
    // backward: L^T X = Y
    for (int i = n - 1; i >= 0; --i) {
        double inv = 1.0 / A[(size_t)i * lda + i];
        for (int j = tid; j < n; j += NT) {
            double s = X[(size_t)i * lda + j];
            for (int k = i + 1; k < n; ++k) s -= A[(size_t)k * lda + i] * X[(size_t)k * lda + j];
            X[(size_t)i * lda + j] = s * inv;
        }
        __syncthreads();
    }
    return ctl[3];
}

}  // namespace la
