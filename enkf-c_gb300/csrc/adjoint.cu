// adjoint.cu -- hand-written adjoint of the local analysis (observation
// impact): gradients of an objective J with respect to every innovation, every
// observation-error variance and the localisation radius.
//
// Forward (per strided point i, reference calc/calcs.c / transforms.c):
//   S_i = diag(lc_i) S,  s_i = diag(lc_i) s      (tapered, standardised)
//   M = I + S_i' S_i = Z diag(l) Z',  b = S_i' s_i
//   w = M^-1 b = Z diag(1/l) Z' b,     T = f(M) (ETKF l^-1/2, DEnKF (1 + 1/l)/2)
//   T_out = I + alpha (T - I)
// with S[o,e] = HA[o,e] / (sigma_o sqrt(m-1)), s[o] = d_o / (sigma_o sqrt(m-1)),
// sigma_o^2 = R_o = estd_o^2 rfactor, lc_io = sum_k wk GC(dist_io / (rho r_k)).
//
// Reverse, given wbar = dJ/dw (and optionally Tbar = dJ/dT_out):
//   lambda = M^-1 wbar
//   Mbar   = -lambda w'                                     (through w)
//          + Z (F o (Z' Gbar Z)) Z',  Gbar = alpha Tbar      (through T)
//     the second term is the Daleckii-Krein form of the Frechet derivative
//     of f(M): F_ij = (f(l_i) - f(l_j)) / (l_i - l_j), F_ii = f'(l_i),
//     evaluated in closed forms that do not cancel for close eigenvalues.  The
//     eigendecomposition is recomputed here rather than stored by the forward.
//   P = Mbar + Mbar'.  For each local observation o (untapered row u = S[o,:],
//   untapered innovation su = s[o]):
//     a = u . lambda,  c = u . w,  q = u P u'
//     dJ/dlc_io  = 2 lc a (su - c) + lc q
//     dJ/dd_o   += lc^2 a / (sigma_o sqrt(m-1))
//     dJ/dR_o   += -lc dJ/dlc_io / (2 R_o)      (S_i and s_i scale like R^-1/2)
//     dJ/drho   += dJ/dlc_io * d lc_io / d rho,  d lc/d rho = -sum_k wk x GC'(x),
//                  x = dist / r_k (the radius enters through x only; GC and
//                  GC' vanish at x = 1, so obs entering or leaving the
//                  neighbourhood contribute nothing).
// Gradients with respect to estd^2 (the variance the obs file carries) are
// dJ/dR_o * rfactor.  The kernel is a template on the arithmetic type F:
// double (FP64 throughout: the form checked against finite differences) or
// float (the production form, enkfg_calc_params.precision = mixed: the
// recomputed S'S, eigendecomposition, Daleckii-Krein products and
// per-observation passes in FP32; the taper, its derivative and the
// gradient accumulators stay FP64).
//
// The mean-update part (update.c:405-410, x_a = x_f + A w_cell, w_cell the
// stride-interpolated w) is reversed by k_adj_mean: wbar_i = sum over cells of
// the interpolation weight times g_c A_c, g_c = dJ/dx_a at cell c.
#include "calc_common.cuh"

// derivative dGC/dx of the Gaspari-Cohn function with support at x = 1
__device__ __forceinline__ double gc_deriv(double x)
{
    if (x >= 1.0 || x < 0.0) return 0.0;
    const double z = 2.0 * x, z2 = z * z, z3 = z2 * z, z4 = z3 * z;
    double fz;
    if (z < 1.0) fz = -1.25 * z4 + 2.0 * z3 + 1.875 * z2 - (10.0 / 3.0) * z;
    else fz = (5.0 / 12.0) * z4 - 2.0 * z3 + 1.875 * z2 + (10.0 / 3.0) * z - 5.0 + (2.0 / 3.0) / z2;
    return 2.0 * fz;
}

struct AdjArgs {
    CalcArgs c;
    const double* wbar;        // [npts][m]
    const double* Tbar;        // [npts][md][m] or null
    const double* sig;         // [nsorted] sigma_o sqrt(m-1) in sorted order
    const double* R;           // [nsorted] R_o in sorted order
    const int* sid;            // sorted position -> obs id
    double* dinn;              // [nobs]
    double* dvar;              // [nobs] (dJ/dR_o)
    double* drho;              // [1]
};

template <typename F>
struct AdjProc {
    const AdjArgs& A;
    const PointScratch& s;
    F* tile;                   // [KC_MAX][MP] untapered S rows of the chunk
    const F* lam;              // M^-1 wbar
    const F* w;                // w
    const F* P;                // Mbar + Mbar' (null: no T term)
    int lda;
    int mp;
    double qx, qy, qz;
    double rho_acc;
    __device__ AdjProc(const AdjArgs& A_, const PointScratch& s_, F* tile_, const F* lam_, const F* w_, const F* P_,
                       int lda_, int mp_, double qx_, double qy_, double qz_)
        : A(A_), s(s_), tile(tile_), lam(lam_), w(w_), P(P_), lda(lda_), mp(mp_), qx(qx_), qy(qy_), qz(qz_),
          rho_acc(0.0) {}
    __device__ void chunk(int nc, int t)
    {
        const CalcArgs& a = A.c;
        const int tid = threadIdx.x, m = a.m, lane = tid & 31, wid = tid >> 5;
        for (int i = tid; i < nc * mp; i += CALC_NT) {
            int o = i / mp, e = i - o * mp;
            tile[i] = (e < m) ? (F)a.St[(size_t)s.lid[o] * a.mpad + e] : F(0);
        }
        __syncthreads();
        const TypeIndex& ti = a.types[t];
        // one warp per observation of the chunk
        for (int o = wid; o < nc; o += CALC_NT / 32) {
            const F* u = tile + (size_t)o * mp;
            F av = F(0), cv = F(0), qv = F(0);
            for (int e = lane; e < m; e += 32) {
                av = fma(u[e], lam[e], av);
                cv = fma(u[e], w[e], cv);
                if (P != nullptr) {
                    F pu = F(0);
                    for (int k = 0; k < m; ++k) pu = fma(P[(size_t)e * lda + k], u[k], pu);
                    qv = fma(u[e], pu, qv);
                }
            }
            for (int d = 16; d > 0; d >>= 1) {
                av += __shfl_xor_sync(0xffffffffu, av, d);
                cv += __shfl_xor_sync(0xffffffffu, cv, d);
                qv += __shfl_xor_sync(0xffffffffu, qv, d);
            }
            if (lane == 0) {
                const int p = s.lid[o];
                const double lc = s.llc[o];
                const double su = a.ss[p];
                const double dlc = 2.0 * lc * (double)av * (su - (double)cv) + lc * (double)qv;
                const int id = A.sid[p];
                atomicAdd(&A.dinn[id], lc * lc * (double)av / A.sig[p]);
                atomicAdd(&A.dvar[id], -lc * dlc / (2.0 * A.R[p]));
                // d lc / d rho
                const double d2 = a.ndim == 2 ? exact::dist2(a.sx[p], a.sy[p], qx, qy)
                                              : exact::dist3(a.sx[p], a.sy[p], a.sz[p], qx, qy, qz);
                const double dist = sqrt(d2);
                double dl = 0.0;
                for (int k = 0; k < ti.nlocrad; ++k) {
                    const double x = dist / ti.locrad[k];
                    dl -= ti.locweight[k] * x * gc_deriv(x);
                }
                rho_acc += dlc * dl;
            }
        }
        __syncthreads();
    }
    __device__ void type_end(int) {}
};

// products rounded to nearest in F: FP64 with the forward kernel's explicit
// rounding, FP32 plainly
__device__ __forceinline__ double adj_mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float adj_mul(float a, float b) { return __fmul_rn(a, b); }

template <int R, typename F>
struct GramProcAdj {
    // S'S and S's in F (FP64: the same arithmetic as the FP64 forward kernel)
    const CalcArgs& a;
    const PointScratch& s;
    F* tile;
    F* sloc;
    F acc[R][R];
    F bacc;
    __device__ GramProcAdj(const CalcArgs& a_, const PointScratch& s_, F* tile_, F* sloc_)
        : a(a_), s(s_), tile(tile_), sloc(sloc_), bacc(F(0))
    {
#pragma unroll
        for (int i = 0; i < R; ++i)
#pragma unroll
            for (int j = 0; j < R; ++j) acc[i][j] = F(0);
    }
    __device__ void chunk(int nc, int)
    {
        constexpr int MP = 16 * R;
        const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4, m = a.m;
        for (int i = tid; i < nc * MP; i += CALC_NT) {
            int o = i / MP, e = i - o * MP;
            tile[i] = (e < m) ? adj_mul((F)a.St[(size_t)s.lid[o] * a.mpad + e], (F)s.llc[o]) : F(0);
        }
        if (tid < nc) sloc[tid] = adj_mul((F)a.ss[s.lid[tid]], (F)s.llc[tid]);
        __syncthreads();
        if (tx >= ty)
            for (int o = 0; o < nc; ++o) {
                F av[R], bv[R];
#pragma unroll
                for (int i = 0; i < R; ++i) av[i] = tile[o * MP + ty * R + i];
#pragma unroll
                for (int j = 0; j < R; ++j) bv[j] = tile[o * MP + tx * R + j];
#pragma unroll
                for (int i = 0; i < R; ++i)
#pragma unroll
                    for (int j = 0; j < R; ++j) acc[i][j] = fma(av[i], bv[j], acc[i][j]);
            }
        if (tid < m)
            for (int o = 0; o < nc; ++o) bacc = fma(tile[o * MP + tid], sloc[o], bacc);
        __syncthreads();
    }
    __device__ void type_end(int) {}
};

template <int R, typename F>
__global__ void __launch_bounds__(CALC_NT) k_adjoint(AdjArgs A)
{
    constexpr int MP = 16 * R, LDA = MP + 1;
    constexpr size_t FS = sizeof(F);
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const CalcArgs& a = A.c;
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    const int m = a.m, md = a.md;
    unsigned char* sp = smem_raw;
    double* llc = (double*)sp;    sp += (size_t)LIST_EXTRA * 8;
    F* tile = (F*)sp;             sp += (size_t)KC_MAX * MP * FS;
    F* sloc = (F*)sp;             sp += (size_t)KC_MAX * FS;
    F* Z = (F*)sp;                sp += (size_t)MP * LDA * FS;    // M, then its eigenvectors
    F* W = (F*)sp;                sp += (size_t)MP * LDA * FS;    // work (Z'GZ, then P)
    F* b = (F*)sp;                sp += MP * FS;
    F* d = (F*)sp;                sp += MP * FS;
    F* e = (F*)sp;                sp += MP * FS;
    F* cs = (F*)sp;               sp += MP * FS;
    F* sn = (F*)sp;               sp += MP * FS;
    F* w = (F*)sp;                sp += MP * FS;
    F* lam = (F*)sp;              sp += MP * FS;
    F* fred = (F*)sp;             sp += MP * FS;                  // (CALC_NT / 32 <= MP) block sums in F
    sp = (unsigned char*)(((uintptr_t)sp + 7) & ~(uintptr_t)7);
    double* tss = (double*)sp;    sp += ENKFG_MAXTYPES * 8;
    double* tpd = (double*)sp;    sp += ENKFG_MAXTYPES * 8;
    double* red = (double*)sp;    sp += (CALC_NT / 32) * 8;
    int* lid = (int*)sp;          sp += LIST_EXTRA * 4;
    int* tcount = (int*)sp;       sp += ENKFG_MAXTYPES * 4;
    int* ictl = (int*)sp;
    const PointScratch s{ lid, llc, ictl, tcount, tss, tpd, red };

    const int pt = blockIdx.x;
    const double qx = a.qx[pt], qy = a.qy[pt], qz = a.ndim == 3 ? a.qz[pt] : 0.0;
    const double* wb = A.wbar + (size_t)pt * m;
    const double* Tb = A.Tbar ? A.Tbar + (size_t)pt * md * m : nullptr;
    // skip points with no incoming gradient
    {
        double nz = 0.0;
        for (int i = tid; i < m; i += CALC_NT) nz += fabs(wb[i]);
        if (Tb)
            for (int i = tid; i < md * m; i += CALC_NT) nz += fabs(Tb[i]);
        nz = la::block_sum<CALC_NT>(nz, red);
        if (nz == 0.0) return;
    }
    // 1. forward recomputation: M, b, eigendecomposition, w
    GramProcAdj<R, F> gp(a, s, tile, sloc);
    const int p = enumerate_obs<0>(a, pt, a.kc, qx, qy, qz, s, gp, true);
    if (p == 0) return;
    if (tx >= ty)
#pragma unroll
        for (int i = 0; i < R; ++i)
#pragma unroll
            for (int j = 0; j < R; ++j) {
                int r = ty * R + i, c = tx * R + j;
                if (r < m && c < m) {
                    Z[r * LDA + c] = gp.acc[i][j];
                    Z[c * LDA + r] = gp.acc[i][j];
                }
            }
    if (tid < m) b[tid] = gp.bacc;
    __syncthreads();
    if (tid < m) Z[tid * LDA + tid] += F(1);
    __syncthreads();
    int rc = la::eig_sym<CALC_NT>(Z, m, LDA, d, e, cs, sn, ictl + 16, fred);
    if (rc != 0) {
        if (tid == 0) a.status[pt] = rc;
        return;
    }
    // w = Z diag(1/l) Z' b ; lam = Z diag(1/l) Z' wbar
    if (tid < m) {
        F cb = F(0), cw = F(0);
        for (int q = 0; q < m; ++q) {
            cb = fma(Z[q * LDA + tid], b[q], cb);
            cw = fma(Z[q * LDA + tid], (F)wb[q], cw);
        }
        cs[tid] = cb / d[tid];
        sn[tid] = cw / d[tid];
    }
    __syncthreads();
    if (tid < m) {
        F x = F(0), y = F(0);
        for (int k = 0; k < m; ++k) {
            x = fma(Z[tid * LDA + k], cs[k], x);
            y = fma(Z[tid * LDA + k], sn[k], y);
        }
        w[tid] = x;
        lam[tid] = y;
    }
    __syncthreads();
    // 2. T term (Daleckii-Krein): P = Mbar_T + Mbar_T', Mbar_T = Z (F o Z' G Z) Z'
    const F* Pp = nullptr;
    if (Tb != nullptr && a.mode != ENKFG_MODE_ENOI) {
        const bool etkf = (a.scheme == ENKFG_SCHEME_ETKF);
        // W = G Z, G = alpha Tbar on rows e1 < md (T[e1][e2] is column e1 of the
        // reference's T; f(M) is symmetric, so G can be taken row-wise)
        for (int idx = tid; idx < m * m; idx += CALC_NT) {
            int r = idx / m, c = idx - r * m;
            F v = F(0);
            if (r < md)
                for (int k = 0; k < m; ++k) v = fma((F)(a.alpha * Tb[(size_t)r * m + k]), Z[k * LDA + c], v);
            W[r * LDA + c] = v;
        }
        __syncthreads();
        // The products below run in place in W, in batches of at most KC_MAX
        // columns (or rows) staged through the tile region (KC_MAX x MP):
        // column c of Z' W and of Z X depends on column c of W only, row r of
        // Y Z' on row r of Y only.
        // W <- F o (Z' W): F the divided differences of f on the eigenvalues
        for (int c0 = 0; c0 < m; c0 += KC_MAX) {
            const int nb = (m - c0 < KC_MAX) ? m - c0 : KC_MAX;
            for (int idx = tid; idx < m * nb; idx += CALC_NT) {
                const int r = idx / nb, cc = idx - r * nb, c = c0 + cc;
                F v = F(0);
                for (int k = 0; k < m; ++k) v = fma(Z[k * LDA + r], W[k * LDA + c], v);
                // divided differences in closed form (no cancellation when
                // l_i ~ l_j, exact limit f'(l) on the diagonal):
                //   ETKF  f = l^-1/2:        F = -1 / (sqrt(li) sqrt(lj) (sqrt(li) + sqrt(lj)))
                //   DEnKF f = (1 + 1/l) / 2: F = -1 / (2 li lj)
                const F li = d[r], lj = d[c];
                F dd;
                if (etkf) {
                    const F qi = sqrt(li), qj = sqrt(lj);
                    dd = F(-1) / (qi * qj * (qi + qj));
                } else {
                    dd = F(-0.5) / (li * lj);
                }
                tile[(size_t)cc * MP + r] = dd * v;
            }
            __syncthreads();
            for (int idx = tid; idx < m * nb; idx += CALC_NT) {
                const int r = idx / nb, cc = idx - r * nb;
                W[r * LDA + c0 + cc] = tile[(size_t)cc * MP + r];
            }
            __syncthreads();
        }
        // W <- Z W
        for (int c0 = 0; c0 < m; c0 += KC_MAX) {
            const int nb = (m - c0 < KC_MAX) ? m - c0 : KC_MAX;
            for (int idx = tid; idx < m * nb; idx += CALC_NT) {
                const int r = idx / nb, cc = idx - r * nb, c = c0 + cc;
                F v = F(0);
                for (int k = 0; k < m; ++k) v = fma(Z[r * LDA + k], W[k * LDA + c], v);
                tile[(size_t)cc * MP + r] = v;
            }
            __syncthreads();
            for (int idx = tid; idx < m * nb; idx += CALC_NT) {
                const int r = idx / nb, cc = idx - r * nb;
                W[r * LDA + c0 + cc] = tile[(size_t)cc * MP + r];
            }
            __syncthreads();
        }
        // W <- W Z' = Mbar_T (row batches)
        for (int r0 = 0; r0 < m; r0 += KC_MAX) {
            const int nb = (m - r0 < KC_MAX) ? m - r0 : KC_MAX;
            for (int idx = tid; idx < nb * m; idx += CALC_NT) {
                const int rr = idx / m, c = idx - rr * m, r = r0 + rr;
                F v = F(0);
                for (int k = 0; k < m; ++k) v = fma(W[r * LDA + k], Z[c * LDA + k], v);
                tile[(size_t)rr * MP + c] = v;
            }
            __syncthreads();
            for (int idx = tid; idx < nb * m; idx += CALC_NT) {
                const int rr = idx / m, c = idx - rr * m;
                W[(r0 + rr) * LDA + c] = tile[(size_t)rr * MP + c];
            }
            __syncthreads();
        }
        // P = Mbar_T + Mbar_T' in place (one thread per unordered pair)
        for (int idx = tid; idx < m * m; idx += CALC_NT) {
            const int r = idx / m, c = idx - r * m;
            if (c < r) continue;
            const F v = W[r * LDA + c] + W[c * LDA + r];
            W[r * LDA + c] = v;
            W[c * LDA + r] = v;
        }
        __syncthreads();
        Pp = W;
    }
    // 3. per-observation sensitivities (second pass over the local obs; the
    //    chunks are staged in the tile region, P stays in W)
    AdjProc<F> ap(A, s, tile, lam, w, Pp, LDA, MP, qx, qy, qz);
    enumerate_obs<0>(a, pt, a.kc, qx, qy, qz, s, ap, false);
    double rs = la::block_sum<CALC_NT>(ap.rho_acc, red);
    if (tid == 0 && rs != 0.0) atomicAdd(A.drho, rs);
}

// adjoint of the mean update and of the stride interpolation: for every
// cell with g_c = dJ/dx_a != 0, wbar at the (up to four) strided points it
// interpolates from += weight * g_c * A_c (A_c the forecast anomalies of the
// cell, update.c:381-392)
__global__ void k_adj_mean(int m, int md, int mni, int mnj, int ni, int nj, int stride, int periodic_i,
                           const float* __restrict__ field, const double* __restrict__ g, double* __restrict__ wbar)
{
    const long long cell = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (cell >= (long long)mni * mnj) return;
    const double gc = g[cell];
    if (gc == 0.0) return;
    const int j = (int)(cell / mni), i = (int)(cell - (long long)j * mni);
    const size_t plane = (size_t)mni * mnj;
    double sm = 0.0;
    for (int e = lane; e < md; e += 32) sm += (double)field[(size_t)e * plane + cell];
    for (int d = 16; d > 0; d >>= 1) sm += __shfl_xor_sync(0xffffffffu, sm, d);
    const double mean = sm / (double)md;
    // corner weights (the forward uses these float weights, update.c:220-265)
    const int jj = j / stride, stepj = j % stride, ii = i / stride, stepi = i % stride;
    int rows[2] = { jj, jj };
    double wr[2] = { 1.0, 0.0 };
    if (stride > 1 && stepj > 0) {
        float w2 = __fdiv_rn((float)stepj, (float)stride), w1 = __fsub_rn(1.0f, w2);
        rows[1] = (jj < nj - 1) ? jj + 1 : jj;
        wr[0] = w1;
        wr[1] = w2;
    }
    int cols[2] = { ii, ii };
    double wc[2] = { 1.0, 0.0 };
    if (stride > 1 && stepi > 0) {
        float u2 = __fdiv_rn((float)stepi, (float)stride), u1 = __fsub_rn(1.0f, u2);
        cols[1] = (ii < ni - 1) ? ii + 1 : (periodic_i ? (ii + 1) % ni : ii);
        wc[0] = u1;
        wc[1] = u2;
    }
    for (int e = lane; e < m; e += 32) {
        const double an = (double)(float)((double)field[(size_t)e * plane + cell] - mean);
        const double v = gc * an;
        for (int r = 0; r < 2; ++r)
            for (int c = 0; c < 2; ++c) {
                const double wt = wr[r] * wc[c];
                if (wt != 0.0) atomicAdd(&wbar[((size_t)rows[r] * ni + cols[c]) * m + e], wt * v);
            }
    }
}

__global__ void k_adj_sorted(int nsorted, const int* __restrict__ sid, const float* __restrict__ estd,
                             const short* __restrict__ type, const double* __restrict__ sqrt_rfac, double mult,
                             double* __restrict__ sig, double* __restrict__ R)
{
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nsorted) return;
    int o = sid[p];
    double sg = (double)estd[o] * sqrt_rfac[type[o]];
    sig[p] = sg * mult;
    R[p] = sg * sg;
}

template <int R, typename F>
static enkfg_status launch_adj(enkfg_ctx* ctx, AdjArgs& A, cudaStream_t st)
{
    constexpr int MP = 16 * R, LDA = MP + 1;
    constexpr size_t FS = sizeof(F);
    size_t smem = LIST_EXTRA * 8 + (size_t)KC_MAX * MP * FS + KC_MAX * FS + 2 * (size_t)MP * LDA * FS +
                  8 * MP * FS + 8 + 2 * ENKFG_MAXTYPES * 8 + (CALC_NT / 32) * 8 + LIST_EXTRA * 4 +
                  ENKFG_MAXTYPES * 4 + 256;
    if (smem > 227 * 1024) {
        set_err(ctx, "adjoint: nmem = %d needs too much shared memory", A.c.m);
        return ENKFG_EUNSUPPORTED;
    }
    CK(cudaFuncSetAttribute(k_adjoint<R, F>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_adjoint<R, F><<<A.c.npts, CALC_NT, smem, st>>>(A);
    CKL();
    return ENKFG_OK;
}

enkfg_status run_adjoint(enkfg_ctx* ctx, const enkfg_calc_params* p, const double* d_wbar, const double* d_Tbar,
                         double* d_dinn, double* d_dvar, double* d_drho, cudaStream_t st)
{
    enkfg_status s;
    const int m = ctx->nmem;
    if (m > 96) {
        set_err(ctx, "the adjoint supports nmem <= 96 (got %d)", m);
        return ENKFG_EUNSUPPORTED;
    }
    if ((s = prepare_search(ctx, st))) return s;
    if (!ctx->gather_valid && (s = build_gather(ctx, st))) return s;
    const int npts = ctx->nj * ctx->ni;
    if ((s = ensure(ctx, &ctx->d_status_pt, &ctx->status_cap, (size_t)npts))) return s;
    CK(cudaMemsetAsync(ctx->d_status_pt, 0, (size_t)npts * sizeof(int), st));
    double *sig, *R;
    CK(cudaMalloc(&sig, (size_t)(ctx->nsorted > 0 ? ctx->nsorted : 1) * sizeof(double)));
    CK(cudaMalloc(&R, (size_t)(ctx->nsorted > 0 ? ctx->nsorted : 1) * sizeof(double)));
    if (ctx->nsorted > 0) {
        k_adj_sorted<<<div_up(ctx->nsorted, 256), 256, 0, st>>>(ctx->nsorted, ctx->d_sid, ctx->d_estd, ctx->d_type,
                                                               ctx->d_rfac_sqrt, sqrt((double)m - 1), sig, R);
        CKL();
    }
    AdjArgs A;
    memset(&A, 0, sizeof(A));
    CalcArgs& a = A.c;
    a.npts = npts;
    a.nitems = npts;
    a.ntypes = ctx->ntypes;
    a.ndim = ctx->geographic ? 3 : 2;
    a.m = m;
    a.md = ctx->nmem_dyn;
    a.mode = p->mode;
    a.scheme = p->scheme;
    a.alpha = p->alpha;
    a.wait_ns = ctx->wait_ns;
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
    a.sid = ctx->d_sid;
    a.cut = any_nlobsmax(ctx) ? ctx->d_cut : nullptr;
    a.status = ctx->d_status_pt;
    A.wbar = d_wbar;
    A.Tbar = d_Tbar;
    A.sig = sig;
    A.R = R;
    A.sid = ctx->d_sid;
    A.dinn = d_dinn;
    A.dvar = d_dvar;
    A.drho = d_drho;
    const bool f32 = (p->precision == ENKFG_PREC_MIXED);
    if (m <= 32) s = f32 ? launch_adj<2, float>(ctx, A, st) : launch_adj<2, double>(ctx, A, st);
    else if (m <= 48) s = f32 ? launch_adj<3, float>(ctx, A, st) : launch_adj<3, double>(ctx, A, st);
    else if (m <= 64) s = f32 ? launch_adj<4, float>(ctx, A, st) : launch_adj<4, double>(ctx, A, st);
    else s = f32 ? launch_adj<6, float>(ctx, A, st) : launch_adj<6, double>(ctx, A, st);
    cudaError_t e = cudaStreamSynchronize(st);
    cudaFree(sig);
    cudaFree(R);
    if (s) return s;
    if (e != cudaSuccess) return cuda_fail(ctx, e, "adjoint", __LINE__);
    return ENKFG_OK;
}

enkfg_status run_adj_mean(enkfg_ctx* ctx, int m, int md, const float* d_field, const double* d_g, double* d_wbar,
                          cudaStream_t st)
{
    const long long cells = (long long)ctx->mni * ctx->mnj;
    k_adj_mean<<<div_up(cells, 8), 256, 0, st>>>(m, md, ctx->mni, ctx->mnj, ctx->ni, ctx->nj, ctx->stride,
                                                 ctx->periodic_i, d_field, d_g, d_wbar);
    CKL();
    return ENKFG_OK;
}
