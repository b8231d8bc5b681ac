// index.cu -- device spatial index of the observations and the local
// observation search (obs_findlocal, reference common/observations.c:
// 1837-1927; kd-tree range search common/kdtree.c:516-574).
//
// The reference walks one kd-tree per observation type for every local
// analysis.  Here the observations of each type are bucketed on a uniform
// cell grid (cell edge >= the type's largest radius), buckets numbered in
// Morton order, so the observations within range of a point are found by
// scanning the 3x3 (3x3x3 on the sphere) cells around it.  Membership uses
// the reference's predicate bit for bit: distsq = sum of squared coordinate
// differences in FP64, accumulated in axis order, compared `<= r*r`; all of
// it with round-to-nearest intrinsics so that no multiply-add is fused.
#include "internal.cuh"
#include "exact.cuh"

// ---------------------------------------------------------------------------
// Morton codes
// ---------------------------------------------------------------------------
__host__ __device__ static inline unsigned int spread2(unsigned int v)
{
    v &= 0x0000ffffu;
    v = (v | (v << 8)) & 0x00ff00ffu;
    v = (v | (v << 4)) & 0x0f0f0f0fu;
    v = (v | (v << 2)) & 0x33333333u;
    v = (v | (v << 1)) & 0x55555555u;
    return v;
}

__host__ __device__ static inline unsigned int spread3(unsigned int v)
{
    v &= 0x000003ffu;
    v = (v | (v << 16)) & 0x030000ffu;
    v = (v | (v << 8)) & 0x0300f00fu;
    v = (v | (v << 4)) & 0x030c30c3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

__device__ __forceinline__ long long bucket_of(const TypeIndex& t, int ndim, int cx, int cy, int cz)
{
    unsigned int code = (ndim == 2) ? (spread2(cx) | (spread2(cy) << 1))
                                    : (spread3(cx) | (spread3(cy) << 1) | (spread3(cz) << 2));
    return t.bucket_base + (long long)code;
}

__device__ __forceinline__ int cell_coord(double v, double v0, double inv_cell)
{
    return (int)floor((v - v0) * inv_cell);
}

// ---------------------------------------------------------------------------
// bounding boxes per type (order-preserving integer encoding of doubles)
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned long long dkey(double d)
{
    long long b = __double_as_longlong(d);
    return b >= 0 ? ((unsigned long long)b ^ 0x8000000000000000ull) : ~(unsigned long long)b;
}

static double dkey_inv(unsigned long long k)
{
    long long b = (k & 0x8000000000000000ull) ? (long long)(k ^ 0x8000000000000000ull) : (long long)~k;
    double d;
    memcpy(&d, &b, 8);
    return d;
}

// Per type: the bounding box of the valid observations as ordered keys
// (box[t*6 + 2a] min, box[t*6 + 2a + 1] max of axis a) and their number
// (box[ntypes*6 + t]).  A thread keeps the running bounds and count of a run
// of observations of one type (a grid-stride sweep) and flushes them to the
// block's shared copy when the type changes; each block then merges into the
// global box once per entry.
#define BBOX_T 256
__global__ void __launch_bounds__(BBOX_T) k_bbox(int nobs, int ndim, int ntypes, const double* __restrict__ ox,
                                                 const double* __restrict__ oy, const double* __restrict__ oz,
                                                 const short* __restrict__ type, const short* __restrict__ status,
                                                 unsigned long long* __restrict__ box)
{
    __shared__ unsigned long long sb[ENKFG_MAXTYPES * 6];
    __shared__ unsigned long long sn[ENKFG_MAXTYPES];
    for (int i = threadIdx.x; i < ntypes * 6; i += BBOX_T) sb[i] = (i & 1) ? 0ull : ~0ull;
    for (int i = threadIdx.x; i < ntypes; i += BBOX_T) sn[i] = 0ull;
    __syncthreads();
    int cur = -1;
    unsigned long long cnt = 0;
    unsigned long long lo[3] = { ~0ull, ~0ull, ~0ull }, hi[3] = { 0ull, 0ull, 0ull };
    auto flush = [&]() {
        if (cur < 0) return;
        for (int a = 0; a < ndim; ++a) {
            atomicMin(&sb[cur * 6 + 2 * a], lo[a]);
            atomicMax(&sb[cur * 6 + 2 * a + 1], hi[a]);
            lo[a] = ~0ull;
            hi[a] = 0ull;
        }
        atomicAdd(&sn[cur], cnt);
        cnt = 0;
    };
    for (int o = blockIdx.x * BBOX_T + threadIdx.x; o < nobs; o += gridDim.x * BBOX_T) {
        if (status[o] != 0) continue;
        const int t = type[o];
        if (t != cur) {
            flush();
            cur = t;
        }
        ++cnt;
        const double v[3] = { ox[o], oy[o], ndim == 3 ? oz[o] : 0.0 };
        for (int a = 0; a < ndim; ++a) {
            const unsigned long long k = dkey(v[a]);
            lo[a] = k < lo[a] ? k : lo[a];
            hi[a] = k > hi[a] ? k : hi[a];
        }
    }
    flush();
    __syncthreads();
    for (int i = threadIdx.x; i < ntypes * 6; i += BBOX_T) {
        if (i & 1) {
            if (sb[i] != 0ull) atomicMax(&box[i], sb[i]);
        } else if (sb[i] != ~0ull) {
            atomicMin(&box[i], sb[i]);
        }
    }
    for (int i = threadIdx.x; i < ntypes; i += BBOX_T)
        if (sn[i] != 0ull) atomicAdd(&box[ntypes * 6 + i], sn[i]);
}

__global__ void k_keys(int nobs, int ndim, const double* __restrict__ ox, const double* __restrict__ oy,
                       const double* __restrict__ oz, const short* __restrict__ type,
                       const short* __restrict__ status, const TypeIndex* __restrict__ types,
                       int* __restrict__ key, int* __restrict__ bcount)
{
    int o = blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= nobs) return;
    if (status[o] != 0) {
        key[o] = -1;
        return;
    }
    const TypeIndex& t = types[type[o]];
    int cx = min(max(cell_coord(ox[o], t.x0, t.inv_cell), 0), t.ncx - 1);
    int cy = min(max(cell_coord(oy[o], t.y0, t.inv_cell), 0), t.ncy - 1);
    int cz = 0;
    if (ndim == 3) cz = min(max(cell_coord(oz[o], t.z0, t.inv_cell), 0), t.ncz - 1);
    long long b = bucket_of(t, ndim, cx, cy, cz);
    key[o] = (int)b;
    atomicAdd(&bcount[b], 1);
}

__global__ void k_scatter(int nobs, const int* __restrict__ key, const long long* __restrict__ bstart,
                          int* __restrict__ bfill, int* __restrict__ sid)
{
    int o = blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= nobs) return;
    int b = key[o];
    if (b < 0) return;
    long long pos = bstart[b] + atomicAdd(&bfill[b], 1);
    sid[pos] = o;
}

// sort the ids inside each bucket (deterministic order): bitonic in shared
// memory for buckets up to 8192 entries, rank sort for larger ones.
#define BSORT_CAP 8192
__global__ void k_bucket_sort(long long nbuckets, const long long* __restrict__ bstart, int* __restrict__ sid,
                              int* __restrict__ tmp)
{
    __shared__ int s[BSORT_CAP];
    for (long long b = blockIdx.x; b < nbuckets; b += gridDim.x) {
        long long b0 = bstart[b], b1 = bstart[b + 1];
        int n = (int)(b1 - b0);
        if (n <= 1) continue;
        if (n <= BSORT_CAP) {
            int np2 = 1;
            while (np2 < n) np2 <<= 1;
            for (int i = threadIdx.x; i < np2; i += blockDim.x) s[i] = i < n ? sid[b0 + i] : 0x7fffffff;
            __syncthreads();
            for (int k = 2; k <= np2; k <<= 1) {
                for (int j = k >> 1; j > 0; j >>= 1) {
                    for (int i = threadIdx.x; i < np2; i += blockDim.x) {
                        int l = i ^ j;
                        if (l > i) {
                            int a = s[i], c = s[l];
                            bool up = ((i & k) == 0);
                            if ((a > c) == up) {
                                s[i] = c;
                                s[l] = a;
                            }
                        }
                    }
                    __syncthreads();
                }
            }
            for (int i = threadIdx.x; i < n; i += blockDim.x) sid[b0 + i] = s[i];
            __syncthreads();
        } else {
            for (int i = threadIdx.x; i < n; i += blockDim.x) {
                int v = sid[b0 + i], r = 0;
                for (int k = 0; k < n; ++k) r += sid[b0 + k] < v;
                tmp[b0 + r] = v;
            }
            __syncthreads();
            for (int i = threadIdx.x; i < n; i += blockDim.x) sid[b0 + i] = tmp[b0 + i];
            __syncthreads();
        }
    }
}

__global__ void k_sorted_coords(int nsorted, const int* __restrict__ sid, const double* __restrict__ ox,
                                const double* __restrict__ oy, const double* __restrict__ oz,
                                const short* __restrict__ type, double* __restrict__ sx, double* __restrict__ sy,
                                double* __restrict__ sz, float* __restrict__ sxf, float* __restrict__ syf,
                                short* __restrict__ stype)
{
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nsorted) return;
    int o = sid[p];
    sx[p] = ox[o];
    sy[p] = oy[o];
    if (sz) sz[p] = oz[o];
    if (sxf) {
        sxf[p] = (float)ox[o];
        syf[p] = (float)oy[o];
    }
    stype[p] = type[o];
}

// S [nmem][nobs] -> St [nsorted][mpad] (sorted order, member-contiguous):
// tiled transpose into T1 [nobs][mpad] then a row gather.
__global__ void k_transpose_S(int nmem, int nobs, int mpad, const float* __restrict__ S, float* __restrict__ St)
{
    __shared__ float tile[32][33];
    int o0 = blockIdx.x * 32, e0 = blockIdx.y * 32;
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
        int e = e0 + k, o = o0 + threadIdx.x;
        tile[k][threadIdx.x] = (e < nmem && o < nobs) ? S[(size_t)e * nobs + o] : 0.0f;
    }
    __syncthreads();
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
        int o = o0 + k, e = e0 + threadIdx.x;
        if (o < nobs && e < mpad) St[(size_t)o * mpad + e] = (e < nmem) ? tile[threadIdx.x][k] : 0.0f;
    }
}

__global__ void k_gather_rows(int nsorted, int mpad, const int* __restrict__ sid, const float* __restrict__ src,
                              const double* __restrict__ s, float* __restrict__ St, double* __restrict__ ss,
                              float* __restrict__ ssf)
{
    // one warp per sorted row, float4 copies
    int p = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    if (p >= nsorted) return;
    int o = sid[p];
    const float4* a = (const float4*)(src + (size_t)o * mpad);
    float4* b = (float4*)(St + (size_t)p * mpad);
    for (int k = lane; k < mpad / 4; k += 32) b[k] = a[k];
    if (lane == 0) {
        ss[p] = s[o];
        ssf[p] = (float)s[o];
    }
}

// Largest |St| per member over all sorted rows (float bits: non-negative
// floats order like their bit patterns), for the mixed path's quantum.
__global__ void k_member_max(long long n4, int mpad, const float4* __restrict__ St, unsigned int* __restrict__ smax)
{
    __shared__ unsigned int sm[ENKFG_MAXMEM];
    for (int r = threadIdx.x; r < mpad; r += blockDim.x) sm[r] = 0u;
    __syncthreads();
    const int q4 = mpad / 4;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += (long long)gridDim.x * blockDim.x) {
        const float4 v = St[i];
        const int r = 4 * (int)(i % q4);
        atomicMax(&sm[r], __float_as_uint(fabsf(v.x)));
        atomicMax(&sm[r + 1], __float_as_uint(fabsf(v.y)));
        atomicMax(&sm[r + 2], __float_as_uint(fabsf(v.z)));
        atomicMax(&sm[r + 3], __float_as_uint(fabsf(v.w)));
    }
    __syncthreads();
    for (int r = threadIdx.x; r < mpad; r += blockDim.x)
        if (sm[r]) atomicMax(&smax[r], sm[r]);
}

// Per-member quantum of the mixed path's split: the power of two q with
// bound <= 256 q, bound = max |St| x (largest sum of taper weights) x
// (1 + 2^-20) (the FP32 product S * taper may round up).  Then every tapered
// value v of the member satisfies |rint(v / q)| <= 256.
__global__ void k_quantum(int m, float lcmax, const unsigned int* __restrict__ smax, float* __restrict__ qscale)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= m) return;
    const float bound = __uint_as_float(smax[r]) * lcmax * (1.0f + 9.5367431640625e-7f);
    float q = 1.0f;
    if (bound > 0.0f && isfinite(bound)) {
        int e;
        frexpf(bound, &e);               // bound = f 2^e, f in [0.5, 1)
        q = ldexpf(1.0f, e - 8);
    }
    qscale[r] = q;
    qscale[ENKFG_MAXMEM + r] = 1.0f / q;
}

// ---------------------------------------------------------------------------
// exclusive scan (int -> long long)
// ---------------------------------------------------------------------------
#define SCAN_T 1024
#define SCAN_IPT 4
__global__ void k_scan_block(const int* __restrict__ in, long long n, long long* __restrict__ out,
                             long long* __restrict__ bsum)
{
    __shared__ long long ws[32];
    long long base = (long long)blockIdx.x * SCAN_T * SCAN_IPT + (long long)threadIdx.x * SCAN_IPT;
    long long v[SCAN_IPT];
    long long acc = 0;
    for (int k = 0; k < SCAN_IPT; ++k) {
        long long i = base + k;
        v[k] = (i < n) ? in[i] : 0;
        acc += v[k];
    }
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    long long x = acc;
    for (int d = 1; d < 32; d <<= 1) {
        long long y = __shfl_up_sync(0xffffffffu, x, d);
        if (lane >= d) x += y;
    }
    if (lane == 31) ws[wid] = x;
    __syncthreads();
    if (wid == 0) {
        long long w = (lane < (SCAN_T >> 5)) ? ws[lane] : 0;
        for (int d = 1; d < 32; d <<= 1) {
            long long y = __shfl_up_sync(0xffffffffu, w, d);
            if (lane >= d) w += y;
        }
        ws[lane] = w;
    }
    __syncthreads();
    long long excl = x - acc + (wid > 0 ? ws[wid - 1] : 0);
    for (int k = 0; k < SCAN_IPT; ++k) {
        long long i = base + k;
        if (i < n) out[i] = excl;
        excl += v[k];
    }
    if (threadIdx.x == SCAN_T - 1) bsum[blockIdx.x] = excl;
}

__global__ void k_scan_add(long long* __restrict__ out, long long n, const long long* __restrict__ boff)
{
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long per = SCAN_T * SCAN_IPT;
    if (i < n) out[i] += boff[i / per];
}

// scan of long long block sums, serial in one thread per chunk (few blocks)
__global__ void k_scan_ll_small(const long long* __restrict__ in, long long n, long long* __restrict__ out)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    long long acc = 0;
    for (long long i = 0; i < n; ++i) {
        long long v = in[i];
        out[i] = acc;
        acc += v;
    }
    out[n] = acc;
}

enkfg_status scan_counts(enkfg_ctx* ctx, const int* d_in, long long* d_out, long long n, cudaStream_t st)
{
    long long per = SCAN_T * SCAN_IPT;
    long long nb = (n + per - 1) / per;
    if (nb < 1) nb = 1;
    size_t need = (size_t)(2 * nb + 2) * sizeof(long long);
    enkfg_status s = ensure(ctx, (char**)&ctx->d_scratch, &ctx->scratch_cap, need);
    if (s) return s;
    long long* bsum = (long long*)ctx->d_scratch;
    long long* boff = bsum + nb;
    k_scan_block<<<(unsigned)nb, SCAN_T, 0, st>>>(d_in, n, d_out, bsum);
    CKL();
    k_scan_ll_small<<<1, 32, 0, st>>>(bsum, nb, boff);
    CKL();
    k_scan_add<<<div_up(n + 1, 256), 256, 0, st>>>(d_out, n, boff);
    CKL();
    // total
    CK(cudaMemcpyAsync(d_out + n, boff + nb, sizeof(long long), cudaMemcpyDeviceToDevice, st));
    return ENKFG_OK;
}

// ---------------------------------------------------------------------------
// build the index
// ---------------------------------------------------------------------------
enkfg_status build_index(enkfg_ctx* ctx, cudaStream_t st)
{
    int nobs = ctx->nobs, ntypes = ctx->ntypes, ndim = ctx->geographic ? 3 : 2;
    enkfg_status s;

    // bounding boxes
    unsigned long long* d_box;
    const size_t box_bytes = (size_t)ntypes * 7 * sizeof(unsigned long long);
    CK(cudaMalloc(&d_box, box_bytes));
    {
        unsigned long long* h = (unsigned long long*)malloc(box_bytes);
        for (int t = 0; t < ntypes; ++t) {
            for (int a = 0; a < 3; ++a) {
                h[t * 6 + 2 * a] = ~0ull;
                h[t * 6 + 2 * a + 1] = 0ull;
            }
            h[ntypes * 6 + t] = 0ull;
        }
        cudaMemcpyAsync(d_box, h, box_bytes, cudaMemcpyHostToDevice, st);
        if (nobs > 0) {
            const int nb = div_up(nobs, BBOX_T * 8) < 2 * 152 ? div_up(nobs, BBOX_T * 8) : 2 * 152;
            k_bbox<<<nb, BBOX_T, 0, st>>>(nobs, ndim, ntypes, ctx->d_ox, ctx->d_oy, ctx->d_oz, ctx->d_type,
                                          ctx->d_status, d_box);
            ctx->launches++;
        }
        cudaMemcpyAsync(h, d_box, box_bytes, cudaMemcpyDeviceToHost, st);
        cudaError_t e = cudaStreamSynchronize(st);
        cudaFree(d_box);
        if (e != cudaSuccess) {
            free(h);
            return cuda_fail(ctx, e, "bbox", __LINE__);
        }
        long long base = 0;
        for (int t = 0; t < ntypes; ++t) {
            TypeIndex& ti = ctx->h_types[t];
            memset(&ti, 0, sizeof(ti));
            ti.nlocrad = ctx->nlocrad[t];
            double rmax = 0.0;
            for (int k = 0; k < ti.nlocrad; ++k) {
                ti.locrad[k] = ctx->locrad[t][k];
                ti.locweight[k] = ctx->locweight[t][k];
                if (ti.locrad[k] > rmax) rmax = ti.locrad[k];
            }
            ti.rmax = rmax;
            ti.rmax2 = rmax * rmax;
            for (int k = 0; k < ti.nlocrad; ++k) {
                ti.locrad_f[k] = (float)ti.locrad[k];
                ti.r2_f[k] = (float)(ti.locrad[k] * ti.locrad[k]);
                ti.r2_fl[k] = (float)(ti.locrad[k] * ti.locrad[k] - (double)ti.r2_f[k]);
                ti.locweight_f[k] = (float)ti.locweight[k];
            }
            // the FP32 squared distance (the high part of the double-float
            // one) is within a few units of 2^-24 of the exact one; 2e-6
            // relative leaves a margin of about 8x
            ti.rmax2_lo = (float)(ti.rmax2 * (1.0 - 2e-6));
            ti.rmax2_hi = (float)(ti.rmax2 * (1.0 + 2e-6));
            ti.nlobsmax = ctx->nlobsmax[t];
            bool empty = (h[t * 6] == ~0ull);
            double lo[3] = { 0, 0, 0 }, hi[3] = { 0, 0, 0 };
            if (!empty)
                for (int a = 0; a < ndim; ++a) {
                    lo[a] = dkey_inv(h[t * 6 + 2 * a]);
                    hi[a] = dkey_inv(h[t * 6 + 2 * a + 1]);
                }
            // cell edge: at least the radius (slightly enlarged so that
            // rounding in the cell arithmetic cannot skip a neighbour cell),
            // and no more cells per axis than 4000 (2-D) / 1000 (3-D) or
            // than the type's observation count allows: about 4 cells per
            // observation in 2-D and one per two in 3-D, so that the bucket
            // table (a power of two per axis) stays within a small multiple
            // of the observations however small the radius is against the
            // extent (a sphere's bounding cube is mostly empty)
            double ext = 0.0;
            for (int a = 0; a < ndim; ++a) ext = fmax(ext, hi[a] - lo[a]);
            const double nt = (double)(h[ntypes * 6 + t] > 0 ? h[ntypes * 6 + t] : 1);
            double axis = ndim == 2 ? fmin(4000.0, floor(sqrt(4.0 * nt))) : fmin(1000.0, floor(cbrt(0.5 * nt)));
            if (axis < 1.0) axis = 1.0;
            double cell = fmax(rmax * (1.0 + 1e-9), ext / axis);
            if (!(cell > 0.0)) cell = 1.0;
            ti.inv_cell = 1.0 / cell;
            ti.x0 = lo[0];
            ti.y0 = lo[1];
            ti.z0 = lo[2];
            ti.ncx = empty ? 1 : (int)floor((hi[0] - lo[0]) * ti.inv_cell) + 1;
            ti.ncy = empty ? 1 : (int)floor((hi[1] - lo[1]) * ti.inv_cell) + 1;
            ti.ncz = (ndim == 3 && !empty) ? (int)floor((hi[2] - lo[2]) * ti.inv_cell) + 1 : 1;
            int nmax = ti.ncx > ti.ncy ? ti.ncx : ti.ncy;
            if (ti.ncz > nmax) nmax = ti.ncz;
            int mb = 0;
            while ((1 << mb) < nmax) mb++;
            ti.mbits = mb;
            ti.nbuckets = 1ll << (ndim * mb);
            ti.bucket_base = base;
            base += ti.nbuckets;
        }
        free(h);
        ctx->nbuckets = base;
    }
    if (ctx->nbuckets > (1ll << 30)) {
        set_err(ctx, "spatial index too large (%lld buckets)", ctx->nbuckets);
        return ENKFG_ECAPACITY;
    }
    if (ctx->d_types == nullptr) CK(cudaMalloc(&ctx->d_types, sizeof(TypeIndex) * ENKFG_MAXTYPES));
    CK(cudaMemcpyAsync(ctx->d_types, ctx->h_types, sizeof(TypeIndex) * ntypes, cudaMemcpyHostToDevice, st));

    // bucket counts, scan, scatter, sort
    if ((s = ensure(ctx, &ctx->d_bstart, &ctx->bstart_cap, (size_t)ctx->nbuckets + 1))) return s;
    if ((s = ensure(ctx, &ctx->d_bfill, &ctx->bfill_cap, (size_t)ctx->nbuckets))) return s;
    if ((s = ensure(ctx, &ctx->d_key, &ctx->key_cap, (size_t)(nobs > 0 ? nobs : 1)))) return s;
    CK(cudaMemsetAsync(ctx->d_bfill, 0, ctx->nbuckets * sizeof(int), st));
    if (nobs > 0) {
        k_keys<<<div_up(nobs, 256), 256, 0, st>>>(nobs, ndim, ctx->d_ox, ctx->d_oy, ctx->d_oz, ctx->d_type,
                                                 ctx->d_status, ctx->d_types, ctx->d_key, ctx->d_bfill);
        CKL();
    }
    if ((s = scan_counts(ctx, ctx->d_bfill, ctx->d_bstart, ctx->nbuckets, st))) return s;
    long long total = 0;
    CK(cudaMemcpyAsync(&total, ctx->d_bstart + ctx->nbuckets, sizeof(long long), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    ctx->nsorted = (int)total;
    size_t ns = ctx->nsorted > 0 ? (size_t)ctx->nsorted : 1;
    if ((s = ensure(ctx, &ctx->d_sid, &ctx->sid_cap, ns))) return s;
    if ((s = ensure(ctx, &ctx->d_sx, &ctx->sx_cap, ns))) return s;
    if ((s = ensure(ctx, &ctx->d_sy, &ctx->sy_cap, ns))) return s;
    if ((s = ensure(ctx, &ctx->d_stype, &ctx->stype_cap, ns))) return s;
    if (ndim == 3) {
        if ((s = ensure(ctx, &ctx->d_sz, &ctx->sz_cap, ns))) return s;
        // the FP32 search copies exist for 2-D only
        cudaFree(ctx->d_sxf);
        cudaFree(ctx->d_syf);
        ctx->d_sxf = ctx->d_syf = nullptr;
        ctx->sxf_cap = ctx->syf_cap = 0;
    } else {
        cudaFree(ctx->d_sz);
        ctx->d_sz = nullptr;
        ctx->sz_cap = 0;
        if ((s = ensure(ctx, &ctx->d_sxf, &ctx->sxf_cap, ns))) return s;
        if ((s = ensure(ctx, &ctx->d_syf, &ctx->syf_cap, ns))) return s;
    }
    CK(cudaMemsetAsync(ctx->d_bfill, 0, ctx->nbuckets * sizeof(int), st));
    if (nobs > 0) {
        k_scatter<<<div_up(nobs, 256), 256, 0, st>>>(nobs, ctx->d_key, ctx->d_bstart, ctx->d_bfill, ctx->d_sid);
        CKL();
        int grid = (int)(ctx->nbuckets < 65536 ? ctx->nbuckets : 65536);
        k_bucket_sort<<<grid, 512, 0, st>>>(ctx->nbuckets, ctx->d_bstart, ctx->d_sid, ctx->d_key);
        CKL();
    }
    if (ctx->nsorted > 0) {
        k_sorted_coords<<<div_up(ctx->nsorted, 256), 256, 0, st>>>(ctx->nsorted, ctx->d_sid, ctx->d_ox, ctx->d_oy,
                                                                  ctx->d_oz, ctx->d_type, ctx->d_sx, ctx->d_sy,
                                                                  ctx->d_sz, ctx->d_sxf, ctx->d_syf, ctx->d_stype);
        CKL();
    }
    // per-type sorted ranges (bucket_base ranges are contiguous by type)
    for (int t = 0; t < ntypes; ++t) {
        long long r[2];
        CK(cudaMemcpyAsync(&r[0], ctx->d_bstart + ctx->h_types[t].bucket_base, sizeof(long long),
                           cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(&r[1], ctx->d_bstart + ctx->h_types[t].bucket_base + ctx->h_types[t].nbuckets,
                           sizeof(long long), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        ctx->h_types[t].pos_begin = (int)r[0];
        ctx->h_types[t].pos_end = (int)r[1];
    }
    if ((s = upload_types(ctx, st))) return s;
    ctx->index_valid = true;
    ctx->gather_valid = false;
    ctx->cut_valid = false;
    return ENKFG_OK;
}

enkfg_status upload_types(enkfg_ctx* ctx, cudaStream_t st)
{
    // observations.c:1877-1892: a type whose domains do not include the
    // grid's is skipped by obs_findlocal; here its position range is empty
    for (int t = 0; t < ctx->ntypes; ++t) {
        ctx->h_types_up[t] = ctx->h_types[t];
        ctx->h_types_up[t].nlobsmax = ctx->nlobsmax[t];
        if (ctx->hidden[t]) ctx->h_types_up[t].pos_end = ctx->h_types_up[t].pos_begin;
    }
    CK(cudaMemcpyAsync(ctx->d_types, ctx->h_types_up, sizeof(TypeIndex) * ctx->ntypes, cudaMemcpyHostToDevice, st));
    return ENKFG_OK;
}

enkfg_status build_gather(enkfg_ctx* ctx, cudaStream_t st)
{
    int m = ctx->nmem, nobs = ctx->nobs;
    int mpad = (m + 3) & ~3;
    ctx->mpad = mpad;
    size_t ns = ctx->nsorted > 0 ? (size_t)ctx->nsorted : 1;
    enkfg_status s;
    if ((s = ensure(ctx, &ctx->d_St, &ctx->St_cap, ns * mpad))) return s;
    if ((s = ensure(ctx, &ctx->d_ss, &ctx->ss_cap, ns))) return s;
    if ((s = ensure(ctx, &ctx->d_ssf, &ctx->ssf_cap, ns))) return s;
    if (nobs > 0 && ctx->nsorted > 0) {
        if ((s = ensure(ctx, &ctx->d_gtmp, &ctx->gtmp_cap, (size_t)nobs * mpad))) return s;
        dim3 g(div_up(nobs, 32), div_up(mpad, 32));
        k_transpose_S<<<g, dim3(32, 8), 0, st>>>(m, nobs, mpad, ctx->d_S, ctx->d_gtmp);
        CKL();
        k_gather_rows<<<div_up((long long)ctx->nsorted * 32, 256), 256, 0, st>>>(ctx->nsorted, mpad, ctx->d_sid,
                                                                               ctx->d_gtmp, ctx->d_s, ctx->d_St,
                                                                               ctx->d_ss, ctx->d_ssf);
        CKL();
    }
    // the mixed path's per-member quantum
    {
        double lcmax = 0.0;
        for (int t = 0; t < ctx->ntypes; ++t) {
            double sw = 0.0;
            for (int k = 0; k < ctx->nlocrad[t]; ++k) sw += fabs(ctx->locweight[t][k]);
            if (sw > lcmax) lcmax = sw;
        }
        CK(cudaMemsetAsync(ctx->d_smax, 0, ENKFG_MAXMEM * sizeof(unsigned int), st));
        const long long n4 = (long long)ctx->nsorted * (mpad / 4);
        if (n4 > 0) {
            k_member_max<<<304, 256, 0, st>>>(n4, mpad, (const float4*)ctx->d_St, ctx->d_smax);
            CKL();
        }
        k_quantum<<<1, ENKFG_MAXMEM, 0, st>>>(m, (float)lcmax, ctx->d_smax, ctx->d_qscale);
        CKL();
    }
    ctx->gather_valid = true;
    return ENKFG_OK;
}

// ---------------------------------------------------------------------------
// local observation count / list
// ---------------------------------------------------------------------------

// Neighbour cells of a query point for type t: returns the number of cells
// and fills the bucket ids (at most 27).
__device__ __forceinline__ int neighbour_buckets(const TypeIndex& t, int ndim, double qx, double qy, double qz,
                                                 long long* b)
{
    // query cell (as a double first: the query can be far outside the grid)
    double fx = floor((qx - t.x0) * t.inv_cell), fy = floor((qy - t.y0) * t.inv_cell);
    double fz = ndim == 3 ? floor((qz - t.z0) * t.inv_cell) : 0.0;
    int n = 0;
    if (fx < -1.0 || fx > (double)t.ncx || fy < -1.0 || fy > (double)t.ncy) return 0;
    if (ndim == 3 && (fz < -1.0 || fz > (double)t.ncz)) return 0;
    int cx = (int)fx, cy = (int)fy, cz = (int)fz;
    int zlo = ndim == 3 ? cz - 1 : 0, zhi = ndim == 3 ? cz + 1 : 0;
    for (int z = zlo; z <= zhi; ++z) {
        if (z < 0 || z >= t.ncz) continue;
        for (int y = cy - 1; y <= cy + 1; ++y) {
            if (y < 0 || y >= t.ncy) continue;
            for (int x = cx - 1; x <= cx + 1; ++x) {
                if (x < 0 || x >= t.ncx) continue;
                b[n++] = bucket_of(t, ndim, x, y, z);
            }
        }
    }
    return n;
}

// one warp per strided point
__global__ void k_count_local(int npts, int ntypes, int ndim, const TypeIndex* __restrict__ types,
                              const long long* __restrict__ bstart, const double* __restrict__ sx,
                              const double* __restrict__ sy, const double* __restrict__ sz,
                              const double* __restrict__ qx, const double* __restrict__ qy,
                              const double* __restrict__ qz, const int* __restrict__ sid,
                              const CutKey* __restrict__ cut, int* __restrict__ counts, int* __restrict__ pcounts)
{
    int pt = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    if (pt >= npts) return;
    double x = qx[pt], y = qy[pt], z = ndim == 3 ? qz[pt] : 0.0;
    int total = 0;
    for (int t = 0; t < ntypes; ++t) {
        const TypeIndex& ti = types[t];
        int nt = 0;
        if (ti.pos_end > ti.pos_begin) {
            const bool cut_on = cut != nullptr && ti.nlobsmax > 0;
            CutKey ck{};
            if (cut_on) ck = cut[(size_t)t * npts + pt];
            long long bk[27];
            int nb = neighbour_buckets(ti, ndim, x, y, z, bk);
            for (int k = 0; k < nb; ++k) {
                long long b0 = bstart[bk[k]], b1 = bstart[bk[k] + 1];
                for (long long base = b0; base < b1; base += 32) {
                    long long p = base + lane;
                    bool in = false;
                    if (p < b1) {
                        double d2 = ndim == 2 ? exact::dist2(sx[p], sy[p], x, y)
                                              : exact::dist3(sx[p], sy[p], sz[p], x, y, z);
                        in = d2 <= ti.rmax2;
                        if (cut_on && in) in = cut_keeps(d2, sid[p], ck);
                    }
                    nt += __popc(__ballot_sync(0xffffffffu, in));
                }
            }
        }
        if (pcounts != nullptr && lane == 0) pcounts[(size_t)t * npts + pt] = nt;
        total += nt;
    }
    if (lane == 0) counts[pt] = total;
}

// Candidate count of every strided point: the observations in its
// neighbour buckets (the search's candidates, no distance tests).  The
// batched path orders its work queue and picks the round size by this
// count, which is proportional to the local count at a fraction of the
// cost; one thread per point.
__global__ void k_count_candidates(int npts, int ntypes, int ndim, const TypeIndex* __restrict__ types,
                                   const long long* __restrict__ bstart, const double* __restrict__ qx,
                                   const double* __restrict__ qy, const double* __restrict__ qz,
                                   int* __restrict__ counts)
{
    const int pt = blockIdx.x * blockDim.x + threadIdx.x;
    if (pt >= npts) return;
    const double x = qx[pt], y = qy[pt], z = ndim == 3 ? qz[pt] : 0.0;
    long long total = 0;
    for (int t = 0; t < ntypes; ++t) {
        const TypeIndex& ti = types[t];
        if (ti.pos_end <= ti.pos_begin) continue;
        long long bk[27];
        const int nb = neighbour_buckets(ti, ndim, x, y, z, bk);
        for (int k = 0; k < nb; ++k) total += bstart[bk[k] + 1] - bstart[bk[k]];
    }
    counts[pt] = total < 0x7fffffffll ? (int)total : 0x7fffffff;
}

enkfg_status count_candidates(enkfg_ctx* ctx, int* d_counts, cudaStream_t st)
{
    int npts = ctx->nj * ctx->ni;
    int ndim = ctx->geographic ? 3 : 2;
    k_count_candidates<<<div_up(npts, 256), 256, 0, st>>>(npts, ctx->ntypes, ndim, ctx->d_types, ctx->d_bstart,
                                                          ctx->d_qx, ctx->d_qy, ctx->d_qz, d_counts);
    CKL();
    return ENKFG_OK;
}

enkfg_status count_local(enkfg_ctx* ctx, int* d_counts, int* d_pcounts, cudaStream_t st)
{
    int npts = ctx->nj * ctx->ni;
    int ndim = ctx->geographic ? 3 : 2;
    k_count_local<<<div_up((long long)npts * 32, 256), 256, 0, st>>>(
        npts, ctx->ntypes, ndim, ctx->d_types, ctx->d_bstart, ctx->d_sx, ctx->d_sy, ctx->d_sz, ctx->d_qx, ctx->d_qy,
        ctx->d_qz, ctx->d_sid, any_nlobsmax(ctx) ? ctx->d_cut : nullptr, d_counts, d_pcounts);
    CKL();
    return ENKFG_OK;
}

// One CTA per point: collect (id, taper) of every local obs, sort by id and
// write the CSR row.  Capacity LIST_CAP entries per point (a power of two,
// so that the bitonic network never leaves the arrays).
#define LIST_CAP 8192
#define LIST_T 256
__global__ void __launch_bounds__(LIST_T) k_list_local(int npts, int ntypes, int ndim,
                                                       const TypeIndex* __restrict__ types,
                                                       const long long* __restrict__ bstart,
                                                       const double* __restrict__ sx, const double* __restrict__ sy,
                                                       const double* __restrict__ sz, const int* __restrict__ sid,
                                                       const double* __restrict__ qx, const double* __restrict__ qy,
                                                       const double* __restrict__ qz,
                                                       const CutKey* __restrict__ cut,
                                                       const long long* __restrict__ offsets, int* __restrict__ ids,
                                                       double* __restrict__ coeffs, int* __restrict__ err)
{
    extern __shared__ unsigned char smem[];
    int* kid = (int*)smem;
    double* kc = (double*)(smem + LIST_CAP * sizeof(int));
    __shared__ int wsum[LIST_T / 32];
    __shared__ int n_sh;
    int pt = blockIdx.x;
    if (pt >= npts) return;
    double x = qx[pt], y = qy[pt], z = ndim == 3 ? qz[pt] : 0.0;
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (threadIdx.x == 0) n_sh = 0;
    __syncthreads();
    for (int t = 0; t < ntypes; ++t) {
        const TypeIndex& ti = types[t];
        if (ti.pos_end <= ti.pos_begin) continue;
        const bool cut_on = cut != nullptr && ti.nlobsmax > 0;
        CutKey ck{};
        if (cut_on) ck = cut[(size_t)t * npts + pt];
        long long bk[27];
        int nb = neighbour_buckets(ti, ndim, x, y, z, bk);
        for (int k = 0; k < nb; ++k) {
            long long b0 = bstart[bk[k]], b1 = bstart[bk[k] + 1];
            for (long long base = b0; base < b1; base += LIST_T) {
                long long p = base + threadIdx.x;
                bool in = false;
                double d2 = 0.0;
                if (p < b1) {
                    d2 = ndim == 2 ? exact::dist2(sx[p], sy[p], x, y) : exact::dist3(sx[p], sy[p], sz[p], x, y, z);
                    in = d2 <= ti.rmax2;
                    if (cut_on && in) in = cut_keeps(d2, sid[p], ck);
                }
                unsigned bal = __ballot_sync(0xffffffffu, in);
                if (lane == 0) wsum[wid] = __popc(bal);
                __syncthreads();
                int before = 0, tot = 0;
                for (int w = 0; w < LIST_T / 32; ++w) {
                    if (w < wid) before += wsum[w];
                    tot += wsum[w];
                }
                int pos = n_sh + before + __popc(bal & ((1u << lane) - 1));
                if (in && pos < LIST_CAP) {
                    kid[pos] = sid[p];
                    kc[pos] = exact::calclcoeff(ti.nlocrad, ti.locrad, ti.locweight, __dsqrt_rn(d2));
                }
                __syncthreads();
                if (threadIdx.x == 0) n_sh += tot;
                __syncthreads();
            }
        }
    }
    int n = n_sh;
    if (n > LIST_CAP) {
        if (threadIdx.x == 0) atomicMax(err, n);
        return;
    }
    int np2 = 1;
    while (np2 < n) np2 <<= 1;
    for (int i = n + threadIdx.x; i < np2; i += LIST_T) kid[i] = 0x7fffffff;
    __syncthreads();
    for (int k = 2; k <= np2; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = threadIdx.x; i < np2; i += LIST_T) {
                int l = i ^ j;
                if (l > i) {
                    int a = kid[i], c = kid[l];
                    bool up = ((i & k) == 0);
                    if ((a > c) == up) {
                        double tmp = kc[i];
                        kid[i] = c;
                        kid[l] = a;
                        kc[i] = kc[l];
                        kc[l] = tmp;
                    }
                }
            }
            __syncthreads();
        }
    }
    long long o0 = offsets[pt];
    for (int i = threadIdx.x; i < n; i += LIST_T) {
        ids[o0 + i] = kid[i];
        coeffs[o0 + i] = kc[i];
    }
}

enkfg_status list_local(enkfg_ctx* ctx, const long long* d_offsets, int* d_ids, double* d_coeffs, cudaStream_t st)
{
    int npts = ctx->nj * ctx->ni;
    int ndim = ctx->geographic ? 3 : 2;
    size_t smem = LIST_CAP * (sizeof(int) + sizeof(double));
    CK(cudaFuncSetAttribute(k_list_local, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    CK(cudaMemsetAsync(ctx->d_qhead, 0, 2 * sizeof(int), st));
    k_list_local<<<npts, LIST_T, smem, st>>>(npts, ctx->ntypes, ndim, ctx->d_types, ctx->d_bstart, ctx->d_sx,
                                             ctx->d_sy, ctx->d_sz, ctx->d_sid, ctx->d_qx, ctx->d_qy, ctx->d_qz,
                                             any_nlobsmax(ctx) ? ctx->d_cut : nullptr, d_offsets, d_ids, d_coeffs,
                                             ctx->d_qhead + 1);
    CKL();
    int over = 0;
    CK(cudaMemcpyAsync(&over, ctx->d_qhead + 1, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (over > 0) {
        set_err(ctx, "a point has %d local observations, above the list capacity %d", over, LIST_CAP);
        return ENKFG_ECAPACITY;
    }
    return ENKFG_OK;
}

// ---------------------------------------------------------------------------
// NLOBSMAX cuts (observations.c:1899-1901, kdtree.c:558-574: with a limit the
// range results of a type are sorted by squared distance and the first
// nlobsmax kept).  One CTA per point: for each type with a limit, the
// nlobsmax-th smallest key (d2, id) among the observations in range, by a
// radix select (8-bit digits) over the 64 bits of the FP64 squared distance
// (non-negative, so its bit pattern orders as the value) and then, among the
// observations at that distance, over the 32 bits of the id.  Keys are staged
// in shared memory when they fit (CUT_CAP); otherwise every pass runs the
// search again.  Equal distances are ordered by id.
// ---------------------------------------------------------------------------
#define CUT_T 256
#define CUT_CAP 8192

struct CutSmem {
    unsigned long long kd[CUT_CAP];   // FP64 bits of d2
    int kid[CUT_CAP];                 // observation id
    int hist[256];
    int wsum[CUT_T / 32];
    int n;                            // keys of the type in range
    int rank;                         // rank still to find (1-based)
    int sel;                          // selected digit
    int tie;                          // keys in the selected digit
};

__global__ void __launch_bounds__(CUT_T) k_cut_local(int npts, int ntypes, int ndim,
                                                     const TypeIndex* __restrict__ types,
                                                     const long long* __restrict__ bstart,
                                                     const double* __restrict__ sx, const double* __restrict__ sy,
                                                     const double* __restrict__ sz, const int* __restrict__ sid,
                                                     const double* __restrict__ qx, const double* __restrict__ qy,
                                                     const double* __restrict__ qz, CutKey* __restrict__ cut)
{
    extern __shared__ unsigned char smem_raw[];
    CutSmem& sm = *reinterpret_cast<CutSmem*>(smem_raw);
    const int pt = blockIdx.x, tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    if (pt >= npts) return;
    const double x = qx[pt], y = qy[pt], z = ndim == 3 ? qz[pt] : 0.0;
    for (int t = 0; t < ntypes; ++t) {
        const TypeIndex& ti = types[t];
        CutKey res;
        res.d2 = __longlong_as_double(0x7ff0000000000000ll);   // +inf: keep all
        res.id = 0x7fffffff;
        res.pad = 0;
        if (ti.nlobsmax <= 0 || ti.pos_end <= ti.pos_begin) {
            if (tid == 0) cut[(size_t)t * npts + pt] = res;
            continue;
        }
        long long bk[27];
        const int nb = neighbour_buckets(ti, ndim, x, y, z, bk);
        // every observation of the type in range, as (d2 bits, id), in
        // passes over the candidates (staged: from shared memory)
        auto search = [&](auto&& f) {
            for (int k = 0; k < nb; ++k) {
                const long long b0 = bstart[bk[k]], b1 = bstart[bk[k] + 1];
                for (long long p = b0 + tid; p < b1; p += CUT_T) {
                    const double d2 = ndim == 2 ? exact::dist2(sx[p], sy[p], x, y)
                                                : exact::dist3(sx[p], sy[p], sz[p], x, y, z);
                    if (d2 <= ti.rmax2) f((unsigned long long)__double_as_longlong(d2), sid[p]);
                }
            }
        };
        // count and stage
        if (tid == 0) sm.n = 0;
        __syncthreads();
        for (int k = 0; k < nb; ++k) {
            const long long b0 = bstart[bk[k]], b1 = bstart[bk[k] + 1];
            for (long long base = b0; base < b1; base += CUT_T) {
                const long long p = base + tid;
                bool in = false;
                double d2 = 0.0;
                if (p < b1) {
                    d2 = ndim == 2 ? exact::dist2(sx[p], sy[p], x, y) : exact::dist3(sx[p], sy[p], sz[p], x, y, z);
                    in = d2 <= ti.rmax2;
                }
                const unsigned bal = __ballot_sync(0xffffffffu, in);
                if (lane == 0) sm.wsum[wid] = __popc(bal);
                __syncthreads();
                int before = 0, tot = 0;
                for (int w = 0; w < CUT_T / 32; ++w) {
                    before += (w < wid) ? sm.wsum[w] : 0;
                    tot += sm.wsum[w];
                }
                const int pos = sm.n + before + __popc(bal & ((1u << lane) - 1));
                if (in && pos < CUT_CAP) {
                    sm.kd[pos] = (unsigned long long)__double_as_longlong(d2);
                    sm.kid[pos] = sid[p];
                }
                __syncthreads();
                if (tid == 0) sm.n += tot;
                __syncthreads();
            }
        }
        const int n = sm.n;
        if (n <= ti.nlobsmax) {
            if (tid == 0) cut[(size_t)t * npts + pt] = res;
            __syncthreads();
            continue;
        }
        const bool staged = n <= CUT_CAP;
        auto each_key = [&](auto&& f) {
            if (staged) {
                for (int i = tid; i < n; i += CUT_T) f(sm.kd[i], sm.kid[i]);
            } else {
                search(f);
            }
        };
        // warp 0 finds the digit holding the rank-th key and updates the rank
        auto pick = [&]() {
            if (wid == 0) {
                int c[8], s = 0;
#pragma unroll
                for (int i = 0; i < 8; ++i) {
                    c[i] = sm.hist[lane * 8 + i];
                    s += c[i];
                }
                int incl = s;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int v = __shfl_up_sync(0xffffffffu, incl, o);
                    if (lane >= o) incl += v;
                }
                const int r = sm.rank;
                const unsigned hit = __ballot_sync(0xffffffffu, incl >= r);
                const int L = __ffs(hit) - 1;   // the rank is at most the count: some lane hits
                if (lane == L) {
                    int cum = incl - s;
                    for (int i = 0; i < 8; ++i) {
                        if (cum + c[i] >= r) {
                            sm.sel = lane * 8 + i;
                            sm.tie = c[i];
                            sm.rank = r - cum;
                            break;
                        }
                        cum += c[i];
                    }
                }
            }
            __syncthreads();
        };
        if (tid == 0) sm.rank = ti.nlobsmax;
        unsigned long long dpre = 0;
        for (int shift = 56; shift >= 0; shift -= 8) {
            sm.hist[tid] = 0;
            __syncthreads();
            const unsigned long long hmask = shift == 56 ? 0ull : (~0ull << (shift + 8));
            each_key([&](unsigned long long kd, int) {
                if ((kd & hmask) == dpre) atomicAdd(&sm.hist[(int)((kd >> shift) & 255ull)], 1);
            });
            __syncthreads();
            pick();
            dpre |= (unsigned long long)sm.sel << shift;
        }
        res.d2 = __longlong_as_double((long long)dpre);
        if (sm.rank < sm.tie) {
            // among the keys at distance d2, the rank-th smallest id
            unsigned ipre = 0;
            for (int shift = 24; shift >= 0; shift -= 8) {
                sm.hist[tid] = 0;
                __syncthreads();
                const unsigned imask = shift == 24 ? 0u : (~0u << (shift + 8));
                each_key([&](unsigned long long kd, int id) {
                    if (kd == dpre && ((unsigned)id & imask) == ipre)
                        atomicAdd(&sm.hist[(int)(((unsigned)id >> shift) & 255u)], 1);
                });
                __syncthreads();
                pick();
                ipre |= (unsigned)sm.sel << shift;
            }
            res.id = (int)ipre;
        }
        if (tid == 0) cut[(size_t)t * npts + pt] = res;
        __syncthreads();
    }
}

bool any_nlobsmax(const enkfg_ctx* ctx)
{
    for (int t = 0; t < ctx->ntypes; ++t)
        if (ctx->nlobsmax[t] > 0 && !ctx->hidden[t]) return true;
    return false;
}

enkfg_status prepare_search(enkfg_ctx* ctx, cudaStream_t st)
{
    enkfg_status s;
    if (!ctx->index_valid && (s = build_index(ctx, st))) return s;
    if (!any_nlobsmax(ctx) || ctx->cut_valid) return ENKFG_OK;
    const int npts = ctx->nj * ctx->ni, ndim = ctx->geographic ? 3 : 2;
    if ((s = ensure(ctx, &ctx->d_cut, &ctx->cut_cap, (size_t)ctx->ntypes * npts))) return s;
    const size_t smem = sizeof(CutSmem);
    CK(cudaFuncSetAttribute(k_cut_local, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_cut_local<<<npts, CUT_T, smem, st>>>(npts, ctx->ntypes, ndim, ctx->d_types, ctx->d_bstart, ctx->d_sx,
                                           ctx->d_sy, ctx->d_sz, ctx->d_sid, ctx->d_qx, ctx->d_qy, ctx->d_qz,
                                           ctx->d_cut);
    CKL();
    ctx->cut_valid = true;
    return ENKFG_OK;
}
