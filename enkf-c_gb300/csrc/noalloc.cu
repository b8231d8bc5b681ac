// noalloc.cu -- CSR offsets of local-observation counts without any device
// allocation.
//
// The offsets enkfg_local_obs returns (offsets[k] = counts[0] + ... +
// counts[k-1], offsets[n] = total) come from a three-step scan whose block
// sums live in scratch the context allocates.  Some callers cannot allocate
// device memory at all -- code running under a memory pool that owns the
// whole device, real-time or embedded hosts that forbid allocation after
// start-up, or a caller that must not trigger an implicit synchronisation
// from cudaMalloc/cudaFree.  enkfg_local_offsets_noalloc gives them the same
// offsets with the block sums in the fixed array below instead.
//
// The array is a file-scope __device__ object: every GPU that loads this
// library keeps it (512 KiB) until the process exits.  Host code cannot use
// the array's name as a device address; the address comes from
// cudaGetSymbolAddress, called with the caller's device (context) current.
// Outside stream capture every call looks the address up again (a symbol
// lookup, no allocation), so a device reset, which reloads the module, or a
// caller's own driver-API context on the same device, where the array has
// another address, always gets the right one.  The address is also recorded
// per CUDA context, and a call made while `stream` is being captured uses the
// recorded one: the first call in a context must therefore come before any
// capture in it (otherwise ENKFG_ESTATE), and after a device reset one
// uncaptured call must come before the next capture.  All calls share the
// array: calls that overlap on the GPU (different streams, or different host
// threads on the same device) race on it and must be serialised by the
// caller.  The array keeps the previous call's block sums; nothing in it
// needs to start at zero, because each call writes every entry it reads (its
// nb block sums, then their nb + 1 offsets) before reading it.
#include "internal.cuh"
#include <cuda.h>
#include <mutex>

#define NA_T 1024
#define NA_IPT 4
#define NA_PER (NA_T * NA_IPT)                   // counts per scan block
#define NA_MAX_BLOCKS 32768                      // -> at most 134,217,728 counts
#define NA_MAX_CONTEXTS 64

// block sums [NA_MAX_BLOCKS] followed by their exclusive scan [NA_MAX_BLOCKS + 1]
static __device__ __align__(256) long long g_noalloc_scratch[2 * NA_MAX_BLOCKS + 2];

static std::mutex g_noalloc_mu;
// the scratch array's address in each CUDA context seen so far
struct NaContextAddr {
    CUcontext cx;
    long long* ptr;
};
static NaContextAddr g_noalloc_addr[NA_MAX_CONTEXTS];
static int g_noalloc_naddr = 0;
typedef CUresult (*NaCtxGetCurrent)(CUcontext*);
static NaCtxGetCurrent g_ctx_get_current = nullptr;

// The scratch array's address in the current context (see the file comment).
static enkfg_status noalloc_scratch(cudaStream_t st, long long** out)
{
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st, &cs) != cudaSuccess) {
        cudaGetLastError();
        return ENKFG_ECUDA;
    }
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (g_ctx_get_current == nullptr) {
        if (cs != cudaStreamCaptureStatusNone) return ENKFG_ESTATE;
        void* fn = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess || fn == nullptr) {
            cudaGetLastError();
            return ENKFG_ECUDA;
        }
        g_ctx_get_current = (NaCtxGetCurrent)fn;
    }
    void* p = nullptr;
    if (cs == cudaStreamCaptureStatusNone) {
        // this also makes the device's primary context current if the
        // caller has not touched the device yet
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || p == nullptr) {
            cudaGetLastError();
            return ENKFG_ECUDA;
        }
    }
    CUcontext cx = nullptr;
    if (g_ctx_get_current(&cx) != CUDA_SUCCESS || cx == nullptr) return ENKFG_ECUDA;
    int k = 0;
    while (k < g_noalloc_naddr && g_noalloc_addr[k].cx != cx) ++k;
    if (cs != cudaStreamCaptureStatusNone) {
        if (k == g_noalloc_naddr) return ENKFG_ESTATE;   // no uncaptured call in this context yet
        *out = g_noalloc_addr[k].ptr;
        return ENKFG_OK;
    }
    if (k == g_noalloc_naddr) {
        if (g_noalloc_naddr < NA_MAX_CONTEXTS) {
            ++g_noalloc_naddr;
        } else {
            k = NA_MAX_CONTEXTS - 1;   // table full: the newest entry is replaced
        }
        g_noalloc_addr[k].cx = cx;
    }
    g_noalloc_addr[k].ptr = (long long*)p;
    *out = (long long*)p;
    return ENKFG_OK;
}

__global__ void k_na_scan_block(const int* __restrict__ in, long long n, long long* __restrict__ out,
                                long long* __restrict__ bsum)
{
    __shared__ long long ws[NA_T / 32];
    long long base = (long long)blockIdx.x * NA_PER + (long long)threadIdx.x * NA_IPT;
    long long v[NA_IPT], acc = 0;
#pragma unroll
    for (int k = 0; k < NA_IPT; ++k) {
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
        long long t = ws[lane];
        for (int d = 1; d < 32; d <<= 1) {
            long long y = __shfl_up_sync(0xffffffffu, t, d);
            if (lane >= d) t += y;
        }
        ws[lane] = t;
    }
    __syncthreads();
    long long excl = x - acc + (wid > 0 ? ws[wid - 1] : 0);
#pragma unroll
    for (int k = 0; k < NA_IPT; ++k) {
        long long i = base + k;
        if (i < n) out[i] = excl;
        excl += v[k];
    }
    if (threadIdx.x == NA_T - 1) bsum[blockIdx.x] = excl;   // every block writes its sum
}

// exclusive scan of nb <= NA_MAX_BLOCKS block sums in one CTA; boff[nb] = total
__global__ void k_na_scan_sums(const long long* __restrict__ bsum, int nb, long long* __restrict__ boff)
{
    __shared__ long long ws[NA_T / 32];
    __shared__ long long carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int base = 0; base < nb; base += NA_T) {
        int i = base + threadIdx.x;
        long long v = (i < nb) ? bsum[i] : 0, x = v;
        for (int d = 1; d < 32; d <<= 1) {
            long long y = __shfl_up_sync(0xffffffffu, x, d);
            if (lane >= d) x += y;
        }
        if (lane == 31) ws[wid] = x;
        __syncthreads();
        if (wid == 0) {
            long long t = ws[lane];
            for (int d = 1; d < 32; d <<= 1) {
                long long y = __shfl_up_sync(0xffffffffu, t, d);
                if (lane >= d) t += y;
            }
            ws[lane] = t;
        }
        __syncthreads();
        long long incl = x + (wid > 0 ? ws[wid - 1] : 0);
        if (i < nb) boff[i] = carry + incl - v;
        __syncthreads();
        if (threadIdx.x == NA_T - 1) carry += incl;
        __syncthreads();
    }
    if (threadIdx.x == 0) boff[nb] = carry;
}

__global__ void k_na_scan_add(long long* __restrict__ out, long long n, const long long* __restrict__ boff, int nb)
{
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] += boff[i / NA_PER];
    if (i == 0) out[n] = boff[nb];
}

extern "C" ENKFG_API enkfg_status enkfg_local_offsets_noalloc(const int* counts_dev, long long n,
                                                             long long* offsets_dev, void* stream)
{
    if ((counts_dev == nullptr && n > 0) || offsets_dev == nullptr || n < 0) return ENKFG_EINVAL;
    if (n > (long long)NA_MAX_BLOCKS * NA_PER) return ENKFG_ECAPACITY;
    cudaStream_t st = (cudaStream_t)stream;
    long long* scratch = nullptr;
    enkfg_status s0 = noalloc_scratch(st, &scratch);
    if (s0 != ENKFG_OK) return s0;
    int nb = (int)((n + NA_PER - 1) / NA_PER);
    if (nb < 1) nb = 1;
    long long* bsum = scratch;                 // fully written by k_na_scan_block
    long long* boff = scratch + NA_MAX_BLOCKS; // fully written by k_na_scan_sums
    k_na_scan_block<<<nb, NA_T, 0, st>>>(counts_dev, n, offsets_dev, bsum);
    k_na_scan_sums<<<1, NA_T, 0, st>>>(bsum, nb, boff);
    k_na_scan_add<<<(unsigned)((n + 256) / 256), 256, 0, st>>>(offsets_dev, n, boff, nb);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? ENKFG_OK : ENKFG_ECUDA;
}
