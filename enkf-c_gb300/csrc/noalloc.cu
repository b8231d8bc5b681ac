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
// library keeps it (512 KiB) until the process exits.  Host
// code cannot use the array's name as a device address, so the address is
// looked up once per device with cudaGetSymbolAddress, on the first call
// made with that device current; that first call should therefore be made
// before any stream capture.  All calls share the array: calls that overlap
// on the GPU (different streams, or different host threads on the same
// device) race on it and must be serialised by the caller.  The array keeps
// the previous call's block sums; nothing in it needs to start at zero,
// because each call writes every entry it reads (its nb block sums, then
// their nb + 1 offsets) before reading it.
#include "internal.cuh"
#include <mutex>

#define NA_T 1024
#define NA_IPT 4
#define NA_PER (NA_T * NA_IPT)                   // counts per scan block
#define NA_MAX_BLOCKS 32768                      // -> at most 134,217,728 counts
#define NA_MAX_DEVICES 64

// block sums [NA_MAX_BLOCKS] followed by their exclusive scan [NA_MAX_BLOCKS + 1]
static __device__ __align__(256) long long g_noalloc_scratch[2 * NA_MAX_BLOCKS + 2];

static std::mutex g_noalloc_mu;
static long long* g_noalloc_ptr[NA_MAX_DEVICES];

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
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= NA_MAX_DEVICES) {
        cudaGetLastError();
        return ENKFG_ECUDA;
    }
    long long* scratch;
    {
        // set-up, once per device: the device address of the scratch array
        std::lock_guard<std::mutex> lock(g_noalloc_mu);
        if (g_noalloc_ptr[dev] == nullptr) {
            void* p = nullptr;
            if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || p == nullptr) {
                cudaGetLastError();
                return ENKFG_ECUDA;
            }
            g_noalloc_ptr[dev] = (long long*)p;
        }
        scratch = g_noalloc_ptr[dev];
    }
    cudaStream_t st = (cudaStream_t)stream;
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
