// pk_sort.cuh — stable LSD radix sort of (u64 key, u64 value) pairs whose element count lives in
// device memory, so the launches can be captured in a CUDA graph once and replayed every step.
//
// One pass per 8-bit digit, three kernels per pass:
//   hist    : each CTA in use counts the digits of its contiguous chunk    -> hist[digit][cta]
//   scan    : one CTA per digit turns its row into exclusive offsets and records the row total
//   scatter : each CTA scans the 256 digit totals into digit bases, then walks its chunk in
//             256-element tiles, ranks equal digits inside a warp with __match_any_sync, combines
//             warps through shared-memory counters, and writes each element to digit base + row
//             offset + running count + rank (stable).
// Traffic per pass and element: read key+value twice (hist reads keys only), write key+value once.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace pk
{

constexpr int kSortThreads = 256;
constexpr int kSortRadix = 256;

// Chunking of [0, n) over at most `nblocks` CTAs, at least kSortMinChunk elements per CTA, so
// a short list touches one CTA and a short digit table (the cost of a pass follows n, not the
// capacity the launches were sized for). CTAs at or past `used` have no chunk.
constexpr int kSortMinChunk = 4096;

__device__ __forceinline__ int sort_per(int n, int nblocks)
{
    int per = (n + nblocks - 1) / nblocks;
    per = per > kSortMinChunk ? per : kSortMinChunk;
    return (per + kSortThreads - 1) / kSortThreads * kSortThreads;
}

__device__ __forceinline__ int sort_used(int n, int nblocks)
{
    int per = sort_per(n, nblocks);
    return (n + per - 1) / per;
}

__device__ __forceinline__ void sort_chunk(int n, int nblocks, int b, int &lo, int &hi)
{
    int per = sort_per(n, nblocks);
    lo = min(n, b * per);
    hi = min(n, lo + per);
}

static __global__ void __launch_bounds__(kSortThreads) k_sort_hist(const uint64_t *__restrict__ keys, const int *n_ptr,
                                                            int shift, uint32_t *__restrict__ hist)
{
    __shared__ uint32_t h[kSortRadix];
    const int n = *n_ptr;
    const int used = sort_used(n, gridDim.x);
    if (int(blockIdx.x) >= used) return;
    h[threadIdx.x] = 0;
    __syncthreads();
    int lo, hi;
    sort_chunk(n, gridDim.x, blockIdx.x, lo, hi);
    for (int i = lo + threadIdx.x; i < hi; i += kSortThreads)
        atomicAdd(&h[(keys[i] >> shift) & 0xFF], 1u);
    __syncthreads();
    hist[threadIdx.x * used + blockIdx.x] = h[threadIdx.x];
}

// Block-wide exclusive scan of one value per thread (kSortThreads threads); returns the total.
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t &excl)
{
    __shared__ uint32_t wtot[kSortThreads / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t incl = v;
    for (int o = 1; o < 32; o <<= 1)
    {
        uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) wtot[warp] = incl;
    __syncthreads();
    uint32_t before = 0, total = 0;
    for (int k = 0; k < kSortThreads / 32; ++k)
    {
        uint32_t t = wtot[k];
        before += k < warp ? t : 0u;
        total += t;
    }
    __syncthreads();
    excl = before + incl - v;
    return total;
}

// Row `blockIdx.x` (one digit) of the digit table: exclusive offsets across the CTAs in use, and
// the row total into tot[digit].
static __global__ void __launch_bounds__(kSortThreads) k_sort_scan(uint32_t *__restrict__ hist, const int *n_ptr,
                                                                   int nblocks, uint32_t *__restrict__ tot)
{
    const int used = sort_used(*n_ptr, nblocks);
    uint32_t *row = hist + size_t(blockIdx.x) * used;
    uint32_t run = 0;
    for (int base = 0; base < used; base += kSortThreads)
    {
        const int i = base + int(threadIdx.x);
        uint32_t v = i < used ? row[i] : 0u, ex;
        uint32_t t = block_exclusive_scan(v, ex);
        if (i < used) row[i] = run + ex;
        run += t;
    }
    if (threadIdx.x == 0) tot[blockIdx.x] = run;
}

template <class V>
__global__ void __launch_bounds__(kSortThreads)
    k_sort_scatter(const uint64_t *__restrict__ kin, const V *__restrict__ vin, uint64_t *__restrict__ kout,
                   V *__restrict__ vout, const int *n_ptr, int shift, const uint32_t *__restrict__ hist,
                   const uint32_t *__restrict__ tot)
{
    constexpr int W = kSortThreads / 32;
    __shared__ uint32_t base[kSortRadix];
    __shared__ uint32_t running[kSortRadix];
    __shared__ uint32_t wcnt[W][kSortRadix + 1];
    __shared__ uint32_t tile_total[kSortRadix];
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const int n = *n_ptr;
    const int used = sort_used(n, gridDim.x);
    if (int(blockIdx.x) >= used) return;
    uint32_t digit_base;
    block_exclusive_scan(tot[t], digit_base);
    base[t] = digit_base + hist[t * used + blockIdx.x];
    running[t] = 0;
    int lo, hi;
    sort_chunk(n, gridDim.x, blockIdx.x, lo, hi);
    const unsigned lt_mask = (1u << lane) - 1u;
    for (int tile = lo; tile < hi; tile += kSortThreads)
    {
        for (int w = 0; w < W; ++w) wcnt[w][t] = 0;
        if (t == 0)
            for (int w = 0; w < W; ++w) wcnt[w][kSortRadix] = 0;
        __syncthreads();
        int i = tile + t;
        bool valid = i < hi;
        uint64_t k = valid ? kin[i] : 0;
        V v = valid ? vin[i] : V(0);
        int d = valid ? int((k >> shift) & 0xFF) : kSortRadix;
        unsigned same = __match_any_sync(0xFFFFFFFFu, d);
        int rank = __popc(same & lt_mask);
        if (rank == 0) wcnt[warp][d] = __popc(same);
        __syncthreads();
        {
            uint32_t s = 0;
            for (int w = 0; w < W; ++w)
            {
                uint32_t c = wcnt[w][t];
                wcnt[w][t] = s;
                s += c;
            }
            tile_total[t] = s;
        }
        __syncthreads();
        if (valid)
        {
            uint32_t dst = base[d] + running[d] + wcnt[warp][d] + uint32_t(rank);
            kout[dst] = k;
            vout[dst] = v;
        }
        __syncthreads();
        running[t] += tile_total[t];
        __syncthreads();
    }
}

// Host-side launcher. Sorts [0, *n_dev) of (k0, v0) by the low `bits` bits of the key; ping-pongs
// with (k1, v1); `hist` holds kSortRadix * (nblocks + 1) counters. Returns true when the result
// ends in (k1, v1).
template <class V>
inline bool radix_sort(uint64_t *k0, V *v0, uint64_t *k1, V *v1, const int *n_dev, int bits, int nblocks,
                       uint32_t *hist, cudaStream_t st)
{
    int passes = (bits + 7) / 8;
    if (passes < 1) passes = 1;
    uint64_t *ka = k0, *kb = k1;
    V *va = v0, *vb = v1;
    for (int p = 0; p < passes; ++p)
    {
        int shift = 8 * p;
        k_sort_hist<<<nblocks, kSortThreads, 0, st>>>(ka, n_dev, shift, hist);
        k_sort_scan<<<kSortRadix, kSortThreads, 0, st>>>(hist, n_dev, nblocks, hist + size_t(kSortRadix) * nblocks);
        k_sort_scatter<V><<<nblocks, kSortThreads, 0, st>>>(ka, va, kb, vb, n_dev, shift, hist,
                                                           hist + size_t(kSortRadix) * nblocks);
        uint64_t *tk = ka;
        ka = kb;
        kb = tk;
        V *tv = va;
        va = vb;
        vb = tv;
    }
    return (passes & 1) != 0;
}

} // namespace pk
