// pk_sort.cuh — stable LSD radix sort of (u64 key, u64 value) pairs whose element count lives in
// device memory, so the launches can be captured in a CUDA graph once and replayed every step.
//
// One pass per 8-bit digit, three kernels per pass:
//   hist    : each CTA in use counts the digits of its contiguous chunk    -> hist[digit][cta]
//   scan    : one CTA per digit turns its row into exclusive offsets and records the row total
//   scatter : each CTA scans the 256 digit totals into digit bases, then walks its chunk in tiles
//             of kSortTile elements: every warp ranks its contiguous sub-tile (equal digits inside a
//             warp through ballots of the digit bits, across its rounds through per-warp counters),
//             the CTA combines the warps, sorts the tile by digit in shared memory and writes each
//             digit's run out contiguously (stable). Runs of ~16 elements per digit per tile keep
//             the writes of the low, near-random digits in whole sectors.
// Traffic per pass and element: read key+value twice (hist reads keys only), write key+value once.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace pk
{

constexpr int kSortThreads = 256;
constexpr int kSortRadix = 256;
constexpr int kSortItems = 16;                        // elements per thread and tile
constexpr int kSortTile = kSortThreads * kSortItems; // elements per tile
constexpr size_t kSortSmem = size_t(kSortTile) * 16; // tile keys + values in dynamic shared memory

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
                                                            int shift, uint32_t *__restrict__ hist, const int *skip)
{
    __shared__ uint32_t h[kSortRadix];
    if (skip && *skip) return;
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

// Lanes of the warp holding the same 8-bit digit as this lane (d = kSortRadix marks an empty lane,
// which matches only other empty lanes): one ballot per digit bit plus one for emptiness.
__device__ __forceinline__ unsigned digit_peers(int d)
{
    unsigned m = __ballot_sync(0xFFFFFFFFu, d == kSortRadix);
    if (d != kSortRadix) m = ~m;
#pragma unroll
    for (int b = 0; b < 8; ++b)
    {
        const unsigned v = __ballot_sync(0xFFFFFFFFu, (d >> b) & 1);
        m &= ((d >> b) & 1) ? v : ~v;
    }
    return m;
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
                                                                   int nblocks, uint32_t *__restrict__ tot, const int *skip)
{
    if (skip && *skip) return;
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
__global__ void __launch_bounds__(kSortThreads, 2)
    k_sort_scatter(const uint64_t *__restrict__ kin, const V *__restrict__ vin, uint64_t *__restrict__ kout,
                   V *__restrict__ vout, const int *n_ptr, int shift, const uint32_t *__restrict__ hist,
                   const uint32_t *__restrict__ tot, const int *skip)
{
    static_assert(sizeof(V) == 8, "tile staging holds 8-byte values");
    if (skip && *skip) return;
    constexpr int W = kSortThreads / 32;
    extern __shared__ uint64_t sort_tile[];
    uint64_t *skey = sort_tile;
    V *sval = reinterpret_cast<V *>(sort_tile + kSortTile);
    __shared__ uint32_t base[kSortRadix];    // output position of this CTA's next element of each digit
    __shared__ uint32_t tstart[kSortRadix];  // first tile position of each digit
    __shared__ uint32_t wcnt[W][kSortRadix]; // per-warp digit counts, then offsets across warps
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const int n = *n_ptr;
    const int used = sort_used(n, gridDim.x);
    if (int(blockIdx.x) >= used) return;
    uint32_t digit_base;
    block_exclusive_scan(tot[t], digit_base);
    base[t] = digit_base + hist[t * used + blockIdx.x];
    int lo, hi;
    sort_chunk(n, gridDim.x, blockIdx.x, lo, hi);
    const unsigned lt_mask = (1u << lane) - 1u;
    for (int tile = lo; tile < hi; tile += kSortTile)
    {
        for (int w = 0; w < W; ++w) wcnt[w][t] = 0;
        __syncthreads();
        // warp `warp` owns elements [wb, wb + 32 * kSortItems) of the tile, round r holding
        // wb + 32 r + lane, so (round, lane) order is element order
        const int wb = tile + warp * 32 * kSortItems;
        uint64_t k[kSortItems];
        V v[kSortItems];
#pragma unroll
        for (int r = 0; r < kSortItems; ++r)
        {
            const int i = wb + 32 * r + lane;
            k[r] = i < hi ? kin[i] : 0;
            v[r] = i < hi ? vin[i] : V(0);
        }
        uint32_t rk[kSortItems];
#pragma unroll
        for (int r = 0; r < kSortItems; ++r)
        {
            const int i = wb + 32 * r + lane;
            const int d = i < hi ? int((k[r] >> shift) & 0xFF) : kSortRadix;
            const unsigned same = digit_peers(d);
            const uint32_t before = d < kSortRadix ? wcnt[warp][d] : 0u;
            __syncwarp();
            if (d < kSortRadix && (same & lt_mask) == 0) wcnt[warp][d] = before + uint32_t(__popc(same));
            __syncwarp();
            rk[r] = before + uint32_t(__popc(same & lt_mask));
        }
        __syncthreads();
        uint32_t cnt = 0; // this tile's count of digit t
        for (int w = 0; w < W; ++w)
        {
            const uint32_t c = wcnt[w][t];
            wcnt[w][t] = cnt;
            cnt += c;
        }
        uint32_t ts;
        block_exclusive_scan(cnt, ts);
        tstart[t] = ts;
        __syncthreads();
#pragma unroll
        for (int r = 0; r < kSortItems; ++r)
        {
            const int i = wb + 32 * r + lane;
            if (i < hi)
            {
                const int d = int((k[r] >> shift) & 0xFF);
                const uint32_t pos = tstart[d] + wcnt[warp][d] + rk[r];
                skey[pos] = k[r];
                sval[pos] = v[r];
            }
        }
        __syncthreads();
        const int tn = min(kSortTile, hi - tile);
        for (int j = t; j < tn; j += kSortThreads)
        {
            const uint64_t kk = skey[j];
            const int d = int((kk >> shift) & 0xFF);
            const uint32_t dst = base[d] + uint32_t(j) - tstart[d];
            kout[dst] = kk;
            vout[dst] = sval[j];
        }
        __syncthreads();
        base[t] += cnt;
    }
}

// The scatter's tile staging exceeds the default dynamic shared-memory limit; call once per device
// before the first sort.
template <class V> inline cudaError_t radix_sort_prepare()
{
    return cudaFuncSetAttribute(k_sort_scatter<V>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kSortSmem));
}

// Host-side launcher. Sorts [0, *n_dev) of (k0, v0) by the low `bits` bits of the key; ping-pongs
// with (k1, v1); `hist` holds kSortRadix * (nblocks + 1) counters. The first `skip_passes` passes
// (an even number, so the buffers still alternate as planned) do nothing while *skip is non-zero
// at run time: the result is then ordered by the higher digits only, stably. Returns true when the
// result ends in (k1, v1).
template <class V>
inline bool radix_sort(uint64_t *k0, V *v0, uint64_t *k1, V *v1, const int *n_dev, int bits, int nblocks,
                       uint32_t *hist, cudaStream_t st, const int *skip = nullptr, int skip_passes = 0)
{
    int passes = (bits + 7) / 8;
    if (passes < 1) passes = 1;
    uint64_t *ka = k0, *kb = k1;
    V *va = v0, *vb = v1;
    for (int p = 0; p < passes; ++p)
    {
        int shift = 8 * p;
        const int *sk = (skip && p < (skip_passes & ~1)) ? skip : nullptr;
        k_sort_hist<<<nblocks, kSortThreads, 0, st>>>(ka, n_dev, shift, hist, sk);
        k_sort_scan<<<kSortRadix, kSortThreads, 0, st>>>(hist, n_dev, nblocks, hist + size_t(kSortRadix) * nblocks, sk);
        k_sort_scatter<V><<<nblocks, kSortThreads, kSortSmem, st>>>(ka, va, kb, vb, n_dev, shift, hist,
                                                                   hist + size_t(kSortRadix) * nblocks, sk);
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
