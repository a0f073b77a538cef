// colo_prims.cu -- device-wide scan and a stable LSD radix sort (hand-written,
// no library).  The reference uses thrust::exclusive_scan / sort_by_key
// (Codes/DeviceProcess.cu:342-344); these are their replacements.
#include "colo_device.cuh"
#include "colo_internal.h"

namespace colo {

thread_local uint64_t g_launches = 0;
thread_local KTimer* g_ktimer = nullptr;

namespace {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

template <class Tin, class Tout>
__global__ void k_tile_sums(const Tin* __restrict__ in, uint64_t n, Tout* __restrict__ partial) {
    uint64_t base = (uint64_t)blockIdx.x * kScanTile + (uint64_t)threadIdx.x * kScanItems;
    Tout s = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i)
        if (base + i < n) s += (Tout)in[base + i];
    Tout tot;
    block_excl_scan<Tout>(s, &tot);
    if (threadIdx.x == 0) partial[blockIdx.x] = tot;
}

// Single block: exclusive scan of partial[0..m) in place; partial[m] = total.
template <class T>
__global__ void k_scan_partials(T* partial, uint64_t m) {
    T carry = 0;
    for (uint64_t base = 0; base < m; base += (uint64_t)blockDim.x * kScanItems) {
        uint64_t i0 = base + (uint64_t)threadIdx.x * kScanItems;
        T v[kScanItems];
        T s = 0;
#pragma unroll
        for (int i = 0; i < kScanItems; ++i) {
            v[i] = (i0 + i < m) ? partial[i0 + i] : T(0);
            s += v[i];
        }
        T tot;
        T ex = block_excl_scan<T>(s, &tot) + carry;
#pragma unroll
        for (int i = 0; i < kScanItems; ++i) {
            if (i0 + i < m) partial[i0 + i] = ex;
            ex += v[i];
        }
        carry += tot;
    }
    if (threadIdx.x == 0) partial[m] = carry;
}

template <class Tin, class Tout>
__global__ void k_scan_tiles(const Tin* __restrict__ in, Tout* __restrict__ out, uint64_t n,
                             const Tout* __restrict__ partial) {
    uint64_t base = (uint64_t)blockIdx.x * kScanTile + (uint64_t)threadIdx.x * kScanItems;
    Tout v[kScanItems];
    Tout s = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        v[i] = (base + i < n) ? (Tout)in[base + i] : Tout(0);
        s += v[i];
    }
    Tout tot;
    Tout ex = block_excl_scan<Tout>(s, &tot) + partial[blockIdx.x];
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        if (base + i < n) out[base + i] = ex;
        ex += v[i];
    }
}

__global__ void k_sum_u32(const uint32_t* __restrict__ in, uint64_t n, unsigned long long* __restrict__ out) {
    unsigned long long v = 0;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        v += in[i];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    __shared__ unsigned long long ws[32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) ws[wid] = v;
    __syncthreads();
    if (wid == 0) {
        v = lane < (int)(blockDim.x >> 5) ? ws[lane] : 0ull;
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0 && v) atomicAdd(out, v);
    }
}

template <class Tin, class Tout>
void scan_impl(const Tin* in, Tout* out, uint64_t n, cudaStream_t s, Tout* total_host) {
    KScope ks("scan");
    uint64_t tiles = (n + kScanTile - 1) / kScanTile;
    if (tiles == 0) tiles = 1;
    DevBuf<Tout> partial;
    partial.alloc(tiles + 1, s);
    if (n > 0) {
        k_tile_sums<Tin, Tout><<<(unsigned)tiles, kScanThreads, 0, s>>>(in, n, partial.get());
        COLO_LAUNCH_CHECK();
        count_launch();
    } else {
        partial.zero(s);
    }
    k_scan_partials<Tout><<<1, 1024, 0, s>>>(partial.get(), n > 0 ? tiles : 0);
    COLO_LAUNCH_CHECK();
    count_launch();
    if (n > 0) {
        k_scan_tiles<Tin, Tout><<<(unsigned)tiles, kScanThreads, 0, s>>>(in, out, n, partial.get());
        COLO_LAUNCH_CHECK();
        count_launch();
    }
    if (total_host) {
        COLO_CUDA(cudaMemcpyAsync(total_host, partial.get() + (n > 0 ? tiles : 0), sizeof(Tout),
                                  cudaMemcpyDeviceToHost, s));
        COLO_CUDA(cudaStreamSynchronize(s));
    }
}

// ---------------------------------------------------------------------------
// Radix sort
// ---------------------------------------------------------------------------

constexpr int kRadixBits = 8;
constexpr int kRadix = 1 << kRadixBits;
constexpr int kSortThreads = 256;
constexpr int kSortWarps = kSortThreads / 32;
constexpr int kSortRounds = 8;                          // items per lane
constexpr int kSortTile = kSortThreads * kSortRounds;   // 2048

template <class KT>
__global__ void k_radix_hist(const KT* __restrict__ keys, uint64_t n, int shift,
                             uint32_t* __restrict__ hist, uint32_t nblocks) {
    __shared__ uint32_t h[kRadix];
    for (int i = threadIdx.x; i < kRadix; i += blockDim.x) h[i] = 0;
    __syncthreads();
    uint64_t base = (uint64_t)blockIdx.x * kSortTile;
    for (int r = 0; r < kSortRounds; ++r) {
        uint64_t i = base + (uint64_t)r * kSortThreads + threadIdx.x;
        if (i < n) atomicAdd(&h[(uint32_t)(keys[i] >> shift) & (kRadix - 1)], 1u);
    }
    __syncthreads();
    for (int d = threadIdx.x; d < kRadix; d += blockDim.x) hist[(uint64_t)d * nblocks + blockIdx.x] = h[d];
}

// Stable scatter: items of a tile are ranked in (warp, round, lane) order,
// which is their input order.
template <class KT>
__global__ void k_radix_scatter(const KT* __restrict__ kin, const uint32_t* __restrict__ vin,
                                KT* __restrict__ kout, uint32_t* __restrict__ vout,
                                uint64_t n, int shift, const uint32_t* __restrict__ offs,
                                uint32_t nblocks) {
    __shared__ uint32_t wh[kSortWarps][kRadix];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int i = threadIdx.x; i < kSortWarps * kRadix; i += blockDim.x) (&wh[0][0])[i] = 0;
    __syncthreads();
    uint64_t base = (uint64_t)blockIdx.x * kSortTile + (uint64_t)w * (32 * kSortRounds);
    KT key[kSortRounds];
    uint32_t val[kSortRounds];
    uint32_t rank[kSortRounds];
    const uint32_t lt = (1u << lane) - 1u;
#pragma unroll
    for (int r = 0; r < kSortRounds; ++r) {
        uint64_t i = base + (uint64_t)r * 32 + lane;
        bool ok = i < n;
        key[r] = ok ? kin[i] : 0;
        val[r] = ok ? vin[i] : 0;
        uint32_t d = ok ? ((uint32_t)(key[r] >> shift) & (kRadix - 1)) : 0xFFFFu;
        uint32_t peers = __match_any_sync(0xffffffffu, d);
        int leader = __ffs(peers) - 1;
        uint32_t old = 0;
        if (ok && lane == leader) {
            old = wh[w][d];
            wh[w][d] = old + __popc(peers);
        }
        old = __shfl_sync(0xffffffffu, old, leader);
        rank[r] = ok ? old + __popc(peers & lt) : 0xFFFFFFFFu;
        __syncwarp();
    }
    __syncthreads();
    for (int d = threadIdx.x; d < kRadix; d += blockDim.x) {
        uint32_t run = 0;
        for (int ww = 0; ww < kSortWarps; ++ww) {
            uint32_t t = wh[ww][d];
            wh[ww][d] = run;
            run += t;
        }
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < kSortRounds; ++r) {
        if (rank[r] == 0xFFFFFFFFu) continue;
        uint32_t d = (uint32_t)(key[r] >> shift) & (kRadix - 1);
        uint64_t pos = (uint64_t)offs[(uint64_t)d * nblocks + blockIdx.x] + wh[w][d] + rank[r];
        kout[pos] = key[r];
        vout[pos] = val[r];
    }
}

}  // namespace

void scan_partials_u64(uint64_t* partial, uint64_t m, cudaStream_t s, uint64_t* total_host) {
    k_scan_partials<uint64_t><<<1, 1024, 0, s>>>(partial, m);
    COLO_LAUNCH_CHECK();
    count_launch();
    if (total_host) {
        COLO_CUDA(cudaMemcpyAsync(total_host, partial + m, sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
        COLO_CUDA(cudaStreamSynchronize(s));
    }
}

uint64_t sum_u32(const uint32_t* in, uint64_t n, cudaStream_t s) {
    KScope ks("sum");
    DevBuf<unsigned long long> acc;
    acc.alloc(1, s);
    acc.zero(s);
    if (n) {
        uint64_t blocks = (n + 255) / 256;
        if (blocks > 2048) blocks = 2048;
        k_sum_u32<<<(unsigned)blocks, 256, 0, s>>>(in, n, acc.get());
        COLO_LAUNCH_CHECK();
        count_launch();
    }
    unsigned long long h = 0;
    COLO_CUDA(cudaMemcpyAsync(&h, acc.get(), 8, cudaMemcpyDeviceToHost, s));
    COLO_CUDA(cudaStreamSynchronize(s));
    return h;
}

void scan_u32_to_u64(const uint32_t* in, uint64_t* out, uint64_t n, cudaStream_t s,
                     uint64_t* total_host) {
    scan_impl<uint32_t, uint64_t>(in, out, n, s, total_host);
}

void scan_u32_to_u32(const uint32_t* in, uint32_t* out, uint64_t n, cudaStream_t s,
                     uint32_t* total_host) {
    scan_impl<uint32_t, uint32_t>(in, out, n, s, total_host);
}

void scan_u64_to_u64(const uint64_t* in, uint64_t* out, uint64_t n, cudaStream_t s,
                     uint64_t* total_host) {
    scan_impl<uint64_t, uint64_t>(in, out, n, s, total_host);
}

namespace {

template <class KT>
void radix_sort_impl(KT* keys, uint32_t* vals, uint64_t n, int bits, cudaStream_t s, const char* name) {
    if (n <= 1 || bits <= 0) return;
    if (n >= (1ull << 32)) throw StatusError{COLO_ERR_CAPACITY, "radix sort supports < 2^32 items"};
    uint32_t nblocks = (uint32_t)((n + kSortTile - 1) / kSortTile);
    DevBuf<KT> k2;
    DevBuf<uint32_t> v2, hist, offs;
    k2.alloc(n, s);
    v2.alloc(n, s);
    hist.alloc((uint64_t)kRadix * nblocks, s);
    offs.alloc((uint64_t)kRadix * nblocks, s);
    KT* ka = keys;
    uint32_t* va = vals;
    KT* kb = k2.get();
    uint32_t* vb = v2.get();
    int passes = (bits + kRadixBits - 1) / kRadixBits;
    for (int p = 0; p < passes; ++p) {
        int shift = p * kRadixBits;
        KScope ks(name);
        k_radix_hist<KT><<<nblocks, kSortThreads, 0, s>>>(ka, n, shift, hist.get(), nblocks);
        COLO_LAUNCH_CHECK();
        count_launch();
        scan_u32_to_u32(hist.get(), offs.get(), (uint64_t)kRadix * nblocks, s, nullptr);
        k_radix_scatter<KT><<<nblocks, kSortThreads, 0, s>>>(ka, va, kb, vb, n, shift, offs.get(), nblocks);
        COLO_LAUNCH_CHECK();
        count_launch();
        std::swap(ka, kb);
        std::swap(va, vb);
    }
    if (ka != keys) {
        COLO_CUDA(cudaMemcpyAsync(keys, ka, n * sizeof(KT), cudaMemcpyDeviceToDevice, s));
        COLO_CUDA(cudaMemcpyAsync(vals, va, n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, s));
    }
}

}  // namespace

void radix_sort_u64_u32(uint64_t* keys, uint32_t* vals, uint64_t n, int bits, cudaStream_t s, const char* name) {
    radix_sort_impl<uint64_t>(keys, vals, n, bits, s, name);
}

void radix_sort_u32_u32(uint32_t* keys, uint32_t* vals, uint64_t n, int bits, cudaStream_t s, const char* name) {
    radix_sort_impl<uint32_t>(keys, vals, n, bits > 32 ? 32 : bits, s, name);
}

}  // namespace colo
