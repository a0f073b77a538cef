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
constexpr int kScanItems = 8;   // per thread in the one-block partials scan

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

// Single-pass scan (decoupled look-back): a block takes the next tile number
// from a counter, sums its 4096 items, publishes the sum, and warp 0 reads its
// predecessors' published words 32 at a time, back to the nearest inclusive
// prefix; the tile then publishes its own inclusive prefix and writes its
// items.  Tiles are numbered in the order blocks start, so a tile only waits
// on tiles whose blocks are already running.  The wait is bounded: past the
// limit the tile sums its predecessors' items itself (slow, but exact), so a
// scan never yields a wrong offset.  A warp reads its segment 32 consecutive
// items per round (coalesced loads and stores).
constexpr int kScan1Items = 16;
constexpr int kScan1Tile = kScanThreads * kScan1Items;
constexpr unsigned long long kScanA = 1ull << 62;   // tile sum published
constexpr unsigned long long kScanP = 2ull << 62;   // inclusive prefix published
constexpr unsigned long long kScanVal = (1ull << 62) - 1;
constexpr uint32_t kScanSpin = 1u << 20;

// Decoupled look-back by one full warp for tile `tile` of a single-pass scan:
// publishes the tile's sum `agg`, reads the predecessors' words 32 at a time
// back to the nearest inclusive prefix, publishes the tile's own inclusive
// prefix and returns the exclusive one.  Past the poll limit it returns false
// and publishes nothing more; the caller then computes the prefix itself and
// publishes it with lookback_publish.
__device__ __forceinline__ bool warp_lookback(unsigned long long* status, uint32_t tile, unsigned long long agg,
                                              unsigned long long& prefix) {
    const int lane = threadIdx.x & 31;
    prefix = 0;
    volatile unsigned long long* st = status + tile;
    if (tile == 0) {
        if (lane == 0) *st = kScanP | agg;
        return true;
    }
    if (lane == 0) *st = kScanA | agg;
    int64_t base = (int64_t)tile - 1;
    uint32_t spins = 0;
    while (true) {
        const int64_t t = base - lane;
        const unsigned long long sv = t >= 0 ? *(volatile const unsigned long long*)(status + t) : kScanP;
        const unsigned long long flag = sv & ~kScanVal;
        const uint32_t pm = __ballot_sync(0xffffffffu, flag == kScanP);
        const uint32_t zm = __ballot_sync(0xffffffffu, flag == 0);
        const int fp = pm ? __ffs(pm) - 1 : 32;   // nearest inclusive prefix
        const uint32_t upto = fp == 32 ? 0xffffffffu : ((2u << fp) - 1u);
        if (zm & upto) {   // a predecessor has not published yet
            if (++spins > kScanSpin) return false;
            __nanosleep(32);
            continue;
        }
        unsigned long long add = ((upto >> lane) & 1u) ? (sv & kScanVal) : 0ull;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) add += __shfl_xor_sync(0xffffffffu, add, o);
        prefix += add;
        if (fp < 32) break;
        base -= 32;
    }
    if (lane == 0) *st = kScanP | (prefix + agg);
    return true;
}

__device__ __forceinline__ void lookback_publish(unsigned long long* status, uint32_t tile, unsigned long long incl) {
    if ((threadIdx.x & 31) == 0) *(volatile unsigned long long*)(status + tile) = kScanP | incl;
}

template <class Tin, class Tout>
__global__ void __launch_bounds__(kScanThreads, 5) k_scan_1p(const Tin* __restrict__ in, Tout* __restrict__ out,
                                                          uint64_t n, unsigned long long* __restrict__ status,
                                                          uint32_t* __restrict__ ticket, Tout* __restrict__ total) {
    __shared__ uint32_t s_tile;
    __shared__ unsigned long long s_prefix;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (threadIdx.x == 0) s_tile = atomicAdd(ticket, 1u);
    __syncthreads();
    const uint32_t tile = s_tile;
    const uint64_t seg = (uint64_t)tile * kScan1Tile + (uint64_t)w * (32 * kScan1Items);
    Tin v[kScan1Items];   // kept in the input type (half the registers for 32-bit counts)
    Tout sum = 0;
#pragma unroll
    for (int i = 0; i < kScan1Items; ++i) {
        const uint64_t p = seg + (uint64_t)i * 32 + lane;
        v[i] = p < n ? in[p] : Tin(0);
        sum += (Tout)v[i];
    }
    Tout tot;
    const Tout ex_thread = block_excl_scan<Tout>(sum, &tot);
    if (w == 0) {
        unsigned long long prefix;
        if (!warp_lookback(status, tile, (unsigned long long)tot, prefix)) {   // the predecessors' items, summed here
            unsigned long long add = 0;
            for (uint64_t p = lane; p < (uint64_t)tile * kScan1Tile; p += 32) add += (unsigned long long)(Tout)in[p];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) add += __shfl_xor_sync(0xffffffffu, add, o);
            prefix = add;
            lookback_publish(status, tile, prefix + (unsigned long long)tot);
        }
        if (lane == 0) s_prefix = prefix;
    }
    __syncthreads();
    Tout carry = __shfl_sync(0xffffffffu, ex_thread, 0) + (Tout)s_prefix;
#pragma unroll
    for (int i = 0; i < kScan1Items; ++i) {
        const Tout x = (Tout)v[i];
        const Tout inc = warp_incl_scan(x);
        const uint64_t p = seg + (uint64_t)i * 32 + lane;
        if (p < n) out[p] = carry + inc - x;
        carry += __shfl_sync(0xffffffffu, inc, 31);
    }
    if (total && threadIdx.x == 0 && (uint64_t)(tile + 1) * kScan1Tile >= n) *total = (Tout)s_prefix + tot;
}

// The join's two run scans in one pass: per run r the active anchors
// act_r = rcnt[r] when the run has targets (run_L[r] > 0) and the single-pass
// layout's capacity cap_r = rcnt[r] * run_L[r] (both 0 otherwise), scanned
// exclusively, with the totals; warps 0 and 1 look back for the two scans at
// once.  Tiles of 2048 runs (two values per run in registers).  The anchors
// are listed in the same pass: the active anchors of a warp's 32 runs fill one
// contiguous range of act_pos / act_run / act_base (their sorted positions,
// runs and single-pass list starts: the run's capacity offset plus the
// anchor's index in the run times run_L), which the warp writes 32 entries at
// a time, each lane finding its entry's run by a binary search over the
// warp's inclusive counts.
constexpr int kRunItems = 8;
constexpr int kRunTile = kScanThreads * kRunItems;

// Six blocks per SM (40 registers, a few spilled): the scan waits on its look-back at the
// barrier, so more resident tiles help -- the scans of the 20M workload took 0.316 ms per
// step against 0.342 ms at four blocks (62 registers).
__global__ void __launch_bounds__(kScanThreads, 6) k_run_scans(uint64_t Rn, const uint32_t* __restrict__ rcnt,
                                                            const uint32_t* __restrict__ run_L,
                                                            const uint32_t* __restrict__ rstart,
                                                            uint32_t* __restrict__ act_pos, uint32_t* __restrict__ act_run,
                                                            uint64_t* __restrict__ act_base,
                                                            unsigned long long* __restrict__ status,
                                                            uint32_t* __restrict__ ticket, uint32_t* __restrict__ act_total,
                                                            uint64_t* __restrict__ cap_total) {
    __shared__ uint32_t s_tile;
    __shared__ unsigned long long s_prefix[2];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (threadIdx.x == 0) s_tile = atomicAdd(ticket, 1u);
    __syncthreads();
    const uint32_t tile = s_tile;
    const uint64_t ntiles = (Rn + kRunTile - 1) / kRunTile;
    unsigned long long* st_act = status;
    unsigned long long* st_cap = status + ntiles;
    const uint64_t seg = (uint64_t)tile * kRunTile + (uint64_t)w * (32 * kRunItems);
    uint32_t a[kRunItems], L[kRunItems];
    uint32_t asum = 0;
    uint64_t csum = 0;
#pragma unroll
    for (int i = 0; i < kRunItems; ++i) {
        const uint64_t p = seg + (uint64_t)i * 32 + lane;
        const uint32_t l = p < Rn ? run_L[p] : 0u;
        a[i] = l ? rcnt[p] : 0u;
        L[i] = l;
        asum += a[i];
        csum += (uint64_t)a[i] * l;
    }
    uint32_t atot;
    uint64_t ctot;
    const uint32_t aex = block_excl_scan<uint32_t>(asum, &atot);
    const uint64_t cex = block_excl_scan<uint64_t>(csum, &ctot);
    if (w < 2) {
        unsigned long long* st = w == 0 ? st_act : st_cap;
        const unsigned long long agg = w == 0 ? (unsigned long long)atot : (unsigned long long)ctot;
        unsigned long long prefix;
        if (!warp_lookback(st, tile, agg, prefix)) {   // the predecessors' runs, summed here
            unsigned long long add = 0;
            for (uint64_t p = lane; p < (uint64_t)tile * kRunTile; p += 32) {
                const uint32_t l = run_L[p];
                const uint64_t av = l ? rcnt[p] : 0u;
                add += w == 0 ? av : av * l;
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) add += __shfl_xor_sync(0xffffffffu, add, o);
            prefix = add;
            lookback_publish(st, tile, prefix + agg);
        }
        if (lane == 0) s_prefix[w] = prefix;
    }
    __syncthreads();
    uint32_t acarry = __shfl_sync(0xffffffffu, aex, 0) + (uint32_t)s_prefix[0];
    uint64_t ccarry = __shfl_sync(0xffffffffu, cex, 0) + (uint64_t)s_prefix[1];
#pragma unroll
    for (int i = 0; i < kRunItems; ++i) {
        const uint64_t cv = (uint64_t)a[i] * L[i];
        const uint32_t ainc = warp_incl_scan(a[i]);
        const uint64_t cinc = warp_incl_scan(cv);
        const uint64_t p = seg + (uint64_t)i * 32 + lane;
        const uint32_t wa = __shfl_sync(0xffffffffu, ainc, 31);   // the warp's anchors this round
        if (wa) {
            const uint32_t st = a[i] ? rstart[p] : 0u;
            const uint32_t aex = ainc - a[i];
            const uint64_t cex = ccarry + cinc - cv;
            for (uint32_t t0 = 0; t0 < wa; t0 += 32) {
                const uint32_t t = t0 + lane;
                // j = the number of runs whose inclusive count is <= t: the run of entry t
                uint32_t j = 0;
#pragma unroll
                for (uint32_t step = 16; step > 0; step >>= 1)
                    if (__shfl_sync(0xffffffffu, ainc, j + step - 1) <= t) j += step;
                const uint32_t jst = __shfl_sync(0xffffffffu, st, j);
                const uint32_t jex = __shfl_sync(0xffffffffu, aex, j);
                const uint32_t jL = __shfl_sync(0xffffffffu, L[i], j);
                const uint64_t jcex = __shfl_sync(0xffffffffu, cex, j);
                if (t < wa) {
                    act_pos[acarry + t] = jst + (t - jex);
                    act_run[acarry + t] = (uint32_t)(seg + (uint64_t)i * 32 + j);
                    act_base[acarry + t] = jcex + (uint64_t)(t - jex) * jL;
                }
            }
        }
        acarry += wa;
        ccarry += __shfl_sync(0xffffffffu, cinc, 31);
    }
    if (threadIdx.x == 0 && (uint64_t)(tile + 1) * kRunTile >= Rn) {
        *act_total = (uint32_t)s_prefix[0] + atot;
        *cap_total = (uint64_t)s_prefix[1] + ctot;
    }
}

template <class Tin, class Tout>
void scan_impl(const Tin* in, Tout* out, uint64_t n, cudaStream_t s, Tout* total_host, Tout* total_dev) {
    KScope ks("scan");
    const uint64_t tiles = n ? (n + kScan1Tile - 1) / kScan1Tile : 0;
    if (tiles >= (1ull << 32)) throw StatusError{COLO_ERR_CAPACITY, "scan supports < 2^32 tiles"};
    // status words, then the tile counter and the total: one clear
    DevBuf<unsigned long long> st;
    st.alloc(tiles + 2, s);
    st.zero(s);
    uint32_t* ticket = reinterpret_cast<uint32_t*>(st.get() + tiles);
    Tout* tot = reinterpret_cast<Tout*>(st.get() + tiles + 1);
    if (tiles) {
        k_scan_1p<Tin, Tout><<<(unsigned)tiles, kScanThreads, 0, s>>>(in, out, n, st.get(), ticket, tot);
        COLO_LAUNCH_CHECK();
        count_launch();
    }
    if (total_dev) COLO_CUDA(cudaMemcpyAsync(total_dev, tot, sizeof(Tout), cudaMemcpyDeviceToDevice, s));
    if (total_host) {
        COLO_CUDA(cudaMemcpyAsync(total_host, tot, sizeof(Tout), cudaMemcpyDeviceToHost, s));
        stream_wait(s);
    }
}

// ---------------------------------------------------------------------------
// Radix sort
// ---------------------------------------------------------------------------

constexpr int kMaxRadixBits = 8;                        // digits of at most 8 bits
static_assert((1 << kMaxRadixBits) == kRadixDigits, "digit count");
constexpr int kMaxRadix = kRadixDigits;
constexpr int kMaxPasses = kRadixMaxPasses;
// Tile shape: 512 threads of 8 items (4096-key tiles) and four resident blocks
// per SM (32 registers for 32-bit keys, a few spilled; 4 x 51 KB of shared
// memory).  A pass is bound by its look-back: each tile walks back over its
// predecessors' published counts (about 30 tiles on the 20M workload) one
// dependent load at a time, so fewer, larger tiles at the same occupancy finish
// sooner: 0.704 ms per sort against 0.763 ms for 2048-key tiles of 256 threads
// (eight blocks per SM) and 0.753 ms for 8192-key tiles of 1024 threads (two);
// 4096-key tiles of 256 threads x 16 items (three blocks per SM, 80 registers)
// were slower than either.
template <class KT>
struct SortShape {
    static constexpr int threads = 512, rounds = 8, min_blocks = 4;
};

// Shared memory of one sort block (dynamic): the tile's keys and ids (bulk-copy
// targets, 16-byte aligned), each digit's global base, the per-warp digit
// counts and each digit's tile-local start.
template <class KT, int RB>
struct SortSmem {
    static constexpr int T = SortShape<KT>::threads, W = T / 32, R = 1 << RB;
    static constexpr int tile = T * SortShape<KT>::rounds;
    static constexpr size_t key_at = 0;
    static constexpr size_t val_at = key_at + (size_t)tile * sizeof(KT);
    static constexpr size_t base_at = val_at + (size_t)tile * sizeof(uint32_t);
    static constexpr size_t wh_at = base_at + (size_t)R * sizeof(unsigned long long);
    static constexpr size_t off_at = wh_at + (size_t)W * R * sizeof(uint32_t);
    static constexpr size_t bytes = off_at + (size_t)R * sizeof(uint32_t);
    static_assert(val_at % 16 == 0 && base_at % 8 == 0, "alignment");
};


// ---------------------------------------------------------------------------
// One-sweep LSD radix sort: the digit histograms of every pass from one read
// of the keys, then one kernel per pass.  A block takes the next tile number
// from a counter, ranks its keys stably, publishes its per-digit counts, and
// looks back over the preceding tiles' published counts (a tile that has
// finished its own look-back publishes its inclusive prefix, which ends the
// walk) to place its keys.  Tiles are numbered in the order blocks start, so
// a block only waits on tiles of blocks already running.  Every wait is
// bounded: past the limit the block sets *err, uses what it has and finishes
// (the host reports COLO_ERR_TIMEOUT).  The key's bits are split evenly over
// the fewest passes of at most 8 bits (25 bits: 7 + 6 + 6 + 6): narrower
// digits leave more keys per digit in a tile, so the scatter writes longer
// runs.
// ---------------------------------------------------------------------------

constexpr unsigned long long kFlagA = 1ull << 62;   // tile count published
constexpr unsigned long long kFlagP = 2ull << 62;   // inclusive prefix published
constexpr unsigned long long kValMask = (1ull << 62) - 1;
constexpr uint32_t kSpinLimit = 1u << 22;

template <class KT>
__global__ void k_digit_hist(const KT* __restrict__ keys, uint64_t n, RadixPlan plan,
                             unsigned long long* __restrict__ ghist) {
    __shared__ uint32_t h[kMaxPasses * kMaxRadix];
    for (int i = threadIdx.x; i < plan.n * kMaxRadix; i += blockDim.x) h[i] = 0;
    __syncthreads();
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const KT k = keys[i];
        for (int p = 0; p < plan.n; ++p)
            atomicAdd(&h[p * kMaxRadix + ((uint32_t)(k >> plan.shift[p]) & ((1u << plan.width[p]) - 1u))], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < plan.n * kMaxRadix; i += blockDim.x) {
        const uint32_t v = h[i];
        if (v) atomicAdd(&ghist[i], (unsigned long long)v);
    }
}

// Exclusive scan of each pass's counters in place (one block of kMaxRadix).
__global__ void k_digit_scan(unsigned long long* __restrict__ ghist, int passes) {
    __shared__ unsigned long long sh[kMaxRadix];
    for (int p = 0; p < passes; ++p) {
        const unsigned long long v = ghist[p * kMaxRadix + threadIdx.x];
        sh[threadIdx.x] = v;
        __syncthreads();
        for (int o = 1; o < kMaxRadix; o <<= 1) {
            unsigned long long t = threadIdx.x >= (unsigned)o ? sh[threadIdx.x - o] : 0ull;
            __syncthreads();
            sh[threadIdx.x] += t;
            __syncthreads();
        }
        ghist[p * kMaxRadix + threadIdx.x] = sh[threadIdx.x] - v;
        __syncthreads();
    }
}

// Bulk (TMA engine) copy of a full tile from global to shared memory,
// completing on an mbarrier: one thread issues it, every thread waits.
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}
// dst and src 16-byte aligned, bytes a multiple of 16
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}
// Waits for phase `parity` of the barrier at most `limit` polls; false when it gave up.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint32_t limit) {
    for (uint32_t it = 0; it < limit; ++it) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
            : "=r"(done)
            : "r"(smem_addr(bar)), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// A full tile's keys and ids come into shared memory by one bulk copy each
// (bulk != 0: the host checked that both arrays are 16-byte aligned); the
// ranking reads them from there, and the same buffers then stage the tile
// in digit order.  vin == nullptr: the ids are the input positions (the first
// pass over keys in id order), generated rather than read.
template <class KT, int RB, int kSortThreads = SortShape<KT>::threads, int kSortRounds = SortShape<KT>::rounds>
__global__ void __launch_bounds__(kSortThreads, SortShape<KT>::min_blocks) k_onesweep(
    const KT* __restrict__ kin, const uint32_t* __restrict__ vin, KT* __restrict__ kout, uint32_t* __restrict__ vout,
    uint64_t n, int shift, uint32_t dmask, const unsigned long long* __restrict__ gofs,
    unsigned long long* __restrict__ status, uint32_t* __restrict__ ticket, uint32_t* __restrict__ err, int bulk,
    uint32_t spin_limit, int withhold, int pass) {
    constexpr int R = 1 << RB;
    constexpr int kSortWarps = kSortThreads / 32;
    constexpr int kSortTile = kSortThreads * kSortRounds;
    // digits per thread in the look-back (1 or 2); with more threads than digits the
    // first R threads take one each
    constexpr int D = R >= kSortThreads ? R / kSortThreads : 1;
    static_assert(R < kSortThreads || D * kSortThreads == R, "digit count");
    using SM = SortSmem<KT, RB>;
    static_assert(SM::T == kSortThreads && SM::tile == kSortTile, "shape");
    extern __shared__ __align__(16) unsigned char s_dyn[];
    KT* s_key = reinterpret_cast<KT*>(s_dyn + SM::key_at);
    uint32_t* s_val = reinterpret_cast<uint32_t*>(s_dyn + SM::val_at);
    unsigned long long* s_base = reinterpret_cast<unsigned long long*>(s_dyn + SM::base_at);  // digit's global base
    uint32_t (*wh)[R] = reinterpret_cast<uint32_t (*)[R]>(s_dyn + SM::wh_at);                 // per-warp digit counts
    uint32_t* s_off = reinterpret_cast<uint32_t*>(s_dyn + SM::off_at);                       // digit's tile-local start
    const bool owner = (int)threadIdx.x * D < R;   // this thread owns digits in the look-back
    __shared__ alignas(8) uint64_t s_bar;
    __shared__ uint32_t s_tile, s_skip;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (threadIdx.x == 0) {
        // an earlier pass that timed out left keys whose digit counts no longer match the
        // histograms, so its positions could leave the array: every later pass writes nothing
        // (the word holds the failed pass + 1; the previous launch has finished, so every
        // block of this pass reads the same value)
        const uint32_t e = *(volatile const uint32_t*)err;
        s_skip = e != 0u && e < (uint32_t)pass + 1u;
        s_tile = atomicAdd(ticket, 1u);
        if (bulk && !s_skip) mbar_init(&s_bar, 1);
    }
    for (int i = threadIdx.x; i < kSortWarps * R; i += blockDim.x) (&wh[0][0])[i] = 0;
    __syncthreads();
    if (s_skip) return;
    const uint32_t tile = s_tile;
    const uint64_t tile0 = (uint64_t)tile * kSortTile;
    const uint64_t base = tile0 + (uint64_t)w * (32 * kSortRounds);
    const bool staged = bulk && n - tile0 >= (uint64_t)kSortTile;   // full tiles only (uniform in the block)
    if (staged) {
        if (threadIdx.x == 0) {
            mbar_expect_tx(&s_bar, kSortTile * (uint32_t)(sizeof(KT) + (vin ? sizeof(uint32_t) : 0)));
            bulk_g2s(s_key, kin + tile0, kSortTile * (uint32_t)sizeof(KT), &s_bar);
            if (vin) bulk_g2s(s_val, vin + tile0, kSortTile * (uint32_t)sizeof(uint32_t), &s_bar);
        }
        const bool done = mbar_wait(&s_bar, 0, kSpinLimit);
        if (!__syncthreads_and(done ? 1 : 0)) {
            // the copy did not complete for every thread in time: report it, give it one
            // more bounded wait (it writes into this block's shared memory) and leave, the
            // whole block together; the host turns err into a timeout
            if (threadIdx.x == 0) atomicCAS(err, 0u, (uint32_t)pass + 1u);
            mbar_wait(&s_bar, 0, kSpinLimit);
            return;
        }
    }
    KT key[kSortRounds];
    uint32_t val[kSortRounds];
    uint32_t rank[kSortRounds];
    const uint32_t lt = (1u << lane) - 1u;
#pragma unroll
    for (int r = 0; r < kSortRounds; ++r) {
        const uint64_t i = base + (uint64_t)r * 32 + lane;
        const bool ok = i < n;
        const uint32_t li = (uint32_t)(i - tile0);
        key[r] = ok ? (staged ? s_key[li] : kin[i]) : 0;
        val[r] = !ok ? 0u : !vin ? (uint32_t)i : staged ? s_val[li] : vin[i];
        const uint32_t d = ok ? ((uint32_t)(key[r] >> shift) & dmask) : 0xFFFFu;
        const uint32_t peers = __match_any_sync(0xffffffffu, d);
        const int leader = __ffs(peers) - 1;
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
    {
        // thread t owns digits t*D .. t*D + D-1
        uint32_t cnt[D], sum = 0;
#pragma unroll
        for (int i = 0; i < D; ++i) {
            const int d = threadIdx.x * D + i;
            uint32_t c = 0;
            if (owner)
                for (int ww = 0; ww < kSortWarps; ++ww) {
                    const uint32_t t = wh[ww][d];
                    wh[ww][d] = c;
                    c += t;
                }
            cnt[i] = c;
            sum += c;
        }
        uint32_t tot;
        uint32_t ex = block_excl_scan<uint32_t>(sum, &tot);
        // status words and look-back for the dmask + 1 digits in use only (a tile's words
        // are kMaxRadix apart: packing them closer measured slower)
        const uint32_t nd = dmask + 1;
#pragma unroll
        for (int i = 0; i < D; ++i) {
            const int d = threadIdx.x * D + i;
            if (!owner) break;
            s_off[d] = ex;
            ex += cnt[i];
            if ((uint32_t)d >= nd) continue;
            volatile unsigned long long* st = status + (uint64_t)tile * R + d;
            unsigned long long prefix = 0;
            if (tile == 0) {
                if (!withhold) *st = kFlagP | cnt[i];   // withhold: a test of the bounded wait below
            } else {
                *st = kFlagA | cnt[i];
                uint32_t spins = 0;
                for (int64_t t = (int64_t)tile - 1; t >= 0;) {
                    const unsigned long long v = *(volatile const unsigned long long*)(status + (uint64_t)t * R + d);
                    const unsigned long long flag = v & ~kValMask;
                    if (flag == 0) {
                        if (++spins > spin_limit) {   // give up: positions from a partial prefix
                            atomicCAS(err, 0u, (uint32_t)pass + 1u);   // stay below the true ones
                            break;
                        }
                        __nanosleep(64);
                        continue;
                    }
                    prefix += v & kValMask;
                    if (flag == kFlagP) break;
                    --t;
                }
                *st = kFlagP | (prefix + cnt[i]);
            }
            s_base[d] = gofs[d] + prefix;
        }
    }
    __syncthreads();
    // stage the tile in digit order, then write it out: consecutive threads
    // write consecutive positions of one digit's range
#pragma unroll
    for (int r = 0; r < kSortRounds; ++r) {
        if (rank[r] == 0xFFFFFFFFu) continue;
        const uint32_t d = (uint32_t)(key[r] >> shift) & dmask;
        const uint32_t lp = s_off[d] + wh[w][d] + rank[r];
        s_key[lp] = key[r];
        s_val[lp] = val[r];
    }
    __syncthreads();
    const uint32_t valid = (uint32_t)(n - tile0 < (uint64_t)kSortTile ? n - tile0 : (uint64_t)kSortTile);
    for (uint32_t i = threadIdx.x; i < valid; i += kSortThreads) {
        const KT k = s_key[i];
        const uint32_t d = (uint32_t)(k >> shift) & dmask;
        const uint64_t pos = s_base[d] + (i - s_off[d]);
        kout[pos] = k;
        vout[pos] = s_val[i];
    }
}

}  // namespace

void scan_partials_u64(uint64_t* partial, uint64_t m, cudaStream_t s, uint64_t* total_host) {
    k_scan_partials<uint64_t><<<1, 1024, 0, s>>>(partial, m);
    COLO_LAUNCH_CHECK();
    count_launch();
    if (total_host) {
        COLO_CUDA(cudaMemcpyAsync(total_host, partial + m, sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
        stream_wait(s);
    }
}

void run_scans(const uint32_t* rcnt, const uint32_t* run_L, const uint32_t* rstart, uint32_t* act_pos,
               uint32_t* act_run, uint64_t* act_base, uint64_t Rn, cudaStream_t s, uint32_t* act_total,
               uint64_t* cap_total) {
    KScope ks("scan");
    const uint64_t tiles = Rn ? (Rn + kRunTile - 1) / kRunTile : 0;
    if (tiles >= (1ull << 31)) throw StatusError{COLO_ERR_CAPACITY, "scan supports < 2^31 tiles"};
    DevBuf<unsigned long long> st;   // two status words per tile, then the tile counter
    st.alloc(2 * tiles + 1, s);
    st.zero(s);
    if (!tiles) {
        COLO_CUDA(cudaMemsetAsync(act_total, 0, 4, s));
        COLO_CUDA(cudaMemsetAsync(cap_total, 0, 8, s));
        return;
    }
    k_run_scans<<<(unsigned)tiles, kScanThreads, 0, s>>>(Rn, rcnt, run_L, rstart, act_pos, act_run, act_base, st.get(),
                                                          reinterpret_cast<uint32_t*>(st.get() + 2 * tiles), act_total,
                                                          cap_total);
    COLO_LAUNCH_CHECK();
    count_launch();
}

void scan_u32_to_u64(const uint32_t* in, uint64_t* out, uint64_t n, cudaStream_t s,
                     uint64_t* total_host, uint64_t* total_dev) {
    scan_impl<uint32_t, uint64_t>(in, out, n, s, total_host, total_dev);
}

void scan_u32_to_u32(const uint32_t* in, uint32_t* out, uint64_t n, cudaStream_t s,
                     uint32_t* total_host, uint32_t* total_dev) {
    scan_impl<uint32_t, uint32_t>(in, out, n, s, total_host, total_dev);
}

void scan_u64_to_u64(const uint64_t* in, uint64_t* out, uint64_t n, cudaStream_t s,
                     uint64_t* total_host, uint64_t* total_dev) {
    scan_impl<uint64_t, uint64_t>(in, out, n, s, total_host, total_dev);
}

namespace {

template <class KT>
void radix_sort_impl(DevBuf<KT>& keys, DevBuf<uint32_t>& vals, uint64_t n, int bits, cudaStream_t s,
                     const char* name, unsigned long long* hist_in, uint32_t* err_dev, uint32_t test_spin,
                     bool iota_vals) {
    if (n <= 1 || bits <= 0) return;   // no pass: vals is left as given, iota_vals or not
    if (n >= (1ull << 32)) throw StatusError{COLO_ERR_CAPACITY, "radix sort supports < 2^32 items"};
    const RadixPlan plan = radix_plan(bits);
    using SM = SortSmem<KT, kMaxRadixBits>;
    const uint32_t ntiles = (uint32_t)((n + SM::tile - 1) / SM::tile);
    DevBuf<KT> k2;
    DevBuf<uint32_t> v2, tickets, err;
    DevBuf<unsigned long long> ghist, status;
    k2.alloc(n, s);
    v2.alloc(n, s);
    if (!hist_in) ghist.alloc((uint64_t)plan.n * kMaxRadix, s);
    unsigned long long* hist = hist_in ? hist_in : ghist.get();
    status.alloc((uint64_t)ntiles * kMaxRadix, s);
    tickets.alloc(plan.n, s);
    tickets.zero(s);
    if (!err_dev) {
        err.alloc(1, s);
        err.zero(s);
    }
    uint32_t* errp = err_dev ? err_dev : err.get();
    {
        KScope ks("radix_hist");
        if (!hist_in) {
            ghist.zero(s);
            uint64_t blocks = (n + 255) / 256;
            if (blocks > 1024) blocks = 1024;
            k_digit_hist<KT><<<(unsigned)blocks, 256, 0, s>>>(keys.get(), n, plan, hist);
            COLO_LAUNCH_CHECK();
            count_launch();
        }
        k_digit_scan<<<1, kMaxRadix, 0, s>>>(hist, plan.n);
        COLO_LAUNCH_CHECK();
        count_launch();
    }
    KT* ka = keys.get();
    uint32_t* va = vals.get();
    KT* kb = k2.get();
    uint32_t* vb = v2.get();
    // several blocks per SM: ask for the largest shared-memory carveout
    COLO_CUDA(cudaFuncSetAttribute((const void*)k_onesweep<KT, kMaxRadixBits>,
                                   cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared));
    COLO_CUDA(cudaFuncSetAttribute((const void*)k_onesweep<KT, kMaxRadixBits>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SM::bytes));
    for (int p = 0; p < plan.n; ++p) {
        KScope ks(name);   // one timed launch per digit pass
        const uint32_t dm = (1u << plan.width[p]) - 1u;
        // the words of the digits in use are cleared for every pass (a pitched clear:
        // a tile's words stay kMaxRadix apart, which spreads the polled lines over L2)
        COLO_CUDA(cudaMemset2DAsync(status.get(), kMaxRadix * 8, 0, ((size_t)1 << plan.width[p]) * 8, ntiles, s));
        const int bulk = ((uintptr_t)ka % 16 == 0 && (uintptr_t)va % 16 == 0) ? 1 : 0;
        // the first pass of a sort of positions generates them (no read)
        const uint32_t* vin = (iota_vals && p == 0) ? nullptr : va;
        k_onesweep<KT, kMaxRadixBits><<<ntiles, SM::T, SM::bytes, s>>>(ka, vin, kb, vb, n, plan.shift[p], dm,
                                                                     hist + p * kMaxRadix, status.get(),
                                                                     tickets.get() + p, errp, bulk,
                                                                     test_spin ? test_spin : kSpinLimit,
                                                                     test_spin && p == 0 ? 1 : 0, p);
        COLO_LAUNCH_CHECK();
        count_launch();
        std::swap(ka, kb);
        std::swap(va, vb);
    }
    if (ka != keys.get()) {   // an odd number of passes: the result is in the second buffers
        keys.swap(k2);
        vals.swap(v2);
    }
    // the caller reads the error word at its next wait; until then its kernels read the
    // output with ids checked against n (a timed-out pass leaves ids unwritten)
    if (err_dev) return;
    uint32_t herr = 0;
    COLO_CUDA(cudaMemcpyAsync(&herr, err.get(), 4, cudaMemcpyDeviceToHost, s));
    stream_wait(s);
    if (herr) throw StatusError{COLO_ERR_TIMEOUT, "radix sort: a tile waited too long for its predecessors"};
}

}  // namespace

RadixPlan radix_plan(int bits) {
    // fewest passes of at most 8 bits, widths as even as possible (25 bits: 7 + 6 + 6 + 6)
    RadixPlan plan{};
    if (bits <= 0) return plan;
    plan.n = (bits + kMaxRadixBits - 1) / kMaxRadixBits;
    for (int p = 0, sh = 0; p < plan.n; ++p) {
        plan.width[p] = bits / plan.n + (p < bits % plan.n ? 1 : 0);
        plan.shift[p] = sh;
        sh += plan.width[p];
    }
    return plan;
}

void radix_sort(DevBuf<uint64_t>& keys, DevBuf<uint32_t>& vals, uint64_t n, int bits, cudaStream_t s,
                const char* name, unsigned long long* hist, uint32_t* err_dev, uint32_t test_spin, bool iota_vals) {
    radix_sort_impl<uint64_t>(keys, vals, n, bits, s, name, hist, err_dev, test_spin, iota_vals);
}

void radix_sort(DevBuf<uint32_t>& keys, DevBuf<uint32_t>& vals, uint64_t n, int bits, cudaStream_t s,
                const char* name, unsigned long long* hist, uint32_t* err_dev, uint32_t test_spin, bool iota_vals) {
    radix_sort_impl<uint32_t>(keys, vals, n, bits > 32 ? 32 : bits, s, name, hist, err_dev, test_spin, iota_vals);
}

}  // namespace colo
