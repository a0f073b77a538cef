// colo_static.cu -- colo_table_pi_static: the participation index of one
// candidate from an instance table already in device memory, computed with
// no device allocation.
//
// Who needs it: hosts that own all of a GPU's memory through their own pool
// (a database or GIS server that reserves the device memory at start-up and
// hands out sub-buffers) cannot let a library call cudaMalloc behind their
// back -- the call fails once the pool holds the memory, or breaks the pool's
// accounting -- and latency-bound services cannot accept cudaFree, which
// synchronises the whole device.  Such callers pass device buffers for the
// inputs and outputs; the only other device memory used is the file-scope
// scratch array below.
//
// The scratch array (kCtrlWords + COLO_TABLE_PI_STATIC_WORDS 32-bit words,
// about 4 MiB) is part of this library's device code: every GPU on which the
// library's kernels are loaded holds it until the process exits.  All calls
// share it and it keeps the last call's contents, so each call clears the
// words it uses before use, and calls whose kernels overlap on the GPU (on
// different streams, or from different host threads without ordering) race
// on it and give wrong results.
//
// The computation is that of k_level_pi in colo_level.cu (the reference's
// getParticipationIndex window sums, Codes/DeviceProcess.cu:108-132), with the
// participation bitmaps built here from the table columns instead of by the
// level kernels.
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>

#include "colo.h"

namespace {

constexpr uint32_t kMaxMembers = 32;
constexpr uint32_t kCtrlWords = 512;   // [0] invalid ids, [1] block ticket, u64 stats from word 256
constexpr uint32_t kStatsWord = 256;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) uint32_t g_table_pi_scratch[kCtrlWords + COLO_TABLE_PI_STATIC_WORDS];

struct Members {
    uint32_t k;
    uint32_t fstart[kMaxMembers];
    uint32_t fcount[kMaxMembers];
    uint32_t bm_off[kMaxMembers];   // word offset of member j's bitmap after the control words
};

__global__ void k_static_clear(uint32_t* __restrict__ w, uint64_t nwords) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nwords;
         i += (uint64_t)gridDim.x * blockDim.x)
        w[i] = 0u;
}

// One entry of the row-major table per thread step: set the member's bit.
// An id outside the member's instance range is not written; it raises the
// invalid flag (a flag, not a count, so no number of bad ids can wrap it).
__global__ void k_static_mark(const uint32_t* __restrict__ table, uint64_t entries, Members m,
                              uint32_t* __restrict__ scratch) {
    uint32_t* bits = scratch + kCtrlWords;
    uint32_t bad = 0;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < entries;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t j = (uint32_t)(i % m.k);
        const uint32_t local = table[i] - m.fstart[j];
        if (local >= m.fcount[j]) {
            ++bad;
            continue;
        }
        atomicOr(&bits[m.bm_off[j] + (local >> 5)], 1u << (local & 31));
    }
    if (bad) atomicOr(&scratch[0], 1u);
}

// Block j counts member j's bitmap: A = bits in [0, n-2], last = bit n-1,
// first = bit 0, full = all bits.  The last block to finish combines the
// members into the numerators and the PI exactly as the mining loop does.
__global__ void __launch_bounds__(1024) k_static_pi(Members m, uint32_t* __restrict__ scratch,
                                                    unsigned long long* __restrict__ num, float* __restrict__ pi) {
    const uint32_t j = blockIdx.x;
    const uint32_t n = m.fcount[j];
    const uint32_t* w = scratch + kCtrlWords + m.bm_off[j];
    unsigned long long* stats = reinterpret_cast<unsigned long long*>(scratch + kStatsWord);
    __shared__ unsigned long long red[32];
    __shared__ bool is_last;
    const uint32_t nw = (n + 31) / 32, lim = n - 1;
    unsigned long long cA = 0, cF = 0;
    for (uint32_t i = threadIdx.x; i < nw; i += blockDim.x) {
        const uint32_t v = w[i], wb = i * 32;
        const uint32_t mask = wb + 32 <= lim ? 0xffffffffu : (wb >= lim ? 0u : (1u << (lim - wb)) - 1u);
        cF += __popc(v);
        cA += __popc(v & mask);
    }
    for (int o = 16; o > 0; o >>= 1) {
        cA += __shfl_down_sync(0xffffffffu, cA, o);
        cF += __shfl_down_sync(0xffffffffu, cF, o);
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) red[wid] = cA | (cF << 32);
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long A = 0, Fu = 0;
        for (int q = 0; q < (int)(blockDim.x >> 5); ++q) {
            A += red[q] & 0xffffffffull;
            Fu += red[q] >> 32;
        }
        stats[j * 4 + 0] = A;
        stats[j * 4 + 1] = (w[(n - 1) >> 5] >> ((n - 1) & 31)) & 1u;
        stats[j * 4 + 2] = w[0] & 1u;
        stats[j * 4 + 3] = Fu;
        __threadfence();
        is_last = atomicAdd(&scratch[1], 1u) == m.k - 1;
    }
    __syncthreads();
    if (!is_last || threadIdx.x != 0) return;
    __threadfence();
    const volatile unsigned long long* st = stats;
    const bool invalid = *(volatile uint32_t*)&scratch[0] != 0;
    float PI = 1.0f;
    for (uint32_t t = 0; t < m.k; ++t) {
        unsigned long long v;
        if (m.k == 2)
            v = t == 0 ? st[0] : (st[4 + 3] - st[4 + 2]) + ((st[4 + 2] | st[1]) ? 1ull : 0ull);
        else
            v = t == 0 ? st[0] : st[(t - 1) * 4 + 1] + st[t * 4 + 0];
        num[t] = invalid ? ~0ull : v;
        const float pr = (float)v / (float)m.fcount[t];
        if (pr < PI) PI = pr;
    }
    if (pi) *pi = invalid ? __int_as_float(0x7fc00000) : PI;
}

std::mutex g_setup_mu;
uint32_t* g_scratch_ptr[kMaxDevices] = {};

// Device address of the scratch array on the current device, looked up once
// per device (cudaGetSymbolAddress; the symbol's host-side name is only a
// handle, never a device address).  The address is cached for the life of
// the process: a cudaDeviceReset of that device after its first call would
// leave it dangling, which is why the header rules out calls after a reset.
colo_status scratch_for_current_device(uint32_t** out) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) return COLO_ERR_NO_DEVICE;
    if (dev >= kMaxDevices) return COLO_ERR_ARG;
    std::lock_guard<std::mutex> lk(g_setup_mu);
    if (!g_scratch_ptr[dev]) {
        uint32_t* p = nullptr;
        if (cudaGetSymbolAddress((void**)&p, g_table_pi_scratch) != cudaSuccess || !p) return COLO_ERR_CUDA;
        g_scratch_ptr[dev] = p;
    }
    *out = g_scratch_ptr[dev];
    return COLO_OK;
}

}  // namespace

extern "C" colo_status colo_table_pi_static(const uint32_t* table, uint64_t rows, uint32_t k, const uint32_t* fstart,
                                            const uint32_t* fcount, uint64_t* num, float* pi, void* stream) {
    if (k < 2 || k > kMaxMembers || !fstart || !fcount || !num || (rows && !table)) return COLO_ERR_ARG;
    if (rows > UINT64_MAX / k) return COLO_ERR_ARG;
    Members m{};
    m.k = k;
    uint64_t words = 0;
    for (uint32_t j = 0; j < k; ++j) {
        if (fcount[j] == 0 || (uint64_t)fstart[j] + fcount[j] > 0x100000000ull) return COLO_ERR_ARG;
        m.fstart[j] = fstart[j];
        m.fcount[j] = fcount[j];
        m.bm_off[j] = (uint32_t)words;
        words += (fcount[j] + 31u) / 32u;
        if (words > COLO_TABLE_PI_STATIC_WORDS) return COLO_ERR_CAPACITY;
    }
    uint32_t* scratch = nullptr;
    colo_status st;
    try {
        st = scratch_for_current_device(&scratch);
    } catch (...) {
        return COLO_ERR_INTERNAL;
    }
    if (st != COLO_OK) return st;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const uint64_t clear = kCtrlWords + words;
    k_static_clear<<<(unsigned)((clear + 1023) / 1024 < 1024 ? (clear + 1023) / 1024 : 1024), 1024, 0, s>>>(scratch,
                                                                                                          clear);
    if (cudaGetLastError() != cudaSuccess) return COLO_ERR_CUDA;
    const uint64_t entries = rows * k;
    if (entries) {
        uint64_t blocks = (entries + 255) / 256;
        if (blocks > 4096) blocks = 4096;
        k_static_mark<<<(unsigned)blocks, 256, 0, s>>>(table, entries, m, scratch);
        if (cudaGetLastError() != cudaSuccess) return COLO_ERR_CUDA;
    }
    k_static_pi<<<k, 1024, 0, s>>>(m, scratch, reinterpret_cast<unsigned long long*>(num), pi);
    if (cudaGetLastError() != cudaSuccess) return COLO_ERR_CUDA;
    return COLO_OK;
}
