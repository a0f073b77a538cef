// colo_internal.h -- shared types of libcolo (device layout, launch helpers).
//
// Device layout of one mining batch (one or more independent jobs):
//   points      x[N], y[N] f32, feat[N] u32 (global feature index; features of
//               a job are contiguous and a job's points are contiguous); xy[N]
//               packed coordinates by id
//   features    fstart[F], fcount[F], fjob[F]
//   jobs        JobGrid[J] (the reference grid of each job, R^2, threshold)
//   bucketed    points sorted by (job cell key, point id): sid/sxy/sfeat/scell
//   cells       occupied cells ckey[M], cstart[M+1] (sorted positions),
//               crun[M+1] (run ranges), nb9[M*9] (geometric 3x3 neighbours),
//               cmask[M*W] (feature bit masks, local feature index),
//               qmask[M*4*W] (masks of the 4 quads containing the cell)
//   runs        (cell, feature) runs rfeat/rstart/rcnt/rcell[Rn], cell-major;
//               runs per feature on the host (h_frun_off prefix)
//   NRL         per cell, the runs of its adjacent cells with a feature above
//               the cell's lowest own feature, ordered by (feature, cell):
//               nrl_off[M+1], nrl_ent (start, count); per run the start of its
//               higher-feature suffix run_sfx and its size run_L
//   neighbours  N+(a) = nb[nb_beg[a] .. nb_beg[a] + nb_cnt[a]) by point id
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <chrono>
#include <string>
#include <vector>

#include "colo.h"

namespace colo {

constexpr int kMaxK = 32;          // largest pattern size handled by the level kernels
constexpr int kMaxMembersFiltered = 8;  // filter counts members j < 8 (block (8,2,2) in the reference)

struct JobGrid {
    float min_x, min_y, w;       // grid origin and cell width (= R)
    float R2;                    // R*R in float
    float R2hu;                  // half an ulp of R2 (the rounding gap above R2)
    float thr;                   // PI threshold
    uint32_t gx, gy;
    uint64_t total;              // gx*gy
    uint64_t key_base;           // first cell key of this job in the batch
    uint64_t row_base;           // first grid row of this job in the batch's row table
    int32_t compat32;            // 32-bit reference cell arithmetic is exact
    uint32_t f0, nf;             // global feature range of the job
};

// Error carrier for kernels: bounded waits and range checks record here.
struct DevFlags {
    uint32_t out_of_grid;        // points whose cell is outside [0, total)
    uint32_t overflow;           // capacity overflows (learned presize)
    uint32_t timeout;            // a bounded wait gave up (the sort stores its failed pass + 1)
    uint32_t internal;           // consistency checks
};

__host__ __device__ inline uint32_t ceil_div_u32(uint64_t a, uint64_t b) {
    return (uint32_t)((a + b - 1) / b);
}

// ---------------------------------------------------------------------------
// Host-side helpers
// ---------------------------------------------------------------------------

struct CudaError {
    cudaError_t err;
    std::string where;
};

#define COLO_CUDA(call)                                                          \
    do {                                                                         \
        cudaError_t e__ = (call);                                                \
        if (e__ != cudaSuccess) throw ::colo::CudaError{e__, std::string(#call) + " @ " + __FILE__ + ":" + std::to_string(__LINE__)}; \
    } while (0)

#define COLO_LAUNCH_CHECK()                                                      \
    do {                                                                         \
        cudaError_t e__ = cudaGetLastError();                                    \
        if (e__ != cudaSuccess) throw ::colo::CudaError{e__, std::string("kernel launch @ ") + __FILE__ + ":" + std::to_string(__LINE__)}; \
    } while (0)

struct StatusError {
    colo_status st;
    std::string msg;
};

// Stream-ordered device buffer (cudaMallocAsync / cudaFreeAsync).
template <class T>
struct DevBuf {
    T* p = nullptr;
    size_t n = 0;
    cudaStream_t s = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    DevBuf(DevBuf&& o) noexcept { swap(o); }
    DevBuf& operator=(DevBuf&& o) noexcept { release(); swap(o); return *this; }
    ~DevBuf() { release(); }
    void swap(DevBuf& o) { std::swap(p, o.p); std::swap(n, o.n); std::swap(s, o.s); }
    void alloc(size_t count, cudaStream_t st) {
        release();
        s = st;
        n = count;
        if (count == 0) return;
        cudaError_t e = cudaMallocAsync((void**)&p, count * sizeof(T), st);
        if (e != cudaSuccess) {
            p = nullptr;
            n = 0;
            cudaGetLastError();
            throw StatusError{COLO_ERR_NOMEM, "device allocation of " + std::to_string(count * sizeof(T)) + " bytes failed"};
        }
    }
    void zero(cudaStream_t st) {
        if (n) COLO_CUDA(cudaMemsetAsync(p, 0, n * sizeof(T), st));
    }
    void release() {
        if (p) cudaFreeAsync(p, s);
        p = nullptr;
        n = 0;
    }
    T* get() const { return p; }
    size_t bytes() const { return n * sizeof(T); }
};

// Instance-table storage: device memory, or pinned host memory mapped into
// the device's address space when asked for or when the device allocation
// fails (on Grace the kernels then read and write them over NVLink-C2C).
struct TableBuf {
    DevBuf<uint32_t> dev;
    void* host = nullptr;
    uint32_t* p = nullptr;
    size_t n = 0;
    cudaStream_t s = 0;
    TableBuf() = default;
    TableBuf(const TableBuf&) = delete;
    TableBuf& operator=(const TableBuf&) = delete;
    void alloc(size_t count, cudaStream_t st, bool on_host) {
        release();
        s = st;
        n = count;
        if (!on_host) {
            try {
                dev.alloc(count, st);
                p = dev.get();
                return;
            } catch (const StatusError& e) {
                if (e.st != COLO_ERR_NOMEM) throw;
            }
        }
        if (cudaHostAlloc(&host, (count ? count : 1) * sizeof(uint32_t), cudaHostAllocMapped) != cudaSuccess) {
            host = nullptr;
            cudaGetLastError();
            throw StatusError{COLO_ERR_NOMEM, "pinned host allocation of " + std::to_string(count * 4) +
                                                  " bytes for instance tables failed"};
        }
        void* d = nullptr;
        COLO_CUDA(cudaHostGetDevicePointer(&d, host, 0));
        p = static_cast<uint32_t*>(d);
    }
    void release() {
        if (host) {
            cudaStreamSynchronize(s);   // kernels of this stream may still use the tables
            cudaFreeHost(host);
            host = nullptr;
        }
        dev.release();
        p = nullptr;
        n = 0;
    }
    ~TableBuf() { release(); }
    uint32_t* get() const { return p; }
    bool on_host() const { return host != nullptr; }
};

// Launch counter (kernels of this library launched by the current mine).
extern thread_local uint64_t g_launches;
inline void count_launch(uint64_t n = 1) { g_launches += n; }

// Optional per-kernel CUDA-event timing on the launching stream (enabled per
// mine; used by the benchmark for its roofline figures).
struct KernelStat {
    std::string name;
    uint64_t launches = 0;
    double ms = 0;
};

struct KTimer {
    bool on = false;
    cudaStream_t s = 0;
    struct Pending {
        int slot;
        cudaEvent_t a, b;
    };
    std::vector<Pending> pend;
    std::vector<KernelStat> stats;
    std::vector<cudaEvent_t> pool;
    int open_slot = -1;
    int depth = 0;                  // nested scopes: the outermost one is timed
    cudaEvent_t open_a = nullptr;
    cudaEvent_t get() {
        if (!pool.empty()) {
            cudaEvent_t e = pool.back();
            pool.pop_back();
            return e;
        }
        cudaEvent_t e;
        COLO_CUDA(cudaEventCreate(&e));
        return e;
    }
    int slot(const char* name) {
        for (size_t i = 0; i < stats.size(); ++i)
            if (stats[i].name == name) return (int)i;
        stats.push_back(KernelStat{name, 0, 0});
        return (int)stats.size() - 1;
    }
    // Host time from the last wait's return to the next timed launch, charged to
    // "host <scope>": the part of a gap that the host spends preparing the launch.
    std::chrono::steady_clock::time_point waited{};
    bool after_wait = false;
    void note_wait() {
        if (!on) return;
        waited = std::chrono::steady_clock::now();
        after_wait = true;
    }
    // Host time between two marks of the level loop, charged to "part <name>"
    // (profile mode): where the host spends the time between a wait and a launch.
    std::chrono::steady_clock::time_point marked{};
    void mark(const char* name) {
        if (!on) return;
        const auto now = std::chrono::steady_clock::now();
        if (marked.time_since_epoch().count()) {
            KernelStat& h = stats[slot((std::string("part ") + name).c_str())];
            h.ms += std::chrono::duration<double, std::milli>(now - marked).count();
            h.launches++;
        }
        marked = now;
    }
    void begin(const char* name) {
        if (!on || depth++ > 0) return;
        if (after_wait) {
            const double ms =
                std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - waited).count();
            KernelStat& h = stats[slot((std::string("host ") + name).c_str())];
            h.ms += ms;
            h.launches++;
            after_wait = false;
        }
        open_slot = slot(name);
        open_a = get();
        COLO_CUDA(cudaEventRecord(open_a, s));
    }
    void end() {
        if (!on || --depth > 0 || open_slot < 0) return;
        cudaEvent_t b = get();
        COLO_CUDA(cudaEventRecord(b, s));
        pend.push_back({open_slot, open_a, b});
        open_slot = -1;
    }
    // Stream time between the end of one timed scope and the start of the next,
    // charged to "gap <next scope>": the GPU waiting for the host (a wait and
    // the launches after it) plus any untimed copy or clear between them.
    cudaEvent_t last_b = nullptr;
    void resolve() {
        if (pend.empty()) return;
        COLO_CUDA(cudaStreamSynchronize(s));
        for (auto& p : pend) {
            float ms = 0;
            COLO_CUDA(cudaEventElapsedTime(&ms, p.a, p.b));
            stats[p.slot].ms += ms;
            stats[p.slot].launches++;
            if (last_b) {
                float gap = 0;
                COLO_CUDA(cudaEventElapsedTime(&gap, last_b, p.a));
                KernelStat& g = stats[slot(("gap " + stats[p.slot].name).c_str())];
                g.ms += gap;
                g.launches++;
                pool.push_back(last_b);
            }
            pool.push_back(p.a);
            last_b = p.b;
        }
        pend.clear();
    }
    ~KTimer() {
        for (auto& p : pend) {
            cudaEventDestroy(p.a);
            cudaEventDestroy(p.b);
        }
        if (last_b) cudaEventDestroy(last_b);
        for (auto e : pool) cudaEventDestroy(e);
    }
};
extern thread_local KTimer* g_ktimer;

// A host wait on the stream (noted by the kernel timer in profile mode).
inline void stream_wait(cudaStream_t s) {
    COLO_CUDA(cudaStreamSynchronize(s));
    if (g_ktimer) g_ktimer->note_wait();
}
struct KScope {
    explicit KScope(const char* name) {
        if (g_ktimer) g_ktimer->begin(name);
    }
    ~KScope() {
        if (g_ktimer) g_ktimer->end();
    }
};

// ---------------------------------------------------------------------------
// Primitives (colo_prims.cu)
// ---------------------------------------------------------------------------

// In place: exclusive scan of partial[0..m), partial[m] = total (read back
// when total_host != nullptr).
void scan_partials_u64(uint64_t* partial, uint64_t m, cudaStream_t s, uint64_t* total_host);
// out[i] = sum(in[0..i)).  The total is read back (with a wait) when
// total_host is given, and copied to device memory (no wait) when total_dev is.
void scan_u32_to_u64(const uint32_t* in, uint64_t* out, uint64_t n, cudaStream_t s,
                     uint64_t* total_host, uint64_t* total_dev = nullptr);
void scan_u32_to_u32(const uint32_t* in, uint32_t* out, uint64_t n, cudaStream_t s,
                     uint32_t* total_host, uint32_t* total_dev = nullptr);
void scan_u64_to_u64(const uint64_t* in, uint64_t* out, uint64_t n, cudaStream_t s,
                     uint64_t* total_host, uint64_t* total_dev = nullptr);
// The join's run scans in one pass: act_r = rcnt[r] if run_L[r] > 0 else 0 and
// cap_r = act_r * run_L[r].  The active anchors are listed in run order:
// act_pos (sorted positions rstart[r] .. rstart[r] + act_r - 1), act_run (r)
// and act_base (the exclusive scan of cap over the runs before r, plus the
// anchor's index in its run times run_L[r]: its list start in the single-pass
// layout); they need room for the sum of act_r.  The totals (sum of act_r,
// sum of cap_r) land in device memory (no wait).
void run_scans(const uint32_t* rcnt, const uint32_t* run_L, const uint32_t* rstart, uint32_t* act_pos,
               uint32_t* act_run, uint64_t* act_base, uint64_t Rn, cudaStream_t s, uint32_t* act_total,
               uint64_t* cap_total);
// Digit split of a radix sort: pass p sorts width[p] (<= 8) bits from shift[p].
constexpr int kRadixDigits = 256;
constexpr int kRadixMaxPasses = 8;
struct RadixPlan {
    int n;
    int shift[kRadixMaxPasses];
    int width[kRadixMaxPasses];
};
RadixPlan radix_plan(int bits);
// Stable LSD radix sort of (key, val) pairs by the low `bits` bits of key.
// The sorted pairs are in keys/vals on return (the buffers may have been
// exchanged for the sort's second buffers, which avoids a copy back).
// hist, when given, holds every pass's digit counts of the keys
// (hist[p * kRadixDigits + d], radix_plan(bits) passes), counted by the
// caller while it wrote the keys; the sort then skips its own count.
// err_dev, when given, receives the timeout flag of a look-back wait (the
// caller checks it at its next wait); otherwise the sort waits and throws.
// test_spin != 0 (tests of the timeout path only): the look-back gives up
// after test_spin polls, and in the first pass tile 0 withholds its counts,
// so tile 1's wait runs out; every wait stays bounded and the sort ends with
// the timeout flag set (its output is discarded by the caller).
// iota_vals: the values are the positions 0 .. n-1, which the first pass
// generates instead of reading (vals must still hold n items).  With no pass
// (n <= 1 or bits <= 0) vals is left as given, so the caller writes them then.
void radix_sort(DevBuf<uint64_t>& keys, DevBuf<uint32_t>& vals, uint64_t n, int bits, cudaStream_t s,
                const char* name = "radix_sort", unsigned long long* hist = nullptr, uint32_t* err_dev = nullptr,
                uint32_t test_spin = 0, bool iota_vals = false);
void radix_sort(DevBuf<uint32_t>& keys, DevBuf<uint32_t>& vals, uint64_t n, int bits, cudaStream_t s,
                const char* name = "radix_sort", unsigned long long* hist = nullptr, uint32_t* err_dev = nullptr,
                uint32_t test_spin = 0, bool iota_vals = false);

}  // namespace colo
