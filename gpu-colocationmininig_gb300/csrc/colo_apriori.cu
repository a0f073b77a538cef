// colo_apriori.cu -- level-k candidate generation on the device.
//
// candidateColocationGeneral (Codes/colocationFinder.cpp:517-557) with
// generateandCheckSubsets / subsetGen / checkSubset (cpp:598-679): over the
// lexicographically ordered prevalent (k-1)-patterns P, pattern i joins each
// later pattern j with the same (k-2)-prefix and a larger last feature; the
// candidate P_i + last(P_j) is kept when all its (k-1)-subsets are prevalent.
// The reference breaks out of the j loop at the first j whose prefix differs
// (cpp:551-552) and at the first candidate with a missing subset (cpp:541-542),
// so the candidates of i are exactly j = i+1 .. i+c_i for a count c_i.
//
// One thread per pattern i counts c_i (subsets found by binary search over
// the job's sorted patterns), an exclusive scan places the rows, and a second
// pass writes them: candidates in the reference's generation order (i, then
// j), each with its prefix pattern i.  Jobs are independent: rows of the jobs
// of a batch are concatenated and a thread joins only within its own job.
#include <algorithm>
#include <vector>

#include "colo_batch.h"
#include "colo_device.cuh"

namespace colo {
namespace {

// Job of row i: last job whose first row is <= i.
__device__ __forceinline__ uint32_t job_of_row(uint64_t i, const uint64_t* __restrict__ jstart, uint32_t J) {
    uint32_t lo = 0, hi = J;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (jstart[mid] <= i) lo = mid;
        else hi = mid;
    }
    return lo;
}

// Lexicographic comparison of pattern row r (km1 features) with s.
__device__ __forceinline__ int cmp_row(const uint32_t* __restrict__ rows, uint64_t r, uint32_t km1,
                                       const uint32_t* s) {
    const uint32_t* a = rows + r * km1;
    for (uint32_t t = 0; t < km1; ++t)
        if (a[t] != s[t]) return a[t] < s[t] ? -1 : 1;
    return 0;
}

__device__ bool has_row(const uint32_t* __restrict__ rows, uint64_t lo, uint64_t hi, uint32_t km1,
                        const uint32_t* s) {
    while (lo < hi) {
        const uint64_t mid = (lo + hi) >> 1;
        const int c = cmp_row(rows, mid, km1, s);
        if (c == 0) return true;
        if (c < 0) lo = mid + 1;
        else hi = mid;
    }
    return false;
}

__global__ void k_apriori_count(const uint32_t* __restrict__ rows, uint64_t P, uint32_t km1,
                                const uint64_t* __restrict__ jstart, uint32_t J, uint32_t* __restrict__ cnt) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P) return;
    const uint32_t job = job_of_row(i, jstart, J);
    const uint64_t js = jstart[job], je = jstart[job + 1];
    const uint32_t k = km1 + 1;
    const uint32_t* pi = rows + i * km1;
    uint32_t cand[kMaxK], sub[kMaxK];
    for (uint32_t t = 0; t < km1; ++t) cand[t] = pi[t];
    uint32_t c = 0;
    for (uint64_t j = i + 1; j < je; ++j) {
        const uint32_t* pj = rows + j * km1;
        bool same = true;
        for (uint32_t t = 0; t + 1 < km1 && same; ++t) same = pi[t] == pj[t];
        if (!same || !(pi[km1 - 1] < pj[km1 - 1])) break;
        cand[km1] = pj[km1 - 1];
        // the subsets that drop positions k-3 .. 0 (dropping k-2 or k-1 gives P_j or P_i)
        bool ok = true;
        for (int drop = (int)k - 3; drop >= 0 && ok; --drop) {
            uint32_t q = 0;
            for (uint32_t t = 0; t < k; ++t)
                if ((int)t != drop) sub[q++] = cand[t];
            ok = has_row(rows, js, je, km1, sub);
        }
        if (!ok) break;
        ++c;
    }
    cnt[i] = c;
}

__global__ void k_apriori_write(const uint32_t* __restrict__ rows, uint64_t P, uint32_t km1,
                                const uint64_t* __restrict__ jstart, uint32_t J, const uint32_t* __restrict__ cnt,
                                const uint64_t* __restrict__ off, uint32_t* __restrict__ out,
                                uint32_t* __restrict__ parent) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P) return;
    const uint32_t c = cnt[i];
    if (!c) return;
    const uint32_t job = job_of_row(i, jstart, J);
    const uint32_t k = km1 + 1;
    const uint32_t* pi = rows + i * km1;
    for (uint32_t t = 0; t < c; ++t) {
        uint32_t* o = out + (off[i] + t) * k;
        for (uint32_t q = 0; q < km1; ++q) o[q] = pi[q];
        o[km1] = rows[(i + 1 + t) * km1 + km1 - 1];
        parent[off[i] + t] = (uint32_t)(i - jstart[job]);
    }
}

}  // namespace

void apriori_device(cudaStream_t s, const std::vector<const std::vector<uint32_t>*>& prev, uint32_t km1,
                    std::vector<std::vector<uint32_t>>& out, std::vector<std::vector<uint32_t>>& parent) {
    const uint32_t J = (uint32_t)prev.size();
    out.assign(J, {});
    parent.assign(J, {});
    if (km1 == 0 || km1 + 1 > (uint32_t)kMaxK) throw StatusError{COLO_ERR_CAPACITY, "patterns larger than 32 features"};
    std::vector<uint64_t> jstart(J + 1, 0);
    for (uint32_t j = 0; j < J; ++j) jstart[j + 1] = jstart[j] + (prev[j] ? prev[j]->size() / km1 : 0);
    const uint64_t P = jstart[J];
    if (P < 2) return;
    if (P >= (1ull << 32)) throw StatusError{COLO_ERR_CAPACITY, "at most 2^32-1 patterns per level"};
    std::vector<uint32_t> rows;
    rows.reserve(P * km1);
    for (uint32_t j = 0; j < J; ++j)
        if (prev[j]) rows.insert(rows.end(), prev[j]->begin(), prev[j]->end());
    DevBuf<uint32_t> drows, dcnt;
    DevBuf<uint64_t> djs, doff;
    drows.alloc(rows.size(), s);
    djs.alloc(J + 1, s);
    dcnt.alloc(P, s);
    doff.alloc(P, s);
    COLO_CUDA(cudaMemcpyAsync(drows.get(), rows.data(), rows.size() * 4, cudaMemcpyHostToDevice, s));
    COLO_CUDA(cudaMemcpyAsync(djs.get(), jstart.data(), (J + 1) * 8, cudaMemcpyHostToDevice, s));
    const unsigned grid = (unsigned)((P + 127) / 128);
    {
        KScope ks("apriori");
        k_apriori_count<<<grid, 128, 0, s>>>(drows.get(), P, km1, djs.get(), J, dcnt.get());
        COLO_LAUNCH_CHECK();
        count_launch();
    }
    uint64_t total = 0;
    scan_u32_to_u64(dcnt.get(), doff.get(), P, s, &total);
    std::vector<uint64_t> hoff(P);
    COLO_CUDA(cudaMemcpyAsync(hoff.data(), doff.get(), P * 8, cudaMemcpyDeviceToHost, s));
    if (total) {
        const uint32_t k = km1 + 1;
        DevBuf<uint32_t> dout, dpar;
        dout.alloc(total * k, s);
        dpar.alloc(total, s);
        {
            KScope ks("apriori");
            k_apriori_write<<<grid, 128, 0, s>>>(drows.get(), P, km1, djs.get(), J, dcnt.get(), doff.get(), dout.get(),
                                                 dpar.get());
            COLO_LAUNCH_CHECK();
            count_launch();
        }
        std::vector<uint32_t> hout(total * k), hpar(total);
        COLO_CUDA(cudaMemcpyAsync(hout.data(), dout.get(), hout.size() * 4, cudaMemcpyDeviceToHost, s));
        COLO_CUDA(cudaMemcpyAsync(hpar.data(), dpar.get(), hpar.size() * 4, cudaMemcpyDeviceToHost, s));
        stream_wait(s);
        for (uint32_t j = 0; j < J; ++j) {
            const uint64_t a = jstart[j] < P ? hoff[jstart[j]] : total;
            const uint64_t b = jstart[j + 1] < P ? hoff[jstart[j + 1]] : total;
            out[j].assign(hout.begin() + a * k, hout.begin() + b * k);
            parent[j].assign(hpar.begin() + a, hpar.begin() + b);
        }
    } else {
        stream_wait(s);
    }
}

}  // namespace colo
