// ref_harness.cpp -- runs the reference's own Begin() (Codes/colocationFinder.cpp)
// on the CPU under the host execution model and records, through wrappers of
// the reference's extern "C" device API (Codes/DeviceProcess.h), every
// level's candidates, filter bounds and verdicts, row counts, participation
// window sums, PI values and instance tables.  TEST INFRASTRUCTURE: the
// output is a golden-vector JSON file.
//
// The reference's degree-2 filter kernel (filter2_2_Kernel) indexes its
// output with an uninitialised variable; this harness routes degree 2 through
// the degree>=3 filter (filter2) instead, the only behavioural change.
#include <cstdio>
#include <map>
#include <string>
#include <vector>

#include "colocationFinder.h"
#include "DeviceProcess.h"

// renamed originals (compiled from the reference's DeviceProcess.cu)
extern "C" {
StatusType colo_ref_degree2InstanceTableSlotCounter(size_t, Integer*, size_t, size_t, size_t, Integer*, Integer);
StatusType colo_ref_degree2InstanceTableGenerator(size_t, Integer*, Index64*, Integer*, size_t, size_t, Integer);
StatusType colo_ref_generalInstanceTableSlotCounter(size_t, Integer*, Integer, Integer*, Integer*, Integer*, Integer);
StatusType colo_ref_calcInstanceTableGeneral(size_t, Integer*, Index64*, Integer*, Integer, Integer*, size_t, Integer);
Real colo_ref_getParticipationIndex(Integer*&, Integer, size_t, vector<Integer>, Integer*&, Integer*&, Integer*&);
void colo_ref_filter2(int*, SInteger*, gridBox, Integer, Integer*, Real, Integer*, Integer, Integer, Integer*);
}

namespace {
struct Refined {
    unsigned long long rows = 0;
    std::vector<unsigned long long> num;
    float pi = 0;
};
struct Level {
    unsigned k = 0;
    std::vector<unsigned> cand;
    std::vector<unsigned long long> ub;
    std::vector<int> pass;
    std::map<size_t, Refined> refined;
    std::vector<std::pair<std::vector<unsigned>, std::vector<unsigned>>> tables;   // members, rows
};
std::vector<Level> g_levels;
unsigned long long g_pending_rows = 0;
std::vector<unsigned long long> g_sums;
std::vector<unsigned long long> g_pending_ub;
colocationFinder* g_finder = nullptr;

void hook_threshold(const unsigned int* countMap, unsigned int degree, unsigned int n) {
    g_pending_ub.assign(countMap, countMap + (size_t)degree * n);
}
void hook_reduce(size_t, unsigned long long s) { g_sums.push_back(s); }

unsigned long long sum_slots(const Integer* s, size_t n) {
    unsigned long long t = 0;
    for (size_t i = 0; i < n; ++i) t += s[i];
    return t;
}

unsigned feature_of(Integer id) { return g_finder->instanceList[id]; }

void record_filter(Integer* coloc, Integer n, Integer degree, Integer* countMap) {
    Level L;
    L.k = degree;
    L.cand.assign(coloc, coloc + (size_t)n * degree);
    L.ub.assign(g_pending_ub.begin(), g_pending_ub.end());
    for (Integer c = 0; c < n; ++c) L.pass.push_back(countMap[(size_t)c * degree] ? 1 : 0);
    g_levels.push_back(L);
}

void record_table(const Integer* tab, unsigned long long rows, unsigned k) {
    if (g_levels.empty()) return;
    std::vector<unsigned> members;
    std::vector<unsigned> t(tab, tab + rows * k);
    if (rows)
        for (unsigned j = 0; j < k; ++j) members.push_back(feature_of(tab[j]));
    g_levels.back().tables.push_back({members, t});
}
}  // namespace

extern "C" {
StatusType degree2InstanceTableSlotCounter(size_t maxCount, Integer* slots, size_t start, size_t end,
                                           size_t secondstart, Integer* d_bitmap, Integer combiningFeatureID) {
    StatusType st = colo_ref_degree2InstanceTableSlotCounter(maxCount, slots, start, end, secondstart, d_bitmap,
                                                              combiningFeatureID);
    g_pending_rows = sum_slots(slots, maxCount);
    return st;
}
StatusType generalInstanceTableSlotCounter(size_t n, Integer* slots, Integer degree, Integer* table1,
                                           Integer* d_bitmap, Integer* coloc, Integer lastFeatureID) {
    StatusType st = colo_ref_generalInstanceTableSlotCounter(n, slots, degree, table1, d_bitmap, coloc, lastFeatureID);
    g_pending_rows = sum_slots(slots, n);
    return st;
}
Real getParticipationIndex(Integer*& d_bitmap, Integer degree, size_t i, vector<Integer> cands,
                           Integer*& fstart, Integer*& fend, Integer*& fcount) {
    g_sums.clear();
    Real pi = colo_ref_getParticipationIndex(d_bitmap, degree, i, cands, fstart, fend, fcount);
    if (!g_levels.empty()) {
        Refined r;
        r.rows = g_pending_rows;
        r.num = g_sums;
        r.pi = pi;
        g_levels.back().refined[i] = r;
    }
    return pi;
}
StatusType degree2InstanceTableGenerator(size_t maxCount, Integer* slots, Index64* indexes, Integer* d_intermediate,
                                         size_t start, size_t end, Integer combiningFeatureID) {
    StatusType st = colo_ref_degree2InstanceTableGenerator(maxCount, slots, indexes, d_intermediate, start, end,
                                                            combiningFeatureID);
    record_table(d_intermediate, sum_slots(slots, maxCount), 2);
    return st;
}
StatusType calcInstanceTableGeneral(size_t n, Integer* slots, Index64* indexes, Integer* d_intermediate,
                                    Integer degree, Integer* table1, size_t startFrom, Integer lastFeatureID) {
    StatusType st = colo_ref_calcInstanceTableGeneral(n, slots, indexes, d_intermediate, degree, table1, startFrom,
                                                       lastFeatureID);
    record_table(d_intermediate, sum_slots(slots, n), degree);
    return st;
}
void filter2(int* isCellProcessed, SInteger* cnt, gridBox g, Integer F, Integer* fcount, Real thr, Integer* coloc,
             Integer n, Integer degree, Integer* countMap) {
    colo_ref_filter2(isCellProcessed, cnt, g, F, fcount, thr, coloc, n, degree, countMap);
    record_filter(coloc, n, degree, countMap);
}
// degree 2: the same rule as the higher levels (see the file comment)
void filter2_2(int* isCellProcessed, SInteger* cnt, gridBox g, Integer F, Integer* fcount, Real thr, Integer* coloc,
               Integer n, Integer degree, Integer* countMap) {
    filter2(isCellProcessed, cnt, g, F, fcount, thr, coloc, n, degree, countMap);
}
}

int main(int argc, char** argv) {
    if (argc < 3) {
        std::fprintf(stderr, "usage: ref_harness <config.txt> <out.json>\n");
        return 2;
    }
    colo_emu_hook_threshold = hook_threshold;
    colo_emu_hook_reduce = hook_reduce;
    g_finder = new colocationFinder();
    char* av[2] = {argv[0], argv[1]};
    g_finder->Begin(2, av);
    FILE* f = std::fopen(argv[2], "w");
    if (!f) return 1;
    std::fprintf(f, "{\"features\": [");
    for (size_t i = 0; i < g_finder->featureTypes.size(); ++i)
        std::fprintf(f, "%s\"%s\"", i ? ", " : "", g_finder->featureTypes[i].c_str());
    std::fprintf(f, "], \"levels\": [");
    for (size_t li = 0; li < g_levels.size(); ++li) {
        const Level& L = g_levels[li];
        std::fprintf(f, "%s{\"k\": %u, \"cand\": [", li ? ", " : "", L.k);
        for (size_t i = 0; i < L.cand.size(); ++i) std::fprintf(f, "%s%u", i ? ", " : "", L.cand[i]);
        std::fprintf(f, "], \"ub\": [");
        for (size_t i = 0; i < L.ub.size(); ++i) std::fprintf(f, "%s%llu", i ? ", " : "", L.ub[i]);
        std::fprintf(f, "], \"pass\": [");
        for (size_t i = 0; i < L.pass.size(); ++i) std::fprintf(f, "%s%d", i ? ", " : "", L.pass[i]);
        std::fprintf(f, "], \"refined\": {");
        bool first = true;
        for (const auto& kv : L.refined) {
            std::fprintf(f, "%s\"%zu\": {\"rows\": %llu, \"pi_bits\": %u, \"num\": [", first ? "" : ", ", kv.first,
                         kv.second.rows, *(const unsigned*)&kv.second.pi);
            for (size_t j = 0; j < kv.second.num.size(); ++j)
                std::fprintf(f, "%s%llu", j ? ", " : "", kv.second.num[j]);
            std::fprintf(f, "]}");
            first = false;
        }
        std::fprintf(f, "}, \"tables\": [");
        for (size_t t = 0; t < L.tables.size(); ++t) {
            std::fprintf(f, "%s{\"members\": [", t ? ", " : "");
            for (size_t j = 0; j < L.tables[t].first.size(); ++j)
                std::fprintf(f, "%s%u", j ? ", " : "", L.tables[t].first[j]);
            std::fprintf(f, "], \"rows\": [");
            for (size_t j = 0; j < L.tables[t].second.size(); ++j)
                std::fprintf(f, "%s%u", j ? ", " : "", L.tables[t].second[j]);
            std::fprintf(f, "]}");
        }
        std::fprintf(f, "]}");
    }
    std::fprintf(f, "]}\n");
    std::fclose(f);
    return 0;
}
