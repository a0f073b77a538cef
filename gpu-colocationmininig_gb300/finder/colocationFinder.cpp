// colocationFinder.cpp -- drop-in front end over libcolo's C ABI.
#include "colocationFinder.h"

#include <chrono>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>

namespace {
using Clock = std::chrono::steady_clock;
double ms_since(Clock::time_point t) { return std::chrono::duration<double, std::milli>(Clock::now() - t).count(); }
}  // namespace

colocationFinder::colocationFinder(void) {
    colo_params_default(&params_);
    params_.mode = COLO_MODE_BATCHED;
    status = colo_create(&ctx_, 0);
    if (status != COLO_OK) error = colo_status_string(status);
}

colocationFinder::~colocationFinder(void) {
    if (res_) colo_result_free(res_);
    if (ds_) colo_dataset_free(ds_);
    if (ctx_) colo_destroy(ctx_);
}

void colocationFinder::LoadParameter(std::string parameterFileName) {
    colo_params p = params_;
    colo_status st = colo_read_params(parameterFileName.c_str(), &p);
    if (st != COLO_OK) {
        status = st;
        error = "Parameter file missing...";
        return;
    }
    params_.distance = p.distance;
    params_.pi_threshold = p.pi_threshold;
    params_.filter_flag = p.filter_flag;
}

void colocationFinder::populateData(std::string datasetFilename) {
    if (!ctx_) return;
    auto t0 = Clock::now();
    dataset_ = datasetFilename;
    if (ds_) colo_dataset_free(ds_);
    ds_ = nullptr;
    // A dataset named *.colo is a binary point file (colo_csv_to_binary); any
    // other name is the reference's CSV.
    const bool binary = datasetFilename.size() > 5 &&
                        datasetFilename.compare(datasetFilename.size() - 5, 5, ".colo") == 0;
    status = binary ? colo_dataset_from_binary(ctx_, datasetFilename.c_str(), &ds_)
                    : colo_dataset_from_csv(ctx_, datasetFilename.c_str(), &ds_);
    if (status != COLO_OK) {
        error = colo_last_error(ctx_);
        return;
    }
    featureTypes.clear();
    for (uint32_t f = 0; f < colo_dataset_num_features(ds_); ++f) featureTypes.push_back(colo_dataset_feature_name(ds_, f));
    ioMs_ = ms_since(t0);
    if (res_) colo_result_free(res_);
    res_ = nullptr;
}

void colocationFinder::ensureMined() {
    if (res_ || !ctx_ || !ds_ || status != COLO_OK) return;
    status = colo_mine(ctx_, ds_, &params_, &res_);
    if (status != COLO_OK) error = colo_last_error(ctx_);
}

void colocationFinder::selectLevel(Integer degree) {
    ensureMined();
    h_candiColocations.clear();
    h_prevalantColocations.clear();
    candiColocCounter = 0;
    h_prevelentColocationCount = 0;
    if (!res_) return;
    for (uint32_t li = 0; li < colo_result_num_levels(res_); ++li) {
        if (colo_result_level_size(res_, li) != degree) continue;
        uint64_t n = colo_result_level_candidates(res_, li);
        std::vector<uint32_t> cand(n * degree);
        std::vector<uint8_t> prev(n);
        colo_result_level(res_, li, cand.data(), nullptr, nullptr, nullptr, nullptr, nullptr, prev.data(), nullptr);
        candiColocCounter = (Integer)n;
        h_candiColocations.assign(cand.begin(), cand.end());
        for (uint64_t c = 0; c < n; ++c)
            if (prev[c]) {
                h_prevalantColocations.insert(h_prevalantColocations.end(), cand.begin() + c * degree,
                                              cand.begin() + (c + 1) * degree);
                h_prevelentColocationCount++;
            }
    }
}

void colocationFinder::degree2Processing() { selectLevel(2); }
void colocationFinder::generatePrevalentPatternsGeneral(Integer degree) { selectLevel(degree); }
void colocationFinder::generateInstanceTableGeneral(Integer degree) { selectLevel(degree); }
void colocationFinder::candidateColocationGeneral(Integer degree) { selectLevel(degree); }

void colocationFinder::savetoFileGen(Integer) {
    ensureMined();
    if (res_ && ds_) colo_result_write_patterns(res_, ds_, location_.c_str());
}

int colocationFinder::Begin(Integer argc, char** argv) {
    auto t_all = Clock::now();
    if (argc <= 1) {
        std::cout << "Configuration file missing...";
        return 1;
    }
    if (!ctx_) {
        std::cerr << "There is no device supporting CUDA (" << error << ")\n";
        return 1;
    }
    char lines[5][4096];
    status = colo_read_config(argv[1], lines[0], lines[1], lines[2], lines[3], lines[4], sizeof(lines[0]));
    if (status != COLO_OK) {
        std::cerr << "cannot read configuration file " << argv[1] << "\n";
        return 1;
    }
    location_ = lines[0];
    outputLocation_ = lines[3];
    outputFile_ = lines[4];
    LoadParameter(lines[1]);
    if (status != COLO_OK) {
        std::cout << error << std::endl;
        return 1;
    }
    populateData(lines[2]);
    if (status != COLO_OK) {
        std::cerr << "dataset: " << error << "\n";
        return 1;
    }
    ensureMined();
    if (status != COLO_OK) {
        std::cerr << "mining failed: " << colo_status_string(status) << ": " << error << "\n";
        return 1;
    }
    savetoFileGen(0);
    if (!outputLocation_.empty() && !outputFile_.empty()) {
        std::ofstream out(outputLocation_ + outputFile_);
        out << "k\tpattern\trows\tnumerators\tcounts\tPI\n";
        for (uint32_t li = 0; li < colo_result_num_levels(res_); ++li) {
            uint32_t k = colo_result_level_size(res_, li);
            uint64_t n = colo_result_level_candidates(res_, li);
            std::vector<uint32_t> cand(n * k);
            std::vector<uint64_t> rows(n), num(n * k);
            std::vector<float> pi(n);
            std::vector<uint8_t> prev(n);
            colo_result_level(res_, li, cand.data(), nullptr, nullptr, rows.data(), num.data(), pi.data(), prev.data(),
                              nullptr);
            for (uint64_t c = 0; c < n; ++c) {
                if (!prev[c]) continue;
                out << k << "\t";
                for (uint32_t j = 0; j < k; ++j) out << (j ? "|" : "") << featureTypes[cand[c * k + j]];
                out << "\t" << rows[c] << "\t";
                for (uint32_t j = 0; j < k; ++j) out << (j ? "," : "") << num[c * k + j];
                out << "\t";
                for (uint32_t j = 0; j < k; ++j) out << (j ? "," : "") << colo_dataset_feature_count(ds_, cand[c * k + j]);
                char buf[64];
                std::snprintf(buf, sizeof buf, "\t%.9g\n", (double)pi[c]);
                out << buf;
            }
        }
    }
    double t[8];
    colo_result_times(res_, t);
    // The reference's summary line (colocationFinder.cpp:1144), milliseconds:
    // dataset, executable, PI threshold, io, transfer, grid, filter, refine, t1, e2e
    std::cout << std::endl
              << dataset_ << " , " << "GPU_GB300" << " , " << params_.pi_threshold << " , " << ioMs_ << " , " << t[1]
              << " , " << (t[2] + t[3]) << " , " << t[4] << " , " << t[5] << " , " << (t[6] + t[7]) << " , "
              << ms_since(t_all) << std::endl;
    return 0;
}
