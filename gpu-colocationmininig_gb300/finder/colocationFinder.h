// colocationFinder.h -- drop-in C++ front end with the reference's class
// interface (Codes/colocationFinder.h:11-184), implemented over the C ABI
// of libcolo (include/colo.h).
//
// The reference mines one level per call and keeps instance tables on the
// host between calls; here the whole level loop runs inside colo_mine with
// the tables resident on the GPU.  The per-level methods therefore trigger
// the mining once (on first use) and then read that level's results.
#pragma once
#include <stdint.h>

#include <string>
#include <vector>

#include "colo.h"

typedef unsigned int Integer;   // Codes/DataTypes.h:5
typedef float Real;             // Codes/DataTypes.h:11

class colocationFinder {
public:
    colocationFinder(void);
    ~colocationFinder(void);

    // Begin (colocationFinder.cpp:1068-1147): argv[1] is the five-line config
    // file.  Mines, writes <location>ColocationDegree_<k>.txt for every level,
    // a per-pattern report to <outputLocation><outputFile> when both are set,
    // and prints the reference's timing line.  Returns 0 on success.
    int Begin(Integer argc, char** argv);
    // LoadParameter (colocationFinder.cpp:57-74)
    void LoadParameter(std::string parameterFileName);
    // populateData (colocationFinder.cpp:139-254)
    void populateData(std::string datasetFilename);
    // degree2Processing (colocationFinder.cpp:256-425): level 2 results.
    void degree2Processing();
    // generatePrevalentPatternsGeneral (colocationFinder.cpp:736-854)
    void generatePrevalentPatternsGeneral(Integer degree);
    // generateInstanceTableGeneral (colocationFinder.cpp:856-909): tables stay on the GPU.
    void generateInstanceTableGeneral(Integer degree);
    // candidateColocationGeneral (colocationFinder.cpp:517-557): candidates of `degree`.
    void candidateColocationGeneral(Integer degree);
    // savetoFileGen (colocationFinder.cpp:979-997) for every mined level.
    void savetoFileGen(Integer degree);

    // results of the last call
    Integer candiColocCounter = 0;                 // candidates of the current level
    std::vector<Integer> h_candiColocations;       // flattened candidates
    std::vector<Integer> h_prevalantColocations;   // flattened prevalent patterns of the level
    Integer h_prevelentColocationCount = 0;
    std::vector<std::string> featureTypes;         // feature names (CSV ids)
    colo_status status = COLO_OK;
    std::string error;

private:
    void ensureMined();
    void selectLevel(Integer degree);
    colo_ctx* ctx_ = nullptr;
    colo_dataset* ds_ = nullptr;
    colo_result* res_ = nullptr;
    colo_params params_{};
    std::string location_, outputLocation_, outputFile_, dataset_;
    double ioMs_ = 0;
};
