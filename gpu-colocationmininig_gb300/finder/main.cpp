// main.cpp -- the GPU-Colocation command line (Codes/main.cpp:8-48):
//   GPU-Colocation <config.txt>
#include <cstdio>

#include "colocationFinder.h"

int main(int argc, char** argv) {
    colocationFinder finder;
    if (finder.status != COLO_OK) {
        std::printf("There is no device supporting CUDA\n");
        return -1;
    }
    return finder.Begin((Integer)argc, argv);
}
