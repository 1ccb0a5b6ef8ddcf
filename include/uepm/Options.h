// Options.h -- the reference's run options (src/EPP/Options.h, Options.cpp:5-31): defaults and the
// 17 canned symmetry-point paths, unchanged in meaning.
#pragma once

#include <string>
#include <vector>

class Options {
 public:
    Options();
    void print_options();

    int         nrThreads;
    std::string materialName;
    int         nrPoints;
    int         nearestNeighbors;
    int         nrLevels;
    int         pathNo;

    std::vector<std::vector<std::string>> paths;
};
