// SymmetryPoints.h -- uepm::pseudopotential::SymmetryPoint(s) (src/EPP/SymmetryPoints.h:8-43): the
// fcc high-symmetry points L, G, X, W, K, U and the path generator (uepm_generate_path).
#pragma once

#include <map>
#include <string>
#include <vector>

#include "Vector3D.h"

namespace uepm::pseudopotential {

class SymmetryPoint {
 public:
    SymmetryPoint() {}
    SymmetryPoint(const std::string& Name, const Vector3D<double> pos) : name(Name), position(pos) {}
    std::string      name;
    Vector3D<double> position;
};

class SymmetryPoints {
 public:
    SymmetryPoints();
    std::map<std::string, SymmetryPoint> symmetryPoints;

    // Throws std::invalid_argument for fewer than two nodes, nrPoints below the node count or an
    // unknown label, like the reference.
    std::vector<Vector3D<double>> GeneratePoints(const std::vector<std::string>& path, unsigned int nrPoints,
                                                 std::vector<unsigned int>& symmetryPointsPositions);
};

}  // namespace uepm::pseudopotential
