// ref_driver.cpp -- CHECKER ONLY. A thin extern "C" shim, compiled together with the reference's
// own sources (read in place from the reference tree by oracle/Makefile, never copied), so that
// tests can compare the oracle's restatement with the reference's code on the same inputs.
//
// Only the hot-path pieces that compile from their own files are built: bessel_func.hpp,
// Pseudopotential.cpp, SymmetryPoints.cpp and Vector3D. Hamiltonian.cpp, Material.cpp,
// SpinOrbitFunctional.cpp and BandStructure.cpp need Eigen and yaml-cpp, which the reference
// fetches at configure time and which are absent here, so they are not built.
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "Pseudopotential.h"
#include "SymmetryPoints.h"
#include "Vector3D.h"
#include "bessel_func.hpp"

extern "C" {

double ref_cyl_bessel(double nu, double x) { return generalized_bessel_cylindrical(nu, x); }

// generalized_bessel throws std::invalid_argument for x < 0; report that as NaN.
double ref_sph_bessel(double nu, double x) {
    try {
        return generalized_bessel(nu, x);
    } catch (const std::invalid_argument&) {
        return __builtin_nan("");
    }
}

double ref_bessel_i2(double x) { return bessel_2nd_order_first_kind(x); }

// Pseudopotential::GetValue(G, tau, a) with V in eV.
void ref_pp_value(const double* V8, int gx, int gy, int gz, const double* tau, double a, double* out) {
    uepm::pseudopotential::Pseudopotential pp(V8[0], V8[1], V8[2], V8[3], V8[4], V8[5], V8[6], V8[7]);
    const Vector3D<int>    G(gx, gy, gz);
    const Vector3D<double> t(tau[0], tau[1], tau[2]);
    const auto             v = pp.GetValue(G, t, a);
    out[0]                   = v.real();
    out[1]                   = v.imag();
}

// SymmetryPoints::GeneratePoints; returns the count, or -1 where the reference throws.
int ref_generate_path(const char* labels, unsigned nrPoints, double* out, int capacity, uint32_t* sympos, int sym_capacity) {
    std::vector<std::string> path;
    for (const char* c = labels; *c; ++c) path.emplace_back(1, *c);
    uepm::pseudopotential::SymmetryPoints sp;
    std::vector<unsigned int>             pos;
    std::vector<Vector3D<double>>         pts;
    try {
        pts = sp.GeneratePoints(path, nrPoints, pos);
    } catch (const std::invalid_argument&) {
        return -1;
    }
    for (size_t i = 0; i < pts.size() && (int)i < capacity; ++i) {
        out[3 * i]     = pts[i].X;
        out[3 * i + 1] = pts[i].Y;
        out[3 * i + 2] = pts[i].Z;
    }
    for (size_t i = 0; i < pos.size() && (int)i < sym_capacity; ++i) sympos[i] = pos[i];
    return (int)pts.size();
}

}  // extern "C"
