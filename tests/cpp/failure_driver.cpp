// failure_driver.cpp -- the adapter's error behaviour on a failed solve, as the reference's: with a
// non-finite k-point, Hamiltonian::Diagonalize and BandStructure::Compute_parallel throw
// std::runtime_error (Hamiltonian.cpp:129-133 throws "Eigenvalue decomposition failed").
//   failure_driver <yaml> <material> <shells>
// Prints one line per case: "<case> runtime_error" / "<case> other" / "<case> none".
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <stdexcept>
#include <string>
#include <vector>

#include "BandStructure.h"
#include "Hamiltonian.h"
#include "Material.h"

using namespace uepm::pseudopotential;

template <typename F>
static void run(const char* name, F f) {
    try {
        f();
        std::printf("%s none\n", name);
    } catch (const std::runtime_error&) {
        std::printf("%s runtime_error\n", name);
    } catch (...) {
        std::printf("%s other\n", name);
    }
}

int main(int argc, char** argv) {
    if (argc != 4) return 2;
    Materials mats;
    mats.load_material_parameters(argv[1]);
    const Material& mat    = mats.materials.at(argv[2]);
    const int       shells = std::atoi(argv[3]);
    const double    nan    = std::nan("");
    BandStructure   ok;
    ok.Initialize(mat, 8, std::vector<Vector3D<double>>{Vector3D<double>(0.1, 0.2, 0.3)}, shells, false, false);
    run("finite_compute", [&] { ok.Compute_parallel(false, 1); });
    run("hamiltonian_nan_k", [&] {
        Hamiltonian h(mat, ok.get_basis_vectors());
        h.SetMatrix(Vector3D<double>(nan, 0.0, 0.0));
        h.Diagonalize(false);
    });
    run("compute_parallel_nan_k", [&] {
        BandStructure bs;
        bs.Initialize(mat, 8, std::vector<Vector3D<double>>{Vector3D<double>(0.1, 0.2, 0.3), Vector3D<double>(nan, 0.5, 0.5)},
                      shells, false, false);
        bs.Compute_parallel(true, 4);
    });
    return 0;
}
