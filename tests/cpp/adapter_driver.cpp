// adapter_driver.cpp -- exercises the C++ adapter the way the reference's apps use src/EPP:
// Materials -> BandStructure::Initialize(path) -> Compute_parallel(true) -> AdjustValues -> export,
// and Hamiltonian::SetMatrix / Diagonalize(true) / compute_gradient_at_level at one k-point, and the
// same loop over a few k-points after Hamiltonian::PrepareBatch against the per-k solves.
//   adapter_driver <yaml> <material> <path> <npoints> <nbands> <shells> <nl 0|1> <soc 0|1> <fp64|mixed> <out_prefix>
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "BandStructure.h"
#include "Hamiltonian.h"
#include "Material.h"

using namespace uepm::pseudopotential;

int main(int argc, char** argv) {
    if (argc != 11) {
        std::fprintf(stderr, "usage: adapter_driver yaml material path npoints nbands shells nl soc prec out\n");
        return 2;
    }
    const std::string yaml = argv[1], name = argv[2], path = argv[3], prec = argv[9], out = argv[10];
    const int         npts = std::atoi(argv[4]), nbands = std::atoi(argv[5]), shells = std::atoi(argv[6]);
    const bool        nl = std::atoi(argv[7]) != 0, soc = std::atoi(argv[8]) != 0;
    Materials mats;
    mats.load_material_parameters(yaml);
    const Material&          mat = mats.materials.at(name);
    std::vector<std::string> labels;
    for (char c : path) labels.emplace_back(1, c);
    BandStructure bs;
    bs.Initialize(mat, nbands, labels, npts, shells, nl, soc);
    if (prec == "mixed") bs.set_precision(SolvePrecision::mixed);
    bs.Compute_parallel(true, 4);
    FILE* f = std::fopen((out + "_raw.txt").c_str(), "w");
    const auto& E = bs.get_band_energies();
    const auto& g = bs.get_band_energy_gradients();
    for (size_t k = 0; k < E.size(); ++k)
        for (size_t b = 0; b < E[k].size(); ++b)
            std::fprintf(f, "%zu %zu %.17g %.17g %.17g %.17g\n", k, b, E[k][b], g[k][b].X, g[k][b].Y, g[k][b].Z);
    std::fclose(f);
    const double gap = bs.AdjustValues();
    bs.export_result_in_file(out + "_bands.txt");
    // one k-point through Hamiltonian directly, all eigenvalues and vectors
    Hamiltonian h(mat, bs.get_basis_vectors());
    const Vector3D<double> k0(0.11, 0.27, -0.05);
    const bool sym_before = h.check_matrix_is_symmetric();
    h.SetMatrix(k0, nl, soc);
    h.Diagonalize(true);
    std::printf("symmetric %d %d\n", sym_before ? 1 : 0, h.check_matrix_is_symmetric() ? 1 : 0);
    std::printf("gradrows %zu %zu\n", g.size(), g.empty() ? (size_t)0 : g.front().size());
    FILE* fh = std::fopen((out + "_ham.txt").c_str(), "w");
    const auto& ev = h.eigenvalues();
    for (long i = 0; i < ev.size(); ++i) std::fprintf(fh, "E %.17g\n", ev(i));
    for (unsigned lvl = 0; lvl < 4; ++lvl) {
        const Vector3D<double> gr = h.compute_gradient_at_level(k0, lvl);
        std::fprintf(fh, "G %u %.17g %.17g %.17g\n", lvl, gr.X, gr.Y, gr.Z);
    }
    std::fclose(fh);
    // a caller's loop over k-points (bz_states.cpp:30-47) after one batched solve, against per-k solves
    std::vector<Vector3D<double>> ks;
    for (int q = 0; q < 6; ++q) ks.emplace_back(0.11 - 0.05 * q, 0.27 + 0.03 * q, -0.05 + 0.02 * q);
    Hamiltonian hb(mat, bs.get_basis_vectors()), h1(mat, bs.get_basis_vectors());
    hb.PrepareBatch(ks, nl, soc, true);
    double dv = 0.0, dx = 0.0;
    for (const auto& kq : ks) {
        hb.SetMatrix(kq, nl, soc);
        hb.Diagonalize(true);
        h1.SetMatrix(kq, nl, soc);
        h1.Diagonalize(true);
        for (long i = 0; i < h1.eigenvalues().size(); ++i) dv = std::max(dv, std::fabs(hb.eigenvalues()(i) - h1.eigenvalues()(i)));
        for (long b = 0; b < h1.get_eigenvectors().cols(); ++b)
            for (long r = 0; r < h1.get_eigenvectors().rows(); ++r)
                dx = std::max(dx, std::abs(hb.get_eigenvectors()(r, b) - h1.get_eigenvectors()(r, b)));
    }
    std::printf("batchdiff %.17g %.17g\n", dv, dx);
    std::printf("gap %.17g\nfile %s\n", gap, bs.path_band_filename().c_str());
    return 0;
}
