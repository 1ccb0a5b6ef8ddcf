// adapter_bands.cpp -- Hamiltonian and BandStructure of the C++ adapter over the C ABI.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <complex>
#include <fstream>
#include <iostream>
#include <stdexcept>
#include <vector>

#include "BandStructure.h"
#include "Hamiltonian.h"
#include "uepm_gb300.h"

namespace uepm::pseudopotential {

namespace {

void throw_for(int rc, const char* what) {
    if (rc == UEPM_OK) return;
    const std::string msg = std::string(what) + ": " + uepm_last_error();
    if (rc == UEPM_ERR_INVALID) throw std::invalid_argument(msg);
    if (rc == UEPM_ERR_OUT_OF_RANGE) throw std::out_of_range(msg);
    throw std::runtime_error(msg);
}

std::vector<int32_t> flat_basis(const std::vector<Vector3D<int>>& G) {
    std::vector<int32_t> g(3 * G.size());
    for (size_t i = 0; i < G.size(); ++i) {
        g[3 * i]     = G[i].X;
        g[3 * i + 1] = G[i].Y;
        g[3 * i + 2] = G[i].Z;
    }
    return g;
}

uepm_ctx* make_context(const Material& mat, const std::vector<Vector3D<int>>& G, bool nl, bool soc) {
    const std::vector<int32_t> g   = flat_basis(G);
    uepm_ctx*                  ctx = nullptr;
    const uint32_t             fl  = (nl ? UEPM_NONLOCAL : 0u) | (soc ? UEPM_SOC : 0u);
    throw_for(uepm_ctx_create(&mat.raw(), g.data(), (int)G.size(), fl, &ctx), "Hamiltonian");
    return ctx;
}

}  // namespace

// ------------------------------------------------------------------------------------------------
Hamiltonian::Hamiltonian(const Material& material, const std::vector<Vector3D<int>>& basisVectors)
    : m_material(material), m_basisVectors(basisVectors) {}

Hamiltonian::Hamiltonian(const Hamiltonian& o) : m_material(o.m_material), m_basisVectors(o.m_basisVectors) {}

Hamiltonian::~Hamiltonian() {
    for (auto*& c : m_ctx)
        if (c) uepm_ctx_destroy(c);
}

uepm_ctx* Hamiltonian::context(bool nl, bool soc) const {
    uepm_ctx*& c = m_ctx[(nl ? 1 : 0) + (soc ? 2 : 0)];
    if (!c) c = make_context(m_material, m_basisVectors, nl, soc);
    return c;
}

void Hamiltonian::SetMatrix(const Vector3D<double>& k, bool add_non_local_correction, bool enable_soc) {
    m_k   = k;
    m_nl  = add_non_local_correction;
    m_soc = enable_soc;
    m_set = true;
}

bool Hamiltonian::check_matrix_is_symmetric() const {
    if (!m_set) return true;
    // uepm_ctx_force_complex(ctx, 0) leaves the automatic choice and reports whether H(k) is real
    return uepm_ctx_force_complex(context(m_nl, m_soc), 0) == 1;
}

void Hamiltonian::PrepareBatch(const std::vector<Vector3D<double>>& kpoints, bool add_non_local_correction,
                               bool enable_soc, bool keep_eigenvectors) {
    ClearBatch();
    if (kpoints.empty()) return;
    uepm_ctx*           ctx = context(add_non_local_correction, enable_soc);
    const int           n   = uepm_ctx_order(ctx);
    const size_t        nk  = kpoints.size();
    std::vector<double> k(3 * nk), E(nk * (size_t)n), X(keep_eigenvectors ? nk * 2 * (size_t)n * n : 0);
    std::vector<int32_t> st(nk, 0);
    for (size_t i = 0; i < nk; ++i) {
        k[3 * i]     = kpoints[i].X;
        k[3 * i + 1] = kpoints[i].Y;
        k[3 * i + 2] = kpoints[i].Z;
    }
    const int rc = uepm_solve(ctx, k.data(), nk, n, keep_eigenvectors ? UEPM_WANT_VECTORS : 0u, E.data(),
                              keep_eigenvectors ? X.data() : nullptr, nullptr, st.data());
    // k-points whose solve failed are left out: their own Diagonalize re-solves and throws
    if (rc != UEPM_ERR_NOT_CONVERGED) throw_for(rc, "Hamiltonian::PrepareBatch");
    for (size_t i = 0; i < nk; ++i)
        if (st[i] == 0) m_batch_row.emplace(std::make_tuple(k[3 * i], k[3 * i + 1], k[3 * i + 2]), i);
    m_batch_nl  = add_non_local_correction;
    m_batch_soc = enable_soc;
    m_batch_vec = keep_eigenvectors;
    m_batch_n   = n;
    m_batch_E   = std::move(E);
    m_batch_X   = std::move(X);
}

void Hamiltonian::ClearBatch() {
    m_batch_row.clear();
    m_batch_E.clear();
    m_batch_E.shrink_to_fit();
    m_batch_X.clear();
    m_batch_X.shrink_to_fit();
    m_batch_n = 0;
}

void Hamiltonian::Diagonalize(bool keep_eigenvectors) {
    if (m_batch_n > 0 && m_nl == m_batch_nl && m_soc == m_batch_soc && (!keep_eigenvectors || m_batch_vec)) {
        const auto it = m_batch_row.find(std::make_tuple(m_k.X, m_k.Y, m_k.Z));
        if (it != m_batch_row.end()) {
            const int    n   = m_batch_n;
            const size_t row = it->second;
            m_values.resize(n);
            for (int i = 0; i < n; ++i) m_values(i) = m_batch_E[row * n + i];
            if (keep_eigenvectors) {
                const double* X = m_batch_X.data() + row * 2 * (size_t)n * n;
                m_vectors.resize(n, n);
                for (int b = 0; b < n; ++b)
                    for (int r = 0; r < n; ++r)
                        m_vectors(r, b) = std::complex<double>(X[2 * ((size_t)b * n + r)], X[2 * ((size_t)b * n + r) + 1]);
            } else {
                m_vectors.resize(0, 0);
            }
            return;
        }
    }
    uepm_ctx*         ctx = context(m_nl, m_soc);
    const int         n   = uepm_ctx_order(ctx);
    const double      k[3] = {m_k.X, m_k.Y, m_k.Z};
    std::vector<double> E((size_t)n), X(keep_eigenvectors ? (size_t)2 * n * n : 0);
    int32_t           st  = 0;
    const int rc = uepm_solve(ctx, k, 1, n, keep_eigenvectors ? UEPM_WANT_VECTORS : 0u, E.data(),
                              keep_eigenvectors ? X.data() : nullptr, nullptr, &st);
    if (rc == UEPM_ERR_NOT_CONVERGED || st != 0) throw std::runtime_error("Eigenvalue decomposition failed");
    throw_for(rc, "Hamiltonian::Diagonalize");
    m_values.resize(n);
    for (int i = 0; i < n; ++i) m_values(i) = E[(size_t)i];
    if (keep_eigenvectors) {
        m_vectors.resize(n, n);
        for (int b = 0; b < n; ++b)
            for (int r = 0; r < n; ++r)
                m_vectors(r, b) = std::complex<double>(X[2 * ((size_t)b * n + r)], X[2 * ((size_t)b * n + r) + 1]);
    } else {
        m_vectors.resize(0, 0);
    }
}

Vector3D<double> Hamiltonian::compute_gradient_at_level(const Vector3D<double>& k_point, unsigned int level_index) const {
    // Hellmann-Feynman on the kinetic term, from the kept eigenvector (Hamiltonian.cpp:146-194)
    const long Nb = (long)m_basisVectors.size();
    if (m_vectors.size() == 0)
        throw std::runtime_error("compute_gradient_at_level: eigenvectors not available. Call Diagonalize(true) first.");
    if (level_index >= (unsigned)m_vectors.cols()) throw std::out_of_range("compute_gradient_at_level: level_index out of range");
    constexpr double h = 6.62607015e-34, q_e = 1.602176634e-19, m_e = 9.1093837015e-31;
    constexpr double pi = 3.141592653589793238462643383279502884, h_bar = h / (2.0 * pi);
    constexpr double diag_factor   = (h_bar * h_bar) / (2.0 * m_e * q_e);
    const double     two_pi_over_a = 2.0 * M_PI / m_material.get_lattice_constant_meter();
    const double     pref_frac     = 2.0 * diag_factor * (two_pi_over_a * two_pi_over_a);
    const bool       spin          = m_vectors.rows() == 2 * Nb;
    Vector3D<double> s(0.0, 0.0, 0.0);
    for (long i = 0; i < Nb; ++i) {
        double w = std::norm(m_vectors(i, level_index));
        if (spin) w = w + std::norm(m_vectors(i + Nb, level_index));
        s += (k_point + m_basisVectors[(size_t)i]) * w;
    }
    return (s * pref_frac) * (1.0 / two_pi_over_a);
}

// ------------------------------------------------------------------------------------------------
std::string BandStructure::get_path_as_string() const {
    std::string p;
    for (const auto& s : m_path) p += s;
    return p;
}

bool BandStructure::GenerateBasisVectors(unsigned int nn) {
    const int n = uepm_generate_basis(nn, nullptr, 0);
    if (n < 0) {
        std::cout << "Error: nearestNeighborsNumber must be between 2 and 116" << std::endl;
        return false;
    }
    std::vector<int32_t> g(3 * (size_t)n);
    uepm_generate_basis(nn, g.data(), n);
    basisVectors.resize((size_t)n);
    for (int i = 0; i < n; ++i) basisVectors[(size_t)i] = Vector3D<int>(g[3 * i], g[3 * i + 1], g[3 * i + 2]);
    return true;
}

void BandStructure::Initialize(const Material& material, std::size_t nb_bands, const std::vector<std::string>& path,
                               unsigned int nbPoints, unsigned int nearestNeighborsNumber, bool enable_non_local_correction,
                               bool enable_soc) {
    m_material                    = material;
    m_nb_bands                    = (unsigned)nb_bands;
    m_path                        = path;
    m_nb_points                   = nbPoints;
    m_nearestNeighborsNumber      = nearestNeighborsNumber;
    m_enable_non_local_correction = enable_non_local_correction;
    m_enable_spin_orbit_coupling  = enable_soc;
    m_kpoints.clear();
    m_energies.clear();
    if (m_enable_spin_orbit_coupling) {
        m_nb_bands *= 2;
        std::cout << "Spin-orbit coupling enabled. Number of bands doubled to " << m_nb_bands << std::endl;
    }
    if (!GenerateBasisVectors(nearestNeighborsNumber))
        throw std::runtime_error("BandStructure::Initialize: GenerateBasisVectors failed");
    m_kpoints   = symmetryPoints.GeneratePoints(m_path, m_nb_points, symmetryPointsPositions);
    m_nb_points = (unsigned)m_kpoints.size();
    if (m_nb_points == 0) throw std::runtime_error("BandStructure::Initialize: GeneratePoints failed. No points generated.");
}

void BandStructure::Initialize(const Material& material, std::size_t nb_bands, const std::vector<Vector3D<double>>& list_k_points,
                               unsigned int nearestNeighborsNumber, bool enable_non_local_correction, bool enable_soc) {
    m_material                    = material;
    m_nb_bands                    = (unsigned)nb_bands;
    m_nb_points                   = (unsigned)list_k_points.size();
    m_nearestNeighborsNumber      = nearestNeighborsNumber;
    m_enable_non_local_correction = enable_non_local_correction;
    m_enable_spin_orbit_coupling  = enable_soc;
    if (m_enable_spin_orbit_coupling) {
        m_nb_bands *= 2;
        std::cout << "Spin-orbit coupling enabled. Number of bands doubled to " << m_nb_bands << std::endl;
    }
    m_kpoints = list_k_points;
    m_energies.clear();
    if (!GenerateBasisVectors(nearestNeighborsNumber))
        throw std::runtime_error("BandStructure::Initialize: GenerateBasisVectors failed");
}

void BandStructure::run(bool compute_gradient) {
    const auto start = std::chrono::high_resolution_clock::now();
    m_nb_points      = (unsigned)m_kpoints.size();
    uepm_ctx* ctx    = make_context(m_material, basisVectors, m_enable_non_local_correction, m_enable_spin_orbit_coupling);
    const int n      = uepm_ctx_order(ctx);
    const int nb     = std::min<int>((int)m_nb_bands, n);
    if (m_precision == SolvePrecision::mixed) uepm_ctx_set_precision(ctx, UEPM_PREC_MIXED);
    const size_t        nk = m_kpoints.size();
    std::vector<double> k(3 * nk), E(nk * nb), g(compute_gradient ? nk * nb * 3 : 0);
    for (size_t i = 0; i < nk; ++i) {
        k[3 * i]     = m_kpoints[i].X;
        k[3 * i + 1] = m_kpoints[i].Y;
        k[3 * i + 2] = m_kpoints[i].Z;
    }
    const int rc = uepm_solve(ctx, k.data(), nk, nb, compute_gradient ? UEPM_WANT_GRADIENT : 0u, E.data(), nullptr,
                              compute_gradient ? g.data() : nullptr, nullptr);
    uepm_ctx_destroy(ctx);
    if (rc == UEPM_ERR_NOT_CONVERGED) throw std::runtime_error("Eigenvalue decomposition failed");
    throw_for(rc, "BandStructure::Compute");
    m_energies.assign(nk, std::vector<double>((size_t)nb));
    // The reference sizes the gradient array [nk * nb] rows of nb and fills the first nk rows
    // (BandStructure.cpp:158-166, :186-187); kept, so get_band_energy_gradients().size() matches.
    if (compute_gradient) m_energies_gradient.assign(nk * m_nb_bands, std::vector<Vector3D<double>>((size_t)m_nb_bands));
    for (size_t i = 0; i < nk; ++i)
        for (int b = 0; b < nb; ++b) {
            m_energies[i][(size_t)b] = E[i * nb + b];
            if (compute_gradient) {
                const double* gg                  = &g[(i * nb + b) * 3];
                m_energies_gradient[i][(size_t)b] = Vector3D<double>(gg[0], gg[1], gg[2]);
            }
        }
    const auto end       = std::chrono::high_resolution_clock::now();
    m_computation_time_s = (double)std::chrono::duration_cast<std::chrono::seconds>(end - start).count();
}

void BandStructure::Compute(bool) {
    std::cout << "Computing band structure..." << std::endl;
    run(false);  // the reference's serial Compute keeps no gradients (BandStructure.cpp:124-149)
}

void BandStructure::Compute_parallel(bool compute_gradient, int nb_threads) {
    std::cout << "Computing band structure with " << nb_threads << " threads..." << std::endl;
    run(compute_gradient);
}

double BandStructure::AdjustValues(bool minConductionBandToZero) {
    if (m_energies.empty()) return 0.0;
    const size_t        nk = m_energies.size(), nb = m_energies.front().size();
    std::vector<double> E(nk * nb);
    for (size_t i = 0; i < nk; ++i) std::copy(m_energies[i].begin(), m_energies[i].end(), E.begin() + i * nb);
    double gap   = 0.0;
    int    found = 0;
    uepm_adjust_values(E.data(), nk, (int)nb, m_enable_spin_orbit_coupling ? 1 : 0, minConductionBandToZero ? 1 : 0, &gap,
                       &found);
    for (size_t i = 0; i < nk; ++i) std::copy(E.begin() + i * nb, E.begin() + (i + 1) * nb, m_energies[i].begin());
    std::cout << "Band gap found: " << gap << " eV" << std::endl;
    return gap;
}

std::vector<double> BandStructure::get_band(unsigned int band_index) const {
    std::vector<double> r;
    r.reserve(m_energies.size());
    for (const auto& p : m_energies) r.push_back(p[band_index]);
    return r;
}

void BandStructure::print_results() const {
    for (const auto& p : m_energies) {
        for (double v : p) std::cout << v << " ";
        std::cout << std::endl;
    }
}

void BandStructure::export_k_points_to_file(std::string filename) const {
    std::ofstream f(filename);
    for (const auto& p : m_kpoints) f << p.Y << " " << p.X << " " << p.Z << std::endl;
}

// Band file read by python/plots/plot_band_structure.py (BandStructure.cpp:290-314 layout).
void BandStructure::export_result_in_file(const std::string& filename) const {
    std::cout << "Exporting band structure to file:     " << filename << std::endl;
    std::ofstream f(filename);
    f << "# Material " << m_material.get_name() << std::endl;
    f << "# NBands " << m_nb_bands << std::endl;
    f << "# Nonlocal " << (m_enable_non_local_correction ? "Yes" : "No") << std::endl;
    f << "# Path " << get_path_as_string() << std::endl;
    f << "# Symmetry points:";
    for (unsigned p : symmetryPointsPositions) f << " " << p;
    f << std::endl;
    const size_t nb = m_energies.front().size();
    for (size_t i = 0; i + 1 < nb; ++i) f << "band_" << i << ",";
    f << "band_" << nb - 1 << std::endl;
    for (unsigned k = 0; k < m_nb_points; ++k) {
        for (size_t b = 0; b < nb; ++b) f << (b ? "," : "") << m_energies[k][b];
        f << std::endl;
    }
}

void BandStructure::export_result_in_file_with_kpoints(const std::string& filename) const {
    std::cout << "Exporting band structure to file:     " << filename << std::endl;
    std::ofstream f(filename);
    f << "kx,ky,kz,";
    const size_t nb = m_energies.front().size();
    for (size_t i = 0; i + 1 < nb; ++i) f << "band_" << i << ",";
    f << "band_" << nb - 1 << std::endl;
    for (unsigned k = 0; k < m_nb_points; ++k) {
        f << m_kpoints[k].Y << "," << m_kpoints[k].X << "," << m_kpoints[k].Z << ",";
        for (size_t b = 0; b < nb; ++b) f << (b ? "," : "") << m_energies[k][b];
        f << std::endl;
    }
}

std::string BandStructure::path_band_filename() const {
    return "EPM_" + m_material.get_name() + "_nb_bands_" + std::to_string(m_energies.front().size()) + "_path_" +
           get_path_as_string() + "_size_basis_" + std::to_string(basisVectors.size());
}

void export_vector_bands_result_in_file(const std::string& filename, std::vector<std::vector<double>> results) {
    std::cout << "Exporting band structure to file:     " << filename << std::endl;
    std::ofstream f(filename);
    for (const auto& p : results) {
        for (double v : p) f << v << ",";
        f << std::endl;
    }
}

}  // namespace uepm::pseudopotential
