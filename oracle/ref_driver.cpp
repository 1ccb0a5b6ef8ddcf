// ref_driver.cpp -- CHECKER ONLY. A thin extern "C" shim, compiled together with the reference's
// own sources (read in place from the reference tree by oracle/Makefile, never copied), so that
// tests can compare the oracle's restatement with the reference's code on the same inputs.
//
// Built from the reference: bessel_func.hpp, Pseudopotential.cpp, SymmetryPoints.cpp, Vector3D,
// and -- against the project-written Eigen and yaml-cpp subsets in oracle/shim/ (the reference
// fetches both at configure time; neither is present here) -- Material.cpp (the YAML loader and
// the nonlocal correction), SpinOrbitFunctional.cpp, Hamiltonian.cpp and BandStructure.cpp. The
// shim's SelfAdjointEigenSolver is the oracle's restated Eigen solver (or_eigh), so eigenvalues
// from this library pin the assembly and the host logic, not the solver.
#include <cstdint>
#include <cstring>
#include <exception>
#include <map>
#include <string>
#include <vector>

#include "BandStructure.h"
#include "Hamiltonian.h"
#include "Material.h"
#include "Pseudopotential.h"
#include "SpinOrbitFunctional.hpp"
#include "SymmetryPoints.h"
#include "Vector3D.h"
#include "bessel_func.hpp"

namespace up = uepm::pseudopotential;

namespace {

// The loaded fields in the layout of the oracle's or_material (and the product's uepm_material).
struct RefMaterial {
    double   lattice_constant;
    double   V3S, V4S, V8S, V11S, V3A, V4A, V8A, V11A;
    int32_t  nl_well;
    int32_t  has_nonlocal;
    double   alpha0_cation, beta0_cation, A2_cation, alpha0_anion, beta0_anion, A2_anion;
    double   R0_cation, R2_cation, R0_anion, R2_anion;
    uint32_t period_anion, period_cation;
    int32_t  has_soc;
    int32_t  _pad;
    double   radial_extent_anion, radial_extent_cation, alpha_soc, mu_soc;
};

// Read access to the reference classes' protected fields, through derived copies.
struct PPFields : up::Pseudopotential {
    explicit PPFields(const up::Pseudopotential& p) : up::Pseudopotential(p) {}
    void fill(RefMaterial& o) const {
        o.V3S  = m_V3S;
        o.V4S  = m_V4S;
        o.V8S  = m_V8S;
        o.V11S = m_V11S;
        o.V3A  = m_V3A;
        o.V4A  = m_V4A;
        o.V8A  = m_V8A;
        o.V11A = m_V11A;
    }
};
struct MatFields : up::Material {
    explicit MatFields(const up::Material& m) : up::Material(m) {}
    void fill(RefMaterial& o) const {
        std::memset(&o, 0, sizeof(o));
        o.lattice_constant = m_lattice_constant;
        PPFields(m_pseudopotential).fill(o);
        const up::NonLocalParameters& nl = m_non_local_parameters;
        o.has_nonlocal                  = m_is_non_local_parameters_populated ? 1 : 0;
        o.nl_well = nl.m_well_type == up::non_local_well_type::square ? 1 : nl.m_well_type == up::non_local_well_type::gaussian ? 2 : 0;
        o.alpha0_cation = nl.m_alpha_0_cation;
        o.beta0_cation  = nl.m_beta_0_cation;
        o.A2_cation     = nl.m_A2_cation;
        o.alpha0_anion  = nl.m_alpha_0_anion;
        o.beta0_anion   = nl.m_beta_0_anion;
        o.A2_anion      = nl.m_A2_anion;
        o.R0_cation     = nl.m_R0_cation;
        o.R2_cation     = nl.m_R2_cation;
        o.R0_anion      = nl.m_R0_anion;
        o.R2_anion      = nl.m_R2_anion;
        const up::SpinOrbitParameters& so = m_spin_orbit_parameters;
        o.has_soc                         = m_is_spin_orbit_parameters_populated ? 1 : 0;
        o.period_anion                    = so.m_period_anion;
        o.period_cation                   = so.m_period_cation;
        o.radial_extent_anion             = so.m_radial_extent_anion;
        o.radial_extent_cation            = so.m_radial_extent_cation;
        o.alpha_soc                       = so.m_alpha;
        o.mu_soc                          = so.m_mu;
    }
};

// Hamiltonian with its (protected) matrix readable.
struct HamAccess : up::Hamiltonian {
    using up::Hamiltonian::Hamiltonian;
    const Eigen::MatrixXcd& H() const { return matrix; }
};

std::map<std::string, up::Material> load(const char* path) {
    up::Materials m;
    m.load_material_parameters(path);
    return m.materials;
}

std::vector<Vector3D<int>> basis_of(const int32_t* G, int N) {
    std::vector<Vector3D<int>> b;
    for (int i = 0; i < N; ++i) b.emplace_back(G[3 * i], G[3 * i + 1], G[3 * i + 2]);
    return b;
}

}  // namespace

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

// Materials::load_material_parameters on `path`; the fields of `symbol` in the oracle's layout.
// Returns 0, -1 when the symbol is absent, -2 when the loader throws.
int ref_material(const char* path, const char* symbol, RefMaterial* out) {
    try {
        auto mats = load(path);
        auto it   = mats.find(symbol);
        if (it == mats.end()) return -1;
        MatFields(it->second).fill(*out);
        return 0;
    } catch (const std::exception&) {
        return -2;
    }
}

int ref_material_size(void) { return (int)sizeof(RefMaterial); }

// Hamiltonian(material, basis); per k: SetMatrix(k, nl, soc), Diagonalize(false), then the
// hermitised matrix Diagonalize leaves behind. H: nk x n x n complex, column-major, (re, im).
// Returns n, or -1 (unknown symbol), -2 (a reference exception).
int ref_hamiltonian(const char* path, const char* symbol, const int32_t* G, int N, const double* k, int nk, int nl, int soc,
                    double* H) {
    try {
        auto mats = load(path);
        auto it   = mats.find(symbol);
        if (it == mats.end()) return -1;
        const auto basis = basis_of(G, N);
        HamAccess  ham(it->second, basis);
        int        n = 0;
        for (int q = 0; q < nk; ++q) {
            ham.SetMatrix(Vector3D<double>(k[3 * q], k[3 * q + 1], k[3 * q + 2]), nl != 0, soc != 0);
            ham.Diagonalize(false);
            const auto& M = ham.H();
            n             = (int)M.rows();
            std::memcpy(H + (size_t)q * 2 * n * n, M.data(), sizeof(double) * 2 * (size_t)n * n);
        }
        return n;
    } catch (const std::exception&) {
        return -2;
    }
}

// Material::compute_pseudopotential_non_local_correction(K1, K2, tau), K in reduced units, tau in m.
int ref_nl_correction(const char* path, const char* symbol, const double* K1, const double* K2, const double* tau,
                      double* out) {
    try {
        auto mats = load(path);
        auto it   = mats.find(symbol);
        if (it == mats.end()) return -1;
        const auto v = it->second.compute_pseudopotential_non_local_correction(Vector3D<double>(K1[0], K1[1], K1[2]),
                                                                              Vector3D<double>(K2[0], K2[1], K2[2]),
                                                                              Vector3D<double>(tau[0], tau[1], tau[2]));
        out[0] = v.real();
        out[1] = v.imag();
        return 0;
    } catch (const std::exception&) {
        return -2;
    }
}

// SpinOrbitCorrection(material, params).compute_soc_contribution(K, Kp, G, Gp, tau): the 2x2 block
// row-major as (re, im) pairs.
int ref_soc_block(const char* path, const char* symbol, const double* K, const double* Kp, const double* G,
                  const double* Gp, const double* tau, double* out) {
    try {
        auto mats = load(path);
        auto it   = mats.find(symbol);
        if (it == mats.end()) return -1;
        up::SpinOrbitCorrection soc(it->second, it->second.get_spin_orbit_parameters());
        const auto              b = soc.compute_soc_contribution(Vector3D<double>(K[0], K[1], K[2]),
                                                    Vector3D<double>(Kp[0], Kp[1], Kp[2]),
                                                    Vector3D<double>(G[0], G[1], G[2]),
                                                    Vector3D<double>(Gp[0], Gp[1], Gp[2]),
                                                    Vector3D<double>(tau[0], tau[1], tau[2]));
        for (int r = 0; r < 2; ++r)
            for (int c = 0; c < 2; ++c) {
                out[2 * (2 * r + c)]     = b(r, c).real();
                out[2 * (2 * r + c) + 1] = b(r, c).imag();
            }
        return 0;
    } catch (const std::exception&) {
        return -2;
    }
}

// BandStructure::Initialize(material, nb, path, n_points, shells, nl, soc), Compute(false),
// AdjustValues(min_cond_zero), export_result_in_file(out_file). E receives up to `capacity` values
// of the [nk][nb] energies; returns nk * nb (nb after the reference's SOC doubling), or -1 / -2.
int ref_band_file(const char* path, const char* symbol, int nb, const char* labels, unsigned n_points, unsigned shells,
                  int nl, int soc, int min_cond_zero, const char* out_file, double* E, int capacity) {
    try {
        auto mats = load(path);
        auto it   = mats.find(symbol);
        if (it == mats.end()) return -1;
        std::vector<std::string> p;
        for (const char* c = labels; *c; ++c) p.emplace_back(1, *c);
        up::BandStructure bs;
        bs.Initialize(it->second, (size_t)nb, p, n_points, shells, nl != 0, soc != 0);
        bs.Compute(false);
        bs.AdjustValues(min_cond_zero != 0);
        bs.export_result_in_file(out_file);
        const auto& en = bs.get_band_energies();
        int         q  = 0;
        for (const auto& row : en)
            for (double v : row)
                if (q < capacity) E[q++] = v;
                else ++q;
        return q;
    } catch (const std::exception&) {
        return -2;
    }
}

// BandStructure::Compute_parallel(true, 1) on a k list: the shape of get_band_energy_gradients()
// (rows, and the length of each row), and the gradients of the first `rows_out` rows.
int ref_gradient_shape(const char* path, const char* symbol, int nb, const double* k, int nk, unsigned shells, int* rows,
                       int* row_len, double* grad, int rows_out) {
    try {
        auto mats = load(path);
        auto it   = mats.find(symbol);
        if (it == mats.end()) return -1;
        std::vector<Vector3D<double>> ks;
        for (int q = 0; q < nk; ++q) ks.emplace_back(k[3 * q], k[3 * q + 1], k[3 * q + 2]);
        up::BandStructure bs;
        bs.Initialize(it->second, (size_t)nb, ks, shells, false, false);
        bs.Compute_parallel(true, 1);
        const auto& g = bs.get_band_energy_gradients();
        *rows         = (int)g.size();
        *row_len      = g.empty() ? 0 : (int)g.front().size();
        for (int r = 0; r < rows_out && r < (int)g.size(); ++r)
            for (size_t b = 0; b < g[r].size(); ++b) {
                grad[((size_t)r * g[r].size() + b) * 3]     = g[r][b].X;
                grad[((size_t)r * g[r].size() + b) * 3 + 1] = g[r][b].Y;
                grad[((size_t)r * g[r].size() + b) * 3 + 2] = g[r][b].Z;
            }
        return 0;
    } catch (const std::exception&) {
        return -2;
    }
}

}  // extern "C"
