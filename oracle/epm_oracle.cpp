// epm_oracle.cpp -- CPU ORACLE (test infrastructure; never part of the product path).
//
// A plain, sequential restatement of UltimateEPM's per-k-point band-structure path, used only by
// tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as the checker. Every function
// cites the reference file:line it restates (paths relative to the reference project root).
//
// Numerics policy: compiled with -ffp-contract=off and without -ffast-math, and every expression
// keeps the reference's operand order, so that on the same inputs the arithmetic is the IEEE
// evaluation of the reference's own formulas. The Bessel functions call libstdc++'s
// std::cyl_bessel_j / std::cyl_neumann exactly as src/EPP/bessel_func.hpp:17-45 does.
//
// The dense eigensolver lives in a third-party library that is absent from the reference tree:
// Eigen 5.0.0 (CPM pin, CMakeLists.txt:95-101), class SelfAdjointEigenSolver, called at
// src/EPP/Hamiltonian.cpp:125-134. Its published algorithm is restated here in our own code:
// scale by the largest |a_ij| of the lower triangle, Householder reduction to real symmetric
// tridiagonal form, implicit symmetric QR with a Wilkinson shift and Givens bulge chasing
// (Golub & Van Loan, Matrix Computations, Alg. 8.3.2/8.3.3), Eigen's deflation test
// |e_i| <= eps*sqrt(|d_i|+|d_i+1|), 30*n iteration cap, then an ascending selection sort.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <limits>
#include <numeric>
#include <string>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

typedef std::complex<double> cd;

// ------------------------------------------------------------------------------------------------
// Constants: src/Common/physical_constants.hpp:18-44 (same constexpr expressions, same values).
namespace orc {
constexpr double h           = 6.62607015e-34;
constexpr double q_e         = 1.602176634e-19;
constexpr double pi          = 3.141592653589793238462643383279502884;  // std::numbers::pi_v<double>
constexpr double h_bar       = h / (2.0 * pi);
constexpr double m_e         = 9.1093837015e-31;
constexpr double bohr_radius = 5.29177210903e-11;
constexpr double Hartree_to_J  = 4.3597447222071e-18;
constexpr double Hartree_to_eV = Hartree_to_J / q_e;
constexpr double Ryd_to_eV     = Hartree_to_eV / 2.0;
}  // namespace orc

extern "C" {

// Material parameters, in the units the reference holds them after loading
// (src/EPP/Material.cpp:33-71, src/EPP/NonLocalParameters.hpp:91-116,
// src/EPP/SpinOrbitParameters.hpp:74-81): V* in eV, alpha_0 and A2 in eV, beta_0 raw, radii in m,
// SOC radial extents and mu/alpha raw. Layout is identical to the product's uepm_material.
struct or_material {
    double   lattice_constant;  // Angstrom
    double   V3S, V4S, V8S, V11S, V3A, V4A, V8A, V11A;
    int32_t  nl_well;           // 0 unknown, 1 square, 2 gaussian
    int32_t  has_nonlocal;
    double   alpha0_cation, beta0_cation, A2_cation, alpha0_anion, beta0_anion, A2_anion;
    double   R0_cation, R2_cation, R0_anion, R2_anion;
    uint32_t period_anion, period_cation;
    int32_t  has_soc;
    int32_t  _pad;
    double   radial_extent_anion, radial_extent_cation, alpha_soc, mu_soc;
};

int or_material_size(void) { return (int)sizeof(or_material); }

// Material::get_lattice_constant_meter, src/EPP/Material.h:108-111
static double lattice_m(const or_material* m) {
    constexpr double angstrom_to_m = 1.0e-10;
    return angstrom_to_m * m->lattice_constant;
}
// Material::get_atomic_volume, src/EPP/Material.h:130
static double atomic_volume(const or_material* m) { return (1.0 / 8.0) * pow(lattice_m(m), 3.0); }
// Material::get_fermi_momentum, src/EPP/Material.h:170
static double fermi_momentum(const or_material* m) { return pow(96 * M_PI * M_PI, 1.0 / 3.0) / lattice_m(m); }

// Vector3D<T>::operator* (dot), src/EPP/Vector3D.inl:66-70, and Length, :117-120
static inline double dot3(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
static inline double len3(const double* a) {
    const double w = dot3(a, a);
    return sqrt(w);
}
// compute_cos_angle, src/EPP/Vector3D.h:75-79
static inline double cos_angle3(const double* a, const double* b) {
    double dp = dot3(a, b);
    double np = len3(a) * len3(b);
    return (np < 1.0e-13) ? 1.0 : dp / (len3(a) * len3(b));
}

// ------------------------------------------------------------------------------------------------
// a1: BandStructure::GenerateBasisVectors, src/EPP/BandStructure.cpp:26-57.
static const unsigned kG2[] = {
    0,   3,   4,   8,   11,  12,  16,  19,  20,  24,  27,  32,  35,  36,  40,  43,  44,  48,  51,  52,  56,  59,  67,  68,
    75,  76,  80,  83,  84,  88,  96,  99,  104, 107, 108, 115, 116, 120, 123, 128, 131, 132, 136, 139, 140, 144, 147, 152,
    155, 160, 163, 164, 168, 171, 172, 176, 179, 180, 184, 187, 192, 195, 196, 200, 203, 204, 208, 211, 212, 216, 219, 224,
    227, 228, 232, 236, 243, 244, 248, 251, 259, 260, 264, 267, 268, 272, 275, 276, 280, 283, 291, 296, 299, 300, 304, 307,
    308, 312, 315, 320, 323, 324, 331, 332, 339, 355, 356, 360, 363, 371, 376, 384, 387, 395, 420, 451};

int or_shell_table_size(void) { return (int)(sizeof(kG2) / sizeof(kG2[0])); }

// Returns the basis size (writes min(size, capacity) vectors), or -1 if the shell count is outside
// [2, table size] (the reference prints an error and returns false there).
int or_generate_basis(unsigned nn, int32_t* G, int capacity) {
    const unsigned tsize = sizeof(kG2) / sizeof(kG2[0]);
    if (nn < 2 || nn > tsize) return -1;
    const unsigned cut  = kG2[nn - 1];
    const int      size = static_cast<int>(ceil(sqrt(static_cast<double>(cut))));
    int count = 0;
    for (int i = -size; i <= size; ++i)
        for (int j = -size; j <= size; ++j)
            for (int k = -size; k <= size; ++k) {
                // b1 = (-1,1,1), b2 = (1,-1,1), b3 = (1,1,-1)
                const int x = -i + j + k, y = i - j + k, z = i + j - k;
                const double sq = x * x + y * y + z * z;
                if (sq <= cut) {
                    if (count < capacity) {
                        G[3 * count + 0] = x;
                        G[3 * count + 1] = y;
                        G[3 * count + 2] = z;
                    }
                    ++count;
                }
            }
    return count;
}

// ------------------------------------------------------------------------------------------------
// a2: Pseudopotential::GetValue, src/EPP/Pseudopotential.cpp:24-56.
void or_pp_value(const or_material* m, int gx, int gy, int gz, const double* tau, double a, double* out) {
    const int    G2   = gx * gx + gy * gy + gz * gz;
    const double kfac = 2.0 * orc::pi / a;
    const double Gtau = kfac * (tau[0] * gx + tau[1] * gy + tau[2] * gz);
    double VS = 0.0, VA = 0.0;
    switch (G2) {
        case 3: VS = m->V3S; VA = m->V3A; break;
        case 4: VS = m->V4S; VA = m->V4A; break;
        case 8: VS = m->V8S; VA = m->V8A; break;
        case 11: VS = m->V11S; VA = m->V11A; break;
        default: break;
    }
    const double c = std::cos(Gtau);
    const double s = std::sin(Gtau);
    out[0] = VS * c;
    out[1] = VA * s;
}

// ------------------------------------------------------------------------------------------------
// a5 helpers: src/EPP/bessel_func.hpp:17-52.
static double J_neg_v(double v, double x) {
    return std::cos(-v * M_PI) * std::cyl_bessel_j(-v, x) - std::sin(-v * M_PI) * std::cyl_neumann(-v, x);
}
double or_cyl_bessel(double nu, double x) {  // generalized_bessel_cylindrical
    if (nu >= 0) return std::cyl_bessel_j(nu, x);
    return J_neg_v(nu, x);
}
// generalized_bessel: spherical j_nu(x) = sqrt(pi/2x) J_{nu+1/2}(x). The reference throws on x<0;
// the oracle returns NaN there.
double or_sph_bessel(double nu, double x) {
    constexpr double epsilon = 1e-14;
    if (x < 0) return std::numeric_limits<double>::quiet_NaN();
    if (x < epsilon && nu == 0) return 1.0;
    if (x < epsilon && nu == 1) return 0.0;
    if (x < epsilon && nu >= 2) return 0.0;
    return sqrt(M_PI / (2.0 * x)) * or_cyl_bessel(nu + 0.5, x);
}
// bessel_2nd_order_first_kind (modified spherical i_2, closed form), bessel_func.hpp:47-52
double or_bessel_i2(double x) {
    if (x == 0.0) return 0.0;
    return ((x * x + 3) * sinh(x) - 3 * x * cosh(x)) / (x * x * x);
}

// F_l_function, src/EPP/Material.cpp:87-109 (K in 1/m).
double or_F_l(const double* K1, const double* K2, double R, int l) {
    constexpr double EPSILON = 1.0e-4;
    const double     n1      = len3(K1);
    const double     n2      = len3(K2);
    if (fabs(n1 - n2) > EPSILON) {
        const double pre = pow(R, 2.0) / (n1 * n1 - n2 * n2);
        const double F   = n1 * or_sph_bessel(l + 1, n1 * R) * or_sph_bessel(l, n2 * R) -
                         n2 * or_sph_bessel(l + 1, n2 * R) * or_sph_bessel(l, n1 * R);
        return pre * F;
    } else if (n1 > EPSILON) {
        const double pre = pow(R, 3.0) / (2.0);
        const double F   = pow(or_sph_bessel(l, n1 * R), 2.0) - or_sph_bessel(l - 1, n1 * R) * or_sph_bessel(l + 1, n1 * R);
        return pre * F;
    } else {
        return (l == 0) ? pow(R, 3.0) / (3.0) : 0.0;
    }
}

// F_2_function_gaussian, src/EPP/Material.cpp:111-116.
double or_F2_gauss(const double* K1, const double* K2, double R) {
    const double n1  = len3(K1);
    const double n2  = len3(K2);
    const double arg = 0.5 * (R * R) * n1 * n2;
    return or_bessel_i2(arg) * exp(-0.25 * (n1 * n1 + n2 * n2) * R * R);
}

// a5: Material::compute_pseudopotential_non_local_correction, src/EPP/Material.cpp:139-208.
// K1n, K2n are k+G in reduced units (2pi/a); tau in metres.
void or_nl_correction(const or_material* m, const double* K1n, const double* K2n, const double* tau, double* out) {
    const double diag_factor    = pow(orc::h_bar, 2) / (2.0 * orc::m_e * orc::q_e);
    const double fourier_factor = 2.0 * M_PI / lattice_m(m);
    const double Gd[3]          = {K1n[0] - K2n[0], K1n[1] - K2n[1], K1n[2] - K2n[2]};
    const double K1[3]          = {K1n[0] * fourier_factor, K1n[1] * fourier_factor, K1n[2] * fourier_factor};
    const double K2[3]          = {K2n[0] * fourier_factor, K2n[1] * fourier_factor, K2n[2] * fourier_factor};
    const double norm_K1        = len3(K1);
    const double norm_K2        = len3(K2);
    const double cosang         = cos_angle3(K1, K2);
    const double V_pre          = 4.0 * M_PI / atomic_volume(m);
    const double legendre_0     = 1.0;
    const double legendre_2     = 0.5 * (3 * cosang * cosang - 1);
    const bool   square         = (m->nl_well == 1);

    double       V_anion   = 0;
    const double A_0_anion = m->alpha0_anion + diag_factor * m->beta0_anion * (norm_K1 * norm_K2 - pow(fermi_momentum(m), 2.0));
    const double F_0_anion = (m->R0_anion == 0.0) ? 0.0 : or_F_l(K1, K2, m->R0_anion, 0);
    V_anion += V_pre * A_0_anion * (2 * 0 + 1) * 1.0 * F_0_anion;
    if (m->A2_anion != 0) {
        const double A_2 = m->A2_anion;
        double       V2;
        if (square) {
            const double F2 = or_F_l(K1, K2, m->R2_anion, 2);
            V2              = V_pre * A_2 * (2 * 2 + 1) * legendre_2 * F2;
        } else {
            const double F2 = or_F2_gauss(K1, K2, m->R2_anion);
            V2 = 5.0 * pow(M_PI, 1.5) * (pow(m->R2_anion, 3.0) / atomic_volume(m)) * A_2 * legendre_2 * F2;
        }
        V_anion += V2;
    }

    double       V_cation   = 0;
    const double F_0_cation = (m->R0_cation == 0) ? 0.0 : or_F_l(K1, K2, m->R0_cation, 0);
    const double A_0_cation = m->alpha0_cation + m->beta0_cation * diag_factor * (norm_K1 * norm_K2 - pow(fermi_momentum(m), 2.0));
    V_cation += V_pre * A_0_cation * (2 * 0 + 1) * legendre_0 * F_0_cation;
    if (m->A2_cation != 0.0) {
        const double A_2 = m->A2_cation;
        double       V2;
        if (square) {
            const double F2 = or_F_l(K1, K2, m->R2_cation, 2);
            V2              = V_pre * A_2 * (2 * 2 + 1) * legendre_2 * F2;
        } else {
            const double F2 = or_F2_gauss(K1, K2, m->R2_cation);
            V2 = 5.0 * pow(M_PI, 1.5) * (pow(m->R2_cation, 3.0) / atomic_volume(m)) * A_2 * legendre_2 * F2;
        }
        V_cation += V2;
    }

    const double Vs   = 1.0 * (V_anion + V_cation) / 2.0;
    const double Va   = 1.0 * (V_anion - V_cation) / 2.0;
    const double a    = lattice_m(m);
    const double ta[3] = {tau[0] / a, tau[1] / a, tau[2] / a};
    const double Gtau = dot3(ta, Gd);
    out[0]            = cos(2.0 * M_PI * Gtau) * Vs;
    out[1]            = sin(2.0 * M_PI * Gtau) * Va;
}

// ------------------------------------------------------------------------------------------------
// a6: SpinOrbitCorrection, src/EPP/SpinOrbitFunctional.cpp:20-138. Returns 0, or -1 for an
// unsupported atomic period (the reference throws std::runtime_error, :58-60 and :70-72).
static double soc_B(unsigned period, const double* K, double r) {
    const double kappa = len3(K) * orc::bohr_radius / r;
    if (period == 2) return 1.0 / std::pow(1.0 + kappa * kappa, 3.0);
    if (period == 3) return (5.0 - kappa * kappa) / (5.0 * std::pow(1.0 + kappa * kappa, 4.0));
    return (5.0 - 3.0 * kappa * kappa) / (5.0 * std::pow(1.0 + kappa * kappa, 5.0));
}
static int soc_lambda(const or_material* m, const double* K, const double* Kp, double* l1, double* l2) {
    if (m->period_cation < 2 || m->period_cation > 4) return -1;
    if (m->period_anion < 2 || m->period_anion > 4) return -1;
    *l1 = m->mu_soc * soc_B(m->period_cation, K, m->radial_extent_cation) * soc_B(m->period_cation, Kp, m->radial_extent_cation);
    *l2 = m->alpha_soc * m->mu_soc * soc_B(m->period_anion, K, m->radial_extent_anion) *
          soc_B(m->period_anion, Kp, m->radial_extent_anion);
    return 0;
}
// out: 2x2 complex block, row-major [s00, s01, s10, s11] as (re, im) pairs.
int or_soc_block(const or_material* m, const double* K, const double* Kp, const double* G, const double* Gp, const double* tau,
                 double* out) {
    const double a      = lattice_m(m);
    const double kfac   = (2.0 * M_PI) / a;
    const double Kph[3] = {K[0] * kfac, K[1] * kfac, K[2] * kfac};
    const double Kpph[3] = {Kp[0] * kfac, Kp[1] * kfac, Kp[2] * kfac};
    double       l1, l2;
    if (soc_lambda(m, Kph, Kpph, &l1, &l2) != 0) return -1;
    const double ls = (l1 + l2) / 2.0;
    const double la = (l1 - l2) / 2.0;
    // compute_pauli_state_dot_product, :100-109
    const double cz   = K[0] * Kp[1] - K[1] * Kp[0];
    const double cx   = K[1] * Kp[2] - K[2] * Kp[1];
    const double cy   = K[0] * Kp[2] - K[2] * Kp[0];
    const cd     a00(cz, 0.0), a01(cx, cy), a10(cx, -cy), a11(-cz, 0.0);
    const double dG[3] = {G[0] - Gp[0], G[1] - Gp[1], G[2] - Gp[2]};
    const double Gtau  = kfac * dot3(tau, dG);
    // phase = (-1i * ls * cos) + (la * sin), :133
    const cd phase(la * std::sin(Gtau), -ls * std::cos(Gtau));
    const cd r[4] = {a00 * phase, a01 * phase, a10 * phase, a11 * phase};
    for (int q = 0; q < 4; ++q) {
        out[2 * q]     = r[q].real();
        out[2 * q + 1] = r[q].imag();
    }
    return 0;
}

// ------------------------------------------------------------------------------------------------
// a3+a4+a5+a6: Hamiltonian ctor / SetConstantNonDiagonalMatrix / SetMatrix, then the
// hermitisation of Diagonalize (src/EPP/Hamiltonian.cpp:18-48, :50-123, :127).
// H: n x n complex, column-major, interleaved (re, im); n = N, or 2N with SOC.
// Returns 0, or -1 on an unsupported SOC period.
int or_assemble(const or_material* m, const int32_t* G, int N, const double* k, int nl, int soc, double* Hout) {
    const double a = lattice_m(m);
    const double one_eight = 1.0 / 8.0;
    const double tau[3] = {one_eight * a, one_eight * a, one_eight * a};
    const double two_pi_over_a = 2.0 * M_PI / a;
    const double diag_factor = (orc::h_bar * orc::h_bar) / (2.0 * orc::m_e * orc::q_e);
    std::vector<cd> Hs((size_t)N * N);
    for (int j = 0; j < N; ++j)
        for (int i = 0; i < N; ++i) {
            double v[2];
            or_pp_value(m, G[3 * i] - G[3 * j], G[3 * i + 1] - G[3 * j + 1], G[3 * i + 2] - G[3 * j + 2], tau, a, v);
            Hs[(size_t)j * N + i] = cd(v[0], v[1]);
        }
    std::vector<double> kg((size_t)3 * N);
    for (int i = 0; i < N; ++i)
        for (int c = 0; c < 3; ++c) kg[3 * i + c] = k[c] + G[3 * i + c];
    for (int i = 0; i < N; ++i) {
        const double KG2 = two_pi_over_a * two_pi_over_a * diag_factor * dot3(&kg[3 * i], &kg[3 * i]);
        Hs[(size_t)i * N + i] += cd(KG2, 0.0);
    }
    if (nl) {
        for (int i = 0; i < N; ++i)
            for (int j = 0; j < N; ++j) {
                double v[2];
                or_nl_correction(m, &kg[3 * i], &kg[3 * j], tau, v);
                Hs[(size_t)j * N + i] += cd(v[0], v[1]);
            }
    }
    const int n = soc ? 2 * N : N;
    std::vector<cd> M((size_t)n * n);
    if (!soc) {
        M = Hs;
    } else {
        for (int j = 0; j < N; ++j)
            for (int i = 0; i < N; ++i) {
                const double Gi[3] = {(double)G[3 * i], (double)G[3 * i + 1], (double)G[3 * i + 2]};
                const double Gj[3] = {(double)G[3 * j], (double)G[3 * j + 1], (double)G[3 * j + 2]};
                double s[8];
                if (or_soc_block(m, &kg[3 * i], &kg[3 * j], Gi, Gj, tau, s) != 0) return -1;
                const cd h = Hs[(size_t)j * N + i];
                M[(size_t)j * n + i]             = h + cd(s[0], s[1]);  // UU
                M[(size_t)(j + N) * n + i]       = cd(0.0, 0.0) + cd(s[2], s[3]);  // UD
                M[(size_t)j * n + (i + N)]       = cd(0.0, 0.0) + cd(s[4], s[5]);  // DU
                M[(size_t)(j + N) * n + (i + N)] = h + cd(s[6], s[7]);  // DD
            }
    }
    // Diagonalize: matrix = 0.5 * (matrix + matrix.adjoint())
    for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) {
            const cd s = M[(size_t)j * n + i] + std::conj(M[(size_t)i * n + j]);
            Hout[2 * ((size_t)j * n + i)]     = 0.5 * s.real();
            Hout[2 * ((size_t)j * n + i) + 1] = 0.5 * s.imag();
        }
    return 0;
}

// ------------------------------------------------------------------------------------------------
// a7: the dense Hermitian eigensolver (restatement of Eigen 5.0.0 SelfAdjointEigenSolver, see
// the file header). A: n x n complex column-major (lower triangle used, destroyed). w: n
// ascending eigenvalues. Z (optional): n x n eigenvectors, column c = eigenvalue c.
// Returns 0 on success, 1 if the QR iteration hit its cap (Eigen's NoConvergence).
static void givens(double x, double z, double* c, double* s) {
    if (z == 0.0) {
        *c = (x < 0) ? -1.0 : 1.0;
        *s = 0.0;
        return;
    }
    if (x == 0.0) {
        *c = 0.0;
        *s = (z < 0) ? -1.0 : 1.0;
        return;
    }
    const double r = std::hypot(x, z);
    *c = x / r;
    *s = z / r;
}

static void qr_sweep(double* d, double* e, int start, int end, cd* Z, int n) {
    // Wilkinson shift from the trailing 2x2 block of the unreduced segment.
    const double td = (d[end - 1] - d[end]) * 0.5;
    const double ee = e[end - 1];
    double       mu = d[end];
    if (td == 0.0) {
        mu -= std::fabs(ee);
    } else if (ee != 0.0) {
        const double e2 = ee * ee;
        const double h  = std::hypot(td, ee);
        const double dn = td + (td > 0.0 ? h : -h);
        if (e2 == 0.0) mu -= ee / (dn / ee);
        else mu -= e2 / dn;
    }
    double x = d[start] - mu;
    double z = e[start];
    for (int k = start; k < end && z != 0.0; ++k) {
        double c, s;
        givens(x, z, &c, &s);
        if (k > start) e[k - 1] = c * e[k - 1] + s * z;
        const double a = d[k], b = e[k], f = d[k + 1];
        const double p = c * a + s * b, q = c * b + s * f;
        const double u = -s * a + c * b, v = -s * b + c * f;
        d[k]     = p * c + q * s;
        e[k]     = -p * s + q * c;
        d[k + 1] = -u * s + v * c;
        x        = e[k];
        if (k < end - 1) {
            z        = s * e[k + 1];
            e[k + 1] = c * e[k + 1];
        }
        if (Z) {
            cd* zk  = Z + (size_t)k * n;
            cd* zk1 = Z + (size_t)(k + 1) * n;
            for (int r = 0; r < n; ++r) {
                const cd t0 = zk[r], t1 = zk1[r];
                zk[r]       = c * t0 + s * t1;
                zk1[r]      = -s * t0 + c * t1;
            }
        }
    }
}

// Householder reduction A = Q T Q^H (lower storage). On return d, e hold T; A's strictly-lower
// part below the subdiagonal holds the reflector tails and tq the reflector scalars, so that
// Q = H_0 H_1 ... H_{n-2}, H_i = I - tq_i v_i v_i^H, v_i = (0..0, 1, A[i+2:, i]).
static void tridiagonalize(int n, cd* A, double* d, double* e, cd* tq) {
    std::vector<cd> w(n);
    for (int i = 0; i < n - 1; ++i) {
        const int m = n - i - 1;
        cd*       v = A + (size_t)i * n + (i + 1);
        double tail2 = 0.0;
        for (int r = 1; r < m; ++r) tail2 += std::norm(v[r]);
        const cd c0 = v[0];
        double beta;
        cd     h;
        if (tail2 <= DBL_MIN && c0.imag() * c0.imag() <= DBL_MIN) {
            h    = 0.0;
            beta = c0.real();
            for (int r = 1; r < m; ++r) v[r] = 0.0;
        } else {
            beta = std::sqrt(std::norm(c0) + tail2);
            if (c0.real() >= 0.0) beta = -beta;
            const cd den = c0 - beta;
            for (int r = 1; r < m; ++r) v[r] /= den;
            h = std::conj((beta - c0) / beta);
        }
        v[0]        = 1.0;
        const cd th = std::conj(h);
        // w = th * A22 * v (Hermitian product from the lower triangle, real diagonal)
        for (int r = 0; r < m; ++r) w[r] = 0.0;
        for (int c = 0; c < m; ++c) {
            const cd* col = A + (size_t)(i + 1 + c) * n + (i + 1);
            w[c] += col[c].real() * v[c];
            for (int r = c + 1; r < m; ++r) {
                w[r] += col[r] * v[c];
                w[c] += std::conj(col[r]) * v[r];
            }
        }
        for (int r = 0; r < m; ++r) w[r] *= th;
        cd dp = 0.0;
        for (int r = 0; r < m; ++r) dp += std::conj(w[r]) * v[r];
        const cd alpha = th * (-0.5) * dp;
        for (int r = 0; r < m; ++r) w[r] += alpha * v[r];
        // A22 -= v w^H + w v^H (lower triangle)
        for (int c = 0; c < m; ++c) {
            cd* col = A + (size_t)(i + 1 + c) * n + (i + 1);
            for (int r = c; r < m; ++r) col[r] -= v[r] * std::conj(w[c]) + w[r] * std::conj(v[c]);
        }
        v[0]  = beta;
        tq[i] = th;
    }
    for (int r = 0; r < n; ++r) d[r] = A[(size_t)r * n + r].real();
    for (int r = 0; r < n - 1; ++r) e[r] = A[(size_t)r * n + r + 1].real();
}

int or_eigh(int n, double* Ain, double* w, double* Zout) {
    cd* A = reinterpret_cast<cd*>(Ain);
    if (n <= 0) return 0;
    if (n == 1) {
        w[0] = A[0].real();
        if (Zout) { Zout[0] = 1.0; Zout[1] = 0.0; }
        return 0;
    }
    double scale = 0.0;
    for (int j = 0; j < n; ++j)
        for (int i = j; i < n; ++i) scale = std::max(scale, std::abs(A[(size_t)j * n + i]));
    if (scale == 0.0) scale = 1.0;
    for (int j = 0; j < n; ++j)
        for (int i = j; i < n; ++i) A[(size_t)j * n + i] /= scale;
    std::vector<double> d(n), e(n - 1);
    std::vector<cd>     tq(n - 1);
    tridiagonalize(n, A, d.data(), e.data(), tq.data());
    cd* Z = reinterpret_cast<cd*>(Zout);
    if (Z) {
        // Q = H_0 (H_1 (... H_{n-2})), built backwards on the trailing block.
        for (size_t q = 0; q < (size_t)n * n; ++q) Z[q] = 0.0;
        for (int r = 0; r < n; ++r) Z[(size_t)r * n + r] = 1.0;
        for (int i = n - 2; i >= 0; --i) {
            const int m = n - i - 1;
            std::vector<cd> v(m);
            v[0] = 1.0;
            for (int r = 1; r < m; ++r) v[r] = A[(size_t)i * n + i + 1 + r];
            for (int c = i + 1; c < n; ++c) {
                cd* col = Z + (size_t)c * n + (i + 1);
                cd  s   = 0.0;
                for (int r = 0; r < m; ++r) s += std::conj(v[r]) * col[r];
                s *= tq[i];
                for (int r = 0; r < m; ++r) col[r] -= s * v[r];
            }
        }
    }
    // Implicit symmetric QR (Eigen's computeFromTridiagonal_impl structure).
    const int    maxIter = 30;
    const double considerAsZero = DBL_MIN;
    const double precision_inv  = 1.0 / DBL_EPSILON;
    int end = n - 1, start = 0, iter = 0;
    while (end > 0) {
        for (int i = start; i < end; ++i) {
            if (std::fabs(e[i]) < considerAsZero) e[i] = 0.0;
            else {
                const double sc = precision_inv * e[i];
                if (sc * sc <= (std::fabs(d[i]) + std::fabs(d[i + 1]))) e[i] = 0.0;
            }
        }
        while (end > 0 && e[end - 1] == 0.0) end--;
        if (end <= 0) break;
        iter++;
        if (iter > maxIter * n) break;
        start = end - 1;
        while (start > 0 && e[start - 1] != 0.0) start--;
        qr_sweep(d.data(), e.data(), start, end, Z, n);
    }
    const int info = (iter <= maxIter * n) ? 0 : 1;
    if (info == 0) {
        for (int i = 0; i < n - 1; ++i) {
            int kmin = i;
            for (int j = i + 1; j < n; ++j)
                if (d[j] < d[kmin]) kmin = j;
            if (kmin != i) {
                std::swap(d[i], d[kmin]);
                if (Z)
                    for (int r = 0; r < n; ++r) std::swap(Z[(size_t)i * n + r], Z[(size_t)kmin * n + r]);
            }
        }
    }
    for (int i = 0; i < n; ++i) w[i] = d[i] * scale;
    return info;
}

// ------------------------------------------------------------------------------------------------
// a8: Hamiltonian::compute_gradient_at_level, src/EPP/Hamiltonian.cpp:146-194 (eV*m).
// ev: eigenvector of length n (N, or 2N with SOC), complex interleaved.
void or_gradient(const or_material* m, const int32_t* G, int N, const double* k, const double* ev, int n, double* grad) {
    const double two_pi_over_a = 2.0 * M_PI / lattice_m(m);
    constexpr double diag_factor = (orc::h_bar * orc::h_bar) / (2.0 * orc::m_e * orc::q_e);
    const double pref_frac = 2.0 * diag_factor * (two_pi_over_a * two_pi_over_a);
    double s[3] = {0.0, 0.0, 0.0};
    const bool has_spin = (n == 2 * N);
    for (int i = 0; i < N; ++i) {
        const double kg[3] = {k[0] + G[3 * i], k[1] + G[3 * i + 1], k[2] + G[3 * i + 2]};
        double wgt = ev[2 * i] * ev[2 * i] + ev[2 * i + 1] * ev[2 * i + 1];
        if (has_spin) {
            const double* e2 = ev + 2 * (i + N);
            wgt = wgt + (e2[0] * e2[0] + e2[1] * e2[1]);
        }
        for (int c = 0; c < 3; ++c) s[c] = s[c] + kg[c] * wgt;
    }
    const double frac_to_phys = 1.0 / two_pi_over_a;
    for (int c = 0; c < 3; ++c) grad[c] = (s[c] * pref_frac) * frac_to_phys;
}

// ------------------------------------------------------------------------------------------------
// a9: BandStructure::Compute_parallel, src/EPP/BandStructure.cpp:151-201.
// E: nk x nb (row-major). grad (optional): nk x nb x 3. vecs (optional): nk x nb x n complex.
// status: nk ints (0 ok, 1 no convergence, -1 unsupported SOC period).
int or_band_structure(const or_material* m, const int32_t* G, int N, const double* kpts, int64_t nk, int nb, int nl, int soc,
                      int want_grad, int nthreads, double* E, double* grad, double* vecs, int32_t* status) {
    const int n = soc ? 2 * N : N;
    const bool want_vec = (grad != nullptr && want_grad) || vecs != nullptr;
    int bad = 0;
#pragma omp parallel num_threads(nthreads > 0 ? nthreads : 1) reduction(+ : bad)
    {
        std::vector<double> H((size_t)2 * n * n), w(n), Z(want_vec ? (size_t)2 * n * n : 0);
#pragma omp for schedule(dynamic)
        for (int64_t ik = 0; ik < nk; ++ik) {
            const double* k = kpts + 3 * ik;
            int st = or_assemble(m, G, N, k, nl, soc, H.data());
            if (st == 0) st = or_eigh(n, H.data(), w.data(), want_vec ? Z.data() : nullptr);
            if (status) status[ik] = st;
            if (st != 0) { ++bad; continue; }
            for (int b = 0; b < nb && b < n; ++b) {
                E[ik * nb + b] = w[b];
                if (want_grad && grad) or_gradient(m, G, N, k, &Z[(size_t)2 * b * n], n, &grad[(ik * nb + b) * 3]);
                if (vecs) std::memcpy(&vecs[((size_t)ik * nb + b) * 2 * n], &Z[(size_t)2 * b * n], sizeof(double) * 2 * n);
            }
        }
    }
    return bad;
}

// ------------------------------------------------------------------------------------------------
// a10: BandStructure::FindBandGap + AdjustValues, src/EPP/BandStructure.cpp:203-262.
// Returns the band gap; shifts E in place. found (optional) receives FindBandGap's result.
double or_adjust_values(double* E, int64_t nk, int nb, int soc, int minCondZero, int* found) {
    double maxVal = 0.0, minCond = 0.0;  // uninitialised in the reference when nothing is found early
    bool   ok     = false;
    if (!(nk == 0 || nb < 2)) {
        maxVal = std::numeric_limits<double>::lowest();
        minCond = std::numeric_limits<double>::infinity();
        double fallback = maxVal;
        for (int lo = 2; lo + 1 < nb; ++lo) {
            maxVal = std::numeric_limits<double>::lowest();
            minCond = std::numeric_limits<double>::infinity();
            for (int64_t ik = 0; ik < nk; ++ik) {
                maxVal = std::max(maxVal, E[ik * nb + lo]);
                minCond = std::min(minCond, E[ik * nb + lo + 1]);
            }
            if (lo == 3) fallback = maxVal;
            if (maxVal + 0.35 < minCond) { ok = true; break; }
        }
        if (!ok) maxVal = fallback;
    }
    double gap = ok ? (minCond - maxVal) : 0.0;
    const int nval = soc ? 8 : 4;
    for (int64_t ik = 0; ik < nk; ++ik)
        for (int b = 0; b < nb; ++b) {
            if (b < nval) E[ik * nb + b] -= maxVal;
            else if (minCondZero) E[ik * nb + b] -= minCond;
            else E[ik * nb + b] -= maxVal;
        }
    if (found) *found = ok ? 1 : 0;
    return gap;
}

// ------------------------------------------------------------------------------------------------
// a12: SymmetryPoints ctor + GeneratePoints, src/EPP/SymmetryPoints.cpp:21-28, :47-147.
// labels: one character per node from {L,G,X,W,K,U}. Returns the number of points written
// (<= capacity), or -1 on invalid arguments (the reference throws std::invalid_argument).
static bool sym_point(char c, double* p) {
    switch (c) {
        case 'L': p[0] = 0.5; p[1] = 0.5; p[2] = 0.5; return true;
        case 'G': p[0] = 0.; p[1] = 0.; p[2] = 0.; return true;
        case 'X': p[0] = 1.; p[1] = 0.; p[2] = 0.; return true;
        case 'W': p[0] = 1.; p[1] = 0.5; p[2] = 0.; return true;
        case 'K': p[0] = 0.75; p[1] = 0.75; p[2] = 0.; return true;
        case 'U': p[0] = 1.; p[1] = 0.25; p[2] = 0.25; return true;
        default: return false;
    }
}
int or_generate_path(const char* labels, unsigned nrPoints, double* out, int capacity, uint32_t* sympos) {
    const size_t M = std::strlen(labels);
    if (M < 2 || nrPoints < M) return -1;
    std::vector<double> nodes(3 * M);
    for (size_t i = 0; i < M; ++i)
        if (!sym_point(labels[i], &nodes[3 * i])) return -1;
    std::vector<double> segLen(M - 1, 0.0);
    for (size_t i = 1; i < M; ++i) {
        const double d[3] = {nodes[3 * i] - nodes[3 * i - 3], nodes[3 * i + 1] - nodes[3 * i - 2], nodes[3 * i + 2] - nodes[3 * i - 1]};
        segLen[i - 1] = len3(d);
    }
    const double totalLen = std::accumulate(segLen.begin(), segLen.end(), 0.0);
    const unsigned R = nrPoints - (unsigned)M;
    int cnt = 0;
    auto push = [&](const double* p) {
        if (cnt < capacity) std::memcpy(out + 3 * cnt, p, 3 * sizeof(double));
        ++cnt;
    };
    int nsym = 0;
    if (totalLen == 0.0) {
        for (size_t j = 0; j < M; ++j) { sympos[nsym++] = cnt; push(&nodes[3 * j]); }
        for (unsigned i = 0; i < R; ++i) push(&nodes[3 * (M - 1)]);
        return cnt;
    }
    std::vector<unsigned> mseg(M - 1, 0);
    std::vector<double>   want(M - 1, 0.0);
    std::vector<size_t>   order(M - 1);
    for (size_t s = 0; s < M - 1; ++s) {
        want[s]  = (segLen[s] / totalLen) * static_cast<double>(R);
        mseg[s]  = static_cast<unsigned>(std::floor(want[s]));
        order[s] = s;
    }
    const unsigned assigned = std::accumulate(mseg.begin(), mseg.end(), 0u);
    const unsigned rem = R - assigned;
    std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) {
        return (want[a] - std::floor(want[a])) > (want[b] - std::floor(want[b]));
    });
    for (unsigned i = 0; i < rem; ++i) ++mseg[order[i]];
    sympos[nsym++] = cnt;
    push(&nodes[0]);
    for (size_t s = 0; s < M - 1; ++s) {
        const double* A = &nodes[3 * s];
        const double* B = &nodes[3 * s + 3];
        const unsigned ms = mseg[s];
        if (ms > 0) {
            const double d[3] = {B[0] - A[0], B[1] - A[1], B[2] - A[2]};
            const double denom = static_cast<double>(ms + 1);
            for (unsigned i = 1; i <= ms; ++i) {
                const double t = static_cast<double>(i) / denom;
                const double p[3] = {A[0] + d[0] * t, A[1] + d[1] * t, A[2] + d[2] * t};
                push(p);
            }
        }
        sympos[nsym++] = cnt;
        push(B);
    }
    return cnt;
}

// MeshBZ::is_irreducible_wedge (src/BZ_MESH/bz_mesh.cpp:1176-1183), on a reduced k-point.
int or_is_irreducible_wedge(const double* kr) {
    const double eps = 1e-12;
    const double x = kr[0], y = kr[1], z = kr[2];
    return (z >= -eps) && (z <= y + eps) && (y <= x + eps) && (x <= 1.0 + eps) && ((x + y + z) <= 1.5 + eps);
}

// apply_same_symmetry_operation (src/BZ_MESH/bz_mesh.cpp:1312-1381): the signed permutation that
// maps k_iw onto k_bz, found component by component of k_bz (the first unused component of k_iw
// whose magnitude matches within 1e-8 * max(1, largest magnitude)); perm[j] and sign[j] such that
// v_bz[j] = sign[j] * v[perm[j]]. Returns 0 (and the identity) when no signed permutation matches,
// where the reference returns v unchanged.
int or_symmetry_operation(const double* a, const double* b, int* perm, int* sign) {
    const double eps = 1e-8;
    int          used[3] = {0, 0, 0};
    double       scale = 0.0;
    for (int q = 0; q < 3; ++q) {
        scale = std::max(scale, std::fabs(a[q]));
        scale = std::max(scale, std::fabs(b[q]));
    }
    if (scale < 1.0) scale = 1.0;
    const double tol = eps * scale;
    for (int jb = 0; jb < 3; ++jb) {
        int found = 0;
        for (int ia = 0; ia < 3; ++ia) {
            if (used[ia]) continue;
            if (std::fabs(std::fabs(a[ia]) - std::fabs(b[jb])) <= tol) {
                perm[jb] = ia;
                used[ia] = 1;
                if (std::fabs(a[ia]) > tol) {
                    const int sa = (a[ia] >= 0.0) ? 1 : -1;
                    const int sb = (b[jb] >= 0.0) ? 1 : -1;
                    sign[jb]     = sb * sa;
                } else {
                    sign[jb] = (b[jb] >= 0.0) ? 1 : -1;
                }
                found = 1;
                break;
            }
        }
        if (!found) {
            for (int q = 0; q < 3; ++q) {
                perm[q] = q;
                sign[q] = 1;
            }
            return 0;
        }
    }
    return 1;
}

}  // extern "C"
