// assemble.cu -- H(k) assembly on the device (local + kinetic + nonlocal + spin-orbit), FP64.
//
// Replaces, per k-point, Hamiltonian::SetMatrix (src/EPP/Hamiltonian.cpp:50-123) with
// Pseudopotential::GetValue (Pseudopotential.cpp:24-56, precomputed per context on the host),
// Material::compute_pseudopotential_non_local_correction + F_l_function + F_2_function_gaussian
// (Material.cpp:87-208), the spherical Bessel helpers (bessel_func.hpp:17-52) and
// SpinOrbitCorrection::compute_soc_contribution (SpinOrbitFunctional.cpp:20-138).
//
// This translation unit is compiled with --fmad=false: every product and sum is rounded
// separately, in the reference's operand order, so the kinetic diagonal, |K| and the F_l branch
// selection (|K1|-|K2| > 1e-4) are bit-identical to an IEEE evaluation of the reference's code.
//
// Two kernels per chunk of k-points:
//   k_rows      one thread per (k, G_i): k+G, K = (k+G) 2pi/a, |K|, the kinetic term and all
//               quantities that depend on a single plane wave (spherical Bessel values at |K| R,
//               gaussian-well exponentials, spin-orbit radial factors B(|K|)).
//   k_assemble_tiles (no spin-orbit) one CTA per 32 x 32 tile of the lower triangle of the N x N
//               matrix: the tile and, through a shared-memory transpose, its Hermitian mirror are
//               written with coalesced stores into the FULL column-major H;
//   k_assemble  (spin-orbit) one thread per lower-triangle element (i >= j) of the scalar N x N
//               problem, writing the four spin blocks [[UU, UD], [DU, DD]] of the 2N x 2N matrix
//               and their mirrors.
//   Both optionally write an FP32 copy for the mixed path, and store H itself as FP64 or as FP32
//   (hi, lo) pairs (the mixed path's Rayleigh-Ritz operand). When H(k) is exactly real (no SOC, no
//   antisymmetric form factors, identical anion/cation nonlocal parameters) only real parts are
//   stored.
#include <type_traits>

#include "uepm_common.cuh"
#include "ctx_internal.h"
#include "uepm_kernels.h"

namespace uepm {

// ------------------------------------------------------------------------------------------------
// Spherical Bessel functions j_nu(x), nu = -1..3, with the reference's generalized_bessel edge
// cases (bessel_func.hpp:29-45): for x < 1e-14, j_0 = 1 and j_{nu>=1} = 0. Written from the
// mathematics (Abramowitz & Stegun 10.1.2 power series for x < 2.5, the closed forms / upward
// recurrence j_{n+1} = (2n+1)/x j_n - j_{n-1} above), not from any library's code.
__device__ __forceinline__ double sph_series(int nu, double x) {
    // x^nu / (2nu+1)!! * sum_k (-x^2/2)^k / (k! (2nu+3)(2nu+5)...(2nu+2k+1))
    const double h    = -0.5 * x * x;
    double       term = 1.0, sum = 1.0;
#pragma unroll
    for (int k = 1; k <= 16; ++k) {
        term = term * h / (double)(k * (2 * nu + 2 * k + 1));
        sum  = sum + term;
    }
    double pre = 1.0;
    double dfac = 1.0;
    for (int q = 1; q <= nu; ++q) {
        pre  = pre * x;
        dfac = dfac * (double)(2 * q + 1);
    }
    return pre / dfac * sum;
}

// Fills j[0..2] with j_{l-1}, j_l, j_{l+1} at x, for l = 0 or l = 2.
__device__ void sph_triple(int l, double x, double* j) {
    constexpr double eps14 = 1e-14;
    if (x < eps14) {
        // generalized_bessel: nu == 0 -> 1, nu >= 1 -> 0; nu == -1 is not special-cased there
        // and evaluates cos(x)/x (only reachable with x > 1e-14 from F_l's branches).
        if (l == 0) {
            j[0] = cos(x) / x;
            j[1] = 1.0;
            j[2] = 0.0;
        } else {
            j[0] = j[1] = j[2] = 0.0;
        }
        return;
    }
    double s, c;
    sincos(x, &s, &c);
    // j_{-1} = cos(0.5 pi) j_0 + cos(x)/x: the reference's J_{-1/2} via J_neg_v keeps the
    // cos(0.5 pi) = 6.123233995736766e-17 weight of J_{1/2}.
    const double jm1 = c / x;
    const double j0  = (x < 2.5) ? sph_series(0, x) : s / x;
    if (l == 0) {
        j[0] = jm1 + 6.123233995736766e-17 * j0;
        j[1] = j0;
        j[2] = (x < 2.5) ? sph_series(1, x) : j0 / x - jm1;
        return;
    }
    if (x < 2.5) {
        j[0] = sph_series(1, x);
        j[1] = sph_series(2, x);
        j[2] = sph_series(3, x);
    } else {
        const double j1 = j0 / x - jm1;
        const double j2 = 3.0 * j1 / x - j0;
        const double j3 = 5.0 * j2 / x - j1;
        j[0] = j1;
        j[1] = j2;
        j[2] = j3;
    }
}

// Modified spherical i_2 by the reference's closed form (bessel_func.hpp:47-52).
// bessel_2nd_order_first_kind (bessel_func.hpp:47-52): i2(x) = ((x^2 + 3) sinh x - 3 x cosh x) / x^3,
// the reference's closed form. Above x = 2 sinh and cosh come from one exponential,
// (e^x -+ e^-x) / 2 (relative error ~ eps there, the numerator cancels by < 10x); below, the
// library's sinh and cosh (the closed form cancels to ~3 eps / x^2 near 0).
__device__ __forceinline__ double bessel_i2(double x) {
    if (x == 0.0) return 0.0;
    double sh, ch;
    if (x > 2.0) {
        const double E = exp(x), Ei = 1.0 / E;
        sh             = 0.5 * (E - Ei);
        ch             = 0.5 * (E + Ei);
    } else {
        sh = sinh(x);
        ch = cosh(x);
    }
    return ((x * x + 3) * sh - 3 * x * ch) / (x * x * x);
}

__device__ __forceinline__ double soc_B(unsigned period, double nK, double bohr, double r) {
    const double kappa = nK * bohr / r;
    const double q     = 1.0 + kappa * kappa;
    if (period == 2) return 1.0 / pow(q, 3.0);
    if (period == 3) return (5.0 - kappa * kappa) / (5.0 * pow(q, 4.0));
    return (5.0 - 3.0 * kappa * kappa) / (5.0 * pow(q, 5.0));
}

__global__ void k_rows(const DevParams P, const double* __restrict__ kpts, const int* __restrict__ G,
                       double* __restrict__ rows, int batch, float2* __restrict__ rows32) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= batch * P.N) return;
    const int     b = idx / P.N, i = idx - b * P.N;
    const double* k = kpts + 3 * (size_t)b;
    double*       R = rows + (size_t)idx * ROW_STRIDE;
    const double  kg[3] = {k[0] + G[3 * i], k[1] + G[3 * i + 1], k[2] + G[3 * i + 2]};
    R[RF_KGX] = kg[0];
    R[RF_KGY] = kg[1];
    R[RF_KGZ] = kg[2];
    R[RF_KIN] = P.kin_pref * (kg[0] * kg[0] + kg[1] * kg[1] + kg[2] * kg[2]);
    if (!P.nl && !P.soc) return;
    const double K[3] = {kg[0] * P.ff, kg[1] * P.ff, kg[2] * P.ff};
    const double nK   = sqrt(K[0] * K[0] + K[1] * K[1] + K[2] * K[2]);
    R[RF_KX] = K[0];
    R[RF_KY] = K[1];
    R[RF_KZ] = K[2];
    R[RF_NK] = nK;
    if (P.nl) {  // the cation's values only where its parameters differ (nl_element reads them then)
        R[P.square ? RF_INVK_SQUARE : RF_INVK_GAUSS] = (nK > 0.0) ? 1.0 / nK : 0.0;
        if (P.has_R0a) sph_triple(0, nK * P.R0a, R + RF_J0A);
        if (P.has_R0c && !P.same_nl) sph_triple(0, nK * P.R0c, R + RF_J0C);
        if (P.square) {
            if (P.has_A2a) sph_triple(2, nK * P.R2a, R + RF_J2A);
            if (P.has_A2c && !P.same_nl) sph_triple(2, nK * P.R2c, R + RF_J2C);
        } else {
            R[RF_GEA] = exp(-0.25 * (nK * nK) * P.R2a * P.R2a);
            if (!P.same_nl) R[RF_GEC] = exp(-0.25 * (nK * nK) * P.R2c * P.R2c);
        }
    }
    if (P.soc) {
        R[RF_BC] = soc_B(P.pc, nK, P.bohr, P.rc);
        R[RF_BA] = soc_B(P.pa, nK, P.bohr, P.ra);
    }
    if (rows32 && (P.nl || P.soc)) {  // double-single copy for the mixed path's FP32-pipe element
        float2* R32 = rows32 + (size_t)idx * ROW_STRIDE;
        auto    put = [&](int f) {
            const ds v = ds_of_double(R[f]);
            R32[f]     = make_float2(v.h, v.l);
        };
        put(RF_KIN);
        if (P.soc) {
            put(RF_KGX);
            put(RF_KGY);
            put(RF_KGZ);
            put(RF_BC);
            put(RF_BA);
        }
    }
    if (rows32 && P.nl) {
        float2* R32 = rows32 + (size_t)idx * ROW_STRIDE;
        auto    put = [&](int f) {
            const ds v = ds_of_double(R[f]);
            R32[f]     = make_float2(v.h, v.l);
        };
        put(RF_KX);
        put(RF_KY);
        put(RF_KZ);
        put(RF_NK);
        put(P.square ? RF_INVK_SQUARE : RF_INVK_GAUSS);
        const ds ns = ds_of_double(nK / P.ff);
        R32[P.square ? RF_NKS32_SQUARE : RF_NKS32_GAUSS] = make_float2(ns.h, ns.l);
        for (int q = 0; q < 3; ++q) {
            if (P.has_R0a) put(RF_J0A + q);
            if (P.has_R0c && !P.same_nl) put(RF_J0C + q);
            if (P.square && P.has_A2a) put(RF_J2A + q);
            if (P.square && P.has_A2c && !P.same_nl) put(RF_J2C + q);
        }
        if (!P.square) {
            put(RF_GEA);
            if (!P.same_nl) put(RF_GEC);
        }
    }
}

// F_l_function (Material.cpp:87-109) from per-row Bessel triples ja (row i) and jb (row j). The
// branch (|n1 - n2| > 1e-4, evaluated on bit-identical |K|) is the reference's; in the first branch
// R^2 / (n1^2 - n2^2) is taken as R^2 times the reciprocal inv = 1 / (n1^2 - n2^2) that all F_l
// terms of the element share (one FP64 division instead of one per term; the product differs from
// the quotient by at most an ulp).
__device__ __forceinline__ bool F_l_far(double n1, double n2) { return fabs(n1 - n2) > 1.0e-4; }
__device__ __forceinline__ double F_l(int l, double n1, double n2, bool far, double inv, const double* ja, const double* jb,
                                      double R2, double R3h, double R3t) {
    constexpr double EPSILON = 1.0e-4;
    if (far) {
        const double pre = R2 * inv;
        const double F   = n1 * ja[2] * jb[1] - n2 * jb[2] * ja[1];
        return pre * F;
    } else if (n1 > EPSILON) {
        const double F = ja[1] * ja[1] - ja[0] * ja[2];
        return R3h * F;
    }
    return (l == 0) ? R3t : 0.0;
}

// compute_pseudopotential_non_local_correction (Material.cpp:139-208); (pc, ps) = cos, sin of the
// structure phase 2 pi (tau/a).(G_i - G_j). Where anion and cation carry the same parameters their
// two terms are equal bit for bit (the same operations on the same values), so the cation's is not
// recomputed: Vs = (Va + Va) / 2 = Va and Vas = 0 exactly.
// The angle's cosine takes the per-row reciprocals of |K| (one product instead of an FP64 division per
// element, within 2 ulp of dp / (n1 n2)), and the F_l reciprocal is formed only where an F_l term
// exists (an l = 0 well, or square l = 2 wells).
__device__ cx<double> nl_element(const DevParams& P, const double* Ri, const double* Rj, double pc, double ps) {
    const double n1   = Ri[RF_NK], n2 = Rj[RF_NK];
    const double dp   = Ri[RF_KX] * Rj[RF_KX] + Ri[RF_KY] * Rj[RF_KY] + Ri[RF_KZ] * Rj[RF_KZ];
    const double np   = n1 * n2;
    const int    fi   = P.square ? RF_INVK_SQUARE : RF_INVK_GAUSS;
    const double ca   = (np < 1.0e-13) ? 1.0 : dp * (Ri[fi] * Rj[fi]);
    const double lg2  = 0.5 * (3 * ca * ca - 1);
    const double t    = n1 * n2 - P.kF2;
    const bool   far  = F_l_far(n1, n2);
    const bool   F_on = P.has_R0a || P.has_R0c || (P.square && (P.has_A2a || P.has_A2c));
    const double inv  = (far && F_on) ? 1.0 / (n1 * n1 - n2 * n2) : 0.0;

    double       Va  = 0.0;
    const double A0a = P.alpha0a + P.nl_df * P.beta0a * t;
    const double F0a = P.has_R0a ? F_l(0, n1, n2, far, inv, Ri + RF_J0A, Rj + RF_J0A, P.R0a2, P.R0a3h, P.R0a3t) : 0.0;
    Va               = Va + P.Vpre * A0a * F0a;
    if (P.has_A2a) {
        double V2;
        if (P.square) {
            const double F2 = F_l(2, n1, n2, far, inv, Ri + RF_J2A, Rj + RF_J2A, P.R2a2, P.R2a3h, 0.0);
            V2              = P.Vpre * P.A2a * 5 * lg2 * F2;
        } else {
            const double arg = 0.5 * (P.R2a * P.R2a) * n1 * n2;
            const double F2  = bessel_i2(arg) * (Ri[RF_GEA] * Rj[RF_GEA]);
            V2               = P.gpre_a * P.A2a * lg2 * F2;
        }
        Va = Va + V2;
    }
    if (P.same_nl) return mk(pc * Va, ps * 0.0);
    double       Vc  = 0.0;
    const double F0c = P.has_R0c ? F_l(0, n1, n2, far, inv, Ri + RF_J0C, Rj + RF_J0C, P.R0c2, P.R0c3h, P.R0c3t) : 0.0;
    const double A0c = P.alpha0c + P.beta0c * P.nl_df * t;
    Vc               = Vc + P.Vpre * A0c * F0c;
    if (P.has_A2c) {
        double V2;
        if (P.square) {
            const double F2 = F_l(2, n1, n2, far, inv, Ri + RF_J2C, Rj + RF_J2C, P.R2c2, P.R2c3h, 0.0);
            V2              = P.Vpre * P.A2c * 5 * lg2 * F2;
        } else {
            const double arg = 0.5 * (P.R2c * P.R2c) * n1 * n2;
            const double F2  = bessel_i2(arg) * (Ri[RF_GEC] * Rj[RF_GEC]);
            V2               = P.gpre_c * P.A2c * lg2 * F2;
        }
        Vc = Vc + V2;
    }
    const double Vs  = 1.0 * (Va + Vc) / 2.0;
    const double Vas = 1.0 * (Va - Vc) / 2.0;
    return mk(pc * Vs, ps * Vas);
}

// The square-well element of nl_element in double-single arithmetic on the FP32 pipe (the mixed
// path's matrix for the Rayleigh-Ritz products, which it stores as FP32 pairs anyway): the same
// formula and branches (taken on the double-single values), from the rows' double-single copies
// (rows32) and the structure phase's (pc, ps). The F_l terms are carried times 4 pi / volume (VF_l
// below) and the far branch in norms of units 2 pi / a, so every intermediate stays inside FP32's
// exponent range; the regrouped products differ from the FP64 element by a few units of 2^-46.
__device__ __forceinline__ ds rd(const float2* R, int f) { return ds{R[f].x, R[f].y}; }
// Vpre F_l; n1s, n2s: the norms in units of 2 pi / a; inv = 1 / (n1s^2 - n2s^2).
__device__ __forceinline__ ds VF_l_ds(int l, ds n1s, bool far, bool big, ds inv, const float2* Ri, const float2* Rj,
                                      int f, ds n2s, ds VR2s, ds VR3h, ds VR3t) {
    if (far) {
        const ds F = ds_sub(ds_mul(ds_mul(n1s, rd(Ri, f + 2)), rd(Rj, f + 1)), ds_mul(ds_mul(n2s, rd(Rj, f + 2)), rd(Ri, f + 1)));
        return ds_mul(ds_mul(VR2s, inv), F);
    } else if (big) {
        const ds F = ds_sub(ds_mul(rd(Ri, f + 1), rd(Ri, f + 1)), ds_mul(rd(Ri, f), rd(Ri, f + 2)));
        return ds_mul(VR3h, F);
    }
    return (l == 0) ? VR3t : ds{0.f, 0.f};
}
// Double-single constants from double values (rounded at compile time): ln 2 in three FP32 parts
// (the first of 16 bits, so that k L1 is exact for |k| < 256) from the double-double value of ln 2,
// and the reciprocal factorials of the exponential's Taylor series.
constexpr double kLn2Hi = 0.6931471805599453, kLn2Lo = 2.3190468138462996e-17;
constexpr float  kLn2P1 = 0.693145751953125f;  // 45426 / 65536
constexpr float  kLn2P2 = (float)(kLn2Hi - 0.693145751953125);
constexpr float  kLn2P3 = (float)((kLn2Hi - 0.693145751953125 - (double)kLn2P2) + kLn2Lo);
__host__ __device__ constexpr double inv_fact(int j) { return j <= 1 ? 1.0 : inv_fact(j - 1) / j; }
// Horner steps p <- p y + 1 / J!, ..., p y + 1 / 0! with the coefficients split into FP32 pairs at
// compile time
template <int J>
__device__ __forceinline__ ds horner_exp_ds(ds p, ds y) {
    constexpr double c  = inv_fact(J);
    constexpr float  ch = (float)c, cl = (float)(c - (double)(float)c);
    p = ds_add(ds_mul(p, y), ds{ch, cl});
    if constexpr (J > 0) return horner_exp_ds<J - 1>(p, y);
    else return p;
}

// e^x for 2 < x <= 80 in double-single arithmetic: Cody and Waite's argument reduction
// (W. J. Cody, W. Waite, Software Manual for the Elementary Functions, 1980) x = k ln 2 + r with
// |r| <= ln 2 / 2, the Taylor series of e^r to degree 13 by Horner's rule (remainder below 2^-50),
// then 2^k. Relative error about 2^-47 (checked against a 40-digit reference over the range).
__device__ __forceinline__ ds ds_exp_pos(ds x) {
    const float k = rintf(__fmul_rn(x.h, 1.4426950408889634f));
    ds          r = ds_add(x, ds{-k * kLn2P1, 0.f});  // k L1 exact; the difference exact (close operands)
    r             = ds_add(r, ds_mulf(ds{-kLn2P2, -kLn2P3}, k));
    constexpr float c13h = (float)inv_fact(13), c13l = (float)(inv_fact(13) - (double)(float)inv_fact(13));
    const ds  p    = horner_exp_ds<12>(ds{c13h, c13l}, r);
    const int ki   = (int)k;
    return ds{ldexpf(p.h, ki), ldexpf(p.l, ki)};
}

// The gaussian well's i2(x) = ((x^2 + 3) sinh x - 3 x cosh x) / x^3 (the modified spherical Bessel
// function of order 2; the reference's closed form, bessel_func.hpp:47-52) for 2 < x <= 80, in
// double-single with e^x from ds_exp_pos. At x <= 2 the closed form cancels (absolute error ~3 eps /
// x^2 in the reference's FP64 evaluation): callers take the FP64 bessel_i2 of the FP64 argument
// there, the very value the FP64 path (and the reference) uses, so that the two paths do not differ
// by that cancellation; x > 80 goes to the FP64 element (e^x would leave FP32's range).
__device__ __forceinline__ ds i2_ds(ds x) {
    const ds E  = ds_exp_pos(x);
    const ds Ei = ds_div(ds{1.f, 0.f}, E);
    const ds sh = ds_mulf(ds_sub(E, Ei), 0.5f), ch = ds_mulf(ds_add(E, Ei), 0.5f);
    const ds x2 = ds_mul(x, x);
    const ds num = ds_sub(ds_mul(ds_add(x2, ds{3.f, 0.f}), sh), ds_mulf(ds_mul(x, ch), 3.f));
    return ds_div(num, ds_mul(x2, x));
}

// i2 of the gaussian well with radius R: x = R^2 / 2 n1 n2, from the FP64 norms where x <= 2 (the
// FP64 element's own operands and function), else in double-single (R2h = R^2 / 2 as a pair, np =
// n1 n2 in double-single).
__device__ __forceinline__ ds i2_gauss(double R, ds R2h, ds np, double n1d, double n2d) {
    const double argd = 0.5 * (R * R) * n1d * n2d;
    return argd <= 2.0 ? ds_of_double(bessel_i2(argd)) : i2_ds(ds_mul(R2h, np));
}

// far: the reference's branch |n1 - n2| > 1e-4, decided on the FP64 norms by the caller (the
// double-single difference is not resolved finely enough for it).
// n1d, n2d: the FP64 norms (the gaussian well's argument at x <= 2, as the FP64 element forms it).
__device__ void nl_element_ds(const DevParams& P, const DevParamsDS& Q, const float2* Ri, const float2* Rj, ds pc, ds ps,
                              bool far, double n1d, double n2d, ds& re, ds& im) {
    const ds   n1  = rd(Ri, RF_NK), n2 = rd(Rj, RF_NK);
    const ds   dp  = ds_add(ds_add(ds_mul(rd(Ri, RF_KX), rd(Rj, RF_KX)), ds_mul(rd(Ri, RF_KY), rd(Rj, RF_KY))),
                            ds_mul(rd(Ri, RF_KZ), rd(Rj, RF_KZ)));
    const ds   np  = ds_mul(n1, n2);
    const int  fi  = Q.square ? RF_INVK_SQUARE : RF_INVK_GAUSS;
    const int  fs  = Q.square ? RF_NKS32_SQUARE : RF_NKS32_GAUSS;
    const ds   ca  = (np.h < 1.0e-13f) ? ds{1.f, 0.f} : ds_mul(dp, ds_mul(rd(Ri, fi), rd(Rj, fi)));
    const ds   lg2 = ds_mulf(ds_sub(ds_mulf(ds_mul(ca, ca), 3.f), ds{1.f, 0.f}), 0.5f);
    const ds   t   = ds_sub(np, Q.kF2);
    const ds   n1s = rd(Ri, fs), n2s = rd(Rj, fs);
    const bool big = n1.h > 1.0e-4f;
    const ds   inv = far ? ds_div(ds{1.f, 0.f}, ds_sub(ds_mul(n1s, n1s), ds_mul(n2s, n2s))) : ds{0.f, 0.f};
    ds         Va  = ds{0.f, 0.f};
    const ds   A0a = ds_add(Q.alpha0a, ds_mul(Q.nl_df_beta0a, t));
    if (Q.has_R0a) Va = ds_mul(A0a, VF_l_ds(0, n1s, far, big, inv, Ri, Rj, RF_J0A, n2s, Q.VR0a2s, Q.VR0a3h, Q.VR0a3t));
    if (Q.has_A2a) {
        if (Q.square)
            Va = ds_add(Va, ds_mul(ds_mul(Q.A2a_5, lg2),
                                   VF_l_ds(2, n1s, far, big, inv, Ri, Rj, RF_J2A, n2s, Q.VR2a2s, Q.VR2a3h, ds{0.f, 0.f})));
        else
            Va = ds_add(Va, ds_mul(ds_mul(Q.gA2a, lg2), ds_mul(i2_gauss(P.R2a, Q.R2a2h, np, n1d, n2d), ds_mul(rd(Ri, RF_GEA), rd(Rj, RF_GEA)))));
    }
    if (Q.same_nl) {
        re = ds_mul(pc, Va);
        im = ds{0.f, 0.f};
        return;
    }
    ds       Vc  = ds{0.f, 0.f};
    const ds A0c = ds_add(Q.alpha0c, ds_mul(Q.beta0c_nl_df, t));
    if (Q.has_R0c) Vc = ds_mul(A0c, VF_l_ds(0, n1s, far, big, inv, Ri, Rj, RF_J0C, n2s, Q.VR0c2s, Q.VR0c3h, Q.VR0c3t));
    if (Q.has_A2c) {
        if (Q.square)
            Vc = ds_add(Vc, ds_mul(ds_mul(Q.A2c_5, lg2),
                                   VF_l_ds(2, n1s, far, big, inv, Ri, Rj, RF_J2C, n2s, Q.VR2c2s, Q.VR2c3h, ds{0.f, 0.f})));
        else
            Vc = ds_add(Vc, ds_mul(ds_mul(Q.gA2c, lg2), ds_mul(i2_gauss(P.R2c, Q.R2c2h, np, n1d, n2d), ds_mul(rd(Ri, RF_GEC), rd(Rj, RF_GEC)))));
    }
    re = ds_mul(pc, ds_mulf(ds_add(Va, Vc), 0.5f));
    im = ds_mul(ps, ds_mulf(ds_sub(Va, Vc), 0.5f));
}

// compute_soc_contribution (SpinOrbitFunctional.cpp:111-138). s[0..3] = s00, s01, s10, s11.
__device__ void soc_element(const DevParams& P, const double* Ri, const double* Rj, double pc, double ps, cx<double>* s) {
    const double l1 = P.mu_soc * Ri[RF_BC] * Rj[RF_BC];
    const double l2 = P.alpha_soc * P.mu_soc * Ri[RF_BA] * Rj[RF_BA];
    const double ls = (l1 + l2) / 2.0;
    const double la = (l1 - l2) / 2.0;
    const double Kx = Ri[RF_KGX], Ky = Ri[RF_KGY], Kz = Ri[RF_KGZ];
    const double Qx = Rj[RF_KGX], Qy = Rj[RF_KGY], Qz = Rj[RF_KGZ];
    const double cz = Kx * Qy - Ky * Qx;
    const double cxv = Ky * Qz - Kz * Qy;
    const double cyv = Kx * Qz - Kz * Qx;
    const double phr = la * ps, phi = -ls * pc;
    // (a + ib)(phr + i phi) with the naive complex product
    s[0] = mk(cz * phr - 0.0 * phi, cz * phi + 0.0 * phr);
    s[1] = mk(cxv * phr - cyv * phi, cxv * phi + cyv * phr);
    s[2] = mk(cxv * phr - (-cyv) * phi, cxv * phi + (-cyv) * phr);
    s[3] = mk((-cz) * phr - 0.0 * phi, (-cz) * phi + 0.0 * phr);
}

__device__ __forceinline__ ds2 split_fp32(double v) {
    const float hi = __double2float_rn(v);
    return ds2{hi, __double2float_rn(v - (double)hi)};
}
__device__ __forceinline__ cx<double> conjd(cx<double> a) { return mk(a.x, -a.y); }

// Element (i, j), i >= j, of the scalar N x N problem: local form factor, kinetic diagonal and the
// nonlocal correction, in the reference's order of operations.
template <bool NL>
__device__ __forceinline__ cx<double> scalar_element(const DevParams& P, const cx<double>* __restrict__ Vloc,
                                                     const double2* __restrict__ phNL, const double* __restrict__ rows,
                                                     int b, int i, int j) {
    const int     N  = P.N;
    const double* Ri = rows + ((size_t)b * N + i) * ROW_STRIDE;
    const double* Rj = rows + ((size_t)b * N + j) * ROW_STRIDE;
    cx<double>    h  = Vloc[(size_t)j * N + i];
    if (i == j) h.x = h.x + Ri[RF_KIN];
    if (NL) {
        const double2    ph = phNL[(size_t)j * N + i];
        const cx<double> v  = nl_element(P, Ri, Rj, ph.x, ph.y);
        h.x                 = h.x + v.x;
        h.y                 = h.y + v.y;
    }
    return h;
}

// The stored form of an element (FP64, or the FP32 pair whose hi part is also the FP32 copy), its
// Hermitian conjugate, and the FP32 copy: each element is converted once and its mirror and copy are
// written from that form (conversions between FP64 and FP32 run at the FP64 rate).
__device__ __forceinline__ double stored(double*, cx<double> h) { return h.x; }
__device__ __forceinline__ cx<double> stored(cx<double>*, cx<double> h) { return h; }
__device__ __forceinline__ ds2 stored(ds2*, cx<double> h) { return split_fp32(h.x); }
__device__ __forceinline__ ds4 stored(ds4*, cx<double> h) {
    const ds2 r = split_fp32(h.x), i = split_fp32(h.y);
    return ds4{r.hi, r.lo, i.hi, i.lo};
}
__device__ __forceinline__ float stored(float*, cx<double> h) { return (float)h.x; }
__device__ __forceinline__ cx<float> stored(cx<float>*, cx<double> h) { return mk((float)h.x, (float)h.y); }
__device__ __forceinline__ float conj_stored(float v) { return v; }
__device__ __forceinline__ cx<float> conj_stored(cx<float> v) { return mk(v.x, -v.y); }
__device__ __forceinline__ float copy32(float v) { return v; }
__device__ __forceinline__ cx<float> copy32(cx<float> v) { return v; }
__device__ __forceinline__ double conj_stored(double v) { return v; }
__device__ __forceinline__ cx<double> conj_stored(cx<double> v) { return conjd(v); }
__device__ __forceinline__ ds2 conj_stored(ds2 v) { return v; }
__device__ __forceinline__ ds4 conj_stored(ds4 v) { return ds4{v.rhi, v.rlo, -v.ihi, -v.ilo}; }
__device__ __forceinline__ float copy32(ds2 v) { return v.hi; }
__device__ __forceinline__ cx<float> copy32(ds4 v) { return mk(v.rhi, v.ihi); }
__device__ __forceinline__ float copy32(double v) { return (float)v; }
__device__ __forceinline__ cx<float> copy32(cx<double> v) { return mk((float)v.x, (float)v.y); }

// Without spin-orbit coupling: one CTA per 32 x 32 tile of the lower triangle, 32 x 8 threads, four
// elements per thread. The tile is written directly (coalesced down its columns) and, through a
// shared-memory transpose, as its Hermitian mirror (coalesced down the mirror's columns), so no
// store is strided and no thread idles on the upper triangle.
template <bool NL, typename SO>
__global__ void __launch_bounds__(256) k_assemble_tiles(const DevParams P, const cx<double>* __restrict__ Vloc,
                                                        const double2* __restrict__ phNL, const double* __restrict__ rows,
                                                        SO* __restrict__ H, int ld, size_t mstride,
                                                        typename Lower<SO>::type* __restrict__ H32, size_t mstride32,
                                                        int batch) {
    using SF = typename Lower<SO>::type;
    __shared__ SO tile[32][33];  // tile[jl][il] = stored form of h(i, j)
    const int b = blockIdx.y;
    if (b >= batch) return;
    // lower tile index -> (ti, tj), ti >= tj, row-major over the lower triangle of tiles
    int t = blockIdx.x, ti = 0;
    while (t > ti) {
        t -= ti + 1;
        ++ti;
    }
    const int tj = t;
    const int N  = P.N;
    const int tx = threadIdx.x, ty = threadIdx.y;
    SO*       Hb = H + (size_t)b * mstride;
    SF*       Fb = H32 ? H32 + (size_t)b * mstride32 : nullptr;
#pragma unroll
    for (int s = 0; s < 4; ++s) {
        const int jl = ty + 8 * s, i = ti * 32 + tx, j = tj * 32 + jl;
        if (i < N && j < N && i >= j) {
            const SO v   = stored(Hb, scalar_element<NL>(P, Vloc, phNL, rows, b, i, j));
            tile[jl][tx] = v;
            Hb[(size_t)j * ld + i] = v;
            if (Fb) Fb[(size_t)j * ld + i] = copy32(v);
        }
    }
    __syncthreads();
#pragma unroll
    for (int s = 0; s < 4; ++s) {
        // mirror (row j, column i) = conj h(i, j) for i > j: threads run down the rows j
        const int il = ty + 8 * s, j = tj * 32 + tx, i = ti * 32 + il;
        if (i < N && j < N && i > j) {
            const SO v = conj_stored(tile[tx][il]);
            Hb[(size_t)i * ld + j] = v;
            if (Fb) Fb[(size_t)i * ld + j] = copy32(v);
        }
    }
}

// Whether the double-single nonlocal element must give way to the FP64 one for the pair of norms
// (n1, n2): where the reference's far branch divides rounding-level differences (|n1 - n2| within
// 1e-5 of the norms), and for gaussian wells where i2's argument x exceeds 80 (e^x beyond FP32's
// range). far returns the reference's branch.
__device__ __forceinline__ bool nl_needs_fp64(const DevParams& P, double n1, double n2, bool& far) {
    const double dn = fabs(n1 - n2);
    far             = F_l_far(n1, n2);
    if (far && dn < 1.0e-5 * fmax(n1, n2)) return true;
    if (!P.square) {
        if (P.has_A2a && 0.5 * (P.R2a * P.R2a) * (n1 * n2) > 80.0) return true;
        if (!P.same_nl && P.has_A2c && 0.5 * (P.R2c * P.R2c) * (n1 * n2) > 80.0) return true;
    }
    return false;
}

// compute_soc_contribution (SpinOrbitFunctional.cpp:111-138) in double-single: sv = (re, im) of
// s00, s01, s10, s11, as soc_element.
__device__ __forceinline__ void soc_element_ds(const DevParamsDS& Q, const float2* Ri, const float2* Rj, ds pc, ds ps,
                                               ds* sv) {
    const ds l1  = ds_mul(ds_mul(Q.mu_soc, rd(Ri, RF_BC)), rd(Rj, RF_BC));
    const ds l2  = ds_mul(ds_mul(Q.alpha_mu_soc, rd(Ri, RF_BA)), rd(Rj, RF_BA));
    const ds ls  = ds_mulf(ds_add(l1, l2), 0.5f);
    const ds la  = ds_mulf(ds_sub(l1, l2), 0.5f);
    const ds Kx = rd(Ri, RF_KGX), Ky = rd(Ri, RF_KGY), Kz = rd(Ri, RF_KGZ);
    const ds Qx = rd(Rj, RF_KGX), Qy = rd(Rj, RF_KGY), Qz = rd(Rj, RF_KGZ);
    const ds cz  = ds_sub(ds_mul(Kx, Qy), ds_mul(Ky, Qx));
    const ds cxv = ds_sub(ds_mul(Ky, Qz), ds_mul(Kz, Qy));
    const ds cyv = ds_sub(ds_mul(Kx, Qz), ds_mul(Kz, Qx));
    const ds phr = ds_mul(la, ps), phi = ds_neg(ds_mul(ls, pc));
    sv[0] = ds_mul(cz, phr);
    sv[1] = ds_mul(cz, phi);
    sv[2] = ds_sub(ds_mul(cxv, phr), ds_mul(cyv, phi));
    sv[3] = ds_add(ds_mul(cxv, phi), ds_mul(cyv, phr));
    sv[4] = ds_add(ds_mul(cxv, phr), ds_mul(cyv, phi));
    sv[5] = ds_sub(ds_mul(cxv, phi), ds_mul(cyv, phr));
    sv[6] = ds_neg(sv[0]);
    sv[7] = ds_neg(sv[1]);
}

template <typename SO>
__device__ __forceinline__ SO make_stored(ds re, ds im);
template <>
__device__ __forceinline__ ds2 make_stored<ds2>(ds re, ds) {
    return ds2{re.h, re.l};
}
template <>
__device__ __forceinline__ ds4 make_stored<ds4>(ds re, ds im) {
    return ds4{re.h, re.l, im.h, im.l};
}

// The mixed path without spin-orbit coupling and with square nonlocal wells: the same tiles, each
// element formed in double-single arithmetic (nl_element_ds) from the k-independent V and structure
// phase in FP32 pairs (Vloc32, phNL32: re hi, re lo, im hi, im lo) and the rows' double-single copy,
// stored directly as its FP32 pair, with the pair's hi part as the FP32 copy. No FP64 instruction.
// An element whose two norms are far apart by the reference's test but within 1e-5 of each other
// (high-symmetry k, where |k + G_i| = |k + G_j| in exact arithmetic and the rounding of the FP64
// norms takes the reference's far branch, dividing one rounding-level difference by another) is
// formed by the FP64 element instead: double-single cannot follow that cancellation.
template <typename SO>
__global__ void __launch_bounds__(256) k_assemble_tiles_ds(const DevParams P, const DevParamsDS Q, const float4* __restrict__ Vloc32,
                                                           const float4* __restrict__ phNL32, const float2* __restrict__ rows32,
                                                           const cx<double>* __restrict__ Vloc, const double2* __restrict__ phNL,
                                                           const double* __restrict__ rows,
                                                           SO* __restrict__ H, int ld, size_t mstride,
                                                           typename Lower<SO>::type* __restrict__ H32, size_t mstride32,
                                                           int batch) {
    using SF = typename Lower<SO>::type;
    __shared__ SO tile[32][33];
    const int b = blockIdx.y;
    if (b >= batch) return;
    int t = blockIdx.x, ti = 0;
    while (t > ti) {
        t -= ti + 1;
        ++ti;
    }
    const int tj = t;
    const int N  = P.N;
    const int tx = threadIdx.x, ty = threadIdx.y;
    SO*       Hb = H + (size_t)b * mstride;
    SF*       Fb = H32 ? H32 + (size_t)b * mstride32 : nullptr;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int jl = ty + 8 * q, i = ti * 32 + tx, j = tj * 32 + jl;
        if (i < N && j < N && i >= j) {
            const double  n1 = rows[((size_t)b * N + i) * ROW_STRIDE + RF_NK];
            const double  n2 = rows[((size_t)b * N + j) * ROW_STRIDE + RF_NK];
            bool          far;
            SO            v;
            if (nl_needs_fp64(P, n1, n2, far)) {
                v = stored(Hb, scalar_element<true>(P, Vloc, phNL, rows, b, i, j));
            } else {
                const float2* Ri = rows32 + ((size_t)b * N + i) * ROW_STRIDE;
                const float2* Rj = rows32 + ((size_t)b * N + j) * ROW_STRIDE;
                const float4  vl = Vloc32[(size_t)j * N + i];
                const float4  ph = phNL32[(size_t)j * N + i];
                ds            vr, vi;
                nl_element_ds(P, Q, Ri, Rj, ds{ph.x, ph.y}, ds{ph.z, ph.w}, far, n1, n2, vr, vi);
                ds hr = ds{vl.x, vl.y}, hi = ds{vl.z, vl.w};
                if (i == j) hr = ds_add(hr, rd(Ri, RF_KIN));
                hr = ds_add(hr, vr);
                hi = ds_add(hi, vi);
                if constexpr (std::is_same<SO, ds2>::value) v = ds2{hr.h, hr.l};
                else v = ds4{hr.h, hr.l, hi.h, hi.l};
            }
            tile[jl][tx]           = v;
            Hb[(size_t)j * ld + i] = v;
            if (Fb) Fb[(size_t)j * ld + i] = copy32(v);
        }
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int il = ty + 8 * q, j = tj * 32 + tx, i = ti * 32 + il;
        if (i < N && j < N && i > j) {
            const SO v             = conj_stored(tile[tx][il]);
            Hb[(size_t)i * ld + j] = v;
            if (Fb) Fb[(size_t)i * ld + j] = copy32(v);
        }
    }
}

template <typename SO>
void launch_assemble_ds(const DevParams& P, const DevParamsDS& Q, const float4* Vloc32, const float4* phNL32,
                        const float2* rows32, const cx<double>* Vloc, const double2* phNL, const double* rows, SO* H,
                        int ld, size_t mstride, typename Lower<SO>::type* H32, size_t mstride32, int batch,
                        cudaStream_t s) {
    const int T = (P.N + 31) / 32;
    dim3      grd(T * (T + 1) / 2, batch), blk(32, 8);
    k_assemble_tiles_ds<SO><<<grd, blk, 0, s>>>(P, Q, Vloc32, phNL32, rows32, Vloc, phNL, rows, H, ld, mstride, H32,
                                                mstride32, batch);
    count_launch();
}
template void launch_assemble_ds<ds2>(const DevParams&, const DevParamsDS&, const float4*, const float4*, const float2*,
                                      const cx<double>*, const double2*, const double*, ds2*, int, size_t, float*, size_t,
                                      int, cudaStream_t);
template void launch_assemble_ds<ds4>(const DevParams&, const DevParamsDS&, const float4*, const float4*, const float2*,
                                      const cx<double>*, const double2*, const double*, ds4*, int, size_t, cx<float>*,
                                      size_t, int, cudaStream_t);

// With spin-orbit coupling: the same tiling over the scalar problem's lower triangle. Each scalar
// element (i, j), i >= j, yields four blocks' elements, UU(i, j) = h + s00, DD(i, j) = h + s11,
// DU(i, j) = s10 and UD(i, j) = s01 (i > j), written directly at (i, j), (i + N, j + N), (i + N, j)
// and (i, j + N), coalesced down their columns; their Hermitian mirrors (j, i), (j + N, i + N),
// (j, i + N) and (j + N, i) go through a shared-memory transpose. On the diagonal (i = j) the
// mirror of DU(i, i) fills (i, i + N), as in the element-per-thread form.
// DSM (the mixed path, SO = ds2 / ds4): the four values in double-single arithmetic on the FP32
// pipe from the FP32-pair tables (Vloc32, phNL32, phSO32) and rows32, the nonlocal part by
// nl_element_ds, and the FP64 element where that one routes an element to FP64.
template <bool NL, bool DSM, typename SO>
__global__ void __launch_bounds__(256) k_assemble_soc_tiles(const DevParams P, const cx<double>* __restrict__ Vloc,
                                                            const double2* __restrict__ phNL,
                                                            const double2* __restrict__ phSO, const double* __restrict__ rows,
                                                            SO* __restrict__ H, int ld, size_t mstride,
                                                            typename Lower<SO>::type* __restrict__ H32,
                                                            size_t mstride32, int batch, const DevParamsDS Q,
                                                            const float4* __restrict__ Vloc32, const float4* __restrict__ phNL32,
                                                            const float4* __restrict__ phSO32, const float2* __restrict__ rows32) {
    using SF = typename Lower<SO>::type;
    extern __shared__ __align__(16) unsigned char smraw[];
    SO(*tile)[32][33] = reinterpret_cast<SO(*)[32][33]>(smraw);  // [4][jl][il]: UU, DD, DU, UD of h(i, j)
    const int b = blockIdx.y;
    if (b >= batch) return;
    int t = blockIdx.x, ti = 0;
    while (t > ti) {
        t -= ti + 1;
        ++ti;
    }
    const int tj = t;
    const int N  = P.N;
    const int tx = threadIdx.x, ty = threadIdx.y;
    SO*       Hb = H + (size_t)b * mstride;
    SF*       Fb = H32 ? H32 + (size_t)b * mstride32 : nullptr;
    auto put = [&](int r, int c, SO v) {
        Hb[(size_t)c * ld + r] = v;
        if (Fb) Fb[(size_t)c * ld + r] = copy32(v);
    };
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int jl = ty + 8 * q, i = ti * 32 + tx, j = tj * 32 + jl;
        if (i < N && j < N && i >= j) {
            SO   uu, dd, du, ud;
            bool fp64 = true;
            if constexpr (DSM) {
                const float2* Ri32 = rows32 + ((size_t)b * N + i) * ROW_STRIDE;
                const float2* Rj32 = rows32 + ((size_t)b * N + j) * ROW_STRIDE;
                const float4  vl   = Vloc32[(size_t)j * N + i];
                ds            hr = ds{vl.x, vl.y}, hm = ds{vl.z, vl.w};
                if (i == j) hr = ds_add(hr, rd(Ri32, RF_KIN));
                fp64 = false;
                if (NL) {
                    const double n1 = rows[((size_t)b * N + i) * ROW_STRIDE + RF_NK];
                    const double n2 = rows[((size_t)b * N + j) * ROW_STRIDE + RF_NK];
                    bool         far;
                    fp64 = nl_needs_fp64(P, n1, n2, far);
                    if (!fp64) {
                        const float4 pn = phNL32[(size_t)j * N + i];
                        ds           vr, vi;
                        nl_element_ds(P, Q, Ri32, Rj32, ds{pn.x, pn.y}, ds{pn.z, pn.w}, far, n1, n2, vr, vi);
                        hr = ds_add(hr, vr);
                        hm = ds_add(hm, vi);
                    }
                }
                if (!fp64) {
                    const float4 ps = phSO32[(size_t)j * N + i];
                    ds           sv[8];
                    soc_element_ds(Q, Ri32, Rj32, ds{ps.x, ps.y}, ds{ps.z, ps.w}, sv);
                    uu = make_stored<SO>(ds_add(hr, sv[0]), ds_add(hm, sv[1]));
                    dd = make_stored<SO>(ds_add(hr, sv[6]), ds_add(hm, sv[7]));
                    du = make_stored<SO>(sv[4], sv[5]);
                    ud = make_stored<SO>(sv[2], sv[3]);
                }
            }
            if (fp64) {
                const cx<double> h  = scalar_element<NL>(P, Vloc, phNL, rows, b, i, j);
                const double*    Ri = rows + ((size_t)b * N + i) * ROW_STRIDE;
                const double*    Rj = rows + ((size_t)b * N + j) * ROW_STRIDE;
                const double2    ph = phSO[(size_t)j * N + i];
                cx<double>       sv[4];
                soc_element(P, Ri, Rj, ph.x, ph.y, sv);
                uu = stored(Hb, mk(h.x + sv[0].x, h.y + sv[0].y));
                dd = stored(Hb, mk(h.x + sv[3].x, h.y + sv[3].y));
                du = stored(Hb, sv[2]);
                ud = stored(Hb, sv[1]);
            }
            put(i, j, uu);
            put(i + N, j + N, dd);
            put(i + N, j, du);
            tile[0][jl][tx] = uu;
            tile[1][jl][tx] = dd;
            tile[2][jl][tx] = du;
            if (i > j) {
                put(i, j + N, ud);
                tile[3][jl][tx] = ud;
            }
        }
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        // mirrors: threads run down the rows j (coalesced down column i, i + N)
        const int il = ty + 8 * q, j = tj * 32 + tx, i = ti * 32 + il;
        if (i < N && j < N && i >= j) {
            put(j, i + N, conj_stored(tile[2][tx][il]));  // UD(j, i) = conj DU(i, j)
            if (i > j) {
                put(j, i, conj_stored(tile[0][tx][il]));          // UU(j, i)
                put(j + N, i + N, conj_stored(tile[1][tx][il]));  // DD(j, i)
                put(j + N, i, conj_stored(tile[3][tx][il]));      // DU(j, i) = conj UD(i, j)
            }
        }
    }
}

// ------------------------------------------------------------------------------------------------
void launch_rows(const DevParams& P, const double* d_k, const int* d_G, double* d_rows, int batch, cudaStream_t s,
                 float2* d_rows32) {
    const int total = batch * P.N;
    k_rows<<<(total + 127) / 128, 128, 0, s>>>(P, d_k, d_G, d_rows, batch, d_rows32);
    count_launch();
}

template <typename SO>
void launch_assemble(const DevParams& P, const cx<double>* Vloc, const double2* phNL, const double2* phSO, const double* rows,
                     SO* H, int ld, size_t mstride, typename Lower<SO>::type* H32, size_t mstride32, int batch,
                     cudaStream_t s) {
    dim3 blk(32, 8);
    if (!P.soc) {
        const int T = (P.N + 31) / 32;
        dim3      grd(T * (T + 1) / 2, batch);
        if (P.nl) k_assemble_tiles<true, SO><<<grd, blk, 0, s>>>(P, Vloc, phNL, rows, H, ld, mstride, H32, mstride32, batch);
        else k_assemble_tiles<false, SO><<<grd, blk, 0, s>>>(P, Vloc, phNL, rows, H, ld, mstride, H32, mstride32, batch);
        count_launch();
        return;
    }
    const int    T    = (P.N + 31) / 32;
    dim3         grd(T * (T + 1) / 2, batch);
    const size_t smem = sizeof(SO) * 4 * 32 * 33;
    auto         kern = P.nl ? k_assemble_soc_tiles<true, false, SO> : k_assemble_soc_tiles<false, false, SO>;
    if (smem > 48 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    kern<<<grd, blk, smem, s>>>(P, Vloc, phNL, phSO, rows, H, ld, mstride, H32, mstride32, batch, DevParamsDS{}, nullptr,
                                nullptr, nullptr, nullptr);
    count_launch();
}

template void launch_assemble<double>(const DevParams&, const cx<double>*, const double2*, const double2*, const double*,
                                      double*, int, size_t, float*, size_t, int, cudaStream_t);
template void launch_assemble<cx<double>>(const DevParams&, const cx<double>*, const double2*, const double2*, const double*,
                                          cx<double>*, int, size_t, cx<float>*, size_t, int, cudaStream_t);
template void launch_assemble<float>(const DevParams&, const cx<double>*, const double2*, const double2*, const double*,
                                     float*, int, size_t, float*, size_t, int, cudaStream_t);
template void launch_assemble<cx<float>>(const DevParams&, const cx<double>*, const double2*, const double2*, const double*,
                                         cx<float>*, int, size_t, cx<float>*, size_t, int, cudaStream_t);
template void launch_assemble<ds2>(const DevParams&, const cx<double>*, const double2*, const double2*, const double*, ds2*,
                                   int, size_t, float*, size_t, int, cudaStream_t);
template void launch_assemble<ds4>(const DevParams&, const cx<double>*, const double2*, const double2*, const double*, ds4*,
                                   int, size_t, cx<float>*, size_t, int, cudaStream_t);

template <typename SO>
void launch_assemble_soc_ds(const DevParams& P, const DevParamsDS& Q, const float4* Vloc32, const float4* phNL32,
                            const float4* phSO32, const float2* rows32, const cx<double>* Vloc, const double2* phNL,
                            const double2* phSO, const double* rows, SO* H, int ld, size_t mstride,
                            typename Lower<SO>::type* H32, size_t mstride32, int batch, cudaStream_t s) {
    const int    T    = (P.N + 31) / 32;
    dim3         grd(T * (T + 1) / 2, batch), blk(32, 8);
    const size_t smem = sizeof(SO) * 4 * 32 * 33;
    auto         kern = P.nl ? k_assemble_soc_tiles<true, true, SO> : k_assemble_soc_tiles<false, true, SO>;
    if (smem > 48 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    kern<<<grd, blk, smem, s>>>(P, Vloc, phNL, phSO, rows, H, ld, mstride, H32, mstride32, batch, Q, Vloc32, phNL32, phSO32,
                                rows32);
    count_launch();
}
template void launch_assemble_soc_ds<ds4>(const DevParams&, const DevParamsDS&, const float4*, const float4*, const float4*,
                                          const float2*, const cx<double>*, const double2*, const double2*, const double*,
                                          ds4*, int, size_t, cx<float>*, size_t, int, cudaStream_t);

// ---- diagnostics: the mixed path's double-single special functions on device values -----------
__global__ void k_ds_special(int fn, const double* __restrict__ x, size_t n, double* __restrict__ y) {
    const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const ds v = ds_of_double(x[t]);
    const ds r = fn == 0 ? ds_exp_pos(v) : i2_ds(v);  // both for 2 < x <= 80
    y[t]       = (double)r.h + (double)r.l;
}

}  // namespace uepm

extern "C" int uepm_ds_special_device(int fn, const double* d_x, size_t n, double* d_y, void* stream) {
    if ((fn != 0 && fn != 1) || (n && (!d_x || !d_y))) {
        uepm::set_error("uepm_ds_special_device: fn must be 0 (e^x) or 1 (i2), and the buffers non-null");
        return UEPM_ERR_INVALID;
    }
    if (n == 0) return UEPM_OK;
    const unsigned blocks = (unsigned)((n + 255) / 256);
    uepm::k_ds_special<<<blocks, 256, 0, (cudaStream_t)stream>>>(fn, d_x, n, d_y);
    uepm::count_launch();
    return cudaGetLastError() == cudaSuccess ? UEPM_OK : UEPM_ERR_CUDA;
}

