// uepm_common.cuh -- shared device types and helpers for the sm_103a band-structure kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cfloat>

namespace uepm {

// ------------------------------------------------------------------------------------------------
// Complex arithmetic on (re, im) pairs, written with explicit fused multiply-adds: on GB300 every
// FP64 instruction (add, mul or fma) costs one slot of the narrow FP64 pipe, so a complex
// multiply-accumulate is exactly 4 FMAs and nothing else.
template <typename T>
struct cx {
    T x, y;
};

template <typename T>
__host__ __device__ __forceinline__ cx<T> mk(T x, T y) {
    cx<T> r;
    r.x = x;
    r.y = y;
    return r;
}
template <typename T>
__device__ __forceinline__ cx<T> cadd(cx<T> a, cx<T> b) {
    return mk(a.x + b.x, a.y + b.y);
}
template <typename T>
__device__ __forceinline__ cx<T> csub(cx<T> a, cx<T> b) {
    return mk(a.x - b.x, a.y - b.y);
}
template <typename T>
__device__ __forceinline__ cx<T> cmul(cx<T> a, cx<T> b) {
    return mk(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}
// c + a * b
template <typename T>
__device__ __forceinline__ cx<T> cfma(cx<T> a, cx<T> b, cx<T> c) {
    return mk(fma(a.x, b.x, fma(-a.y, b.y, c.x)), fma(a.x, b.y, fma(a.y, b.x, c.y)));
}
// c + conj(a) * b
template <typename T>
__device__ __forceinline__ cx<T> cfmac(cx<T> a, cx<T> b, cx<T> c) {
    return mk(fma(a.x, b.x, fma(a.y, b.y, c.x)), fma(a.x, b.y, fma(-a.y, b.x, c.y)));
}
// c - a * conj(b)
template <typename T>
__device__ __forceinline__ cx<T> cfms_conjb(cx<T> a, cx<T> b, cx<T> c) {
    return mk(fma(-a.x, b.x, fma(-a.y, b.y, c.x)), fma(-a.y, b.x, fma(a.x, b.y, c.y)));
}
template <typename T>
__device__ __forceinline__ cx<T> cscale(cx<T> a, T s) {
    return mk(a.x * s, a.y * s);
}

// 16-byte (double) / 8-byte (float) vector loads and stores of one complex element.
__device__ __forceinline__ cx<double> ldc(const cx<double>* p) {
    double2 v = *reinterpret_cast<const double2*>(p);
    return mk(v.x, v.y);
}
__device__ __forceinline__ cx<float> ldc(const cx<float>* p) {
    float2 v = *reinterpret_cast<const float2*>(p);
    return mk(v.x, v.y);
}
__device__ __forceinline__ void stc(cx<double>* p, cx<double> a) { *reinterpret_cast<double2*>(p) = make_double2(a.x, a.y); }
__device__ __forceinline__ void stc(cx<float>* p, cx<float> a) { *reinterpret_cast<float2*>(p) = make_float2(a.x, a.y); }

// Real-scalar counterparts of the complex helpers: the same kernel templates serve real symmetric
// matrices (H(k) is exactly real for diamond-structure local / symmetric-nonlocal EPM without SOC).
__device__ __forceinline__ double cadd(double a, double b) { return a + b; }
__device__ __forceinline__ float cadd(float a, float b) { return a + b; }
__device__ __forceinline__ double csub(double a, double b) { return a - b; }
__device__ __forceinline__ float csub(float a, float b) { return a - b; }
__device__ __forceinline__ double cmul(double a, double b) { return a * b; }
__device__ __forceinline__ float cmul(float a, float b) { return a * b; }
__device__ __forceinline__ double cfma(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float cfma(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double cfmac(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float cfmac(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double cfms_conjb(double a, double b, double c) { return fma(-a, b, c); }
__device__ __forceinline__ float cfms_conjb(float a, float b, float c) { return fmaf(-a, b, c); }
__device__ __forceinline__ double cscale(double a, double s) { return a * s; }
__device__ __forceinline__ float cscale(float a, float s) { return a * s; }
__device__ __forceinline__ double ldc(const double* p) { return *p; }
__device__ __forceinline__ float ldc(const float* p) { return *p; }
__device__ __forceinline__ void stc(double* p, double a) { *p = a; }
__device__ __forceinline__ void stc(float* p, float a) { *p = a; }

// Scalar traits: R = the real type, and the few operations that differ between real and complex.
template <typename S>
struct ST;
template <>
struct ST<double> {
    using R = double;
    static constexpr bool cplx = false;
    static __device__ __forceinline__ double zero() { return 0.0; }
    static __device__ __forceinline__ double one() { return 1.0; }
    static __device__ __forceinline__ double re(double a) { return a; }
    static __device__ __forceinline__ double im(double) { return 0.0; }
    static __device__ __forceinline__ double make(double r, double) { return r; }
    static __device__ __forceinline__ double conj(double a) { return a; }
    static __device__ __forceinline__ double norm(double a) { return a * a; }
    static __device__ __forceinline__ double neg(double a) { return -a; }
};
template <>
struct ST<float> {
    using R = float;
    static constexpr bool cplx = false;
    static __device__ __forceinline__ float zero() { return 0.f; }
    static __device__ __forceinline__ float one() { return 1.f; }
    static __device__ __forceinline__ float re(float a) { return a; }
    static __device__ __forceinline__ float im(float) { return 0.f; }
    static __device__ __forceinline__ float make(float r, float) { return r; }
    static __device__ __forceinline__ float conj(float a) { return a; }
    static __device__ __forceinline__ float norm(float a) { return a * a; }
    static __device__ __forceinline__ float neg(float a) { return -a; }
};
template <typename T>
struct ST<cx<T>> {
    using R = T;
    static constexpr bool cplx = true;
    static __device__ __forceinline__ cx<T> zero() { return mk<T>(0, 0); }
    static __device__ __forceinline__ cx<T> one() { return mk<T>(1, 0); }
    static __device__ __forceinline__ T re(cx<T> a) { return a.x; }
    static __device__ __forceinline__ T im(cx<T> a) { return a.y; }
    static __device__ __forceinline__ cx<T> make(T r, T i) { return mk<T>(r, i); }
    static __device__ __forceinline__ cx<T> conj(cx<T> a) { return mk<T>(a.x, -a.y); }
    static __device__ __forceinline__ T norm(cx<T> a) { return fma(a.x, a.x, a.y * a.y); }
    static __device__ __forceinline__ cx<T> neg(cx<T> a) { return mk<T>(-a.x, -a.y); }
};

// Lower-precision counterpart of a scalar type (FP64 -> FP32), for the mixed path.
template <typename S>
struct Lower;
template <>
struct Lower<double> {
    using type = float;
};
template <>
struct Lower<cx<double>> {
    using type = cx<float>;
};

// An FP64 matrix element carried as the unevaluated sum of two FP32 values, hi = fl32(v) and
// lo = fl32(v - hi) (about 48 significant bits, same size as the FP64 element): the mixed path's copy
// of H for the Rayleigh-Ritz products, which then run on the FP32 pipe.
struct __align__(8) ds2 {
    float hi, lo;
};
struct __align__(16) ds4 {
    float rhi, rlo, ihi, ilo;
};
template <typename S>
struct Split;
template <>
struct Split<double> {
    using type = ds2;
};
template <>
struct Split<cx<double>> {
    using type = ds4;
};
template <>
struct Lower<float> {
    using type = float;
};
template <>
struct Lower<cx<float>> {
    using type = cx<float>;
};
template <>
struct Lower<ds2> {
    using type = float;
};
template <>
struct Lower<ds4> {
    using type = cx<float>;
};

// Double-single accumulation (Dekker's exact product, Knuth's two-sum) with operations the compiler
// does not contract: acc += (xh + xl) * y with xh * y exact, carried as acc.h + acc.l.
struct dsacc {
    float h, l;
};
__device__ __forceinline__ void ds_add_prod(dsacc& a, float xh, float xl, float y) {
    const float p  = __fmul_rn(xh, y);
    const float pe = fmaf(xh, y, -p);
    const float s  = __fadd_rn(a.h, p);
    const float z  = __fsub_rn(s, a.h);
    const float er = __fadd_rn(__fsub_rn(a.h, __fsub_rn(s, z)), __fsub_rn(p, z));
    a.h            = s;
    a.l            = fmaf(xl, y, __fadd_rn(a.l, __fadd_rn(er, pe)));
}
// acc += x * y for FP32 x, y (the product exactly)
__device__ __forceinline__ void ds_add_prod(dsacc& a, float x, float y) {
    const float p  = __fmul_rn(x, y);
    const float pe = fmaf(x, y, -p);
    const float s  = __fadd_rn(a.h, p);
    const float z  = __fsub_rn(s, a.h);
    const float er = __fadd_rn(__fsub_rn(a.h, __fsub_rn(s, z)), __fsub_rn(p, z));
    a.h            = s;
    a.l            = __fadd_rn(a.l, __fadd_rn(er, pe));
}
__device__ __forceinline__ double ds_value(dsacc a) { return (double)a.h + (double)a.l; }

// Double-single numbers (an FP32 pair h + l, |l| <= ulp(h) / 2, about 48 significant bits) with the
// classical error-free transformations (Dekker, Knuth) on non-contracted FP32 operations: the mixed
// path evaluates the nonlocal matrix elements on the FP32 pipe with them instead of the FP64 pipe.
struct ds {
    float h, l;
};
__host__ __device__ inline ds ds_of_double(double v) {
    const float h = (float)v;
    return ds{h, (float)(v - (double)h)};
}
__device__ __forceinline__ ds ds_quick(float s, float e) {  // |s| >= |e|
    const float t = __fadd_rn(s, e);
    return ds{t, __fsub_rn(e, __fsub_rn(t, s))};
}
__device__ __forceinline__ ds ds_add(ds a, ds b) {
    const float s  = __fadd_rn(a.h, b.h);
    const float bb = __fsub_rn(s, a.h);
    const float e  = __fadd_rn(__fsub_rn(a.h, __fsub_rn(s, bb)), __fsub_rn(b.h, bb));
    return ds_quick(s, __fadd_rn(e, __fadd_rn(a.l, b.l)));
}
__device__ __forceinline__ ds ds_neg(ds a) { return ds{-a.h, -a.l}; }
__device__ __forceinline__ ds ds_sub(ds a, ds b) { return ds_add(a, ds_neg(b)); }
__device__ __forceinline__ ds ds_mul(ds a, ds b) {
    const float p = __fmul_rn(a.h, b.h);
    const float e = fmaf(a.h, b.h, -p);
    return ds_quick(p, fmaf(a.h, b.l, fmaf(a.l, b.h, e)));
}
__device__ __forceinline__ ds ds_mulf(ds a, float b) {  // times an exact FP32 value
    const float p = __fmul_rn(a.h, b);
    const float e = fmaf(a.h, b, -p);
    return ds_quick(p, fmaf(a.l, b, e));
}
__device__ __forceinline__ ds ds_div(ds a, ds b) {  // long division, two quotient digits
    const float q1 = __fdiv_rn(a.h, b.h);
    const ds    r  = ds_sub(a, ds_mulf(b, q1));
    const float q2 = __fdiv_rn(r.h, b.h);
    return ds_quick(q1, q2);
}
__device__ __forceinline__ float ds_abs_hi(ds a) { return fabsf(a.h); }

// cp.async of one naturally aligned element of B = 4 or 8 bytes, global -> shared
template <int B>
__device__ __forceinline__ void cp_async_elem(void* dst, const void* src) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2;\n" ::"r"(sa), "l"(src), "n"(B) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
template <typename T>
__device__ __forceinline__ cx<T> warp_sum(cx<T> v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
        v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
    }
    return v;
}
template <typename T>
__device__ __forceinline__ T warp_max(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
template <typename T>
__device__ __forceinline__ T warp_min(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

template <typename T>
struct num;
template <>
struct num<double> {
    static __host__ __device__ constexpr double eps() { return DBL_EPSILON; }
    static __host__ __device__ constexpr double tiny() { return DBL_MIN; }
};
template <>
struct num<float> {
    static __host__ __device__ constexpr float eps() { return FLT_EPSILON; }
    static __host__ __device__ constexpr float tiny() { return FLT_MIN; }
};

// ------------------------------------------------------------------------------------------------
// Device-side material constants. Every derived constant is computed on the host in double with the
// reference's own expression (Material.h / Material.cpp / Hamiltonian.cpp / SpinOrbitFunctional.cpp),
// so the kernels start from bit-identical constants.
struct DevParams {
    int N;        // scalar basis size
    int n;        // matrix order (N or 2N)
    int nl;       // nonlocal correction on
    int soc;      // spin-orbit blocks on
    int square;   // nonlocal well: 1 square, 0 gaussian
    int has_R0a, has_R0c, has_A2a, has_A2c;
    int same_nl;  // anion and cation carry the same nonlocal parameters (their terms are equal)
    double kin_pref;      // two_pi_over_a * two_pi_over_a * diag_factor      (Hamiltonian.cpp:68-72)
    double grad_pref;     // 2 * diag_factor * (2pi/a)^2                      (Hamiltonian.cpp:167)
    double frac_to_phys;  // 1 / (2pi/a)                                      (Hamiltonian.cpp:190)
    // nonlocal (Material.cpp:139-208)
    double ff;            // fourier factor 2pi/a (1/m)
    double nl_df;         // pow(h_bar,2)/(2 m_e q_e)
    double Vpre;          // 4 pi / atomic volume
    double kF2;           // pow(fermi momentum, 2)
    double alpha0a, beta0a, A2a, alpha0c, beta0c, A2c;
    double R0a, R0c, R2a, R2c;
    double R0a2, R0c2, R2a2, R2c2;         // pow(R, 2.0)
    double R0a3h, R0c3h, R2a3h, R2c3h;     // pow(R, 3.0) / 2
    double R0a3t, R0c3t;                   // pow(R, 3.0) / 3
    double gpre_a, gpre_c;                 // 5 pi^1.5 (R2^3 / volume)
    // spin-orbit (SpinOrbitFunctional.cpp:20-138)
    unsigned pa, pc;
    double ra, rc, alpha_soc, mu_soc, kfac, bohr;
};

// The nonlocal constants of DevParams as double-single numbers, for the mixed path's square-well
// element on the FP32 pipe; products the FP64 element forms first are formed on the host in FP64
// (the same order of operations) and then split.
struct DevParamsDS {
    int  has_R0a, has_R0c, has_A2a, has_A2c, same_nl;
    ds   kF2;
    ds   alpha0a, nl_df_beta0a, alpha0c, beta0c_nl_df;  // A0 = alpha0 + (nl_df beta0) t
    ds   A2a_5, A2c_5;                                  // A2 5 (eV)
    // The F_l terms times Vpre = 4 pi / volume, so that every intermediate stays well inside FP32's
    // exponent range (R^2 / (n1^2 - n2^2) ~ 1e-41 in SI units is not): VR2s = Vpre R^2 / (2 pi / a)
    // for the far branch, whose norms are taken in units of 2 pi / a, VR3h = Vpre R^3 / 2 and
    // VR3t = Vpre R^3 / 3 for the near branch and its K = 0 limit.
    ds   VR0a2s, VR0c2s, VR2a2s, VR2c2s;
    ds   VR0a3h, VR0c3h, VR2a3h, VR2c3h, VR0a3t, VR0c3t;
    // gaussian d-wells: V2 = (gpre A2) P2 i2(x) e_i e_j with x = (R2^2 / 2) n1 n2
    int  square;
    ds   gA2a, gA2c, R2a2h, R2c2h;  // gpre A2, R2^2 / 2
    // spin-orbit: lambda_1 = mu B_c B_c', lambda_2 = (alpha mu) B_a B_a'
    ds   mu_soc, alpha_mu_soc;
};

// Per-(k, basis vector) quantities computed once per k in the row kernel and read by the
// element kernel. Layout: rows[(b * N + i) * ROW_STRIDE + field].
enum RowField {
    RF_KGX = 0, RF_KGY, RF_KGZ,   // k + G_i, reduced
    RF_KX, RF_KY, RF_KZ,          // (k + G_i) * 2pi/a, 1/m
    RF_NK,                        // |K_i|
    RF_KIN,                       // kinetic diagonal C |k+G_i|^2
    RF_J0A,                       // j_{-1}, j_0, j_1 at |K| R0_anion
    RF_J0C = RF_J0A + 3,          // j_{-1}, j_0, j_1 at |K| R0_cation
    RF_J2A = RF_J0C + 3,          // j_1, j_2, j_3 at |K| R2_anion (square well)
    RF_J2C = RF_J2A + 3,          // j_1, j_2, j_3 at |K| R2_cation (square well)
    RF_GEA = RF_J2C + 3,          // exp(-0.25 |K|^2 R2a^2) (gaussian well)
    RF_GEC,                       // exp(-0.25 |K|^2 R2c^2)
    RF_BC,                        // SOC radial factor B_period(|K|), cation
    RF_BA,                        // anion
    ROW_STRIDE = 24,
    // 1 / |K_i| (0 where K = 0), in a slot the well type leaves free: the gaussian exponentials'
    // slot for square wells, the l = 2 Bessel slot for gaussian wells
    RF_INVK_SQUARE = RF_GEA,
    RF_INVK_GAUSS  = RF_J2A,
    // in the mixed path's double-single copy of the rows only: |K_i| in units of 2 pi / a, in the
    // slot the well type leaves free
    RF_NKS32_SQUARE = RF_GEC,
    RF_NKS32_GAUSS  = RF_J2C
};

}  // namespace uepm
