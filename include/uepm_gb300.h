/*
 * uepm_gb300.h -- C ABI of the GB300 (sm_103a) band-structure engine.
 *
 * This is the drop-in boundary for UltimateEPM's per-k-point hot path: H(k) assembly plus the
 * Hermitian eigensolve, batched over k-points on one GPU. Every entry point takes plain pointers and
 * sizes and returns an int status; the C++ adapter (include/uepm/*.h) rethrows the same exception
 * types the reference throws. Energies are in eV, k in reduced units of 2*pi/a, gradients in eV*m,
 * exactly as in the reference's src/EPP.
 *
 * Reference interfaces replaced (paths relative to the reference project root):
 *   uepm_generate_basis        BandStructure::GenerateBasisVectors     src/EPP/BandStructure.cpp:26-57
 *   uepm_generate_path         SymmetryPoints::GeneratePoints          src/EPP/SymmetryPoints.cpp:47-147
 *   uepm_materials_load        Materials::load_material_parameters     src/EPP/Material.cpp:33-71
 *   uepm_ctx_create            Hamiltonian::Hamiltonian + SetConstantNonDiagonalMatrix
 *                                                                       src/EPP/Hamiltonian.cpp:18-48
 *   uepm_solve / _device       BandStructure::Compute_parallel, i.e. per k: Hamiltonian::SetMatrix
 *                              + Diagonalize + compute_gradient_at_level
 *                                                                       src/EPP/BandStructure.cpp:151-201,
 *                                                                       src/EPP/Hamiltonian.cpp:50-194
 *   uepm_assemble_device       Hamiltonian::SetMatrix + the hermitisation in Diagonalize
 *                                                                       src/EPP/Hamiltonian.cpp:50-127
 *   uepm_adjust_values         BandStructure::AdjustValues / FindBandGap
 *                                                                       src/EPP/BandStructure.cpp:203-262
 */
#ifndef UEPM_GB300_H
#define UEPM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Return codes. The C++ adapter maps them onto the reference's exception types. */
#define UEPM_OK 0
#define UEPM_ERR_INVALID (-1)      /* std::invalid_argument (bad path label, x < 0, ...)       */
#define UEPM_ERR_RUNTIME (-2)      /* std::runtime_error (bad basis, unsupported SOC period)  */
#define UEPM_ERR_OUT_OF_RANGE (-3) /* std::out_of_range (band index)                          */
#define UEPM_ERR_CUDA (-4)         /* a CUDA call failed; uepm_last_error() has the text      */
#define UEPM_ERR_NOMEM (-5)        /* device allocation failed                               */
#define UEPM_ERR_NOT_CONVERGED (-6)/* at least one k-point reported a non-zero status        */

/* Per-k-point status values written by the solve. */
#define UEPM_K_OK 0
#define UEPM_K_NOCONVERGE 1 /* an iteration cap was reached                                   */
#define UEPM_K_NONFINITE 2  /* NaN/Inf appeared in H(k) or in the reduction                  */

/* Context flags (Hamiltonian::SetMatrix's add_non_local_correction / enable_soc). */
#define UEPM_NONLOCAL 1u
#define UEPM_SOC 2u

/* What a solve computes. Values are always produced. */
#define UEPM_WANT_VALUES 1u
#define UEPM_WANT_VECTORS 2u  /* X: the nb lowest eigenvectors                              */
#define UEPM_WANT_GRADIENT 4u /* Hellmann-Feynman kinetic gradient, as compute_gradient_at_level */

/* Arithmetic of the solve. */
#define UEPM_PREC_FP64 0  /* plain FP64 path: the drop-in                                   */
#define UEPM_PREC_MIXED 1 /* FP32 reduction + FP64 residual and Rayleigh-Ritz refinement    */

/*
 * Material parameters in the units the reference holds after loading a YAML file
 * (src/EPP/Material.cpp:33-71, NonLocalParameters.hpp:91-116, SpinOrbitParameters.hpp:74-81):
 * lattice constant in Angstrom; V* in eV; alpha_0 and A2 in eV; beta_0 raw; radii in metres;
 * spin-orbit periods, radial extents (bohr units), alpha and mu raw. nl_well: 0 unknown,
 * 1 square, 2 gaussian.
 */
typedef struct uepm_material {
    double lattice_constant;
    double V3S, V4S, V8S, V11S, V3A, V4A, V8A, V11A;
    int32_t nl_well;
    int32_t has_nonlocal;
    double alpha0_cation, beta0_cation, A2_cation, alpha0_anion, beta0_anion, A2_anion;
    double R0_cation, R2_cation, R0_anion, R2_anion;
    uint32_t period_anion, period_cation;
    int32_t has_soc;
    int32_t _pad;
    double radial_extent_anion, radial_extent_cation, alpha_soc, mu_soc;
} uepm_material;

typedef struct uepm_ctx uepm_ctx;

/* Library identity and the last error message of the calling thread. */
int uepm_version(void);
const char* uepm_last_error(void);
int uepm_material_size(void);

/* BandStructure::GenerateBasisVectors: writes up to `capacity` int32 triples (x,y,z) in the
 * reference's i->j->k loop order and returns the basis size N, or UEPM_ERR_RUNTIME when `shells`
 * is outside [2, table size]. Pass capacity 0 to query N. Host-only. */
int uepm_generate_basis(unsigned shells, int32_t* G, int capacity);

/* SymmetryPoints::GeneratePoints for single-letter labels from {L,G,X,W,K,U} (e.g. "LGXWKULWXKG"):
 * writes up to `capacity` k triples and strlen(labels) node positions, returns the point count or
 * UEPM_ERR_INVALID where the reference throws std::invalid_argument. Host-only. */
int uepm_generate_path(const char* labels, unsigned n_points, double* k, int capacity, uint32_t* sym_pos);

/* Materials::load_material_parameters: parses the reference's YAML layout. Writes up to
 * `capacity` materials and their symbols (each `symbol_stride` bytes, NUL-terminated) in file
 * order; returns the number of materials in the file or a negative code. Host-only. */
int uepm_materials_load(const char* path, uepm_material* out, char* symbols, int symbol_stride, int capacity);

/* Hamiltonian ctor: uploads the material and the basis G (N int32 triples) to the current CUDA
 * device and precomputes the k-independent local form-factor matrix. flags: UEPM_NONLOCAL,
 * UEPM_SOC. Fails with UEPM_ERR_RUNTIME for SOC on a material whose atomic periods are not 2-4
 * (the reference throws from SpinOrbitCorrection::compute_lambda_1/2). */
int uepm_ctx_create(const uepm_material* mat, const int32_t* G, int N, uint32_t flags, uepm_ctx** out);
int uepm_ctx_destroy(uepm_ctx* ctx);
int uepm_ctx_set_precision(uepm_ctx* ctx, int precision);
/* Matrix order n: N, or 2N with SOC. */
int uepm_ctx_order(const uepm_ctx* ctx);
/* Upper bound, in bytes, of device workspace a solve may hold (default 8 GiB). */
int uepm_ctx_set_workspace_limit(uepm_ctx* ctx, size_t bytes);
/* When H(k) is exactly real for the context's material and flags (no SOC, all antisymmetric form
 * factors zero, identical anion/cation nonlocal parameters: elemental diamond-structure crystals),
 * the solve runs real-symmetric kernels, a quarter of the complex arithmetic, with the same results.
 * on != 0 forces the complex kernels (for cross-checks). Returns 1 if the real kernels will run,
 * 0 otherwise. */
int uepm_ctx_force_complex(uepm_ctx* ctx, int on);

/*
 * Batched solve over nk k-points (reduced units, nk x 3 row-major), keeping the nb lowest bands:
 *   E      nk x nb, ascending per k                                   (required)
 *   X      nk x nb x n complex128 (re, im interleaved), eigenvector b of k in X[k][b][:]
 *                                                       (UEPM_WANT_VECTORS, else may be NULL)
 *   grad   nk x nb x 3, eV*m                             (UEPM_WANT_GRADIENT, else may be NULL)
 *   status nk int32 per-k status                         (may be NULL)
 * nb must be in [1, n]. uepm_solve takes HOST buffers and copies in and out; uepm_solve_device
 * takes DEVICE buffers and enqueues on `stream` (a cudaStream_t, NULL = legacy default stream)
 * without synchronising. A mixed-precision solve of 1024 or more k-points that fits one pipeline
 * pass splits the batch between `stream` and a second stream of the context, forked from and joined
 * back to `stream` (work enqueued on `stream` afterwards waits for both; the results are the same;
 * uepm_tuning.streams). With profiling on, the two halves of a kernel count as one launch, timed
 * from the first start to the last end.
 */
int uepm_solve(uepm_ctx* ctx, const double* k, size_t nk, int nb, uint32_t want, double* E, double* X, double* grad,
               int32_t* status);
int uepm_solve_device(uepm_ctx* ctx, const double* d_k, size_t nk, int nb, uint32_t want, double* d_E, double* d_X,
                      double* d_grad, int32_t* d_status, void* stream);

/* H(k) after SetMatrix and Diagonalize's hermitisation, for nk k-points: d_H is nk x n x n
 * complex128, column-major per k, both triangles filled. Device buffers, enqueued on `stream`. */
int uepm_assemble_device(uepm_ctx* ctx, const double* d_k, size_t nk, double* d_H, void* stream);

/* H(k) assembly that allocates nothing (no counterpart in the reference). Same inputs, output and
 * results as uepm_assemble_device, for callers that must not allocate device memory when they call
 * (a serving loop with memory reserved at start-up, a host program whose device memory belongs to its
 * own allocator): the per-plane-wave row table lives in a fixed 16 MiB device array of the library,
 * present on every GPU that loads it until exit, instead of a workspace grown on demand. Limit:
 * nk * N * 24 * 8 bytes <= UEPM_NOALLOC_SCRATCH_BYTES (e.g. 637 k-points per call for basis 137)
 * and nk <= 32768; larger requests fail with UEPM_ERR_INVALID. The first call on a device looks up
 * the array's device address (with that device current) and should come before any stream capture;
 * the address is kept for the life of the process, so after cudaDeviceReset on a device this entry
 * point must not be used there again. All calls share the array: calls that overlap on the GPU race.
 * The context must have been created (which allocates) beforehand, with the same device current. */
#define UEPM_NOALLOC_SCRATCH_BYTES (16u << 20)
int uepm_assemble_device_noalloc(uepm_ctx* ctx, const double* d_k, size_t nk, double* d_H, void* stream);

/* BandStructure::AdjustValues (FindBandGap + shift) on host E (nk x nb). Returns the gap via *gap
 * and whether FindBandGap succeeded via *found. soc selects 8 instead of 4 valence bands. */
int uepm_adjust_values(double* E, size_t nk, int nb, int soc, int min_cond_zero, double* gap, int* found);

/* Diagnostics (no reference counterpart): the FP64 Sturm count's pivot step, r = 1 / guard(q), for
 * n device values q (guard: a pivot within pivmin becomes -pivmin, as in the bisection), written to
 * device r, enqueued on `stream`. Exposes the refined hardware reciprocal the bisection uses so that
 * tests can bound it against the correctly rounded 1.0 / q. pivmin must be positive. */
int uepm_pivot_reciprocal_device(const double* d_q, double pivmin, size_t n, double* d_r, void* stream);

/* Diagnostics (no reference counterpart): the double-single special functions the mixed path's
 * gaussian-well elements use, on n device values x (rounded to FP32 pairs), written to device y as
 * h + l, enqueued on `stream`. fn 0: e^x for 2 < x <= 80 (Cody-Waite reduction and a degree-13
 * Taylor series); fn 1: i2(x) = ((x^2 + 3) sinh x - 3 x cosh x) / x^3 for 2 < x <= 80, the closed
 * form bessel_func.hpp:47-52 defines, with that e^x. Lets tests bound them against high-precision
 * values. */
int uepm_ds_special_device(int fn, const double* d_x, size_t n, double* d_y, void* stream);

/* Launch counters (kernels enqueued by this library since load), for launch accounting. */
uint64_t uepm_kernel_launches(void);

/* Per-kernel device timing for profiling (no reference counterpart; the reference only has
 * whole-second wall timers, BandStructure.cpp:126-148). When on, every kernel a solve enqueues is
 * bracketed by CUDA events on the launching stream. uepm_ctx_read_profile waits for the recorded
 * events and returns, per kernel kind, the accumulated milliseconds and launch counts since
 * profiling was switched on. Kinds: see uepm_kernel_name (0..UEPM_KERNEL_KINDS-1). */
#define UEPM_KERNEL_KINDS 10
int uepm_ctx_set_profiling(uepm_ctx* ctx, int on);
int uepm_ctx_read_profile(uepm_ctx* ctx, double* ms, uint64_t* launches, int capacity);
const char* uepm_kernel_name(int kind);

/* Calibration (no reference counterpart): sustained FMA throughput of the current device's FP64
 * pipe (precision UEPM_PREC_FP64) or FP32 pipe (UEPM_PREC_MIXED), in TFLOP/s, measured with a
 * pure-FMA kernel. Used as the roofline denominator of the compute-bound kernels. */
int uepm_measure_peak(int precision, double* tflops);

/* ---- Tuning (no reference counterpart) -------------------------------------------------------
 * Kernel-shape choices of a context. 0 in a field means "automatic":
 *   reduction     the Householder reduction kernel: 1 register-resident (FP32 real matrices, n <= 176),
 *                 2 one CTA per matrix (shared memory where the matrix fits, else global memory with
 *                 a persistent grid), 3 one thread-block cluster per matrix, the matrix spread over
 *                 the cluster's shared memory (orders beyond one SM), 4 one CTA per matrix in global
 *                 memory with each step's update fused into the next step's product (FP32 matrices
 *                 beyond the on-chip sizes, n <= 512), 5 the same with every other update deferred
 *                 to the next pass (a read-only pass, then a rank-4 pass: 3 passes per two steps), 6 blocked:
 *                 panels of 16 columns whose updates are applied once per panel, only the lower
 *                 triangle read and written, one matrix per SM (FP32, n <= 512);
 *                 automatic: 1 where it applies, 6 for the FP32 orders 200..512 (real: 300..512), 5 for the other FP32
 *                 matrices, else 2
 *   ctas_per_sm   CTAs per SM of the global-memory reduction (its L2 working set), 1..8
 *   vector_lanes  lanes per eigenvector in the back-transformation: 8, 16 or 32
 *   chunk         k-points per pipeline pass (smaller keeps H(k) resident in L2 between the
 *                 kernels of a pass), 64..32768
 *   cluster       CTAs per cluster of reduction 3: 2, 4, 8 or 16
 *   max_iter      iteration cap (0..1000) of the iterative kernels: bisection steps per phase
 *                 (automatic 64 / 200), inverse-iteration solves per vector (automatic 4 FP32, 5 FP64)
 *                 and projected-Jacobi sweeps (automatic 12). A k-point whose iteration the cap ends
 *                 before it converged gets UEPM_K_NOCONVERGE, and uepm_solve returns
 *                 UEPM_ERR_NOT_CONVERGED (the reference throws "Eigenvalue decomposition failed"
 *                 when Eigen reports NoConvergence, Hamiltonian.cpp:129-133). Not a shape: the
 *                 autotuner keeps the context's value.
 *   tensor_cores  0 (automatic): the mixed path's complex contractions run on the tensor cores
 *                 (tcgen05) where they apply: the blocked reduction's panel updates (TF32 with
 *                 hi/lo operand splits, FP32-level products) and, from order 150, the Rayleigh-Ritz
 *                 product H X (BF16 integer slices of H and X, exact to double-single level);
 *                 1: every product on the FP32 pipe (SIMT). Kept by the autotuner.
 *   streams       0 (automatic): a mixed-precision uepm_solve_device / uepm_solve of 1024 or more
 *                 k-points that fits one pipeline pass runs as two halves on two streams (the
 *                 caller's and one of the context, forked and joined on the caller's stream), so
 *                 that one half's later kernels run beside the other half's reduction; 1: one
 *                 stream; 2: two streams for any solve of two or more k-points, consecutive passes
 *                 alternating. The results are the same bits. Kept by the autotuner.
 * Every choice gives results within the parity tolerances; a given choice is deterministic.
 * uepm_ctx_autotune times candidate shapes on sample_k seeded random first-zone k-points (coordinate
 * descent over the fields, CUDA events on `stream`) and keeps the fastest; results are cached
 * process-wide per (device, n, real/complex, precision, nb, vectors) so that contexts of the same
 * shape reuse them. It allocates and synchronises: call it before capturing work into a graph. */
typedef struct uepm_tuning {
    int32_t reduction;
    int32_t ctas_per_sm;
    int32_t vector_lanes;
    int32_t chunk;
    int32_t cluster;
    int32_t max_iter;
    int32_t tensor_cores;
    int32_t streams;
} uepm_tuning;
int uepm_ctx_get_tuning(const uepm_ctx* ctx, uepm_tuning* out);
int uepm_ctx_set_tuning(uepm_ctx* ctx, const uepm_tuning* t);
int uepm_ctx_autotune(uepm_ctx* ctx, int nb, uint32_t want, size_t sample_k, void* stream);

/* ---- Uneven batches (no reference counterpart; the reference runs one material at a time,
 * BandStructure::Compute_parallel, BandStructure.cpp:162-201) ---------------------------------
 * A batch holds groups: (context, device k-points, nb, want, device outputs), each with the meaning
 * and layout of uepm_solve_device. Contexts may differ in material, basis, SOC and precision.
 * uepm_batch_run enqueues every group on `stream`: each distinct context gets its own internal
 * stream (forked from and joined back to `stream`), so groups of different shapes run concurrently
 * and fill the GPU together; groups of the same context run in order (they share its workspace).
 * With graphs on (the default), the first run captures the whole fork/join pipeline into a CUDA
 * graph and later runs replay it with one launch, as long as the groups are unchanged (the k-points
 * and outputs are read and written through the registered device pointers at every run). Workspaces
 * are allocated before capture. Adding or clearing groups drops the graph. Not thread-safe per
 * batch; a context must not be used by another call while a run of the batch is in flight. */
typedef struct uepm_batch uepm_batch;
int  uepm_batch_create(uepm_batch** out);
void uepm_batch_destroy(uepm_batch* b);
int  uepm_batch_add(uepm_batch* b, uepm_ctx* ctx, const double* d_k, size_t nk, int nb, uint32_t want, double* d_E,
                    double* d_X, double* d_grad, int32_t* d_status);
int  uepm_batch_clear(uepm_batch* b);
int  uepm_batch_set_graph(uepm_batch* b, int on);
int  uepm_batch_run(uepm_batch* b, void* stream);
/* Kernels enqueued by one run of the batch (counted while capturing). */
uint64_t uepm_batch_kernels_per_run(const uepm_batch* b);

/* Irreducible wedge -> full Brillouin zone (MeshBZ::distribute_energies_from_iw_wedge_to_full_bz,
 * src/BZ_MESH/bz_mesh.cpp:1383-1414), as a device gather after the solve of the wedge vertices:
 * for each of n_full vertices v, E_full[v][:] = E_iw[src[v]][:] and, when gradients are given,
 * grad_full[v][b][j] = s_j * grad_iw[src[v]][b][p_j], the signed permutation (p, s) that maps the
 * wedge k-point onto vertex v (apply_same_symmetry_operation, bz_mesh.cpp:1312-1381), packed in
 * op[v] as p_0 | p_1 << 2 | p_2 << 4 | (s_0 < 0) << 6 | (s_1 < 0) << 7 | (s_2 < 0) << 8.
 * All pointers are device pointers; E is [.][nb], gradients [.][nb][3]; enqueued on `stream`. */
int uepm_star_expand_device(const double* d_E_iw, const double* d_grad_iw, const int64_t* d_src, const uint16_t* d_op,
                            size_t n_full, int nb, double* d_E_full, double* d_grad_full, void* stream);

/* Dielectric function from the eigenstates at k and k + q: the per-q body of
 * DielectricFunction::compute_dielectric_function (src/EPP/DielectricFunction.cpp:92-150), and,
 * with per-vertex weights (the volume / 4 of each tetrahedron holding the vertex), the tetrahedron
 * sums of BZ_States::compute_dielectric_function (src/BZ_MESH/bz_states.cpp:101-140). For each of
 * nk k-points, the P = (nb - first_cond) * first_cond squared overlaps
 * O_cv = |sum_i u_c(k+q)_i u_v(k)_i|^2 (conduction c in [first_cond, nb) at k + q, valence
 * v < first_cond at k; no factor conjugated, as the reference's Eigen expression
 * col(c).adjoint().dot(col(v)) evaluates, which equals |<u_c|u_v>|^2 for a real H) and
 * differences dE_cv = E_c(k+q) - E_v(k) give, at each of ne energies w,
 *   s_k(w) = sum_{c,v} O_cv [(dE - w) / ((dE - w)^2 + eta^2) + (dE + w) / ((dE + w)^2 + eta^2)],
 * and weights[k] * s_k(w) (weights NULL: 1) is ADDED to sums[w]. X_k, X_kq: [nk][nb][n] complex
 * (re, im doubles: the layout uepm_solve writes), E_k, E_kq: [nk][nb], energies [ne], sums [ne];
 * all device pointers, enqueued on `stream` with stream-ordered scratch (2 * SMs * ne doubles).
 * ne <= 4096; nb * n complex must fit one CTA's shared memory (n <= ~780 at nb = 16). The sums are
 * deterministic (fixed reduction order). */
int uepm_dielectric_sums_device(const double* d_Xk, const double* d_Xkq, const double* d_Ek, const double* d_Ekq,
                                size_t nk, int nb, int n, int first_cond, const double* d_energies, int ne, double eta,
                                const double* d_weights, double* d_sums, void* stream);
/* Host: the packed signed permutations op[q] mapping k_src[q] onto k_dst[q] (n pairs of reduced or
 * SI k-points, the rule of apply_same_symmetry_operation); found[q] = 0 (optional) where none
 * exists, with the identity written. */
int uepm_star_operations(const double* k_src, const double* k_dst, size_t n, uint16_t* op, int32_t* found);

/* ---- Serving (no reference counterpart; the reference's full-band Monte Carlo interpolates bands
 * on a mesh, src/FBMC/particle.cpp:52-63) -------------------------------------------------------
 * A query server over resident contexts (all on one device; not owned: keep them alive and unused
 * by other calls until the server is destroyed). A scheduler thread cuts each request into work
 * items of at most max_chunk k-points and runs them on `slots` streams, admitting an item only when
 * a slot is free and a sub-range of the device arena (hbm_budget bytes, allocated here once) can hold
 * its footprint: the solve workspace plus its k-points, energies and status. Items of requests that
 * arrive while others run are admitted as slots and memory free up (continuous batching); results
 * are the same whether a request runs alone or in the mix.
 * uepm_server_submit copies k (nk x 3, reduced units) and returns a request id (>= 0) at once; the
 * server writes E (nk x nb, eV), status (nk, optional) and, with UEPM_SERVE_VELOCITY, the group
 * velocities V (nk x nb x 3, m/s) by central differences of step fd_step (reduced units) along each
 * axis (7 solves per k-point). The host buffers must stay valid until uepm_server_wait returns for the
 * id (UEPM_OK when done, 1 on timeout; timeout_s < 0 waits indefinitely). uepm_server_stats reports
 * the latency (submission to completion) percentiles of the requests completed since the last reset,
 * how many, their k-points and the span from the first submission to the last completion. */
#define UEPM_SERVE_VELOCITY 1u
typedef struct uepm_server uepm_server;
int     uepm_server_create(uepm_ctx* const* ctxs, int nctx, size_t hbm_budget, int slots, size_t max_chunk, int max_nb,
                           uepm_server** out);
int     uepm_server_destroy(uepm_server* sv);
int64_t uepm_server_submit(uepm_server* sv, int ctx_index, const double* k, size_t nk, int nb, uint32_t flags,
                           double fd_step, double* E, double* V, int32_t* status);
int     uepm_server_wait(uepm_server* sv, int64_t id, double timeout_s);
int     uepm_server_stats(uepm_server* sv, double* p50_ms, double* p99_ms, uint64_t* completed, uint64_t* kpoints,
                          double* span_s);
int     uepm_server_reset_stats(uepm_server* sv);

#ifdef __cplusplus
}
#endif
#endif /* UEPM_GB300_H */
