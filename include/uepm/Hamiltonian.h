// Hamiltonian.h -- uepm::pseudopotential::Hamiltonian (src/EPP/Hamiltonian.h:10-32) on the GB300
// library: SetMatrix records k and the flags, Diagonalize solves H(k) on the GPU (all n eigenvalues,
// and all eigenvectors when asked, like Eigen's SelfAdjointEigenSolver), the results are kept on the
// host with the reference's accessors. Like the reference, it keeps references to the material and
// the basis (the caller keeps them alive) and one instance is not thread-safe.
#pragma once

#include <map>
#include <memory>
#include <tuple>
#include <vector>

#include "DenseTypes.h"
#include "Material.h"
#include "Vector3D.h"

struct uepm_ctx;

namespace uepm::pseudopotential {

class Hamiltonian {
 public:
    Hamiltonian(const Material& material, const std::vector<Vector3D<int>>& basisVectors);
    Hamiltonian(const Hamiltonian& other);
    Hamiltonian& operator=(const Hamiltonian&) = delete;
    ~Hamiltonian();

    // k-independent part: built on the GPU when the context is created; kept for API parity
    void SetConstantNonDiagonalMatrix() {}

    void SetMatrix(const Vector3D<double>& k, bool add_non_local_correction = false, bool enable_soc = false);
    // Throws std::runtime_error("Eigenvalue decomposition failed") on a non-finite solve.
    void Diagonalize(bool keep_eigenvectors = false);

    // No reference counterpart: solves every k of `kpoints` in one batched device solve and keeps the
    // results, so that a caller's loop SetMatrix(k, nl, soc) / Diagonalize(keep) over these k-points
    // (bz_states.cpp:30-47, DielectricFunction.cpp:92-119) takes them from the batch instead of one
    // launch per k. The results are bit-identical to the per-k solve (the same kernels per matrix).
    // A k (compared exactly) or flags not in the batch, or eigenvectors asked when the batch kept
    // none, fall back to the per-k solve. Host memory: n doubles per k, plus n x n complex per k with
    // keep_eigenvectors. A new call replaces the batch; ClearBatch() drops it.
    void PrepareBatch(const std::vector<Vector3D<double>>& kpoints, bool add_non_local_correction = false,
                      bool enable_soc = false, bool keep_eigenvectors = false);
    void ClearBatch();

    const RealVector&    get_eigenvalues() const { return m_values; }
    const ComplexMatrix& get_eigenvectors() const { return m_vectors; }
    const RealVector&    eigenvalues() const { return m_values; }
    // The reference compares the stored H(k) with its transpose (Hamiltonian.h:22), so it answers
    // true for a real H(k) and false for a complex one (spin-orbit, antisymmetric form factors,
    // unequal anion / cation nonlocal parameters); the same answer here, from the context's type.
    // True before the first SetMatrix.
    bool check_matrix_is_symmetric() const;
    // Hellmann-Feynman kinetic gradient of band level_index at k_point, from the kept eigenvectors
    // (src/EPP/Hamiltonian.cpp:146-194); throws std::runtime_error / std::out_of_range like the reference.
    Vector3D<double> compute_gradient_at_level(const Vector3D<double>& k_point, unsigned int level_index) const;

 protected:
    const Material&                   m_material;
    const std::vector<Vector3D<int>>& m_basisVectors;

 private:
    uepm_ctx*         context(bool nl, bool soc) const;
    mutable uepm_ctx* m_ctx[4] = {nullptr, nullptr, nullptr, nullptr};  // per (nl, soc)
    Vector3D<double>  m_k;
    bool              m_nl = false, m_soc = false, m_set = false;
    RealVector       m_values;
    ComplexMatrix    m_vectors;
    // the prefetched batch: k -> row, its flags, values [nk][n] and vectors [nk][n][n] (re, im)
    std::map<std::tuple<double, double, double>, size_t> m_batch_row;
    bool                m_batch_nl = false, m_batch_soc = false, m_batch_vec = false;
    int                 m_batch_n  = 0;
    std::vector<double> m_batch_E, m_batch_X;
};

}  // namespace uepm::pseudopotential
