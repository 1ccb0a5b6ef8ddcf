// Hamiltonian.h -- uepm::pseudopotential::Hamiltonian (src/EPP/Hamiltonian.h:10-32) on the GB300
// library: SetMatrix records k and the flags, Diagonalize solves H(k) on the GPU (all n eigenvalues,
// and all eigenvectors when asked, like Eigen's SelfAdjointEigenSolver), the results are kept on the
// host with the reference's accessors. Like the reference, it keeps references to the material and
// the basis (the caller keeps them alive) and one instance is not thread-safe.
#pragma once

#include <memory>
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
};

}  // namespace uepm::pseudopotential
