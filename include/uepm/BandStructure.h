// BandStructure.h -- uepm::pseudopotential::BandStructure (src/EPP/BandStructure.h:11-110) on the
// GB300 library: Compute / Compute_parallel run the whole k batch as one device solve. Same members,
// same quirks (SOC doubles the number of bands, AdjustValues shifts 4 or 8 valence bands, the
// computation time is kept in whole seconds) and the same exceptions.
#pragma once

#include <string>
#include <vector>

#include "Material.h"
#include "SymmetryPoints.h"
#include "Vector3D.h"

namespace uepm::pseudopotential {

enum class SolvePrecision { fp64, mixed };

class BandStructure {
 public:
    BandStructure() : m_nb_points(0), m_nb_bands(10), m_nearestNeighborsNumber(10), m_computation_time_s(-1.0) {}

    void Initialize(const Material& material, std::size_t nb_bands, const std::vector<std::string>& path,
                    unsigned int nrPoints, unsigned int nearestNeighborsNumber, bool enable_non_local_correction,
                    bool enable_soc);
    void Initialize(const Material& material, std::size_t nb_bands, const std::vector<Vector3D<double>>& list_k_points,
                    unsigned int nearestNeighborsNumber, bool enable_non_local_correction, bool enable_soc);

    const std::vector<std::string>& GetPath() const { return m_path; }
    std::string                     get_path_as_string() const;
    unsigned int                    GetPointsNumber() const { return static_cast<unsigned int>(m_kpoints.size()); }
    void                            Compute(bool compute_gradient = false);
    // nb_threads is accepted for source compatibility; the batch runs on the GPU.
    void   Compute_parallel(bool compute_gradient = false, int nb_threads = 1);
    double AdjustValues(bool minConductionBandToZero = false);

    void        print_results() const;
    std::string path_band_filename() const;
    void        export_k_points_to_file(std::string filename) const;
    void        export_result_in_file(const std::string& filename) const;
    void        export_result_in_file_with_kpoints(const std::string& filename) const;

    unsigned int        get_number_of_bands() const { return m_nb_bands; }
    std::vector<double> get_band(unsigned int band_index) const;
    double get_energy_at_k_band(unsigned int band_index, unsigned int index_k) const { return m_energies[index_k][band_index]; }

    const std::vector<Vector3D<int>>&                 get_basis_vectors() const { return basisVectors; }
    const std::vector<Vector3D<double>>&              get_kpoints() const { return m_kpoints; }
    const std::vector<std::vector<double>>&           get_band_energies() const { return m_energies; }
    const std::vector<std::vector<Vector3D<double>>>& get_band_energy_gradients() const { return m_energies_gradient; }

    void set_kpoints(const std::vector<Vector3D<double>>& kpoints) { m_kpoints = kpoints; }

    double get_computation_time_s() const { return m_computation_time_s; }
    bool   is_soc_enabled() const { return m_enable_spin_orbit_coupling; }

    // GB300 extension: FP64 (default, the drop-in) or mixed precision (<= 1e-6 eV from FP64)
    void           set_precision(SolvePrecision p) { m_precision = p; }
    SolvePrecision get_precision() const { return m_precision; }

 private:
    SymmetryPoints            symmetryPoints;
    std::vector<unsigned int> symmetryPointsPositions;
    std::vector<std::string>  m_path;
    unsigned int              m_nb_points;

    Material     m_material;
    unsigned int m_nb_bands;
    unsigned int m_nearestNeighborsNumber;
    bool         m_enable_non_local_correction = false;
    bool         m_enable_spin_orbit_coupling  = false;

    std::vector<Vector3D<int>>                 basisVectors;
    std::vector<Vector3D<double>>              m_kpoints;
    std::vector<std::vector<double>>           m_energies;
    std::vector<std::vector<Vector3D<double>>> m_energies_gradient;

    double         m_computation_time_s;
    SolvePrecision m_precision = SolvePrecision::fp64;

    bool GenerateBasisVectors(unsigned int nearestNeighborsNumber);
    void run(bool compute_gradient);
};

void export_vector_bands_result_in_file(const std::string& filename, std::vector<std::vector<double>>);

}  // namespace uepm::pseudopotential
