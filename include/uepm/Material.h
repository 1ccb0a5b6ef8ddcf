// Material.h -- uepm::pseudopotential::Material / Materials (src/EPP/Material.h:14-187), over the
// GB300 library's material record. Same constructor, getters and YAML loading semantics (form
// factors, alpha_0 and A2 converted from Ry to eV, radii from Angstrom to m). The members that take
// yaml-cpp nodes (populate_*_parameters(const YAML::Node&)) are not provided: this build has no
// yaml-cpp; load_material_parameters parses the same files itself.
#pragma once

#include <cmath>
#include <map>
#include <string>

#include "Vector3D.h"
#include "uepm_gb300.h"

namespace uepm::pseudopotential {

enum class non_local_well_type { square, gaussian, unknown };

struct NonLocalParameters {
    double              m_alpha_0_cation = 0, m_beta_0_cation = 0, m_A2_cation = 0;
    double              m_alpha_0_anion = 0, m_beta_0_anion = 0, m_A2_anion = 0;
    double              m_R0_cation = 0, m_R2_cation = 0, m_R0_anion = 0, m_R2_anion = 0;
    non_local_well_type m_well_type = non_local_well_type::unknown;
};

struct SpinOrbitParameters {
    unsigned int m_period_anion = 0, m_period_cation = 0;
    double       m_radial_extent_cation = 0, m_radial_extent_anion = 0, m_alpha = 0, m_mu = 0;
    void         print_parameters() const;
};

class Material {
 public:
    Material() { raw_.lattice_constant = 0; }
    // form factors in eV, as the reference's constructor takes them
    Material(const std::string& Name, double a, double V3S, double V4S, double V8S, double V11S, double V3A = 0,
             double V4A = 0, double V8A = 0, double V11A = 0);
    explicit Material(const std::string& name, const uepm_material& raw) : m_name(name), raw_(raw) {}

    const std::string& get_name() const { return m_name; }
    double get_lattice_constant_meter() const { return 1.0e-10 * raw_.lattice_constant; }
    double get_fourier_factor() const { return 2.0 * M_PI / (1.0e-10 * raw_.lattice_constant); }
    double get_atomic_volume_angstrom() const { return (1.0 / 8.0) * std::pow(raw_.lattice_constant, 3.0); }
    double get_atomic_volume() const { return (1.0 / 8.0) * std::pow(get_lattice_constant_meter(), 3.0); }
    double get_fermi_momentum() const { return std::pow(96 * M_PI * M_PI, 1.0 / 3.0) / get_lattice_constant_meter(); }

    bool is_non_local_parameters_populated() const { return raw_.has_nonlocal != 0; }
    bool is_spin_orbit_parameters_populated() const { return raw_.has_soc != 0; }
    void set_is_non_local_parameters_populated(bool v) { raw_.has_nonlocal = v ? 1 : 0; }
    void set_is_spin_orbit_parameters_populated(bool v) { raw_.has_soc = v ? 1 : 0; }

    NonLocalParameters  get_non_local_parameters() const;
    SpinOrbitParameters get_spin_orbit_parameters() const;

    // the record the GB300 library takes (units as after loading a YAML file)
    const uepm_material& raw() const { return raw_; }
    uepm_material&       raw() { return raw_; }

 private:
    std::string   m_name;
    uepm_material raw_{};
};

class Materials {
 public:
    Materials() = default;
    // Materials::load_material_parameters (src/EPP/Material.cpp:33-71); throws std::runtime_error.
    void load_material_parameters(const std::string& filename);

    std::map<std::string, Material> materials;

    void print_materials_list() const;
    void print_material_parameters(const std::string& material_name) const;
    void print_material_parameters() const;
};

}  // namespace uepm::pseudopotential
