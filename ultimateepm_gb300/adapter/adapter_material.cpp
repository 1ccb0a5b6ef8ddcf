// adapter_material.cpp -- Material / Materials / SymmetryPoints / Options of the C++ adapter.
#include <cstring>
#include <iostream>
#include <stdexcept>
#include <vector>

#include "Material.h"
#include "Options.h"
#include "SymmetryPoints.h"
#include "uepm_gb300.h"

namespace uepm::pseudopotential {

Material::Material(const std::string& Name, double a, double V3S, double V4S, double V8S, double V11S, double V3A,
                   double V4A, double V8A, double V11A)
    : m_name(Name) {
    std::memset(&raw_, 0, sizeof(raw_));
    raw_.lattice_constant = a;
    raw_.V3S              = V3S;
    raw_.V4S              = V4S;
    raw_.V8S              = V8S;
    raw_.V11S             = V11S;
    raw_.V3A              = V3A;
    raw_.V4A              = V4A;
    raw_.V8A              = V8A;
    raw_.V11A             = V11A;
}

NonLocalParameters Material::get_non_local_parameters() const {
    NonLocalParameters p;
    p.m_alpha_0_cation = raw_.alpha0_cation;
    p.m_beta_0_cation  = raw_.beta0_cation;
    p.m_A2_cation      = raw_.A2_cation;
    p.m_alpha_0_anion  = raw_.alpha0_anion;
    p.m_beta_0_anion   = raw_.beta0_anion;
    p.m_A2_anion       = raw_.A2_anion;
    p.m_R0_cation      = raw_.R0_cation;
    p.m_R2_cation      = raw_.R2_cation;
    p.m_R0_anion       = raw_.R0_anion;
    p.m_R2_anion       = raw_.R2_anion;
    p.m_well_type      = raw_.nl_well == 1   ? non_local_well_type::square
                         : raw_.nl_well == 2 ? non_local_well_type::gaussian
                                             : non_local_well_type::unknown;
    return p;
}

SpinOrbitParameters Material::get_spin_orbit_parameters() const {
    SpinOrbitParameters p;
    p.m_period_anion         = raw_.period_anion;
    p.m_period_cation        = raw_.period_cation;
    p.m_radial_extent_anion  = raw_.radial_extent_anion;
    p.m_radial_extent_cation = raw_.radial_extent_cation;
    p.m_alpha                = raw_.alpha_soc;
    p.m_mu                   = raw_.mu_soc;
    return p;
}

void SpinOrbitParameters::print_parameters() const {
    std::cout << "Spin-Orbit Coupling parameters:" << std::endl;
    std::cout << "Period anion: " << m_period_anion << std::endl;
    std::cout << "Period cation: " << m_period_cation << std::endl;
    std::cout << "Radial extent anion: " << m_radial_extent_anion << std::endl;
    std::cout << "Radial extent cation: " << m_radial_extent_cation << std::endl;
    std::cout << "Alpha: " << m_alpha << std::endl;
    std::cout << "Mu: " << m_mu << std::endl;
}

void Materials::load_material_parameters(const std::string& filename) {
    const int cnt = uepm_materials_load(filename.c_str(), nullptr, nullptr, 0, 0);
    if (cnt < 0) throw std::runtime_error(uepm_last_error());
    constexpr int              stride = 64;
    std::vector<uepm_material> mats((size_t)cnt);
    std::vector<char>          syms((size_t)cnt * stride);
    uepm_materials_load(filename.c_str(), mats.data(), syms.data(), stride, cnt);
    for (int i = 0; i < cnt; ++i) {
        const std::string sym(&syms[(size_t)i * stride]);
        materials[sym] = Material(sym, mats[(size_t)i]);
    }
}

void Materials::print_materials_list() const {
    for (const auto& m : materials) std::cout << m.first << std::endl;
}

void Materials::print_material_parameters(const std::string& name) const {
    if (materials.find(name) == materials.end()) {
        std::cout << "Material " << name << " not found" << std::endl;
        return;
    }
    std::cout << "Material: " << name << std::endl;
    std::cout << "Lattice constant: " << materials.at(name).get_lattice_constant_meter() << " Bohr" << std::endl;
    std::cout << "-------------------------------------" << std::endl;
}

void Materials::print_material_parameters() const {
    for (const auto& m : materials) print_material_parameters(m.first);
}

SymmetryPoints::SymmetryPoints() {
    symmetryPoints["L"] = SymmetryPoint("L", Vector3D<double>(0.5, 0.5, 0.5));
    symmetryPoints["G"] = SymmetryPoint("G", Vector3D<double>(0., 0., 0.));
    symmetryPoints["X"] = SymmetryPoint("X", Vector3D<double>(1., 0., 0.));
    symmetryPoints["W"] = SymmetryPoint("W", Vector3D<double>(1., 0.5, 0.));
    symmetryPoints["K"] = SymmetryPoint("K", Vector3D<double>(0.75, 0.75, 0.));
    symmetryPoints["U"] = SymmetryPoint("U", Vector3D<double>(1., 0.25, 0.25));
}

std::vector<Vector3D<double>> SymmetryPoints::GeneratePoints(const std::vector<std::string>& path, unsigned int nrPoints,
                                                             std::vector<unsigned int>& symmetryPointsPositions) {
    std::string labels;
    for (const auto& p : path) {
        if (p.size() != 1 || symmetryPoints.find(p) == symmetryPoints.end())
            throw std::invalid_argument("Unknown symmetry point label: " + p);
        labels += p;
    }
    std::vector<double>   k(3 * (size_t)std::max(nrPoints, 1u));
    std::vector<uint32_t> pos(std::max<size_t>(labels.size(), 1));
    const int             cnt = uepm_generate_path(labels.c_str(), nrPoints, k.data(), (int)nrPoints, pos.data());
    if (cnt < 0) throw std::invalid_argument(uepm_last_error());
    std::vector<Vector3D<double>> out((size_t)cnt);
    for (int i = 0; i < cnt; ++i) out[(size_t)i] = Vector3D<double>(k[3 * i], k[3 * i + 1], k[3 * i + 2]);
    symmetryPointsPositions.assign(pos.begin(), pos.begin() + labels.size());
    return out;
}

}  // namespace uepm::pseudopotential

Options::Options()
    : nrThreads(4), materialName("Si"), nrPoints(60), nearestNeighbors(12), nrLevels(30), pathNo(1),
      paths{{
          {"K", "W", "X", "G", "L", "W"},
          {"W", "G", "X", "W", "L", "G"},
          {"W", "L", "G", "X", "W", "K"},
          {"L", "G", "X", "K", "G"},
          {"L", "G", "X", "W", "K", "G"},
          {"L", "G", "X", "U", "K", "G"},
          {"L", "G", "X", "U", "G"},
          {"L", "K", "W", "G", "X", "W", "L", "G", "K"},
          {"G", "X", "K", "G", "L", "K", "W", "X"},
          {"G", "X", "W", "L", "G", "K", "W", "U"},
          {"G", "X", "W", "L", "G", "K"},
          {"G", "X", "W", "L", "G", "K", "X"},
          {"G", "X", "W", "L", "G", "X"},
          {"G", "X", "W", "G", "U", "X"},
          {"G", "X", "W", "K", "L", "G"},
          {"G", "X", "W", "K", "G", "L", "U", "W", "L", "K"},
          {"G", "X", "U", "K", "G", "L", "W", "X"},
      }} {}

void Options::print_options() {
    std::cout << "Options:" << std::endl;
    std::cout << "nrThreads: " << nrThreads << std::endl;
    std::cout << "materialName: " << materialName << std::endl;
    std::cout << "nrPoints: " << nrPoints << std::endl;
    std::cout << "nearestNeighbors: " << nearestNeighbors << std::endl;
    std::cout << "nrLevels: " << nrLevels << std::endl;
    std::cout << "pathNo: " << pathNo << std::endl;
}
