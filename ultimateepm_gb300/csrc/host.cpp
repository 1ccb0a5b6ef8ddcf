// host.cpp -- host-side pieces of the C ABI that need no GPU: basis generation, the symmetry-point
// path, the material YAML loader and the band-gap shift. Plain C++17, no CUDA.
#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <fstream>
#include <limits>
#include <map>
#include <memory>
#include <numeric>
#include <sstream>
#include <string>
#include <vector>

#include "uepm_gb300.h"

namespace uepm {
void set_error(const std::string& msg);
}

namespace {

// The 116 squared lengths of fcc reciprocal-lattice shells (units of (2pi/a)^2) that
// BandStructure::GenerateBasisVectors (src/EPP/BandStructure.cpp:27-32) uses as cut-offs.
const unsigned kShellG2[] = {
    0,   3,   4,   8,   11,  12,  16,  19,  20,  24,  27,  32,  35,  36,  40,  43,  44,  48,  51,  52,  56,  59,  67,  68,
    75,  76,  80,  83,  84,  88,  96,  99,  104, 107, 108, 115, 116, 120, 123, 128, 131, 132, 136, 139, 140, 144, 147, 152,
    155, 160, 163, 164, 168, 171, 172, 176, 179, 180, 184, 187, 192, 195, 196, 200, 203, 204, 208, 211, 212, 216, 219, 224,
    227, 228, 232, 236, 243, 244, 248, 251, 259, 260, 264, 267, 268, 272, 275, 276, 280, 283, 291, 296, 299, 300, 304, 307,
    308, 312, 315, 320, 323, 324, 331, 332, 339, 355, 356, 360, 363, 371, 376, 384, 387, 395, 420, 451};
constexpr unsigned kShellCount = sizeof(kShellG2) / sizeof(kShellG2[0]);

// ------------------------------------------------------------------------------------------------
// A small reader for the block-style YAML subset of the material files: nested maps, a sequence
// of maps, plain or quoted scalars, comments and the document marker.
struct YNode {
    enum Kind { Scalar, Map, Seq } kind = Scalar;
    std::string                                   value;
    std::vector<std::pair<std::string, YNode>>    map;
    std::vector<YNode>                            seq;
    const YNode* get(const std::string& key) const {
        for (const auto& kv : map)
            if (kv.first == key) return &kv.second;
        return nullptr;
    }
};

struct YLine {
    int         indent;
    std::string text;
};

std::string trim(const std::string& s) {
    size_t a = 0, b = s.size();
    while (a < b && std::isspace((unsigned char)s[a])) ++a;
    while (b > a && std::isspace((unsigned char)s[b - 1])) --b;
    return s.substr(a, b - a);
}

std::string unquote(const std::string& s) {
    if (s.size() >= 2 && (s.front() == '"' || s.front() == '\'') && s.back() == s.front()) return s.substr(1, s.size() - 2);
    return s;
}

class YParser {
 public:
    explicit YParser(std::vector<YLine> lines) : L(std::move(lines)) {}
    YNode parse() { return L.empty() ? YNode{} : block(L[0].indent); }

 private:
    std::vector<YLine> L;
    size_t             pos = 0;

    static bool is_item(const std::string& t) { return t == "-" || (t.size() >= 2 && t[0] == '-' && t[1] == ' '); }

    YNode block(int indent) {
        YNode node;
        if (pos < L.size() && is_item(L[pos].text)) {
            node.kind = YNode::Seq;
            while (pos < L.size() && L[pos].indent == indent && is_item(L[pos].text)) {
                std::string rest = trim(L[pos].text.substr(1));
                if (rest.empty()) {
                    ++pos;
                    node.seq.push_back(pos < L.size() ? block(L[pos].indent) : YNode{});
                } else {
                    // "- key: value" opens a map whose keys sit two columns to the right
                    L[pos].indent += 2;
                    L[pos].text = rest;
                    node.seq.push_back(block(indent + 2));
                }
            }
            return node;
        }
        node.kind = YNode::Map;
        while (pos < L.size() && L[pos].indent == indent && !is_item(L[pos].text)) {
            const std::string t     = L[pos].text;
            const size_t      colon = t.find(':');
            const std::string key   = trim(t.substr(0, colon));
            const std::string val   = colon == std::string::npos ? std::string() : trim(t.substr(colon + 1));
            ++pos;
            YNode child;
            if (!val.empty()) {
                child.value = unquote(val);
            } else if (pos < L.size() && L[pos].indent > indent) {
                child = block(L[pos].indent);
            } else if (pos < L.size() && L[pos].indent == indent && is_item(L[pos].text)) {
                child = block(indent);
            }
            node.map.emplace_back(key, std::move(child));
        }
        return node;
    }
};

bool read_yaml(const char* path, YNode* out, std::string* err) {
    std::ifstream f(path);
    if (!f) {
        *err = std::string("cannot open ") + path;
        return false;
    }
    std::vector<YLine> lines;
    std::string        raw;
    while (std::getline(f, raw)) {
        // strip comments that are not inside quotes
        bool   inq = false;
        char   q   = 0;
        size_t cut = raw.size();
        for (size_t i = 0; i < raw.size(); ++i) {
            const char c = raw[i];
            if (inq) {
                if (c == q) inq = false;
            } else if (c == '"' || c == '\'') {
                inq = true;
                q   = c;
            } else if (c == '#') {
                cut = i;
                break;
            }
        }
        std::string line = raw.substr(0, cut);
        while (!line.empty() && std::isspace((unsigned char)line.back())) line.pop_back();
        const std::string t = trim(line);
        if (t.empty() || t == "---" || t == "...") continue;
        int ind = 0;
        while (ind < (int)line.size() && line[ind] == ' ') ++ind;
        lines.push_back({ind, t});
    }
    *out = YParser(std::move(lines)).parse();
    return true;
}

bool as_double(const YNode* n, double* v) {
    if (!n || n->kind != YNode::Scalar) return false;
    char*        end = nullptr;
    const double d   = std::strtod(n->value.c_str(), &end);
    if (end == n->value.c_str()) return false;
    *v = d;
    return true;
}

}  // namespace

extern "C" {

int uepm_material_size(void) { return (int)sizeof(uepm_material); }

int uepm_generate_basis(unsigned shells, int32_t* G, int capacity) {
    if (shells < 2 || shells > kShellCount) {
        uepm::set_error("BandStructure::Initialize: GenerateBasisVectors failed (shell count must be between 2 and " +
                        std::to_string(kShellCount) + ")");
        return UEPM_ERR_RUNTIME;
    }
    const unsigned cut  = kShellG2[shells - 1];
    const int      half = (int)std::ceil(std::sqrt((double)cut));
    int            n    = 0;
    // G = i b1 + j b2 + k b3 with b1 = (-1,1,1), b2 = (1,-1,1), b3 = (1,1,-1), in i -> j -> k order:
    // this order fixes the row/column order of H.
    for (int i = -half; i <= half; ++i)
        for (int j = -half; j <= half; ++j)
            for (int k = -half; k <= half; ++k) {
                const int gx = -i + j + k, gy = i - j + k, gz = i + j - k;
                if ((unsigned)(gx * gx + gy * gy + gz * gz) <= cut) {
                    if (n < capacity && G) {
                        G[3 * n]     = gx;
                        G[3 * n + 1] = gy;
                        G[3 * n + 2] = gz;
                    }
                    ++n;
                }
            }
    return n;
}

int uepm_generate_path(const char* labels, unsigned n_points, double* k, int capacity, uint32_t* sym_pos) {
    struct P3 {
        double x, y, z;
    };
    auto lookup = [](char c, P3* p) {
        switch (c) {
            case 'L': *p = {0.5, 0.5, 0.5}; return true;
            case 'G': *p = {0.0, 0.0, 0.0}; return true;
            case 'X': *p = {1.0, 0.0, 0.0}; return true;
            case 'W': *p = {1.0, 0.5, 0.0}; return true;
            case 'K': *p = {0.75, 0.75, 0.0}; return true;
            case 'U': *p = {1.0, 0.25, 0.25}; return true;
            default: return false;
        }
    };
    const size_t M = labels ? std::strlen(labels) : 0;
    if (M < 2) {
        uepm::set_error("Path must contain at least two symmetry points.");
        return UEPM_ERR_INVALID;
    }
    if (n_points < M) {
        uepm::set_error("nrPoints must be at least the number of nodes in the path.");
        return UEPM_ERR_INVALID;
    }
    std::vector<P3> nodes(M);
    for (size_t i = 0; i < M; ++i)
        if (!lookup(labels[i], &nodes[i])) {
            uepm::set_error(std::string("Unknown symmetry point label: ") + labels[i]);
            return UEPM_ERR_INVALID;
        }
    int  count = 0;
    auto emit  = [&](const P3& p) {
        if (count < capacity && k) {
            k[3 * count]     = p.x;
            k[3 * count + 1] = p.y;
            k[3 * count + 2] = p.z;
        }
        ++count;
    };
    std::vector<double> seg(M - 1);
    for (size_t i = 1; i < M; ++i) {
        const double dx = nodes[i].x - nodes[i - 1].x, dy = nodes[i].y - nodes[i - 1].y, dz = nodes[i].z - nodes[i - 1].z;
        seg[i - 1]      = std::sqrt(dx * dx + dy * dy + dz * dz);
    }
    const double   total = std::accumulate(seg.begin(), seg.end(), 0.0);
    const unsigned rest  = n_points - (unsigned)M;
    size_t         ns    = 0;
    if (total == 0.0) {
        for (size_t j = 0; j < M; ++j) {
            if (sym_pos) sym_pos[ns] = (uint32_t)count;
            ++ns;
            emit(nodes[j]);
        }
        for (unsigned i = 0; i < rest; ++i) emit(nodes.back());
        return count;
    }
    // largest-remainder apportionment of the interior points to the segments by length
    std::vector<unsigned> share(M - 1);
    std::vector<double>   exact(M - 1);
    std::vector<size_t>   order(M - 1);
    unsigned              given = 0;
    for (size_t s = 0; s < M - 1; ++s) {
        exact[s] = (seg[s] / total) * (double)rest;
        share[s] = (unsigned)std::floor(exact[s]);
        given += share[s];
        order[s] = s;
    }
    std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) {
        return (exact[a] - std::floor(exact[a])) > (exact[b] - std::floor(exact[b]));
    });
    for (unsigned i = 0; i < rest - given; ++i) ++share[order[i]];
    if (sym_pos) sym_pos[ns] = (uint32_t)count;
    ++ns;
    emit(nodes[0]);
    for (size_t s = 0; s < M - 1; ++s) {
        const P3& A = nodes[s];
        const P3& B = nodes[s + 1];
        const P3  d = {B.x - A.x, B.y - A.y, B.z - A.z};
        for (unsigned i = 1; i <= share[s]; ++i) {
            const double t = (double)i / (double)(share[s] + 1);
            emit({A.x + d.x * t, A.y + d.y * t, A.z + d.z * t});
        }
        if (sym_pos) sym_pos[ns] = (uint32_t)count;
        ++ns;
        emit(B);
    }
    return count;
}

int uepm_materials_load(const char* path, uepm_material* out, char* symbols, int symbol_stride, int capacity) {
    YNode       root;
    std::string err;
    if (!path || !read_yaml(path, &root, &err)) {
        uepm::set_error(err.empty() ? "no path" : err);
        return UEPM_ERR_INVALID;
    }
    const YNode* list = root.get("materials");
    if (!list || list->kind != YNode::Seq) {
        uepm::set_error("YAML file has no 'materials' sequence");
        return UEPM_ERR_RUNTIME;
    }
    // Ry -> eV as in Material.cpp:40-53 (physical_constants.hpp:33-37)
    constexpr double q_e       = 1.602176634e-19;
    constexpr double Ryd_to_eV = (4.3597447222071e-18 / q_e) / 2.0;
    constexpr double ang_to_m  = 1e-10;
    int              idx       = 0;
    for (const YNode& m : list->seq) {
        uepm_material mat;
        std::memset(&mat, 0, sizeof(mat));
        const YNode* sym = m.get("symbol");
        const YNode* pp  = m.get("pseudo-potential-parameters");
        if (!sym || !pp || !as_double(m.get("lattice-constant"), &mat.lattice_constant)) {
            uepm::set_error("material entry lacks symbol, lattice-constant or pseudo-potential-parameters");
            return UEPM_ERR_RUNTIME;
        }
        const char* must[] = {"V3S", "V8S", "V11S", "V3A", "V4A", "V11A"};
        double*     dst[]  = {&mat.V3S, &mat.V8S, &mat.V11S, &mat.V3A, &mat.V4A, &mat.V11A};
        for (int q = 0; q < 6; ++q) {
            double v;
            if (!as_double(pp->get(must[q]), &v)) {
                uepm::set_error(std::string("missing form factor ") + must[q] + " for " + sym->value);
                return UEPM_ERR_RUNTIME;
            }
            *dst[q] = Ryd_to_eV * v;
        }
        double v;
        if (as_double(pp->get("V4S"), &v)) mat.V4S = Ryd_to_eV * v;
        if (as_double(pp->get("V8A"), &v)) mat.V8A = Ryd_to_eV * v;
        if (const YNode* nl = m.get("non-local-parameters")) {
            struct F {
                const char* key;
                double*     dst;
                double      scale;
            } fs[] = {{"alpha_0_cation", &mat.alpha0_cation, Ryd_to_eV}, {"alpha_0_anion", &mat.alpha0_anion, Ryd_to_eV},
                      {"beta_0_cation", &mat.beta0_cation, 1.0},         {"beta_0_anion", &mat.beta0_anion, 1.0},
                      {"A2_cation", &mat.A2_cation, Ryd_to_eV},          {"A2_anion", &mat.A2_anion, Ryd_to_eV},
                      {"R0_cation", &mat.R0_cation, 0.0},                {"R2_cation", &mat.R2_cation, 0.0},
                      {"R0_anion", &mat.R0_anion, 0.0},                  {"R2_anion", &mat.R2_anion, 0.0}};
            for (const F& f : fs) {
                if (!as_double(nl->get(f.key), &v)) {
                    uepm::set_error(std::string("missing non-local parameter ") + f.key);
                    return UEPM_ERR_RUNTIME;
                }
                // radii: Angstrom -> m after reading (NonLocalParameters.hpp:112-115)
                *f.dst = (f.scale == 0.0) ? v * ang_to_m : f.scale * v;
            }
            const YNode* wt = nl->get("well_type");
            if (wt && wt->value == "square") mat.nl_well = 1;
            else if (wt && wt->value == "gaussian") mat.nl_well = 2;
            else {
                uepm::set_error("Unknown non-local well type");
                return UEPM_ERR_RUNTIME;
            }
            mat.has_nonlocal = 1;
        }
        if (const YNode* so = m.get("spin-orbit-parameters")) {
            double pa, pc;
            if (!as_double(so->get("period_anion"), &pa) || !as_double(so->get("period_cation"), &pc) ||
                !as_double(so->get("radial_extent_anion"), &mat.radial_extent_anion) ||
                !as_double(so->get("radial_extent_cation"), &mat.radial_extent_cation) ||
                !as_double(so->get("alpha_soc"), &mat.alpha_soc) || !as_double(so->get("mu_soc"), &mat.mu_soc)) {
                uepm::set_error("incomplete spin-orbit-parameters");
                return UEPM_ERR_RUNTIME;
            }
            mat.period_anion  = (uint32_t)pa;
            mat.period_cation = (uint32_t)pc;
            mat.has_soc       = 1;
        }
        if (idx < capacity) {
            if (out) out[idx] = mat;
            if (symbols && symbol_stride > 0) {
                std::strncpy(symbols + (size_t)idx * symbol_stride, sym->value.c_str(), (size_t)symbol_stride - 1);
                symbols[(size_t)idx * symbol_stride + symbol_stride - 1] = '\0';
            }
        }
        ++idx;
    }
    return idx;
}

int uepm_adjust_values(double* E, size_t nk, int nb, int soc, int min_cond_zero, double* gap, int* found) {
    // FindBandGap (BandStructure.cpp:230-262): scan band pairs (l, l+1) from l = 2 for a gap above
    // 0.35 eV; without one, fall back to the band-3 maximum.
    double vbm = 0.0, cbm = 0.0;
    bool   ok  = false;
    if (nk > 0 && nb >= 2) {
        double fallback = std::numeric_limits<double>::lowest();
        for (int l = 2; l + 1 < nb; ++l) {
            vbm = std::numeric_limits<double>::lowest();
            cbm = std::numeric_limits<double>::infinity();
            for (size_t q = 0; q < nk; ++q) {
                vbm = std::max(vbm, E[q * nb + l]);
                cbm = std::min(cbm, E[q * nb + l + 1]);
            }
            if (l == 3) fallback = vbm;
            if (vbm + 0.35 < cbm) {
                ok = true;
                break;
            }
        }
        if (!ok) {
            if (nb <= 3) cbm = std::numeric_limits<double>::infinity();
            vbm = fallback;
        }
    }
    const int nval = soc ? 8 : 4;
    for (size_t q = 0; q < nk; ++q)
        for (int b = 0; b < nb; ++b) {
            if (b < nval) E[q * nb + b] -= vbm;
            else if (min_cond_zero) E[q * nb + b] -= cbm;
            else E[q * nb + b] -= vbm;
        }
    if (gap) *gap = ok ? cbm - vbm : 0.0;
    if (found) *found = ok ? 1 : 0;
    return UEPM_OK;
}

// The signed permutation that maps each k_src[q] onto k_dst[q] (component by component of k_dst: the
// first unused component of k_src whose magnitude matches within 1e-8 * max(1, largest magnitude),
// the sign from the two components' signs, or from k_dst's where the component vanishes), the rule
// of apply_same_symmetry_operation (src/BZ_MESH/bz_mesh.cpp:1312-1381), packed for
// uepm_star_expand_device. found[q] = 0 where no signed permutation matches (identity written; the
// reference leaves the vector unchanged there).
int uepm_star_operations(const double* k_src, const double* k_dst, size_t n, uint16_t* op, int32_t* found) {
    if (n && (!k_src || !k_dst || !op)) return UEPM_ERR_INVALID;
    for (size_t q = 0; q < n; ++q) {
        const double* a = k_src + 3 * q;
        const double* b = k_dst + 3 * q;
        double        scale = 1.0;
        for (int c = 0; c < 3; ++c) scale = std::max(scale, std::max(std::fabs(a[c]), std::fabs(b[c])));
        const double tol = 1e-8 * scale;
        bool         used[3] = {false, false, false}, ok = true;
        unsigned     packed  = 0;
        for (int j = 0; j < 3 && ok; ++j) {
            int p = -1;
            for (int i = 0; i < 3; ++i)
                if (!used[i] && std::fabs(std::fabs(a[i]) - std::fabs(b[j])) <= tol) {
                    p = i;
                    break;
                }
            if (p < 0) {
                ok = false;
                break;
            }
            used[p]        = true;
            const bool neg = std::fabs(a[p]) > tol ? ((a[p] >= 0.0) != (b[j] >= 0.0)) : (b[j] < 0.0);
            packed |= (unsigned)p << (2 * j);
            if (neg) packed |= 1u << (6 + j);
        }
        op[q] = ok ? (uint16_t)packed : (uint16_t)(0 | 1 << 2 | 2 << 4);
        if (found) found[q] = ok ? 1 : 0;
    }
    return UEPM_OK;
}

}  // extern "C"
