// yaml-cpp/yaml.h -- CHECKER ONLY (test infrastructure; never part of the product path).
//
// The reference's material loader (src/EPP/Material.cpp:33-71, NonLocalParameters.hpp:91-116,
// SpinOrbitParameters.hpp:74-81) reads its parameter files through yaml-cpp, which its CMake fetches
// at configure time (CMakeLists.txt:86-92) and which is absent here. This header supplies, written
// for this project, the part of yaml-cpp's API those files use, so that they compile unchanged into
// oracle/_ref/libref.so: YAML::LoadFile, YAML::Node with operator[] (a missing key gives an
// undefined node, false in a condition, as in yaml-cpp), iteration over a sequence, and
// as<std::string / double / unsigned int / int>(), converting the scalar text with a
// std::istringstream as yaml-cpp's conversions do.
//
// The parser covers the block-style subset the reference's parameter files are written in:
// nested mappings by indentation, sequences of "- " entries (each a mapping or a scalar), plain and
// quoted scalars, comments, and the "---" / "..." document markers.
#pragma once

#include <fstream>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace YAML {

struct NodeData {
    enum Kind { Null, Scalar, Map, Seq } kind = Null;
    std::string                                                   scalar;
    std::vector<std::pair<std::string, std::shared_ptr<NodeData>>> map;
    std::vector<std::shared_ptr<NodeData>>                        seq;
};

class Node {
 public:
    Node() = default;
    explicit Node(std::shared_ptr<NodeData> d) : d_(std::move(d)) {}

    explicit operator bool() const { return d_ != nullptr; }
    bool IsDefined() const { return d_ != nullptr; }
    bool IsMap() const { return d_ && d_->kind == NodeData::Map; }
    bool IsSequence() const { return d_ && d_->kind == NodeData::Seq; }
    bool IsScalar() const { return d_ && d_->kind == NodeData::Scalar; }

    Node operator[](const std::string& key) const {
        if (d_ && d_->kind == NodeData::Map)
            for (const auto& kv : d_->map)
                if (kv.first == key) return Node(kv.second);
        return Node();
    }
    Node operator[](const char* key) const { return (*this)[std::string(key)]; }

    template <typename T>
    T as() const {
        if (!d_ || d_->kind != NodeData::Scalar) throw std::runtime_error("YAML shim: bad conversion (not a scalar)");
        if constexpr (std::is_same_v<T, std::string>) {
            return d_->scalar;
        } else {
            std::istringstream in(d_->scalar);
            T                  v{};
            in >> v;
            if (in.fail()) throw std::runtime_error("YAML shim: bad conversion of '" + d_->scalar + "'");
            return v;
        }
    }

    class const_iterator {
     public:
        const_iterator(const std::vector<std::shared_ptr<NodeData>>* s, size_t i) : s_(s), i_(i) {}
        Node            operator*() const { return Node((*s_)[i_]); }
        const_iterator& operator++() {
            ++i_;
            return *this;
        }
        bool operator!=(const const_iterator& o) const { return i_ != o.i_; }

     private:
        const std::vector<std::shared_ptr<NodeData>>* s_;
        size_t                                        i_;
    };
    const_iterator begin() const { return const_iterator(seq(), 0); }
    const_iterator end() const { return const_iterator(seq(), seq() ? seq()->size() : 0); }

 private:
    const std::vector<std::shared_ptr<NodeData>>* seq() const {
        return (d_ && d_->kind == NodeData::Seq) ? &d_->seq : nullptr;
    }
    std::shared_ptr<NodeData> d_;
};

namespace shim_detail {

struct Line {
    int         indent;
    std::string text;
};

inline std::string trim(const std::string& s) {
    size_t a = s.find_first_not_of(" \t\r");
    if (a == std::string::npos) return "";
    size_t b = s.find_last_not_of(" \t\r");
    return s.substr(a, b - a + 1);
}

// Drops a comment: '#' at the start of the text or after a blank, outside quotes.
inline std::string strip_comment(const std::string& s) {
    char quote = 0;
    for (size_t i = 0; i < s.size(); ++i) {
        const char c = s[i];
        if (quote) {
            if (c == quote) quote = 0;
        } else if (c == '"' || c == '\'') {
            quote = c;
        } else if (c == '#' && (i == 0 || s[i - 1] == ' ' || s[i - 1] == '\t')) {
            return s.substr(0, i);
        }
    }
    return s;
}

inline std::shared_ptr<NodeData> scalar(const std::string& raw) {
    auto        d = std::make_shared<NodeData>();
    std::string t = trim(raw);
    if (t.size() >= 2 && (t.front() == '"' || t.front() == '\'') && t.back() == t.front()) t = t.substr(1, t.size() - 2);
    d->kind   = NodeData::Scalar;
    d->scalar = t;
    return d;
}

inline bool is_item(const std::string& t) { return t == "-" || (t.size() >= 2 && t[0] == '-' && t[1] == ' '); }

inline std::shared_ptr<NodeData> parse_block(std::vector<Line>& L, size_t& i, int indent);

inline std::shared_ptr<NodeData> parse_seq(std::vector<Line>& L, size_t& i, int indent) {
    auto d  = std::make_shared<NodeData>();
    d->kind = NodeData::Seq;
    while (i < L.size() && L[i].indent == indent && is_item(L[i].text)) {
        const std::string rest = L[i].text.size() > 1 ? L[i].text.substr(2) : "";
        const size_t      lead = rest.find_first_not_of(' ');
        if (lead == std::string::npos) {  // "-" alone: the entry is the block below
            ++i;
            d->seq.push_back(i < L.size() && L[i].indent > indent ? parse_block(L, i, L[i].indent)
                                                                  : std::make_shared<NodeData>());
            continue;
        }
        // The entry's content starts a block at the column after "- ".
        L[i].indent = indent + 2 + (int)lead;
        L[i].text   = rest.substr(lead);
        if (L[i].text.find(": ") == std::string::npos && L[i].text.back() != ':' && !is_item(L[i].text)) {
            d->seq.push_back(scalar(L[i].text));
            ++i;
        } else {
            d->seq.push_back(parse_block(L, i, L[i].indent));
        }
    }
    return d;
}

inline std::shared_ptr<NodeData> parse_map(std::vector<Line>& L, size_t& i, int indent) {
    auto d  = std::make_shared<NodeData>();
    d->kind = NodeData::Map;
    while (i < L.size() && L[i].indent == indent && !is_item(L[i].text)) {
        const std::string& t     = L[i].text;
        size_t             colon = t.find(": ");
        if (colon == std::string::npos && !t.empty() && t.back() == ':') colon = t.size() - 1;
        if (colon == std::string::npos) throw std::runtime_error("YAML shim: expected 'key: value' in '" + t + "'");
        const std::string key  = trim(t.substr(0, colon));
        const std::string rest = trim(t.substr(colon + 1));
        ++i;
        if (!rest.empty()) {
            d->map.emplace_back(key, scalar(rest));
        } else if (i < L.size() && (L[i].indent > indent || (L[i].indent == indent && is_item(L[i].text)))) {
            d->map.emplace_back(key, parse_block(L, i, L[i].indent));
        } else {
            d->map.emplace_back(key, std::make_shared<NodeData>());
        }
    }
    return d;
}

inline std::shared_ptr<NodeData> parse_block(std::vector<Line>& L, size_t& i, int indent) {
    return is_item(L[i].text) ? parse_seq(L, i, indent) : parse_map(L, i, indent);
}

}  // namespace shim_detail

inline Node Load(std::istream& in) {
    std::vector<shim_detail::Line> L;
    std::string                    raw;
    while (std::getline(in, raw)) {
        const std::string s = shim_detail::strip_comment(raw);
        const std::string t = shim_detail::trim(s);
        if (t.empty() || t == "---" || t == "...") continue;
        L.push_back({(int)s.find_first_not_of(' '), t});
    }
    if (L.empty()) return Node(std::make_shared<NodeData>());
    size_t i = 0;
    return Node(shim_detail::parse_block(L, i, L[0].indent));
}

inline Node LoadFile(const std::string& filename) {
    std::ifstream in(filename);
    if (!in) throw std::runtime_error("YAML shim: bad file: " + filename);
    return Load(in);
}

}  // namespace YAML
