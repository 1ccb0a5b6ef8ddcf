// Minimal stand-in for the fmt library (test infrastructure): fmt::print with "{}" placeholders only,
// enough to compile the reference's apps against the adapter headers.
#pragma once
#include <iostream>
#include <sstream>
#include <string>
namespace fmt {
inline void format_into(std::ostringstream& os, const char* f) { os << f; }
template <typename T, typename... Rest>
void format_into(std::ostringstream& os, const char* f, const T& v, const Rest&... rest) {
    for (; *f; ++f) {
        if (f[0] == '{' && f[1] == '}') {
            os << v;
            format_into(os, f + 2, rest...);
            return;
        }
        os << *f;
    }
}
template <typename... Args>
void print(const char* f, const Args&... args) {
    std::ostringstream os;
    format_into(os, f, args...);
    std::cout << os.str();
}
}  // namespace fmt
