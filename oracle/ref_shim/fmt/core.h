// Minimal stand-in for fmt::format, as used by libBICOS's CPU backend for
// one error message.  TEST INFRASTRUCTURE ONLY (oracle/_ref checker build).
// Replaces each "{}" in order with the streamed argument.
#pragma once

#include <sstream>
#include <string>

namespace fmt {

namespace detail {
inline void format_into(std::ostringstream& os, const char* s) { os << s; }

template<typename A, typename... Rest>
void format_into(std::ostringstream& os, const char* s, const A& a, const Rest&... rest) {
    for (; *s; ++s) {
        if (s[0] == '{' && s[1] == '}') {
            os << a;
            format_into(os, s + 2, rest...);
            return;
        }
        os << *s;
    }
}
} // namespace detail

template<typename... Args>
std::string format(const char* s, const Args&... args) {
    std::ostringstream os;
    detail::format_into(os, s, args...);
    return os.str();
}

} // namespace fmt
