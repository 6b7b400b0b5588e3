// Test-only stand-in for the few Boost string algorithms the reference's sources call (boost::split with
// is_any_of / is_space and token_compress_on, trim, iequals, erase_first_copy, erase_last_copy), so that the
// reference's Blob.cpp and its script readers compile without Boost for the oracle's reference build. The
// semantics follow Boost's documentation: split cuts at every separator character, giving empty tokens between
// adjacent separators unless they are compressed (an empty input gives one empty token); trim removes leading
// and trailing white space; the erase_*_copy functions remove the first / last occurrence of a substring.
#pragma once
#include <algorithm>
#include <cctype>
#include <string>

namespace boost {
namespace algorithm {
enum token_compress_mode_type { token_compress_on, token_compress_off };

struct is_any_of_pred {
    std::string set;
    bool operator()(char c) const { return set.find(c) != std::string::npos; }
};
struct is_space_pred {
    bool operator()(char c) const { return std::isspace((unsigned char)c) != 0; }
};
inline is_any_of_pred is_any_of(const std::string &s) { return is_any_of_pred{s}; }
inline is_space_pred is_space() { return is_space_pred{}; }

template <class Seq, class Pred>
Seq &split(Seq &out, const std::string &in, Pred pred, token_compress_mode_type mode = token_compress_off) {
    out.clear();
    std::string cur;
    size_t i = 0;
    while (i <= in.size()) {
        if (i == in.size()) {
            out.push_back(cur);
            break;
        }
        if (pred(in[i])) {
            out.push_back(cur);
            cur.clear();
            ++i;
            if (mode == token_compress_on)
                while (i < in.size() && pred(in[i])) ++i;
            continue;
        }
        cur += in[i++];
    }
    return out;
}

inline void trim(std::string &s) {
    size_t b = 0, e = s.size();
    while (b < e && std::isspace((unsigned char)s[b])) ++b;
    while (e > b && std::isspace((unsigned char)s[e - 1])) --e;
    s = s.substr(b, e - b);
}

inline bool iequals(const std::string &a, const std::string &b) {
    if (a.size() != b.size()) return false;
    for (size_t i = 0; i < a.size(); ++i)
        if (std::tolower((unsigned char)a[i]) != std::tolower((unsigned char)b[i])) return false;
    return true;
}

inline std::string erase_first_copy(const std::string &s, const std::string &sub) {
    const size_t p = s.find(sub);
    if (p == std::string::npos || sub.empty()) return s;
    return s.substr(0, p) + s.substr(p + sub.size());
}

inline std::string erase_last_copy(const std::string &s, const std::string &sub) {
    const size_t p = s.rfind(sub);
    if (p == std::string::npos || sub.empty()) return s;
    return s.substr(0, p) + s.substr(p + sub.size());
}
}  // namespace algorithm
using algorithm::erase_first_copy;
using algorithm::erase_last_copy;
using algorithm::iequals;
using algorithm::is_any_of;
using algorithm::is_space;
using algorithm::split;
using algorithm::token_compress_off;
using algorithm::token_compress_on;
using algorithm::trim;
}  // namespace boost
