// Test-only stand-in for boost::lexical_cast as the reference's readers use it (string to number or string,
// number to string): the whole source must convert, else bad_lexical_cast is thrown, as Boost documents.
#pragma once
#include <sstream>
#include <stdexcept>
#include <string>
#include <type_traits>

namespace boost {
struct bad_lexical_cast : std::bad_cast {
    const char *what() const noexcept override { return "bad lexical cast"; }
};

template <class T, class S>
T lexical_cast(const S &src) {
    std::stringstream ss;
    ss.precision(17);
    ss << src;
    if constexpr (std::is_same<T, std::string>::value) {
        return ss.str();
    } else {
        T out{};
        ss >> out;
        if (ss.fail() || ss.peek() != std::char_traits<char>::eof()) throw bad_lexical_cast();
        return out;
    }
}
}  // namespace boost
