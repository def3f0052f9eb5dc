// Minimal stand-in for boost::hash_range, enough to compile the reference's
// std::hash<Vec3f> specialisation (include/af/eigen_extension.h).  Test build only.
#pragma once
#include <cstddef>
#include <functional>
namespace boost {
template <class It>
std::size_t hash_range(It first, It last) {
    std::size_t seed = 0;
    for (; first != last; ++first)
        seed ^= std::hash<typename std::decay<decltype(*first)>::type>()(*first) + 0x9e3779b9 + (seed << 6) + (seed >> 2);
    return seed;
}
}  // namespace boost
