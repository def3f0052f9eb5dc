// Minimal stand-in for boost::tuple (only named in an unused typedef by the reference).
#pragma once
#include <tuple>
namespace boost {
template <class... T>
using tuple = std::tuple<T...>;
}
