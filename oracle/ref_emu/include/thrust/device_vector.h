// Minimal stand-in for thrust::device_vector on host memory (test build only).
#pragma once
#include <vector>
#include "device_ptr.h"
namespace thrust {
template <class T>
struct device_vector : std::vector<T> {
    using std::vector<T>::vector;
    device_ptr<T> data() { return device_ptr<T>{std::vector<T>::data()}; }
    device_ptr<const T> data() const { return device_ptr<const T>{std::vector<T>::data()}; }
};
}  // namespace thrust
