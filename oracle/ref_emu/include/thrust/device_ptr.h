#pragma once
namespace thrust {
template <class T>
struct device_ptr {
    T* p;
    T* get() const { return p; }
};
}  // namespace thrust
