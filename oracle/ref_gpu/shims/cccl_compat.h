// Pre-included into the reference's CUDA sources for the baseline build.  The reference orders
// Vec2i and Vec3f for thrust::sort / thrust::sort_by_key with operator< overloads declared in
// namespace thrust (include/af/eigen_extension.cuh:6-27), which older thrust's default comparator
// found by unqualified lookup.  In CUDA 13's CCCL the default comparator is cuda::std::less, whose
// lookup no longer reaches namespace thrust, so the two comparators are named here, forwarding to
// the reference's own operators (declared here, defined by the reference's header).  The default
// equality of thrust::unique / reduce_by_key is named likewise (below).
#pragma once
#ifndef WIN64
#define EIGEN_DONT_ALIGN_STATICALLY
#endif
#include <Eigen/Dense>
#include <cuda/std/functional>

namespace thrust {
__host__ __device__ inline bool operator<(const Eigen::Vector2i& a, const Eigen::Vector2i& b);
__host__ __device__ inline bool operator<(const Eigen::Vector3f& a, const Eigen::Vector3f& b);
}  // namespace thrust

template <>
struct cuda::std::less<Eigen::Vector2i> {
    __host__ __device__ bool operator()(const Eigen::Vector2i& a, const Eigen::Vector2i& b) const {
        return thrust::operator<(a, b);
    }
};

template <>
struct cuda::std::less<Eigen::Vector3f> {
    __host__ __device__ bool operator()(const Eigen::Vector3f& a, const Eigen::Vector3f& b) const {
        return thrust::operator<(a, b);
    }
};

// The same lookup change breaks the default equality of thrust::unique and thrust::reduce_by_key
// on these types (with CUDA 13, unique on Eigen::Vector3f keys returns an empty range); name it
// too, component by component as Eigen's operator== compares.
template <>
struct cuda::std::equal_to<Eigen::Vector2i> {
    __host__ __device__ bool operator()(const Eigen::Vector2i& a, const Eigen::Vector2i& b) const {
        return a[0] == b[0] && a[1] == b[1];
    }
};

template <>
struct cuda::std::equal_to<Eigen::Vector3f> {
    __host__ __device__ bool operator()(const Eigen::Vector3f& a, const Eigen::Vector3f& b) const {
        return a[0] == b[0] && a[1] == b[1] && a[2] == b[2];
    }
};
