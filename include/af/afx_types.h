/*
 * af/afx_types.h -- the small value types of the af:: C++ surface.
 *
 * The reference spells its arguments with Eigen aliases (include/af/eigen_extension.h:10-41:
 * Vec3f = Eigen::Vector3f, Mat4f = Eigen::Matrix4f, Vecui<K> = Eigen::Matrix<unsigned, K, 1>, ...).
 * When Eigen is included before this header the af:: names below are exactly those Eigen types,
 * so a caller's existing values and buffers pass straight through.  Without Eigen they are plain
 * structs with the same memory layout (packed vectors, column-major matrices) and the few members
 * the surface itself uses ([], (r, c), data(), Zero(), Identity()), so the headers need no Eigen.
 */
#ifndef AF_AFX_TYPES_H
#define AF_AFX_TYPES_H

#include <cstddef>
#include <cstdint>
#include <type_traits>

namespace af {

#ifdef EIGEN_WORLD_VERSION

using Vec2i = Eigen::Matrix<int, 2, 1>;
using Vec3i = Eigen::Matrix<int, 3, 1>;
using Vec2f = Eigen::Matrix<float, 2, 1>;
using Vec3f = Eigen::Matrix<float, 3, 1>;
using Vec4f = Eigen::Matrix<float, 4, 1>;
using Vec6f = Eigen::Matrix<float, 6, 1>;
using Vec3d = Eigen::Matrix<double, 3, 1>;
using Mat3f = Eigen::Matrix<float, 3, 3>;
using Mat4f = Eigen::Matrix<float, 4, 4>;
using Mat6f = Eigen::Matrix<float, 6, 6>;
template <int K>
using Vecf = Eigen::Matrix<float, K, 1>;
template <int K>
using Vecui = Eigen::Matrix<unsigned int, K, 1>;

#else

// N packed values of T.
template <class T, int N>
struct SmallVec {
    using value_type = T;
    using Scalar = T;
    T v[N];

    SmallVec() = default;
    template <class... A, class = typename std::enable_if<sizeof...(A) == N && (N > 1)>::type>
    SmallVec(A... a) : v{static_cast<T>(a)...} {}

    T& operator[](int i) { return v[i]; }
    const T& operator[](int i) const { return v[i]; }
    T& operator()(int i) { return v[i]; }
    const T& operator()(int i) const { return v[i]; }
    T* data() { return v; }
    const T* data() const { return v; }
    static constexpr int size() { return N; }
    void fill(T c) {
        for (int i = 0; i < N; ++i) v[i] = c;
    }
    static SmallVec Constant(T c) {
        SmallVec r;
        r.fill(c);
        return r;
    }
    static SmallVec Zero() { return Constant(T(0)); }
    bool operator==(const SmallVec& o) const {
        for (int i = 0; i < N; ++i)
            if (!(v[i] == o.v[i])) return false;
        return true;
    }
    bool operator!=(const SmallVec& o) const { return !(*this == o); }
};

// N x N values of T, column-major as Eigen stores them: (r, c) is data()[c * N + r].
template <class T, int N>
struct SmallMat {
    using value_type = T;
    using Scalar = T;
    T m[N * N];

    T& operator()(int r, int c) { return m[c * N + r]; }
    const T& operator()(int r, int c) const { return m[c * N + r]; }
    T* data() { return m; }
    const T* data() const { return m; }
    static constexpr int rows() { return N; }
    static constexpr int cols() { return N; }
    static SmallMat Zero() {
        SmallMat r;
        for (int i = 0; i < N * N; ++i) r.m[i] = T(0);
        return r;
    }
    static SmallMat Identity() {
        SmallMat r = Zero();
        for (int i = 0; i < N; ++i) r.m[i * N + i] = T(1);
        return r;
    }
};

using Vec2i = SmallVec<int, 2>;
using Vec3i = SmallVec<int, 3>;
using Vec2f = SmallVec<float, 2>;
using Vec3f = SmallVec<float, 3>;
using Vec4f = SmallVec<float, 4>;
using Vec6f = SmallVec<float, 6>;
using Vec3d = SmallVec<double, 3>;
using Mat3f = SmallMat<float, 3>;
using Mat4f = SmallMat<float, 4>;
using Mat6f = SmallMat<float, 6>;
template <int K>
using Vecf = SmallVec<float, K>;
template <int K>
using Vecui = SmallVec<unsigned int, K>;

static_assert(sizeof(Vec3f) == 12 && sizeof(Mat4f) == 64 && sizeof(Vecui<6>) == 24, "packed layout");
static_assert(std::is_trivially_copyable<Vec3f>::value && std::is_trivially_copyable<Mat4f>::value,
              "device buffers are copied bytewise");

#endif

// include/af/Constants.h:11-18: neighbours per point (skinning) and per node (regularisation).
struct Constants {
    static constexpr std::size_t motionGraphKNN = 6;
    static constexpr std::size_t energyMRegKNN = 4;
};

}  // namespace af

#endif
