/*
 * af/afx_containers.h -- the reference's af:: device containers over the C ABI (header-only C++17).
 *
 *   DeviceBuffer, DeviceBufferCounted     include/af/DeviceBuffer.cuh:36-115
 *   DeviceImage, DeviceDepthImage         include/af/DeviceImage.cuh:12-68
 *   CameraIntrinsics, CameraDistortion, CameraModel   include/af/CameraModel.h:14-44
 *   DeviceKnn, DeviceKnnWeighted          include/af/DataTypes.cuh:9-62
 *   DeviceMotionGraph                     include/af/DeviceMotionGraph.cuh:10-33
 *   Settings                              include/af/Settings.h:9-47, defaults src/Settings.cpp:8-41
 *
 * They hold raw device arrays where the reference holds thrust vectors; data() returns a handle
 * with get(), so `buf.data().get()` call sites stay, and begin()/end() are device pointers.
 * The objects that compute (DeviceTsdf, MotionGraph, WarpField, TSDFVolume, ...) are in
 * af/afx_classes.h.
 */
#ifndef AF_AFX_CONTAINERS_H
#define AF_AFX_CONTAINERS_H

#include <algorithm>
#include <cmath>
#include <limits>
#include <string>
#include <utility>
#include <vector>

#include "afx_shims.h"

namespace af {

template <class T>
inline void copyToDevice(T* data_d, const T* data, const std::size_t cSize) {
    if (cSize) detail::cuda_check(cudaMemcpy(data_d, data, cSize * sizeof(T), cudaMemcpyHostToDevice), "copyToDevice");
}
template <class T>
inline void copyToHost(T* data, const T* data_d, const std::size_t cSize) {
    if (cSize) detail::cuda_check(cudaMemcpy(data, data_d, cSize * sizeof(T), cudaMemcpyDeviceToHost), "copyToHost");
}

// A device pointer with thrust::device_ptr's get().
template <class T>
struct device_ptr {
    T* p;
    T* get() const { return p; }
    operator T*() const { return p; }
};

// Owned device array of n elements (no construction: the element types are trivially copyable).
template <class T>
class DeviceArray {
public:
    DeviceArray() = default;
    explicit DeviceArray(std::size_t n) { allocate(n); }
    DeviceArray(const DeviceArray& o) { *this = o; }
    DeviceArray& operator=(const DeviceArray& o) {
        if (this != &o) {
            allocate(o.n_);
            if (n_)
                detail::cuda_check(cudaMemcpy(p_, o.p_, n_ * sizeof(T), cudaMemcpyDeviceToDevice), "DeviceArray copy");
        }
        return *this;
    }
    DeviceArray(DeviceArray&& o) noexcept : p_(o.p_), n_(o.n_) {
        o.p_ = nullptr;
        o.n_ = 0;
    }
    DeviceArray& operator=(DeviceArray&& o) noexcept {
        std::swap(p_, o.p_);
        std::swap(n_, o.n_);
        return *this;
    }
    ~DeviceArray() { cudaFree(p_); }

    // Keeps the first min(n, size) elements; new elements are set to x.
    void resize(std::size_t n, const T& x = T()) {
        if (n == n_) return;
        T* q = nullptr;
        if (n) detail::cuda_check(cudaMalloc(reinterpret_cast<void**>(&q), n * sizeof(T)), "cudaMalloc");
        const std::size_t keep = std::min(n, n_);
        if (keep) detail::cuda_check(cudaMemcpy(q, p_, keep * sizeof(T), cudaMemcpyDeviceToDevice), "resize copy");
        if (n > keep) {
            std::vector<T> tail(n - keep, x);
            copyToDevice(q + keep, tail.data(), tail.size());
        }
        cudaFree(p_);
        p_ = q;
        n_ = n;
    }
    T* get() { return p_; }
    const T* get() const { return p_; }
    std::size_t size() const { return n_; }

private:
    void allocate(std::size_t n) {
        if (n == n_) return;
        cudaFree(p_);
        p_ = nullptr;
        n_ = 0;
        if (n) detail::cuda_check(cudaMalloc(reinterpret_cast<void**>(&p_), n * sizeof(T)), "cudaMalloc");
        n_ = n;
    }
    T* p_ = nullptr;
    std::size_t n_ = 0;
};

// ---- include/af/DeviceBuffer.cuh ----
template <class Type>
class DeviceBuffer {
public:
    using value_type = Type;
    using pointer = device_ptr<Type>;
    using const_pointer = device_ptr<const Type>;
    using iterator = Type*;
    using const_iterator = const Type*;
    using size_type = std::size_t;

    DeviceBuffer(unsigned int bufferSize, unsigned int size = 0) : _buffer(bufferSize), _size(size) {
        if (size > bufferSize) throw std::runtime_error("af::DeviceBuffer: size > bufferSize");
    }
    virtual ~DeviceBuffer() = default;

    iterator begin() { return _buffer.get(); }
    const_iterator begin() const { return _buffer.get(); }
    iterator end() { return _buffer.get() + _size; }
    const_iterator end() const { return _buffer.get() + _size; }

    size_type bufferSize() const { return _buffer.size(); }
    void resizeBuffer(size_type new_size, const value_type& x = value_type()) {
        _buffer.resize(new_size, x);
        if (_size > new_size) _size = (unsigned int)new_size;
    }

    Type* bufferPtr() { return _buffer.get(); }
    const Type* bufferPtr() const { return _buffer.get(); }
    pointer data() { return {_buffer.get()}; }
    const_pointer data() const { return {_buffer.get()}; }

    virtual void setSize(unsigned int size) {
        if (size > _buffer.size())
            throw std::runtime_error("af::DeviceBuffer::setSize(): size > bufferSize (" + std::to_string(size) +
                                     " > " + std::to_string(_buffer.size()) + ").");
        _size = size;
    }
    void resetSize() { setSize(0); }
    unsigned int size() const { return _size; }

    // Host transfers (the reference's callers use copyToDevice / thrust::copy for these).
    void upload(const std::vector<Type>& v) {
        if (v.size() > bufferSize()) resizeBuffer(v.size());
        copyToDevice(bufferPtr(), v.data(), v.size());
        setSize((unsigned int)v.size());
    }
    std::vector<Type> download() const {
        std::vector<Type> v(_size);
        copyToHost(v.data(), bufferPtr(), v.size());
        return v;
    }

private:
    DeviceArray<Type> _buffer;
    unsigned int _size;
};

template <class Type>
class DeviceBufferCounted : public DeviceBuffer<Type> {
public:
    DeviceBufferCounted(unsigned int bufferSize, unsigned int size = 0) : DeviceBuffer<Type>(bufferSize, size), _size_d(1) {
        copyToDevice(_size_d.get(), &size, 1);
    }

    void syncHostSize() {
        unsigned int n = 0;
        copyToHost(&n, _size_d.get(), 1);
        DeviceBuffer<Type>::setSize(n);
    }
    void setSize(unsigned int size) override {
        DeviceBuffer<Type>::setSize(size);
        copyToDevice(_size_d.get(), &size, 1);
    }

    unsigned int* size_dPtr() { return _size_d.get(); }
    const unsigned int* size_dPtr() const { return _size_d.get(); }

private:
    DeviceArray<unsigned int> _size_d;
};

// ---- include/af/CameraModel.h:14-44 ----
struct CameraIntrinsics {
    float cx{0.f};
    float cy{0.f};
    float fx{0.f};
    float fy{0.f};
};

struct CameraDistortion {
    float k1{0.f};
    float k2{0.f};
    float k3{0.f};
    float k4{0.f};
    float k5{0.f};
    float k6{0.f};
    float codx{0.f};
    float cody{0.f};
    float p1{0.f};
    float p2{0.f};
    bool is_distorted{false};
};

struct CameraModel {
    unsigned int width{0};
    unsigned int height{0};
    CameraIntrinsics intrinsics;
    CameraDistortion distortion;
    Mat3f depthIntrinsics = Mat3f::Identity();
    Mat4f transfW2C = Mat4f::Identity();
};

// ---- include/af/DeviceImage.cuh ----
template <class Type>
class DeviceImage {
public:
    using iterator = Type*;
    using const_iterator = const Type*;

    DeviceImage() = default;
    DeviceImage(std::size_t height, std::size_t width) : _image_d(height * width), _height(height), _width(width) {}
    virtual ~DeviceImage() = default;

    // Values above upperBound (and below 1e-4, and NaN) become +inf (runFilterDepthKernel).
    void nullifyUpperBound(Type upperBound) { af::runFilterDepthKernel(dataPtr(), (unsigned int)size(), upperBound); }

    Type* dataPtr() { return _image_d.get(); }
    const Type* dataPtr() const { return _image_d.get(); }

    void resize(std::size_t height, std::size_t width) {
        _height = height;
        _width = width;
        _image_d.resize(_height * _width);
    }
    iterator begin() { return _image_d.get(); }
    const_iterator begin() const { return _image_d.get(); }
    std::size_t height() const { return _height; }
    std::size_t width() const { return _width; }
    std::size_t size() const { return _height * _width; }

    void upload(const Type* host) { copyToDevice(dataPtr(), host, size()); }
    void download(Type* host) const { copyToHost(host, dataPtr(), size()); }

private:
    DeviceArray<Type> _image_d;
    std::size_t _height = 0;
    std::size_t _width = 0;
};

class DeviceDepthImage : public DeviceImage<float> {
public:
    explicit DeviceDepthImage(const CameraModel& camera) : _camera(camera) {}
    DeviceDepthImage(std::size_t height, std::size_t width, const CameraModel& camera)
        : DeviceImage<float>(height, width), _camera(camera) {}

    const CameraModel& camera() const { return _camera; }
    const Mat3f& depthIntrinsics() const { return _camera.depthIntrinsics; }

private:
    const CameraModel& _camera;
};

// ---- include/af/DataTypes.cuh ----
template <int K>
class DeviceKnn {
public:
    explicit DeviceKnn(std::size_t bufferSize) : _bufferSize(bufferSize), _size(0), _idxs_d(bufferSize), _dists_d(bufferSize) {}
    virtual ~DeviceKnn() = default;

    Vecui<K>* idxsPtr() { return _idxs_d.get(); }
    Vecf<K>* distsPtr() { return _dists_d.get(); }
    const Vecui<K>* idxsPtr() const { return _idxs_d.get(); }
    const Vecf<K>* distsPtr() const { return _dists_d.get(); }

    void setSize(std::size_t size) {
        if (size > _bufferSize) throw std::runtime_error("af::DeviceKnn::setSize(): size > bufferSize.");
        _size = size;
    }
    std::size_t size() const { return _size; }
    virtual void resizeBuffer(std::size_t bufferSize) {
        _bufferSize = bufferSize;
        _idxs_d.resize(_bufferSize);
        _dists_d.resize(_bufferSize);
        if (_size > _bufferSize) _size = _bufferSize;
    }
    std::size_t bufferSize() const { return _bufferSize; }

private:
    std::size_t _bufferSize;
    std::size_t _size;
    DeviceArray<Vecui<K>> _idxs_d;
    DeviceArray<Vecf<K>> _dists_d;
};

template <int K>
class DeviceKnnWeighted : public DeviceKnn<K> {
public:
    explicit DeviceKnnWeighted(std::size_t bufferSize) : DeviceKnn<K>(bufferSize), _weights_d(bufferSize) {}
    void resizeBuffer(std::size_t bufferSize) override {
        DeviceKnn<K>::resizeBuffer(bufferSize);
        _weights_d.resize(bufferSize);
    }
    Vecf<K>* weightsPtr() { return _weights_d.get(); }
    const Vecf<K>* weightsPtr() const { return _weights_d.get(); }

private:
    DeviceArray<Vecf<K>> _weights_d;
};

// ---- include/af/DeviceMotionGraph.cuh ----
class DeviceMotionGraph {
public:
    explicit DeviceMotionGraph(std::size_t size)
        : _points_d(size), _transforms_d(size), _radiuses_d(size), _count_d(1), _size(size), _count(0) {
        setCount(0);
    }

    Vec3f* pointsPtr() { return _points_d.get(); }
    Mat4f* transformsPtr() { return _transforms_d.get(); }
    float* radiusesPtr() { return _radiuses_d.get(); }
    const Vec3f* pointsPtr() const { return _points_d.get(); }
    const Mat4f* transformsPtr() const { return _transforms_d.get(); }
    const float* radiusesPtr() const { return _radiuses_d.get(); }

    std::size_t bufferSize() const { return _size; }
    std::size_t count() const { return _count; }
    void setCount(std::size_t count) {
        if (count > _size) throw std::runtime_error("af::DeviceMotionGraph::setCount(): count > bufferSize.");
        _count = count;
        const int c = (int)count;
        copyToDevice(_count_d.get(), &c, 1);
    }
    // The node count as the afx_* calls read it (device int, kept equal to count()).
    int* countPtr() { return _count_d.get(); }
    const int* countPtr() const { return _count_d.get(); }
    // Re-reads count() after a device call appended nodes.
    void syncCount() {
        int c = 0;
        copyToHost(&c, _count_d.get(), 1);
        _count = (std::size_t)c;
    }

private:
    DeviceArray<Vec3f> _points_d;
    DeviceArray<Mat4f> _transforms_d;
    DeviceArray<float> _radiuses_d;
    DeviceArray<int> _count_d;
    std::size_t _size;
    std::size_t _count;
};

// ---- include/af/Settings.h, defaults of src/Settings.cpp:8-41 ----
struct Settings {
    Vec3f tsdfSize = Vec3f(1.0f, 1.0f, 1.0f);
    Vec3i tsdfDim = Vec3i(400, 400, 400);
    Vec3f tsdfCenter = Vec3f(0.0f, 0.0f, 0.0f);
    Vec3i tsdfRotation = Vec3i(45, -45, 0);
    std::pair<float, float> normExclAngleRange = {1.3f, 2.1f};
    std::pair<int, int> framesRange = {1, 1000};
    int frameBreak = -1;
    std::string dataFolder;
    uint32_t cameraCount = 1;
    std::string depthFilesPattern;
    float depthThreshold = 1.0f;
    bool integrateTsdf = true;
    bool bilateralFiltr = true;
    bool updateGraph = true;
    bool useCopyHack = true;
    bool useCholesky = true;
    int bilateralD = 5;
    float bilateralSigmaI = 75;
    float bilateralSigmaS = 75;
    float bilateralThreshold = 0.025f;
    float energyWeightDepth = 1.f;
    float energyWeightMReg = 2.2f;
    float energyMinStep = 0.0001f;
    int icpIterations = 3;
    float motionGraphRadius = 0.05f;
    float motionGraphSampleDistance = 0.03f;
    float tsdfDelta = 0.01f;
    float correspThreshDist = 0.01f;
    bool isMeshWarped = false;
};

}  // namespace af

#endif
