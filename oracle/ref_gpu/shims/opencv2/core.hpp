// Minimal stand-in for the parts of OpenCV that the reference's fusion loop (src/VolumeFusion.cu)
// touches when it is built as the GPU baseline: an owning cv::Mat of float or uint16 pixels
// (rows, cols, data, total(), clone(), at<T>()), cv::Scalar and the type constants.  Frames are
// handed to the loop by the baseline driver, not read from image files.  Test build only.
#pragma once
#include <cstddef>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <vector>

#define CV_8UC1 0
#define CV_16UC1 2
#define CV_32FC1 5
#define CV_8UC3 16
#define CV_32FC3 21

namespace cv {

struct Scalar {
    double v0 = 0.0;
    Scalar() = default;
    Scalar(double v) : v0(v) {}
};

inline std::size_t elem_size(int type) {
    switch (type) {
        case CV_8UC1: return 1;
        case CV_16UC1: return 2;
        case CV_32FC1: return 4;
        case CV_8UC3: return 3;
        case CV_32FC3: return 12;
    }
    throw std::runtime_error("cv::Mat stand-in: unsupported type");
}

struct Mat {
    unsigned char* data = nullptr;
    int rows = 0, cols = 0;
    int type_ = CV_32FC1;
    std::shared_ptr<std::vector<unsigned char>> store;

    Mat() = default;
    Mat(int r, int c, int type) : rows(r), cols(c), type_(type) {
        store = std::make_shared<std::vector<unsigned char>>((std::size_t)r * c * elem_size(type));
        data = store->data();
    }
    Mat(int r, int c, int type, const Scalar& s) : Mat(r, c, type) {
        if (type == CV_32FC1)
            for (std::size_t i = 0; i < total(); ++i) reinterpret_cast<float*>(data)[i] = (float)s.v0;
    }
    Mat(int r, int c, int type, void* d) : data(static_cast<unsigned char*>(d)), rows(r), cols(c), type_(type) {}
    std::size_t total() const { return (std::size_t)rows * cols; }
    bool empty() const { return data == nullptr || rows == 0 || cols == 0; }
    int type() const { return type_; }
    Mat clone() const {
        Mat m(rows, cols, type_);
        if (!empty()) std::memcpy(m.data, data, total() * elem_size(type_));
        return m;
    }
    template <class T>
    T& at(int i) {
        return reinterpret_cast<T*>(data)[i];
    }
    template <class T>
    T& at(int r, int c) {
        return reinterpret_cast<T*>(data)[(std::size_t)r * cols + c];
    }
    template <class T>
    T* ptr(int r = 0) {
        return reinterpret_cast<T*>(data) + (std::size_t)r * cols;
    }
};

// Only reached when the camera is distorted, which the baseline's frames are not.
inline void undistort(const Mat&, Mat&, const Mat&, const Mat&) {
    throw std::runtime_error("cv::undistort is not part of the baseline build");
}

}  // namespace cv
