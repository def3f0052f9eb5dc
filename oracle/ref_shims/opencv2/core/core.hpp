// Minimal stand-in for cv::Mat: the reference CPU sources compiled for the oracle pins
// only read Mat::data/rows/cols/empty() and write 2-float elements through at<Vec2f>(row, col)
// (a view over the caller's buffer).  Test build only.
#pragma once
#include <cstddef>
namespace cv {
struct Vec2f {
    float v[2];
    Vec2f(float a, float b) : v{a, b} {}
};
struct Mat {
    unsigned char* data = nullptr;
    int rows = 0, cols = 0;
    Mat() = default;
    Mat(int r, int c, void* d) : data(static_cast<unsigned char*>(d)), rows(r), cols(c) {}
    bool empty() const { return data == nullptr || rows == 0 || cols == 0; }
    template <class T>
    T& at(int r, int c) {
        return reinterpret_cast<T*>(data)[(std::size_t)r * cols + c];
    }
};
}  // namespace cv
