// Minimal stand-in for cv::Mat: the reference CPU sources compiled for the oracle pins
// only read Mat::data/rows/cols/empty().  Test build only.
#pragma once
namespace cv {
struct Mat {
    unsigned char* data = nullptr;
    int rows = 0, cols = 0;
    Mat() = default;
    Mat(int r, int c, void* d) : data(static_cast<unsigned char*>(d)), rows(r), cols(c) {}
    bool empty() const { return data == nullptr || rows == 0 || cols == 0; }
};
}  // namespace cv
