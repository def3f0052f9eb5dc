/*
 * af/afx_ingest.h -- the reference's depth-ingest functions over the C ABI (header-only C++17):
 *
 *   insertIntoPattern, loadIntrinsics, loadCameraDistortion    src/dataset.cpp:22-79, 131-150
 *   loadDepthFrame                                             src/dataset.cpp:168-189 (cv::imread of a
 *                                                              16-bit PNG / TIFF, then metres)
 *   DepthUndistorter                                           cv::undistort (src/VolumeFusion.cu:162-180),
 *                                                              initUndistortRectifyMap + remap(INTER_NEAREST)
 *                                                              (src/MeshRecontructionStream.cu:94-101)
 *   create_xy_lookup_table, transformation_unproject / _project  src/CameraCalibration.cpp:220-295
 *
 * The reference's cv::Mat arguments become host vectors or device buffers: loadDepthFrame decodes on
 * the host and converts to metres on the device; the undistortion map and the ray table are device
 * arrays.  Calls block until the GPU work has finished and throw std::runtime_error on failure, as
 * the rest of the af:: surface does.
 */
#ifndef AF_AFX_INGEST_H
#define AF_AFX_INGEST_H

#include <cstdint>
#include <fstream>
#include <iterator>
#include <stdexcept>
#include <string>
#include <vector>

#include "afx_containers.h"

namespace af {

// af::insertIntoPattern (src/dataset.cpp:131-150): the run of all the pattern's '*' replaced by the
// zero-padded index.  The reference prints a message and returns "" for a pattern without that run.
inline std::string insertIntoPattern(const std::string& pattern, std::size_t index) {
    std::vector<char> out(pattern.size() + 32);
    const int rc = afx_depth_file_name(pattern.c_str(), (long)index, out.data(), out.size());
    return rc == AFX_OK ? std::string(out.data()) : std::string();
}

// af::loadIntrinsics (src/dataset.cpp:22-42): nine numbers, row by row.
inline void loadIntrinsics(const std::string& intrinsicsFile, Mat3f& K) {
    if (intrinsicsFile.empty()) throw std::runtime_error("loadIntrinsics(): Intrinsics file name is empty.");
    std::ifstream in(intrinsicsFile.c_str());
    if (!in.is_open())
        throw std::runtime_error("loadIntrinsics(): Intrinsics file " + intrinsicsFile + " couldn't be open.");
    K = Mat3f::Identity();
    float v = 0.f;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            in >> v;
            K(i, j) = v;
        }
}

// af::loadCameraDistortion (src/dataset.cpp:44-79): k1 k2 p1 p2 k3 k4 k5 k6.
inline bool loadCameraDistortion(const std::string& filename, CameraDistortion& d) {
    d.is_distorted = false;
    if (filename.empty()) return false;
    std::ifstream in(filename.c_str());
    if (!in.is_open()) return false;
    float c[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    for (float& x : c) in >> x;
    d.k1 = c[0];
    d.k2 = c[1];
    d.p1 = c[2];
    d.p2 = c[3];
    d.k3 = c[4];
    d.k4 = c[5];
    d.k5 = c[6];
    d.k6 = c[7];
    d.codx = d.cody = 0.f;
    d.is_distorted = true;
    return true;
}

namespace detail {
inline afx_camera_distortion to_afx(const CameraDistortion& d) {
    afx_camera_distortion o;
    o.k1 = d.k1;
    o.k2 = d.k2;
    o.k3 = d.k3;
    o.k4 = d.k4;
    o.k5 = d.k5;
    o.k6 = d.k6;
    o.codx = d.codx;
    o.cody = d.cody;
    o.p1 = d.p1;
    o.p2 = d.p2;
    o.is_distorted = d.is_distorted ? 1 : 0;
    return o;
}
inline void intrinsics4(const CameraIntrinsics& c, float* o) {
    o[0] = c.cx;
    o[1] = c.cy;
    o[2] = c.fx;
    o[3] = c.fy;
}
}  // namespace detail

// The uint16 millimetre image of frame `index` (af::loadDepthFrame before its convertTo).
inline std::vector<uint16_t> loadDepthFrameMm(const std::string& pattern, std::size_t index, int& width,
                                              int& height) {
    const std::string file = insertIntoPattern(pattern, index);
    if (file.empty()) throw std::runtime_error("loadDepthFrame(): file name pattern is not correct");
    std::ifstream in(file.c_str(), std::ios::binary);
    if (!in.is_open()) throw std::runtime_error("loadDepthFrame(): Depth couldn't be loadded");
    std::vector<uint8_t> bytes((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>());
    detail::afx_check(afx_decode_depth_image(bytes.data(), bytes.size(), nullptr, 0, &width, &height),
                      "loadDepthFrame");
    std::vector<uint16_t> mm((std::size_t)width * height);
    detail::afx_check(afx_decode_depth_image(bytes.data(), bytes.size(), mm.data(), (long)mm.size(), &width, &height),
                      "loadDepthFrame");
    return mm;
}

// af::loadDepthFrame (src/dataset.cpp:168-189) into a device depth image in metres.
inline void loadDepthFrame(const std::string& pattern, std::size_t index, DeviceDepthImage& depth) {
    int w = 0, h = 0;
    const std::vector<uint16_t> mm = loadDepthFrameMm(pattern, index, w, h);
    depth.resize((std::size_t)h, (std::size_t)w);
    DeviceArray<uint16_t> mm_d(mm.size());
    copyToDevice(mm_d.get(), mm.data(), mm.size());
    detail::afx_check(afx_depth_from_mm(depth.dataPtr(), mm_d.get(), (long)mm.size(), nullptr), "loadDepthFrame");
}

// The reference's undistortion of a depth frame with the intrinsics as new camera matrix: the map is
// built once (the reference's stream readers rebuild it every frame), apply() remaps a float image.
class DepthUndistorter {
public:
    enum Mode { Linear = AFX_UNDISTORT_LINEAR, Nearest = AFX_UNDISTORT_NEAREST };

    DepthUndistorter(const Mat3f& K, const CameraDistortion& distortion, int width, int height, Mode mode = Linear)
        : _map((std::size_t)width * height * 2), _width(width), _height(height), _mode(mode) {
        float k[9];
        detail::to_m3(K, k);
        const afx_camera_distortion d = detail::to_afx(distortion);
        detail::afx_check(afx_undistort_map(_map.get(), width, height, k, &d, (int)mode, nullptr),
                          "DepthUndistorter");
    }
    // dst = remap(src); both device images of the camera's size, not aliased.
    void apply(const float* src_d, float* dst_d) const {
        detail::afx_check(afx_undistort_depth(dst_d, src_d, _width, _height, _map.get(), (int)_mode, nullptr),
                          "DepthUndistorter::apply");
    }
    // In place on a device depth image, as the reference's callers overwrite their frame.
    void apply(DeviceDepthImage& depth) const {
        DeviceArray<float> tmp(depth.size());
        apply(depth.dataPtr(), tmp.get());
        detail::cuda_check(cudaMemcpy(depth.dataPtr(), tmp.get(), depth.size() * sizeof(float), cudaMemcpyDeviceToDevice),
                           "DepthUndistorter::apply");
    }
    const uint32_t* mapPtr() const { return _map.get(); }

private:
    DeviceArray<uint32_t> _map;
    int _width, _height;
    Mode _mode;
};

// af::create_xy_lookup_table (src/CameraCalibration.cpp:261-295) into a device table of width x height
// Vec2f (the reference fills a host cv::Mat of Vec2f).  False unless fx, fy > 0.
inline bool create_xy_lookup_table(const CameraModel& camera, DeviceBuffer<Vec2f>& xy_table) {
    if (!(camera.intrinsics.fx > 0.f && camera.intrinsics.fy > 0.f)) return false;
    const std::size_t n = (std::size_t)camera.width * camera.height;
    if (xy_table.bufferSize() < n) xy_table.resizeBuffer(n);
    xy_table.setSize((unsigned int)n);
    float intr[4];
    detail::intrinsics4(camera.intrinsics, intr);
    const afx_camera_distortion d = detail::to_afx(camera.distortion);
    detail::afx_check(afx_xy_lookup_table(detail::ff<2>(xy_table.bufferPtr()), (int)camera.width, (int)camera.height,
                                          intr, &d, nullptr),
                      "create_xy_lookup_table");
    return true;
}

// af::transformation_unproject / transformation_project (src/CameraCalibration.cpp:220-259) over
// device arrays of n pixels (Vec2f) + depths -> points (Vec3f) + valid flags, and back.
inline void transformation_unproject(const CameraModel& camera, const Vec2f* points2d_d, const float* depths_d,
                                     std::size_t n, Vec3f* points3d_d, int* valid_d) {
    float intr[4];
    detail::intrinsics4(camera.intrinsics, intr);
    const afx_camera_distortion d = detail::to_afx(camera.distortion);
    detail::afx_check(afx_unproject_points(detail::ff<3>(points3d_d), valid_d, detail::ff<2>(points2d_d), depths_d,
                                           (long)n, intr, &d, nullptr),
                      "transformation_unproject");
}
inline void transformation_project(const CameraModel& camera, const Vec3f* points3d_d, std::size_t n,
                                   Vec2f* points2d_d, int* valid_d) {
    float intr[4];
    detail::intrinsics4(camera.intrinsics, intr);
    const afx_camera_distortion d = detail::to_afx(camera.distortion);
    detail::afx_check(afx_project_points(detail::ff<2>(points2d_d), valid_d, detail::ff<3>(points3d_d), (long)n,
                                         intr, &d, nullptr),
                      "transformation_project");
}

}  // namespace af

#endif
