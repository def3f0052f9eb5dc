// driver.cu -- runs the reference's own per-frame fusion loop, af::runVolumeFusion
// (src/VolumeFusion.cu:223-783), compiled unchanged for this GPU, on frames handed over from
// memory.  Baseline infrastructure only (the "reference GPU kernels" line of the benchmark):
// oracle/ref_gpu/build.py links it with the reference's sources into oracle/_ref/libvfref_gpu.so.
//
// The loop reads its frames through af::loadDepthFrame and its camera through af::loadIntrinsics /
// af::loadCameraDistortion (src/dataset.cpp, not built here); this file provides those three from
// memory -- uint16 millimetres to float metres, as dataset.cpp:188 does -- and records when each
// frame is requested, so the time between two requests is one frame of the loop (every stage of
// the loop ends with cudaDeviceSynchronize).  The viewer hooks of VolumeFusionOutput (stream
// buffers) are sinks that copy nothing, its stepper is disabled (include/af/Stepper.h:63 starts it
// enabled, which makes every frame wait for a viewer), and the loop's console output is kept only
// to report the lines before an exception.
#include <af/CameraModel.h>
#include <af/Settings.h>
#include <af/VolumeFusion.h>
#include <af/dataset.h>

#include <chrono>
#include <cstdint>
#include <cstring>
#include <iostream>
#include <sstream>
#include <vector>

namespace {

using Clock = std::chrono::steady_clock;

struct Feed {
    const uint16_t* frames = nullptr;
    int n = 0, width = 0, height = 0;
    float K[9] = {};
    std::vector<Clock::time_point> requested;
};
Feed g_feed;

template <class T>
struct Sink : af::StreamBufferAbstract<T> {
    void load(const T*, std::size_t) override {}
    void loadFromDevice(const T*, std::size_t) override {}
};

// Keeps the last bytes the loop prints (its own diagnostics precede each of its throws).
struct TailBuf : std::streambuf {
    std::string tail;
    int overflow(int c) override {
        if (c != EOF) {
            tail.push_back((char)c);
            if (tail.size() > 8192) tail.erase(0, tail.size() - 4096);
        }
        return c;
    }
};

}  // namespace

// src/Settings.cpp is not built (its preset loader needs a JSON library); the caller sets every field.
af::Settings::Settings() {}

namespace af {

void loadIntrinsics(const std::string&, Eigen::Matrix3f& K) {
    for (int c = 0; c < 3; ++c)
        for (int r = 0; r < 3; ++r) K(r, c) = g_feed.K[c * 3 + r];
}

bool loadCameraDistortion(const std::string&, af::CameraDistortion& d) {
    d = af::CameraDistortion();
    return true;
}

void loadDepthFrame(const std::string&, size_t index, cv::Mat& depth) {
    if ((int)index >= g_feed.n) throw std::runtime_error("loadDepthFrame: frame index out of range");
    g_feed.requested[index] = Clock::now();
    depth = cv::Mat(g_feed.height, g_feed.width, CV_32FC1);
    const uint16_t* mm = g_feed.frames + (std::size_t)index * g_feed.width * g_feed.height;
    float* out = reinterpret_cast<float*>(depth.data);
    for (std::size_t i = 0; i < depth.total(); ++i) out[i] = (float)(mm[i] * (1.0 / 1000.0));
}

}  // namespace af

extern "C" {

// One run of the loop over frames[0..n) (frame 0 initialises the volume, frames 1..n-1 are
// non-rigid), with the settings given.  frame_ms[i] receives frame i's wall time and *n_nodes the
// motion graph's size at the end.  Returns 0, or 1 when the loop threw (its message and the lines
// the loop printed before it are copied to err).
int ref_gpu_fusion(const uint16_t* frames_mm, int n_frames, int width, int height, const float* K_colmajor,
                   const float* volume_size, float delta, float depth_threshold, int bilateral, int bilateral_d,
                   float sigma_i, float sigma_s, float bilateral_thr, float excl_lo, float excl_hi, float graph_radius,
                   int update_graph, int icp_iterations, float weight_depth, float weight_mreg, float min_step,
                   float corr_thresh, double* frame_ms, int* n_nodes, char* err, int err_len) {
    g_feed.frames = frames_mm;
    g_feed.n = n_frames;
    g_feed.width = width;
    g_feed.height = height;
    std::memcpy(g_feed.K, K_colmajor, sizeof(g_feed.K));
    g_feed.requested.assign((std::size_t)n_frames, Clock::time_point());

    af::Settings s;
    s.tsdfSize = Vec3f(volume_size[0], volume_size[1], volume_size[2]);
    s.tsdfDim = Vec3i(256, 256, 256);
    s.tsdfCenter = Vec3f(0.f, 0.f, 0.f);
    s.tsdfRotation = Vec3i(0, 0, 0);
    s.normExclAngleRange = {excl_lo, excl_hi};
    s.framesRange = {0, n_frames};
    s.frameBreak = -1;
    s.dataFolder = "";
    s.cameraCount = 1;
    s.depthFilesPattern = "";
    s.depthThreshold = depth_threshold;
    s.integrateTsdf = true;
    s.bilateralFiltr = bilateral != 0;
    s.updateGraph = update_graph != 0;
    s.useCopyHack = true;
    s.useCholesky = true;
    s.bilateralD = bilateral_d;
    s.bilateralSigmaI = sigma_i;
    s.bilateralSigmaS = sigma_s;
    s.bilateralThreshold = bilateral_thr;
    s.energyWeightDepth = weight_depth;
    s.energyWeightMReg = weight_mreg;
    s.energyMinStep = min_step;
    s.icpIterations = icp_iterations;
    s.motionGraphRadius = graph_radius;
    s.motionGraphSampleDistance = graph_radius;
    s.tsdfDelta = delta;
    s.correspThreshDist = corr_thresh;
    s.isMeshWarped = false;

    MotionGraph graph;
    Sink<Vec3f> canon, warped, nodes, frame, meshPoints, centroid;
    Sink<Vec3i> faces;
    Sink<Vec2i> corr;
    Sink<Vecui<Constants::energyMRegKNN>> lines;
    af::Stepper stepper;
    std::atomic_flag keepRunning = ATOMIC_FLAG_INIT;
    keepRunning.test_and_set();  // the loop stops when a viewer clears it
    std::mutex mu;
    Mesh mesh;
    af::VolumeFusionOutput out{graph, canon, warped, nodes, frame, meshPoints, faces, corr, lines, centroid,
                               stepper,  keepRunning, mu, mesh};

    TailBuf tail;
    std::streambuf* saved = std::cout.rdbuf(&tail);
    stepper.enable(false);  // a Stepper starts enabled: the loop would wait for a viewer's step() each frame
    int rc = 0;
    try {
        af::runVolumeFusion(out, s);
    } catch (const std::exception& e) {
        rc = 1;
        if (err && err_len > 0) {
            std::string msg = std::string(e.what()) + " | " +
                              tail.tail.substr(tail.tail.size() > 3500 ? tail.tail.size() - 3500 : 0);
            std::strncpy(err, msg.c_str(), (std::size_t)err_len - 1);
            err[err_len - 1] = 0;
        }
    }
    const Clock::time_point end = Clock::now();
    std::cout.rdbuf(saved);
    if (n_nodes) *n_nodes = (int)graph.graph().size();
    for (int i = 0; i < n_frames; ++i) {
        const Clock::time_point next = i + 1 < n_frames ? g_feed.requested[(std::size_t)i + 1] : end;
        frame_ms[i] = std::chrono::duration<double, std::milli>(next - g_feed.requested[(std::size_t)i]).count();
    }
    return rc;
}

}  // extern "C"

// ---- a check of the build: frame 0 through the loop's own first steps ----
#include <af/MarchingCubes.cuh>
#include <af/TSDFIntegration.cuh>
#include <thrust/count.h>
#include <thrust/device_vector.h>
#include <thrust/extrema.h>

namespace af {
// src/VolumeFusion.cu:151-221 (defined there, not declared in a header)
void loadProcessFrame(cv::Mat& depth, thrust::device_vector<float>& depthFrame_d, thrust::device_vector<Vec3f>& depthMesh_d,
                      thrust::device_vector<Vec3f>& depthMeshNormals_d, Vec3f& centroid, size_t index,
                      const Mat3f& cDepthIntrinsics, const af::CameraDistortion& cDepthDistortion, af::Settings settings);
}  // namespace af

namespace {
struct FiniteDepth {
    __host__ __device__ bool operator()(float d) const { return d > 1.e-4f && d < 1.e30f; }
};
struct Positive {
    __host__ __device__ bool operator()(float w) const { return w > 0.f; }
};
}  // namespace

extern "C" int ref_gpu_frame0_check(const uint16_t* frame_mm, int width, int height, const float* K_colmajor,
                                    const float* volume_size, float delta, float depth_threshold, int bilateral,
                                    int bilateral_d, float sigma_i, float sigma_s, float bilateral_thr, float excl_lo,
                                    float excl_hi, double* out /* [8] */) {
    g_feed.frames = frame_mm;
    g_feed.n = 1;
    g_feed.width = width;
    g_feed.height = height;
    std::memcpy(g_feed.K, K_colmajor, sizeof(g_feed.K));
    g_feed.requested.assign(1, Clock::time_point());
    af::Settings s;
    s.depthThreshold = depth_threshold;
    s.bilateralFiltr = bilateral != 0;
    s.bilateralD = bilateral_d;
    s.bilateralSigmaI = sigma_i;
    s.bilateralSigmaS = sigma_s;
    s.bilateralThreshold = bilateral_thr;
    s.normExclAngleRange = {excl_lo, excl_hi};
    s.dataFolder = "";
    s.depthFilesPattern = "";
    Mat3f K;
    af::loadIntrinsics("", K);
    af::CameraDistortion dist;
    cv::Mat depth;
    thrust::device_vector<float> depth_d;
    thrust::device_vector<Vec3f> mesh_d, normals_d;
    Vec3f c;
    TailBuf tail;
    std::streambuf* saved = std::cout.rdbuf(&tail);
    int rc = 0;
    try {
        af::loadProcessFrame(depth, depth_d, mesh_d, normals_d, c, 0, K, dist, s);
        const Vec3i dims(256, 256, 256);
        const Vec3f size(volume_size[0], volume_size[1], volume_size[2]);
        const Vec3f vs = size.cwiseQuotient(dims.cast<float>());
        const std::size_t S = 256ull * 256 * 256;
        thrust::device_vector<float> tsdf(S, -1.f), w(S, 0.f);
        af::runIntegrateTSDFFromFrameKernel(tsdf.data().get(), w.data().get(), depth_d.data().get(),
                                            Vec2i(depth.cols, depth.rows), delta, dims, vs, size, Mat3f::Identity(), c, K);
        thrust::device_vector<Vec3f> pts(4000000);
        thrust::device_vector<unsigned int> n(1, 0);
        af::runMarchingCubesMeshKernel(pts.data().get(), n.data().get(), tsdf.data().get(), w.data().get(), dims, vs,
                                       size, 0.f);
        out[0] = (double)thrust::count_if(depth_d.begin(), depth_d.end(), FiniteDepth());
        out[1] = c[0];
        out[2] = c[1];
        out[3] = c[2];
        out[4] = (double)thrust::count_if(w.begin(), w.end(), Positive());
        out[5] = *thrust::min_element(tsdf.begin(), tsdf.end());
        out[6] = *thrust::max_element(tsdf.begin(), tsdf.end());
        out[7] = (double)(unsigned int)n[0];
    } catch (const std::exception& e) {
        rc = 1;
    }
    std::cout.rdbuf(saved);
    return rc;
}
