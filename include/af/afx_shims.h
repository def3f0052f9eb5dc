/*
 * af/afx_shims.h -- header-only C++ forwarding from the reference's af:: operator names to
 * the C ABI in afx/afx.h.
 *
 * A caller written against the reference's headers (include/af/) keeps its call sites: the
 * functions below take the same arguments in the same order, with the reference's element types.  Buffers of Vec3f, Mat4f, Vec2i, Vecui<K> or Vecf<K> (af/afx_types.h: the
 * caller's Eigen types when Eigen is included first) are passed as such; a pointer to plain
 * float / int / unsigned is accepted as well, with K then given explicitly (default
 * Constants::motionGraphKNN, as the reference's kernels hard-code it).  Value arguments (Vec2i,
 * Vec3i, Vec3f, Mat3f, Mat4f) are accepted through templates: anything indexable with [] for
 * vectors and exposing column-major .data() for matrices.
 *
 * Like the reference, each call blocks until the GPU work has finished (the reference
 * synchronised after every launch) and throws std::runtime_error on failure (the reference's
 * CUDA_CHECK, src/Helper.cu:7-20).  Callers that want asynchronous launches call the afx_*
 * functions directly with a stream.  The classes (DeviceTsdf, WarpField, MotionGraph,
 * TSDFVolume, ...) are in af/afx_classes.h.
 */
#ifndef AF_AFX_SHIMS_H
#define AF_AFX_SHIMS_H

#include <cuda_runtime_api.h>

#include <climits>
#include <cstddef>
#include <cstdint>
#include <limits>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>

#include "../afx/afx.h"
#include "afx_types.h"

namespace af {
namespace detail {

inline void afx_check(int status, const char* what) {
    if (status != AFX_OK) {
        throw std::runtime_error(std::string(what) + ": " + afx_status_string(status));
    }
    cudaError_t e = cudaStreamSynchronize(nullptr);
    if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

inline void cuda_check(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

template <class V>
inline void to_f3(const V& v, float* o) {
    o[0] = (float)v[0];
    o[1] = (float)v[1];
    o[2] = (float)v[2];
}
template <class V>
inline void to_i3(const V& v, int* o) {
    o[0] = (int)v[0];
    o[1] = (int)v[1];
    o[2] = (int)v[2];
}
template <class M>
inline void to_m3(const M& m, float* o) {  // column-major, as Eigen stores it
    const float* d = m.data();
    for (int i = 0; i < 9; ++i) o[i] = d[i];
}
template <class M>
inline void to_m4(const M& m, float* o) {
    const float* d = m.data();
    for (int i = 0; i < 16; ++i) o[i] = d[i];
}

// A buffer of elements T seen as the scalars S it packs: T is S itself or N packed S.
template <class S, int N, class T>
inline typename std::conditional<std::is_const<T>::value, const S*, S*>::type flat(T* p) {
    static_assert(sizeof(T) == N * sizeof(S) || sizeof(T) == sizeof(S),
                  "element type must be the scalar or N packed scalars (Vec3f, Mat4f, Vec2i, ...)");
    return reinterpret_cast<typename std::conditional<std::is_const<T>::value, const S*, S*>::type>(p);
}
template <int N, class T>
inline auto ff(T* p) -> decltype(flat<float, N>(p)) {
    return flat<float, N>(p);
}

// Neighbour slots per point: the element's length for Vecui<K> / Vecf<K> buffers, else K as given
// (K <= 0: the reference's Constants::motionGraphKNN).
template <class T>
inline int slots(int K) {
    static_assert(sizeof(T) % 4 == 0, "neighbour buffers hold 4-byte values");
    const int n = (int)(sizeof(T) / 4);
    if (n == 1) return K > 0 ? K : (int)Constants::motionGraphKNN;
    if (K > 0 && K != n) throw std::invalid_argument("af: K differs from the neighbour element's length");
    return n;
}
template <class T>
inline uint32_t* u32(T* p) {
    return reinterpret_cast<uint32_t*>(p);
}
template <class T>
inline const uint32_t* u32(const T* p) {
    return reinterpret_cast<const uint32_t*>(p);
}

// One int on the device (node counts the afx_* calls read from device memory).
struct DeviceInt {
    int* p = nullptr;
    explicit DeviceInt(int v) {
        cuda_check(cudaMalloc(reinterpret_cast<void**>(&p), sizeof(int)), "cudaMalloc");
        cuda_check(cudaMemcpy(p, &v, sizeof(int), cudaMemcpyHostToDevice), "cudaMemcpy");
    }
    ~DeviceInt() { cudaFree(p); }
    DeviceInt(const DeviceInt&) = delete;
    DeviceInt& operator=(const DeviceInt&) = delete;
    int get() const {
        int v = 0;
        cuda_check(cudaMemcpy(&v, p, sizeof(int), cudaMemcpyDeviceToHost), "cudaMemcpy");
        return v;
    }
};

// Scratch device memory for one call.
struct Workspace {
    void* p = nullptr;
    size_t bytes = 0;
    explicit Workspace(size_t n) : bytes(n) {
        if (n) cuda_check(cudaMalloc(&p, n), "cudaMalloc (workspace)");
    }
    ~Workspace() { cudaFree(p); }
    Workspace(const Workspace&) = delete;
    Workspace& operator=(const Workspace&) = delete;
};

}  // namespace detail

// ---- include/af/VertexManipulation.cuh ----

// fillValue: what replaces rejected values (src/VertexManipulation.cu:6-15).
inline void runFilterDepthKernel(float* depth, unsigned int depthSize, float threshold,
                                 float fillValue = std::numeric_limits<float>::infinity()) {
    detail::afx_check(afx_filter_depth_fill(depth, depthSize, threshold, fillValue, nullptr), "runFilterDepthKernel");
}

template <class P3, class Mat3f>
inline void runDepthToMeshKernel(P3* mesh, const float* cDepth, unsigned int depthWidth, unsigned int depthHeight,
                                 const Mat3f& K) {
    float k[9];
    detail::to_m3(K, k);
    detail::afx_check(afx_depth_to_mesh(detail::ff<3>(mesh), cDepth, (int)depthWidth, (int)depthHeight, k, nullptr),
                      "runDepthToMeshKernel");
}

template <class P3, class Q3>
inline void runDepthVerticesNormalsKernel(P3* normals, Q3* vertices, const float* /*depth*/, int h, int w,
                                          std::pair<float, float> normExclAngleRange) {
    detail::afx_check(afx_depth_vertices_normals(detail::ff<3>(normals), detail::ff<3>(vertices), h, w,
                                                 normExclAngleRange.first, normExclAngleRange.second, nullptr),
                      "runDepthVerticesNormalsKernel");
}

template <class P3, class Q3>
inline void runRemoveDepthWithoutNormalsKernel(P3* normals, Q3* vertices, float* depth, int h, int w) {
    detail::afx_check(afx_remove_depth_without_normals(detail::ff<3>(normals), detail::ff<3>(vertices), depth, h, w,
                                                       nullptr),
                      "runRemoveDepthWithoutNormalsKernel");
}

template <class P3, class Vec3f>
inline void runTranslateKernel(P3* mesh, unsigned int meshSize, const Vec3f& translation) {
    float t[3];
    detail::to_f3(translation, t);
    detail::afx_check(afx_translate(detail::ff<3>(mesh), nullptr, (long)meshSize, t, nullptr), "runTranslateKernel");
}

// knnWeights[i][j] = exp(-d^2 / 2r^2) of slot j (0 at d >= r), normalised to sum 1
// (src/VertexManipulation.cu:105-132).
template <class PW, class PI, class PD>
inline void runComputeWarpWeightsKernel(PW* knnWeights, const float* cMotionGraphRadiuses, const PI* cKnnIdxs,
                                        const PD* cKnnDists, const std::size_t cMeshSize, int K = 0) {
    const int k = detail::slots<PI>(K);
    detail::DeviceInt all(INT_MAX);  // every stored index is a node (empty slots hold 0xFFFFFFFF)
    detail::afx_check(afx_warp_weights(reinterpret_cast<float*>(knnWeights), cMotionGraphRadiuses, detail::u32(cKnnIdxs),
                                       reinterpret_cast<const float*>(cKnnDists), nullptr, (long)cMeshSize, k, all.p,
                                       nullptr),
                      "runComputeWarpWeightsKernel");
}

// ---- include/af/BilateralFilter.cuh ----
inline void bilateralFilterTextureOpmShared(float* output, const float* input, int height, int width, int r, double sI,
                                            double sS, float thr) {
    detail::afx_check(afx_bilateral_filter(output, input, height, width, r, sI, sS, thr, nullptr),
                      "bilateralFilterTextureOpmShared");
}

// ---- include/af/TSDFIntegration.cuh ----
template <class Vec2i, class Vec3i, class Vec3f, class Mat3f, class Vec3t>
inline void runIntegrateTSDFFromFrameKernel(float* tsdf, float* tsdfWeights, const float* cDepthFrame,
                                            const Vec2i cFrameDims, const float cDelta, const Vec3i cDims,
                                            const Vec3f cVoxelSize, const Vec3f cVolumeSize,
                                            const Mat3f cVolumeRotate, const Vec3t cVolumeTranslate,
                                            const Mat3f cDepthIntrinsics) {
    int dims[3];
    float vs[3], size[3], R[9], t[3], K[9];
    detail::to_i3(cDims, dims);
    detail::to_f3(cVoxelSize, vs);
    detail::to_f3(cVolumeSize, size);
    detail::to_m3(cVolumeRotate, R);
    detail::to_f3(cVolumeTranslate, t);
    detail::to_m3(cDepthIntrinsics, K);
    detail::afx_check(afx_integrate_tsdf(tsdf, tsdfWeights, cDepthFrame, (int)cFrameDims[0], (int)cFrameDims[1],
                                         cDelta, dims, vs, size, R, t, K, nullptr),
                      "runIntegrateTSDFFromFrameKernel");
}

template <class P3, class Vec3f, class Vec3i, class Mat3f>
inline void runCountCollisionsPerVoxelKernel(int* collisionCounts, const P3* tsdfVertices, const int* cKnnCounts,
                                             const Vec3f cVoxelSize, const Vec3f cVolumeSize, const Vec3i cVolumeDim,
                                             const Mat3f cVolumeRotate, const Vec3f cVolumeTranslate) {
    int dims[3];
    float vs[3], size[3], R[9], t[3];
    detail::to_i3(cVolumeDim, dims);
    detail::to_f3(cVoxelSize, vs);
    detail::to_f3(cVolumeSize, size);
    detail::to_m3(cVolumeRotate, R);
    detail::to_f3(cVolumeTranslate, t);
    detail::afx_check(afx_count_collisions(collisionCounts, detail::ff<3>(tsdfVertices), cKnnCounts, vs, size, dims, R,
                                           t, nullptr),
                      "runCountCollisionsPerVoxelKernel");
}

template <class P3, class Vec2i, class Vec3f, class Vec3i, class Mat3f>
inline void runIntegrateWarpedTSDFFromFrameKernel(float* tsdf, float* tsdfWeights, const P3* cTsdfVertices,
                                                  const int* collisionCounts, const int* cKnnCounts,
                                                  const float* cDepthFrame, const Vec2i cFrameDims,
                                                  const float cDelta, const Vec3f cVoxelSize,
                                                  const Vec3f cVolumeSize, const Vec3i cVolumeDim,
                                                  const Mat3f cVolumeRotate, const Vec3f cVolumeTranslate,
                                                  const Mat3f cDepthIntrinsics) {
    int dims[3];
    float vs[3], size[3], R[9], t[3], K[9];
    detail::to_i3(cVolumeDim, dims);
    detail::to_f3(cVoxelSize, vs);
    detail::to_f3(cVolumeSize, size);
    detail::to_m3(cVolumeRotate, R);
    detail::to_f3(cVolumeTranslate, t);
    detail::to_m3(cDepthIntrinsics, K);
    detail::afx_check(afx_integrate_warped_tsdf(tsdf, tsdfWeights, detail::ff<3>(cTsdfVertices), collisionCounts,
                                                cKnnCounts, cDepthFrame, (int)cFrameDims[0], (int)cFrameDims[1],
                                                cDelta, vs, size, dims, R, t, K, nullptr),
                      "runIntegrateWarpedTSDFFromFrameKernel");
}

// ---- include/af/TSDFWarp.h ----
template <class PI, class PD, class P3, class Vec3f, class Vec3i>
inline void runTsdfKNNGraph(PI* knnIdxs, PD* knnDists, int* knnCounts, const P3* cGraph, const float* cGraphRadiuses,
                            const std::size_t cGraphSize, const Vec3f cVoxelSize, const Vec3f cVolumeSize,
                            const Vec3i cVolumeDim, const Vec3i cVoxelsPerNode, int K = 0) {
    const int k = detail::slots<PI>(K);
    int dims[3], per[3];
    float vs[3], size[3];
    detail::to_i3(cVolumeDim, dims);
    detail::to_i3(cVoxelsPerNode, per);
    detail::to_f3(cVoxelSize, vs);
    detail::to_f3(cVolumeSize, size);
    detail::Workspace ws(afx_tsdf_knn_workspace_size(dims, (int)cGraphSize, per));
    detail::afx_check(afx_tsdf_knn(detail::u32(knnIdxs), reinterpret_cast<float*>(knnDists), knnCounts,
                                   detail::ff<3>(cGraph), cGraphRadiuses, (int)cGraphSize, vs, size, dims, per, k,
                                   ws.p, ws.bytes, nullptr),
                      "runTsdfKNNGraph");
}

template <class PW, class PI, class PD>
inline void runComputeTsdfWarpWeightsKernel(PW* cKnnWeights, const float* cMotionGraphRadiuses, const PI* cKnnIdxs,
                                            const PD* cKnnDists, const int* cKnnCounts, const std::size_t cGridSize,
                                            int K = 0) {
    const int k = detail::slots<PI>(K);
    detail::afx_check(afx_tsdf_warp_weights(reinterpret_cast<float*>(cKnnWeights), cMotionGraphRadiuses,
                                            detail::u32(cKnnIdxs), reinterpret_cast<const float*>(cKnnDists),
                                            cKnnCounts, (long)cGridSize, k, nullptr),
                      "runComputeTsdfWarpWeightsKernel");
}

template <class P3, class Vec3f, class Vec3i>
inline void runGenerateTsdfVerticesKernel(P3* tsdfVertices, const Vec3f cVoxelSize, const Vec3f cVolumeSize,
                                          const Vec3i cVolumeDim) {
    int dims[3];
    float vs[3], size[3];
    detail::to_i3(cVolumeDim, dims);
    detail::to_f3(cVoxelSize, vs);
    detail::to_f3(cVolumeSize, size);
    detail::afx_check(afx_tsdf_vertices(detail::ff<3>(tsdfVertices), vs, size, dims, nullptr),
                      "runGenerateTsdfVerticesKernel");
}

template <class P3, class P16, class PI, class PW, class Vec3f, class Vec3i>
inline void runWarpTsdfKernel(P3* tsdfVertices, const P16* cMotionGraph, const PI* cKnnIdxs, const PW* cKnnWeights,
                              const int* cKnnCounts, const Vec3f cVoxelSize, const Vec3f cVolumeSize,
                              const Vec3i cVolumeDim, int K = 0) {
    (void)cVoxelSize;
    (void)cVolumeSize;
    const int k = detail::slots<PI>(K);
    const long n = (long)cVolumeDim[0] * (long)cVolumeDim[1] * (long)cVolumeDim[2];
    detail::afx_check(afx_warp_tsdf(detail::ff<3>(tsdfVertices), detail::ff<16>(cMotionGraph), detail::u32(cKnnIdxs),
                                    reinterpret_cast<const float*>(cKnnWeights), cKnnCounts, n, k, nullptr),
                      "runWarpTsdfKernel");
}

// ---- include/af/MarchingCubes.cuh ----
// The reference's kernels append at *meshSize without a bound (src/MarchingCubes.cu:510-520); the
// overloads without a capacity keep that contract: the buffer must hold every point the volume
// yields (at most 12 per cube).  The overloads with a capacity stop there and report overflow.
template <class P3, class Vec3i, class Vec3f>
inline void runMarchingCubesMeshKernel(P3* mesh, unsigned int* meshSize, std::size_t meshCapacity, const float* cTsdf,
                                       const float* cTsdfWeights, const Vec3i cDims, const Vec3f& cVoxelSize,
                                       const Vec3f& cVolSize, const float cIsoValue) {
    int dims[3];
    float vs[3], size[3];
    detail::to_i3(cDims, dims);
    detail::to_f3(cVoxelSize, vs);
    detail::to_f3(cVolSize, size);
    detail::afx_check(afx_marching_cubes_points(detail::ff<3>(mesh), meshSize, (long)meshCapacity, cTsdf, cTsdfWeights,
                                                dims, vs, size, cIsoValue, nullptr),
                      "runMarchingCubesMeshKernel");
}

template <class Vec3i>
inline std::size_t marching_cubes_bound(const Vec3i& d, int per_cube) {
    const long c = (long)(d[0] > 1 ? d[0] - 1 : 0) * (long)(d[1] > 1 ? d[1] - 1 : 0) * (long)(d[2] > 1 ? d[2] - 1 : 0);
    return (std::size_t)(c * per_cube);
}

template <class P3, class Vec3i, class Vec3f>
inline void runMarchingCubesMeshKernel(P3* mesh, unsigned int* meshSize, const float* cTsdf, const float* cTsdfWeights,
                                       const Vec3i cDims, const Vec3f& cVoxelSize, const Vec3f& cVolSize,
                                       const float cIsoValue) {
    runMarchingCubesMeshKernel(mesh, meshSize, marching_cubes_bound(cDims, 12), cTsdf, cTsdfWeights, cDims, cVoxelSize,
                               cVolSize, cIsoValue);
}

template <class P3, class F3, class Vec3i, class Vec3f>
inline void runMarchingCubesFullKernel(P3* mesh, unsigned int* meshSize, std::size_t meshCapacity, F3* faces,
                                       unsigned int* facesSize, std::size_t facesCapacity, const float* cTsdf,
                                       const float* cTsdfWeights, const Vec3i cDims, const Vec3f& cVoxelSize,
                                       const Vec3f& cVolSize, const float cIsoValue) {
    int dims[3];
    float vs[3], size[3];
    detail::to_i3(cDims, dims);
    detail::to_f3(cVoxelSize, vs);
    detail::to_f3(cVolSize, size);
    detail::afx_check(afx_marching_cubes_mesh(detail::ff<3>(mesh), meshSize, (long)meshCapacity,
                                              detail::flat<int, 3>(faces), facesSize, (long)facesCapacity, cTsdf,
                                              cTsdfWeights, dims, vs, size, cIsoValue, nullptr),
                      "runMarchingCubesFullKernel");
}

// Without capacities: at most 5 triangles (15 vertices) per cube.
template <class P3, class F3, class Vec3i, class Vec3f>
inline void runMarchingCubesFullKernel(P3* mesh, unsigned int* meshSize, F3* faces, unsigned int* facesSize,
                                       const float* cTsdf, const float* cTsdfWeights, const Vec3i cDims,
                                       const Vec3f& cVoxelSize, const Vec3f& cVolSize, const float cIsoValue) {
    runMarchingCubesFullKernel(mesh, meshSize, marching_cubes_bound(cDims, 15), faces, facesSize,
                               marching_cubes_bound(cDims, 5), cTsdf, cTsdfWeights, cDims, cVoxelSize, cVolSize,
                               cIsoValue);
}

// ---- include/af/ComputeCorrespondence.cuh ----
template <class P3, class Q3, class P16, class PI, class PW>
inline void runWarpKernel(P3* warpedMesh, const Q3* cMesh, const P16* cMotionGraph, const PI* cKnnIdxs,
                          const PW* cKnnWeights, const std::size_t cMeshSize, int K = 0) {
    const int k = detail::slots<PI>(K);
    detail::afx_check(afx_warp(detail::ff<3>(warpedMesh), detail::ff<3>(cMesh), detail::ff<16>(cMotionGraph),
                               detail::u32(cKnnIdxs), reinterpret_cast<const float*>(cKnnWeights), nullptr,
                               (long)cMeshSize, k, nullptr),
                      "runWarpKernel");
}

// runWarpKernel with dual-quaternion blending (afx_warp_dqb; no counterpart in the reference).
template <class P3, class Q3, class P16, class PI, class PW>
inline void runWarpDualQuaternionKernel(P3* warpedMesh, const Q3* cMesh, const P16* cMotionGraph, const PI* cKnnIdxs,
                                        const PW* cKnnWeights, const std::size_t cMeshSize, int K = 0) {
    const int k = detail::slots<PI>(K);
    detail::afx_check(afx_warp_dqb(detail::ff<3>(warpedMesh), detail::ff<3>(cMesh), detail::ff<16>(cMotionGraph),
                                   detail::u32(cKnnIdxs), reinterpret_cast<const float*>(cKnnWeights), nullptr,
                                   (long)cMeshSize, k, nullptr),
                      "runWarpDualQuaternionKernel");
}

// One (warped point, pixel) pair per warped point that projects onto a valid pixel whose vertex
// lies within thresholdDist (src/ComputeCorrespondence.cu:33-80), ordered by point index;
// cDepthDim = (rows, cols).  *corrIdxsSize (device) receives the pair count: the reference's kernel
// appends to it, and its callers zero it first.  corrIdxs holds up to cWarpedMeshSize pairs.
template <class P2, class P3, class Mat3f, class Vec2i, class Q3>
inline void runCorrespondencePairsKernel(P2* corrIdxs, unsigned int* corrIdxsSize, const P3* cWarpedMesh,
                                         const std::size_t cWarpedMeshSize, const Mat3f& K,
                                         const float* const cPtrDepth, const Vec2i cDepthDim,
                                         const Q3* const cFrameMesh, const float thresholdDist) {
    float k[9];
    detail::to_m3(K, k);
    detail::Workspace ws(afx_correspondences_workspace_size((long)cWarpedMeshSize));
    detail::afx_check(afx_correspondences(detail::flat<int, 2>(corrIdxs), corrIdxsSize, (long)cWarpedMeshSize,
                                          detail::ff<3>(cWarpedMesh), nullptr, (long)cWarpedMeshSize, k, cPtrDepth,
                                          (int)cDepthDim[0], (int)cDepthDim[1], detail::ff<3>(cFrameMesh),
                                          thresholdDist, ws.p, ws.bytes, nullptr),
                      "runCorrespondencePairsKernel");
}

// ---- include/af/MotionOptimization.cuh ----
// T -= [[x_rot]_x, x_t; 0] per node (src/MotionOptimization.cu:483-506).
template <class P16, class P6>
inline void runUpdateTransformsKernel(P16* transforms, const P6* cUpdates, unsigned int transformsSize) {
    detail::DeviceInt n((int)transformsSize);
    detail::afx_check(afx_update_transforms(detail::ff<16>(transforms), detail::ff<6>(cUpdates), n.p,
                                            (int)transformsSize, nullptr),
                      "runUpdateTransformsKernel");
}

// The reference's wrapper launches the same subtracting kernel as runUpdateTransformsKernel
// (src/MotionOptimization.cu:525-531), so this entry point subtracts too.
template <class P16, class P6>
inline void runUpdateTransformsReverseKernel(P16* transforms, const P6* cUpdates, unsigned int transformsSize) {
    runUpdateTransformsKernel(transforms, cUpdates, transformsSize);
}

/* The reference's whole-frame loop (af::runVolumeFusion, src/VolumeFusion.cu:223) fed frame by frame. */
class VolumeFusionSession {
public:
    explicit VolumeFusionSession(const afx_fusion_params& p) {
        int st = afx_fusion_create(&p, &f_);
        if (st != AFX_OK) throw std::runtime_error(std::string("afx_fusion_create: ") + afx_status_string(st));
    }
    ~VolumeFusionSession() { afx_fusion_destroy(f_); }
    VolumeFusionSession(const VolumeFusionSession&) = delete;
    VolumeFusionSession& operator=(const VolumeFusionSession&) = delete;
    void processHostFrame(const uint16_t* depthMm) {
        detail::afx_check(afx_fusion_process_host(f_, depthMm, nullptr), "afx_fusion_process_host");
    }
    afx_frame_stats stats() {
        afx_frame_stats s;
        int st = afx_fusion_stats(f_, &s, nullptr);
        if (st != AFX_OK) throw std::runtime_error(std::string("afx_fusion_stats: ") + afx_status_string(st));
        return s;
    }
    afx_fusion* handle() { return f_; }

private:
    afx_fusion* f_ = nullptr;
};

}  // namespace af

#endif
