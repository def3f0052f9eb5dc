/*
 * af/afx_shims.h -- header-only C++ forwarding from the reference's af:: operator names to
 * the C ABI in afx/afx.h.
 *
 * A caller written against the reference (include/af/*.cuh, include/af/*.h) keeps its call
 * sites: the functions below take the same arguments in the same order.  Small Eigen values
 * (Vec2i, Vec3i, Vec3f, Mat3f, Mat4f) are accepted through templates -- anything indexable
 * with [] for vectors and exposing column-major .data() for matrices -- so this header does not
 * depend on Eigen.  Like the reference, each call blocks until the GPU work has finished
 * (the reference synchronised after every launch) and throws std::runtime_error on failure
 * (the reference's CUDA_CHECK, src/Helper.cu:7-20).  Callers that want asynchronous launches
 * call the afx_* functions directly with a stream.
 */
#ifndef AF_AFX_SHIMS_H
#define AF_AFX_SHIMS_H

#include <cuda_runtime_api.h>

#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>

#include "../afx/afx.h"

namespace af {
namespace detail {

inline void afx_check(int status, const char* what) {
    if (status != AFX_OK) {
        throw std::runtime_error(std::string(what) + ": " + afx_status_string(status));
    }
    cudaError_t e = cudaStreamSynchronize(nullptr);
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

}  // namespace detail

// include/af/VertexManipulation.cuh
inline void runFilterDepthKernel(float* depth, unsigned int depthSize, float threshold) {
    detail::afx_check(afx_filter_depth(depth, depthSize, threshold, nullptr), "runFilterDepthKernel");
}

template <class Mat3f>
inline void runDepthToMeshKernel(float* mesh, const float* cDepth, unsigned int depthWidth, unsigned int depthHeight,
                                 const Mat3f& K) {
    float k[9];
    detail::to_m3(K, k);
    detail::afx_check(afx_depth_to_mesh(mesh, cDepth, (int)depthWidth, (int)depthHeight, k, nullptr),
                      "runDepthToMeshKernel");
}

inline void runDepthVerticesNormalsKernel(float* normals, float* vertices, const float* /*depth*/, int h, int w,
                                          std::pair<float, float> normExclAngleRange) {
    detail::afx_check(afx_depth_vertices_normals(normals, vertices, h, w, normExclAngleRange.first,
                                                 normExclAngleRange.second, nullptr),
                      "runDepthVerticesNormalsKernel");
}

inline void runRemoveDepthWithoutNormalsKernel(float* normals, float* vertices, float* depth, int h, int w) {
    detail::afx_check(afx_remove_depth_without_normals(normals, vertices, depth, h, w, nullptr),
                      "runRemoveDepthWithoutNormalsKernel");
}

// include/af/BilateralFilter.cuh
inline void bilateralFilterTextureOpmShared(float* output, const float* input, int height, int width, int r, double sI,
                                            double sS, float thr) {
    detail::afx_check(afx_bilateral_filter(output, input, height, width, r, sI, sS, thr, nullptr),
                      "bilateralFilterTextureOpmShared");
}

// include/af/TSDFIntegration.cuh
template <class Vec2i, class Vec3i, class Vec3f, class Mat3f>
inline void runIntegrateTSDFFromFrameKernel(float* tsdf, float* tsdfWeights, const float* cDepthFrame,
                                            const Vec2i cFrameDims, const float cDelta, const Vec3i cDims,
                                            const Vec3f cVoxelSize, const Vec3f cVolumeSize,
                                            const Mat3f cVolumeRotate, const Vec3f cVolumeTranslate,
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

template <class Vec3f, class Vec3i, class Mat3f>
inline void runCountCollisionsPerVoxelKernel(int* collisionCounts, const float* tsdfVertices, const int* cKnnCounts,
                                             const Vec3f cVoxelSize, const Vec3f cVolumeSize, const Vec3i cVolumeDim,
                                             const Mat3f cVolumeRotate, const Vec3f cVolumeTranslate) {
    int dims[3];
    float vs[3], size[3], R[9], t[3];
    detail::to_i3(cVolumeDim, dims);
    detail::to_f3(cVoxelSize, vs);
    detail::to_f3(cVolumeSize, size);
    detail::to_m3(cVolumeRotate, R);
    detail::to_f3(cVolumeTranslate, t);
    detail::afx_check(afx_count_collisions(collisionCounts, tsdfVertices, cKnnCounts, vs, size, dims, R, t, nullptr),
                      "runCountCollisionsPerVoxelKernel");
}

template <class Vec2i, class Vec3f, class Vec3i, class Mat3f>
inline void runIntegrateWarpedTSDFFromFrameKernel(float* tsdf, float* tsdfWeights, const float* cTsdfVertices,
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
    detail::afx_check(afx_integrate_warped_tsdf(tsdf, tsdfWeights, cTsdfVertices, collisionCounts, cKnnCounts,
                                                cDepthFrame, (int)cFrameDims[0], (int)cFrameDims[1], cDelta, vs, size,
                                                dims, R, t, K, nullptr),
                      "runIntegrateWarpedTSDFFromFrameKernel");
}

// include/af/TSDFWarp.h (K = number of slots per voxel)
template <class Vec3f, class Vec3i>
inline void runTsdfKNNGraph(uint32_t* knnIdxs, float* knnDists, int* knnCounts, const float* cGraph,
                            const float* cGraphRadiuses, const std::size_t cGraphSize, const Vec3f cVoxelSize,
                            const Vec3f cVolumeSize, const Vec3i cVolumeDim, const Vec3i cVoxelsPerNode, int K) {
    int dims[3], per[3];
    float vs[3], size[3];
    detail::to_i3(cVolumeDim, dims);
    detail::to_i3(cVoxelsPerNode, per);
    detail::to_f3(cVoxelSize, vs);
    detail::to_f3(cVolumeSize, size);
    std::size_t bytes = afx_tsdf_knn_workspace_size(dims, (int)cGraphSize, per);
    void* ws = nullptr;
    if (cudaMalloc(&ws, bytes) != cudaSuccess) throw std::runtime_error("runTsdfKNNGraph: cudaMalloc");
    int st = afx_tsdf_knn(knnIdxs, knnDists, knnCounts, cGraph, cGraphRadiuses, (int)cGraphSize, vs, size, dims, per, K,
                          ws, bytes, nullptr);
    cudaFree(ws);
    detail::afx_check(st, "runTsdfKNNGraph");
}

inline void runComputeTsdfWarpWeightsKernel(float* cKnnWeights, const float* cMotionGraphRadiuses,
                                            const uint32_t* cKnnIdxs, const float* cKnnDists, const int* cKnnCounts,
                                            const std::size_t cGridSize, int K) {
    detail::afx_check(afx_tsdf_warp_weights(cKnnWeights, cMotionGraphRadiuses, cKnnIdxs, cKnnDists, cKnnCounts,
                                            (long)cGridSize, K, nullptr),
                      "runComputeTsdfWarpWeightsKernel");
}

template <class Vec3f, class Vec3i>
inline void runGenerateTsdfVerticesKernel(float* tsdfVertices, const Vec3f cVoxelSize, const Vec3f cVolumeSize,
                                          const Vec3i cVolumeDim) {
    int dims[3];
    float vs[3], size[3];
    detail::to_i3(cVolumeDim, dims);
    detail::to_f3(cVoxelSize, vs);
    detail::to_f3(cVolumeSize, size);
    detail::afx_check(afx_tsdf_vertices(tsdfVertices, vs, size, dims, nullptr), "runGenerateTsdfVerticesKernel");
}

inline void runWarpTsdfKernel(float* tsdfVertices, const float* cMotionGraph, const uint32_t* cKnnIdxs,
                              const float* cKnnWeights, const int* cKnnCounts, std::size_t gridSize, int K) {
    detail::afx_check(afx_warp_tsdf(tsdfVertices, cMotionGraph, cKnnIdxs, cKnnWeights, cKnnCounts, (long)gridSize, K,
                                    nullptr),
                      "runWarpTsdfKernel");
}

// include/af/MarchingCubes.cuh
template <class Vec3i, class Vec3f>
inline void runMarchingCubesMeshKernel(float* mesh, unsigned int* meshSize, std::size_t meshCapacity, const float* cTsdf,
                                       const float* cTsdfWeights, const Vec3i cDims, const Vec3f& cVoxelSize,
                                       const Vec3f& cVolSize, const float cIsoValue) {
    int dims[3];
    float vs[3], size[3];
    detail::to_i3(cDims, dims);
    detail::to_f3(cVoxelSize, vs);
    detail::to_f3(cVolSize, size);
    detail::afx_check(afx_marching_cubes_points(mesh, meshSize, (long)meshCapacity, cTsdf, cTsdfWeights, dims, vs,
                                                size, cIsoValue, nullptr),
                      "runMarchingCubesMeshKernel");
}

template <class Vec3i, class Vec3f>
inline void runMarchingCubesFullKernel(float* mesh, unsigned int* meshSize, std::size_t meshCapacity, int* faces,
                                       unsigned int* facesSize, std::size_t facesCapacity, const float* cTsdf,
                                       const float* cTsdfWeights, const Vec3i cDims, const Vec3f& cVoxelSize,
                                       const Vec3f& cVolSize, const float cIsoValue) {
    int dims[3];
    float vs[3], size[3];
    detail::to_i3(cDims, dims);
    detail::to_f3(cVoxelSize, vs);
    detail::to_f3(cVolSize, size);
    detail::afx_check(afx_marching_cubes_mesh(mesh, meshSize, (long)meshCapacity, faces, facesSize,
                                              (long)facesCapacity, cTsdf, cTsdfWeights, dims, vs, size, cIsoValue,
                                              nullptr),
                      "runMarchingCubesFullKernel");
}

// include/af/ComputeCorrespondence.cuh
inline void runWarpKernel(float* warpedMesh, const float* cMesh, const float* cMotionGraph, const uint32_t* cKnnIdxs,
                          const float* cKnnWeights, const std::size_t cMeshSize, int K) {
    detail::afx_check(afx_warp(warpedMesh, cMesh, cMotionGraph, cKnnIdxs, cKnnWeights, nullptr, (long)cMeshSize, K,
                               nullptr),
                      "runWarpKernel");
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
