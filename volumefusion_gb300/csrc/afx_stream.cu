// afx_stream.cu -- the rigid multi-camera reconstruction stream (af::startMeshReconstructionStream,
// src/MeshRecontructionStream.cu:115-206), device-resident.
//
// Per frame, for every camera (CameraData::processNextFrame, :88-112): depth from uint16 mm,
// runFilterDepthKernel, the bilateral filter when enabled, and DeviceDepthImage::backProject
// (include/af/DeviceImage.cuh:54-58): runDepthToMeshKernel with the camera's intrinsics, then
// runTransformKernel with the inverse of its world-to-camera transform.  The cameras' clouds are
// concatenated in camera order (every pixel, invalid ones included).  The volume is re-initialised
// (DeviceTsdf::initDefault) and -- as the reference does -- only camera 0's filtered depth is
// integrated, at the volume's centre and rotation (DeviceTsdf::integrate ->
// runIntegrateTSDFFromFrameKernel), and the full marching-cubes mesh is extracted (untranslated).
// Nothing is read back to the host; the outputs are device views.
#include <cstring>
#include <new>

#include "afx_internal.h"

namespace afx {

struct Mat4 {
    float m[16];  // column-major
};

// transformKernel (src/VertexManipulation.cu:89-95): p <- (T * [p; 1]).head(3), in place
__global__ void transform_points_kernel(float* pts, long n, Mat4 T) {
    AFX_GRID_STRIDE(i, n) {
        float p[3] = {pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]}, q[3];
        mat4_point(T.m, p, q);
        pts[3 * i] = q[0];
        pts[3 * i + 1] = q[1];
        pts[3 * i + 2] = q[2];
    }
}

__global__ void stream_init_kernel(float* tsdf, float* weights, long S, unsigned* counts) {
    if (blockIdx.x == 0 && threadIdx.x < 2) counts[threadIdx.x] = 0;
    AFX_GRID_STRIDE(i, S) {
        tsdf[i] = -1.f;
        weights[i] = 0.f;
    }
}

}  // namespace afx

using namespace afx;

struct afx_rigid_stream {
    afx_rigid_stream_params p;
    Volume vol;
    long S = 0, P = 0;
    void* arena = nullptr;
    float* depth;    // [n_cameras * P], the filtered depth of each camera
    float* scratch;  // [P], bilateral input
    float* cloud;    // [n_cameras * P * 3]
    float* tsdf;
    float* weights;
    float* verts;    // [3 * triangle_capacity * 3]
    int* faces;      // [triangle_capacity * 3]
    unsigned* counts;  // faces, vertices
    int* error;
    float* raw;        // [P], a distorted camera's unfiltered metres
    uint32_t* umap;    // [n_cameras * P * 2], undistortion maps of the distorted cameras
};

extern "C" {

void afx_rigid_stream_default_params(afx_rigid_stream_params* p) {
    if (!p) return;
    std::memset(p, 0, sizeof(*p));
    p->n_cameras = 1;
    p->width = 640;
    p->height = 576;
    for (int c = 0; c < AFX_MAX_CAMERAS; ++c) {
        const float K[9] = {504.f, 0.f, 0.f, 0.f, 504.f, 0.f, 320.f, 288.f, 1.f};
        std::memcpy(p->K[c], K, sizeof(K));
        for (int i = 0; i < 16; ++i) p->camera_to_world[c][i] = (i % 5 == 0) ? 1.f : 0.f;
    }
    p->dims[0] = p->dims[1] = p->dims[2] = 400;  // Settings.cpp: tsdfDim
    p->volume_size[0] = p->volume_size[1] = p->volume_size[2] = 1.f;  // tsdfSize
    p->delta = 0.016f;
    for (int i = 0; i < 9; ++i) p->rotation[i] = (i % 4 == 0) ? 1.f : 0.f;
    p->depth_threshold = 1.2f;
    p->bilateral = 1;
    p->bilateral_r = 2;
    p->sigma_i = 0.03f;
    p->sigma_s = 2.f;
    p->bilateral_thr = 0.09f;
    p->triangle_capacity = 4000000;
}

int afx_rigid_stream_create(const afx_rigid_stream_params* params, afx_rigid_stream** out) {
    if (!params || !out) return AFX_ERR_INVALID_ARGUMENT;
    const afx_rigid_stream_params& p = *params;
    if (p.n_cameras < 1 || p.n_cameras > AFX_MAX_CAMERAS || p.width < 3 || p.height < 3 || p.dims[0] < 3 ||
        p.dims[1] < 3 || p.dims[2] < 3 || p.triangle_capacity < 1 || (p.bilateral && p.bilateral_r < 1))
        return AFX_ERR_INVALID_ARGUMENT;
    afx_rigid_stream* s = new (std::nothrow) afx_rigid_stream();
    if (!s) return AFX_ERR_NO_MEMORY;
    s->p = p;
    float vs[3];
    for (int c = 0; c < 3; ++c) vs[c] = p.volume_size[c] / (float)p.dims[c];  // DeviceTsdf::voxelSize
    s->vol = make_volume(p.dims, vs, p.volume_size);
    s->S = (long)p.dims[0] * p.dims[1] * p.dims[2];
    s->P = (long)p.width * p.height;
    auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
    const size_t nc = (size_t)p.n_cameras, P = (size_t)s->P, S = (size_t)s->S, T = (size_t)p.triangle_capacity;
    bool distorted = false;
    for (int c = 0; c < p.n_cameras; ++c) distorted = distorted || p.distortion[c].is_distorted;
    const size_t sizes[] = {nc * P * 4, P * 4, nc * P * 12, S * 4, S * 4, T * 36, T * 12, 64, 64,
                            distorted ? P * 4 : 0, distorted ? nc * P * 8 : 0};
    constexpr int kBuffers = (int)(sizeof(sizes) / sizeof(sizes[0]));
    size_t total = 0;
    for (size_t x : sizes) total += al(x);
    cudaError_t e = cudaMalloc(&s->arena, total);
    if (e != cudaSuccess) {
        note_cuda_error(e);
        delete s;
        return AFX_ERR_NO_MEMORY;
    }
    char* q = static_cast<char*>(s->arena);
    void* ptr[kBuffers];
    for (int i = 0; i < kBuffers; ++i) {
        ptr[i] = q;
        q += al(sizes[i]);
    }
    s->depth = (float*)ptr[0];
    s->scratch = (float*)ptr[1];
    s->cloud = (float*)ptr[2];
    s->tsdf = (float*)ptr[3];
    s->weights = (float*)ptr[4];
    s->verts = (float*)ptr[5];
    s->faces = (int*)ptr[6];
    s->counts = (unsigned*)ptr[7];
    s->error = (int*)ptr[8];
    s->raw = distorted ? (float*)ptr[9] : nullptr;
    s->umap = distorted ? (uint32_t*)ptr[10] : nullptr;
    e = cudaMemset(s->arena, 0, total);
    // each distorted camera's cv::initUndistortRectifyMap(CV_32FC1) map, built once
    // (src/MeshRecontructionStream.cu:97-98 rebuilds the same map every frame)
    int map_rc = AFX_OK;
    for (int c = 0; c < p.n_cameras && e == cudaSuccess && !map_rc; ++c)
        if (p.distortion[c].is_distorted)
            map_rc = undistort_map_impl(s->umap + (size_t)c * P * 2, p.width, p.height, p.K[c], &p.distortion[c],
                                        AFX_UNDISTORT_NEAREST, nullptr);
    if (e == cudaSuccess && !map_rc) e = cudaStreamSynchronize(nullptr);
    if (map_rc) {
        cudaFree(s->arena);
        delete s;
        return map_rc;
    }
    if (e != cudaSuccess) {
        cudaFree(s->arena);
        delete s;
        return note_cuda_error(e);
    }
    *out = s;
    return AFX_OK;
}

int afx_rigid_stream_destroy(afx_rigid_stream* s) {
    if (!s) return AFX_ERR_INVALID_ARGUMENT;
    cudaDeviceSynchronize();
    const cudaError_t e = cudaFree(s->arena);
    delete s;
    return note_cuda_error(e);
}

int afx_rigid_stream_process(afx_rigid_stream* s, const uint16_t* const* depth_mm, void* stream) {
    if (!s || !depth_mm) return AFX_ERR_INVALID_ARGUMENT;
    const afx_rigid_stream_params& p = s->p;
    for (int c = 0; c < p.n_cameras; ++c)
        if (!depth_mm[c]) return AFX_ERR_INVALID_ARGUMENT;
    cudaStream_t st = as_stream(stream);
    const long P = s->P;
    for (int c = 0; c < p.n_cameras; ++c) {
        float* d = s->depth + c * P;
        float* in = p.bilateral ? s->scratch : d;
        int rc;
        if (p.distortion[c].is_distorted) {
            // the filtered device frame is overwritten by the host frame's undistortion: the unfiltered
            // metres remapped (src/MeshRecontructionStream.cu:91-101)
            rc = afx_depth_from_mm(s->raw, depth_mm[c], P, st);
            if (!rc) rc = undistort_apply_impl(in, s->raw, p.width, p.height, s->umap + (size_t)c * P * 2,
                                               AFX_UNDISTORT_NEAREST, st);
        } else {
            rc = afx_depth_from_mm(in, depth_mm[c], P, st);
            if (!rc) rc = afx_filter_depth(in, P, p.depth_threshold, st);
        }
        if (!rc && p.bilateral)
            rc = afx_bilateral_filter(d, in, p.height, p.width, p.bilateral_r, p.sigma_i, p.sigma_s, p.bilateral_thr, st);
        float* cloud = s->cloud + 3 * c * P;
        if (!rc) rc = afx_depth_to_mesh(cloud, d, p.width, p.height, p.K[c], st);
        if (rc) return rc;
        Mat4 T;
        std::memcpy(T.m, p.camera_to_world[c], sizeof(T.m));
        transform_points_kernel<<<grid_for(P, 256), 256, 0, st>>>(cloud, P, T);
        AFX_LAUNCH_CHECK();
    }
    // DeviceTsdf::initDefault + integrate(cameras[0]): one write-only pass where the layout allows
    AFX_CUDA(cudaMemsetAsync(s->counts, 0, 8, st));
    int rc = integrate_fresh_impl(s->tsdf, s->weights, s->depth, p.width, p.height, p.delta, s->vol, p.rotation,
                                  p.center, p.K[0], st);
    if (rc == AFX_ERR_UNSUPPORTED) {
        stream_init_kernel<<<grid_for(s->S, 256), 256, 0, st>>>(s->tsdf, s->weights, s->S, s->counts);
        AFX_LAUNCH_CHECK();
        rc = integrate_rigid_impl(s->tsdf, s->weights, kVoxF32, s->depth, p.width, p.height, p.delta, s->vol,
                                  p.rotation, p.center, p.K[0], st);
    }
    if (rc) return rc;
    const long T = p.triangle_capacity;
    rc = mc_fused_impl(s->tsdf, s->weights, kVoxF32, s->vol, 0.f, nullptr, nullptr, 0, s->verts, s->counts + 1, T * 3,
                       s->faces, s->counts, T, st, s->error);
    return rc;
}

int afx_rigid_stream_outputs(afx_rigid_stream* s, float** cloud, long* cloud_points, float** vertices,
                             unsigned** vertex_count, int** faces, unsigned** face_count, float** tsdf, float** weights) {
    if (!s) return AFX_ERR_INVALID_ARGUMENT;
    if (cloud) *cloud = s->cloud;
    if (cloud_points) *cloud_points = s->P * s->p.n_cameras;
    if (vertices) *vertices = s->verts;
    if (vertex_count) *vertex_count = s->counts + 1;
    if (faces) *faces = s->faces;
    if (face_count) *face_count = s->counts;
    if (tsdf) *tsdf = s->tsdf;
    if (weights) *weights = s->weights;
    return AFX_OK;
}

}  // extern "C"
