// afx_common.cuh -- shared device helpers for the sm_103a fusion kernels.
//
// Floating point: the library is compiled with -fmad=false, so every binary32 product
// and sum below is rounded separately, in the order written, which is the order the
// reference's Eigen expressions evaluate in (3-term dots / norms a0+(a1+a2), Mat4*[p;1]
// rows ((a0+a1)+a2)+a3).  Fused multiply-adds appear only where written explicitly.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/afx/afx.h"

#define AFX_HD __host__ __device__ __forceinline__
#define AFX_D __device__ __forceinline__

namespace afx {

// Device-side error flags, OR-ed into a session's error word.
enum : int {
    ERRF_CAPACITY = 1,
    ERRF_TIMEOUT = 2,
    ERRF_SINGULAR = 4,
    ERRF_UNSUPPORTED = 8,
    ERRF_TMA = 16,
    ERRF_INDEX = 32,  // an index failed a bounds check; the access was skipped
};

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

int note_cuda_error(cudaError_t e);  // records e for afx_last_cuda_error; returns AFX_ERR_CUDA or AFX_OK
void count_launch();                  // kernel launch accounting for the session statistics
long launches_total();

#define AFX_LAUNCH_CHECK()                                                  \
    do {                                                                    \
        ::afx::count_launch();                                              \
        cudaError_t _e = cudaGetLastError();                                \
        if (_e != cudaSuccess) return ::afx::note_cuda_error(_e);           \
    } while (0)

#define AFX_CUDA(call)                                                      \
    do {                                                                    \
        cudaError_t _e = (call);                                            \
        if (_e != cudaSuccess) return ::afx::note_cuda_error(_e);           \
    } while (0)

inline unsigned blocks_for(long n, int threads) {
    long b = (n + threads - 1) / threads;
    return (unsigned)(b < 1 ? 1 : b);
}

// Grid for a grid-stride kernel over at most n items whose live count is read on the device:
// enough blocks to cover n, capped at kStrideBlocks so that a large capacity with few live
// items costs one short wave of immediately-exiting blocks, not one block per 256 slots.  Two
// blocks per SM cover 78k live items in one pass; the cap is low because a block that only
// reads the count and exits still costs the GPU its dispatch: with many sessions' frames in
// flight, kernels of 1216 such blocks ran at 1.1M kernels/s, of 152 blocks at 4.0M kernels/s.
constexpr long kStrideBlocks = 304;  // 2 blocks per SM on 152 SMs
inline unsigned grid_for(long n, int threads) {
    long b = (n + threads - 1) / threads;
    return (unsigned)(b < 1 ? 1 : (b > kStrideBlocks ? kStrideBlocks : b));
}
// The same for kernels with a long loop per item (one graph node per warp or block): up to 8
// blocks per SM, so that graphs of thousands of nodes still spread over every SM.
constexpr long kNodeBlocks = 1216;
inline unsigned grid_for_nodes(long n, int per_block) {
    long b = (n + per_block - 1) / per_block;
    return (unsigned)(b < 1 ? 1 : (b > kNodeBlocks ? kNodeBlocks : b));
}

// for (i in [start, n)) over the whole grid
#define AFX_GRID_STRIDE(i, n) \
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < (n); i += (long)gridDim.x * blockDim.x)

// ---- Eigen-order small vector arithmetic ----
AFX_HD float dot3(const float* a, const float* b) { return a[0] * b[0] + (a[1] * b[1] + a[2] * b[2]); }
AFX_HD float sqnorm3(const float* a) { return a[0] * a[0] + (a[1] * a[1] + a[2] * a[2]); }
AFX_D float norm3(const float* a) { return sqrtf(sqnorm3(a)); }
// Mat3f (column-major) * Vec3f
AFX_HD void mat3_vec3(const float* R, const float* p, float* o) {
#pragma unroll
    for (int i = 0; i < 3; ++i) o[i] = R[i] * p[0] + (R[3 + i] * p[1] + R[6 + i] * p[2]);
}
// (Mat4f (column-major) * [p;1]).head(3)
AFX_HD void mat4_point(const float* T, const float* p, float* o) {
#pragma unroll
    for (int i = 0; i < 3; ++i) o[i] = ((T[i] * p[0] + T[4 + i] * p[1]) + T[8 + i] * p[2]) + T[12 + i];
}
// nanoflann L2_Simple_Adaptor::evalMetric order: ((0 + d0^2) + d1^2) + d2^2
AFX_HD float l2sq_nanoflann(const float* q, const float* p) {
    float d0 = q[0] - p[0], d1 = q[1] - p[1], d2 = q[2] - p[2];
    return (d0 * d0 + d1 * d1) + d2 * d2;
}

// float -> int with truncation toward zero, saturating, NaN -> 0 (static_cast<int> on the GPU)
AFX_D int f2i(float x) { return __float2int_rz(x); }

// voxelToWorld (src/TSDFIntegration.cu:6-8): v * voxelSize - size/2
AFX_HD void voxel_to_world(int x, int y, int z, const float* vs, const float* half, float* o) {
    o[0] = (float)x * vs[0] - half[0];
    o[1] = (float)y * vs[1] - half[1];
    o[2] = (float)z * vs[2] - half[2];
}

// worldToVoxel (src/TSDFIntegration.cu:10-14) with inv = (float)(1.0 / (double)voxelSize) from the host
AFX_D void world_to_voxel(const float* p, const float* inv, const float* half, int* v) {
#pragma unroll
    for (int c = 0; c < 3; ++c) v[c] = f2i((p[c] + half[c]) * inv[c]);
}

// Own exp: Cody-Waite reduction x = k ln2 + r with ln2 split into a 16-bit head and a
// tail, degree-7 Taylor polynomial for e^r by Horner with fused multiply-adds, then 2^k
// applied in two exact power-of-two steps.  Faithfully rounded (<= 1 ulp); the CPU
// oracle evaluates the identical operation sequence.
AFX_D float afx_expf(float x) {
    if (x != x) return x;
    if (x > 88.7228394f) return __int_as_float(0x7f800000);
    if (x < -103.972084f) return 0.0f;
    const float log2e = (float)1.4426950408889634;
    const float ln2_hi = 0.693145751953125f;
    const float ln2_lo = (float)(0.6931471805599453 - 0.693145751953125);
    float kf = rintf(x * log2e);
    float r = __fmaf_rn(-kf, ln2_hi, x);
    r = __fmaf_rn(-kf, ln2_lo, r);
    float p = (float)(1.0 / 5040.0);
    p = __fmaf_rn(p, r, (float)(1.0 / 720.0));
    p = __fmaf_rn(p, r, (float)(1.0 / 120.0));
    p = __fmaf_rn(p, r, (float)(1.0 / 24.0));
    p = __fmaf_rn(p, r, (float)(1.0 / 6.0));
    p = __fmaf_rn(p, r, 0.5f);
    p = __fmaf_rn(p, r, 1.0f);
    p = __fmaf_rn(p, r, 1.0f);
    int k = (int)kf;
    int k1 = k / 2, k2 = k - k1;
    float s1 = __int_as_float((k1 + 127) << 23);
    float s2 = __int_as_float((k2 + 127) << 23);
    return (p * s1) * s2;
}

// Geometry of a dense volume as the kernels need it.
struct Volume {
    int dims[3];
    float vs[3];    // voxel size = size / dims
    float half[3];  // size * 0.5f
    float inv[3];   // (float)(1.0 / (double)vs)
};

Volume make_volume(const int dims[3], const float voxel_size[3], const float volume_size[3]);

struct Intrinsics {
    float fx, fy, cx, cy;
};
inline Intrinsics make_intrinsics(const float* K) { return Intrinsics{K[0], K[4], K[6], K[7]}; }

// updateTsdf (src/TSDFIntegration.cu:16-67)
AFX_D bool tsdf_update_value(const float* p, const float* depth, int W, int H, float delta, const Intrinsics& K,
                             float* tnew) {
    if (p[2] < 1.e-4f) return false;
    float zInv = 1.0f / p[2];
    float uf = (K.fx * p[0]) * zInv + K.cx;
    float vf = (K.fy * p[1]) * zInv + K.cy;
    int u = f2i(uf + 0.5f);
    int v = f2i(vf + 0.5f);
    if (u < 0 || u >= W || v < 0 || v >= H) return false;
    float D = __ldg(depth + (long)v * W + u);
    if (isinf(D) || D < 1.e-4f) return false;
    float sdf = p[2] - D;
    if (sdf > delta) return false;
    if (sdf < -delta) {  // behind the truncation band: no division (most voxels that update)
        *tnew = -1.0f;
        return true;
    }
    *tnew = sdf / delta;
    return true;
}

AFX_D void tsdf_blend(float& t, float& w, float tnew) {
    const float wnew = 1.0f;
    float told = t, wold = w;
    t = (told * wold + tnew * wnew) / (wold + wnew);
    w = fminf(wold + wnew, 15.0f);
}

// Warp reductions
template <typename T>
AFX_D T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Bounded spin on a device flag / counter; returns false on timeout.
AFX_D bool spin_until_geq(volatile unsigned* p, unsigned target, long max_iter) {
    for (long i = 0; i < max_iter; ++i) {
        if (*p >= target) return true;
        __nanosleep(64);
    }
    return false;
}

}  // namespace afx
