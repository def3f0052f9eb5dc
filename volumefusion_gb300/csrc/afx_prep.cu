// afx_prep.cu -- depth pre-processing: mm -> metres, range filter, bilateral filter,
// back-projection, normals with angle exclusion, removal of pixels without a normal and
// the frame centroid.  The reference runs these as six launches with a blocking sync
// after each (src/VolumeFusion.cu:184-220); here one kernel does all of it per 32x16
// tile, with the uint16 input tile (plus halo) staged into shared memory by TMA.
#include <cuda.h>

#include <cmath>
#include <cstring>
#include <mutex>

#include "afx_common.cuh"
#include "afx_host.h"
#include "afx_tma.h"
#include "afx_undistort.cuh"

namespace afx {

constexpr int kMaxBilateralR = 7;

struct BilateralTables {
    int r;
    float norm_factor;  // (float)(30 / (3 * sigma_i))
    float thr;
    int clr[31];
    float g2d[(2 * kMaxBilateralR + 1) * (2 * kMaxBilateralR + 1)];
};

// updateGaussian16 (src/BilateralFilter.cu:12-50), evaluated on the host as the reference does.
static void make_bilateral_tables(int r, double sI, double sS, float thr, BilateralTables* t) {
    std::memset(t, 0, sizeof(*t));
    t->r = r;
    t->thr = thr;
    t->norm_factor = (float)(30 / (3 * sI));
    float g[2 * kMaxBilateralR + 1];
    for (int i = 0; i < 2 * r + 1; i++) {
        float x = (float)(i - r);
        g[i] = expf((float)((double)(-(x * x)) / (2 * sS * sS)));
    }
    int index = 0;
    for (int dy = -r; dy <= r; dy++)
        for (int dx = -r; dx <= r; dx++) t->g2d[index++] = g[dy + r] * g[dx + r];
    float fc[31];
    for (int i = 0; i <= 30; i++) fc[i] = (float)std::exp(-(std::pow(i / 10.0, 2)) / (2));
    for (int i = 0; i <= 30; i++) t->clr[i] = (int)(fc[i] / fc[30]);
}

// Normal exclusion test of depthVerticesNormalsKernel (src/VertexManipulation.cu:191-199):
// invalid <=> (float)acos(n.z) in (lo, hi).  acos is monotone, so the test becomes
// t_hi < n.z < t_lo with thresholds found here by bisection over binary32 values.
struct AngleThresholds {
    float d_lo;  // smallest d in [-1,1] with (float)acos(d) <= lo  (invalid needs d < d_lo)
    float d_hi;  // largest d in [-1,1] with (float)acos(d) >= hi   (invalid needs d > d_hi)
};

static inline int f_ord(float f) {
    int i;
    std::memcpy(&i, &f, 4);
    return i < 0 ? (int)(0x80000000u - (unsigned)i) : i;
}
static inline float ord_f(int o) {
    int i = o < 0 ? (int)(0x80000000u - (unsigned)o) : o;
    float f;
    std::memcpy(&f, &i, 4);
    return f;
}
static inline float acos_f(float d) { return (float)std::acos((double)d); }

static AngleThresholds make_angle_thresholds(float lo, float hi) {
    AngleThresholds t;
    const int a = f_ord(-1.0f), b = f_ord(1.0f);
    // smallest d with acos_f(d) <= lo (predicate monotone false..true over increasing d)
    if (!(acos_f(1.0f) <= lo)) {
        t.d_lo = -2.0f;  // no d qualifies: "d < d_lo" never holds in [-1, 1]
    } else {
        int L = a, R = b;
        while (L < R) {
            int mid = L + (R - L) / 2;
            if (acos_f(ord_f(mid)) <= lo) R = mid;
            else L = mid + 1;
        }
        t.d_lo = ord_f(L);
    }
    // largest d with acos_f(d) >= hi (predicate monotone true..false)
    if (!(acos_f(-1.0f) >= hi)) {
        t.d_hi = 2.0f;  // "d > d_hi" never holds in [-1, 1]
    } else {
        int L = a, R = b;
        while (L < R) {
            int mid = L + (R - L + 1) / 2;
            if (acos_f(ord_f(mid)) >= hi) L = mid;
            else R = mid - 1;
        }
        t.d_hi = ord_f(L);
    }
    return t;
}

AFX_D bool normal_angle_excluded(float dz, const AngleThresholds& t) {
    return dz >= -1.0f && dz <= 1.0f && dz > t.d_hi && dz < t.d_lo;
}

// Normal at interior pixel from its four neighbours (src/VertexManipulation.cu:160-206).
AFX_D void pixel_normal(const float* c, const float* xl, const float* xr, const float* yt, const float* yb,
                        const AngleThresholds& at, float* n) {
    n[0] = n[1] = n[2] = 0.f;
    if (c[2] < 1.e-4f) return;
    if (xr[2] < 1.e-4f || xl[2] < 1.e-4f || yb[2] < 1.e-4f || yt[2] < 1.e-4f) return;
    float dX[3] = {xr[0] - xl[0], xr[1] - xl[1], xr[2] - xl[2]};
    float dY[3] = {yb[0] - yt[0], yb[1] - yt[1], yb[2] - yt[2]};
    float nx = sqrtf(dX[0] * dX[0] + dX[1] * dX[1]);
    float ny = sqrtf(dY[0] * dY[0] + dY[1] * dY[1]);
    float gX[3] = {dX[0] / nx, dX[1] / nx, dX[2] / nx};
    float gY[3] = {dY[0] / ny, dY[1] / ny, dY[2] / ny};
    float cr[3] = {gY[1] * gX[2] - gY[2] * gX[1], gY[2] * gX[0] - gY[0] * gX[2], gY[0] * gX[1] - gY[1] * gX[0]};
    float s = sqnorm3(cr);
    if (s > 0.f) {
        float q = sqrtf(s);
        cr[0] = cr[0] / q;
        cr[1] = cr[1] / q;
        cr[2] = cr[2] / q;
    }
    float dot = 0.f * cr[0] + (0.f * cr[1] + 1.f * cr[2]);
    if (normal_angle_excluded(dot, at)) return;
    n[0] = cr[0];
    n[1] = cr[1];
    n[2] = cr[2];
}

AFX_D bool normal_is_zero(const float* n) {
    return fabsf(n[0]) <= 1.e-4f && fabsf(n[1]) <= 1.e-4f && fabsf(n[2]) <= 1.e-4f;
}

AFX_D float filter_value(float v, float thr) { return (v > thr || v < 1.e-4f || isnan(v)) ? __int_as_float(0x7f800000) : v; }

// Bilateral response at (x, y) reading a clamped window through `at(xx, yy)`
// (gpuFilterTextureOpmShared, src/BilateralFilter.cu:92-126: a (x offset) outer, b inner).
template <typename At>
AFX_D float bilateral_at(int x, int y, int w, int h, const BilateralTables& T, At at) {
    float centre = at(x, y);
    if (isinf(centre)) return centre;
    const int r = T.r, kd = 2 * r + 1;
    float iF = 0.f, wP = 0.f;
    int ig = 0;
    for (int a = 0; a < kd; ++a) {
        int xx = min(max(x + a - r, 0), w - 1);
        for (int b = 0; b < kd; ++b, ++ig) {
            int yy = min(max(y + b - r, 0), h - 1);
            float cur = at(xx, yy);
            if (isinf(cur)) continue;
            float diff = fabsf(centre - cur);
            if (diff > T.thr) continue;
            int x0 = f2i(fabsf(diff * T.norm_factor));
            if (x0 > 30 || x0 < 0) x0 = 30;
            float wt = T.g2d[ig] * (float)T.clr[x0];
            iF = iF + cur * wt;
            wP = wP + wt;
        }
    }
    return iF / wP;
}

// ------------------------------------------------------------------------------------
// Fused frame preparation
// ------------------------------------------------------------------------------------

constexpr int kTW = 32, kTH = 16;       // output tile
constexpr int kHalo = kMaxBilateralR + 1;
constexpr int kInW = kTW + 2 * ((kHalo + 7) / 8) * 8, kInH = kTH + 2 * kHalo;

struct PrepArgs {
    int width, height;
    Intrinsics K;
    float fxi, fyi;         // 1.0f / fx, 1.0f / fy
    float depth_threshold;
    int bilateral;
    int halo;               // r + 1 (rows above/below the tile held in shared memory)
    int xhalo;              // halo rounded up to 8 columns
    BilateralTables tab;
    AngleThresholds ang;
    float* depth;
    float* vertices;
    float* normals;
    unsigned long long* acc;  // 3 fixed-point sums + count
    int* error;
    const uint32_t* umap;     // cv::undistort map (kSrc == kSrcUndistort)
};

// Where the tile's depth comes from: plain loads of the uint16 frame, one TMA tile copy of it, or
// bilinear samples of its metres through an undistortion map (cv::undistort before the filter,
// src/VolumeFusion.cu:162-190).
constexpr int kSrcLoad = 0, kSrcTma = 1, kSrcUndistort = 2;

AFX_D uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

template <int kSrc>
__global__ void __launch_bounds__(kTW * kTH) prep_kernel(const __grid_constant__ CUtensorMap tmap,
                                                         const uint16_t* __restrict__ mm, PrepArgs A) {
    __shared__ alignas(128) uint16_t raw[kInH * kInW];
    __shared__ float dep[kInH * kInW];
    __shared__ float bil[(kTH + 2) * (kTW + 2)];
    __shared__ float ver[(kTH + 2) * (kTW + 2) * 3];
    __shared__ alignas(8) unsigned long long mbar;
    __shared__ long long red[4][kTW * kTH / 32];

    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * kTW + tx;
    const int x0 = blockIdx.x * kTW, y0 = blockIdx.y * kTH;
    const int W = A.width, H = A.height;
    const int inW = kTW + 2 * A.xhalo, inH = kTH + 2 * A.halo;
    const int gx0 = x0 - A.xhalo, gy0 = y0 - A.halo;  // global coordinates of raw[0][0]

    if (kSrc == kSrcTma) {
        if (tid == 0) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar)));
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        }
        __syncthreads();
        if (tid == 0) {
            const unsigned bytes = (unsigned)(inW * inH * sizeof(uint16_t));
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(&mbar)), "r"(bytes)
                         : "memory");
            asm volatile(
                "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
                "[%4];" ::"r"(smem_u32(raw)),
                "l"(&tmap), "r"(gx0), "r"(gy0), "r"(smem_u32(&mbar))
                : "memory");
        }
        // bounded wait for the tile (phase 0); the give-up decision is uniform across the CTA
        bool done = false;
        for (int it = 0; it < (1 << 22) && !done; ++it) {
            uint32_t ok;
            asm volatile(
                "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0; selp.u32 %0, 1, 0, p; }"
                : "=r"(ok)
                : "r"(smem_u32(&mbar))
                : "memory");
            done = ok != 0;
        }
        if (__syncthreads_or(!done)) {
            if (tid == 0) atomicOr(A.error, ERRF_TMA | ERRF_TIMEOUT);
            // the copy may still land: wait for it (bounded) before the CTA's shared memory goes
            for (int it = 0; it < (1 << 22); ++it) {
                uint32_t ok;
                asm volatile(
                    "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0; selp.u32 %0, 1, 0, p; }"
                    : "=r"(ok)
                    : "r"(smem_u32(&mbar))
                    : "memory");
                if (ok) break;
            }
            return;
        }
    } else if (kSrc == kSrcLoad) {
        for (int i = tid; i < inW * inH; i += kTW * kTH) {
            int gx = gx0 + i % inW, gy = gy0 + i / inW;
            raw[i] = (gx >= 0 && gx < W && gy >= 0 && gy < H) ? mm[(long)gy * W + gx] : (uint16_t)0;
        }
    }
    if (kSrc == kSrcUndistort) {
        // metres (src/dataset.cpp:188), cv::undistort (src/VolumeFusion.cu:179), range filter
        auto metres = [&](int x, int y) { return (float)mm[(long)y * W + x] * 0.001f; };
        for (int i = tid; i < inW * inH; i += kTW * kTH) {
            int gx = gx0 + i % inW, gy = gy0 + i / inW;
            float v = 0.f;
            if (gx >= 0 && gx < W && gy >= 0 && gy < H) {
                const long p = (long)gy * W + gx;
                v = remap_linear_at(A.umap[2 * p], A.umap[2 * p + 1], W, H, metres);
            }
            dep[i] = filter_value(v, A.depth_threshold);
        }
    } else {
        __syncthreads();
        // metres + range filter (src/dataset.cpp:188, src/VertexManipulation.cu:6-15)
        for (int i = tid; i < inW * inH; i += kTW * kTH) dep[i] = filter_value((float)raw[i] * 0.001f, A.depth_threshold);
    }
    __syncthreads();
    auto at_dep = [&](int gx, int gy) -> float { return dep[(gy - gy0) * inW + (gx - gx0)]; };
    // bilateral filter on the tile plus a one-pixel ring
    const int bw = kTW + 2;
    for (int i = tid; i < (kTH + 2) * bw; i += kTW * kTH) {
        int gx = x0 - 1 + i % bw, gy = y0 - 1 + i / bw;
        float v = __int_as_float(0x7f800000);
        if (gx >= 0 && gx < W && gy >= 0 && gy < H)
            v = A.bilateral ? bilateral_at(gx, gy, W, H, A.tab, at_dep) : at_dep(gx, gy);
        bil[i] = v;
        // back-projection (src/VertexManipulation.cu:43-63)
        float* o = ver + 3 * i;
        if (isinf(v) || v < 1.e-4f) {
            o[0] = o[1] = o[2] = 0.f;
        } else {
            float xr = ((float)gx - A.K.cx) * A.fxi;
            float yr = ((float)gy - A.K.cy) * A.fyi;
            o[0] = xr * v;
            o[1] = yr * v;
            o[2] = v;
        }
    }
    __syncthreads();
    const int gx = x0 + tx, gy = y0 + ty;
    long long s0 = 0, s1 = 0, s2 = 0, cnt = 0;
    if (gx < W && gy < H) {
        const int li = (ty + 1) * bw + (tx + 1);
        const float* c = ver + 3 * li;
        float n[3] = {0.f, 0.f, 0.f};
        float d = bil[li];
        float v[3] = {c[0], c[1], c[2]};
        if (gx >= 1 && gx < W - 1 && gy >= 1 && gy < H - 1) {
            pixel_normal(c, ver + 3 * (li - 1), ver + 3 * (li + 1), ver + 3 * (li - bw), ver + 3 * (li + bw), A.ang, n);
            if (normal_is_zero(n)) {  // removeDepthWithoutNormalsKernel (src/VertexManipulation.cu:223-236)
                v[0] = v[1] = v[2] = 0.f;
                d = __int_as_float(0x7f800000);
            }
        }
        const long p = (long)gy * W + gx;
        A.depth[p] = d;
        float* vo = A.vertices + 3 * p;
        float* no = A.normals + 3 * p;
        vo[0] = v[0]; vo[1] = v[1]; vo[2] = v[2];
        no[0] = n[0]; no[1] = n[1]; no[2] = n[2];
        // v * 2^32 is exact in binary32 (a power-of-two scaling of a finite coordinate), so rounding
        // it to an integer from binary32 gives the binary64 path's value without the FP64 pipe
        s0 = __float2ll_rn(v[0] * 4294967296.0f);
        s1 = __float2ll_rn(v[1] * 4294967296.0f);
        s2 = __float2ll_rn(v[2] * 4294967296.0f);
        cnt = v[2] > 1.e-4f ? 1 : 0;
    }
    s0 = warp_sum(s0);
    s1 = warp_sum(s1);
    s2 = warp_sum(s2);
    cnt = warp_sum(cnt);
    const int wid = tid / 32, lane = tid % 32;
    if (lane == 0) {
        red[0][wid] = s0;
        red[1][wid] = s1;
        red[2][wid] = s2;
        red[3][wid] = cnt;
    }
    __syncthreads();
    if (tid < 4) {
        long long s = 0;
        for (int i = 0; i < kTW * kTH / 32; ++i) s += red[tid][i];
        if (s != 0) atomicAdd(A.acc + tid, (unsigned long long)s);
    }
}

__global__ void centroid_finalize_kernel(unsigned long long* acc, float* centroid) {
    long long cnt = (long long)acc[3];
    for (int c = 0; c < 3; ++c) {
        long long s = (long long)acc[c];
        centroid[c] = (float)(((double)s / 4294967296.0) / (double)cnt);
        acc[c] = 0;
    }
    acc[3] = 0;
}

// ---- separate stage kernels (API parity with the reference's individual launches) ----

__global__ void mm_to_m_kernel(float* d, const uint16_t* mm, long n) {
    long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (i < n) d[i] = (float)mm[i] * 0.001f;
}

__global__ void filter_depth_kernel(float* d, long n, float thr) {
    long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (i < n) d[i] = filter_value(d[i], thr);
}

// filterDepthKernel with the caller's fill value (src/VertexManipulation.cu:6-15).
__global__ void filter_depth_fill_kernel(float* d, long n, float thr, float fill) {
    long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (i < n) {
        const float v = d[i];
        if (v > thr || v < 1.e-4f || isnan(v)) d[i] = fill;
    }
}

__global__ void fill_f32_kernel(float* d, long n, float value) {
    AFX_GRID_STRIDE(i, n) d[i] = value;
}

__global__ void bilateral_kernel(float* out, const float* __restrict__ in, int h, int w, BilateralTables T) {
    int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= w || y >= h) return;
    auto at = [&](int xx, int yy) -> float { return __ldg(in + (long)yy * w + xx); };
    out[(long)y * w + x] = bilateral_at(x, y, w, h, T, at);
}

__global__ void depth_to_mesh_kernel(float* mesh, const float* depth, int w, int h, Intrinsics K, float fxi,
                                     float fyi) {
    int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= w || y >= h) return;
    long id = (long)y * w + x;
    float d = depth[id];
    float* o = mesh + 3 * id;
    if (isinf(d) || d < 1.e-4f) {
        o[0] = o[1] = o[2] = 0.f;
        return;
    }
    float xr = ((float)x - K.cx) * fxi, yr = ((float)y - K.cy) * fyi;
    o[0] = xr * d;
    o[1] = yr * d;
    o[2] = d;
}

__global__ void normals_kernel(float* normals, const float* V, int h, int w, AngleThresholds at) {
    int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= w || y >= h) return;
    long id = (long)y * w + x;
    float n[3] = {0.f, 0.f, 0.f};
    if (x >= 1 && x < w - 1 && y >= 1 && y < h - 1)
        pixel_normal(V + 3 * id, V + 3 * (id - 1), V + 3 * (id + 1), V + 3 * (id - w), V + 3 * (id + w), at, n);
    normals[3 * id] = n[0];
    normals[3 * id + 1] = n[1];
    normals[3 * id + 2] = n[2];
}

__global__ void remove_without_normals_kernel(const float* normals, float* V, float* depth, int h, int w) {
    int x = blockIdx.x * blockDim.x + threadIdx.x + 1, y = blockIdx.y * blockDim.y + threadIdx.y + 1;
    if (x >= w - 1 || y >= h - 1) return;
    long id = (long)y * w + x;
    if (normal_is_zero(normals + 3 * id)) {
        V[3 * id] = V[3 * id + 1] = V[3 * id + 2] = 0.f;
        depth[id] = __int_as_float(0x7f800000);
    }
}

// ---- TMA descriptor ----

EncodeTiledFn encode_fn() {
    static EncodeTiledFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
        else
            cudaGetLastError();
    });
    return fn;
}

// 2-D tiled map over a uint16 image; the box is the input tile with its halo.
static bool make_u16_tile_map(CUtensorMap* map, const uint16_t* base, int width, int height, int box_w, int box_h) {
    if (width % 8 != 0 || (reinterpret_cast<uintptr_t>(base) & 15) != 0) return false;
    EncodeTiledFn fn = encode_fn();
    if (!fn) return false;
    cuuint64_t dims[2] = {(cuuint64_t)width, (cuuint64_t)height};
    cuuint64_t strides[1] = {(cuuint64_t)width * sizeof(uint16_t)};
    cuuint32_t box[2] = {(cuuint32_t)box_w, (cuuint32_t)box_h};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_UINT16, 2, const_cast<uint16_t*>(base), dims, strides, box, estr,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_NONE,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
}

// Scratch of the stand-alone afx_frame_prep: centroid accumulators (zero between calls: the
// finalising kernel clears them) and the error word.  One per host thread and device, allocated
// on the thread's first call and kept for the life of the process, so calls from different host
// threads never share it; calls from one thread on different streams must not overlap.
struct PrepScratch {
    unsigned long long acc[4];
    int error;
};

static PrepScratch* prep_scratch() {
    thread_local PrepScratch* s[kMaxDevices] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return nullptr;
    if (!s[dev]) {
        PrepScratch* p = nullptr;
        if (cudaMalloc(&p, sizeof(PrepScratch)) != cudaSuccess) return nullptr;
        if (cudaMemset(p, 0, sizeof(PrepScratch)) != cudaSuccess) {
            cudaFree(p);
            return nullptr;
        }
        s[dev] = p;
    }
    return s[dev];
}

int frame_prep_impl(const uint16_t* mm, int width, int height, const afx_prep_params* p, float* depth, float* vertices,
                    float* normals, float* centroid, unsigned long long* acc, int* error, cudaStream_t st,
                    const uint32_t* undistort_map) {
    if (!mm || !p || !depth || !vertices || !normals || width < 3 || height < 3) return AFX_ERR_INVALID_ARGUMENT;
    if (p->bilateral && (p->bilateral_r < 0 || p->bilateral_r > kMaxBilateralR)) return AFX_ERR_UNSUPPORTED;
    PrepArgs A;
    A.width = width;
    A.height = height;
    A.K = make_intrinsics(p->K);
    A.fxi = 1.0f / p->K[0];
    A.fyi = 1.0f / p->K[4];
    A.depth_threshold = p->depth_threshold;
    A.bilateral = p->bilateral;
    int r = p->bilateral ? p->bilateral_r : 0;
    A.halo = r + 1;
    A.xhalo = ((A.halo + 7) / 8) * 8;
    make_bilateral_tables(r, (double)p->sigma_i, (double)p->sigma_s, p->bilateral_thr, &A.tab);
    A.ang = make_angle_thresholds(p->excl_angle_lo, p->excl_angle_hi);
    A.depth = depth;
    A.vertices = vertices;
    A.normals = normals;
    A.acc = acc;
    A.error = error;
    A.umap = undistort_map;
    CUtensorMap map;
    std::memset(&map, 0, sizeof(map));
    const int inW = kTW + 2 * A.xhalo, inH = kTH + 2 * A.halo;
    dim3 grid((width + kTW - 1) / kTW, (height + kTH - 1) / kTH), block(kTW, kTH);
    if (undistort_map)
        prep_kernel<kSrcUndistort><<<grid, block, 0, st>>>(map, mm, A);
    else if (make_u16_tile_map(&map, mm, width, height, inW, inH))
        prep_kernel<kSrcTma><<<grid, block, 0, st>>>(map, mm, A);
    else
        prep_kernel<kSrcLoad><<<grid, block, 0, st>>>(map, mm, A);
    AFX_LAUNCH_CHECK();
    if (centroid) {
        centroid_finalize_kernel<<<1, 1, 0, st>>>(acc, centroid);
        AFX_LAUNCH_CHECK();
    }
    return AFX_OK;
}

}  // namespace afx

using namespace afx;

extern "C" {

int afx_depth_from_mm(float* depth, const uint16_t* mm, long n, void* stream) {
    if (!depth || !mm || n < 0) return AFX_ERR_INVALID_ARGUMENT;
    if (n == 0) return AFX_OK;
    mm_to_m_kernel<<<blocks_for(n, 256), 256, 0, as_stream(stream)>>>(depth, mm, n);
    AFX_LAUNCH_CHECK();
    return AFX_OK;
}

int afx_filter_depth(float* depth, long n, float threshold, void* stream) {
    if (!depth || n < 0) return AFX_ERR_INVALID_ARGUMENT;
    if (n == 0) return AFX_OK;
    filter_depth_kernel<<<blocks_for(n, 256), 256, 0, as_stream(stream)>>>(depth, n, threshold);
    AFX_LAUNCH_CHECK();
    return AFX_OK;
}

int afx_filter_depth_fill(float* depth, long n, float threshold, float fill, void* stream) {
    if (!depth || n < 0) return AFX_ERR_INVALID_ARGUMENT;
    if (n == 0) return AFX_OK;
    filter_depth_fill_kernel<<<blocks_for(n, 256), 256, 0, as_stream(stream)>>>(depth, n, threshold, fill);
    AFX_LAUNCH_CHECK();
    return AFX_OK;
}

int afx_fill_f32(float* dst, long n, float value, void* stream) {
    if (!dst || n < 0) return AFX_ERR_INVALID_ARGUMENT;
    if (n == 0) return AFX_OK;
    fill_f32_kernel<<<grid_for(n, 256), 256, 0, as_stream(stream)>>>(dst, n, value);
    AFX_LAUNCH_CHECK();
    return AFX_OK;
}

int afx_bilateral_filter(float* out, const float* in, int height, int width, int r, double sigma_i, double sigma_s,
                         float thr, void* stream) {
    if (!out || !in || out == in || height <= 0 || width <= 0) return AFX_ERR_INVALID_ARGUMENT;
    if (r < 0 || r > kMaxBilateralR) return AFX_ERR_UNSUPPORTED;
    BilateralTables T;
    make_bilateral_tables(r, sigma_i, sigma_s, thr, &T);
    dim3 block(32, 8), grid((width + 31) / 32, (height + 7) / 8);
    bilateral_kernel<<<grid, block, 0, as_stream(stream)>>>(out, in, height, width, T);
    AFX_LAUNCH_CHECK();
    return AFX_OK;
}

int afx_depth_to_mesh(float* vertices, const float* depth, int width, int height, const float K[9], void* stream) {
    if (!vertices || !depth || !K || width <= 0 || height <= 0) return AFX_ERR_INVALID_ARGUMENT;
    dim3 block(32, 8), grid((width + 31) / 32, (height + 7) / 8);
    depth_to_mesh_kernel<<<grid, block, 0, as_stream(stream)>>>(vertices, depth, width, height, make_intrinsics(K),
                                                               1.0f / K[0], 1.0f / K[4]);
    AFX_LAUNCH_CHECK();
    return AFX_OK;
}

int afx_depth_vertices_normals(float* normals, const float* vertices, int height, int width, float lo, float hi,
                               void* stream) {
    if (!normals || !vertices || width <= 0 || height <= 0) return AFX_ERR_INVALID_ARGUMENT;
    dim3 block(32, 8), grid((width + 31) / 32, (height + 7) / 8);
    normals_kernel<<<grid, block, 0, as_stream(stream)>>>(normals, vertices, height, width,
                                                         make_angle_thresholds(lo, hi));
    AFX_LAUNCH_CHECK();
    return AFX_OK;
}

int afx_remove_depth_without_normals(const float* normals, float* vertices, float* depth, int height, int width,
                                     void* stream) {
    if (!normals || !vertices || !depth || width <= 0 || height <= 0) return AFX_ERR_INVALID_ARGUMENT;
    if (width < 3 || height < 3) return AFX_OK;
    dim3 block(32, 8), grid((width - 2 + 31) / 32, (height - 2 + 7) / 8);
    remove_without_normals_kernel<<<grid, block, 0, as_stream(stream)>>>(normals, vertices, depth, height, width);
    AFX_LAUNCH_CHECK();
    return AFX_OK;
}

int afx_frame_prep(const uint16_t* depth_mm, int width, int height, const afx_prep_params* params, float* depth,
                   float* vertices, float* normals, float* centroid, void* stream) {
    PrepScratch* s = prep_scratch();
    if (!s) return AFX_ERR_NO_MEMORY;
    return frame_prep_impl(depth_mm, width, height, params, depth, vertices, normals, centroid, s->acc, &s->error,
                           as_stream(stream), nullptr);
}

}  // extern "C"
