// vf_oracle.cpp -- CPU oracle (test infrastructure only; see vf_oracle.h).
//
// Each function restates one step of the reference hot path and cites the reference
// file:line it follows.  Compiled with -ffp-contract=off so that every binary32
// operation is rounded separately, in the order written here.
#include "vf_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

// The arithmetic type of the restatement: float (the reference's binary32, bit for bit) or, for
// the FP64 oracle build (-DVFO_REAL=double, liboracle64.so), double throughout.
typedef VFO_REAL real;

namespace {

// the reference pads KNN distances with FLT_MAX in either build
const real kFltMax = (real)std::numeric_limits<float>::max();
const real kInf = std::numeric_limits<real>::infinity();

// exp of the reference's skinning weights: the oracle's own binary32 exp, or exp in binary64
inline real vexp(real x);

inline float bits_to_float(uint32_t u) {
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}

// ---- Eigen-order vector arithmetic (measured on the vendored Eigen 3.3.90) ----
inline real dot3(const real* a, const real* b) { return a[0] * b[0] + (a[1] * b[1] + a[2] * b[2]); }
inline real sqnorm3(const real* a) { return a[0] * a[0] + (a[1] * a[1] + a[2] * a[2]); }
inline real norm3(const real* a) { return std::sqrt(sqnorm3(a)); }
// Mat3f (column-major) * Vec3f, row i = R(i,0)x + (R(i,1)y + R(i,2)z)
inline void mat3_vec3(const real* R, const real* p, real* o) {
    for (int i = 0; i < 3; ++i) o[i] = R[i] * p[0] + (R[3 + i] * p[1] + R[6 + i] * p[2]);
}
// (Mat4f (column-major) * [p;1]).head(3), row i = ((T(i,0)x + T(i,1)y) + T(i,2)z) + T(i,3)
inline void mat4_point(const real* T, const real* p, real* o) {
    for (int i = 0; i < 3; ++i) o[i] = ((T[i] * p[0] + T[4 + i] * p[1]) + T[8 + i] * p[2]) + T[12 + i];
}
// nanoflann L2_Simple_Adaptor::evalMetric (third_party nanoflann.hpp:432-440): ((0+d0^2)+d1^2)+d2^2
inline real l2sq_nanoflann(const real* q, const real* p) {
    real d0 = q[0] - p[0], d1 = q[1] - p[1], d2 = q[2] - p[2];
    return (d0 * d0 + d1 * d1) + d2 * d2;
}

// voxelToWorld (src/TSDFIntegration.cu:6-8, src/TSDFWarp.cu:8-10, src/MarchingCubes.cu:315-318)
inline void voxel_to_world(int x, int y, int z, const real* vs, const real* size, real* o) {
    o[0] = (real)x * vs[0] - size[0] * 0.5f;
    o[1] = (real)y * vs[1] - size[1] * 0.5f;
    o[2] = (real)z * vs[2] - size[2] * 0.5f;
}
// worldToVoxel (src/TSDFIntegration.cu:10-14, src/TSDFWarp.cu:11-15)
inline void world_to_voxel(const real* p, const real* vs, const real* size, int* v) {
    for (int c = 0; c < 3; ++c) {
        real inv = (real)(1.0 / (double)vs[c]);
        real f = (p[c] + 0.5f * size[c]) * inv;
        v[c] = vfo_f2i_rz(f);
    }
}

// The binary16 value nearest to x (ties to even), as a real: IEEE 754 rounding of the significand
// to the binary16 spacing of x's binade (2^(e-10) for normal binary16 values, 2^-24 below 2^-14).
// |x| stays far below the binary16 maximum here (TSDF values lie in [-1, 1]).
extern "C" float vfo_round_half(float x) {
    uint32_t u;
    std::memcpy(&u, &x, 4);
    const uint32_t sign = u & 0x80000000u, a = u & 0x7fffffffu;
    const int e = (int)(a >> 23) - 127;
    if (a == 0 || e < -40) {  // zero, binary32 subnormals and anything below half the smallest step
        float z = 0.f;
        if (sign) z = -z;
        return z;
    }
    const uint32_t m = (a & 0x7fffffu) | 0x800000u;  // 24-bit significand, value m * 2^(e-23)
    const int k = (e > -14 ? e : -14) - 10;          // exponent of the binary16 spacing
    const int r = k - (e - 23);                      // significand bits below that spacing (13..)
    uint32_t q = r >= 32 ? 0u : (m >> r);
    if (r < 32) {
        const uint32_t rem = m & ((1u << r) - 1u), half = 1u << (r - 1);
        if (rem > half || (rem == half && (q & 1u))) ++q;
    }
    float y = std::ldexp((float)q, k);
    return sign ? -y : y;
}

// updateTsdf (src/TSDFIntegration.cu:16-67), K column-major
inline void update_tsdf(real* tsdf, real* weights, const real* p, long idx, const real* depth, int W, int H,
                        real delta, const real* K, int half) {
    if (p[2] < 1.e-4f) return;
    real zInv = 1.0f / p[2];
    real uf = (K[0] * p[0]) * zInv + K[6];
    real vf = (K[4] * p[1]) * zInv + K[7];
    int u = vfo_f2i_rz(uf + 0.5f);
    int v = vfo_f2i_rz(vf + 0.5f);
    if (u < 0 || u >= W || v < 0 || v >= H) return;
    real D = depth[(long)v * W + u];
    if (std::isinf(D) || D < 1.e-4f) return;
    real sdf = p[2] - D;
    if (sdf > delta) return;
    real tnew = (sdf < -delta) ? -1.0f : sdf / delta;
    real wnew = 1.0f;
    real wold = weights[idx];
    real told = tsdf[idx];
    const real t = (told * wold + tnew * wnew) / (wold + wnew);
    // precision form: the value is stored as FP16 (weights are integer counts, exact either way)
    tsdf[idx] = half ? (real)vfo_round_half((float)t) : t;
    weights[idx] = std::min(wold + wnew, (real)15.0f);
}

struct Cand {
    real key;  // squared distance (graph KNN) or distance (voxel KNN)
    uint32_t idx;
};
inline bool cand_less(const Cand& a, const Cand& b) { return a.key < b.key || (a.key == b.key && a.idx < b.idx); }

// Insert into a sorted list of at most cap candidates.
inline void topk_insert(Cand* list, int& count, int cap, Cand c) {
    if (count == cap && !cand_less(c, list[cap - 1])) return;
    int i = (count < cap) ? count++ : cap - 1;
    while (i > 0 && cand_less(c, list[i - 1])) {
        list[i] = list[i - 1];
        --i;
    }
    list[i] = c;
}

// Marching-cubes corner numbering (src/MarchingCubes.cu:338-379) and edge endpoints (:441-507).
const int kCorner[8][3] = {{1, 1, 0}, {1, 0, 0}, {0, 0, 0}, {0, 1, 0}, {1, 1, 1}, {1, 0, 1}, {0, 0, 1}, {0, 1, 1}};
const int kEdge[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {4, 5}, {5, 6}, {6, 7}, {7, 4}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};
const uint64_t kTriTable[256] = {
#include "mc_tables.inc"
};

int edge_table(int cube) {
    int e = 0;
    for (int i = 0; i < 12; ++i) {
        int a = (cube >> kEdge[i][0]) & 1, b = (cube >> kEdge[i][1]) & 1;
        if (a != b) e |= 1 << i;
    }
    return e;
}

struct McCtx {
    const real* tsdf;
    const real* w;
    int X, Y, Z;
    const real* vs;
    const real* size;
    real iso;
    long at(int x, int y, int z) const { return (long)z * X * Y + (long)y * X + x; }
    // computeLutIndex (src/MarchingCubes.cu:338-379)
    int cube_index(int x, int y, int z) const {
        long off[8];
        for (int c = 0; c < 8; ++c) off[c] = at(x + kCorner[c][0], y + kCorner[c][1], z + kCorner[c][2]);
        for (int c = 0; c < 8; ++c)
            if (w[off[c]] == 0.0f) return 0;
        int idx = 0;
        for (int c = 0; c < 8; ++c)
            if (tsdf[off[c]] > iso) idx |= 1 << c;
        return idx;
    }
    // getVertex + interpolate (src/MarchingCubes.cu:294-336)
    void vertex(int x, int y, int z, int e, real* o) const {
        const int* ca = kCorner[kEdge[e][0]];
        const int* cb = kCorner[kEdge[e][1]];
        int x1 = x + ca[0], y1 = y + ca[1], z1 = z + ca[2];
        int x2 = x + cb[0], y2 = y + cb[1], z2 = z + cb[2];
        real t0 = tsdf[at(x1, y1, z1)], t1 = tsdf[at(x2, y2, z2)];
        real p0[3], p1[3];
        voxel_to_world(x1, y1, z1, vs, size, p0);
        voxel_to_world(x2, y2, z2, vs, size, p1);
        if ((double)std::fabs(iso - t0) < 1e-7) { std::memcpy(o, p0, 3 * sizeof(real)); return; }
        if ((double)std::fabs(iso - t1) < 1e-7) { std::memcpy(o, p1, 3 * sizeof(real)); return; }
        if ((double)std::fabs(t0 - t1) < 1e-7) { std::memcpy(o, p0, 3 * sizeof(real)); return; }
        double mu = (double)((iso - t0) / (t1 - t0));
        if (mu > 1.0) mu = 1.0;
        else if (mu < 0) mu = 0.0;
        for (int c = 0; c < 3; ++c) o[c] = (real)((double)p0[c] + mu * (double)(p1[c] - p0[c]));
    }
};

inline bool vec3_less(const real* a, const real* b) {
    if (a[0] < b[0]) return true;
    if (b[0] < a[0]) return false;
    if (a[1] < b[1]) return true;
    if (b[1] < a[1]) return false;
    return a[2] < b[2];
}

struct P3 {
    real v[3];
};

}  // namespace

extern "C" {

void vfo_set_threads(int n) { omp_set_num_threads(n > 0 ? n : 1); }

int vfo_threads(void) { return omp_get_max_threads(); }

// Own exp: Cody-Waite range reduction x = k*ln2 + r (ln2 split into a 16-bit head and
// a tail), then a degree-7 Taylor polynomial for e^r by Horner with fused
// multiply-adds, then scaling by 2^k in two exact steps.  Faithful (<= 1 ulp).
float vfo_expf(float x) {
    if (x != x) return x;
    if (x > 88.7228394f) return kInf;
    if (x < -103.972084f) return 0.0f;
    const float log2e = (float)1.4426950408889634;
    const float ln2_hi = 0.693145751953125f;
    const float ln2_lo = (float)(0.6931471805599453 - 0.693145751953125);
    float kf = std::rint(x * log2e);
    float r = std::fma(-kf, ln2_hi, x);
    r = std::fma(-kf, ln2_lo, r);
    float p = (float)(1.0 / 5040.0);
    p = std::fma(p, r, (float)(1.0 / 720.0));
    p = std::fma(p, r, (float)(1.0 / 120.0));
    p = std::fma(p, r, (float)(1.0 / 24.0));
    p = std::fma(p, r, (float)(1.0 / 6.0));
    p = std::fma(p, r, 0.5f);
    p = std::fma(p, r, 1.0f);
    p = std::fma(p, r, 1.0f);
    int k = (int)kf;
    int k1 = k / 2, k2 = k - k1;
    float s1 = bits_to_float((uint32_t)(k1 + 127) << 23);
    float s2 = bits_to_float((uint32_t)(k2 + 127) << 23);
    return (p * s1) * s2;
}

}  // extern "C"
namespace {
inline real vexp(real x) {
    if (sizeof(real) == sizeof(float)) return (real)vfo_expf((float)x);
    return (real)std::exp((double)x);
}
}  // namespace
extern "C" {

// real -> int conversion with CUDA's cvt.rzi.s32.f32 semantics (truncate, saturate, NaN -> 0),
// which is what static_cast<int>(real) does in the reference's device code.
int vfo_f2i_rz(real x) {
    if (x != x) return 0;
    if (x >= 2147483648.0f) return 2147483647;
    if (x <= -2147483648.0f) return (int)(-2147483647 - 1);
    return (int)x;
}

void vfo_depth_from_mm(const uint16_t* mm, long n, real* out) {
    // cv::Mat::convertTo(CV_32FC1, 1/1000) after cv::imread (src/dataset.cpp:188)
    for (long i = 0; i < n; ++i) out[i] = (real)mm[i] * 0.001f;
}

void vfo_filter_depth(real* depth, long n, real threshold) {
    // filterDepthKernel (src/VertexManipulation.cu:6-15), fill value +inf
    for (long i = 0; i < n; ++i) {
        real v = depth[i];
        if (v > threshold || v < 1.e-4f || std::isnan(v)) depth[i] = kInf;
    }
}

// updateGaussian16 (src/BilateralFilter.cu:12-50)
static void bilateral_tables(int r, double sd, real* g2d, int* clr) {
    real g[64];
    for (int i = 0; i < 2 * r + 1; i++) {
        real x = (real)(i - r);
        g[i] = expf((real)((double)(-(x * x)) / (2 * sd * sd)));
    }
    int index = 0;
    for (int dy = -r; dy <= r; dy++)
        for (int dx = -r; dx <= r; dx++) g2d[index++] = g[dy + r] * g[dx + r];
    real fc[31];
    for (int i = 0; i <= 30; i++) fc[i] = (real)std::exp(-(std::pow(i / 10.0, 2)) / (2));
    for (int i = 0; i <= 30; i++) clr[i] = (int)(fc[i] / fc[30]);
}

void vfo_bilateral(real* out, const real* in, int h, int w, int r, double sI, double sS, real thr) {
    // gpuFilterTextureOpmShared (src/BilateralFilter.cu:52-127): clamp-to-edge tile, loop a (x) outer, b (y) inner
    std::vector<real> g2d((2 * r + 1) * (2 * r + 1));
    int clr[31];
    bilateral_tables(r, sS, g2d.data(), clr);
    const real normFactor = (real)(30 / (3 * sI));
    const int kd = 2 * r + 1;
#pragma omp parallel for schedule(static)
    for (int y = 0; y < h; ++y) {
        for (int x = 0; x < w; ++x) {
            real centre = in[(long)y * w + x];
            if (std::isinf(centre)) {
                out[(long)y * w + x] = kInf;
                continue;
            }
            real iF = 0, wP = 0;
            int ig = 0;
            for (int a = 0; a < kd; ++a) {
                for (int b = 0; b < kd; ++b, ++ig) {
                    int xx = std::min(std::max(x + a - r, 0), w - 1);
                    int yy = std::min(std::max(y + b - r, 0), h - 1);
                    real cur = in[(long)yy * w + xx];
                    if (std::isinf(cur)) continue;
                    real diff = std::fabs(centre - cur);
                    if (diff > thr) continue;
                    int x0 = vfo_f2i_rz(std::fabs(diff * normFactor));
                    if (x0 > 30 || x0 < 0) x0 = 30;
                    real wt = g2d[ig] * (real)clr[x0];
                    iF += cur * wt;
                    wP += wt;
                }
            }
            out[(long)y * w + x] = iF / wP;
        }
    }
}

void vfo_depth_to_mesh(real* mesh, const real* depth, int width, int height, const real* K) {
    // depthToMeshKernel (src/VertexManipulation.cu:43-63)
    const real fxi = 1.0f / K[0], fyi = 1.0f / K[4];
    for (int y = 0; y < height; ++y)
        for (int x = 0; x < width; ++x) {
            long id = (long)y * width + x;
            real d = depth[id];
            real* m = mesh + 3 * id;
            if (std::isinf(d) || d < 1.e-4f) {
                m[0] = m[1] = m[2] = 0.f;
                continue;
            }
            real x0 = ((real)x - K[6]) * fxi;
            real y0 = ((real)y - K[7]) * fyi;
            m[0] = x0 * d;
            m[1] = y0 * d;
            m[2] = d;
        }
}

void vfo_normals(real* normals, const real* V, int h, int w, real a_lo, real a_hi) {
    // depthVerticesNormalsKernel (src/VertexManipulation.cu:147-207); border pixels get a zero normal
    std::memset(normals, 0, sizeof(real) * 3 * (size_t)w * h);
#pragma omp parallel for schedule(static)
    for (int y = 1; y < h - 1; ++y) {
        for (int x = 1; x < w - 1; ++x) {
            long id = (long)y * w + x;
            real* n = normals + 3 * id;
            if (V[3 * id + 2] < 1.e-4f) continue;
            const real* xl = V + 3 * (id - 1);
            const real* xr = V + 3 * (id + 1);
            const real* yt = V + 3 * (id - w);
            const real* yb = V + 3 * (id + w);
            if (xr[2] < 1.e-4f || xl[2] < 1.e-4f || yb[2] < 1.e-4f || yt[2] < 1.e-4f) continue;
            real dX[3] = {xr[0] - xl[0], xr[1] - xl[1], xr[2] - xl[2]};
            real dY[3] = {yb[0] - yt[0], yb[1] - yt[1], yb[2] - yt[2]};
            real nx = std::sqrt(dX[0] * dX[0] + dX[1] * dX[1]);
            real ny = std::sqrt(dY[0] * dY[0] + dY[1] * dY[1]);
            real gX[3] = {dX[0] / nx, dX[1] / nx, dX[2] / nx};
            real gY[3] = {dY[0] / ny, dY[1] / ny, dY[2] / ny};
            real c[3] = {gY[1] * gX[2] - gY[2] * gX[1], gY[2] * gX[0] - gY[0] * gX[2], gY[0] * gX[1] - gY[1] * gX[0]};
            real s = sqnorm3(c);
            if (s > 0.f) {
                real q = std::sqrt(s);
                c[0] /= q;
                c[1] /= q;
                c[2] /= q;
            }
            real dot = 0.f * c[0] + (0.f * c[1] + 1.f * c[2]);
            real angle = (real)std::acos((double)dot);
            if (angle > a_lo && angle < a_hi) continue;
            n[0] = c[0];
            n[1] = c[1];
            n[2] = c[2];
        }
    }
}

void vfo_remove_without_normals(const real* normals, real* V, real* depth, int h, int w) {
    // removeDepthWithoutNormalsKernel (src/VertexManipulation.cu:223-236), isZero(1e-4)
    for (int y = 1; y < h - 1; ++y)
        for (int x = 1; x < w - 1; ++x) {
            long id = (long)y * w + x;
            const real* n = normals + 3 * id;
            if (std::fabs(n[0]) <= 1.e-4f && std::fabs(n[1]) <= 1.e-4f && std::fabs(n[2]) <= 1.e-4f) {
                V[3 * id] = V[3 * id + 1] = V[3 * id + 2] = 0.f;
                depth[id] = kInf;
            }
        }
}

void vfo_centroid(const real* V, long n, real out[3]) {
    // Sum of all vertices / count of z > 1e-4 (src/VolumeFusion.cu:217-219).  The sum is taken in
    // 2^-32 fixed point so that it does not depend on summation order.
    long long s[3] = {0, 0, 0};
    long cnt = 0;
    for (long i = 0; i < n; ++i) {
        for (int c = 0; c < 3; ++c) s[c] += std::llrint((double)V[3 * i + c] * 4294967296.0);
        if (V[3 * i + 2] > 1.e-4f) ++cnt;
    }
    for (int c = 0; c < 3; ++c) out[c] = (real)(((double)s[c] / 4294967296.0) / (double)cnt);
}

// ---- depth ingest (test infrastructure: restatements of OpenCV 4.x and of src/CameraCalibration.cpp) ----

// cvRound on x86-64: nearest, ties to even; NaN and values outside int32 give INT_MIN.
static int cv_round_d(double v) {
    return (v >= -2147483648.5 && v < 2147483647.5) ? (int)std::nearbyint(v) : (int)(-2147483647 - 1);
}
static int cv_round_f(float v) {
    return (v >= -2147483648.f && v < 2147483648.f) ? (int)std::nearbyintf(v) : (int)(-2147483647 - 1);
}
static uint32_t pack_sxy(int sx, int sy) { return (uint32_t)(uint16_t)(int16_t)sx | ((uint32_t)(uint16_t)(int16_t)sy << 16); }

void vfo_undistort_map(uint32_t* map, int W, int H, const float K[9], const float k_cv[8], int mode) {
    // the camera matrix the reference builds (src/VolumeFusion.cu:163-170): fx, fy, cx, cy, K(2,2)
    double A[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    A[0] = K[0];
    A[4] = K[4];
    A[2] = K[6];
    A[5] = K[7];
    A[8] = K[8];
    double k[8];
    for (int q = 0; q < 8; ++q) k[q] = k_cv[q];
    // cv::undistort (calib3d/src/undistort.dispatch.cpp): stripes of max(1, 4096 / cols) rows, each
    // with the new camera matrix's cy lowered by the stripe's first row; the stream readers' single
    // initUndistortRectifyMap is one stripe
    int stripe = H;
    if (mode == 0) {
        stripe = 4096 / W;
        if (stripe < 1) stripe = 1;
        if (stripe > H) stripe = H;
    }
    for (int i = 0; i < H; ++i) {
        const int y0 = (i / stripe) * stripe;
        double Ar[9];
        std::memcpy(Ar, A, sizeof(Ar));
        if (mode == 0) Ar[5] = A[5] - (double)y0;
        // iR = Ar^-1 (cv::invert, DECOMP_LU, closed form for 3 x 3)
        const double* m = Ar;
        double ir[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        const double det = m[0] * (m[4] * m[8] - m[5] * m[7]) - m[1] * (m[3] * m[8] - m[5] * m[6]) +
                           m[2] * (m[3] * m[7] - m[4] * m[6]);
        if (det != 0.0) {
            const double d = 1.0 / det;
            ir[0] = (m[4] * m[8] - m[5] * m[7]) * d;
            ir[1] = (m[2] * m[7] - m[1] * m[8]) * d;
            ir[2] = (m[1] * m[5] - m[2] * m[4]) * d;
            ir[3] = (m[5] * m[6] - m[3] * m[8]) * d;
            ir[4] = (m[0] * m[8] - m[2] * m[6]) * d;
            ir[5] = (m[2] * m[3] - m[0] * m[5]) * d;
            ir[6] = (m[3] * m[7] - m[4] * m[6]) * d;
            ir[7] = (m[1] * m[6] - m[0] * m[7]) * d;
            ir[8] = (m[0] * m[4] - m[1] * m[3]) * d;
        }
        // initUndistortRectifyMap's row loop: u0, v0, fx, fy from the original camera matrix
        const double u0 = A[2], v0 = A[5], fx = A[0], fy = A[4];
        const double k1 = k[0], k2 = k[1], p1 = k[2], p2 = k[3], k3 = k[4], k4 = k[5], k5 = k[6], k6 = k[7];
        const int row = mode == 0 ? i - y0 : i;
        double X = row * ir[1] + ir[2], Y = row * ir[4] + ir[5], Wh = row * ir[7] + ir[8];
        uint32_t* out = map + 2 * (size_t)i * W;
        for (int j = 0; j < W; ++j, X += ir[0], Y += ir[3], Wh += ir[6]) {
            const double w = 1. / Wh, x = X * w, y = Y * w;
            const double x2 = x * x, y2 = y * y;
            const double r2 = x2 + y2, _2xy = 2 * x * y;
            const double kr = (1 + ((k3 * r2 + k2) * r2 + k1) * r2) / (1 + ((k6 * r2 + k5) * r2 + k4) * r2);
            const double xd = x * kr + p1 * _2xy + p2 * (r2 + 2 * x2);
            const double yd = y * kr + p1 * (r2 + 2 * y2) + p2 * _2xy;
            const double u = fx * xd + u0, v = fy * yd + v0;
            if (mode == 0) {  // CV_16SC2 + CV_16UC1, INTER_BITS = 5
                const int iu = cv_round_d(u * 32.0), iv = cv_round_d(v * 32.0);
                out[2 * j] = pack_sxy((int)(int16_t)(iu >> 5), (int)(int16_t)(iv >> 5));
                out[2 * j + 1] = (uint32_t)((iv & 31) * 32 + (iu & 31));
            } else {  // CV_32FC1, then remap's saturate_cast<short> of each coordinate
                const int sx = cv_round_f((float)u), sy = cv_round_f((float)v);
                out[2 * j] = pack_sxy(std::min(std::max(sx, -32768), 32767), std::min(std::max(sy, -32768), 32767));
                out[2 * j + 1] = 0;
            }
        }
    }
}

void vfo_undistort_depth(real* dst, const real* src, int W, int H, const uint32_t* map, int mode) {
    // cv::remap (imgproc/src/imgwarp.cpp): remapBilinear with the float 32 x 32 weight table, or
    // remapNearest; BORDER_CONSTANT with value 0
    for (long p = 0; p < (long)W * H; ++p) {
        const int sx = (int)(int16_t)(uint16_t)(map[2 * p] & 0xFFFF), sy = (int)(int16_t)(uint16_t)(map[2 * p] >> 16);
        auto at = [&](int x, int y) -> real {
            return ((unsigned)x < (unsigned)W && (unsigned)y < (unsigned)H) ? src[(long)y * W + x] : (real)0;
        };
        if (mode == 0) {
            const uint32_t f = map[2 * p + 1];
            const float ax = (float)(f & 31u) * (1.f / 32.f), ay = (float)((f >> 5) & 31u) * (1.f / 32.f);
            const float bx = 1.f - ax, by = 1.f - ay;
            const real w0 = by * bx, w1 = by * ax, w2 = ay * bx, w3 = ay * ax;
            dst[p] = at(sx, sy) * w0 + at(sx + 1, sy) * w1 + at(sx, sy + 1) * w2 + at(sx + 1, sy + 1) * w3;
        } else {
            dst[p] = at(sx, sy);
        }
    }
}

namespace {

struct BcCam {
    float cx, cy, fx, fy, k1, k2, k3, k4, k5, k6, codx, cody, p1, p2;
};

BcCam bc_cam(const float intr[4], const float d[10]) {
    return BcCam{intr[0], intr[1], intr[2], intr[3], d[0], d[1], d[2], d[3], d[4], d[5], d[6], d[7], d[8], d[9]};
}

// transformation_project_internal (src/CameraCalibration.cpp:9-94); false beyond the radius
bool bc_project(const BcCam& c, float x, float y, float* uv, float* J) {
    float xp = x - c.codx, yp = y - c.cody;
    float xp2 = xp * xp, yp2 = yp * yp, xyp = xp * yp;
    float rs = xp2 + yp2;
    float max_r = 1.7f;
    if (rs > max_r * max_r) return false;
    float rss = rs * rs, rsc = rss * rs;
    float a = 1.f + c.k1 * rs + c.k2 * rss + c.k3 * rsc;
    float b = 1.f + c.k4 * rs + c.k5 * rss + c.k6 * rsc;
    float bi = b != 0.f ? 1.f / b : 1.f;
    float d = a * bi;
    float xp_d = xp * d, yp_d = yp * d;
    float rs_2xp2 = rs + 2.f * xp2, rs_2yp2 = rs + 2.f * yp2;
    xp_d += rs_2xp2 * c.p2 + 2.f * xyp * c.p1;
    yp_d += rs_2yp2 * c.p1 + 2.f * xyp * c.p2;
    uv[0] = (xp_d + c.codx) * c.fx + c.cx;
    uv[1] = (yp_d + c.cody) * c.fy + c.cy;
    if (J) {
        float dudrs = c.k1 + 2.f * c.k2 * rs + 3.f * c.k3 * rss;
        float dvdrs = c.k4 + 2.f * c.k5 * rs + 3.f * c.k6 * rss;
        float bis = bi * bi;
        float dddrs = (dudrs * b - a * dvdrs) * bis;
        float dddrs_2 = dddrs * 2.f;
        float xp_dddrs_2 = xp * dddrs_2;
        float yp_xp_dddrs_2 = yp * xp_dddrs_2;
        J[0] = c.fx * (d + xp * xp_dddrs_2 + 6.f * xp * c.p2 + 2.f * yp * c.p1);
        J[1] = c.fx * (yp_xp_dddrs_2 + 2.f * yp * c.p2 + 2.f * xp * c.p1);
        J[2] = c.fy * (yp_xp_dddrs_2 + 2.f * xp * c.p1 + 2.f * yp * c.p2);
        J[3] = c.fy * (d + yp * yp * dddrs_2 + 6.f * yp * c.p1 + 2.f * xp * c.p2);
    }
    return true;
}

// transformation_unproject_internal + transformation_iterative_unproject (src/CameraCalibration.cpp:106-218)
void bc_unproject(const BcCam& c, float u, float v, float* xy, int* valid) {
    float xp_d = (u - c.cx) / c.fx - c.codx;
    float yp_d = (v - c.cy) / c.fy - c.cody;
    float rs = xp_d * xp_d + yp_d * yp_d;
    float rss = rs * rs, rsc = rss * rs;
    float a = 1.f + c.k1 * rs + c.k2 * rss + c.k3 * rsc;
    float b = 1.f + c.k4 * rs + c.k5 * rss + c.k6 * rsc;
    float ai = a != 0.f ? 1.f / a : 1.f;
    float di = ai * b;
    float x = xp_d * di, y = yp_d * di;
    float two_xy = 2.f * x * y;
    float xx = x * x, yy = y * y;
    x -= (yy + 3.f * xx) * c.p2 + two_xy * c.p1;
    y -= (xx + 3.f * xx) * c.p1 + two_xy * c.p2;  // (xx + 3 xx), as the reference has it
    x += c.codx;
    y += c.cody;
    *valid = 1;
    float bx = 0.f, by = 0.f, best = std::numeric_limits<float>::max();
    for (int pass = 0; pass < 20; ++pass) {
        float p[2], J[4];
        if (!bc_project(c, x, y, p, J)) {
            *valid = 0;
            xy[0] = x;
            xy[1] = y;
            return;
        }
        float ex = u - p[0], ey = v - p[1];
        float err = ex * ex + ey * ey;
        if (err >= best) {
            x = bx;
            y = by;
            break;
        }
        best = err;
        bx = x;
        by = y;
        float det = J[0] * J[3] - J[1] * J[2];
        float inv = 1.f / det;
        float i0 = inv * J[3], i3 = inv * J[0], i1 = -inv * J[1], i2 = -inv * J[2];
        if (pass + 1 == 20 || best < 1e-22f) break;
        x += i0 * ex + i1 * ey;
        y += i2 * ex + i3 * ey;
    }
    if (best > 1e-6f) *valid = 0;
    xy[0] = x;
    xy[1] = y;
}

}  // namespace

void vfo_xy_lookup_table(float* table, int W, int H, const float intr[4], const float dist[10]) {
    // create_xy_lookup_table (src/CameraCalibration.cpp:261-295)
    const BcCam c = bc_cam(intr, dist);
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            float xy[2];
            int valid = 0;
            bc_unproject(c, (float)x, (float)y, xy, &valid);
            float* o = table + 2 * ((size_t)y * W + x);
            o[0] = valid ? xy[0] * 1.f : 0.f;
            o[1] = valid ? xy[1] * 1.f : 0.f;
        }
}

void vfo_bc_unproject(float* pts, int* valid, const float* px, const float* depth, long n, const float intr[4],
                      const float dist[10]) {
    // transformation_unproject (src/CameraCalibration.cpp:220-243)
    const BcCam c = bc_cam(intr, dist);
    for (long i = 0; i < n; ++i) {
        const float d = depth[i];
        if (d == 0.f) {
            pts[3 * i] = pts[3 * i + 1] = pts[3 * i + 2] = 0.f;
            valid[i] = 0;
            continue;
        }
        float xy[2];
        bc_unproject(c, px[2 * i], px[2 * i + 1], xy, &valid[i]);
        pts[3 * i] = xy[0] * d;
        pts[3 * i + 1] = xy[1] * d;
        pts[3 * i + 2] = d;
    }
}

void vfo_bc_project(float* px, int* valid, const float* pts, long n, const float intr[4], const float dist[10]) {
    // transformation_project (src/CameraCalibration.cpp:245-259); beyond the radius the pixel is left as it was
    const BcCam c = bc_cam(intr, dist);
    for (long i = 0; i < n; ++i) {
        const float z = pts[3 * i + 2];
        if (z <= 0.f) {
            px[2 * i] = px[2 * i + 1] = 0.f;
            valid[i] = 0;
            continue;
        }
        float uv[2];
        if (bc_project(c, pts[3 * i] / z, pts[3 * i + 1] / z, uv, nullptr)) {
            px[2 * i] = uv[0];
            px[2 * i + 1] = uv[1];
            valid[i] = 1;
        } else {
            valid[i] = 0;
        }
    }
}

static void frame_prep_from_depth(int width, int height, const real* K, real depth_threshold, int bilateral, int r,
                                  double sigma_i, double sigma_s, real thr, real angle_lo, real angle_hi, real* depth,
                                  real* vertices, real* normals, real centroid[3]) {
    long n = (long)width * height;
    vfo_filter_depth(depth, n, depth_threshold);
    if (bilateral) {
        std::vector<real> tmp(depth, depth + n);
        vfo_bilateral(depth, tmp.data(), height, width, r, sigma_i, sigma_s, thr);
    }
    vfo_depth_to_mesh(vertices, depth, width, height, K);
    vfo_normals(normals, vertices, height, width, angle_lo, angle_hi);
    vfo_remove_without_normals(normals, vertices, depth, height, width);
    vfo_centroid(vertices, n, centroid);
}

void vfo_frame_prep_undistorted(const uint16_t* mm, int width, int height, const real* K, real depth_threshold,
                                int bilateral, int r, double sigma_i, double sigma_s, real thr, real angle_lo,
                                real angle_hi, const uint32_t* map, real* depth, real* vertices, real* normals,
                                real centroid[3]) {
    // af::loadProcessFrame with a distorted camera (src/VolumeFusion.cu:160-220): metres, cv::undistort,
    // then the filter and the rest
    long n = (long)width * height;
    std::vector<real> metres(n);
    vfo_depth_from_mm(mm, n, metres.data());
    vfo_undistort_depth(depth, metres.data(), width, height, map, 0);
    frame_prep_from_depth(width, height, K, depth_threshold, bilateral, r, sigma_i, sigma_s, thr, angle_lo, angle_hi,
                          depth, vertices, normals, centroid);
}

void vfo_frame_prep(const uint16_t* mm, int width, int height, const real* K, real depth_threshold, int bilateral,
                    int r, double sigma_i, double sigma_s, real thr, real angle_lo, real angle_hi, real* depth,
                    real* vertices, real* normals, real centroid[3]) {
    // af::loadProcessFrame (src/VolumeFusion.cu:184-220)
    long n = (long)width * height;
    vfo_depth_from_mm(mm, n, depth);
    vfo_filter_depth(depth, n, depth_threshold);
    if (bilateral) {
        std::vector<real> tmp(depth, depth + n);
        vfo_bilateral(depth, tmp.data(), height, width, r, sigma_i, sigma_s, thr);
    }
    vfo_depth_to_mesh(vertices, depth, width, height, K);
    vfo_normals(normals, vertices, height, width, angle_lo, angle_hi);
    vfo_remove_without_normals(normals, vertices, depth, height, width);
    vfo_centroid(vertices, n, centroid);
}

void vfo_integrate_rigid(real* tsdf, real* weights, const real* depth, int width, int height, real delta,
                         const int dims[3], const real vs[3], const real size[3], const real R[9], const real t[3],
                         const real K[9], int half) {
    // integrateTSDFFromFrameKernel (src/TSDFIntegration.cu:69-96)
    const int X = dims[0], Y = dims[1], Z = dims[2];
#pragma omp parallel for schedule(static)
    for (int z = 0; z < Z; ++z)
        for (int y = 0; y < Y; ++y)
            for (int x = 0; x < X; ++x) {
                real p[3], q[3];
                voxel_to_world(x, y, z, vs, size, p);
                mat3_vec3(R, p, q);
                q[0] = q[0] + t[0];
                q[1] = q[1] + t[1];
                q[2] = q[2] + t[2];
                update_tsdf(tsdf, weights, q, (long)z * X * Y + (long)y * X + x, depth, width, height, delta, K, half);
            }
}

// ---- marching cubes ----

static void mc_slab(const McCtx& m, int z, std::vector<P3>& out) {
    for (int y = 0; y < m.Y - 2; ++y)
        for (int x = 0; x < m.X - 2; ++x) {
            int ci = m.cube_index(x, y, z);
            if (ci == 0 || ci == 255) continue;
            int et = edge_table(ci);
            for (int e = 0; e < 12; ++e)
                if (et & (1 << e)) {
                    P3 p;
                    m.vertex(x, y, z, e, p.v);
                    out.push_back(p);
                }
        }
}

long vfo_mc_pointcloud(const real* tsdf, const real* weights, const int dims[3], const real vs[3],
                       const real size[3], real iso, real* out, long cap) {
    // marchingCubesMeshKernel (src/MarchingCubes.cu:422-508), cubes x,y,z < dim-2, z/y/x loop order
    McCtx m{tsdf, weights, dims[0], dims[1], dims[2], vs, size, iso};
    int nz = std::max(dims[2] - 2, 0);
    std::vector<std::vector<P3>> slabs(nz);
#pragma omp parallel for schedule(dynamic, 4)
    for (int z = 0; z < nz; ++z) mc_slab(m, z, slabs[z]);
    long n = 0;
    for (auto& s : slabs) {
        for (auto& p : s) {
            if (n < cap) std::memcpy(out + 3 * n, p.v, 3 * sizeof(real));
            ++n;
        }
    }
    return n;
}

long vfo_sort_unique_vec3(real* pts, long n) {
    // thrust::sort + thrust::unique with the lexicographic operator< (include/af/eigen_extension.cuh:15-25)
    std::vector<P3> v(n);
    std::memcpy(v.data(), pts, 3 * sizeof(real) * n);
    std::sort(v.begin(), v.end(), [](const P3& a, const P3& b) { return vec3_less(a.v, b.v); });
    long m = 0;
    for (long i = 0; i < n; ++i) {
        if (m > 0 && v[i].v[0] == v[m - 1].v[0] && v[i].v[1] == v[m - 1].v[1] && v[i].v[2] == v[m - 1].v[2]) continue;
        v[m++] = v[i];
    }
    std::memcpy(pts, v.data(), 3 * sizeof(real) * m);
    return m;
}

void vfo_transform_points(real* pts, long n, const real T[16]) {
    // transformKernel (src/VertexManipulation.cu:89-95): p <- (T * [p; 1]).head(3)
    for (long i = 0; i < n; ++i) {
        real q[3];
        mat4_point(T, pts + 3 * i, q);
        std::memcpy(pts + 3 * i, q, 3 * sizeof(real));
    }
}

void vfo_translate(real* pts, long n, const real t[3]) {
    // translateKernel (src/VertexManipulation.cu:73-79)
    for (long i = 0; i < n; ++i)
        for (int c = 0; c < 3; ++c) pts[3 * i + c] = pts[3 * i + c] + t[c];
}

long vfo_mc_full(const real* tsdf, const real* weights, const int dims[3], const real vs[3], const real size[3],
                 real iso, real* verts, long vcap, int* faces, long fcap, long* nfaces) {
    // marchingCubesFullKernel + computeTriangles (src/MarchingCubes.cu:393-420, 526-682), cube order z/y/x
    McCtx m{tsdf, weights, dims[0], dims[1], dims[2], vs, size, iso};
    int nz = std::max(dims[2] - 2, 0);
    std::vector<std::vector<P3>> slabs(nz);
#pragma omp parallel for schedule(dynamic, 4)
    for (int z = 0; z < nz; ++z) {
        for (int y = 0; y < m.Y - 2; ++y)
            for (int x = 0; x < m.X - 2; ++x) {
                int ci = m.cube_index(x, y, z);
                if (ci == 0 || ci == 255) continue;
                int et = edge_table(ci);
                real ep[12][3];
                for (int e = 0; e < 12; ++e)
                    if (et & (1 << e)) m.vertex(x, y, z, e, ep[e]);
                uint64_t tri = kTriTable[ci];
                for (int s = 0;; s += 3) {
                    int e0 = (int)((tri >> (4 * s)) & 0xF);
                    if (e0 == 0xF) break;
                    int e1 = (int)((tri >> (4 * (s + 1))) & 0xF), e2 = (int)((tri >> (4 * (s + 2))) & 0xF);
                    const real *p1 = ep[e0], *p2 = ep[e1], *p3 = ep[e2];
                    auto ne = [](const real* a, const real* b) { return a[0] != b[0] || a[1] != b[1] || a[2] != b[2]; };
                    if (ne(p1, p2) && ne(p1, p3) && ne(p2, p3)) {
                        P3 a, b, c;
                        std::memcpy(a.v, p1, 3 * sizeof(real));
                        std::memcpy(b.v, p2, 3 * sizeof(real));
                        std::memcpy(c.v, p3, 3 * sizeof(real));
                        slabs[z].push_back(a);
                        slabs[z].push_back(b);
                        slabs[z].push_back(c);
                    }
                }
            }
    }
    long nv = 0;
    for (auto& s : slabs)
        for (auto& p : s) {
            if (nv < vcap) std::memcpy(verts + 3 * nv, p.v, 3 * sizeof(real));
            ++nv;
        }
    long nf = nv / 3;
    for (long f = 0; f < nf && f < fcap; ++f) {
        faces[3 * f] = (int)(3 * f);
        faces[3 * f + 1] = (int)(3 * f + 1);
        faces[3 * f + 2] = (int)(3 * f + 2);
    }
    if (nfaces) *nfaces = nf;
    return nv;
}

// ---- motion graph ----

static int knn_query(const real* nodes, int n, const real* q, int k, Cand* out) {
    int cnt = 0;
    for (int j = 0; j < n; ++j) topk_insert(out, cnt, k, Cand{l2sq_nanoflann(q, nodes + 3 * j), (uint32_t)j});
    return cnt;
}

int vfo_build_graph(real* nodes, real* radii, real* T, int n, int cap, const real* mesh, long m, int knn,
                    real radius) {
    // af::buildGraph (src/GraphBuilder.cpp:12-50) with MotionGraph::knnSearch (src/MotionGraph.cpp:43-60)
    static const real I4[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
    if (m == 0) return n;
    if (n == 0) {
        if (cap < 1) return -1;
        std::memcpy(nodes, mesh, 3 * sizeof(real));
        radii[0] = radius;
        std::memcpy(T, I4, 16 * sizeof(real));
        n = 1;
    }
    std::vector<Cand> c(knn);
    for (long i = 0; i < m; ++i) {
        const real* q = mesh + 3 * i;
        int cnt = knn_query(nodes, n, q, knn, c.data());
        bool supported = false;
        for (int j = 0; j < cnt; ++j)
            if (std::sqrt(c[j].key) < radii[c[j].idx]) {
                supported = true;
                break;
            }
        if (supported) continue;
        if (n >= cap) return -1;
        real d0 = std::sqrt(c[0].key);
        real factor = d0 / (0.f + d0);
        const real* Tn = T + 16 * c[0].idx;
        real* Tnew = T + 16 * n;
        for (int e = 0; e < 16; ++e) Tnew[e] = 0.f + Tn[e] * factor;
        std::memcpy(nodes + 3 * n, q, 3 * sizeof(real));
        radii[n] = radius;
        ++n;
    }
    return n;
}

void vfo_knn(const real* nodes, int n, const real* pts, long m, int k, int exclude_closest, uint32_t* idx,
             real* dist) {
    // af::getKnnData<K> + MotionGraph::knnSearch<K> (include/af/GraphBuilder.h:118-130, include/af/MotionGraph.h:50-70).
    // Exact K nearest by nanoflann's squared distance; equal distances are ordered by node index.
    const int kk = k + (exclude_closest ? 1 : 0);
#pragma omp parallel for schedule(static)
    for (long i = 0; i < m; ++i) {
        Cand c[33];
        int cnt = knn_query(nodes, n, pts + 3 * i, kk, c);
        int off = exclude_closest ? 1 : 0;
        int res = std::max(cnt - off, 0);
        for (int s = 0; s < k; ++s) {
            if (s < res) {
                idx[i * k + s] = c[s + off].idx;
                dist[i * k + s] = std::sqrt(c[s + off].key);
            } else {
                idx[i * k + s] = VFO_INVALID_IDX;
                dist[i * k + s] = kFltMax;
            }
        }
    }
}

void vfo_filter_disconnected(uint32_t* idx, real* dist, int n, int k, const real* radii) {
    // af::filterDisconnected<K> (include/af/GraphBuilder.h:132-146)
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < k; ++j) {
            uint32_t nb = idx[i * k + j];
            if (nb >= (uint32_t)n) continue;
            if (dist[i * k + j] <= radii[i] * 1.3f) continue;
            idx[i * k + j] = VFO_INVALID_IDX;
            dist[i * k + j] = kFltMax;
        }
}

void vfo_warp_weights(real* w, const real* radii, const uint32_t* idx, const real* dist, long m, int k,
                      int n_nodes) {
    // computeWarpWeightsKernel + weight() (src/VertexManipulation.cu:105-132): cut off at d >= radius
#pragma omp parallel for schedule(static)
    for (long i = 0; i < m; ++i) {
        real s = 0;
        real* wi = w + i * k;
        for (int j = 0; j < k; ++j) {
            uint32_t nb = idx[i * k + j];
            real wj = 0.f;
            if (nb < (uint32_t)n_nodes) {
                real r = radii[nb], d = dist[i * k + j];
                wj = (d >= r) ? 0.f : vexp(-(d * d) / (2.0f * (r * r)));
            }
            wi[j] = wj;
            s += wj;
        }
        if (s != 0.f)
            for (int j = 0; j < k; ++j) wi[j] = wi[j] / s;
    }
}

// ---- dual-quaternion blending (no counterpart in the reference) ----
// Kavan, Collins, Zara, O'Sullivan, "Skinning with dual quaternions" (I3D 2007).  A node's rigid part
// is the unit quaternion of its transform's upper 3x3 by Shepperd's method (the largest diagonal
// combination under the square root, then normalised) with the translation T[12..14]; the nodes of
// a point are blended as sum_j w_j s_j q_j, s_j = -1 for rotation parts in the other hemisphere from
// the first valid node's, normalised by the rotation part's norm, and applied as one rigid motion.
// Operation order as written (-ffp-contract=off), the library's too.
static void dq_of(const real* T, real* q) {
    const real m00 = T[0], m10 = T[1], m20 = T[2], m01 = T[4], m11 = T[5], m21 = T[6];
    const real m02 = T[8], m12 = T[9], m22 = T[10];
    const real tr = (m00 + m11) + m22;
    real w, x, y, z;
    if (tr > (real)0) {
        const real s = std::sqrt(tr + (real)1) * (real)2;
        w = (real)0.25 * s;
        x = (m21 - m12) / s;
        y = (m02 - m20) / s;
        z = (m10 - m01) / s;
    } else if (m00 > m11 && m00 > m22) {
        const real s = std::sqrt((((real)1 + m00) - m11) - m22) * (real)2;
        w = (m21 - m12) / s;
        x = (real)0.25 * s;
        y = (m01 + m10) / s;
        z = (m02 + m20) / s;
    } else if (m11 > m22) {
        const real s = std::sqrt((((real)1 + m11) - m00) - m22) * (real)2;
        w = (m02 - m20) / s;
        x = (m01 + m10) / s;
        y = (real)0.25 * s;
        z = (m12 + m21) / s;
    } else {
        const real s = std::sqrt((((real)1 + m22) - m00) - m11) * (real)2;
        w = (m10 - m01) / s;
        x = (m02 + m20) / s;
        y = (m12 + m21) / s;
        z = (real)0.25 * s;
    }
    const real n = std::sqrt(((w * w + x * x) + y * y) + z * z);
    w = w / n;
    x = x / n;
    y = y / n;
    z = z / n;
    const real tx = T[12], ty = T[13], tz = T[14];
    q[0] = w;
    q[1] = x;
    q[2] = y;
    q[3] = z;
    q[4] = (real)-0.5 * ((tx * x + ty * y) + tz * z);
    q[5] = (real)0.5 * ((w * tx + ty * z) - tz * y);
    q[6] = (real)0.5 * ((w * ty + tz * x) - tx * z);
    q[7] = (real)0.5 * ((w * tz + tx * y) - ty * x);
}

// out = p moved by the blend of the k slots (skipping VFO_INVALID_IDX); p when the weights are all
// within 1e-5 of zero or the blend's rotation part is zero.
static void dq_point(const real* T, const uint32_t* idx, const real* w, int k, const real* p, real* out) {
    out[0] = p[0];
    out[1] = p[1];
    out[2] = p[2];
    bool zero = true;
    for (int j = 0; j < k; ++j)
        if (!(std::fabs(w[j]) <= (real)1e-5f)) zero = false;
    if (zero) return;
    real b[8] = {0, 0, 0, 0, 0, 0, 0, 0}, r0[4] = {0, 0, 0, 0};
    bool first = true;
    for (int j = 0; j < k; ++j) {
        if (idx[j] == VFO_INVALID_IDX) continue;
        real q[8];
        dq_of(T + 16 * (size_t)idx[j], q);
        if (first) {
            for (int c = 0; c < 4; ++c) r0[c] = q[c];
            first = false;
        }
        const real d = ((r0[0] * q[0] + r0[1] * q[1]) + r0[2] * q[2]) + r0[3] * q[3];
        const real ws = d < (real)0 ? -w[j] : w[j];
        for (int c = 0; c < 8; ++c) b[c] = b[c] + ws * q[c];
    }
    const real n = std::sqrt(((b[0] * b[0] + b[1] * b[1]) + b[2] * b[2]) + b[3] * b[3]);
    if (!(n > (real)0)) return;
    const real rw = b[0] / n, rx = b[1] / n, ry = b[2] / n, rz = b[3] / n;
    const real ew = b[4] / n, ex = b[5] / n, ey = b[6] / n, ez = b[7] / n;
    const real cx = ry * p[2] - rz * p[1], cy = rz * p[0] - rx * p[2], cz = rx * p[1] - ry * p[0];
    const real ccx = ry * cz - rz * cy, ccy = rz * cx - rx * cz, ccz = rx * cy - ry * cx;
    const real tx = (real)2 * ((rw * ex - ew * rx) + (ry * ez - rz * ey));
    const real ty = (real)2 * ((rw * ey - ew * ry) + (rz * ex - rx * ez));
    const real tz = (real)2 * ((rw * ez - ew * rz) + (rx * ey - ry * ex));
    out[0] = ((p[0] + (real)2 * rw * cx) + (real)2 * ccx) + tx;
    out[1] = ((p[1] + (real)2 * rw * cy) + (real)2 * ccy) + ty;
    out[2] = ((p[2] + (real)2 * rw * cz) + (real)2 * ccz) + tz;
}

void vfo_warp_dqb(real* out, const real* pts, long m, const real* T, const uint32_t* idx, const real* w, int k) {
#pragma omp parallel for schedule(static)
    for (long i = 0; i < m; ++i) dq_point(T, idx + i * k, w + i * k, k, pts + 3 * i, out + 3 * i);
}

void vfo_warp(real* out, const real* pts, long m, const real* T, const uint32_t* idx, const real* w, int k) {
    // warpKernel (src/ComputeCorrespondence.cu:5-30): identity when all weights are zero (isZero, 1e-5)
#pragma omp parallel for schedule(static)
    for (long i = 0; i < m; ++i) {
        const real* p = pts + 3 * i;
        const real* wi = w + i * k;
        bool zero = true;
        for (int j = 0; j < k; ++j)
            if (!(std::fabs(wi[j]) <= 1e-5f)) zero = false;
        real acc[3] = {0.f, 0.f, 0.f};
        if (zero) {
            std::memcpy(acc, p, 3 * sizeof(real));
        } else {
            for (int j = 0; j < k; ++j) {
                uint32_t nb = idx[i * k + j];
                if (nb == VFO_INVALID_IDX) continue;
                real q[3];
                mat4_point(T + 16 * (size_t)nb, p, q);
                for (int c = 0; c < 3; ++c) acc[c] = acc[c] + wi[j] * q[c];
            }
        }
        std::memcpy(out + 3 * i, acc, 3 * sizeof(real));
    }
}

long vfo_correspondences(int* corr, long cap, const real* warped, long m, const real* K, const real* depth,
                         int rows, int cols, const real* frame_mesh, real thr) {
    // correspondencePairsKernel (src/ComputeCorrespondence.cu:45-81), output ordered by vertex index
    long n = 0;
    for (long i = 0; i < m; ++i) {
        const real* v = warped + 3 * i;
        real y0 = v[1] / v[2];
        real x0 = v[0] / v[2];
        int y = vfo_f2i_rz(y0 * K[4] + K[7]);
        int x = vfo_f2i_rz(x0 * K[0] + K[6]);
        if (y < 0 || x < 0 || y >= rows || x >= cols) continue;
        long px = (long)y * cols + x;
        real d[3] = {frame_mesh[3 * px] - v[0], frame_mesh[3 * px + 1] - v[1], frame_mesh[3 * px + 2] - v[2]};
        if (norm3(d) > thr) continue;
        if (depth[px] > 1.e-4f) {
            if (n < cap) {
                corr[2 * n] = (int)i;
                corr[2 * n + 1] = (int)px;
            }
            ++n;
        }
    }
    return n;
}

// ---- Gauss-Newton ----

void vfo_residual_depth(real* r, const int* corr, long c, const real* warped, const real* frame_mesh,
                        const real* normals, real lambda) {
    // fill_r_DepthKernel (src/MotionOptimization.cu:163-181)
    for (long i = 0; i < c; ++i) {
        const real* v = warped + 3 * (long)corr[2 * i];
        const real* f = frame_mesh + 3 * (long)corr[2 * i + 1];
        const real* n = normals + 3 * (long)corr[2 * i + 1];
        real d[3] = {v[0] - f[0], v[1] - f[1], v[2] - f[2]};
        r[i] = lambda * dot3(n, d);
    }
}

void vfo_residual_reg(real* r, const real* nodes, const real* T, int n, const uint32_t* gidx, int kreg,
                      real lambda) {
    // fill_r_MRegKernel (src/MotionOptimization.cu:198-227); rows of invalid slots are left untouched (zero)
    for (int i = 0; i < n; ++i) {
        real tc[3];
        mat4_point(T + 16 * (size_t)i, nodes + 3 * i, tc);
        for (int k = 0; k < kreg; ++k) {
            uint32_t nb = gidx[i * kreg + k];
            if (nb >= (uint32_t)n) continue;
            real tn[3];
            mat4_point(T + 16 * (size_t)nb, nodes + 3 * i, tn);
            long row = ((long)i * kreg + k) * 3;
            for (int a = 0; a < 3; ++a) r[row + a] = (tc[a] - tn[a]) * lambda;
        }
    }
}

double vfo_energy(const real* r, long n) {
    // runSquareKernel + thrust::reduce (src/VolumeFusion.cu:585-588), accumulated in FP64
    double e = 0;
    for (long i = 0; i < n; ++i) e += (double)(r[i] * r[i]);
    return e;
}

// d(T p)/d xi rows for the additive update (gradOfTransfVertex, src/MotionOptimization.cu:10-26)
static void grad_rows(const real* p, real G[3][6]) {
    const real Gv[3][6] = {{0, p[2], -p[1], 1, 0, 0}, {-p[2], 0, p[0], 0, 1, 0}, {p[1], -p[0], 0, 0, 0, 1}};
    std::memcpy(G, Gv, sizeof(Gv));
}

int vfo_assemble(double* jtj_dense, real* jtj_blocks, real* jtr, const int* corr, long c, const real* canon,
                 const uint32_t* midx, const real* mw, int k, const real* normals, real lambda_d,
                 const real* nodes, int n, const uint32_t* gidx, int kreg, real lambda_r, const real* r_depth,
                 const real* r_reg) {
    // J^T J and J^T r as assembled by runFill_J_*, runComputeJTJAndJTrContrib*, runMultiply*, reduce_by_key
    // and runFillJTJKernel/runFillJTrKernel (src/MotionOptimization.cu:29-481, src/VolumeFusion.cu:469-646).
    // Per block the contributions are summed in binary32 in the order: depth rows by ascending
    // correspondence, then regularisation rows by ascending row.  Diagonal blocks that receive no
    // contribution keep the identity written by runInitIdentityKernel.  jtj_blocks (optional) is
    // the dense (6n)^2 real matrix, row-major; jtj_dense (optional) is the same in double.
    const long dim = 6L * n;
    std::vector<real> A((size_t)dim * dim, 0.f);
    std::vector<char> touched((size_t)n * n, 0);
    std::vector<real> b((size_t)dim, 0.f);
    auto add_block = [&](int a, int bb, const real* Ja, const real* Jb) {
        touched[(size_t)a * n + bb] = 1;
        for (int i = 0; i < 6; ++i)
            for (int j = 0; j < 6; ++j) {
                real& e = A[(size_t)(6 * a + i) * dim + 6 * bb + j];
                e = e + Ja[i] * Jb[j];
            }
    };
    for (long ci = 0; ci < c; ++ci) {
        int vi = corr[2 * ci], pi = corr[2 * ci + 1];
        const real* nrm = normals + 3 * (long)pi;
        real G[3][6];
        grad_rows(canon + 3 * (long)vi, G);
        real J[32][6];
        for (int s = 0; s < k; ++s) {
            real wgt = mw[(long)vi * k + s];
            for (int q = 0; q < 6; ++q) J[s][q] = 0.f;
            if (wgt < 1.e-4f) continue;
            real nw[3] = {nrm[0] * wgt, nrm[1] * wgt, nrm[2] * wgt};
            for (int q = 0; q < 6; ++q) J[s][q] = (nw[0] * G[0][q] + (nw[1] * G[1][q] + nw[2] * G[2][q])) * lambda_d;
        }
        for (int s = 0; s < k; ++s) {
            if (mw[(long)vi * k + s] == 0.f) continue;
            uint32_t a = midx[(long)vi * k + s];
            for (int t = s; t < k; ++t) {
                if (mw[(long)vi * k + t] == 0.f) continue;
                uint32_t bb = midx[(long)vi * k + t];
                if (a <= bb) add_block((int)a, (int)bb, J[s], J[t]);
                else add_block((int)bb, (int)a, J[t], J[s]);
            }
            for (int q = 0; q < 6; ++q) b[6 * a + q] = b[6 * a + q] + J[s][q] * r_depth[ci];
        }
    }
    for (int i = 0; i < n; ++i) {
        real G[3][6];
        grad_rows(nodes + 3 * i, G);
        for (int kk = 0; kk < kreg; ++kk) {
            uint32_t nb = gidx[i * kreg + kk];
            if (nb >= (uint32_t)n) continue;
            for (int ax = 0; ax < 3; ++ax) {
                long row = ((long)i * kreg + kk) * 3 + ax;
                real g[6], gn[6];
                for (int q = 0; q < 6; ++q) {
                    g[q] = G[ax][q] * lambda_r;
                    gn[q] = -g[q];
                }
                if ((uint32_t)i < nb) add_block(i, (int)nb, g, gn);
                else add_block((int)nb, i, gn, g);
                add_block(i, i, g, g);
                add_block((int)nb, (int)nb, gn, gn);
                for (int q = 0; q < 6; ++q) {
                    b[6 * i + q] = b[6 * i + q] + g[q] * r_reg[row];
                    b[6 * nb + q] = b[6 * nb + q] + gn[q] * r_reg[row];
                }
            }
        }
    }
    int empty = 0;
    for (int a = 0; a < n; ++a) {
        if (!touched[(size_t)a * n + a]) {
            ++empty;
            for (int i = 0; i < 6; ++i) A[(size_t)(6 * a + i) * dim + 6 * a + i] = 1.f;
        }
        for (int bb = a + 1; bb < n; ++bb) {
            if (!touched[(size_t)a * n + bb]) continue;
            for (int i = 0; i < 6; ++i)
                for (int j = 0; j < 6; ++j)
                    A[(size_t)(6 * bb + i) * dim + 6 * a + j] = A[(size_t)(6 * a + j) * dim + 6 * bb + i];
        }
    }
    if (jtj_blocks) std::memcpy(jtj_blocks, A.data(), sizeof(real) * A.size());
    if (jtj_dense)
        for (size_t i = 0; i < A.size(); ++i) jtj_dense[i] = (double)A[i];
    if (jtr) std::memcpy(jtr, b.data(), sizeof(real) * b.size());
    return empty;
}

int vfo_solve_dense(const double* A, const real* b, int dim, double* x) {
    // FP64 Cholesky in place of the reference's FP32 cuSOLVER LU (src/LinearSolver.cu:179-224)
    std::vector<double> L((size_t)dim * dim, 0.0);
    for (int j = 0; j < dim; ++j) {
        double s = A[(size_t)j * dim + j];
        for (int p = 0; p < j; ++p) s -= L[(size_t)j * dim + p] * L[(size_t)j * dim + p];
        if (!(s > 0)) return 1;
        double d = std::sqrt(s);
        L[(size_t)j * dim + j] = d;
        for (int i = j + 1; i < dim; ++i) {
            double t = A[(size_t)i * dim + j];
            for (int p = 0; p < j; ++p) t -= L[(size_t)i * dim + p] * L[(size_t)j * dim + p];
            L[(size_t)i * dim + j] = t / d;
        }
    }
    std::vector<double> y(dim);
    for (int i = 0; i < dim; ++i) {
        double s = b[i];
        for (int p = 0; p < i; ++p) s -= L[(size_t)i * dim + p] * y[p];
        y[i] = s / L[(size_t)i * dim + i];
    }
    for (int i = dim - 1; i >= 0; --i) {
        double s = y[i];
        for (int p = i + 1; p < dim; ++p) s -= L[(size_t)p * dim + i] * x[p];
        x[i] = s / L[(size_t)i * dim + i];
    }
    return 0;
}

static bool inv6(const double* M, double* Minv) {
    double a[6][12];
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 12; ++j) a[i][j] = (j < 6) ? M[i * 6 + j] : (j - 6 == i ? 1.0 : 0.0);
    for (int c = 0; c < 6; ++c) {
        int p = c;
        for (int r = c + 1; r < 6; ++r)
            if (std::fabs(a[r][c]) > std::fabs(a[p][c])) p = r;
        if (a[p][c] == 0.0) return false;
        if (p != c)
            for (int j = 0; j < 12; ++j) std::swap(a[p][j], a[c][j]);
        double d = a[c][c];
        for (int j = 0; j < 12; ++j) a[c][j] /= d;
        for (int r = 0; r < 6; ++r)
            if (r != c) {
                double f = a[r][c];
                for (int j = 0; j < 12; ++j) a[r][j] -= f * a[c][j];
            }
    }
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 6; ++j) Minv[i * 6 + j] = a[i][j + 6];
    return true;
}

int vfo_pcg(const double* A, const real* b, int n, int iters, double tol, double* x, int* iters_done) {
    // Block-Jacobi preconditioned conjugate gradients in FP64 (reference point for the GPU solver)
    const int dim = 6 * n;
    std::vector<double> Minv((size_t)n * 36), r(dim), z(dim), p(dim), Ap(dim);
    for (int a = 0; a < n; ++a) {
        double blk[36];
        for (int i = 0; i < 6; ++i)
            for (int j = 0; j < 6; ++j) blk[i * 6 + j] = A[(size_t)(6 * a + i) * dim + 6 * a + j];
        if (!inv6(blk, &Minv[(size_t)a * 36])) return 1;
    }
    auto precond = [&](const std::vector<double>& in, std::vector<double>& out) {
        for (int a = 0; a < n; ++a)
            for (int i = 0; i < 6; ++i) {
                double s = 0;
                for (int j = 0; j < 6; ++j) s += Minv[(size_t)a * 36 + i * 6 + j] * in[6 * a + j];
                out[6 * a + i] = s;
            }
    };
    double bn = 0;
    for (int i = 0; i < dim; ++i) {
        x[i] = 0;
        r[i] = b[i];
        bn += r[i] * r[i];
    }
    bn = std::sqrt(bn);
    precond(r, z);
    p = z;
    double rz = 0;
    for (int i = 0; i < dim; ++i) rz += r[i] * z[i];
    int it = 0;
    for (; it < iters; ++it) {
        double rn = 0;
        for (int i = 0; i < dim; ++i) rn += r[i] * r[i];
        if (std::sqrt(rn) <= tol * bn) break;
        for (int i = 0; i < dim; ++i) {
            double s = 0;
            for (int j = 0; j < dim; ++j) s += A[(size_t)i * dim + j] * p[j];
            Ap[i] = s;
        }
        double pAp = 0;
        for (int i = 0; i < dim; ++i) pAp += p[i] * Ap[i];
        if (pAp == 0) break;
        double alpha = rz / pAp;
        for (int i = 0; i < dim; ++i) {
            x[i] += alpha * p[i];
            r[i] -= alpha * Ap[i];
        }
        precond(r, z);
        double rz2 = 0;
        for (int i = 0; i < dim; ++i) rz2 += r[i] * z[i];
        double beta = rz2 / rz;
        rz = rz2;
        for (int i = 0; i < dim; ++i) p[i] = z[i] + beta * p[i];
    }
    if (iters_done) *iters_done = it;
    return 0;
}

void vfo_update_transforms(real* T, const real* x, int n) {
    // updateTransformsKernel (src/MotionOptimization.cu:483-498): T <- T - [[xi_rot]x, xi_t; 0 0 0 0]
    for (int i = 0; i < n; ++i) {
        const real* u = x + 6 * i;
        real* t = T + 16 * (size_t)i;
        const real U[16] = {0, u[2], -u[1], 0, -u[2], 0, u[0], 0, u[1], -u[0], 0, 0, u[3], u[4], u[5], 0};  // column-major
        for (int e = 0; e < 16; ++e) t[e] = t[e] - U[e];
    }
}

// ---- voxel warp and warped integration ----

void vfo_tsdf_knn(uint32_t* kidx, real* kdist, int* kcount, const real* nodes, const real* radii, int n,
                  const real vs[3], const real size[3], const int dims[3], const int per_node[3], int k) {
    // tsdfKNNGraph (src/TSDFWarp.cu:23-68).  Support: voxels of the node's cube within 2*radius.
    // Slot rule: the K nearest supporting nodes, ordered by (distance, node index); the reference
    // keeps the first K to arrive, so the two agree whenever a voxel has at most K supporters.
    const int X = dims[0], Y = dims[1], Z = dims[2];
    const long S = (long)X * Y * Z;
    std::vector<int> tot(S, 0);
    std::vector<Cand> best((size_t)S * k);
    for (int j = 0; j < n; ++j) {
        const real* nd = nodes + 3 * j;
        int nv[3];
        world_to_voxel(nd, vs, size, nv);
        for (int oz = 0; oz < per_node[2]; ++oz)
            for (int oy = 0; oy < per_node[1]; ++oy)
                for (int ox = 0; ox < per_node[0]; ++ox) {
                    int v[3] = {nv[0] - (per_node[0] - 1) / 2 + ox, nv[1] - (per_node[1] - 1) / 2 + oy,
                                nv[2] - (per_node[2] - 1) / 2 + oz};
                    if (v[0] < 0 || v[1] < 0 || v[2] < 0 || v[0] >= X || v[1] >= Y || v[2] >= Z) continue;
                    real tp[3];
                    voxel_to_world(v[0], v[1], v[2], vs, size, tp);
                    real d3[3] = {tp[0] - nd[0], tp[1] - nd[1], tp[2] - nd[2]};
                    real dist = norm3(d3);
                    if (dist > radii[j] * 2.0f) continue;
                    long id = (long)v[2] * X * Y + (long)v[1] * X + v[0];
                    int cnt = std::min(tot[id], k);
                    topk_insert(&best[(size_t)id * k], cnt, k, Cand{dist, (uint32_t)j});
                    tot[id]++;
                }
    }
    for (long id = 0; id < S; ++id) {
        int cnt = std::min(tot[id], k);
        kcount[id] = cnt;
        for (int s = 0; s < k; ++s) {
            if (s < cnt) {
                kidx[id * k + s] = best[(size_t)id * k + s].idx;
                kdist[id * k + s] = best[(size_t)id * k + s].key;
            } else {
                kidx[id * k + s] = VFO_INVALID_IDX;
                kdist[id * k + s] = kFltMax;
            }
        }
    }
}

void vfo_tsdf_weights(real* kw, const real* radii, const uint32_t* kidx, const real* kdist, const int* kcount,
                      long s, int k) {
    // computeTsdfWarpWeightsKernel (src/TSDFWarp.cu:88-116): no distance cut-off; zero for empty voxels
#pragma omp parallel for schedule(static)
    for (long i = 0; i < s; ++i) {
        real* w = kw + i * k;
        for (int j = 0; j < k; ++j) w[j] = 0.f;
        int cnt = kcount[i];
        if (!cnt) continue;
        real sum = 0;
        for (int j = 0; j < cnt; ++j) {
            real r = radii[kidx[i * k + j]], d = kdist[i * k + j];
            w[j] = vexp(-(d * d) / (2.0f * (r * r)));
            sum += w[j];
        }
        if (sum != 0.f)
            for (int j = 0; j < k; ++j) w[j] = w[j] / sum;
    }
}

void vfo_tsdf_vertices(real* verts, const real vs[3], const real size[3], const int dims[3]) {
    // generateTsdfVerticesKernel (src/TSDFWarp.cu:131-145)
    const int X = dims[0], Y = dims[1], Z = dims[2];
#pragma omp parallel for schedule(static)
    for (int z = 0; z < Z; ++z)
        for (int y = 0; y < Y; ++y)
            for (int x = 0; x < X; ++x) voxel_to_world(x, y, z, vs, size, verts + 3 * ((long)z * X * Y + (long)y * X + x));
}

void vfo_warp_tsdf(real* verts, const real* T, const uint32_t* kidx, const real* kw, const int* kcount, long s,
                   int k) {
    // warpTsdfKernel (src/TSDFWarp.cu:158-190)
#pragma omp parallel for schedule(static)
    for (long i = 0; i < s; ++i) {
        int cnt = kcount[i];
        if (!cnt) continue;
        const real* w = kw + i * k;
        bool zero = true;
        for (int j = 0; j < k; ++j)
            if (!(std::fabs(w[j]) <= 1e-5f)) zero = false;
        if (zero) continue;
        real p[3];
        std::memcpy(p, verts + 3 * i, 3 * sizeof(real));
        real acc[3] = {0.f, 0.f, 0.f};
        for (int j = 0; j < cnt; ++j) {
            real q[3];
            mat4_point(T + 16 * (size_t)kidx[i * k + j], p, q);
            for (int c = 0; c < 3; ++c) acc[c] = acc[c] + w[j] * q[c];
        }
        std::memcpy(verts + 3 * i, acc, 3 * sizeof(real));
    }
}

static bool warped_target(const real* wp, const real* vs, const real* size, const int* dims, const real* Rinv,
                          const real* t, long* target) {
    real d[3] = {wp[0] - t[0], wp[1] - t[1], wp[2] - t[2]};
    real o[3];
    mat3_vec3(Rinv, d, o);
    int v[3];
    world_to_voxel(o, vs, size, v);
    if (v[0] < 0 || v[1] < 0 || v[2] < 0 || v[0] >= dims[0] || v[1] >= dims[1] || v[2] >= dims[2]) return false;
    *target = (long)v[2] * dims[0] * dims[1] + (long)v[1] * dims[0] + v[0];
    return true;
}

void vfo_count_collisions(int* counts, const real* verts, const int* kcount, const real vs[3], const real size[3],
                          const int dims[3], const real Rinv[9], const real t[3]) {
    // countCollisionsPerVoxelKernel (src/TSDFIntegration.cu:252-283)
    const long S = (long)dims[0] * dims[1] * dims[2];
#pragma omp parallel for schedule(static)
    for (long i = 0; i < S; ++i) {
        if (!kcount[i]) continue;
        long tg;
        if (!warped_target(verts + 3 * i, vs, size, dims, Rinv, t, &tg)) continue;
#pragma omp atomic
        counts[tg]++;
    }
}

void vfo_integrate_warped(real* tsdf, real* weights, const real* verts, const int* collisions, const int* kcount,
                          const real* depth, int width, int height, real delta, const real vs[3],
                          const real size[3], const int dims[3], const real Rinv[9], const real t[3],
                          const real K[9], int half) {
    // integrateWarpedTSDFFromFrameKernel (src/TSDFIntegration.cu:173-226)
    const long S = (long)dims[0] * dims[1] * dims[2];
#pragma omp parallel for schedule(static)
    for (long i = 0; i < S; ++i) {
        if (!kcount[i]) continue;
        long tg;
        if (!warped_target(verts + 3 * i, vs, size, dims, Rinv, t, &tg)) continue;
        if (collisions[tg] > 1) continue;
        update_tsdf(tsdf, weights, verts + 3 * i, i, depth, width, height, delta, K, half);
    }
}

}  // extern "C"

// ---- whole-frame driver ----

struct vfo_fusion {
    vfo_params p;
    long S = 0, P = 0;
    real vs[3] = {0, 0, 0};
    real K[9], vsize[3];  // f->K and f->vsize in the arithmetic type
    int frame = 0;
    std::vector<real> tsdf, weights;
    std::vector<real> depth, verts, normals;
    std::vector<uint32_t> umap;  // cv::undistort map of a distorted camera
    real c0[3] = {0, 0, 0};
    int n = 0;
    std::vector<real> nodes_host, nodes_dev, radii, T;
    std::vector<real> mesh, mesh_out;
    long m = 0, mesh_out_n = 0, ncorr = 0;
    int gn_done = 0;
    double energy = 0;
};

extern "C" {

vfo_fusion* vfo_fusion_create(const vfo_params* p) {
    vfo_fusion* f = new vfo_fusion();
    f->p = *p;
    f->S = (long)p->dims[0] * p->dims[1] * p->dims[2];
    f->P = (long)p->width * p->height;
    for (int c = 0; c < 3; ++c) f->vs[c] = (real)p->volume_size[c] / (real)p->dims[c];
    for (int c = 0; c < 9; ++c) f->K[c] = (real)p->K[c];
    for (int c = 0; c < 3; ++c) f->vsize[c] = (real)p->volume_size[c];
    f->tsdf.assign(f->S, -1.f);
    f->weights.assign(f->S, 0.f);
    f->depth.resize(f->P);
    f->verts.resize(3 * f->P);
    f->normals.resize(3 * f->P);
    f->nodes_host.resize(3 * (size_t)p->node_cap);
    f->nodes_dev.resize(3 * (size_t)p->node_cap);
    f->radii.resize(p->node_cap);
    f->T.resize(16 * (size_t)p->node_cap);
    if (p->distorted) {
        f->umap.resize(2 * (size_t)f->P);
        vfo_undistort_map(f->umap.data(), p->width, p->height, p->K, p->dist_cv, 0);
    }
    return f;
}

void vfo_fusion_destroy(vfo_fusion* f) { delete f; }

int vfo_fusion_process(vfo_fusion* f, const uint16_t* depth_mm) {
    // af::runVolumeFusion per-frame loop (src/VolumeFusion.cu:327-769)
    const vfo_params& p = f->p;
    static const real I3[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    real cen[3];
    if (p.distorted)
        vfo_frame_prep_undistorted(depth_mm, p.width, p.height, f->K, p.depth_threshold, p.bilateral, p.bilateral_r,
                                   p.sigma_i, p.sigma_s, p.bilateral_thr, p.angle_lo, p.angle_hi, f->umap.data(),
                                   f->depth.data(), f->verts.data(), f->normals.data(), cen);
    else
        vfo_frame_prep(depth_mm, p.width, p.height, f->K, p.depth_threshold, p.bilateral, p.bilateral_r, p.sigma_i,
                       p.sigma_s, p.bilateral_thr, p.angle_lo, p.angle_hi, f->depth.data(), f->verts.data(),
                       f->normals.data(), cen);
    if (f->frame == 0) {
        std::memcpy(f->c0, cen, 3 * sizeof(real));
        vfo_integrate_rigid(f->tsdf.data(), f->weights.data(), f->depth.data(), p.width, p.height, p.delta, p.dims,
                            f->vs, f->vsize, I3, f->c0, f->K, p.precision);
        f->frame++;
        return 0;
    }
    // canonical point cloud: MC point cloud, sort + unique, translate by the frame-0 centroid (:372-389)
    f->mesh.resize(3 * (size_t)p.mesh_cap);
    long raw = vfo_mc_pointcloud(f->tsdf.data(), f->weights.data(), p.dims, f->vs, f->vsize, 0.f,
                                 f->mesh.data(), p.mesh_cap);
    if (raw > p.mesh_cap) return -2;
    f->m = vfo_sort_unique_vec3(f->mesh.data(), raw);
    vfo_translate(f->mesh.data(), f->m, f->c0);
    const long m = f->m;
    // motion graph (:392-404)
    int n_old = f->n;
    if (f->frame == 1 || p.update_graph) {
        int nn = vfo_build_graph(f->nodes_host.data(), f->radii.data(), f->T.data(), f->n, p.node_cap, f->mesh.data(),
                                 m, p.knn, p.graph_radius);
        if (nn < 0) return -3;
        f->n = nn;
    }
    const int n = f->n;
    std::memcpy(f->nodes_dev.data() + 3 * n_old, f->nodes_host.data() + 3 * n_old, 3 * sizeof(real) * (size_t)(n - n_old));
    // KNN (:410-419)
    std::vector<uint32_t> midx((size_t)m * p.knn), gidx((size_t)n * p.kreg);
    std::vector<real> mdist((size_t)m * p.knn), gdist((size_t)n * p.kreg), mw((size_t)m * p.knn);
    vfo_knn(f->nodes_host.data(), n, f->mesh.data(), m, p.knn, 0, midx.data(), mdist.data());
    vfo_knn(f->nodes_host.data(), n, f->nodes_host.data(), n, p.kreg, 1, gidx.data(), gdist.data());
    vfo_filter_disconnected(gidx.data(), gdist.data(), n, p.kreg, f->radii.data());
    vfo_warp_weights(mw.data(), f->radii.data(), midx.data(), mdist.data(), m, p.knn, n);
    std::vector<real> warped(3 * (size_t)m);
    (p.blend ? vfo_warp_dqb : vfo_warp)(warped.data(), f->mesh.data(), m, f->T.data(), midx.data(), mw.data(), p.knn);
    // ICP / Gauss-Newton (:434-691)
    std::vector<real> pending(f->T.size());
    f->gn_done = 0;
    for (int icp = 0; icp < p.icp_iterations; ++icp) {
        (p.blend ? vfo_warp_dqb : vfo_warp)(warped.data(), f->mesh.data(), m, f->T.data(), midx.data(), mw.data(), p.knn);
        std::vector<int> corr(2 * (size_t)m);
        long c = vfo_correspondences(corr.data(), m, warped.data(), m, f->K, f->depth.data(), p.height, p.width,
                                     f->verts.data(), p.corr_thresh);
        f->ncorr = c;
        const long jreg = (long)n * p.kreg * 3;
        std::vector<real> rd(c), rr(jreg);
        std::vector<double> A((size_t)36 * n * n);
        std::vector<real> b(6 * (size_t)n), xf(6 * (size_t)n);
        std::vector<double> x(6 * (size_t)n);
        std::copy(f->T.begin(), f->T.begin() + 16 * (size_t)n, pending.begin());
        double E = (double)kFltMax;
        for (int gn = 0; gn < p.gn_iterations; ++gn) {
            vfo_residual_depth(rd.data(), corr.data(), c, warped.data(), f->verts.data(), f->normals.data(),
                               p.lambda_depth);
            std::fill(rr.begin(), rr.end(), 0.f);
            vfo_residual_reg(rr.data(), f->nodes_dev.data(), pending.data(), n, gidx.data(), p.kreg, p.lambda_reg);
            double e = vfo_energy(rd.data(), c) + vfo_energy(rr.data(), jreg);
            f->energy = e;
            if (E - e < (double)p.energy_min_step) break;
            E = e;
            if (gn != 0) std::copy(pending.begin(), pending.begin() + 16 * (size_t)n, f->T.begin());
            vfo_assemble(A.data(), nullptr, b.data(), corr.data(), c, f->mesh.data(), midx.data(), mw.data(), p.knn,
                         f->normals.data(), p.lambda_depth, f->nodes_dev.data(), n, gidx.data(), p.kreg, p.lambda_reg,
                         rd.data(), rr.data());
            int st;
            if (p.solver == 0) st = vfo_solve_dense(A.data(), b.data(), 6 * n, x.data());
            else st = vfo_pcg(A.data(), b.data(), n, p.pcg_iterations, p.pcg_tol, x.data(), nullptr);
            if (st) return -4;
            for (int i = 0; i < 6 * n; ++i) xf[i] = (real)x[i];
            vfo_update_transforms(pending.data(), xf.data(), n);
            (p.blend ? vfo_warp_dqb : vfo_warp)(warped.data(), f->mesh.data(), m, pending.data(), midx.data(), mw.data(),
                                                p.knn);
            f->gn_done = gn + 1;
        }
    }
    // voxel KNN, warp and warped integration (:702-741)
    int per[3];
    for (int c = 0; c < 3; ++c) per[c] = 2 * (vfo_f2i_rz(p.graph_radius / f->vs[c]) + 1) + 1;
    const real negc[3] = {-f->c0[0], -f->c0[1], -f->c0[2]};
    vfo_translate(f->nodes_dev.data(), n, negc);
    const long S = f->S;
    std::vector<uint32_t> kidx((size_t)S * p.knn);
    std::vector<real> kdist((size_t)S * p.knn), kw((size_t)S * p.knn), tv(3 * (size_t)S);
    std::vector<int> kcount(S), coll(S, 0);
    vfo_tsdf_knn(kidx.data(), kdist.data(), kcount.data(), f->nodes_dev.data(), f->radii.data(), n, f->vs,
                 f->vsize, p.dims, per, p.knn);
    vfo_tsdf_weights(kw.data(), f->radii.data(), kidx.data(), kdist.data(), kcount.data(), S, p.knn);
    vfo_tsdf_vertices(tv.data(), f->vs, f->vsize, p.dims);
    vfo_translate(f->nodes_dev.data(), n, f->c0);
    vfo_translate(tv.data(), S, f->c0);
    if (p.blend) {
        // dual-quaternion blend of each supported voxel's nodes (its kcount slots)
#pragma omp parallel for schedule(static)
        for (long i = 0; i < S; ++i) {
            if (!kcount[i]) continue;
            real c[3] = {tv[3 * i], tv[3 * i + 1], tv[3 * i + 2]};
            dq_point(f->T.data(), kidx.data() + i * p.knn, kw.data() + i * p.knn, kcount[i], c, tv.data() + 3 * i);
        }
    } else {
        vfo_warp_tsdf(tv.data(), f->T.data(), kidx.data(), kw.data(), kcount.data(), S, p.knn);
    }
    vfo_count_collisions(coll.data(), tv.data(), kcount.data(), f->vs, f->vsize, p.dims, I3, f->c0);
    if (p.integrate)
        vfo_integrate_warped(f->tsdf.data(), f->weights.data(), tv.data(), coll.data(), kcount.data(), f->depth.data(),
                             p.width, p.height, p.delta, f->vs, f->vsize, p.dims, I3, f->c0, f->K, p.precision);
    f->frame++;
    return 0;
}

int vfo_fusion_num_nodes(const vfo_fusion* f) { return f->n; }
long vfo_fusion_mesh_size(const vfo_fusion* f) { return f->m; }
long vfo_fusion_num_corr(const vfo_fusion* f) { return f->ncorr; }
int vfo_fusion_gn_done(const vfo_fusion* f) { return f->gn_done; }
double vfo_fusion_energy(const vfo_fusion* f) { return f->energy; }
const real* vfo_fusion_tsdf(const vfo_fusion* f) { return f->tsdf.data(); }
const real* vfo_fusion_weights(const vfo_fusion* f) { return f->weights.data(); }
const real* vfo_fusion_nodes(const vfo_fusion* f) { return f->nodes_host.data(); }
const real* vfo_fusion_transforms(const vfo_fusion* f) { return f->T.data(); }
const real* vfo_fusion_centroid(const vfo_fusion* f) { return f->c0; }
const real* vfo_fusion_mesh(const vfo_fusion* f) { return f->mesh.data(); }
void vfo_fusion_set_transforms(vfo_fusion* f, const real* T, int n) {
    std::memcpy(f->T.data(), T, 16 * sizeof(real) * (size_t)std::min(n, f->n));
}

void vfo_fusion_set_tsdf(vfo_fusion* f, const real* tsdf, const real* weights) {
    std::memcpy(f->tsdf.data(), tsdf, sizeof(real) * f->S);
    std::memcpy(f->weights.data(), weights, sizeof(real) * f->S);
}

}  // extern "C"
