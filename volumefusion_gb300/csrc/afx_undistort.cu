// afx_undistort.cu -- depth undistortion on the device: the per-pixel source maps of the reference's
// two OpenCV undistortions, their application to a float depth image, and the Brown-Conrady
// unprojection of src/CameraCalibration.cpp.
//
// Undistortion maps.  Both reference call sites build an OpenCV map with the intrinsics as the new
// camera matrix and the identity rectification, from a camera matrix holding only fx, fy, cx, cy
// and K(2,2) (src/VolumeFusion.cu:163-170, src/MeshRecontructionStream.cu:66-71):
//   - af::loadProcessFrame (src/VolumeFusion.cu:179) calls cv::undistort: fixed-point maps (CV_16SC2
//     + CV_16UC1, 1/32 pixel) computed in stripes of max(1, 4096 / width) rows -- each stripe with the
//     new camera matrix's cy lowered by the stripe's first row -- then cv::remap INTER_LINEAR with a
//     zero border;
//   - the stream readers (src/MeshRecontructionStream.cu:97-99, src/PointCloudStream.cu:111-113) call
//     cv::initUndistortRectifyMap(..., CV_32FC1) once over the whole image and cv::remap
//     INTER_NEAREST with a zero border.
// The map arithmetic restates OpenCV's initUndistortRectifyMap (calib3d, scalar path) in binary64:
// iR = inverse(newK) by the closed-form 3x3 inverse of cv::invert, per row the homogeneous
// coordinates start at i * ir[1] + ir[2] (and likewise for y and w) and advance by ir[0] / ir[3] /
// ir[6] per column; per pixel x = _x / _w, y = _y / _w, the rational radial factor
// kr = (1 + ((k3 r2 + k2) r2 + k1) r2) / (1 + ((k6 r2 + k5) r2 + k4) r2), the tangential terms, and
// u = fx xd + cx, v = fy yd + cy.  The fixed-point map is round(u * 32) split into the integer pixel
// (arithmetic shift) and the 5 + 5 fractional bits; the float map is rounded to the nearest pixel
// (ties to even) and saturated to int16 when remapped.  The map is built once per camera.
#include <climits>
#include <cstring>

#include "afx_internal.h"
#include "afx_undistort.cuh"

namespace afx {

namespace {

struct MapArgs {
    double A[9];        // camera matrix, row-major, binary64
    double k[8];        // k1 k2 p1 p2 k3 k4 k5 k6 (OpenCV order)
    int width, height;
    int stripe;         // rows per map stripe (LINEAR), or the image height (NEAREST)
    int mode;
};

// cv::invert (DECOMP_LU, n = 3, binary64): adjugate times the reciprocal of the determinant; a zero
// matrix when the determinant is 0.
AFX_D void inverse3(const double* m, double* t) {
    const double det = m[0] * (m[4] * m[8] - m[5] * m[7]) - m[1] * (m[3] * m[8] - m[5] * m[6]) +
                       m[2] * (m[3] * m[7] - m[4] * m[6]);
    if (det == 0.0) {
        for (int i = 0; i < 9; ++i) t[i] = 0.0;
        return;
    }
    const double d = 1.0 / det;
    t[0] = (m[4] * m[8] - m[5] * m[7]) * d;
    t[1] = (m[2] * m[7] - m[1] * m[8]) * d;
    t[2] = (m[1] * m[5] - m[2] * m[4]) * d;
    t[3] = (m[5] * m[6] - m[3] * m[8]) * d;
    t[4] = (m[0] * m[8] - m[2] * m[6]) * d;
    t[5] = (m[2] * m[3] - m[0] * m[5]) * d;
    t[6] = (m[3] * m[7] - m[4] * m[6]) * d;
    t[7] = (m[1] * m[6] - m[0] * m[7]) * d;
    t[8] = (m[0] * m[4] - m[1] * m[3]) * d;
}

// cvRound on x86-64 (cvtsd2si / cvtss2si): nearest, ties to even; NaN and values outside int32 give
// INT_MIN.
AFX_D int round_to_int(double v) { return (v >= -2147483648.5 && v < 2147483647.5) ? __double2int_rn(v) : INT_MIN; }
AFX_D int round_to_int(float v) { return (v >= -2147483648.f && v < 2147483648.f) ? __float2int_rn(v) : INT_MIN; }
AFX_D int saturate_short(int v) { return v < -32768 ? -32768 : (v > 32767 ? 32767 : v); }
AFX_D uint32_t pack_xy(int sx, int sy) { return (uint32_t)(uint16_t)(int16_t)sx | ((uint32_t)(uint16_t)(int16_t)sy << 16); }

// One block per row.  The row's homogeneous coordinates are OpenCV's running sums (one addition per
// column, in column order), so thread 0 walks them kMapChunk columns at a time into shared memory and
// the block then maps those columns in parallel: the same values, pixel by pixel, as the sequential
// loop, at the cost of one serial addition chain per row.
constexpr int kMapChunk = 256;

__global__ void __launch_bounds__(kMapChunk) undistort_map_kernel(uint32_t* map, MapArgs a) {
    __shared__ double sx[kMapChunk], sy[kMapChunk], sw[kMapChunk];
    __shared__ double ir[9];
    const int i = blockIdx.x;  // row
    if (i >= a.height) return;
    const int y0 = (i / a.stripe) * a.stripe;  // first row of this row's stripe
    if (threadIdx.x == 0) {
        double Ar[9];
        for (int q = 0; q < 9; ++q) Ar[q] = a.A[q];
        if (a.mode == AFX_UNDISTORT_LINEAR) Ar[5] = a.A[5] - (double)y0;  // cv::undistort: Ar(1,2) = v0 - y
        inverse3(Ar, ir);
    }
    __syncthreads();
    const double u0 = a.A[2], v0 = a.A[5], fx = a.A[0], fy = a.A[4];
    const double k1 = a.k[0], k2 = a.k[1], p1 = a.k[2], p2 = a.k[3], k3 = a.k[4], k4 = a.k[5], k5 = a.k[6], k6 = a.k[7];
    const int row = a.mode == AFX_UNDISTORT_LINEAR ? i - y0 : i;
    double X = row * ir[1] + ir[2], Y = row * ir[4] + ir[5], Wh = row * ir[7] + ir[8];  // thread 0's running sums
    uint32_t* out = map + 2 * (size_t)i * a.width;
    for (int j0 = 0; j0 < a.width; j0 += kMapChunk) {
        const int n = min(kMapChunk, a.width - j0);
        if (threadIdx.x == 0) {
            for (int t = 0; t < n; ++t, X += ir[0], Y += ir[3], Wh += ir[6]) {
                sx[t] = X;
                sy[t] = Y;
                sw[t] = Wh;
            }
        }
        __syncthreads();
        const int t = threadIdx.x;
        if (t < n) {
            const int j = j0 + t;
            const double w = 1. / sw[t], x = sx[t] * w, y = sy[t] * w;
            const double x2 = x * x, y2 = y * y;
            const double r2 = x2 + y2, _2xy = 2 * x * y;
            const double kr = (1 + ((k3 * r2 + k2) * r2 + k1) * r2) / (1 + ((k6 * r2 + k5) * r2 + k4) * r2);
            const double xd = x * kr + p1 * _2xy + p2 * (r2 + 2 * x2);
            const double yd = y * kr + p1 * (r2 + 2 * y2) + p2 * _2xy;
            const double u = fx * xd + u0, v = fy * yd + v0;
            if (a.mode == AFX_UNDISTORT_LINEAR) {
                const int iu = round_to_int(u * 32.0), iv = round_to_int(v * 32.0);
                out[2 * j] = pack_xy((int)(int16_t)(iu >> 5), (int)(int16_t)(iv >> 5));
                out[2 * j + 1] = (uint32_t)((iv & 31) * 32 + (iu & 31));
            } else {
                const float fu = (float)u, fv = (float)v;
                out[2 * j] = pack_xy(saturate_short(round_to_int(fu)), saturate_short(round_to_int(fv)));
                out[2 * j + 1] = 0u;
            }
        }
        __syncthreads();
    }
}

__global__ void undistort_apply_kernel(float* dst, const float* __restrict__ src, const uint32_t* __restrict__ map,
                                       int W, int H, int mode) {
    const long n = (long)W * H;
    auto at = [&](int x, int y) { return src[(long)y * W + x]; };
    AFX_GRID_STRIDE(p, n) {
        const uint32_t w0 = map[2 * p];
        dst[p] = mode == AFX_UNDISTORT_LINEAR ? remap_linear_at(w0, map[2 * p + 1], W, H, at)
                                              : remap_nearest_at(w0, W, H, at);
    }
}

// ---- Brown-Conrady projection (src/CameraCalibration.cpp) ----

struct BcCamera {
    float cx, cy, fx, fy;
    float k1, k2, k3, k4, k5, k6, codx, cody, p1, p2;
};

// transformation_project_internal (src/CameraCalibration.cpp:9-94).  Returns false when the point
// is beyond the projection radius (valid = 0, uv and J untouched).
AFX_D bool bc_project(const BcCamera& c, float x, float y, float* uv, float* J) {
    const float xp = x - c.codx, yp = y - c.cody;
    const float xp2 = xp * xp, yp2 = yp * yp, xyp = xp * yp;
    const float rs = xp2 + yp2;
    const float max_r = 1.7f;
    if (rs > max_r * max_r) return false;
    const float rss = rs * rs, rsc = rss * rs;
    const float a = 1.f + c.k1 * rs + c.k2 * rss + c.k3 * rsc;
    const float b = 1.f + c.k4 * rs + c.k5 * rss + c.k6 * rsc;
    const float bi = b != 0.f ? 1.f / b : 1.f;
    const float d = a * bi;
    float xp_d = xp * d, yp_d = yp * d;
    const float rs_2xp2 = rs + 2.f * xp2, rs_2yp2 = rs + 2.f * yp2;
    xp_d += rs_2xp2 * c.p2 + 2.f * xyp * c.p1;
    yp_d += rs_2yp2 * c.p1 + 2.f * xyp * c.p2;
    const float xp_d_cx = xp_d + c.codx, yp_d_cy = yp_d + c.cody;
    uv[0] = xp_d_cx * c.fx + c.cx;
    uv[1] = yp_d_cy * c.fy + c.cy;
    if (J) {
        const float dudrs = c.k1 + 2.f * c.k2 * rs + 3.f * c.k3 * rss;
        const float dvdrs = c.k4 + 2.f * c.k5 * rs + 3.f * c.k6 * rss;
        const float bis = bi * bi;
        const float dddrs = (dudrs * b - a * dvdrs) * bis;
        const float dddrs_2 = dddrs * 2.f;
        const float xp_dddrs_2 = xp * dddrs_2;
        const float yp_xp_dddrs_2 = yp * xp_dddrs_2;
        J[0] = c.fx * (d + xp * xp_dddrs_2 + 6.f * xp * c.p2 + 2.f * yp * c.p1);
        J[1] = c.fx * (yp_xp_dddrs_2 + 2.f * yp * c.p2 + 2.f * xp * c.p1);
        J[2] = c.fy * (yp_xp_dddrs_2 + 2.f * xp * c.p1 + 2.f * yp * c.p2);
        J[3] = c.fy * (d + yp * yp * dddrs_2 + 6.f * yp * c.p1 + 2.f * xp * c.p2);
    }
    return true;
}

// transformation_unproject_internal + transformation_iterative_unproject (src/CameraCalibration.cpp:
// 106-218): closed-form first guess (with the reference's (xx + 3 xx) p1 term), then up to 20
// Gauss-Newton passes keeping the best point; valid = 0 beyond the projection radius or when the
// best squared pixel error stays above 1e-6.
AFX_D void bc_unproject(const BcCamera& c, float u, float v, float* xy, int* valid) {
    const float xp_d = (u - c.cx) / c.fx - c.codx;
    const float yp_d = (v - c.cy) / c.fy - c.cody;
    const float rs = xp_d * xp_d + yp_d * yp_d;
    const float rss = rs * rs, rsc = rss * rs;
    const float a = 1.f + c.k1 * rs + c.k2 * rss + c.k3 * rsc;
    const float b = 1.f + c.k4 * rs + c.k5 * rss + c.k6 * rsc;
    const float ai = a != 0.f ? 1.f / a : 1.f;
    const float di = ai * b;
    float x = xp_d * di, y = yp_d * di;
    const float two_xy = 2.f * x * y;
    const float xx = x * x, yy = y * y;
    x -= (yy + 3.f * xx) * c.p2 + two_xy * c.p1;
    y -= (xx + 3.f * xx) * c.p1 + two_xy * c.p2;
    x += c.codx;
    y += c.cody;
    *valid = 1;
    float best_x = 0.f, best_y = 0.f, best_err = 3.40282347e+38f;
    for (int pass = 0; pass < 20; ++pass) {
        float p[2], J[4];
        if (!bc_project(c, x, y, p, J)) {
            *valid = 0;
            xy[0] = x;
            xy[1] = y;
            return;
        }
        const float err_x = u - p[0], err_y = v - p[1];
        const float err = err_x * err_x + err_y * err_y;
        if (err >= best_err) {
            x = best_x;
            y = best_y;
            break;
        }
        best_err = err;
        best_x = x;
        best_y = y;
        const float detJ = J[0] * J[3] - J[1] * J[2];
        const float inv_detJ = 1.f / detJ;
        const float Ji0 = inv_detJ * J[3], Ji3 = inv_detJ * J[0], Ji1 = -inv_detJ * J[1], Ji2 = -inv_detJ * J[2];
        if (pass + 1 == 20 || best_err < 1e-22f) break;
        const float dx = Ji0 * err_x + Ji1 * err_y;
        const float dy = Ji2 * err_x + Ji3 * err_y;
        x += dx;
        y += dy;
    }
    if (best_err > 1e-6f) *valid = 0;
    xy[0] = x;
    xy[1] = y;
}

// create_xy_lookup_table (src/CameraCalibration.cpp:261-295): the unit-depth ray per pixel, (0, 0)
// where invalid.
__global__ void xy_table_kernel(float* table, int W, int H, BcCamera c) {
    const long n = (long)W * H;
    AFX_GRID_STRIDE(p, n) {
        const int x = (int)(p % W), y = (int)(p / W);
        float xy[2];
        int valid = 0;
        bc_unproject(c, (float)x, (float)y, xy, &valid);
        // transformation_unproject at depth 1: point = xy * 1
        table[2 * p] = valid ? xy[0] * 1.f : 0.f;
        table[2 * p + 1] = valid ? xy[1] * 1.f : 0.f;
    }
}

// transformation_unproject (src/CameraCalibration.cpp:220-243)
__global__ void unproject_kernel(float* pts, int* valid, const float* __restrict__ px, const float* __restrict__ depth,
                                 long n, BcCamera c) {
    AFX_GRID_STRIDE(i, n) {
        const float d = depth[i];
        if (d == 0.f) {
            pts[3 * i] = pts[3 * i + 1] = pts[3 * i + 2] = 0.f;
            valid[i] = 0;
            continue;
        }
        float xy[2];
        int v = 0;
        bc_unproject(c, px[2 * i], px[2 * i + 1], xy, &v);
        pts[3 * i] = xy[0] * d;
        pts[3 * i + 1] = xy[1] * d;
        pts[3 * i + 2] = d;
        valid[i] = v;
    }
}

// transformation_project (src/CameraCalibration.cpp:245-259); a point beyond the projection radius
// leaves its pixel unwritten, as the reference leaves point2d.
__global__ void project_kernel(float* px, int* valid, const float* __restrict__ pts, long n, BcCamera c) {
    AFX_GRID_STRIDE(i, n) {
        const float z = pts[3 * i + 2];
        if (z <= 0.f) {
            px[2 * i] = px[2 * i + 1] = 0.f;
            valid[i] = 0;
            continue;
        }
        const float x = pts[3 * i] / z, y = pts[3 * i + 1] / z;
        float uv[2];
        if (bc_project(c, x, y, uv, nullptr)) {
            px[2 * i] = uv[0];
            px[2 * i + 1] = uv[1];
            valid[i] = 1;
        } else {
            valid[i] = 0;
        }
    }
}

bool make_bc_camera(const float intr[4], const afx_camera_distortion* d, BcCamera* c) {
    if (!intr || !d) return false;
    c->cx = intr[0];
    c->cy = intr[1];
    c->fx = intr[2];
    c->fy = intr[3];
    c->k1 = d->k1;
    c->k2 = d->k2;
    c->k3 = d->k3;
    c->k4 = d->k4;
    c->k5 = d->k5;
    c->k6 = d->k6;
    c->codx = d->codx;
    c->cody = d->cody;
    c->p1 = d->p1;
    c->p2 = d->p2;
    return c->fx > 0.f && c->fy > 0.f;
}

}  // namespace

int undistort_map_impl(uint32_t* map, int width, int height, const float K[9], const afx_camera_distortion* d, int mode,
                       cudaStream_t st) {
    if (!map || !K || !d || width < 1 || height < 1 || (mode != AFX_UNDISTORT_LINEAR && mode != AFX_UNDISTORT_NEAREST))
        return AFX_ERR_INVALID_ARGUMENT;
    if (width > 32767 || height > 32767) return AFX_ERR_UNSUPPORTED;  // int16 source coordinates
    MapArgs a;
    // the reference's cv::Mat camera matrix: fx, fy, cx, cy and K(2,2); the rest zero
    std::memset(a.A, 0, sizeof(a.A));
    a.A[0] = (double)K[0];
    a.A[4] = (double)K[4];
    a.A[2] = (double)K[6];
    a.A[5] = (double)K[7];
    a.A[8] = (double)K[8];
    const float k[8] = {d->k1, d->k2, d->p1, d->p2, d->k3, d->k4, d->k5, d->k6};
    for (int q = 0; q < 8; ++q) a.k[q] = (double)k[q];
    a.width = width;
    a.height = height;
    a.mode = mode;
    if (mode == AFX_UNDISTORT_LINEAR) {
        int s = 4096 / width;
        s = s < 1 ? 1 : s;
        a.stripe = s < height ? s : height;
    } else {
        a.stripe = height;
    }
    undistort_map_kernel<<<height, kMapChunk, 0, st>>>(map, a);
    AFX_LAUNCH_CHECK();
    return AFX_OK;
}

int undistort_apply_impl(float* dst, const float* src, int width, int height, const uint32_t* map, int mode,
                         cudaStream_t st) {
    if (!dst || !src || !map || width < 1 || height < 1 || dst == src ||
        (mode != AFX_UNDISTORT_LINEAR && mode != AFX_UNDISTORT_NEAREST))
        return AFX_ERR_INVALID_ARGUMENT;
    const long n = (long)width * height;
    undistort_apply_kernel<<<grid_for(n, 256), 256, 0, st>>>(dst, src, map, width, height, mode);
    AFX_LAUNCH_CHECK();
    return AFX_OK;
}

}  // namespace afx

using namespace afx;

extern "C" {

int afx_undistort_map(uint32_t* map, int width, int height, const float K[9], const afx_camera_distortion* d, int mode,
                      void* stream) {
    return undistort_map_impl(map, width, height, K, d, mode, as_stream(stream));
}

int afx_undistort_depth(float* dst, const float* src, int width, int height, const uint32_t* map, int mode,
                        void* stream) {
    return undistort_apply_impl(dst, src, width, height, map, mode, as_stream(stream));
}

int afx_xy_lookup_table(float* table, int width, int height, const float intrinsics[4], const afx_camera_distortion* d,
                        void* stream) {
    BcCamera c;
    if (!table || width < 1 || height < 1 || !make_bc_camera(intrinsics, d, &c)) return AFX_ERR_INVALID_ARGUMENT;
    const long n = (long)width * height;
    xy_table_kernel<<<grid_for(n, 128), 128, 0, as_stream(stream)>>>(table, width, height, c);
    AFX_LAUNCH_CHECK();
    return AFX_OK;
}

int afx_unproject_points(float* points, int* valid, const float* pixels, const float* depths, long n,
                         const float intrinsics[4], const afx_camera_distortion* d, void* stream) {
    BcCamera c;
    if (!points || !valid || !pixels || !depths || n < 0 || !make_bc_camera(intrinsics, d, &c))
        return AFX_ERR_INVALID_ARGUMENT;
    if (n == 0) return AFX_OK;
    unproject_kernel<<<grid_for(n, 128), 128, 0, as_stream(stream)>>>(points, valid, pixels, depths, n, c);
    AFX_LAUNCH_CHECK();
    return AFX_OK;
}

int afx_project_points(float* pixels, int* valid, const float* points, long n, const float intrinsics[4],
                       const afx_camera_distortion* d, void* stream) {
    BcCamera c;
    if (!pixels || !valid || !points || n < 0 || !make_bc_camera(intrinsics, d, &c)) return AFX_ERR_INVALID_ARGUMENT;
    if (n == 0) return AFX_OK;
    project_kernel<<<grid_for(n, 128), 128, 0, as_stream(stream)>>>(pixels, valid, points, n, c);
    AFX_LAUNCH_CHECK();
    return AFX_OK;
}

}  // extern "C"
