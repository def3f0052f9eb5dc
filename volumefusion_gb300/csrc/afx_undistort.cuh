// afx_undistort.cuh -- sampling through an undistortion map (afx_undistort_map): the per-pixel
// part of cv::remap for the two ways the reference undistorts a depth frame.
//
// Map entry per destination pixel (2 x uint32):
//   word 0 = source column sx (int16, low half) | source row sy (int16, high half)
//   word 1 = sub-pixel index (fy * 32 + fx, 1/32 pixel) for AFX_UNDISTORT_LINEAR, 0 for NEAREST.
#pragma once

#include "afx_common.cuh"

namespace afx {

AFX_HD int map_sx(uint32_t w0) { return (int)(int16_t)(uint16_t)(w0 & 0xFFFFu); }
AFX_HD int map_sy(uint32_t w0) { return (int)(int16_t)(uint16_t)(w0 >> 16); }

// INTER_LINEAR with the float table of 32 x 32 sub-pixel positions and a constant-zero border: the
// four taps (sx, sy), (sx+1, sy), (sx, sy+1), (sx+1, sy+1) weighted (1-fy)(1-fx), (1-fy)fx,
// fy(1-fx), fy fx (products of multiples of 1/32, exact in binary32), summed left to right; a tap
// outside the image reads 0 (cv::remap, BORDER_CONSTANT; remapBilinear).  at(x, y) gives the
// source value of an in-image pixel.
template <class At>
AFX_HD float remap_linear_at(uint32_t w0, uint32_t w1, int W, int H, At at) {
    const int sx = map_sx(w0), sy = map_sy(w0);
    const float ax = (float)(w1 & 31u) * (1.f / 32.f), ay = (float)((w1 >> 5) & 31u) * (1.f / 32.f);
    const float bx = 1.f - ax, by = 1.f - ay;
    const float w[4] = {by * bx, by * ax, ay * bx, ay * ax};
    const bool x0 = (unsigned)sx < (unsigned)W, x1 = (unsigned)(sx + 1) < (unsigned)W;
    const bool y0 = (unsigned)sy < (unsigned)H, y1 = (unsigned)(sy + 1) < (unsigned)H;
    const float v0 = (x0 && y0) ? at(sx, sy) : 0.f;
    const float v1 = (x1 && y0) ? at(sx + 1, sy) : 0.f;
    const float v2 = (x0 && y1) ? at(sx, sy + 1) : 0.f;
    const float v3 = (x1 && y1) ? at(sx + 1, sy + 1) : 0.f;
    return v0 * w[0] + v1 * w[1] + v2 * w[2] + v3 * w[3];
}

// INTER_NEAREST with a constant-zero border (remapNearest).
template <class At>
AFX_HD float remap_nearest_at(uint32_t w0, int W, int H, At at) {
    const int sx = map_sx(w0), sy = map_sy(w0);
    return ((unsigned)sx < (unsigned)W && (unsigned)sy < (unsigned)H) ? at(sx, sy) : 0.f;
}

}  // namespace afx
