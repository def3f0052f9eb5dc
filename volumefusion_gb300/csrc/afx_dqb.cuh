// afx_dqb.cuh -- dual-quaternion blending of node transforms (Kavan, Collins, Zara, O'Sullivan:
// "Skinning with dual quaternions", I3D 2007), the session option next to the reference's linear
// blend (warpKernel, src/ComputeCorrespondence.cu:5-30; warpTsdfKernel, src/TSDFWarp.cu:158-190).
//
// A node transform T (column-major 4x4) is updated additively by the Gauss-Newton loop, so its
// upper 3x3 is only close to a rotation.  Its rigid part is taken as the unit quaternion of that
// 3x3 (Shepperd's method: the largest of the four diagonal combinations under the square root,
// then normalised) and the translation T[12..14].  The unit dual quaternion of node j is
// q_j = r_j + e * (0.5 * (0, t_j) (x) r_j).  A point's K nodes are blended as b = sum_j w_j s_j q_j
// with s_j = -1 where the rotation part lies in the other hemisphere from the first valid node's,
// b is divided by the norm of its rotation part, and the point moves by the rigid motion of the
// result: p' = p + 2 w (v x p) + 2 v x (v x p) + 2 (w v_e - w_e v + v x v_e).  As with the linear
// blend, a point whose weights are all within 1e-5 of zero stays where it is, and so does one
// whose blended rotation part is zero.
//
// The order of every operation is written out (the library builds with -fmad=false), so the CPU
// oracle's restatement gives the same bits.
#pragma once

#include <stdint.h>

#include "afx_common.cuh"

namespace afx {

// Unit dual quaternion of the rigid part of T: q[0..3] = rotation (w, x, y, z), q[4..7] = dual part.
AFX_HD void dq_of_transform(const float* T, float* q) {
    // m(r, c) = T[c * 4 + r]
    const float m00 = T[0], m10 = T[1], m20 = T[2];
    const float m01 = T[4], m11 = T[5], m21 = T[6];
    const float m02 = T[8], m12 = T[9], m22 = T[10];
    const float tr = (m00 + m11) + m22;
    float w, x, y, z;
    if (tr > 0.0f) {
        const float s = sqrtf(tr + 1.0f) * 2.0f;
        w = 0.25f * s;
        x = (m21 - m12) / s;
        y = (m02 - m20) / s;
        z = (m10 - m01) / s;
    } else if (m00 > m11 && m00 > m22) {
        const float s = sqrtf(((1.0f + m00) - m11) - m22) * 2.0f;
        w = (m21 - m12) / s;
        x = 0.25f * s;
        y = (m01 + m10) / s;
        z = (m02 + m20) / s;
    } else if (m11 > m22) {
        const float s = sqrtf(((1.0f + m11) - m00) - m22) * 2.0f;
        w = (m02 - m20) / s;
        x = (m01 + m10) / s;
        y = 0.25f * s;
        z = (m12 + m21) / s;
    } else {
        const float s = sqrtf(((1.0f + m22) - m00) - m11) * 2.0f;
        w = (m10 - m01) / s;
        x = (m02 + m20) / s;
        y = (m12 + m21) / s;
        z = 0.25f * s;
    }
    const float n = sqrtf(((w * w + x * x) + y * y) + z * z);
    w = w / n;
    x = x / n;
    y = y / n;
    z = z / n;
    const float tx = T[12], ty = T[13], tz = T[14];
    q[0] = w;
    q[1] = x;
    q[2] = y;
    q[3] = z;
    // 0.5 * (0, t) (x) (w, v) = 0.5 * (-t.v, w t + t x v)
    q[4] = -0.5f * ((tx * x + ty * y) + tz * z);
    q[5] = 0.5f * ((w * tx + ty * z) - tz * y);
    q[6] = 0.5f * ((w * ty + tz * x) - tx * z);
    q[7] = 0.5f * ((w * tz + tx * y) - ty * x);
}

// Blends the K nodes of one point (idx/w: its K slots; AFX_INVALID_INDEX or indices >= n_valid
// are skipped) and moves p into out.  load(node, T) fills T[16] with the node's transform.
// Returns false, leaving out = p, when the blend is empty.
template <class Load>
AFX_HD bool dq_blend_point(Load load, const uint32_t* idx, const float* w, int k, uint32_t n_valid, const float* p,
                           float* out) {
    out[0] = p[0];
    out[1] = p[1];
    out[2] = p[2];
    bool zero = true;
    for (int j = 0; j < k; ++j)
        if (!(fabsf(w[j]) <= 1e-5f)) zero = false;
    if (zero) return false;
    float b[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    float r0[4] = {0.f, 0.f, 0.f, 0.f};
    bool have_first = false;
    for (int j = 0; j < k; ++j) {
        const uint32_t nb = idx[j];
        if (nb == AFX_INVALID_INDEX || nb >= n_valid) continue;
        float T[16], q[8];
        load(nb, T);
        dq_of_transform(T, q);
        if (!have_first) {
            r0[0] = q[0];
            r0[1] = q[1];
            r0[2] = q[2];
            r0[3] = q[3];
            have_first = true;
        }
        const float d = ((r0[0] * q[0] + r0[1] * q[1]) + r0[2] * q[2]) + r0[3] * q[3];
        const float ws = d < 0.0f ? -w[j] : w[j];
        for (int c = 0; c < 8; ++c) b[c] = b[c] + ws * q[c];
    }
    const float n = sqrtf(((b[0] * b[0] + b[1] * b[1]) + b[2] * b[2]) + b[3] * b[3]);
    if (!(n > 0.0f)) return false;
    const float rw = b[0] / n, rx = b[1] / n, ry = b[2] / n, rz = b[3] / n;
    const float ew = b[4] / n, ex = b[5] / n, ey = b[6] / n, ez = b[7] / n;
    // rotation: p + 2 rw (v x p) + 2 v x (v x p), v = (rx, ry, rz)
    const float cx = ry * p[2] - rz * p[1], cy = rz * p[0] - rx * p[2], cz = rx * p[1] - ry * p[0];
    const float ccx = ry * cz - rz * cy, ccy = rz * cx - rx * cz, ccz = rx * cy - ry * cx;
    // translation: 2 (rw v_e - ew v + v x v_e)
    const float tx = 2.0f * ((rw * ex - ew * rx) + (ry * ez - rz * ey));
    const float ty = 2.0f * ((rw * ey - ew * ry) + (rz * ex - rx * ez));
    const float tz = 2.0f * ((rw * ez - ew * rz) + (rx * ey - ry * ex));
    out[0] = ((p[0] + 2.0f * rw * cx) + 2.0f * ccx) + tx;
    out[1] = ((p[1] + 2.0f * rw * cy) + 2.0f * ccy) + ty;
    out[2] = ((p[2] + 2.0f * rw * cz) + 2.0f * ccz) + tz;
    return true;
}

// The same with the transforms read directly from an array.
AFX_HD bool dq_blend_point(const float* transforms, const uint32_t* idx, const float* w, int k, uint32_t n_valid,
                           const float* p, float* out) {
    return dq_blend_point(
        [transforms](uint32_t nb, float* T) {
            for (int e = 0; e < 16; ++e) T[e] = transforms[16 * (long)nb + e];
        },
        idx, w, k, n_valid, p, out);
}

}  // namespace afx
