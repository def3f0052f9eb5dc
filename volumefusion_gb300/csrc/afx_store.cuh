// afx_store.cuh -- voxel storage formats.
//
// kVoxF32: the reference's layout (DeviceTsdf<float>): FP32 TSDF values and FP32 weights, 8 B/voxel.
// kVoxF16 (precision form): FP16 TSDF values and uint16 weights, 4 B/voxel.  Values are widened to
// FP32 exactly on load, every update is computed in FP32 as in the FP32 layout, and the result is
// rounded to the nearest FP16 (ties to even) on store.  Weights are integer counts capped at 15,
// so uint16 holds them exactly.
#pragma once

#include <cuda_fp16.h>

#include "afx_internal.h"

namespace afx {

// read-only loads (marching cubes)
AFX_D float vox_ld_t(const float* p, long i) { return __ldg(p + i); }
AFX_D float vox_ld_t(const __half* p, long i) { return __half2float(__ldg(p + i)); }
AFX_D float vox_ld_w(const float* p, long i) { return __ldg(p + i); }
AFX_D float vox_ld_w(const unsigned short* p, long i) { return (float)__ldg(p + i); }

// read-modify-write access (integration: each voxel is read and written by one thread)
AFX_D float vox_get_t(const float* p, long i) { return p[i]; }
AFX_D float vox_get_t(const __half* p, long i) { return __half2float(p[i]); }
AFX_D float vox_get_w(const float* p, long i) { return p[i]; }
AFX_D float vox_get_w(const unsigned short* p, long i) { return (float)p[i]; }
AFX_D void vox_put(float* t, float* w, long i, float tv, float wv) {
    t[i] = tv;
    w[i] = wv;
}
AFX_D void vox_put(__half* t, unsigned short* w, long i, float tv, float wv) {
    t[i] = __float2half_rn(tv);
    w[i] = (unsigned short)wv;  // an integer in [0, 15]
}

// four consecutive voxels (the base is aligned to four elements)
AFX_D void vox_get4(const float* t, const float* w, long i, float tv[4], float wv[4]) {
    const float4 a = *reinterpret_cast<const float4*>(t + i);
    const float4 b = *reinterpret_cast<const float4*>(w + i);
    tv[0] = a.x; tv[1] = a.y; tv[2] = a.z; tv[3] = a.w;
    wv[0] = b.x; wv[1] = b.y; wv[2] = b.z; wv[3] = b.w;
}
AFX_D void vox_put4(float* t, float* w, long i, const float tv[4], const float wv[4]) {
    *reinterpret_cast<float4*>(t + i) = make_float4(tv[0], tv[1], tv[2], tv[3]);
    *reinterpret_cast<float4*>(w + i) = make_float4(wv[0], wv[1], wv[2], wv[3]);
}
AFX_D void vox_get4(const __half* t, const unsigned short* w, long i, float tv[4], float wv[4]) {
    const uint2 a = *reinterpret_cast<const uint2*>(t + i);
    const uint2 b = *reinterpret_cast<const uint2*>(w + i);
    tv[0] = __half2float(__ushort_as_half((unsigned short)(a.x & 0xffffu)));
    tv[1] = __half2float(__ushort_as_half((unsigned short)(a.x >> 16)));
    tv[2] = __half2float(__ushort_as_half((unsigned short)(a.y & 0xffffu)));
    tv[3] = __half2float(__ushort_as_half((unsigned short)(a.y >> 16)));
    wv[0] = (float)(b.x & 0xffffu);
    wv[1] = (float)(b.x >> 16);
    wv[2] = (float)(b.y & 0xffffu);
    wv[3] = (float)(b.y >> 16);
}
AFX_D void vox_put4(__half* t, unsigned short* w, long i, const float tv[4], const float wv[4]) {
    unsigned h[4], u[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        h[k] = __half_as_ushort(__float2half_rn(tv[k]));
        u[k] = (unsigned)wv[k];
    }
    *reinterpret_cast<uint2*>(t + i) = make_uint2(h[0] | (h[1] << 16), h[2] | (h[3] << 16));
    *reinterpret_cast<uint2*>(w + i) = make_uint2(u[0] | (u[1] << 16), u[2] | (u[3] << 16));
}

// Calls f.template operator()<TsdfT, WeightT>(tsdf, weights) with the typed pointers of a format.
template <class F>
inline auto vox_dispatch(int fmt, void* tsdf, void* weights, F&& f) {
    if (fmt == kVoxF16) return f(static_cast<__half*>(tsdf), static_cast<unsigned short*>(weights));
    return f(static_cast<float*>(tsdf), static_cast<float*>(weights));
}

}  // namespace afx
