// afx_integrate.cu -- TSDF integration: rigid projective integration and the non-rigid
// path (voxel -> node support, skinning weights, voxel warp, collision count, warped
// integration).
//
// The reference materialises per-voxel KNN index/distance/weight arrays and warped
// centres for the whole grid (~1.5 GB at 256^3, src/VolumeFusion.cu:252-260) and fills
// the KNN slots with atomics (first K to arrive, src/TSDFWarp.cu:61-67).  Here the
// active region is gathered brick by brick (8^3 voxels): each node lists the bricks
// its support cube touches, and one CTA per active brick selects, for each of its
// voxels, the K nearest supporting nodes (ties by node index), blends them, warps the
// voxel centre and counts collisions; a second pass integrates.  Only active voxels
// are touched.
#include <cstring>

#include "afx_dqb.cuh"
#include "afx_store.cuh"
#include "afx_voxel.h"

namespace afx {

Volume make_volume(const int dims[3], const float voxel_size[3], const float volume_size[3]) {
    Volume v;
    for (int c = 0; c < 3; ++c) {
        v.dims[c] = dims[c];
        v.vs[c] = voxel_size[c];
        v.half[c] = volume_size[c] * 0.5f;
        v.inv[c] = (float)(1.0 / (double)voxel_size[c]);
    }
    return v;
}

// ------------------------------------------------------------------------------------
// Rigid integration (integrateTSDFFromFrameKernel, src/TSDFIntegration.cu:69-96)
// Each thread owns four consecutive voxels along x: it projects them first and touches
// the volume (one 16-byte load and store per array) only if one of them is updated.
// ------------------------------------------------------------------------------------

struct RigidArgs {
    Volume vol;
    float R[9];
    float t[3];
    const float* t_dev;  // when set, the translation is read from device memory
    Intrinsics K;
    float delta;
    int W, H;
    unsigned char* occ;  // brick occupancy, or null
    int nbx, nby;        // bricks per axis (x, y)
};

// Marks the 8^3 brick of voxel (x, y, z) as holding a voxel with a weight (many threads may store 1).
AFX_D void mark_brick(unsigned char* occ, int nbx, int nby, int x, int y, int z) {
    if (occ) occ[((long)(z >> 3) * nby + (y >> 3)) * nbx + (x >> 3)] = 1;
}

template <class TT, class WT>
__global__ void __launch_bounds__(256) integrate_rigid_x4_kernel(TT* __restrict__ tsdf, WT* __restrict__ weights,
                                                                 const float* __restrict__ depth, RigidArgs a) {
    const int qx = blockIdx.x * blockDim.x + threadIdx.x;  // quad index along x
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int z = blockIdx.z;
    const int X = a.vol.dims[0], Y = a.vol.dims[1];
    if (qx * 4 >= X || y >= Y) return;
    const float t0 = a.t_dev ? a.t_dev[0] : a.t[0], t1 = a.t_dev ? a.t_dev[1] : a.t[1],
                t2 = a.t_dev ? a.t_dev[2] : a.t[2];
    float tn[4];
    unsigned upd = 0;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        float p[3], q[3];
        voxel_to_world(qx * 4 + i, y, z, a.vol.vs, a.vol.half, p);
        mat3_vec3(a.R, p, q);
        q[0] = q[0] + t0;
        q[1] = q[1] + t1;
        q[2] = q[2] + t2;
        if (tsdf_update_value(q, depth, a.W, a.H, a.delta, a.K, &tn[i])) upd |= 1u << i;
    }
    if (!upd) return;
    mark_brick(a.occ, a.nbx, a.nby, qx * 4, y, z);  // the four voxels share a brick
    const long base = ((long)z * Y + y) * X + qx * 4;
    float tv[4], wv[4];
    vox_get4(tsdf, weights, base, tv, wv);
#pragma unroll
    for (int i = 0; i < 4; ++i)
        if (upd & (1u << i)) tsdf_blend(tv[i], wv[i], tn[i]);
    vox_put4(tsdf, weights, base, tv, wv);
}

template <class TT, class WT>
__global__ void integrate_rigid_kernel(TT* tsdf, WT* weights, const float* __restrict__ depth, RigidArgs a) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y, z = blockIdx.z;
    const int X = a.vol.dims[0], Y = a.vol.dims[1];
    if (x >= X || y >= Y) return;
    float p[3], q[3], tn;
    voxel_to_world(x, y, z, a.vol.vs, a.vol.half, p);
    mat3_vec3(a.R, p, q);
    q[0] = q[0] + (a.t_dev ? a.t_dev[0] : a.t[0]);
    q[1] = q[1] + (a.t_dev ? a.t_dev[1] : a.t[1]);
    q[2] = q[2] + (a.t_dev ? a.t_dev[2] : a.t[2]);
    if (!tsdf_update_value(q, depth, a.W, a.H, a.delta, a.K, &tn)) return;
    mark_brick(a.occ, a.nbx, a.nby, x, y, z);
    const long i = ((long)z * Y + y) * X + x;
    float t = vox_get_t(tsdf, i), w = vox_get_w(weights, i);
    tsdf_blend(t, w, tn);
    vox_put(tsdf, weights, i, t, w);
}

// DeviceTsdf::initDefault followed by integrateTSDFFromFrameKernel, in one pass that only writes: a
// freshly initialised voxel (-1, weight 0) that is updated becomes ((-1 * 0) + t * 1) / (0 + 1) = t
// with weight min(0 + 1, 15) = 1 -- exactly, since -0 + t = t and t / 1 = t -- and every other voxel
// stays (-1, 0).  8 B per voxel written instead of 8 written + 16 read and written.
// Threads run over the quads of a z slice in memory order (a slice is contiguous), so no lane idles
// whatever X is.  The blend of a fresh voxel is written out as its result (t, 1): the division by
// (0 + 1) and the products by 0 and 1 change nothing.
__global__ void __launch_bounds__(256) integrate_fresh_x4_kernel(float* __restrict__ tsdf, float* __restrict__ weights,
                                                                 const float* __restrict__ depth, RigidArgs a) {
    const int X = a.vol.dims[0], Y = a.vol.dims[1];
    const int qx_n = X >> 2;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;  // quad within the slice
    if (j >= qx_n * Y) return;
    const int y = j / qx_n, qx = j - y * qx_n, z = blockIdx.y;
    float tv[4], wv[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        float p[3], q[3], tn;
        voxel_to_world(qx * 4 + i, y, z, a.vol.vs, a.vol.half, p);
        mat3_vec3(a.R, p, q);
        q[0] = q[0] + a.t[0];
        q[1] = q[1] + a.t[1];
        q[2] = q[2] + a.t[2];
        const bool upd = tsdf_update_value(q, depth, a.W, a.H, a.delta, a.K, &tn);
        tv[i] = upd ? tn : -1.f;
        wv[i] = upd ? 1.f : 0.f;
    }
    vox_put4(tsdf, weights, ((long)z * Y + y) * X + qx * 4, tv, wv);
}

int integrate_fresh_impl(float* tsdf, float* weights, const float* depth, int W, int H, float delta, const Volume& vol,
                         const float* R, const float* t, const float* K, cudaStream_t st) {
    const int X = vol.dims[0], Y = vol.dims[1], Z = vol.dims[2];
    const bool vec = (X % 4 == 0) && ((reinterpret_cast<uintptr_t>(tsdf) | reinterpret_cast<uintptr_t>(weights)) & 15) == 0;
    if (!vec) return AFX_ERR_UNSUPPORTED;  // callers fall back to initialise + integrate
    RigidArgs a;
    a.vol = vol;
    a.occ = nullptr;
    a.nbx = a.nby = 0;
    for (int i = 0; i < 9; ++i) a.R[i] = R[i];
    for (int i = 0; i < 3; ++i) a.t[i] = t[i];
    a.t_dev = nullptr;
    a.K = make_intrinsics(K);
    a.delta = delta;
    a.W = W;
    a.H = H;
    const long quads = (long)(X / 4) * Y;
    dim3 grid((unsigned)((quads + 255) / 256), (unsigned)Z);
    integrate_fresh_x4_kernel<<<grid, 256, 0, st>>>(tsdf, weights, depth, a);
    AFX_LAUNCH_CHECK();
    return AFX_OK;
}

int integrate_rigid_impl(void* tsdf, void* weights, int fmt, const float* depth, int W, int H, float delta,
                         const Volume& vol, const float* R, const float* t, const float* K, cudaStream_t st,
                         const float* t_dev, unsigned char* occ) {
    RigidArgs a;
    a.vol = vol;
    a.occ = occ;
    {
        const BrickGrid bg = make_bricks(vol);
        a.nbx = bg.nb[0];
        a.nby = bg.nb[1];
    }
    for (int i = 0; i < 9; ++i) a.R[i] = R[i];
    for (int i = 0; i < 3; ++i) a.t[i] = t ? t[i] : 0.f;
    a.t_dev = t_dev;
    a.K = make_intrinsics(K);
    a.delta = delta;
    a.W = W;
    a.H = H;
    const int X = vol.dims[0], Y = vol.dims[1], Z = vol.dims[2];
    const uintptr_t align = 4 * vox_bytes(fmt) - 1;  // four voxels per vector access
    bool vec = (X % 4 == 0) && ((reinterpret_cast<uintptr_t>(tsdf) | reinterpret_cast<uintptr_t>(weights)) & align) == 0;
    vox_dispatch(fmt, tsdf, weights, [&](auto* tp, auto* wp) {
        if (vec) {
            dim3 block(64, 4), grid((X / 4 + 63) / 64, (Y + 3) / 4, Z);
            integrate_rigid_x4_kernel<<<grid, block, 0, st>>>(tp, wp, depth, a);
        } else {
            dim3 block(64, 4), grid((X + 63) / 64, (Y + 3) / 4, Z);
            integrate_rigid_kernel<<<grid, block, 0, st>>>(tp, wp, depth, a);
        }
        return 0;
    });
    AFX_LAUNCH_CHECK();
    return AFX_OK;
}

// ------------------------------------------------------------------------------------
// Brick-sparse voxel support (replaces tsdfKNNGraph, src/TSDFWarp.cu:23-68)
// ------------------------------------------------------------------------------------

// Node support cube: node voxel (worldToVoxel of the translated node), minus (per-1)/2,
// plus [0, per) per axis (src/TSDFWarp.cu:40-50), clipped to the volume.
AFX_D bool node_cube(const float* node_t, const Volume& vol, const int* per, NodeCube* c) {
    int nv[3];
    world_to_voxel(node_t, vol.inv, vol.half, nv);
    bool empty = false;
    for (int a = 0; a < 3; ++a) {
        int lo = nv[a] - (per[a] - 1) / 2;
        int hi = lo + per[a] - 1;
        c->lo[a] = max(lo, 0);
        c->hi[a] = min(hi, vol.dims[a] - 1);
        if (c->lo[a] > c->hi[a]) empty = true;
    }
    return !empty;
}

__global__ void brick_count_kernel(SupportArgs a) {
    const int n = min(*a.n_nodes, a.n_max);
    AFX_GRID_STRIDE(j, n) {
    NodeCube c;
    if (!node_cube(a.nodes + 3 * j, a.vol, a.per, &c)) continue;
    for (int bz = c.lo[2] / kBrick; bz <= c.hi[2] / kBrick; ++bz)
        for (int by = c.lo[1] / kBrick; by <= c.hi[1] / kBrick; ++by)
            for (int bx = c.lo[0] / kBrick; bx <= c.hi[0] / kBrick; ++bx)
                atomicAdd(a.brick_count + ((long)bz * a.bg.nb[1] + by) * a.bg.nb[0] + bx, 1u);
    }
}

__global__ void brick_fill_kernel(SupportArgs a) {
    const int n = min(*a.n_nodes, a.n_max);
    AFX_GRID_STRIDE(j, n) {
    NodeCube c;
    if (!node_cube(a.nodes + 3 * j, a.vol, a.per, &c)) continue;
    for (int bz = c.lo[2] / kBrick; bz <= c.hi[2] / kBrick; ++bz)
        for (int by = c.lo[1] / kBrick; by <= c.hi[1] / kBrick; ++by)
            for (int bx = c.lo[0] / kBrick; bx <= c.hi[0] / kBrick; ++bx) {
                long b = ((long)bz * a.bg.nb[1] + by) * a.bg.nb[0] + bx;
                unsigned pos = a.brick_offset[b] + atomicAdd(a.brick_cursor + b, 1u);
                if (pos < a.pair_capacity) a.brick_nodes[pos] = (unsigned)j;
                else atomicOr(a.error, ERRF_CAPACITY);
            }
    }
}

__global__ void brick_active_kernel(const unsigned* brick_count, long nb, unsigned* active, unsigned* n_active) {
    const long b = blockIdx.x * (long)blockDim.x + threadIdx.x;
    const bool on = b < nb && brick_count[b] > 0;  // every lane takes part in the ballot
    unsigned m = __ballot_sync(0xffffffffu, on);
    unsigned base = 0;
    int lane = threadIdx.x & 31;
    if (lane == 0 && m) base = atomicAdd(n_active, (unsigned)__popc(m));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (on) active[base + __popc(m & ((1u << lane) - 1))] = (unsigned)b;
}

AFX_D void topk_insert(float* kd, int* ki, int& cnt, int cap, float d, int idx) {
    if (cnt == cap && !(d < kd[cap - 1] || (d == kd[cap - 1] && idx < ki[cap - 1]))) return;
    int i = (cnt < cap) ? cnt++ : cap - 1;
    while (i > 0 && (d < kd[i - 1] || (d == kd[i - 1] && idx < ki[i - 1]))) {
        kd[i] = kd[i - 1];
        ki[i] = ki[i - 1];
        --i;
    }
    kd[i] = d;
    ki[i] = idx;
}

AFX_D void coll_add(unsigned* w, unsigned epoch) {
    unsigned old = *w, assumed;
    do {
        assumed = old;
        unsigned nw = ((assumed >> 8) == epoch) ? (((assumed & 255u) < 255u) ? assumed + 1u : assumed) : ((epoch << 8) | 1u);
        old = atomicCAS(w, assumed, nw);
    } while (old != assumed);
}

AFX_D int coll_get(const unsigned* w, unsigned epoch) {
    unsigned v = *w;
    return ((v >> 8) == epoch) ? (int)(v & 255u) : 0;
}

template <int K>
__global__ void __launch_bounds__(kBrickVox) brick_warp_kernel(WarpArgs a) {
    __shared__ float s_pos[kMaxBrickNodes * 3];
    __shared__ float s_rad[kMaxBrickNodes];
    __shared__ int s_lo[kMaxBrickNodes * 3], s_hi[kMaxBrickNodes * 3];
    __shared__ int s_id[kMaxBrickNodes];
    const unsigned n_active = *a.n_active;
    for (unsigned slot = blockIdx.x; slot < n_active; slot += gridDim.x) {
    __syncthreads();  // the previous brick's staged nodes are no longer read
    [&] {
    const unsigned b = a.active[slot];
    const unsigned off = a.brick_offset[b];
    const int nc = min((int)a.brick_count[b], kMaxBrickNodes);
    if (threadIdx.x == 0 && a.brick_count[b] > kMaxBrickNodes) atomicOr(a.error, ERRF_CAPACITY);
    for (int i = threadIdx.x; i < nc; i += blockDim.x) {
        int j = (int)a.brick_nodes[off + i];
        s_id[i] = j;
        const float* p = a.nodes_t + 3 * j;
        s_pos[3 * i] = p[0];
        s_pos[3 * i + 1] = p[1];
        s_pos[3 * i + 2] = p[2];
        s_rad[i] = a.radii[j];
        NodeCube c;
        node_cube(p, a.vol, a.per, &c);
        for (int q = 0; q < 3; ++q) {
            s_lo[3 * i + q] = c.lo[q];
            s_hi[3 * i + q] = c.hi[q];
        }
    }
    __syncthreads();
    const int bx = b % a.bg.nb[0], by = (b / a.bg.nb[0]) % a.bg.nb[1], bz = b / ((unsigned)a.bg.nb[0] * a.bg.nb[1]);
    const int lx = threadIdx.x % kBrick, ly = (threadIdx.x / kBrick) % kBrick, lz = threadIdx.x / (kBrick * kBrick);
    const int x = bx * kBrick + lx, y = by * kBrick + ly, z = bz * kBrick + lz;
    const long local = (long)slot * kBrickVox + threadIdx.x;
    const int X = a.vol.dims[0], Y = a.vol.dims[1], Z = a.vol.dims[2];
    const bool inside = x < X && y < Y && z < Z;
    float kd[K];
    int ki[K];
    int cnt = 0;
    float p[3];
    voxel_to_world(x, y, z, a.vol.vs, a.vol.half, p);
    if (inside) {
        for (int i = 0; i < nc; ++i) {
            if (x < s_lo[3 * i] || x > s_hi[3 * i] || y < s_lo[3 * i + 1] || y > s_hi[3 * i + 1] ||
                z < s_lo[3 * i + 2] || z > s_hi[3 * i + 2])
                continue;
            float d3[3] = {p[0] - s_pos[3 * i], p[1] - s_pos[3 * i + 1], p[2] - s_pos[3 * i + 2]};
            float d = norm3(d3);
            if (d > s_rad[i] * 2.0f) continue;
            topk_insert(kd, ki, cnt, K < a.k ? K : a.k, d, s_id[i]);
        }
    }
    if (a.dense_count && inside) {
        const long v = ((long)z * Y + y) * X + x;
        a.dense_count[v] = cnt;
        for (int s = 0; s < a.k; ++s) {
            a.dense_idx[v * a.k + s] = s < cnt ? (uint32_t)ki[s] : AFX_INVALID_INDEX;
            a.dense_dist[v * a.k + s] = s < cnt ? kd[s] : 3.402823466e+38f;
        }
    }
    if (!a.out) return;
    a.out_count[local] = (unsigned char)cnt;
    if (cnt == 0) return;
    // weights (computeTsdfWarpWeightsKernel, src/TSDFWarp.cu:88-116: no cut-off)
    float w[K];
    float sum = 0.f;
    for (int s = 0; s < cnt; ++s) {
        float r = a.radii[ki[s]], d = kd[s];
        w[s] = afx_expf(-(d * d) / (2.0f * (r * r)));
        sum = sum + w[s];
    }
    if (sum != 0.f)
        for (int s = 0; s < cnt; ++s) w[s] = w[s] / sum;
    bool zero = true;
    for (int s = 0; s < cnt; ++s)
        if (!(fabsf(w[s]) <= 1e-5f)) zero = false;
    // voxel centre in camera space (generateTsdfVertices + translate, src/VolumeFusion.cu:718-723)
    const float cen[3] = {a.centroid_dev[0], a.centroid_dev[1], a.centroid_dev[2]};
    float c[3] = {p[0] + cen[0], p[1] + cen[1], p[2] + cen[2]};
    float q[3] = {c[0], c[1], c[2]};
    if (!zero && a.blend == AFX_BLEND_DQB) {  // dual-quaternion blend (afx_dqb.cuh)
        uint32_t kidx[K];
        for (int s = 0; s < cnt; ++s) kidx[s] = (uint32_t)ki[s];
        dq_blend_point(a.transforms, kidx, w, cnt, AFX_INVALID_INDEX, c, q);
    } else if (!zero) {  // warpTsdfKernel (src/TSDFWarp.cu:158-190)
        q[0] = q[1] = q[2] = 0.f;
        for (int s = 0; s < cnt; ++s) {
            float o[3];
            mat4_point(a.transforms + 16 * (long)ki[s], c, o);
            q[0] = q[0] + w[s] * o[0];
            q[1] = q[1] + w[s] * o[1];
            q[2] = q[2] + w[s] * o[2];
        }
    }
    // target voxel (countCollisionsPerVoxelKernel, src/TSDFIntegration.cu:272-282)
    float dq[3] = {q[0] - cen[0], q[1] - cen[1], q[2] - cen[2]};
    float o[3];
    mat3_vec3(a.Rinv, dq, o);
    int tv[3];
    world_to_voxel(o, a.vol.inv, a.vol.half, tv);
    int target = -1;
    if (tv[0] >= 0 && tv[1] >= 0 && tv[2] >= 0 && tv[0] < X && tv[1] < Y && tv[2] < Z) {
        target = (int)(((long)tv[2] * Y + tv[1]) * X + tv[0]);
        coll_add(a.coll + target, *a.epoch_dev);
    }
    WarpedVoxel wv;
    wv.p[0] = q[0];
    wv.p[1] = q[1];
    wv.p[2] = q[2];
    wv.target = target;
    a.out[local] = wv;
    }();
    }
}

// integrateWarpedTSDFFromFrameKernel (src/TSDFIntegration.cu:173-226) over the active bricks
template <class TT, class WT>
__global__ void __launch_bounds__(kBrickVox) brick_integrate_kernel(WarpedIntegrateArgs a) {
    TT* __restrict__ tsdf = static_cast<TT*>(a.tsdf);
    WT* __restrict__ weights = static_cast<WT*>(a.weights);
    const unsigned n_active = *a.n_active;
    for (unsigned slot = blockIdx.x; slot < n_active; slot += gridDim.x) [&] {
    const long local = (long)slot * kBrickVox + threadIdx.x;
    if (a.in_count[local] == 0) return;
    const WarpedVoxel wv = a.in[local];
    if (wv.target < 0) return;
    if (coll_get(a.coll + wv.target, *a.epoch_dev) > 1) return;
    float tn;
    if (!tsdf_update_value(wv.p, a.depth, a.W, a.H, a.delta, a.K, &tn)) return;
    const unsigned b = a.active[slot];
    const int bx = b % a.bg.nb[0], by = (b / a.bg.nb[0]) % a.bg.nb[1], bz = b / ((unsigned)a.bg.nb[0] * a.bg.nb[1]);
    const int x = bx * kBrick + threadIdx.x % kBrick, y = by * kBrick + (threadIdx.x / kBrick) % kBrick,
              z = bz * kBrick + threadIdx.x / (kBrick * kBrick);
    const long v = ((long)z * a.vol.dims[1] + y) * a.vol.dims[0] + x;
    float t = vox_get_t(tsdf, v), w = vox_get_w(weights, v);
    tsdf_blend(t, w, tn);
    vox_put(tsdf, weights, v, t, w);
    if (a.occ) a.occ[b] = 1;
    }();
}

static size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// Bricks a node's support cube can touch: per axis at most ceil((per - 1) / 8) + 1.
static long pairs_per_node(const int* per) {
    long p = 1;
    for (int c = 0; c < 3; ++c) p *= (per[c] - 1 + kBrick - 1) / kBrick + 1;
    return p;
}

size_t support_workspace_size(const Volume& vol, int n_nodes_max, const int* per) {
    BrickGrid bg = make_bricks(vol);
    size_t scan = scan_workspace_size(bg.n);
    long pairs = (long)n_nodes_max * pairs_per_node(per) + 1024;
    return align256(bg.n * 4) * 3 + align256((bg.n + 1) * 4) + align256(pairs * 4) + align256(bg.n * 4) + 256 +
           align256(scan) + 1024;
}

bool carve_support(void* ws, size_t bytes, const Volume& vol, int n_nodes_max, const int* per, SupportWorkspace* s) {
    if (bytes < support_workspace_size(vol, n_nodes_max, per) || !ws) return false;
    BrickGrid bg = make_bricks(vol);
    char* p = static_cast<char*>(ws);
    auto take = [&](size_t n) {
        char* r = p;
        p += align256(n);
        return r;
    };
    s->brick_count = (unsigned*)take(bg.n * 4);
    s->brick_cursor = (unsigned*)take(bg.n * 4);
    s->brick_offset = (unsigned*)take((bg.n + 1) * 4);
    s->pair_capacity = (long)n_nodes_max * pairs_per_node(per) + 1024;
    s->brick_nodes = (unsigned*)take(s->pair_capacity * 4);
    s->active = (unsigned*)take(bg.n * 4);
    s->n_active = (unsigned*)take(256);
    size_t scan = scan_workspace_size(bg.n);
    s->scan_tmp_bytes = scan;
    s->scan_tmp = take(scan);
    return true;
}

// Builds the brick -> node candidate lists and the active brick list.
int build_support(const SupportWorkspace& s, const Volume& vol, const int* per, const float* nodes_t,
                  const float* radii, const int* n_nodes, int n_max, int* error, cudaStream_t st) {
    BrickGrid bg = make_bricks(vol);
    AFX_CUDA(cudaMemsetAsync(s.brick_count, 0, bg.n * 4, st));
    AFX_CUDA(cudaMemsetAsync(s.brick_cursor, 0, bg.n * 4, st));
    AFX_CUDA(cudaMemsetAsync(s.n_active, 0, 4, st));
    SupportArgs a;
    a.vol = vol;
    a.bg = bg;
    for (int c = 0; c < 3; ++c) a.per[c] = per[c];
    a.nodes = nodes_t;
    a.radii = radii;
    a.n_nodes = n_nodes;
    a.n_max = n_max;
    a.brick_count = s.brick_count;
    a.brick_offset = s.brick_offset;
    a.brick_cursor = s.brick_cursor;
    a.brick_nodes = s.brick_nodes;
    a.pair_capacity = s.pair_capacity;
    a.error = error;
    if (n_max > 0) {
        brick_count_kernel<<<grid_for(n_max, 128), 128, 0, st>>>(a);
        AFX_LAUNCH_CHECK();
    }
    int rc = scan_exclusive(s.brick_count, s.brick_offset, bg.n, nullptr, s.scan_tmp, st);
    if (rc) return rc;
    if (n_max > 0) {
        brick_fill_kernel<<<grid_for(n_max, 128), 128, 0, st>>>(a);
        AFX_LAUNCH_CHECK();
    }
    brick_active_kernel<<<blocks_for(bg.n, 256), 256, 0, st>>>(s.brick_count, bg.n, s.active, s.n_active);
    AFX_LAUNCH_CHECK();
    return AFX_OK;
}

// Block-stride grid over the active bricks (their number is on the device).
static unsigned brick_grid(long max_active) { return (unsigned)(max_active < 608 ? max_active : 608); }

int launch_brick_warp(const WarpArgs& a, long max_active, cudaStream_t st) {
    if (max_active <= 0) return AFX_OK;
    switch (a.k <= 4 ? 4 : 8) {
        case 4: brick_warp_kernel<4><<<brick_grid(max_active), kBrickVox, 0, st>>>(a); break;
        default: brick_warp_kernel<8><<<brick_grid(max_active), kBrickVox, 0, st>>>(a); break;
    }
    AFX_LAUNCH_CHECK();
    return AFX_OK;
}

int launch_brick_integrate(const WarpedIntegrateArgs& a, long max_active, cudaStream_t st) {
    if (max_active <= 0) return AFX_OK;
    if (a.fmt == kVoxF16) brick_integrate_kernel<__half, unsigned short><<<brick_grid(max_active), kBrickVox, 0, st>>>(a);
    else brick_integrate_kernel<float, float><<<brick_grid(max_active), kBrickVox, 0, st>>>(a);
    AFX_LAUNCH_CHECK();
    return AFX_OK;
}

long brick_count_total(const Volume& vol) { return make_bricks(vol).n; }

// ------------------------------------------------------------------------------------
// Dense per-voxel stage kernels (the reference's layouts)
// ------------------------------------------------------------------------------------

__global__ void tsdf_weights_kernel(float* kw, const float* radii, const uint32_t* kidx, const float* kdist,
                                    const int* kcount, long S, int k) {
    long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (i >= S) return;
    int cnt = kcount[i];
    if (!cnt) return;  // as the reference: empty voxels keep whatever the array held
    float w[kMaxK];
    float sum = 0.f;
    for (int s = 0; s < k; ++s) w[s] = 0.f;
    for (int s = 0; s < cnt && s < k; ++s) {
        float r = radii[kidx[i * k + s]], d = kdist[i * k + s];
        w[s] = afx_expf(-(d * d) / (2.0f * (r * r)));
        sum = sum + w[s];
    }
    if (sum != 0.f)
        for (int s = 0; s < k; ++s) w[s] = w[s] / sum;
    for (int s = 0; s < k; ++s) kw[i * k + s] = w[s];
}

__global__ void tsdf_vertices_kernel(float* v, Volume vol) {
    long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
    long S = (long)vol.dims[0] * vol.dims[1] * vol.dims[2];
    if (i >= S) return;
    int x = i % vol.dims[0], y = (i / vol.dims[0]) % vol.dims[1], z = i / ((long)vol.dims[0] * vol.dims[1]);
    voxel_to_world(x, y, z, vol.vs, vol.half, v + 3 * i);
}

__global__ void warp_tsdf_kernel(float* verts, const float* T, const uint32_t* kidx, const float* kw,
                                 const int* kcount, long S, int k) {
    long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (i >= S) return;
    int cnt = kcount[i];
    if (!cnt) return;
    bool zero = true;
    for (int s = 0; s < k; ++s)
        if (!(fabsf(kw[i * k + s]) <= 1e-5f)) zero = false;
    if (zero) return;
    float p[3] = {verts[3 * i], verts[3 * i + 1], verts[3 * i + 2]};
    float q[3] = {0.f, 0.f, 0.f};
    for (int s = 0; s < cnt; ++s) {
        float o[3];
        mat4_point(T + 16 * (long)kidx[i * k + s], p, o);
        float w = kw[i * k + s];
        q[0] = q[0] + w * o[0];
        q[1] = q[1] + w * o[1];
        q[2] = q[2] + w * o[2];
    }
    verts[3 * i] = q[0];
    verts[3 * i + 1] = q[1];
    verts[3 * i + 2] = q[2];
}

AFX_D long warped_target(const float* wp, const Volume& vol, const float* Rinv, const float* t) {
    float d[3] = {wp[0] - t[0], wp[1] - t[1], wp[2] - t[2]};
    float o[3];
    mat3_vec3(Rinv, d, o);
    int v[3];
    world_to_voxel(o, vol.inv, vol.half, v);
    if (v[0] < 0 || v[1] < 0 || v[2] < 0 || v[0] >= vol.dims[0] || v[1] >= vol.dims[1] || v[2] >= vol.dims[2])
        return -1;
    return ((long)v[2] * vol.dims[1] + v[1]) * vol.dims[0] + v[0];
}

struct DenseWarpArgs {
    Volume vol;
    float Rinv[9];
    float t[3];
};

__global__ void count_collisions_kernel(int* counts, const float* verts, const int* kcount, DenseWarpArgs a) {
    long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
    long S = (long)a.vol.dims[0] * a.vol.dims[1] * a.vol.dims[2];
    if (i >= S || !kcount[i]) return;
    long tg = warped_target(verts + 3 * i, a.vol, a.Rinv, a.t);
    if (tg >= 0) atomicAdd(counts + tg, 1);
}

__global__ void integrate_warped_kernel(float* tsdf, float* weights, const float* verts, const int* coll,
                                        const int* kcount, const float* depth, int W, int H, float delta,
                                        Intrinsics K, DenseWarpArgs a) {
    long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
    long S = (long)a.vol.dims[0] * a.vol.dims[1] * a.vol.dims[2];
    if (i >= S || !kcount[i]) return;
    long tg = warped_target(verts + 3 * i, a.vol, a.Rinv, a.t);
    if (tg < 0 || coll[tg] > 1) return;
    float tn;
    if (!tsdf_update_value(verts + 3 * i, depth, W, H, delta, K, &tn)) return;
    float t = tsdf[i], w = weights[i];
    tsdf_blend(t, w, tn);
    tsdf[i] = t;
    weights[i] = w;
}

static void inverse3(const float* R, float* Rinv) {
    // Mat3f::inverse() for the rotations the pipeline passes; identity stays exact
    double a[9];
    for (int i = 0; i < 9; ++i) a[i] = R[i];
    // column-major: a[c*3 + r]
    auto m = [&](int r, int c) { return a[c * 3 + r]; };
    double det = m(0, 0) * (m(1, 1) * m(2, 2) - m(1, 2) * m(2, 1)) - m(0, 1) * (m(1, 0) * m(2, 2) - m(1, 2) * m(2, 0)) +
                 m(0, 2) * (m(1, 0) * m(2, 1) - m(1, 1) * m(2, 0));
    double inv[3][3];
    inv[0][0] = (m(1, 1) * m(2, 2) - m(1, 2) * m(2, 1)) / det;
    inv[0][1] = (m(0, 2) * m(2, 1) - m(0, 1) * m(2, 2)) / det;
    inv[0][2] = (m(0, 1) * m(1, 2) - m(0, 2) * m(1, 1)) / det;
    inv[1][0] = (m(1, 2) * m(2, 0) - m(1, 0) * m(2, 2)) / det;
    inv[1][1] = (m(0, 0) * m(2, 2) - m(0, 2) * m(2, 0)) / det;
    inv[1][2] = (m(0, 2) * m(1, 0) - m(0, 0) * m(1, 2)) / det;
    inv[2][0] = (m(1, 0) * m(2, 1) - m(1, 1) * m(2, 0)) / det;
    inv[2][1] = (m(0, 1) * m(2, 0) - m(0, 0) * m(2, 1)) / det;
    inv[2][2] = (m(0, 0) * m(1, 1) - m(0, 1) * m(1, 0)) / det;
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) Rinv[c * 3 + r] = (float)inv[r][c];
}

void rotation_inverse(const float* R, float* Rinv) { inverse3(R, Rinv); }

}  // namespace afx

using namespace afx;

extern "C" {

int afx_integrate_tsdf(float* tsdf, float* weights, const float* depth, int width, int height, float delta,
                       const int dims[3], const float voxel_size[3], const float volume_size[3], const float rotate[9],
                       const float translate[3], const float K[9], void* stream) {
    if (!tsdf || !weights || !depth || !dims || !voxel_size || !volume_size || !rotate || !translate || !K)
        return AFX_ERR_INVALID_ARGUMENT;
    if (width <= 0 || height <= 0 || dims[0] <= 0 || dims[1] <= 0 || dims[2] <= 0) return AFX_ERR_INVALID_ARGUMENT;
    return integrate_rigid_impl(tsdf, weights, kVoxF32, depth, width, height, delta,
                                make_volume(dims, voxel_size, volume_size),
                                rotate, translate, K, as_stream(stream));
}

int afx_integrate_tsdf_fresh(float* tsdf, float* weights, const float* depth, int width, int height, float delta,
                             const int dims[3], const float voxel_size[3], const float volume_size[3],
                             const float rotate[9], const float translate[3], const float K[9], void* stream) {
    if (!tsdf || !weights || !depth || !dims || !voxel_size || !volume_size || !rotate || !translate || !K)
        return AFX_ERR_INVALID_ARGUMENT;
    if (width <= 0 || height <= 0 || dims[0] <= 0 || dims[1] <= 0 || dims[2] <= 0) return AFX_ERR_INVALID_ARGUMENT;
    return integrate_fresh_impl(tsdf, weights, depth, width, height, delta, make_volume(dims, voxel_size, volume_size),
                                rotate, translate, K, as_stream(stream));
}

size_t afx_tsdf_knn_workspace_size(const int dims[3], int n_nodes, const int voxels_per_node[3]) {
    float one[3] = {1, 1, 1};
    if (!dims || !voxels_per_node) return 0;
    return support_workspace_size(make_volume(dims, one, one), n_nodes, voxels_per_node);
}

int afx_tsdf_knn(uint32_t* knn_idx, float* knn_dist, int* knn_counts, const float* nodes, const float* radii,
                 int n_nodes, const float voxel_size[3], const float volume_size[3], const int dims[3],
                 const int voxels_per_node[3], int k, void* workspace, size_t workspace_bytes, void* stream) {
    if (!knn_idx || !knn_dist || !knn_counts || (!nodes && n_nodes) || !dims || k < 1 || k > kMaxK || n_nodes < 0)
        return AFX_ERR_INVALID_ARGUMENT;
    cudaStream_t st = as_stream(stream);
    Volume vol = make_volume(dims, voxel_size, volume_size);
    SupportWorkspace s;
    if (!carve_support(workspace, workspace_bytes, vol, n_nodes, voxels_per_node, &s)) return AFX_ERR_WORKSPACE;
    const long S = (long)dims[0] * dims[1] * dims[2];
    AFX_CUDA(cudaMemsetAsync(knn_counts, 0, S * sizeof(int), st));
    int* d_n = reinterpret_cast<int*>(s.n_active) + 1;  // spare word in the n_active slot
    int* d_err = reinterpret_cast<int*>(s.n_active) + 2;
    AFX_CUDA(cudaMemcpyAsync(d_n, &n_nodes, sizeof(int), cudaMemcpyHostToDevice, st));
    AFX_CUDA(cudaMemsetAsync(d_err, 0, sizeof(int), st));
    int st_ = build_support(s, vol, voxels_per_node, nodes, radii, d_n, n_nodes, d_err, st);
    if (st_) return st_;
    WarpArgs a;
    std::memset(&a, 0, sizeof(a));
    a.vol = vol;
    a.bg = make_bricks(vol);
    a.k = k;
    a.nodes_t = nodes;
    a.radii = radii;
    a.brick_offset = s.brick_offset;
    a.brick_count = s.brick_count;
    a.brick_nodes = s.brick_nodes;
    a.active = s.active;
    a.n_active = s.n_active;
    for (int c = 0; c < 3; ++c) a.per[c] = voxels_per_node[c];
    a.dense_idx = knn_idx;
    a.dense_dist = knn_dist;
    a.dense_count = knn_counts;
    a.error = d_err;
    int rc = launch_brick_warp(a, a.bg.n, st);
    if (rc) return rc;
    int err = 0;
    AFX_CUDA(cudaMemcpyAsync(&err, d_err, sizeof(int), cudaMemcpyDeviceToHost, st));
    AFX_CUDA(cudaStreamSynchronize(st));
    return err ? AFX_ERR_CAPACITY : AFX_OK;
}

int afx_tsdf_warp_weights(float* knn_weights, const float* radii, const uint32_t* knn_idx, const float* knn_dist,
                          const int* knn_counts, long n_voxels, int k, void* stream) {
    if (!knn_weights || !radii || !knn_idx || !knn_dist || !knn_counts || k < 1 || k > kMaxK)
        return AFX_ERR_INVALID_ARGUMENT;
    if (n_voxels <= 0) return AFX_OK;
    tsdf_weights_kernel<<<blocks_for(n_voxels, 256), 256, 0, as_stream(stream)>>>(knn_weights, radii, knn_idx,
                                                                                  knn_dist, knn_counts, n_voxels, k);
    AFX_LAUNCH_CHECK();
    return AFX_OK;
}

int afx_tsdf_vertices(float* vertices, const float voxel_size[3], const float volume_size[3], const int dims[3],
                      void* stream) {
    if (!vertices || !dims) return AFX_ERR_INVALID_ARGUMENT;
    Volume vol = make_volume(dims, voxel_size, volume_size);
    long S = (long)dims[0] * dims[1] * dims[2];
    tsdf_vertices_kernel<<<blocks_for(S, 256), 256, 0, as_stream(stream)>>>(vertices, vol);
    AFX_LAUNCH_CHECK();
    return AFX_OK;
}

int afx_warp_tsdf(float* vertices, const float* transforms, const uint32_t* knn_idx, const float* knn_weights,
                  const int* knn_counts, long n_voxels, int k, void* stream) {
    if (!vertices || !transforms || !knn_idx || !knn_weights || !knn_counts || k < 1 || k > kMaxK)
        return AFX_ERR_INVALID_ARGUMENT;
    if (n_voxels <= 0) return AFX_OK;
    warp_tsdf_kernel<<<blocks_for(n_voxels, 256), 256, 0, as_stream(stream)>>>(vertices, transforms, knn_idx,
                                                                               knn_weights, knn_counts, n_voxels, k);
    AFX_LAUNCH_CHECK();
    return AFX_OK;
}

int afx_count_collisions(int* counts, const float* vertices, const int* knn_counts, const float voxel_size[3],
                         const float volume_size[3], const int dims[3], const float rotate[9], const float translate[3],
                         void* stream) {
    if (!counts || !vertices || !knn_counts || !dims || !rotate || !translate) return AFX_ERR_INVALID_ARGUMENT;
    DenseWarpArgs a;
    a.vol = make_volume(dims, voxel_size, volume_size);
    rotation_inverse(rotate, a.Rinv);
    for (int c = 0; c < 3; ++c) a.t[c] = translate[c];
    long S = (long)dims[0] * dims[1] * dims[2];
    count_collisions_kernel<<<blocks_for(S, 256), 256, 0, as_stream(stream)>>>(counts, vertices, knn_counts, a);
    AFX_LAUNCH_CHECK();
    return AFX_OK;
}

int afx_integrate_warped_tsdf(float* tsdf, float* weights, const float* vertices, const int* collisions,
                              const int* knn_counts, const float* depth, int width, int height, float delta,
                              const float voxel_size[3], const float volume_size[3], const int dims[3],
                              const float rotate[9], const float translate[3], const float K[9], void* stream) {
    if (!tsdf || !weights || !vertices || !collisions || !knn_counts || !depth || !dims || !K)
        return AFX_ERR_INVALID_ARGUMENT;
    DenseWarpArgs a;
    a.vol = make_volume(dims, voxel_size, volume_size);
    rotation_inverse(rotate, a.Rinv);
    for (int c = 0; c < 3; ++c) a.t[c] = translate[c];
    long S = (long)dims[0] * dims[1] * dims[2];
    integrate_warped_kernel<<<blocks_for(S, 256), 256, 0, as_stream(stream)>>>(
        tsdf, weights, vertices, collisions, knn_counts, depth, width, height, delta, make_intrinsics(K), a);
    AFX_LAUNCH_CHECK();
    return AFX_OK;
}

}  // extern "C"
