// afx_mc.cu -- marching cubes (point-cloud and triangle variants, fused into one pass over
// the volume) with warp-aggregated stream compaction, and the lexicographic sort +
// unique of the canonical point cloud (a merge sort: bitonic 2048-element tiles in
// shared memory, then merge-path passes).
//
// Case index, edge interpolation and triangulation follow src/MarchingCubes.cu:294-420
// (corner bit c set when tsdf > iso, cubes skipped when any corner weight is 0, cubes
// x,y,z < dim-2).  The triangulation table is the reference's (packed re-encoding).
#include <cuda.h>

#include <cstring>

#include "afx_host.h"
#include "afx_internal.h"
#include "afx_store.cuh"
#include "afx_tma.h"

namespace afx {

__constant__ uint64_t c_tri_table[256];
__constant__ unsigned short c_edge_table[256];

static const uint64_t kTriTableHost[256] = {
#include "mc_tables.inc"
};

// Corner c of cube (x,y,z) is at (x,y,z) + kCorner[c]; edge e joins corners kEdge[e][0] -> kEdge[e][1]
// (src/MarchingCubes.cu:338-379 and the getVertex calls at :441-507).
__constant__ int c_corner[8][3] = {{1, 1, 0}, {1, 0, 0}, {0, 0, 0}, {0, 1, 0}, {1, 1, 1}, {1, 0, 1}, {0, 0, 1}, {0, 1, 1}};
__constant__ int c_edge[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {4, 5}, {5, 6}, {6, 7}, {7, 4}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};
static const int kEdgeHost[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {4, 5}, {5, 6}, {6, 7}, {7, 4}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};

// The tables are constant: uploaded once per device context (before the first marching-cubes launch,
// which is never inside a stream capture: a session's first frame runs eagerly).
static int upload_tables() {
    static ContextOnce once;
    return once_per_context(once, [](int) {
        unsigned short et[256];
        for (int c = 0; c < 256; ++c) {
            int e = 0;
            for (int i = 0; i < 12; ++i)
                if (((c >> kEdgeHost[i][0]) & 1) != ((c >> kEdgeHost[i][1]) & 1)) e |= 1 << i;
            et[c] = (unsigned short)e;
        }
        AFX_CUDA(cudaMemcpyToSymbol(c_edge_table, et, sizeof(et)));
        AFX_CUDA(cudaMemcpyToSymbol(c_tri_table, kTriTableHost, sizeof(kTriTableHost)));
        return (int)AFX_OK;
    });
}

struct McArgs {
    Volume vol;
    float iso;
    float* points;
    unsigned* point_count;
    long point_cap;
    float* verts;
    unsigned* face_count;  // triangles; vertex count = 3 * faces
    unsigned* vert_count;
    long face_cap;
    int* faces;
    int* error;  // TMA path: set on a tile-load timeout
    const unsigned char* occ;  // brick occupancy (8^3 voxels), or null: process every tile
    int nbx, nby, nbz;
    unsigned* tile_count;      // persistent grid: occupied tiles listed here (with occ), or null
    unsigned* tile_list;
};


// getVertex + interpolate (src/MarchingCubes.cu:294-336)
template <class TT>
AFX_D void edge_vertex(const TT* __restrict__ tsdf, const Volume& vol, int x, int y, int z, int e, float iso,
                       float* o) {
    const int* ca = c_corner[c_edge[e][0]];
    const int* cb = c_corner[c_edge[e][1]];
    const int X = vol.dims[0], Y = vol.dims[1];
    int x1 = x + ca[0], y1 = y + ca[1], z1 = z + ca[2];
    int x2 = x + cb[0], y2 = y + cb[1], z2 = z + cb[2];
    float t0 = vox_ld_t(tsdf, ((long)z1 * Y + y1) * X + x1);
    float t1 = vox_ld_t(tsdf, ((long)z2 * Y + y2) * X + x2);
    float p0[3], p1[3];
    voxel_to_world(x1, y1, z1, vol.vs, vol.half, p0);
    voxel_to_world(x2, y2, z2, vol.vs, vol.half, p1);
    // (double)v < 1e-7 is v < 1e-7f for every float v: 1e-7f is the smallest float >= 1e-7
    if (fabsf(iso - t0) < 1e-7f) {
        o[0] = p0[0]; o[1] = p0[1]; o[2] = p0[2];
        return;
    }
    if (fabsf(iso - t1) < 1e-7f) {
        o[0] = p1[0]; o[1] = p1[1]; o[2] = p1[2];
        return;
    }
    if (fabsf(t0 - t1) < 1e-7f) {
        o[0] = p0[0]; o[1] = p0[1]; o[2] = p0[2];
        return;
    }
    double mu = (double)((iso - t0) / (t1 - t0));
    if (mu > 1.0) mu = 1.0;
    else if (mu < 0) mu = 0.0;
#pragma unroll
    for (int c = 0; c < 3; ++c) o[c] = (float)__dadd_rn((double)p0[c], __dmul_rn(mu, (double)(p1[c] - p0[c])));
}

AFX_D bool vne(const float* a, const float* b) { return a[0] != b[0] || a[1] != b[1] || a[2] != b[2]; }

// Warp-aggregated append: returns this lane's base index for `n` items.
AFX_D unsigned warp_append(unsigned* counter, unsigned n) {
    const int lane = threadIdx.x & 31;
    unsigned x = n;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        unsigned y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    unsigned total = __shfl_sync(0xffffffffu, x, 31);
    unsigned base = 0;
    if (lane == 31 && total) base = atomicAdd(counter, total);
    base = __shfl_sync(0xffffffffu, base, 31);
    return base + x - n;
}

// Vertices and triangles of one cube (all lanes of the warp call this together: the appends are
// warp-aggregated).  Emits the point-cloud vertices (marchingCubesMeshKernel) and/or the
// triangles (marchingCubesFullKernel).
template <bool kPoints, bool kMesh, class TT>
AFX_D void mc_emit(const TT* __restrict__ tsdf, const McArgs& a, int x, int y, int z, int ci, bool active) {
    const unsigned et = active ? c_edge_table[ci] : 0u;
    float ep[12][3];
    if (active) {
#pragma unroll
        for (int e = 0; e < 12; ++e)
            if (et & (1u << e)) edge_vertex(tsdf, a.vol, x, y, z, e, a.iso, ep[e]);
    }
    if (kPoints) {
        unsigned n = __popc(et);
        unsigned pos = warp_append(a.point_count, n);
        if (active)
            for (int e = 0; e < 12; ++e)
                if (et & (1u << e)) {
                    if (pos < a.point_cap) {
                        float* o = a.points + 3 * (long)pos;
                        o[0] = ep[e][0]; o[1] = ep[e][1]; o[2] = ep[e][2];
                    }
                    ++pos;
                }
    }
    if (kMesh) {
        uint64_t tri = active ? c_tri_table[ci] : 0xFull;
        unsigned nt = 0;
        for (int s = 0; s < 15; s += 3) {
            int e0 = (int)((tri >> (4 * s)) & 0xF);
            if (e0 == 0xF) break;
            int e1 = (int)((tri >> (4 * (s + 1))) & 0xF), e2 = (int)((tri >> (4 * (s + 2))) & 0xF);
            if (vne(ep[e0], ep[e1]) && vne(ep[e0], ep[e2]) && vne(ep[e1], ep[e2])) ++nt;
        }
        unsigned f = warp_append(a.face_count, nt);
        for (int s = 0; s < 15; s += 3) {
            int e0 = (int)((tri >> (4 * s)) & 0xF);
            if (e0 == 0xF) break;
            int e1 = (int)((tri >> (4 * (s + 1))) & 0xF), e2 = (int)((tri >> (4 * (s + 2))) & 0xF);
            if (!(vne(ep[e0], ep[e1]) && vne(ep[e0], ep[e2]) && vne(ep[e1], ep[e2]))) continue;
            if (f < a.face_cap) {
                float* o = a.verts + 9 * (long)f;
                const int es[3] = {e0, e1, e2};
#pragma unroll
                for (int t = 0; t < 3; ++t) {
                    o[3 * t] = ep[es[t]][0];
                    o[3 * t + 1] = ep[es[t]][1];
                    o[3 * t + 2] = ep[es[t]][2];
                }
                int* fo = a.faces + 3 * (long)f;
                fo[0] = (int)(3 * f);
                fo[1] = (int)(3 * f + 1);
                fo[2] = (int)(3 * f + 2);
            }
            ++f;
        }
    }
}

// A CTA covers a 32 x 8 patch of cube columns and a run of kMcZ cubes along z; each thread
// marches its column, keeping the four corner values of the slice it shares with the next cube
// (one new tsdf/weight row pair per step instead of eight corners, no index divisions).  Warps
// are aligned to x rows, so the loads are coalesced and the warp-level append stays converged.
// Emits the point-cloud vertices (marchingCubesMeshKernel) and/or the triangles
// (marchingCubesFullKernel) of each cube.
constexpr int kMcX = 32, kMcY = 8, kMcZ = 16;

// False when no 8^3 brick holding a cube origin of the tile [x0, x0+32) x [y0, y0+8) x [z0, z0+zr)
// has a voxel with a weight.  A cube is active only if all eight corners have a weight, its origin
// corner among them, so such a tile has no active cube.  Every thread evaluates it (same answer).
AFX_D bool tile_occupied(const McArgs& a, int x0, int y0, int z0, int zr) {
    if (!a.occ) return true;
    const int bx1 = min((x0 + kMcX - 1) >> 3, a.nbx - 1), by1 = min((y0 + kMcY - 1) >> 3, a.nby - 1);
    const int bz1 = min((z0 + zr - 1) >> 3, a.nbz - 1);
    for (int bz = z0 >> 3; bz <= bz1; ++bz)
        for (int by = y0 >> 3; by <= by1; ++by)
            for (int bx = x0 >> 3; bx <= bx1; ++bx)
                if (__ldg(a.occ + ((long)bz * a.nby + by) * a.nbx + bx)) return true;
    return false;
}

// tsdf/weight of the corners (x, y), (x+1, y), (x, y+1), (x+1, y+1) of slice z
template <class TT, class WT>
AFX_D void mc_slice(const TT* __restrict__ tsdf, const WT* __restrict__ w, long row0, long X, float t[4],
                    float ww[4]) {
    t[0] = vox_ld_t(tsdf, row0);
    t[1] = vox_ld_t(tsdf, row0 + 1);
    t[2] = vox_ld_t(tsdf, row0 + X);
    t[3] = vox_ld_t(tsdf, row0 + X + 1);
    ww[0] = vox_ld_w(w, row0);
    ww[1] = vox_ld_w(w, row0 + 1);
    ww[2] = vox_ld_w(w, row0 + X);
    ww[3] = vox_ld_w(w, row0 + X + 1);
}

template <class TT, class WT, bool kPoints, bool kMesh>
__global__ void __launch_bounds__(kMcX * kMcY) mc_kernel(const TT* __restrict__ tsdf,
                                                        const WT* __restrict__ weights, McArgs a) {
    const int nx = a.vol.dims[0] - 2, ny = a.vol.dims[1] - 2, nz = a.vol.dims[2] - 2;
    const long X = a.vol.dims[0], XY = X * a.vol.dims[1];
    const int x = blockIdx.x * kMcX + threadIdx.x, y = blockIdx.y * kMcY + threadIdx.y;
    const int z0 = blockIdx.z * kMcZ, z1 = min(z0 + kMcZ, nz);
    if (!tile_occupied(a, blockIdx.x * kMcX, blockIdx.y * kMcY, z0, kMcZ)) return;  // uniform over the CTA
    const bool col = x < nx && y < ny;
    const long base = (long)y * X + x;
    float t0[4] = {0.f, 0.f, 0.f, 0.f}, w0[4] = {0.f, 0.f, 0.f, 0.f};
    if (col) mc_slice(tsdf, weights, (long)z0 * XY + base, X, t0, w0);
    for (int z = z0; z < z1; ++z) {
        float t1[4] = {0.f, 0.f, 0.f, 0.f}, w1[4] = {0.f, 0.f, 0.f, 0.f};
        if (col) mc_slice(tsdf, weights, (long)(z + 1) * XY + base, X, t1, w1);
        int ci = 0;
        if (col) {
            // corners (src/MarchingCubes.cu:338-379): c0 (1,1,0) c1 (1,0,0) c2 (0,0,0) c3 (0,1,0),
            // c4..c7 the same one slice up; slot s of a slice is (x + (s & 1), y + (s >> 1))
            const float ct[8] = {t0[3], t0[1], t0[0], t0[2], t1[3], t1[1], t1[0], t1[2]};
            const float cw[8] = {w0[3], w0[1], w0[0], w0[2], w1[3], w1[1], w1[0], w1[2]};
            bool any_zero = false;
#pragma unroll
            for (int c = 0; c < 8; ++c) any_zero |= (cw[c] == 0.0f);
            if (!any_zero)
#pragma unroll
                for (int c = 0; c < 8; ++c)
                    if (ct[c] > a.iso) ci |= 1 << c;
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            t0[q] = t1[q];
            w0[q] = w1[q];
        }
        const bool active = ci != 0 && ci != 255;
        if (!__any_sync(0xffffffffu, active)) continue;
        mc_emit<kPoints, kMesh>(tsdf, a, x, y, z, ci, active);
    }
}

// Same cubes as mc_kernel, with the CTA's whole brick of corner values -- 40 x 9 x (ZR + 1)
// elements of TSDF and of weights, x padded to a 16-byte multiple -- brought into shared memory by
// two TMA tile loads on one mbarrier, so the march reads no global memory for inactive cubes.
constexpr int kMcTX = 40;  // box width in elements (>= kMcX + 1; 160 B in FP32, 80 B in FP16)
// each brick starts on a 128-byte boundary (TMA destination alignment), plus slack to align the base
__host__ __device__ constexpr size_t mc_brick_bytes(size_t elem, int zr) {
    return ((size_t)kMcTX * (kMcY + 1) * (zr + 1) * elem + 127) / 128 * 128;
}
__host__ __device__ constexpr size_t mc_tma_smem(size_t elem, int zr) { return 2 * mc_brick_bytes(elem, zr) + 128; }

AFX_D uint32_t mc_smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

AFX_D float smem_t(const float* p, int i) { return p[i]; }
AFX_D float smem_t(const __half* p, int i) { return __half2float(p[i]); }
AFX_D bool smem_w_zero(const float* p, int i) { return p[i] == 0.0f; }
AFX_D bool smem_w_zero(const unsigned short* p, int i) { return p[i] == 0; }

// ZR: cubes per CTA along z (the tile depth the autotuner chooses: 8, 16 or 32)
template <class TT, class WT, bool kPoints, bool kMesh, int ZR>
__global__ void __launch_bounds__(kMcX * kMcY) mc_tma_kernel(const __grid_constant__ CUtensorMap map_t,
                                                            const __grid_constant__ CUtensorMap map_w,
                                                            const TT* __restrict__ tsdf, McArgs a) {
    static_assert(sizeof(TT) == sizeof(WT), "value and weight bricks share one layout");
    static_assert(ZR <= 64, "the queue entry keeps z in 6 bits");
    constexpr size_t kMcBrickBytes = mc_brick_bytes(sizeof(TT), ZR);
    extern __shared__ __align__(128) unsigned char mc_raw[];
    __shared__ alignas(8) unsigned long long mbar;
    __shared__ unsigned q[kMcX * kMcY * ZR];  // surface cubes of this CTA: ci | x << 8 | y << 13 | z << 16
    __shared__ unsigned q_n;
    constexpr int kSlice = kMcTX * (kMcY + 1);
    const uint32_t pad = (128u - (mc_smem_u32(mc_raw) & 127u)) & 127u;
    TT* st = reinterpret_cast<TT*>(mc_raw + pad);
    WT* sw = reinterpret_cast<WT*>(mc_raw + pad + kMcBrickBytes);
    const int tid = threadIdx.y * kMcX + threadIdx.x;
    const int x0 = blockIdx.x * kMcX, y0 = blockIdx.y * kMcY, z0 = blockIdx.z * ZR;
    if (!tile_occupied(a, x0, y0, z0, ZR)) return;  // uniform over the CTA, before any barrier or copy
    if (((mc_smem_u32(st) | mc_smem_u32(sw)) & 127u) != 0u) {  // never expected: refuse rather than fault
        if (tid == 0 && a.error) atomicOr(a.error, ERRF_TMA);
        return;
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mc_smem_u32(&mbar)));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        q_n = 0;
    }
    __syncthreads();
    if (tid == 0) {
        const unsigned bytes = (unsigned)(kSlice * (ZR + 1) * (sizeof(TT) + sizeof(WT)));
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mc_smem_u32(&mbar)), "r"(bytes)
                     : "memory");
        asm volatile(
            "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
            "[%5];" ::"r"(mc_smem_u32(st)),
            "l"(&map_t), "r"(x0), "r"(y0), "r"(z0), "r"(mc_smem_u32(&mbar))
            : "memory");
        asm volatile(
            "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
            "[%5];" ::"r"(mc_smem_u32(sw)),
            "l"(&map_w), "r"(x0), "r"(y0), "r"(z0), "r"(mc_smem_u32(&mbar))
            : "memory");
    }
    // bounded wait for the brick (phase 0); the give-up decision is uniform across the CTA
    bool done = false;
    for (int it = 0; it < (1 << 22) && !done; ++it) {
        uint32_t ok;
        asm volatile(
            "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0; selp.u32 %0, 1, 0, p; }"
            : "=r"(ok)
            : "r"(mc_smem_u32(&mbar))
            : "memory");
        done = ok != 0;
    }
    if (__syncthreads_or(!done)) {
        if (tid == 0 && a.error) atomicOr(a.error, ERRF_TMA | ERRF_TIMEOUT);
        // the copies may still land: wait for them (bounded) before the CTA's shared memory goes
        for (int it = 0; it < (1 << 22); ++it) {
            uint32_t ok;
            asm volatile(
                "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0; selp.u32 %0, 1, 0, p; }"
                : "=r"(ok)
                : "r"(mc_smem_u32(&mbar))
                : "memory");
            if (ok) break;
        }
        return;
    }
    const int nx = a.vol.dims[0] - 2, ny = a.vol.dims[1] - 2, nz = a.vol.dims[2] - 2;
    const int x = x0 + threadIdx.x, y = y0 + threadIdx.y;
    const int z1 = min(z0 + ZR, nz);
    const bool col = x < nx && y < ny;
    const int o00 = threadIdx.y * kMcTX + threadIdx.x;  // (x, y) within a slice
    for (int z = z0; z < z1; ++z) {
        const int s0 = (z - z0) * kSlice + o00, s1 = s0 + kSlice;
        int ci = 0;
        if (col) {
            // corners (src/MarchingCubes.cu:338-379): c0 (1,1,0) c1 (1,0,0) c2 (0,0,0) c3 (0,1,0), c4..c7 one slice up
            const int off[8] = {s0 + kMcTX + 1, s0 + 1, s0, s0 + kMcTX, s1 + kMcTX + 1, s1 + 1, s1, s1 + kMcTX};
            bool any_zero = false;
#pragma unroll
            for (int c = 0; c < 8; ++c) any_zero |= smem_w_zero(sw, off[c]);
            if (!any_zero)
#pragma unroll
                for (int c = 0; c < 8; ++c)
                    if (smem_t(st, off[c]) > a.iso) ci |= 1 << c;
        }
        const bool active = ci != 0 && ci != 255;
        // queue the surface cubes (warp-aggregated), processed densely below
        const unsigned bal = __ballot_sync(0xffffffffu, active);
        if (bal) {
            const int lane = threadIdx.x & 31;  // blockDim.x == 32: a warp is one row of x
            unsigned base = 0;
            if (lane == 0) base = atomicAdd(&q_n, (unsigned)__popc(bal));
            base = __shfl_sync(0xffffffffu, base, 0);
            if (active)
                q[base + __popc(bal & ((1u << lane) - 1))] =
                    (unsigned)ci | ((unsigned)threadIdx.x << 8) | ((unsigned)threadIdx.y << 13) | ((unsigned)(z - z0) << 16);
        }
    }
    __syncthreads();
    // edge vertices and triangles of the queued cubes, one per thread: the FP64 interpolation
    // then runs with full warps instead of one or two surface lanes per warp
    const unsigned nq = q_n;
    for (unsigned r0 = 0; r0 < nq; r0 += kMcX * kMcY) {
        const unsigned qi = r0 + tid;
        const bool act = qi < nq;
        const unsigned e = act ? q[qi] : 0u;
        mc_emit<kPoints, kMesh>(tsdf, a, x0 + (int)((e >> 8) & 31u), y0 + (int)((e >> 13) & 7u),
                                z0 + (int)((e >> 16) & 63u), (int)(e & 255u), act);
    }
}

// The same cubes again, by a persistent grid: a CTA walks the tiles blockIdx.x, + gridDim.x, ...
// with two stages of TMA-loaded bricks.  The load of tile k + 2 is issued as soon as tile k's
// classification has read its stage, so loads overlap the FP64 edge interpolation and the appends
// of the tiles before.  Every wait is bounded; on a timeout the CTA flags the error, waits (bounded)
// for the loads it issued and leaves.
AFX_D bool mc_wait(uint32_t bar, uint32_t parity) {
    for (int it = 0; it < (1 << 22); ++it) {
        uint32_t ok;
        asm volatile("{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
                     : "=r"(ok)
                     : "r"(bar), "r"(parity)
                     : "memory");
        if (ok) return true;
    }
    return false;
}

// The occupied tiles of the volume (those tile_occupied accepts), in no particular order.
__global__ void mc_tile_list_kernel(McArgs a, int tx_n, int ty_n, int tz_n, int zr) {
    const long nt = (long)tx_n * ty_n * tz_n;
    AFX_GRID_STRIDE(t, nt) {
        const int tx = (int)(t % tx_n), ty = (int)((t / tx_n) % ty_n), tz = (int)(t / ((long)tx_n * ty_n));
        if (tile_occupied(a, tx * kMcX, ty * kMcY, tz * zr, zr)) a.tile_list[atomicAdd(a.tile_count, 1u)] = (unsigned)t;
    }
}

// Persistent grid over the tiles -- every tile, or with a.tile_list the listed ones -- with two
// stages of TMA bricks: the next tile's brick loads while this one is classified.
template <class TT, class WT, bool kPoints, bool kMesh, int ZR>
__global__ void __launch_bounds__(kMcX * kMcY) mc_pipe_kernel(const __grid_constant__ CUtensorMap map_t,
                                                             const __grid_constant__ CUtensorMap map_w,
                                                             const TT* __restrict__ tsdf, McArgs a, int tx_n, int ty_n,
                                                             int tz_n) {
    static_assert(sizeof(TT) == sizeof(WT), "value and weight bricks share one layout");
    static_assert(ZR <= 64, "the queue entry keeps z in 6 bits");
    constexpr size_t kBrick = mc_brick_bytes(sizeof(TT), ZR);
    constexpr int kSlice = kMcTX * (kMcY + 1);
    constexpr unsigned kBytes = (unsigned)(kSlice * (ZR + 1) * (sizeof(TT) + sizeof(WT)));
    extern __shared__ __align__(128) unsigned char mc_raw[];
    __shared__ alignas(8) unsigned long long mbar[2];
    __shared__ unsigned q[kMcX * kMcY * ZR];
    __shared__ unsigned q_n;
    const uint32_t pad = (128u - (mc_smem_u32(mc_raw) & 127u)) & 127u;
    TT* st[2];
    WT* sw[2];
    for (int k = 0; k < 2; ++k) {
        st[k] = reinterpret_cast<TT*>(mc_raw + pad + (2 * k) * kBrick);
        sw[k] = reinterpret_cast<WT*>(mc_raw + pad + (2 * k + 1) * kBrick);
    }
    const int tid = threadIdx.y * kMcX + threadIdx.x;
    const long nall = (long)tx_n * ty_n * tz_n;
    const long nt = a.tile_list ? min((long)*a.tile_count, nall) : nall;
    if ((mc_smem_u32(st[0]) & 127u) != 0u) {  // never expected: refuse rather than fault
        if (tid == 0 && a.error) atomicOr(a.error, ERRF_TMA);
        return;
    }
    auto origin = [&](long i, int& x0, int& y0, int& z0) {  // i-th tile of this launch
        const long t = a.tile_list ? (long)a.tile_list[i] : i;
        const int tx = (int)(t % tx_n), ty = (int)((t / tx_n) % ty_n), tz = (int)(t / ((long)tx_n * ty_n));
        x0 = tx * kMcX;
        y0 = ty * kMcY;
        z0 = tz * ZR;
    };
    auto issue = [&](int s, long t) {  // one thread
        int x0, y0, z0;
        origin(t, x0, y0, z0);
        const uint32_t bar = mc_smem_u32(&mbar[s]);
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(kBytes) : "memory");
        asm volatile(
            "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
            "[%5];" ::"r"(mc_smem_u32(st[s])),
            "l"(&map_t), "r"(x0), "r"(y0), "r"(z0), "r"(bar)
            : "memory");
        asm volatile(
            "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
            "[%5];" ::"r"(mc_smem_u32(sw[s])),
            "l"(&map_w), "r"(x0), "r"(y0), "r"(z0), "r"(bar)
            : "memory");
    };
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mc_smem_u32(&mbar[0])));
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mc_smem_u32(&mbar[1])));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    const long G = gridDim.x;
    if (tid == 0) {
        if ((long)blockIdx.x < nt) issue(0, blockIdx.x);
        if ((long)blockIdx.x + G < nt) issue(1, blockIdx.x + G);
    }
    const int nx = a.vol.dims[0] - 2, ny = a.vol.dims[1] - 2, nz = a.vol.dims[2] - 2;
    const int o00 = threadIdx.y * kMcTX + threadIdx.x;
    int k = 0;
    for (long t = blockIdx.x; t < nt; t += G, ++k) {
        const int s = k & 1;
        const uint32_t parity = (uint32_t)((k >> 1) & 1);
        const bool ok = mc_wait(mc_smem_u32(&mbar[s]), parity);
        if (__syncthreads_or(!ok)) {
            if (tid == 0 && a.error) atomicOr(a.error, ERRF_TMA | ERRF_TIMEOUT);
            // loads issued and not yet waited for: this tile's (stage s, if it timed out) and the next
            mc_wait(mc_smem_u32(&mbar[s]), parity);
            if (t + G < nt) mc_wait(mc_smem_u32(&mbar[s ^ 1]), (uint32_t)(((k + 1) >> 1) & 1));
            return;
        }
        if (tid == 0) q_n = 0;
        __syncthreads();
        int x0, y0, z0;
        origin(t, x0, y0, z0);
        const int x = x0 + threadIdx.x, y = y0 + threadIdx.y;
        const int z1 = min(z0 + ZR, nz);
        const bool col = x < nx && y < ny;
        for (int z = z0; z < z1; ++z) {
            const int s0 = (z - z0) * kSlice + o00, s1 = s0 + kSlice;
            int ci = 0;
            if (col) {
                const int off[8] = {s0 + kMcTX + 1, s0 + 1, s0, s0 + kMcTX, s1 + kMcTX + 1, s1 + 1, s1, s1 + kMcTX};
                bool any_zero = false;
#pragma unroll
                for (int c = 0; c < 8; ++c) any_zero |= smem_w_zero(sw[s], off[c]);
                if (!any_zero)
#pragma unroll
                    for (int c = 0; c < 8; ++c)
                        if (smem_t(st[s], off[c]) > a.iso) ci |= 1 << c;
            }
            const bool active = ci != 0 && ci != 255;
            const unsigned bal = __ballot_sync(0xffffffffu, active);
            if (bal) {
                const int lane = threadIdx.x & 31;
                unsigned base = 0;
                if (lane == 0) base = atomicAdd(&q_n, (unsigned)__popc(bal));
                base = __shfl_sync(0xffffffffu, base, 0);
                if (active)
                    q[base + __popc(bal & ((1u << lane) - 1))] = (unsigned)ci | ((unsigned)threadIdx.x << 8) |
                                                                 ((unsigned)threadIdx.y << 13) | ((unsigned)(z - z0) << 16);
            }
        }
        __syncthreads();  // stage s has been read: it can take tile t + 2G
        if (tid == 0 && t + 2 * G < nt) issue(s, t + 2 * G);
        const unsigned nq = q_n;
        for (unsigned r0 = 0; r0 < nq; r0 += kMcX * kMcY) {
            const unsigned qi = r0 + tid;
            const bool act = qi < nq;
            const unsigned e = act ? q[qi] : 0u;
            mc_emit<kPoints, kMesh>(tsdf, a, x0 + (int)((e >> 8) & 31u), y0 + (int)((e >> 13) & 7u),
                                    z0 + (int)((e >> 16) & 63u), (int)(e & 255u), act);
        }
        __syncthreads();  // the queue is reused by the next tile
    }
}

__global__ void mc_vert_count_kernel(const unsigned* face_count, unsigned* vert_count) {
    *vert_count = 3u * *face_count;
}

// 3-D tiled map over one voxel array (element type `type`, `elem` bytes); the box is one CTA's
// brick of corner values.
static bool make_volume_map(CUtensorMap* map, const void* base, const Volume& vol, CUtensorMapDataType type,
                            size_t elem, int zr) {
    if ((vol.dims[0] * elem) % 16 != 0 || (reinterpret_cast<uintptr_t>(base) & 15) != 0) return false;
    EncodeTiledFn fn = encode_fn();
    if (!fn) return false;
    cuuint64_t dims[3] = {(cuuint64_t)vol.dims[0], (cuuint64_t)vol.dims[1], (cuuint64_t)vol.dims[2]};
    cuuint64_t strides[2] = {(cuuint64_t)vol.dims[0] * elem, (cuuint64_t)vol.dims[0] * vol.dims[1] * elem};
    cuuint32_t box[3] = {(cuuint32_t)kMcTX, (cuuint32_t)(kMcY + 1), (cuuint32_t)(zr + 1)};
    cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = fn(map, type, 3, const_cast<void*>(base), dims, strides, box, estr,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
}

template <class TT, class WT, bool kPoints, bool kMesh, int ZR>
static void mc_launch_tma(const TT* tsdf, const McArgs& a, const CUtensorMap* mt, const CUtensorMap* mw,
                          cudaStream_t st) {
    constexpr int smem = (int)mc_tma_smem(sizeof(TT), ZR);
    static ContextOnce once;  // per instantiation: the dynamic shared memory opt-in
    once_per_context(once, [](int) {
        return note_cuda_error(cudaFuncSetAttribute(mc_tma_kernel<TT, WT, kPoints, kMesh, ZR>,
                                                    cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    });
    const dim3 grid((unsigned)((a.vol.dims[0] - 2 + kMcX - 1) / kMcX), (unsigned)((a.vol.dims[1] - 2 + kMcY - 1) / kMcY),
                    (unsigned)((a.vol.dims[2] - 2 + ZR - 1) / ZR));
    mc_tma_kernel<TT, WT, kPoints, kMesh, ZR><<<grid, dim3(kMcX, kMcY), smem, st>>>(*mt, *mw, tsdf, a);
}

template <class TT, class WT, bool kPoints, bool kMesh, int ZR>
static void mc_launch_pipe(const TT* tsdf, const McArgs& a, const CUtensorMap* mt, const CUtensorMap* mw,
                           cudaStream_t st) {
    constexpr int smem = (int)(4 * mc_brick_bytes(sizeof(TT), ZR) + 128);
    static ContextOnce once;  // per instantiation: opt-in and resident CTAs per SM, per device
    static int per_sm_dev[kMaxDevices], sms_dev[kMaxDevices];
    once_per_context(once, [](int dev) {
        int per_sm = 0, sms = 0;
        cudaFuncSetAttribute(mc_pipe_kernel<TT, WT, kPoints, kMesh, ZR>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             smem);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, mc_pipe_kernel<TT, WT, kPoints, kMesh, ZR>, kMcX * kMcY,
                                                      smem);
        cudaGetLastError();
        per_sm_dev[dev] = per_sm < 1 ? 1 : per_sm;
        sms_dev[dev] = sms < 1 ? 1 : sms;
        return (int)AFX_OK;
    });
    int dev = 0;
    cudaGetDevice(&dev);
    const int per_sm = per_sm_dev[dev] < 1 ? 1 : per_sm_dev[dev], sms = sms_dev[dev] < 1 ? 1 : sms_dev[dev];
    const int tx = (a.vol.dims[0] - 2 + kMcX - 1) / kMcX, ty = (a.vol.dims[1] - 2 + kMcY - 1) / kMcY,
              tz = (a.vol.dims[2] - 2 + ZR - 1) / ZR;
    const long nt = (long)tx * ty * tz;
    const long grid = nt < (long)sms * per_sm ? nt : (long)sms * per_sm;
    McArgs b = a;
    if (a.occ && a.tile_list && a.tile_count) {
        cudaMemsetAsync(a.tile_count, 0, sizeof(unsigned), st);
        mc_tile_list_kernel<<<grid_for(nt, 256), 256, 0, st>>>(a, tx, ty, tz, ZR);
    } else {
        b.tile_list = nullptr;
    }
    mc_pipe_kernel<TT, WT, kPoints, kMesh, ZR><<<(unsigned)grid, dim3(kMcX, kMcY), smem, st>>>(*mt, *mw, tsdf, b, tx,
                                                                                              ty, tz);
}

// Words of the occupied-tile list for a volume (count + one entry per tile of the shallowest depth, 4).
size_t mc_tile_ws_words(const Volume& vol) {
    const long tx = (vol.dims[0] - 2 + kMcX - 1) / kMcX, ty = (vol.dims[1] - 2 + kMcY - 1) / kMcY,
               tz = (vol.dims[2] - 2 + 4 - 1) / 4;
    return (size_t)(1 + (tx > 0 ? tx : 0) * (ty > 0 ? ty : 0) * (tz > 0 ? tz : 0));
}

// tile: kMcTileTma16 (default), kMcTileTma8, kMcTileTma32 (TMA bricks of that many cubes along z),
// kMcTilePipe8 / kMcTilePipe16 / kMcTilePipe4 (persistent grid with two stages of bricks 8, 16 or 4
// cubes deep) or
// kMcTileColumn (column march from global memory, 16 cubes along z).  mt/mw are the maps encoded for
// that depth, or null (then the column march runs).
template <class TT, class WT, bool kPoints, bool kMesh>
static void mc_launch(const TT* tsdf, const WT* weights, const McArgs& a, const CUtensorMap* mt, const CUtensorMap* mw,
                      int tile, cudaStream_t st) {
    if (mt && tile == kMcTilePipe8) {
        mc_launch_pipe<TT, WT, kPoints, kMesh, 8>(tsdf, a, mt, mw, st);
    } else if (mt && tile == kMcTilePipe4) {
        mc_launch_pipe<TT, WT, kPoints, kMesh, 4>(tsdf, a, mt, mw, st);
    } else if (mt && tile == kMcTilePipe16) {
        mc_launch_pipe<TT, WT, kPoints, kMesh, 16>(tsdf, a, mt, mw, st);
    } else if (mt && tile == kMcTileTma8) {
        mc_launch_tma<TT, WT, kPoints, kMesh, 8>(tsdf, a, mt, mw, st);
    } else if (mt && tile == kMcTileTma32) {
        mc_launch_tma<TT, WT, kPoints, kMesh, 32>(tsdf, a, mt, mw, st);
    } else if (mt) {
        mc_launch_tma<TT, WT, kPoints, kMesh, 16>(tsdf, a, mt, mw, st);
    } else {
        const dim3 grid((unsigned)((a.vol.dims[0] - 2 + kMcX - 1) / kMcX),
                        (unsigned)((a.vol.dims[1] - 2 + kMcY - 1) / kMcY), (unsigned)((a.vol.dims[2] - 2 + kMcZ - 1) / kMcZ));
        mc_kernel<TT, WT, kPoints, kMesh><<<grid, dim3(kMcX, kMcY), 0, st>>>(tsdf, weights, a);
    }
}

template <class TT, class WT>
static void mc_launch_any(const TT* tsdf, const WT* weights, const McArgs& a, const CUtensorMap* mt,
                          const CUtensorMap* mw, bool P, bool M, int tile, cudaStream_t st) {
    if (P && M) mc_launch<TT, WT, true, true>(tsdf, weights, a, mt, mw, tile, st);
    else if (P) mc_launch<TT, WT, true, false>(tsdf, weights, a, mt, mw, tile, st);
    else mc_launch<TT, WT, false, true>(tsdf, weights, a, mt, mw, tile, st);
}

int mc_fused_impl(const void* tsdf, const void* weights, int fmt, const Volume& vol, float iso, float* points,
                  unsigned* point_count, long point_cap, float* verts, unsigned* vert_count, long vert_cap, int* faces,
                  unsigned* face_count, long face_cap, cudaStream_t st, int* error, int tile,
                  const unsigned char* occ, unsigned* tile_ws) {
    int rc = upload_tables();
    if (rc) return rc;
    McArgs a;
    a.vol = vol;
    a.iso = iso;
    a.points = points;
    a.point_count = point_count;
    a.point_cap = point_cap;
    a.verts = verts;
    a.face_count = face_count;
    a.vert_count = vert_count;
    a.face_cap = face_cap < vert_cap / 3 ? face_cap : vert_cap / 3;
    a.faces = faces;
    a.error = error;
    a.occ = occ;
    a.tile_count = tile_ws;
    a.tile_list = tile_ws ? tile_ws + 1 : nullptr;
    a.nbx = (vol.dims[0] + 7) / 8;
    a.nby = (vol.dims[1] + 7) / 8;
    a.nbz = (vol.dims[2] + 7) / 8;
    const long ncubes = (long)(vol.dims[0] - 2) * (vol.dims[1] - 2) * (vol.dims[2] - 2);
    if (ncubes <= 0) return AFX_OK;
    const bool P = points != nullptr, M = verts != nullptr;
    if (!P && !M) return AFX_OK;
    // TMA bricks where the caller can receive a load-timeout report and the maps encode
    CUtensorMap mt, mw;
    const bool f16 = fmt == kVoxF16;
    const size_t elem = vox_bytes(fmt);
    const int zr = (tile == kMcTileTma8 || tile == kMcTilePipe8) ? 8 : tile == kMcTilePipe4 ? 4 : tile == kMcTileTma32 ? 32 : 16;
    const bool tma = error && tile != kMcTileColumn &&
                     make_volume_map(&mt, tsdf, vol, f16 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16 :
                                                           CU_TENSOR_MAP_DATA_TYPE_FLOAT32, elem, zr) &&
                     make_volume_map(&mw, weights, vol, f16 ? CU_TENSOR_MAP_DATA_TYPE_UINT16 :
                                                              CU_TENSOR_MAP_DATA_TYPE_FLOAT32, elem, zr);
    if (f16)
        mc_launch_any(static_cast<const __half*>(tsdf), static_cast<const unsigned short*>(weights), a,
                      tma ? &mt : nullptr, tma ? &mw : nullptr, P, M, tile, st);
    else
        mc_launch_any(static_cast<const float*>(tsdf), static_cast<const float*>(weights), a, tma ? &mt : nullptr,
                      tma ? &mw : nullptr, P, M, tile, st);
    AFX_LAUNCH_CHECK();
    if (M && vert_count) {
        mc_vert_count_kernel<<<1, 1, 0, st>>>(face_count, vert_count);
        AFX_LAUNCH_CHECK();
    }
    return AFX_OK;
}

// ------------------------------------------------------------------------------------
// Lexicographic sort + unique of float triples
// ------------------------------------------------------------------------------------

struct Key3 {
    unsigned k[3];
};

AFX_D unsigned f2key(float f) {
    unsigned u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
AFX_D float key2f(unsigned k) { return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k); }
AFX_D bool key_less(const Key3& a, const Key3& b) {
    if (a.k[0] != b.k[0]) return a.k[0] < b.k[0];
    if (a.k[1] != b.k[1]) return a.k[1] < b.k[1];
    return a.k[2] < b.k[2];
}
AFX_D bool key_le(const Key3& a, const Key3& b) { return !key_less(b, a); }

constexpr int kSortTile = 2048;
constexpr int kSortThreads = 1024;
constexpr int kSortCluster = 16;

AFX_D unsigned sort_rank() {
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
AFX_D unsigned sort_ncta() {
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
    return r;
}
AFX_D void sort_cluster_barrier() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// Bitonic sort of one tile of up to kSortTile points (padding sorts last) into `out`.
AFX_D void sort_tile(const float* __restrict__ pts, Key3* out, long base, long n, Key3* s) {
    __syncthreads();
    for (int i = threadIdx.x; i < kSortTile; i += blockDim.x) {
        const long j = base + i;
        Key3 k;
        if (j < n) {
            k.k[0] = f2key(pts[3 * j]);
            k.k[1] = f2key(pts[3 * j + 1]);
            k.k[2] = f2key(pts[3 * j + 2]);
        } else {
            k.k[0] = k.k[1] = k.k[2] = 0xffffffffu;
        }
        s[i] = k;
    }
    __syncthreads();
    for (int size = 2; size <= kSortTile; size <<= 1)
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            for (int p = threadIdx.x; p < kSortTile / 2; p += blockDim.x) {
                const int i = 2 * stride * (p / stride) + (p % stride), j = i + stride;
                const bool asc = (i & size) == 0;
                const Key3 a = s[i], b = s[j];
                if (key_less(b, a) == asc) {
                    s[i] = b;
                    s[j] = a;
                }
            }
            __syncthreads();
        }
    for (int i = threadIdx.x; i < kSortTile; i += blockDim.x) {
        const long j = base + i;
        if (j < n) out[j] = s[i];
    }
}

// Outputs [o0, o0 + kSortTile) of merging the sorted runs of length L around o0 (merge path).
AFX_D void merge_chunk(const Key3* __restrict__ in, Key3* __restrict__ out, long n, long L, long o0, Key3* s,
                       long* split) {
    const long pair = o0 / (2 * L) * (2 * L);
    const long a0 = pair, na = min(L, n - a0);
    const long b0 = pair + L, nb = max(0L, min(L, n - b0));
    const long d0 = o0 - pair, d1 = min(d0 + kSortTile, na + nb);
    __syncthreads();
    if (threadIdx.x < 2) {
        const long d = threadIdx.x == 0 ? d0 : d1;
        long lo = max(0L, d - nb), hi = min(d, na);
        while (lo < hi) {
            const long mid = (lo + hi) >> 1;
            if (key_le(in[a0 + mid], in[b0 + d - 1 - mid])) lo = mid + 1;
            else hi = mid;
        }
        split[threadIdx.x] = lo;
    }
    __syncthreads();
    const long i0 = split[0], i1 = split[1];
    const long j0 = d0 - i0, j1 = d1 - i1;
    const int la = (int)(i1 - i0), lb = (int)(j1 - j0);
    for (int t = threadIdx.x; t < la + lb; t += blockDim.x) s[t] = t < la ? in[a0 + i0 + t] : in[b0 + j0 + (t - la)];
    __syncthreads();
    const int tot = la + lb;
    const int per = kSortTile / blockDim.x;  // blockDim.x divides kSortTile
    const int q0 = threadIdx.x * per;
    if (q0 < tot) {
        int lo = max(0, q0 - lb), hi = min(q0, la);
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (key_le(s[mid], s[la + q0 - 1 - mid])) lo = mid + 1;
            else hi = mid;
        }
        int ia = lo, ib = q0 - lo;
        for (int q = q0; q < q0 + per && q < tot; ++q) {
            const bool takeA = ib >= lb || (ia < la && key_le(s[ia], s[la + ib]));
            out[o0 + q] = takeA ? s[ia++] : s[la + ib++];
        }
    }
}

AFX_D bool key_same_point(const Key3& a, const Key3& b) {
    return key2f(a.k[0]) == key2f(b.k[0]) && key2f(a.k[1]) == key2f(b.k[1]) && key2f(a.k[2]) == key2f(b.k[2]);
}

// Lexicographic sort + unique of the point cloud in one launch of one thread-block cluster:
// tiles of kSortTile sorted in shared memory, merge-path passes until one run remains (the
// pass count follows the live count on the device), then unique by float equality of
// consecutive points and an ordered compaction back into `pts`.  Phases are separated by the
// hardware cluster barrier.
__global__ void __launch_bounds__(kSortThreads, 1) sort_unique_kernel(float* pts, unsigned* count, long n_max,
                                                                     Key3* buf0, Key3* buf1, unsigned* tile_cnt,
                                                                     const unsigned* only_if) {
    __shared__ Key3 s[kSortTile];
    if (only_if && *only_if == 0u) return;  // the column-bucket sort did the work
    __shared__ long split[2];
    __shared__ unsigned wsum[kSortThreads / 32];
    __shared__ unsigned s_base;
    const long n = min((long)*count, n_max);
    const unsigned rank = sort_rank(), ncta = sort_ncta();
    const long tiles = (n + kSortTile - 1) / kSortTile;
    for (long t = rank; t < tiles; t += ncta) sort_tile(pts, buf0, t * kSortTile, n, s);
    sort_cluster_barrier();
    Key3* src = buf0;
    Key3* dst = buf1;
    for (long L = kSortTile; L < n; L <<= 1) {
        for (long t = rank; t < tiles; t += ncta) merge_chunk(src, dst, n, L, t * kSortTile, s, split);
        sort_cluster_barrier();
        Key3* tmp = src;
        src = dst;
        dst = tmp;
    }
    // unique flags and per-tile counts
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (long t = rank; t < tiles; t += ncta) {
        unsigned c = 0;
        for (long i = t * kSortTile + threadIdx.x; i < min(n, (t + 1) * kSortTile); i += blockDim.x)
            c += (i == 0 || !key_same_point(src[i - 1], src[i])) ? 1u : 0u;
        c = warp_sum(c);
        __syncthreads();
        if (lane == 0) wsum[w] = c;
        __syncthreads();
        if (threadIdx.x == 0) {
            unsigned tot = 0;
            for (int k = 0; k < kSortThreads / 32; ++k) tot += wsum[k];
            tile_cnt[t] = tot;
        }
    }
    sort_cluster_barrier();
    // ordered compaction: tile base = exclusive prefix of the tile counts
    for (long t = rank; t < tiles; t += ncta) {
        __syncthreads();
        if (threadIdx.x == 0) {
            unsigned b = 0;
            for (long k = 0; k < t; ++k) b += __ldcg(tile_cnt + k);
            s_base = b;
        }
        __syncthreads();
        // one element per thread per round, kSortTile / kSortThreads rounds, in index order
        unsigned run = s_base;
        for (long r0 = t * kSortTile; r0 < min(n, (t + 1) * kSortTile); r0 += blockDim.x) {
            const long i = r0 + threadIdx.x;
            const bool keep = i < n && (i == 0 || !key_same_point(src[i - 1], src[i]));
            const unsigned bal = __ballot_sync(0xffffffffu, keep);
            __syncthreads();
            if (lane == 0) wsum[w] = __popc(bal);
            __syncthreads();
            unsigned before = 0, all = 0;
            for (int k = 0; k < kSortThreads / 32; ++k) {
                const unsigned v = wsum[k];
                if (k < w) before += v;
                all += v;
            }
            if (keep) {
                const unsigned pos = run + before + __popc(bal & ((1u << lane) - 1));
                const Key3 k = src[i];
                float* o = pts + 3 * (long)pos;
                o[0] = key2f(k.k[0]);
                o[1] = key2f(k.k[1]);
                o[2] = key2f(k.k[2]);
            }
            run += all;
        }
    }
    sort_cluster_barrier();
    if (rank == 0 && threadIdx.x == 0 && n > 0) {
        unsigned tot = 0;
        for (long k = 0; k < tiles; ++k) tot += __ldcg(tile_cnt + k);
        *count = tot;
    }
}

static size_t al(size_t x) { return (x + 255) & ~(size_t)255; }

size_t sort_unique_workspace_size(long n_max) {
    if (n_max < 1) n_max = 1;
    return 2 * al(n_max * sizeof(Key3)) + al(((n_max + kSortTile - 1) / kSortTile) * 4) + 256;
}

static int sort_cluster_size() {
    static ContextOnce once;
    static int cached_dev[kMaxDevices];
    once_per_context(once, [](int dev) {
        int cached = 0;
        cudaFuncSetAttribute(sort_unique_kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        const int sizes[2] = {kSortCluster, 8};
        for (int c : sizes) {
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = dim3(c);
            cfg.blockDim = dim3(kSortThreads);
            cudaLaunchAttribute at[1];
            at[0].id = cudaLaunchAttributeClusterDimension;
            at[0].val.clusterDim.x = c;
            at[0].val.clusterDim.y = 1;
            at[0].val.clusterDim.z = 1;
            cfg.attrs = at;
            cfg.numAttrs = 1;
            int clusters = 0;
            if (cudaOccupancyMaxActiveClusters(&clusters, sort_unique_kernel, &cfg) == cudaSuccess && clusters > 0) {
                cached = c;
                break;
            }
            cudaGetLastError();
        }
        cached_dev[dev] = cached ? cached : 8;
        return (int)AFX_OK;
    });
    int dev = 0;
    cudaGetDevice(&dev);
    return cached_dev[dev] ? cached_dev[dev] : 8;
}

static int sort_unique_cluster(float* pts, unsigned* count, long n_max, void* ws, size_t ws_bytes, cudaStream_t st,
                               const unsigned* only_if);

int sort_unique_impl(float* pts, unsigned* count, long n_max, void* ws, size_t ws_bytes, cudaStream_t st) {
    return sort_unique_cluster(pts, count, n_max, ws, ws_bytes, st, nullptr);
}

static int sort_unique_cluster(float* pts, unsigned* count, long n_max, void* ws, size_t ws_bytes, cudaStream_t st,
                               const unsigned* only_if) {
    if (n_max <= 0) return AFX_OK;
    if (!ws || ws_bytes < sort_unique_workspace_size(n_max)) return AFX_ERR_WORKSPACE;
    char* p = static_cast<char*>(ws);
    Key3* buf0 = reinterpret_cast<Key3*>(p);
    p += al(n_max * sizeof(Key3));
    Key3* buf1 = reinterpret_cast<Key3*>(p);
    p += al(n_max * sizeof(Key3));
    unsigned* tile_cnt = reinterpret_cast<unsigned*>(p);
    const int c = sort_cluster_size();
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(c);
    cfg.blockDim = dim3(kSortThreads);
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = c;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    AFX_CUDA(cudaLaunchKernelEx(&cfg, sort_unique_kernel, pts, count, n_max, buf0, buf1, tile_cnt, only_if));
    AFX_LAUNCH_CHECK();
    return AFX_OK;
}

// ------------------------------------------------------------------------------------
// Column-bucket sort + unique of a marching-cubes point cloud of a known volume.
//
// Every point of the cloud has x in [-half, half] of the volume, and b(x) = trunc((x + half) * inv)
// (clamped) is monotone in x under IEEE rounding, so bucketing by voxel column keeps the
// lexicographic order between buckets and puts equal points (-0 and +0 included) in one bucket.
// Pipeline: count per bucket, scan, scatter (order within a bucket arbitrary), one CTA per bucket
// sorting it in shared memory and counting its unique points, scan of those counts, ordered
// compaction back into the cloud.  A bucket larger than kBucketCap (a surface lying along one x
// column) is sorted by its CTA in runs of kBucketCap in shared memory that are then merged pairwise
// in global memory (merge path, ties from the left run first) between the key buffer and the second
// buffer of the workspace, so one crowded column no longer sends the whole cloud to the cluster sort.
// ------------------------------------------------------------------------------------

constexpr int kBucketCap = 8192;  // keys per bucket sorted in shared memory (96 KB)
constexpr int kBucketThreads = 512;

struct BucketArgs {
    float half0, inv0;
    int nb;
};

AFX_D int bucket_of(float x, const BucketArgs& a) {
    const float u = (x + a.half0) * a.inv0;
    const int b = u > 0.f ? f2i(u) : 0;
    return b >= a.nb ? a.nb - 1 : b;
}

struct BucketWs {
    unsigned* cnt;     // [nb]
    unsigned* off;     // [nb + 1]
    unsigned* cursor;  // [nb]
    unsigned* ucnt;    // [nb]
    unsigned* uoff;    // [nb + 1]
    unsigned* overflow;
};

__global__ void bucket_count_kernel(const float* __restrict__ pts, const unsigned* count, long n_max, BucketArgs a,
                                    unsigned* cnt) {
    const long n = min((long)*count, n_max);
    AFX_GRID_STRIDE(i, n) atomicAdd(cnt + bucket_of(pts[3 * i], a), 1u);
}

// Exclusive scan of n values by one CTA of 1024 threads (n up to a few thousand); out[n] = total.
// With `overflow`, flags it when a value exceeds `cap`; with `total`, also writes the total there
// unless *skip is set.
__global__ void __launch_bounds__(1024) small_scan_kernel(const unsigned* in, int n, unsigned* out, unsigned* copy,
                                                          unsigned cap, unsigned* overflow, unsigned* total,
                                                          const unsigned* skip) {
    __shared__ unsigned part[1024];
    const int per = (n + 1023) / 1024;
    const int lo = threadIdx.x * per, hi = min(n, lo + per);
    unsigned sum = 0, big = 0;
    for (int i = lo; i < hi; ++i) {
        sum += in[i];
        big |= in[i] > cap;
    }
    if (overflow && __syncthreads_or(big) && threadIdx.x == 0) *overflow = 1u;
    part[threadIdx.x] = sum;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
        const unsigned v = threadIdx.x >= o ? part[threadIdx.x - o] : 0u;
        __syncthreads();
        part[threadIdx.x] += v;
        __syncthreads();
    }
    unsigned run = part[threadIdx.x] - sum;
    for (int i = lo; i < hi; ++i) {
        out[i] = run;
        if (copy) copy[i] = run;
        run += in[i];
    }
    if (threadIdx.x == 1023) {
        out[n] = part[1023];
        if (total && !(skip && *skip)) *total = part[1023];
    }
}

__global__ void bucket_scatter_kernel(const float* __restrict__ pts, const unsigned* count, long n_max, BucketArgs a,
                                      unsigned* cursor, Key3* keys, const unsigned* overflow, int* error) {
    if (*overflow) return;
    const long n = min((long)*count, n_max);
    AFX_GRID_STRIDE(i, n) {
        Key3 k;
        k.k[0] = f2key(pts[3 * i]);
        k.k[1] = f2key(pts[3 * i + 1]);
        k.k[2] = f2key(pts[3 * i + 2]);
        const unsigned pos = atomicAdd(cursor + bucket_of(pts[3 * i], a), 1u);
        if (pos < (unsigned long)n) keys[pos] = k;
        else if (error) atomicOr(error, ERRF_INDEX);
    }
}

// Bitonic sort of m <= kBucketCap keys at g in shared memory (padded to a power of two with keys that
// sort last), written back to g.
AFX_D void bucket_bitonic(Key3* g, unsigned m, Key3* sk) {
    unsigned P = 1;
    while (P < m) P <<= 1;
    __syncthreads();
    for (unsigned i = threadIdx.x; i < P; i += blockDim.x) {
        Key3 k;
        if (i < m) k = g[i];
        else k.k[0] = k.k[1] = k.k[2] = 0xffffffffu;
        sk[i] = k;
    }
    __syncthreads();
    for (unsigned size = 2; size <= P; size <<= 1)
        for (unsigned stride = size >> 1; stride > 0; stride >>= 1) {
            for (unsigned q = threadIdx.x; q < P / 2; q += blockDim.x) {
                const unsigned i = 2 * stride * (q / stride) + (q % stride), j = i + stride;
                const bool asc = (i & size) == 0;
                const Key3 x = sk[i], y = sk[j];
                if (key_less(y, x) == asc) {
                    sk[i] = y;
                    sk[j] = x;
                }
            }
            __syncthreads();
        }
    for (unsigned i = threadIdx.x; i < m; i += blockDim.x) g[i] = sk[i];
    __syncthreads();
}

// Stable merge of the sorted runs A[0, la) and B[0, lb) into out by the whole CTA: each thread finds
// where its share of the output starts on the merge path (binary search: the first i with
// B[k - i - 1] < A[i]) and merges its share sequentially.
AFX_D void cta_merge(const Key3* A, unsigned la, const Key3* B, unsigned lb, Key3* out) {
    const unsigned total = la + lb, per = (total + blockDim.x - 1) / blockDim.x;
    const unsigned k0 = min(total, threadIdx.x * per), k1 = min(total, k0 + per);
    if (k0 >= k1) return;
    unsigned lo = k0 > lb ? k0 - lb : 0u, hi = min(k0, la);
    while (lo < hi) {
        const unsigned mid = (lo + hi) >> 1;
        if (key_less(B[k0 - mid - 1], A[mid])) hi = mid;
        else lo = mid + 1;
    }
    unsigned i = lo, j = k0 - lo;
    for (unsigned k = k0; k < k1; ++k) {
        const bool takeA = i < la && (j >= lb || !key_less(B[j], A[i]));
        out[k] = takeA ? A[i++] : B[j++];
    }
}

// One CTA per bucket: sort it in place (in shared memory, or in runs merged through `scratch` when it
// holds more than kBucketCap points) and count its unique points.
__global__ void __launch_bounds__(kBucketThreads) bucket_sort_kernel(Key3* keys, Key3* scratch, const unsigned* off,
                                                                   unsigned* ucnt, const unsigned* overflow, long n_max,
                                                                   int* error) {
    extern __shared__ Key3 sk[];
    __shared__ unsigned wsum[kBucketThreads / 32];
    if (*overflow) return;
    const int b = blockIdx.x;
    const unsigned lo = off[b], n = off[b + 1] - lo;
    if (lo > off[b + 1] || (long)off[b + 1] > n_max) {  // never expected: skip, flag
        if (threadIdx.x == 0) {
            ucnt[b] = 0;
            if (error) atomicOr(error, ERRF_INDEX);
        }
        return;
    }
    if (n == 0) {
        if (threadIdx.x == 0) ucnt[b] = 0;
        return;
    }
    Key3* g = keys + lo;
    if (n <= (unsigned)kBucketCap) {
        bucket_bitonic(g, n, sk);
    } else {
        for (unsigned c0 = 0; c0 < n; c0 += kBucketCap) bucket_bitonic(g + c0, min((unsigned)kBucketCap, n - c0), sk);
        Key3 *src = g, *dst = scratch + lo;
        for (unsigned L = kBucketCap; L < n; L *= 2) {
            for (unsigned s0 = 0; s0 < n; s0 += 2 * L) {
                const unsigned la = min(L, n - s0), lb = min(L, n - s0 - la);
                cta_merge(src + s0, la, src + s0 + la, lb, dst + s0);
            }
            __syncthreads();
            Key3* t = src;
            src = dst;
            dst = t;
        }
        if (src != g) {
            for (unsigned i = threadIdx.x; i < n; i += blockDim.x) g[i] = src[i];
            __syncthreads();
        }
    }
    unsigned c = 0;
    for (unsigned i = threadIdx.x; i < n; i += blockDim.x) c += (i == 0 || !key_same_point(g[i - 1], g[i])) ? 1u : 0u;
    c = warp_sum(c);
    if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned t = 0;
        for (int w = 0; w < kBucketThreads / 32; ++w) t += wsum[w];
        ucnt[b] = t;
    }
}

// One CTA per bucket: its unique points, in order, at the bucket's place in the output.
__global__ void __launch_bounds__(kBucketThreads) bucket_compact_kernel(const Key3* keys, const unsigned* off,
                                                                      const unsigned* uoff, float* pts, long n_max,
                                                                      const unsigned* overflow, int* error) {
    __shared__ unsigned wsum[kBucketThreads / 32];
    if (*overflow) return;
    const int b = blockIdx.x;
    if (off[b] > off[b + 1] || (long)off[b + 1] > n_max || (long)uoff[b + 1] > n_max) {
        if (threadIdx.x == 0 && error) atomicOr(error, ERRF_INDEX);
        return;
    }
    const unsigned lo = off[b], n = off[b + 1] - lo;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    unsigned run = uoff[b];
    for (unsigned r0 = 0; r0 < n; r0 += blockDim.x) {
        const unsigned i = r0 + threadIdx.x;
        const bool keep = i < n && (i == 0 || !key_same_point(keys[lo + i - 1], keys[lo + i]));
        const unsigned bal = __ballot_sync(0xffffffffu, keep);
        __syncthreads();
        if (lane == 0) wsum[w] = __popc(bal);
        __syncthreads();
        unsigned before = 0, all = 0;
        for (int k = 0; k < kBucketThreads / 32; ++k) {
            const unsigned v = wsum[k];
            if (k < w) before += v;
            all += v;
        }
        if (keep) {
            const Key3 k = keys[lo + i];
            float* o = pts + 3 * (long)(run + before + __popc(bal & ((1u << lane) - 1)));
            o[0] = key2f(k.k[0]);
            o[1] = key2f(k.k[1]);
            o[2] = key2f(k.k[2]);
        }
        run += all;
    }
}

size_t sort_unique_volume_workspace_size(long n_max, int nb) {
    return sort_unique_workspace_size(n_max) + al((size_t)(5 * (nb + 2) + 1) * 4);
}

int sort_unique_volume_impl(float* pts, unsigned* count, long n_max, void* ws, size_t ws_bytes, const Volume& vol,
                            cudaStream_t st, int* error) {
    if (n_max <= 0) return AFX_OK;
    const int nb = vol.dims[0] + 1;
    if (nb > 8 * 1024) return sort_unique_impl(pts, count, n_max, ws, ws_bytes, st);
    if (!ws || ws_bytes < sort_unique_volume_workspace_size(n_max, nb)) return AFX_ERR_WORKSPACE;
    const size_t base = sort_unique_workspace_size(n_max);
    unsigned* u = reinterpret_cast<unsigned*>(static_cast<char*>(ws) + base);
    BucketWs w{u, u + nb, u + 2 * nb + 1, u + 3 * nb + 1, u + 4 * nb + 1, u + 5 * nb + 2};
    Key3* keys = reinterpret_cast<Key3*>(ws);  // the cluster sort's first buffer (it rebuilds it from the cloud)
    BucketArgs a{vol.half[0], vol.inv[0], nb};
    static ContextOnce once;
    once_per_context(once, [](int) {
        return note_cuda_error(cudaFuncSetAttribute(bucket_sort_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                    (int)(kBucketCap * sizeof(Key3))));
    });
    AFX_CUDA(cudaMemsetAsync(w.cnt, 0, nb * 4, st));
    AFX_CUDA(cudaMemsetAsync(w.overflow, 0, 4, st));
    bucket_count_kernel<<<grid_for(n_max, 256), 256, 0, st>>>(pts, count, n_max, a, w.cnt);
    small_scan_kernel<<<1, 1024, 0, st>>>(w.cnt, nb, w.off, w.cursor, 0xffffffffu, nullptr, nullptr, nullptr);
    bucket_scatter_kernel<<<grid_for(n_max, 256), 256, 0, st>>>(pts, count, n_max, a, w.cursor, keys, w.overflow,
                                                                 error);
    Key3* scratch = reinterpret_cast<Key3*>(static_cast<char*>(ws) + al(n_max * sizeof(Key3)));  // the second buffer
    bucket_sort_kernel<<<nb, kBucketThreads, kBucketCap * sizeof(Key3), st>>>(keys, scratch, w.off, w.ucnt, w.overflow,
                                                                              n_max, error);
    small_scan_kernel<<<1, 1024, 0, st>>>(w.ucnt, nb, w.uoff, nullptr, 0xffffffffu, nullptr, count, w.overflow);
    bucket_compact_kernel<<<nb, kBucketThreads, 0, st>>>(keys, w.off, w.uoff, pts, n_max, w.overflow, error);
    AFX_LAUNCH_CHECK();
    return sort_unique_cluster(pts, count, n_max, ws, ws_bytes, st, w.overflow);
}

__global__ void translate_kernel(float* pts, const unsigned* count, long n_max, float tx, float ty, float tz) {
    long n = count ? min((long)*count, n_max) : n_max;
    long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    pts[3 * i] = pts[3 * i] + tx;
    pts[3 * i + 1] = pts[3 * i + 1] + ty;
    pts[3 * i + 2] = pts[3 * i + 2] + tz;
}

__global__ void translate_dev_kernel(float* dst, const float* src, const unsigned* count, long n_max, const float* t,
                                     float sign) {
    const long n = count ? min((long)*count, n_max) : n_max;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        for (int c = 0; c < 3; ++c) dst[3 * i + c] = src[3 * i + c] + sign * t[c];
}

int translate_dev_impl(float* dst, const float* src, const unsigned* count, long n_max, const float* t_dev, float sign,
                       cudaStream_t st) {
    if (n_max <= 0) return AFX_OK;
    translate_dev_kernel<<<grid_for(n_max, 256), 256, 0, st>>>(dst, src, count, n_max, t_dev, sign);
    AFX_LAUNCH_CHECK();
    return AFX_OK;
}

int translate_impl(float* pts, const unsigned* count, long n_max, const float* t, cudaStream_t st) {
    if (n_max <= 0) return AFX_OK;
    translate_kernel<<<blocks_for(n_max, 256), 256, 0, st>>>(pts, count, n_max, t[0], t[1], t[2]);
    AFX_LAUNCH_CHECK();
    return AFX_OK;
}

}  // namespace afx

using namespace afx;

extern "C" {

int afx_marching_cubes_points(float* points, unsigned* count, long capacity, const float* tsdf, const float* weights,
                              const int dims[3], const float voxel_size[3], const float volume_size[3], float iso,
                              void* stream) {
    if (!points || !count || !tsdf || !weights || !dims || capacity < 0) return AFX_ERR_INVALID_ARGUMENT;
    return mc_fused_impl(tsdf, weights, kVoxF32, make_volume(dims, voxel_size, volume_size), iso, points, count, capacity,
                         nullptr, nullptr, 0, nullptr, nullptr, 0, as_stream(stream));
}

int afx_marching_cubes_mesh(float* vertices, unsigned* vertex_count, long vertex_capacity, int* faces,
                            unsigned* face_count, long face_capacity, const float* tsdf, const float* weights,
                            const int dims[3], const float voxel_size[3], const float volume_size[3], float iso,
                            void* stream) {
    if (!vertices || !vertex_count || !faces || !face_count || !tsdf || !weights || !dims)
        return AFX_ERR_INVALID_ARGUMENT;
    return mc_fused_impl(tsdf, weights, kVoxF32, make_volume(dims, voxel_size, volume_size), iso, nullptr, nullptr, 0, vertices,
                         vertex_count, vertex_capacity, faces, face_count, face_capacity, as_stream(stream));
}

size_t afx_sort_unique_points_workspace_size(long n_max) { return sort_unique_workspace_size(n_max); }

int afx_sort_unique_points(float* points, unsigned* count, long n_max, void* workspace, size_t workspace_bytes,
                           void* stream) {
    if (!points || !count || n_max < 0) return AFX_ERR_INVALID_ARGUMENT;
    return sort_unique_impl(points, count, n_max, workspace, workspace_bytes, as_stream(stream));
}

size_t afx_sort_unique_volume_points_workspace_size(long n_max, const int dims[3]) {
    if (!dims || dims[0] < 1) return 0;
    return sort_unique_volume_workspace_size(n_max < 1 ? 1 : n_max, dims[0] + 1);
}

int afx_sort_unique_volume_points(float* points, unsigned* count, long n_max, const int dims[3],
                                  const float voxel_size[3], const float volume_size[3], void* workspace,
                                  size_t workspace_bytes, void* stream) {
    if (!points || !count || n_max < 0 || !dims || !voxel_size || !volume_size || dims[0] < 1)
        return AFX_ERR_INVALID_ARGUMENT;
    return sort_unique_volume_impl(points, count, n_max, workspace, workspace_bytes,
                                   make_volume(dims, voxel_size, volume_size), as_stream(stream), nullptr);
}

int afx_extract_point_cloud(float* points, unsigned* count, long capacity, const float* tsdf, const float* weights,
                            const int dims[3], const float voxel_size[3], const float volume_size[3], float iso,
                            void* workspace, size_t workspace_bytes, void* stream) {
    if (!points || !count || !tsdf || !weights || !dims) return AFX_ERR_INVALID_ARGUMENT;
    cudaStream_t st = as_stream(stream);
    AFX_CUDA(cudaMemsetAsync(count, 0, sizeof(unsigned), st));
    int rc = mc_fused_impl(tsdf, weights, kVoxF32, make_volume(dims, voxel_size, volume_size), iso, points, count, capacity,
                           nullptr, nullptr, 0, nullptr, nullptr, 0, st);
    if (rc) return rc;
    return sort_unique_impl(points, count, capacity, workspace, workspace_bytes, st);
}

int afx_translate(float* points, const unsigned* count, long n_max, const float t[3], void* stream) {
    if (!points || !t || n_max < 0) return AFX_ERR_INVALID_ARGUMENT;
    return translate_impl(points, count, n_max, t, as_stream(stream));
}

}  // extern "C"
