// afx_mc.cu -- marching cubes (point-cloud and triangle variants, fused into one pass over
// the volume) with warp-aggregated stream compaction, and the lexicographic sort +
// unique of the canonical point cloud (a merge sort: bitonic 2048-element tiles in
// shared memory, then merge-path passes).
//
// Case index, edge interpolation and triangulation follow src/MarchingCubes.cu:294-420
// (corner bit c set when tsdf > iso, cubes skipped when any corner weight is 0, cubes
// x,y,z < dim-2).  The triangulation table is the reference's (packed re-encoding).
#include <cstring>

#include "afx_internal.h"

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

static int upload_tables() {
    static bool done = false;  // tables are constant; one upload per process and device 0 context
    static int dev_done = -1;
    int dev = 0;
    cudaGetDevice(&dev);
    if (done && dev_done == dev) return AFX_OK;
    unsigned short et[256];
    for (int c = 0; c < 256; ++c) {
        int e = 0;
        for (int i = 0; i < 12; ++i)
            if (((c >> kEdgeHost[i][0]) & 1) != ((c >> kEdgeHost[i][1]) & 1)) e |= 1 << i;
        et[c] = (unsigned short)e;
    }
    AFX_CUDA(cudaMemcpyToSymbol(c_edge_table, et, sizeof(et)));
    AFX_CUDA(cudaMemcpyToSymbol(c_tri_table, kTriTableHost, sizeof(kTriTableHost)));
    done = true;
    dev_done = dev;
    return AFX_OK;
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
};

// getVertex + interpolate (src/MarchingCubes.cu:294-336)
AFX_D void edge_vertex(const float* __restrict__ tsdf, const Volume& vol, int x, int y, int z, int e, float iso,
                       float* o) {
    const int* ca = c_corner[c_edge[e][0]];
    const int* cb = c_corner[c_edge[e][1]];
    const int X = vol.dims[0], Y = vol.dims[1];
    int x1 = x + ca[0], y1 = y + ca[1], z1 = z + ca[2];
    int x2 = x + cb[0], y2 = y + cb[1], z2 = z + cb[2];
    float t0 = __ldg(tsdf + ((long)z1 * Y + y1) * X + x1);
    float t1 = __ldg(tsdf + ((long)z2 * Y + y2) * X + x2);
    float p0[3], p1[3];
    voxel_to_world(x1, y1, z1, vol.vs, vol.half, p0);
    voxel_to_world(x2, y2, z2, vol.vs, vol.half, p1);
    if ((double)fabsf(iso - t0) < 1e-7) {
        o[0] = p0[0]; o[1] = p0[1]; o[2] = p0[2];
        return;
    }
    if ((double)fabsf(iso - t1) < 1e-7) {
        o[0] = p1[0]; o[1] = p1[1]; o[2] = p1[2];
        return;
    }
    if ((double)fabsf(t0 - t1) < 1e-7) {
        o[0] = p0[0]; o[1] = p0[1]; o[2] = p0[2];
        return;
    }
    double mu = (double)((iso - t0) / (t1 - t0));
    if (mu > 1.0) mu = 1.0;
    else if (mu < 0) mu = 0.0;
#pragma unroll
    for (int c = 0; c < 3; ++c) o[c] = (float)__dadd_rn((double)p0[c], __dmul_rn(mu, (double)(p1[c] - p0[c])));
}

AFX_D int cube_index(const float* __restrict__ tsdf, const float* __restrict__ w, const Volume& vol, int x, int y,
                     int z, float iso) {
    const int X = vol.dims[0], Y = vol.dims[1];
    long off[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) off[c] = ((long)(z + c_corner[c][2]) * Y + (y + c_corner[c][1])) * X + x + c_corner[c][0];
    bool any_zero = false;
#pragma unroll
    for (int c = 0; c < 8; ++c) any_zero |= (__ldg(w + off[c]) == 0.0f);
    if (any_zero) return 0;
    int idx = 0;
#pragma unroll
    for (int c = 0; c < 8; ++c)
        if (__ldg(tsdf + off[c]) > iso) idx |= 1 << c;
    return idx;
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

// One thread per cube, x fastest.  Emits the point-cloud vertices (marchingCubesMeshKernel)
// and/or the triangles (marchingCubesFullKernel) of its cube.
template <bool kPoints, bool kMesh>
__global__ void __launch_bounds__(256) mc_kernel(const float* __restrict__ tsdf, const float* __restrict__ weights,
                                                 McArgs a) {
    const int nx = a.vol.dims[0] - 2, ny = a.vol.dims[1] - 2, nz = a.vol.dims[2] - 2;
    const long ncubes = (long)nx * ny * nz;
    const long stride = (long)gridDim.x * blockDim.x;
    const long start = blockIdx.x * (long)blockDim.x + threadIdx.x;
    // all lanes of a warp iterate together so the warp-level append stays converged
    for (long base = start - (threadIdx.x & 31); base < ncubes; base += stride) {
        long cid = base + (threadIdx.x & 31);
        int ci = 0, x = 0, y = 0, z = 0;
        if (cid < ncubes) {
            x = (int)(cid % nx);
            y = (int)((cid / nx) % ny);
            z = (int)(cid / ((long)nx * ny));
            ci = cube_index(tsdf, weights, a.vol, x, y, z, a.iso);
        }
        const bool active = ci != 0 && ci != 255;
        if (!__any_sync(0xffffffffu, active)) continue;
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
}

__global__ void mc_vert_count_kernel(const unsigned* face_count, unsigned* vert_count) {
    *vert_count = 3u * *face_count;
}

int mc_fused_impl(const float* tsdf, const float* weights, const Volume& vol, float iso, float* points,
                  unsigned* point_count, long point_cap, float* verts, unsigned* vert_count, long vert_cap, int* faces,
                  unsigned* face_count, long face_cap, cudaStream_t st) {
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
    const long ncubes = (long)(vol.dims[0] - 2) * (vol.dims[1] - 2) * (vol.dims[2] - 2);
    if (ncubes <= 0) return AFX_OK;
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    long want = (ncubes + 255) / 256;
    unsigned grid = (unsigned)(want < (long)sms * 16 ? want : (long)sms * 16);
    const bool P = points != nullptr, M = verts != nullptr;
    if (P && M) mc_kernel<true, true><<<grid, 256, 0, st>>>(tsdf, weights, a);
    else if (P) mc_kernel<true, false><<<grid, 256, 0, st>>>(tsdf, weights, a);
    else if (M) mc_kernel<false, true><<<grid, 256, 0, st>>>(tsdf, weights, a);
    else return AFX_OK;
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

__device__ __forceinline__ long dev_n(const unsigned* count, long n_max) { return min((long)*count, n_max); }

__global__ void __launch_bounds__(1024) sort_tiles_kernel(const float* __restrict__ pts, Key3* out,
                                                          const unsigned* count, long n_max) {
    __shared__ Key3 s[kSortTile];
    const long n = dev_n(count, n_max);
    const long base = (long)blockIdx.x * kSortTile;
    if (base >= n) return;
    for (int i = threadIdx.x; i < kSortTile; i += blockDim.x) {
        long j = base + i;
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
    for (int size = 2; size <= kSortTile; size <<= 1) {
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            int p = threadIdx.x;  // one pair per thread (1024 pairs)
            int i = 2 * stride * (p / stride) + (p % stride);
            int j = i + stride;
            bool asc = (i & size) == 0;
            Key3 a = s[i], b = s[j];
            if (key_less(b, a) == asc) {
                s[i] = b;
                s[j] = a;
            }
            __syncthreads();
        }
    }
    for (int i = threadIdx.x; i < kSortTile; i += blockDim.x) {
        long j = base + i;
        if (j < n) out[j] = s[i];
    }
}

// One merge pass: runs of length L in `in` merged pairwise into `out`.  Each CTA produces
// kSortTile outputs; a pass with L >= n leaves the data where it is (flag in *state).
__global__ void __launch_bounds__(512) merge_pass_kernel(const Key3* __restrict__ in, Key3* __restrict__ out,
                                                         const unsigned* count, long n_max, long L) {
    __shared__ Key3 s[kSortTile];
    const long n = dev_n(count, n_max);
    if (L >= n) return;
    const long o0 = (long)blockIdx.x * kSortTile;
    if (o0 >= n) return;
    const long pair = o0 / (2 * L) * (2 * L);
    const long a0 = pair, na = min(L, n - a0);
    const long b0 = pair + L, nb = max(0L, min(L, n - b0));
    const long d0 = o0 - pair, d1 = min(d0 + kSortTile, na + nb);
    __shared__ long split[2];
    if (threadIdx.x < 2) {
        long d = threadIdx.x == 0 ? d0 : d1;
        long lo = max(0L, d - nb), hi = min(d, na);
        while (lo < hi) {
            long mid = (lo + hi) >> 1;
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
    // each thread merges 4 consecutive outputs of the tile
    const int tot = la + lb;
    const int q0 = threadIdx.x * 4;
    if (q0 >= tot) return;
    int lo = max(0, q0 - lb), hi = min(q0, la);
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (key_le(s[mid], s[la + q0 - 1 - mid])) lo = mid + 1;
        else hi = mid;
    }
    int ia = lo, ib = q0 - lo;
    for (int q = q0; q < q0 + 4 && q < tot; ++q) {
        bool takeA = ib >= lb || (ia < la && key_le(s[ia], s[la + ib]));
        out[o0 + q] = takeA ? s[ia++] : s[la + ib++];
    }
}

__global__ void unique_flags_kernel(const Key3* buf0, const Key3* buf1, const unsigned* count, long n_max, int passes,
                                    unsigned* flags) {
    const long n = dev_n(count, n_max);
    // the sorted data is in buf0 after an even number of effective passes, else in buf1
    int eff = 0;
    for (long L = kSortTile; L < n && eff < passes; L <<= 1) ++eff;
    const Key3* buf = (eff & 1) ? buf1 : buf0;
    long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    unsigned f = 1;
    if (i > 0) {
        Key3 a = buf[i - 1], b = buf[i];
        float ax = key2f(a.k[0]), ay = key2f(a.k[1]), az = key2f(a.k[2]);
        float bx = key2f(b.k[0]), by = key2f(b.k[1]), bz = key2f(b.k[2]);
        f = (ax == bx && ay == by && az == bz) ? 0u : 1u;
    }
    flags[i] = f;
}

__global__ void unique_scatter_kernel(const Key3* buf0, const Key3* buf1, unsigned* count, long n_max, int passes,
                                      const unsigned* flags, const unsigned* pos, const unsigned* total, float* pts) {
    const long n = dev_n(count, n_max);
    int eff = 0;
    for (long L = kSortTile; L < n && eff < passes; L <<= 1) ++eff;
    const Key3* buf = (eff & 1) ? buf1 : buf0;
    long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (i < n && flags[i]) {
        Key3 k = buf[i];
        float* o = pts + 3 * (long)pos[i];
        o[0] = key2f(k.k[0]);
        o[1] = key2f(k.k[1]);
        o[2] = key2f(k.k[2]);
    }
}

__global__ void set_count_kernel(unsigned* count, const unsigned* total, long n_max) {
    if (min((long)*count, n_max) > 0) *count = *total;
}

static size_t al(size_t x) { return (x + 255) & ~(size_t)255; }

size_t sort_unique_workspace_size(long n_max) {
    if (n_max < 1) n_max = 1;
    return 2 * al(n_max * sizeof(Key3)) + 2 * al(n_max * 4) + al(scan_workspace_size(n_max)) + 256;
}

int sort_unique_impl(float* pts, unsigned* count, long n_max, void* ws, size_t ws_bytes, cudaStream_t st) {
    if (n_max <= 0) return AFX_OK;
    if (!ws || ws_bytes < sort_unique_workspace_size(n_max)) return AFX_ERR_WORKSPACE;
    char* p = static_cast<char*>(ws);
    Key3* buf0 = reinterpret_cast<Key3*>(p);
    p += al(n_max * sizeof(Key3));
    Key3* buf1 = reinterpret_cast<Key3*>(p);
    p += al(n_max * sizeof(Key3));
    unsigned* flags = reinterpret_cast<unsigned*>(p);
    p += al(n_max * 4);
    unsigned* pos = reinterpret_cast<unsigned*>(p);
    p += al(n_max * 4);
    void* scan_ws = p;
    p += al(scan_workspace_size(n_max));
    unsigned* total = reinterpret_cast<unsigned*>(p);
    const long tiles = (n_max + kSortTile - 1) / kSortTile;
    sort_tiles_kernel<<<(unsigned)tiles, 1024, 0, st>>>(pts, buf0, count, n_max);
    AFX_LAUNCH_CHECK();
    int passes = 0;
    Key3* src = buf0;
    Key3* dst = buf1;
    for (long L = kSortTile; L < n_max; L <<= 1, ++passes) {
        merge_pass_kernel<<<(unsigned)tiles, 512, 0, st>>>(src, dst, count, n_max, L);
        AFX_LAUNCH_CHECK();
        Key3* t = src;
        src = dst;
        dst = t;
    }
    unique_flags_kernel<<<blocks_for(n_max, 256), 256, 0, st>>>(buf0, buf1, count, n_max, passes, flags);
    AFX_LAUNCH_CHECK();
    int rc = scan_exclusive_dev(flags, pos, count, n_max, total, scan_ws, st);
    if (rc) return rc;
    unique_scatter_kernel<<<blocks_for(n_max, 256), 256, 0, st>>>(buf0, buf1, count, n_max, passes, flags, pos, total,
                                                                  pts);
    AFX_LAUNCH_CHECK();
    set_count_kernel<<<1, 1, 0, st>>>(count, total, n_max);
    AFX_LAUNCH_CHECK();
    return AFX_OK;
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
    long n = count ? min((long)*count, n_max) : n_max;
    long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (int c = 0; c < 3; ++c) dst[3 * i + c] = src[3 * i + c] + sign * t[c];
}

int translate_dev_impl(float* dst, const float* src, const unsigned* count, long n_max, const float* t_dev, float sign,
                       cudaStream_t st) {
    if (n_max <= 0) return AFX_OK;
    translate_dev_kernel<<<blocks_for(n_max, 256), 256, 0, st>>>(dst, src, count, n_max, t_dev, sign);
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
    return mc_fused_impl(tsdf, weights, make_volume(dims, voxel_size, volume_size), iso, points, count, capacity,
                         nullptr, nullptr, 0, nullptr, nullptr, 0, as_stream(stream));
}

int afx_marching_cubes_mesh(float* vertices, unsigned* vertex_count, long vertex_capacity, int* faces,
                            unsigned* face_count, long face_capacity, const float* tsdf, const float* weights,
                            const int dims[3], const float voxel_size[3], const float volume_size[3], float iso,
                            void* stream) {
    if (!vertices || !vertex_count || !faces || !face_count || !tsdf || !weights || !dims)
        return AFX_ERR_INVALID_ARGUMENT;
    return mc_fused_impl(tsdf, weights, make_volume(dims, voxel_size, volume_size), iso, nullptr, nullptr, 0, vertices,
                         vertex_count, vertex_capacity, faces, face_count, face_capacity, as_stream(stream));
}

size_t afx_sort_unique_points_workspace_size(long n_max) { return sort_unique_workspace_size(n_max); }

int afx_sort_unique_points(float* points, unsigned* count, long n_max, void* workspace, size_t workspace_bytes,
                           void* stream) {
    if (!points || !count || n_max < 0) return AFX_ERR_INVALID_ARGUMENT;
    return sort_unique_impl(points, count, n_max, workspace, workspace_bytes, as_stream(stream));
}

int afx_extract_point_cloud(float* points, unsigned* count, long capacity, const float* tsdf, const float* weights,
                            const int dims[3], const float voxel_size[3], const float volume_size[3], float iso,
                            void* workspace, size_t workspace_bytes, void* stream) {
    if (!points || !count || !tsdf || !weights || !dims) return AFX_ERR_INVALID_ARGUMENT;
    cudaStream_t st = as_stream(stream);
    AFX_CUDA(cudaMemsetAsync(count, 0, sizeof(unsigned), st));
    int rc = mc_fused_impl(tsdf, weights, make_volume(dims, voxel_size, volume_size), iso, points, count, capacity,
                           nullptr, nullptr, 0, nullptr, nullptr, 0, st);
    if (rc) return rc;
    return sort_unique_impl(points, count, capacity, workspace, workspace_bytes, st);
}

int afx_translate(float* points, const unsigned* count, long n_max, const float t[3], void* stream) {
    if (!points || !t || n_max < 0) return AFX_ERR_INVALID_ARGUMENT;
    return translate_impl(points, count, n_max, t, as_stream(stream));
}

}  // extern "C"
