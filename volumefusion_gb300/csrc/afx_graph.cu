// afx_graph.cu -- motion graph on the device: greedy radius subsampling (af::buildGraph),
// exact K-nearest-node queries (af::getKnnData), graph-edge pruning
// (af::filterDisconnected), skinning weights, linear-blend warp and projective
// correspondences.  The reference does the first three on the host with nanoflann,
// copying the point cloud down and the results up every frame (src/VolumeFusion.cu:392-419).
#include <cfloat>
#include <cstring>
#include <mutex>

#include "afx_dqb.cuh"
#include "afx_host.h"
#include "afx_internal.h"

namespace afx {

// ------------------------------------------------------------------------------------
// Graph build
// ------------------------------------------------------------------------------------
//
// af::buildGraph visits the sorted point cloud in order and inserts a point as a node
// when none of its K nearest nodes lies closer than that node's radius.  With one radius
// for all nodes (what the pipeline uses) that is: insert p_i iff no node -- existing, or
// inserted earlier in the same call -- is within distance < r.  The device version keeps
// that order exactly:
//   1. points already covered by existing nodes are dropped in parallel;
//   2. the remaining candidates are walked in order by one CTA in chunks of 1024: each
//      chunk is first tested in parallel against the nodes inserted by earlier chunks
//      (uniform grid in global memory), then the still-uncovered ones are resolved in
//      order by one warp against the nodes inserted earlier in the same chunk.
// A new node copies the transform of its nearest node at insertion time
// (src/GraphBuilder.cpp:38-48); equal distances go to the lower node index.

constexpr int kGridSlots = 32;
constexpr int kGridMaxCells = 1 << 18;
constexpr int kChunk = 1024;
constexpr int kNearestBrute = 1024;  // nearest existing node by a scan below this many nodes

struct Grid {
    float org[3];
    float cell;
    int dims[3];
    int* cnt;    // [cells]
    int* slots;  // [cells * kGridSlots]
};

struct GraphState {
    float* nodes;
    float* radii;
    float* T;
    int* n_nodes;
    int cap;
    const float* mesh;
    const unsigned* mesh_count;
    long mesh_max;
    float r;
    Grid g;
    unsigned* flags;     // [mesh_max]
    unsigned* pos;       // [mesh_max]
    unsigned* cand;      // [mesh_max]
    unsigned* ncand;     // [1]
    int* bbox;           // [6] ordered-int min/max
    int* error;          // [1]
    int* n_old;          // [1]
};

AFX_D int ford(float f) {
    int i = __float_as_int(f);
    return i < 0 ? (int)(0x80000000u - (unsigned)i) : i;
}
AFX_D float ordf(int o) { return __int_as_float(o < 0 ? (int)(0x80000000u - (unsigned)o) : o); }

__global__ void graph_bbox_init(int* bbox) {
    if (threadIdx.x < 3) {
        bbox[threadIdx.x] = 0x7fffffff;
        bbox[3 + threadIdx.x] = (int)0x80000000;
    }
}

// Bounding box of the point cloud and the existing nodes: grid-stride over the live counts,
// block reduction, one atomic per block and axis.
__global__ void __launch_bounds__(256) graph_bbox_kernel(GraphState s) {
    __shared__ int smn[3][8], smx[3][8];
    const long m = min((long)*s.mesh_count, s.mesh_max);
    const int n = min(*s.n_nodes, s.cap);
    int mn[3] = {0x7fffffff, 0x7fffffff, 0x7fffffff}, mx[3] = {(int)0x80000000, (int)0x80000000, (int)0x80000000};
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < m + n; i += (long)gridDim.x * blockDim.x) {
        const float* p = i < m ? s.mesh + 3 * i : s.nodes + 3 * (i - m);
        for (int c = 0; c < 3; ++c) {
            int o = ford(p[c]);
            mn[c] = min(mn[c], o);
            mx[c] = max(mx[c], o);
        }
    }
    for (int c = 0; c < 3; ++c) {
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            mn[c] = min(mn[c], __shfl_xor_sync(0xffffffffu, mn[c], off));
            mx[c] = max(mx[c], __shfl_xor_sync(0xffffffffu, mx[c], off));
        }
    }
    if ((threadIdx.x & 31) == 0)
        for (int c = 0; c < 3; ++c) {
            smn[c][threadIdx.x >> 5] = mn[c];
            smx[c][threadIdx.x >> 5] = mx[c];
        }
    __syncthreads();
    if (threadIdx.x < 3) {
        int a = 0x7fffffff, b = (int)0x80000000;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
            a = min(a, smn[threadIdx.x][w]);
            b = max(b, smx[threadIdx.x][w]);
        }
        atomicMin(s.bbox + threadIdx.x, a);
        atomicMax(s.bbox + 3 + threadIdx.x, b);
    }
}

// Chooses the grid from the bounding box, seeds the first node when the graph is empty
// (src/GraphBuilder.cpp:19-20) and checks the radii.
__global__ void graph_setup_kernel(GraphState s, Grid* gout) {
    long m = min((long)*s.mesh_count, s.mesh_max);
    int n = *s.n_nodes;
    *s.n_old = n;
    Grid g = s.g;
    float lo[3], hi[3], ext = 0.f;
    for (int c = 0; c < 3; ++c) {
        lo[c] = ordf(s.bbox[c]);
        hi[c] = ordf(s.bbox[3 + c]);
        if (!(lo[c] <= hi[c])) lo[c] = hi[c] = 0.f;
        ext = fmaxf(ext, hi[c] - lo[c]);
    }
    float cell = s.r > 0.f ? s.r : 1.f;
    if (!(ext < 1e6f)) {  // non-finite coordinates: refuse rather than size a grid from them
        atomicOr(s.error, ERRF_UNSUPPORTED);
        for (int c = 0; c < 3; ++c) lo[c] = hi[c] = 0.f;
    }
    for (int guard = 0; guard < 200; ++guard) {
        long cells = 1;
        for (int c = 0; c < 3; ++c) cells *= (long)((hi[c] - lo[c]) / cell) + 2;
        if (cells <= kGridMaxCells) break;
        cell *= 1.25f;
    }
    g.cell = cell;
    for (int c = 0; c < 3; ++c) {
        g.org[c] = lo[c] - cell * 0.5f;
        g.dims[c] = (int)((hi[c] - lo[c]) / cell) + 2;
    }
    if (cell > 2.0f * s.r) atomicOr(s.error, ERRF_CAPACITY);  // more than 32 nodes per cell possible
    *gout = g;
    if (n == 0 && m > 0) {
        if (s.cap < 1) {
            atomicOr(s.error, ERRF_CAPACITY);
            return;
        }
        for (int c = 0; c < 3; ++c) s.nodes[c] = s.mesh[c];
        s.radii[0] = s.r;
        for (int e = 0; e < 16; ++e) s.T[e] = (e % 5 == 0) ? 1.f : 0.f;
        *s.n_nodes = 1;
    }
}

AFX_D int grid_cell(const Grid& g, const float* p, int* c3) {
    for (int c = 0; c < 3; ++c) {
        int v = (int)floorf((p[c] - g.org[c]) / g.cell);
        c3[c] = min(max(v, 0), g.dims[c] - 1);
    }
    return (c3[2] * g.dims[1] + c3[1]) * g.dims[0] + c3[0];
}

AFX_D void grid_insert(const Grid& g, const float* p, int idx, int* error) {
    int c3[3];
    int cell = grid_cell(g, p, c3);
    int k = atomicAdd(g.cnt + cell, 1);
    if (k < kGridSlots) g.slots[(long)cell * kGridSlots + k] = idx;
    else atomicOr(error, ERRF_CAPACITY);
}

__global__ void graph_check_radii_kernel(GraphState s) {
    const int n = min(*s.n_nodes, s.cap);
    AFX_GRID_STRIDE(i, n) if (s.radii[i] != s.r) atomicOr(s.error, ERRF_UNSUPPORTED);
}

__global__ void graph_insert_existing_kernel(GraphState s, const Grid* gp) {
    const int n = min(*s.n_nodes, s.cap);
    AFX_GRID_STRIDE(i, n) grid_insert(*gp, s.nodes + 3 * i, (int)i, s.error);
}

// Any node in the grid with distance < r?  (radius test of src/GraphBuilder.cpp:28-34)
AFX_D bool grid_covered(const Grid& g, const float* nodes, const float* p, float r) {
    int c3[3];
    grid_cell(g, p, c3);
    for (int dz = -1; dz <= 1; ++dz)
        for (int dy = -1; dy <= 1; ++dy)
            for (int dx = -1; dx <= 1; ++dx) {
                int x = c3[0] + dx, y = c3[1] + dy, z = c3[2] + dz;
                if (x < 0 || y < 0 || z < 0 || x >= g.dims[0] || y >= g.dims[1] || z >= g.dims[2]) continue;
                int cell = (z * g.dims[1] + y) * g.dims[0] + x;
                int c = min(((volatile int*)g.cnt)[cell], kGridSlots);
                for (int k = 0; k < c; ++k) {
                    int j = ((volatile int*)g.slots)[(long)cell * kGridSlots + k];
                    if (sqrtf(l2sq_nanoflann(p, nodes + 3 * j)) < r) return true;
                }
            }
    return false;
}

// flags[i] = 1 for live points no node covers (only the live range is read afterwards)
__global__ void graph_candidates_kernel(GraphState s, const Grid* gp) {
    const long m = min((long)*s.mesh_count, s.mesh_max);
    AFX_GRID_STRIDE(i, m) s.flags[i] = grid_covered(*gp, s.nodes, s.mesh + 3 * i, s.r) ? 0u : 1u;
}

__global__ void graph_compact_kernel(GraphState s, const unsigned* total) {
    const long m = min((long)*s.mesh_count, s.mesh_max);
    AFX_GRID_STRIDE(i, m) if (s.flags[i]) s.cand[s.pos[i]] = (unsigned)i;
    if (blockIdx.x == 0 && threadIdx.x == 0) *s.ncand = *total;
}

// Exact nearest node by expanding rings of grid cells; ties to the lower index.
AFX_D int nearest_node(const Grid& g, const float* nodes, const float* p, float* best_sq) {
    int c3[3];
    grid_cell(g, p, c3);
    float bs = FLT_MAX;
    int bi = -1;
    const int maxr = max(g.dims[0], max(g.dims[1], g.dims[2]));
    for (int ring = 0; ring <= maxr; ++ring) {
        for (int dz = -ring; dz <= ring; ++dz)
            for (int dy = -ring; dy <= ring; ++dy)
                for (int dx = -ring; dx <= ring; ++dx) {
                    if (max(abs(dx), max(abs(dy), abs(dz))) != ring) continue;
                    int x = c3[0] + dx, y = c3[1] + dy, z = c3[2] + dz;
                    if (x < 0 || y < 0 || z < 0 || x >= g.dims[0] || y >= g.dims[1] || z >= g.dims[2]) continue;
                    int cell = (z * g.dims[1] + y) * g.dims[0] + x;
                    int c = min(((volatile int*)g.cnt)[cell], kGridSlots);
                    for (int k = 0; k < c; ++k) {
                        int j = ((volatile int*)g.slots)[(long)cell * kGridSlots + k];
                        float d = l2sq_nanoflann(p, nodes + 3 * j);
                        if (d < bs || (d == bs && j < bi)) {
                            bs = d;
                            bi = j;
                        }
                    }
                }
        // every node outside the examined rings is farther than ring * cell
        if (bi >= 0 && sqrtf(bs) < (float)ring * g.cell) break;
    }
    *best_sq = bs;
    return bi;
}

// While the graph has at most kGreedyCache nodes their positions are also kept in shared memory,
// and the coverage test and the nearest-node search scan them there (the same answers as the grid:
// every node within r is examined, ties go to the lower index); the grid stays up to date and takes
// over if the graph outgrows the cache.  The first build of a sequence walks every point of the
// cloud, and there a grid lookup's chain of dependent global loads set the pace.
constexpr int kGreedyCache = 1000;  // with the chunk arrays, within the 48 KB of static shared memory

AFX_D bool covered_smem(const float* sn, int n, const float* p, float r) {
    for (int j = 0; j < n; ++j)
        if (sqrtf(l2sq_nanoflann(p, sn + 3 * j)) < r) return true;
    return false;
}

__global__ void __launch_bounds__(kChunk) graph_greedy_kernel(GraphState s, const Grid* gp) {
    __shared__ float s_nodes[kGreedyCache * 3];  // node positions while they fit
    __shared__ int s_ncache;                     // nodes in s_nodes (= all nodes, or -1 once outgrown)
    __shared__ unsigned uncovered[kChunk];
    __shared__ int s_nu;
    __shared__ int s_sel[kChunk];
    __shared__ float s_fac[kChunk];
    __shared__ float s_upos[kChunk * 3];  // positions of the uncovered candidates
    __shared__ float s_spos[kChunk * 3];  // positions of the points selected in this chunk
    __shared__ int s_nsel;
    __shared__ int s_stop;
    const Grid g = *gp;
    const unsigned nc = *s.ncand;
    const int tid = threadIdx.x, lane = tid & 31;
    if (tid == 0) s_stop = 0;
    {
        const int n_start = *s.n_nodes;
        const bool fits = n_start <= kGreedyCache;
        if (fits)
            for (int i = tid; i < 3 * n_start; i += blockDim.x) s_nodes[i] = s.nodes[i];
        if (tid == 0) s_ncache = fits ? n_start : -1;
    }
    __syncthreads();
    for (unsigned start = 0; start < nc && !s_stop; start += kChunk) {
        // (a) drop candidates covered by nodes inserted by earlier chunks
        unsigned ci = start + tid;
        bool unc = false;
        const int ncache = s_ncache;
        if (ci < nc) {
            const float* pc = s.mesh + 3 * (long)s.cand[ci];
            unc = ncache >= 0 ? !covered_smem(s_nodes, ncache, pc, s.r) : !grid_covered(g, s.nodes, pc, s.r);
        }
        // ordered compaction of the uncovered candidates
        unsigned bal = __ballot_sync(0xffffffffu, unc);
        __shared__ int wcount[kChunk / 32];
        if (lane == 0) wcount[tid >> 5] = __popc(bal);
        if (tid == 0) s_nsel = 0;
        __syncthreads();
        if (tid == 0) {
            int acc = 0;
            for (int w = 0; w < kChunk / 32; ++w) {
                int c = wcount[w];
                wcount[w] = acc;
                acc += c;
            }
            s_nu = acc;
        }
        __syncthreads();
        if (unc) {
            const int slot = wcount[tid >> 5] + __popc(bal & ((1u << lane) - 1));
            const unsigned v = s.cand[ci];
            uncovered[slot] = v;
            s_upos[3 * slot] = s.mesh[3 * (long)v];
            s_upos[3 * slot + 1] = s.mesh[3 * (long)v + 1];
            s_upos[3 * slot + 2] = s.mesh[3 * (long)v + 2];
        }
        __syncthreads();
        // (b) in-order resolution against the nodes selected earlier in this chunk (warp 0, all
        // positions in shared memory), 32 candidates at a time: each lane tests its candidate against
        // every node selected so far, then the survivors are taken in lane order, each one selected
        // removing the later survivors within r of it -- the same selections as one candidate at a
        // time, with one step per selected node instead of one per candidate.
        if (tid < 32) {
            int nsel = 0;
            const int nu = s_nu;
            for (int base = 0; base < nu; base += 32) {
                const int u = base + lane;
                const bool valid = u < nu;
                float pu[3] = {0.f, 0.f, 0.f};
                bool hit = !valid;
                if (valid) {
                    pu[0] = s_upos[3 * u];
                    pu[1] = s_upos[3 * u + 1];
                    pu[2] = s_upos[3 * u + 2];
                    for (int k = 0; k < nsel && !hit; ++k)
                        if (sqrtf(l2sq_nanoflann(pu, s_spos + 3 * k)) < s.r) hit = true;
                }
                unsigned live = __ballot_sync(0xffffffffu, !hit);
                while (live) {
                    const int j = __ffs(live) - 1;  // the earliest survivor: selected
                    const float pj[3] = {__shfl_sync(0xffffffffu, pu[0], j), __shfl_sync(0xffffffffu, pu[1], j),
                                         __shfl_sync(0xffffffffu, pu[2], j)};
                    if (lane == j) {
                        s_spos[3 * nsel] = pu[0];
                        s_spos[3 * nsel + 1] = pu[1];
                        s_spos[3 * nsel + 2] = pu[2];
                        s_sel[nsel] = (int)uncovered[u];
                    }
                    ++nsel;
                    if (lane > j && !hit && sqrtf(l2sq_nanoflann(pu, pj)) < s.r) hit = true;
                    live = __ballot_sync(0xffffffffu, !hit) & ~((2u << j) - 1u);
                }
                __syncwarp();
            }
            if (lane == 0) s_nsel = nsel;
        }
        __syncthreads();
        // (c) append the selected points as nodes, in order, each with the transform of its nearest
        // node among all nodes before it.  The nearest node is found in parallel: the grid holds
        // the nodes from before this chunk; the ones selected earlier in the chunk are scanned
        // directly, after them, so equal distances still go to the lower index.
        const int n0 = *s.n_nodes;
        const int take = min(s_nsel, max(s.cap - n0, 0));
        if (tid < take) {
            const float* p = s_spos + 3 * tid;
            float bs = FLT_MAX;
            int j = -1;
            if (ncache >= 0) {  // every node in shared memory
                for (int q = 0; q < n0; ++q) {
                    const float d = l2sq_nanoflann(p, s_nodes + 3 * q);
                    if (d < bs) {
                        bs = d;
                        j = q;
                    }
                }
            } else if (n0 <= kNearestBrute) {  // few nodes: a scan beats expanding rings over a sparse grid
                for (int q = 0; q < n0; ++q) {
                    const float d = l2sq_nanoflann(p, s.nodes + 3 * (long)q);
                    if (d < bs) {
                        bs = d;
                        j = q;
                    }
                }
            } else {
                j = nearest_node(g, s.nodes, p, &bs);
            }
            for (int q = 0; q < tid; ++q) {
                const float d = l2sq_nanoflann(p, s_spos + 3 * q);
                if (d < bs) {
                    bs = d;
                    j = n0 + q;
                }
            }
            uncovered[tid] = (unsigned)j;  // reuse: nearest node of selected point tid
            const float d = sqrtf(bs);
            s_fac[tid] = d / (0.f + d);
            const int n = n0 + tid;
            s.nodes[3 * n] = p[0];
            s.nodes[3 * n + 1] = p[1];
            s.nodes[3 * n + 2] = p[2];
            s.radii[n] = s.r;
            if (ncache >= 0 && n < kGreedyCache) {
                s_nodes[3 * n] = p[0];
                s_nodes[3 * n + 1] = p[1];
                s_nodes[3 * n + 2] = p[2];
            }
        }
        __syncthreads();
        // transforms in order (a node may copy from one selected earlier in the chunk): lane e of
        // warp 0 owns entry e, so each copy reads what the same lane wrote before
        if (tid < 16)
            for (int k = 0; k < take; ++k) {
                const long j = (long)uncovered[k];
                s.T[16 * (long)(n0 + k) + tid] = 0.f + s.T[16 * j + tid] * s_fac[k];
            }
        __threadfence();
        __syncthreads();
        if (tid < take) grid_insert(g, s.mesh + 3 * (long)s_sel[tid], n0 + tid, s.error);
        __threadfence();
        __syncthreads();
        if (tid == 0) {
            *s.n_nodes = n0 + take;
            if (s_ncache >= 0) s_ncache = n0 + take <= kGreedyCache ? n0 + take : -1;
            if (take < s_nsel) {
                atomicOr(s.error, ERRF_CAPACITY);
                s_stop = 1;
            }
        }
        __syncthreads();
    }
}

static size_t al(size_t x) { return (x + 255) & ~(size_t)255; }

size_t build_graph_ws(long mesh_max) {
    return 3 * al(mesh_max * 4) + al(scan_workspace_size(mesh_max)) + al((size_t)kGridMaxCells * 4) +
           al((size_t)kGridMaxCells * kGridSlots * 4) + al(sizeof(Grid)) + 1024;
}

int build_graph_impl(float* nodes, float* radii, float* T, int* n_nodes, int cap, const float* mesh,
                     const unsigned* mesh_count, long mesh_max, float r, void* ws, size_t ws_bytes, int* error,
                     cudaStream_t st) {
    if (ws_bytes < build_graph_ws(mesh_max) || !ws) return AFX_ERR_WORKSPACE;
    char* p = static_cast<char*>(ws);
    auto take = [&](size_t n) {
        char* q = p;
        p += al(n);
        return q;
    };
    GraphState s;
    s.nodes = nodes;
    s.radii = radii;
    s.T = T;
    s.n_nodes = n_nodes;
    s.cap = cap;
    s.mesh = mesh;
    s.mesh_count = mesh_count;
    s.mesh_max = mesh_max;
    s.r = r;
    s.flags = (unsigned*)take(mesh_max * 4);
    s.pos = (unsigned*)take(mesh_max * 4);
    s.cand = (unsigned*)take(mesh_max * 4);
    void* scan_ws = take(scan_workspace_size(mesh_max));
    s.g.cnt = (int*)take((size_t)kGridMaxCells * 4);
    s.g.slots = (int*)take((size_t)kGridMaxCells * kGridSlots * 4);
    Grid* gdev = (Grid*)take(sizeof(Grid));
    int* misc = (int*)take(256);
    s.ncand = (unsigned*)misc;
    s.bbox = misc + 2;
    s.n_old = misc + 8;
    unsigned* total = (unsigned*)(misc + 9);
    s.error = error;
    AFX_CUDA(cudaMemsetAsync(s.g.cnt, 0, (size_t)kGridMaxCells * 4, st));
    graph_bbox_init<<<1, 32, 0, st>>>(s.bbox);
    AFX_LAUNCH_CHECK();
    graph_bbox_kernel<<<128, 256, 0, st>>>(s);
    AFX_LAUNCH_CHECK();
    graph_check_radii_kernel<<<grid_for(cap, 256), 256, 0, st>>>(s);
    AFX_LAUNCH_CHECK();
    graph_setup_kernel<<<1, 1, 0, st>>>(s, gdev);
    AFX_LAUNCH_CHECK();
    graph_insert_existing_kernel<<<grid_for(cap, 256), 256, 0, st>>>(s, gdev);
    AFX_LAUNCH_CHECK();
    graph_candidates_kernel<<<grid_for(mesh_max, 256), 256, 0, st>>>(s, gdev);
    AFX_LAUNCH_CHECK();
    int rc = scan_exclusive_dev(s.flags, s.pos, mesh_count, mesh_max, total, scan_ws, st);
    if (rc) return rc;
    graph_compact_kernel<<<grid_for(mesh_max, 256), 256, 0, st>>>(s, total);
    AFX_LAUNCH_CHECK();
    graph_greedy_kernel<<<1, kChunk, 0, st>>>(s, gdev);
    AFX_LAUNCH_CHECK();
    return AFX_OK;
}

// ------------------------------------------------------------------------------------
// KNN (getKnnData<K>): brute force over node tiles in shared memory, per-thread sorted
// top-(K[+1]) list by (nanoflann squared distance, node index).
// ------------------------------------------------------------------------------------

constexpr int kKnnTile = 1024;
constexpr int kKnnThreads = 128;

// One thread per query point (grid-stride over blocks of points, so a block that has no points
// left loads no nodes).  The running list holds the best KK (distance, index) pairs in
// registers: a candidate that beats the last entry (or fills an empty slot) replaces it and
// bubbles up past strictly larger distances, so equal distances keep the earlier index, as the
// ordered insertion did.  Empty slots carry index -1 and sort last.
template <int KK>
__global__ void __launch_bounds__(kKnnThreads) knn_kernel(uint32_t* idx, float* dist, const float* __restrict__ nodes,
                                                          const int* n_nodes, int n_max, const float* __restrict__ pts,
                                                          const unsigned* count, long m_max, int k, int excl) {
    __shared__ float s_n[kKnnTile * 3];
    const int n = min(*n_nodes, n_max);
    const long m = count ? min((long)*count, m_max) : m_max;
    for (long blk = blockIdx.x; blk * kKnnThreads < m; blk += gridDim.x) {
        const long i = blk * kKnnThreads + threadIdx.x;
        float q[3] = {0.f, 0.f, 0.f};
        if (i < m) {
            q[0] = pts[3 * i];
            q[1] = pts[3 * i + 1];
            q[2] = pts[3 * i + 2];
        }
        float bd[KK];
        int bi[KK];
#pragma unroll
        for (int s = 0; s < KK; ++s) {
            bd[s] = 0.f;
            bi[s] = -1;
        }
        for (int base = 0; base < n; base += kKnnTile) {
            const int nt = min(kKnnTile, n - base);
            __syncthreads();
            for (int t = threadIdx.x; t < nt * 3; t += blockDim.x) s_n[t] = nodes[3 * (long)base + t];
            __syncthreads();
            if (i < m)
                for (int j = 0; j < nt; ++j) {
                    const float d = l2sq_nanoflann(q, s_n + 3 * j);
                    if (bi[KK - 1] >= 0 && !(d < bd[KK - 1])) continue;
                    bd[KK - 1] = d;
                    bi[KK - 1] = base + j;
#pragma unroll
                    for (int p = KK - 1; p > 0; --p) {
                        if (bi[p - 1] < 0 || bd[p] < bd[p - 1]) {
                            const float td = bd[p];
                            bd[p] = bd[p - 1];
                            bd[p - 1] = td;
                            const int ti = bi[p];
                            bi[p] = bi[p - 1];
                            bi[p - 1] = ti;
                        }
                    }
                }
        }
        if (i < m)
#pragma unroll
            for (int s = 0; s < KK; ++s) {
                const int o = s - excl;
                if (o < 0 || o >= k) continue;
                if (bi[s] >= 0) {
                    idx[i * k + o] = (uint32_t)bi[s];
                    dist[i * k + o] = sqrtf(bd[s]);
                } else {
                    idx[i * k + o] = AFX_INVALID_INDEX;
                    dist[i * k + o] = FLT_MAX;
                }
            }
    }
}

int knn_impl(uint32_t* idx, float* dist, const float* nodes, const int* n_nodes, int n_max, const float* pts,
             const unsigned* count, long m_max, int k, int excl, cudaStream_t st) {
    if (m_max <= 0) return AFX_OK;
    const int e = excl ? 1 : 0;
    const int kk = k + e;
    // grid-stride over the live points; the search loop is long, so up to 8 blocks per SM
    const long want = (m_max + kKnnThreads - 1) / kKnnThreads;
    const unsigned blocks = (unsigned)(want < 1216 ? want : 1216);
#define AFX_KNN(KK)                                                                                              \
    knn_kernel<KK><<<blocks, kKnnThreads, 0, st>>>(idx, dist, nodes, n_nodes, n_max, pts, count, m_max, k, e); \
    break
    switch (kk) {
        case 1: AFX_KNN(1);
        case 2: AFX_KNN(2);
        case 3: AFX_KNN(3);
        case 4: AFX_KNN(4);
        case 5: AFX_KNN(5);
        case 6: AFX_KNN(6);
        case 7: AFX_KNN(7);
        case 8: AFX_KNN(8);
        case 9: AFX_KNN(9);
        default:
            if (kk <= 12) {
                AFX_KNN(12);
            } else if (kk <= 17) {
                AFX_KNN(17);
            } else {
                return AFX_ERR_UNSUPPORTED;
            }
    }
#undef AFX_KNN
    AFX_LAUNCH_CHECK();
    return AFX_OK;
}

__global__ void filter_disconnected_kernel(uint32_t* idx, float* dist, const int* n_nodes, int n_max, int k,
                                           const float* radii) {
    const int n = min(*n_nodes, n_max);
    AFX_GRID_STRIDE(t, (long)n * k) {
        const long i = t / k;
        const uint32_t nb = idx[t];
        if (nb >= (uint32_t)n) continue;
        if (dist[t] <= radii[i] * 1.3f) continue;
        idx[t] = AFX_INVALID_INDEX;
        dist[t] = FLT_MAX;
    }
}

// computeWarpWeightsKernel (src/VertexManipulation.cu:105-132)
__global__ void warp_weights_kernel(float* w, const float* radii, const uint32_t* idx, const float* dist,
                                    const unsigned* count, long m_max, int k, const int* n_nodes) {
    const long m = count ? min((long)*count, m_max) : m_max;
    const int n = *n_nodes;
    AFX_GRID_STRIDE(i, m) {
        float ws[17];
        float sum = 0.f;
        for (int j = 0; j < k; ++j) {
            uint32_t nb = idx[i * k + j];
            float wj = 0.f;
            if (nb < (uint32_t)n) {
                float r = radii[nb], d = dist[i * k + j];
                wj = (d >= r) ? 0.f : afx_expf(-(d * d) / (2.0f * (r * r)));
            }
            ws[j] = wj;
            sum = sum + wj;
        }
        for (int j = 0; j < k; ++j) w[i * k + j] = (sum != 0.f) ? ws[j] / sum : ws[j];
    }
}

// warpKernel (src/ComputeCorrespondence.cu:5-30)
__global__ void warp_kernel(float* out, const float* __restrict__ pts, const float* __restrict__ T,
                            const uint32_t* __restrict__ idx, const float* __restrict__ w, const unsigned* count,
                            long m_max, int k) {
    long m = count ? min((long)*count, m_max) : m_max;
    AFX_GRID_STRIDE(i, m) {
        float p[3] = {pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]};
        bool zero = true;
        for (int j = 0; j < k; ++j)
            if (!(fabsf(w[i * k + j]) <= 1e-5f)) zero = false;
        float acc[3] = {p[0], p[1], p[2]};
        if (!zero) {
            acc[0] = acc[1] = acc[2] = 0.f;
            for (int j = 0; j < k; ++j) {
                uint32_t nb = idx[i * k + j];
                if (nb == AFX_INVALID_INDEX) continue;
                float o[3];
                mat4_point(T + 16 * (long)nb, p, o);
                float wj = w[i * k + j];
                acc[0] = acc[0] + wj * o[0];
                acc[1] = acc[1] + wj * o[1];
                acc[2] = acc[2] + wj * o[2];
            }
        }
        out[3 * i] = acc[0];
        out[3 * i + 1] = acc[1];
        out[3 * i + 2] = acc[2];
    }
}

int warp_weights_impl(float* w, const float* radii, const uint32_t* idx, const float* dist, const unsigned* count,
                      long m_max, int k, const int* n_nodes, cudaStream_t st) {
    if (m_max <= 0) return AFX_OK;
    if (k > 17) return AFX_ERR_UNSUPPORTED;
    warp_weights_kernel<<<grid_for(m_max, 256), 256, 0, st>>>(w, radii, idx, dist, count, m_max, k, n_nodes);
    AFX_LAUNCH_CHECK();
    return AFX_OK;
}

// The same points moved by the dual-quaternion blend of their nodes (afx_dqb.cuh).
__global__ void warp_dqb_kernel(float* out, const float* __restrict__ pts, const float* __restrict__ T,
                                const uint32_t* __restrict__ idx, const float* __restrict__ w, const unsigned* count,
                                long m_max, int k) {
    long m = count ? min((long)*count, m_max) : m_max;
    AFX_GRID_STRIDE(i, m) {
        const float p[3] = {pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]};
        float o[3];
        dq_blend_point(T, idx + i * k, w + i * k, k, AFX_INVALID_INDEX, p, o);
        out[3 * i] = o[0];
        out[3 * i + 1] = o[1];
        out[3 * i + 2] = o[2];
    }
}

int warp_impl(float* out, const float* pts, const float* T, const uint32_t* idx, const float* w, const unsigned* count,
              long m_max, int k, cudaStream_t st, int blend) {
    if (m_max <= 0) return AFX_OK;
    if (blend == AFX_BLEND_DQB) {
        warp_dqb_kernel<<<grid_for(m_max, 256), 256, 0, st>>>(out, pts, T, idx, w, count, m_max, k);
        AFX_LAUNCH_CHECK();
        return AFX_OK;
    }
    warp_kernel<<<grid_for(m_max, 256), 256, 0, st>>>(out, pts, T, idx, w, count, m_max, k);
    AFX_LAUNCH_CHECK();
    return AFX_OK;
}

// ------------------------------------------------------------------------------------
// Correspondences (correspondencePairsKernel, src/ComputeCorrespondence.cu:45-81),
// compacted in vertex order.
// ------------------------------------------------------------------------------------

struct CorrArgs {
    const float* warped;
    const unsigned* count;
    long m_max;
    Intrinsics K;
    const float* depth;
    int rows, cols;
    const float* frame;
    float thresh;
};

AFX_D int corr_pixel(const CorrArgs& a, long i) {
    const float* v = a.warped + 3 * i;
    float y0 = v[1] / v[2];
    float x0 = v[0] / v[2];
    int y = f2i(y0 * a.K.fy + a.K.cy);
    int x = f2i(x0 * a.K.fx + a.K.cx);
    if (y < 0 || x < 0 || y >= a.rows || x >= a.cols) return -1;
    long px = (long)y * a.cols + x;
    const float* f = a.frame + 3 * px;
    float d[3] = {f[0] - v[0], f[1] - v[1], f[2] - v[2]};
    if (norm3(d) > a.thresh) return -1;
    if (!(a.depth[px] > 1.e-4f)) return -1;
    return (int)px;
}

__global__ void corr_flags_kernel(CorrArgs a, unsigned* flags, int* pix) {
    long m = a.count ? min((long)*a.count, a.m_max) : a.m_max;
    AFX_GRID_STRIDE(i, m) {
        int px = corr_pixel(a, i);
        pix[i] = px;
        flags[i] = px >= 0 ? 1u : 0u;
    }
}

__global__ void corr_scatter_kernel(CorrArgs a, const unsigned* flags, const int* pix, const unsigned* pos, int* corr,
                                    long cap, int* corr_of_vertex) {
    long m = a.count ? min((long)*a.count, a.m_max) : a.m_max;
    AFX_GRID_STRIDE(i, m) {
        if (flags[i]) {
            unsigned p = pos[i];
            if (p < cap) {
                corr[2 * (long)p] = (int)i;
                corr[2 * (long)p + 1] = pix[i];
            }
            if (corr_of_vertex) corr_of_vertex[i] = (int)p;
        } else if (corr_of_vertex) {
            corr_of_vertex[i] = -1;
        }
    }
}

size_t corr_ws(long m_max) { return 3 * al(m_max * 4) + al(scan_workspace_size(m_max)) + 256; }

int correspondences_impl(int* corr, unsigned* corr_count, long cap, const float* warped, const unsigned* count,
                         long m_max, const float* K, const float* depth, int rows, int cols, const float* frame,
                         float thresh, int* corr_of_vertex, void* ws, size_t ws_bytes, cudaStream_t st) {
    if (ws_bytes < corr_ws(m_max) || !ws) return AFX_ERR_WORKSPACE;
    if (m_max <= 0) {
        AFX_CUDA(cudaMemsetAsync(corr_count, 0, 4, st));
        return AFX_OK;
    }
    char* p = static_cast<char*>(ws);
    unsigned* flags = (unsigned*)p;
    p += al(m_max * 4);
    int* pix = (int*)p;
    p += al(m_max * 4);
    unsigned* pos = (unsigned*)p;
    p += al(m_max * 4);
    void* scan_ws = p;
    CorrArgs a;
    a.warped = warped;
    a.count = count;
    a.m_max = m_max;
    a.K = make_intrinsics(K);
    a.depth = depth;
    a.rows = rows;
    a.cols = cols;
    a.frame = frame;
    a.thresh = thresh;
    corr_flags_kernel<<<grid_for(m_max, 256), 256, 0, st>>>(a, flags, pix);
    AFX_LAUNCH_CHECK();
    int rc = scan_exclusive_dev(flags, pos, count, m_max, corr_count, scan_ws, st);
    if (rc) return rc;
    corr_scatter_kernel<<<grid_for(m_max, 256), 256, 0, st>>>(a, flags, pix, pos, corr, cap, corr_of_vertex);
    AFX_LAUNCH_CHECK();
    return AFX_OK;
}

// Device scratch of the stand-alone entry points (error word, node count copy): one per host
// thread and device, allocated on the thread's first call and kept for the life of the process,
// so calls from different host threads never share it.
struct CallScratch {
    int error;
    int n;
    unsigned count;
};

static CallScratch* call_scratch() {
    thread_local CallScratch* s[kMaxDevices] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return nullptr;
    if (!s[dev]) {
        CallScratch* p = nullptr;
        if (cudaMalloc(&p, sizeof(CallScratch)) != cudaSuccess) return nullptr;
        if (cudaMemset(p, 0, sizeof(CallScratch)) != cudaSuccess) {
            cudaFree(p);
            return nullptr;
        }
        s[dev] = p;
    }
    return s[dev];
}

}  // namespace afx

using namespace afx;

extern "C" {

size_t afx_build_graph_workspace_size(long mesh_max, int node_capacity) {
    (void)node_capacity;
    return build_graph_ws(mesh_max);
}

int afx_build_graph(float* nodes, float* radii, float* transforms, int* n_nodes, int node_capacity, const float* mesh,
                    const unsigned* mesh_count, long mesh_max, int knn, float radius, void* workspace,
                    size_t workspace_bytes, void* stream) {
    if (!nodes || !radii || !transforms || !n_nodes || !mesh || !mesh_count || knn < 1 || node_capacity < 1 ||
        mesh_max < 0 || !(radius > 0.f))
        return AFX_ERR_INVALID_ARGUMENT;
    cudaStream_t st = as_stream(stream);
    CallScratch* cs = call_scratch();
    if (!cs) return AFX_ERR_NO_MEMORY;
    AFX_CUDA(cudaMemsetAsync(&cs->error, 0, sizeof(int), st));
    int rc = build_graph_impl(nodes, radii, transforms, n_nodes, node_capacity, mesh, mesh_count, mesh_max, radius,
                              workspace, workspace_bytes, &cs->error, st);
    if (rc) return rc;
    int err = 0;
    AFX_CUDA(cudaMemcpyAsync(&err, &cs->error, sizeof(int), cudaMemcpyDeviceToHost, st));
    AFX_CUDA(cudaStreamSynchronize(st));
    if (err & ERRF_UNSUPPORTED) return AFX_ERR_UNSUPPORTED;
    if (err & ERRF_CAPACITY) return AFX_ERR_CAPACITY;
    return AFX_OK;
}

int afx_knn(uint32_t* idx, float* dist, const float* nodes, const int* n_nodes, int n_nodes_max, const float* points,
            const unsigned* count, long n_points_max, int k, int exclude_closest, void* stream) {
    if (!idx || !dist || !nodes || !n_nodes || !points || k < 1 || n_points_max < 0) return AFX_ERR_INVALID_ARGUMENT;
    return knn_impl(idx, dist, nodes, n_nodes, n_nodes_max, points, count, n_points_max, k, exclude_closest,
                    as_stream(stream));
}

int afx_filter_disconnected(uint32_t* idx, float* dist, const int* n_nodes, int n_nodes_max, int k, const float* radii,
                            void* stream) {
    if (!idx || !dist || !n_nodes || !radii || k < 1) return AFX_ERR_INVALID_ARGUMENT;
    if (n_nodes_max <= 0) return AFX_OK;
    filter_disconnected_kernel<<<grid_for((long)n_nodes_max * k, 256), 256, 0, as_stream(stream)>>>(
        idx, dist, n_nodes, n_nodes_max, k, radii);
    AFX_LAUNCH_CHECK();
    return AFX_OK;
}

int afx_warp_weights(float* weights, const float* radii, const uint32_t* idx, const float* dist, const unsigned* count,
                     long n_points_max, int k, const int* n_nodes, void* stream) {
    if (!weights || !radii || !idx || !dist || !n_nodes || k < 1) return AFX_ERR_INVALID_ARGUMENT;
    return warp_weights_impl(weights, radii, idx, dist, count, n_points_max, k, n_nodes, as_stream(stream));
}

int afx_warp(float* warped, const float* points, const float* transforms, const uint32_t* idx, const float* weights,
             const unsigned* count, long n_points_max, int k, void* stream) {
    if (!warped || !points || !transforms || !idx || !weights || k < 1) return AFX_ERR_INVALID_ARGUMENT;
    return warp_impl(warped, points, transforms, idx, weights, count, n_points_max, k, as_stream(stream));
}

int afx_warp_dqb(float* warped, const float* points, const float* transforms, const uint32_t* idx,
                 const float* weights, const unsigned* count, long n_points_max, int k, void* stream) {
    if (!warped || !points || !transforms || !idx || !weights || k < 1) return AFX_ERR_INVALID_ARGUMENT;
    return warp_impl(warped, points, transforms, idx, weights, count, n_points_max, k, as_stream(stream),
                     AFX_BLEND_DQB);
}

size_t afx_correspondences_workspace_size(long n_points_max) { return corr_ws(n_points_max); }

int afx_correspondences(int* corr, unsigned* corr_count, long capacity, const float* warped, const unsigned* count,
                        long n_points_max, const float K[9], const float* depth, int rows, int cols,
                        const float* frame_vertices, float thresh, void* workspace, size_t workspace_bytes,
                        void* stream) {
    if (!corr || !corr_count || !warped || !K || !depth || !frame_vertices || rows <= 0 || cols <= 0)
        return AFX_ERR_INVALID_ARGUMENT;
    return correspondences_impl(corr, corr_count, capacity, warped, count, n_points_max, K, depth, rows, cols,
                                frame_vertices, thresh, nullptr, workspace, workspace_bytes, as_stream(stream));
}

}  // extern "C"

// ------------------------------------------------------------------------------------
// Correspondence search without any allocation: the same three steps as
// afx_correspondences (flag kernel, exclusive scan, scatter kernel), with the scratch in a
// fixed file-scope device array instead of a caller-provided workspace.  Every scratch word
// is written before it is read within one call (flags and pixels for every live vertex,
// scan block sums, scan output), so nothing has to start at zero and nothing is cleared.
// The array is shared by all calls on a device: calls that overlap in time race on it.
// ------------------------------------------------------------------------------------

namespace afx {

constexpr long kCorrStaticMaxPoints = AFX_CORR_STATIC_MAX_POINTS;
// flags, pixels, scan output (4 bytes each per vertex) + scan block sums + alignment slack
constexpr size_t kCorrStaticBytes = 3 * (size_t)kCorrStaticMaxPoints * 4 + 64 * 1024;

static __device__ __align__(256) unsigned char g_corr_static_scratch[kCorrStaticBytes];

constexpr int kCorrStaticMaxDevices = 64;
static std::mutex g_corr_static_mu;
struct CorrStaticSlot {
    unsigned long long ctx_id = 0;  // context the address belongs to (0: none yet)
    void* ptr = nullptr;
};
static CorrStaticSlot g_corr_static[kCorrStaticMaxDevices];

// Device address of the scratch array in the current device's context.  The lookup
// (cudaGetSymbolAddress, which loads the module into the context if needed and allocates
// nothing) runs on the first call in each context -- once per device unless the device is
// reset -- and its result is kept with the context's identifier, so an address from a
// context that has since been destroyed is never reused.
static int corr_static_scratch(void** out) {
    int dev = 0;
    AFX_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kCorrStaticMaxDevices) return AFX_ERR_UNSUPPORTED;
    std::lock_guard<std::mutex> lock(g_corr_static_mu);
    CorrStaticSlot& slot = g_corr_static[dev];
    const unsigned long long id = current_context_id();
    if (!slot.ptr || id == 0 || id != slot.ctx_id) {
        void* p = nullptr;
        AFX_CUDA(cudaGetSymbolAddress(&p, g_corr_static_scratch));
        slot.ptr = p;
        slot.ctx_id = current_context_id();  // the lookup above made the context current if it was not
    }
    *out = slot.ptr;
    return AFX_OK;
}

}  // namespace afx

extern "C" int afx_correspondences_static(int* corr, unsigned* corr_count, long capacity, const float* warped,
                                          const unsigned* count, long n_points_max, const float K[9],
                                          const float* depth, int rows, int cols, const float* frame_vertices,
                                          float thresh, void* stream) {
    if (!corr || !corr_count || !warped || !K || !depth || !frame_vertices || rows <= 0 || cols <= 0)
        return AFX_ERR_INVALID_ARGUMENT;
    if (n_points_max > kCorrStaticMaxPoints) return AFX_ERR_CAPACITY;
    if (corr_ws(n_points_max) > kCorrStaticBytes) return AFX_ERR_CAPACITY;
    void* scratch = nullptr;
    int rc = corr_static_scratch(&scratch);
    if (rc) return rc;
    return correspondences_impl(corr, corr_count, capacity, warped, count, n_points_max, K, depth, rows, cols,
                                frame_vertices, thresh, nullptr, scratch, kCorrStaticBytes, as_stream(stream));
}
