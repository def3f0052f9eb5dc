// afx_fusion.cu -- the per-frame non-rigid fusion loop (af::runVolumeFusion,
// src/VolumeFusion.cu:223-769) as a device-resident session, plus the library's
// status / error plumbing.
//
// Every stage runs on the session's stream with its sizes kept in device memory, so a
// frame needs no host synchronisation: the canonical point cloud, motion graph,
// correspondences and Gauss-Newton control (energy test, commit of pending transforms)
// all stay on the GPU.  The reference blocks on cudaDeviceSynchronize and copies the
// point cloud and graph to the host every frame.
#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <new>
#include <vector>

#include <cuda.h>
#include <cuda_fp16.h>

#include "afx_gn.h"
#include "afx_host.h"
#include "afx_voxel.h"

namespace afx {

static thread_local int g_last_cuda_error = 0;
static std::atomic<long> g_launches{0};

int note_cuda_error(cudaError_t e) {
    if (e == cudaSuccess) return AFX_OK;
    g_last_cuda_error = (int)e;
    return AFX_ERR_CUDA;
}
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
long launches_total() { return g_launches.load(std::memory_order_relaxed); }

using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);

unsigned long long current_context_id() {
    static CtxGetCurrentFn get_current = nullptr;
    static CtxGetIdFn get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = reinterpret_cast<CtxGetCurrentFn>(p);
        p = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<CtxGetIdFn>(p);
        cudaGetLastError();
    });
    if (!get_current || !get_id) return 0;
    CUcontext c = nullptr;
    if (get_current(&c) != CUDA_SUCCESS || !c) return 0;
    unsigned long long id = 0;
    return get_id(c, &id) == CUDA_SUCCESS ? id : 0;
}

struct FrameStats {
    int frame;
    int n_nodes;
    int new_nodes;
    unsigned mesh_points;
    unsigned correspondences;
    int gn_iterations_done;
    double energy;
    unsigned mesh_vertices, mesh_faces;
    int error;
};

// The streams an object has enqueued work on, each with an event recorded after its latest work
// there, so that tearing the object down waits for its own work only (not the whole device).
struct WorkMarks {
    std::vector<std::pair<cudaStream_t, cudaEvent_t>> marks;
    bool lost = false;  // an event could not be created: teardown waits for the device instead

    // Called after enqueueing work on `st` (never while `st` is capturing).
    void note(cudaStream_t st) {
        for (auto& m : marks)
            if (m.first == st) {
                if (cudaEventRecord(m.second, st) != cudaSuccess) lost = true;
                return;
            }
        cudaEvent_t e = nullptr;
        if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventRecord(e, st) != cudaSuccess) {
            if (e) cudaEventDestroy(e);
            cudaGetLastError();
            lost = true;
            return;
        }
        marks.push_back({st, e});
    }
    // Waits for every marked piece of work, then forgets the marks.
    cudaError_t wait_and_clear() {
        cudaError_t r = cudaSuccess;
        if (lost) r = cudaDeviceSynchronize();
        for (auto& m : marks) {
            const cudaError_t e = cudaEventSynchronize(m.second);
            if (r == cudaSuccess) r = e;
            cudaEventDestroy(m.second);
        }
        marks.clear();
        lost = false;
        return r;
    }
};

}  // namespace afx

using namespace afx;

struct afx_fusion {
    afx_fusion_params p;
    Volume vol;
    long S = 0, P = 0;
    int per[3];
    int frame = 0;
    long launches_at_create = 0;
    // device buffers
    void* arena = nullptr;
    size_t arena_bytes = 0;
    int fmt = kVoxF32;     // voxel storage: kVoxF32, or kVoxF16 (precision form)
    void* tsdf;
    void* weights;
    unsigned* coll;
    uint16_t* depth_mm;
    float* depth;
    float* verts;
    float* normals;
    float* centroid0;      // frame-0 centroid (volume translation)
    float* centroid;       // current frame centroid
    unsigned long long* acc;
    int* error;
    unsigned* epoch;
    float* points;         // canonical point cloud
    unsigned* npoints;
    float* nodes_host;     // positions used for graph build / KNN (the reference's CPU copy)
    float* nodes_dev;      // positions used on the device (the reference's motionGraph_d)
    float* nodes_t;        // translated copy for the voxel support
    float* radii;
    float* T;              // committed transforms
    float* Tp;             // pending transforms
    int* n_nodes;
    int* n_old;
    uint32_t* midx;
    float* mdist;
    float* mw;
    uint32_t* gidx;
    float* gdist;
    float* warped;
    int* corr;
    unsigned* ncorr;
    int* corr_of_vertex;
    float* mverts;
    int* mfaces;
    unsigned* nmverts;
    uint32_t* vidx;        // output-mesh warp: KNN and weights per mesh vertex (warp_mesh only)
    float* vdist;
    float* vw;
    unsigned* nmfaces;
    WarpedVoxel* wvox;
    unsigned char* wcount;
    unsigned char* occ;    // per 8^3 brick: 1 once any voxel of it has a weight (marching cubes skips the rest)
    unsigned* mc_tiles;    // marching cubes on the persistent grid: count + occupied tiles
    uint32_t* umap;        // undistortion map of a distorted camera (null otherwise)
    FrameStats* stats;
    void* ws_sort;
    size_t ws_sort_bytes;
    void* ws_graph;
    size_t ws_graph_bytes;
    void* ws_corr;
    size_t ws_corr_bytes;
    void* ws_support;
    size_t ws_support_bytes;
    void* ws_gn;
    size_t ws_gn_bytes;
    SupportWorkspace sup;
    GnBuffers gn;
    // optional per-stage timing (the reference's TimeMap, include/af/TimeMap.h)
    bool timing = false;
    std::vector<cudaEvent_t> ev_pool;                  // recorded-and-read events for reuse
    std::vector<std::pair<int, cudaEvent_t>> marks;    // (stage started at this event, event); -1 = stage end
    // canonical point cloud double buffer: marching cubes at the end of a frame writes the
    // next frame's raw points into points_buf[cur ^ 1] while points_buf[cur] keeps this frame's
    int cur = 0;
    float* points_buf[2];
    unsigned* npoints_buf[2];
    unsigned* mesh_used;   // canonical point count used by the last frame
    int* frame_dev;        // frame index on the device (written into the statistics)
    // non-rigid frames replayed from CUDA graphs, one per (graph built or not, buffer parity),
    // captured on first use; per-stage timing runs eagerly instead
    bool graphs = true;
    cudaStream_t cap_stream = nullptr;
    // the voxel support is built on a side stream while the Gauss-Newton stages run (fork after the
    // graph build, join before the voxel warp); created with the session, outside any capture
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    // host frames (afx_fusion_process_host): two device input buffers filled on a copy stream, so the
    // next frame's copy overlaps the frame in flight
    uint16_t* in_buf[2] = {nullptr, nullptr};
    cudaStream_t copy_st = nullptr;
    cudaEvent_t ev_in_ready[2] = {nullptr, nullptr}, ev_in_free[2] = {nullptr, nullptr};
    cudaGraphExec_t gexec[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
    cudaGraph_t graph[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};  // kept for batch graphs
    unsigned graph_epoch = 0;  // advanced whenever the captured graphs are dropped
    int mc_tile = kMcTileTma16;  // marching-cubes tile (afx_fusion_autotune)
    long glaunches[2][2] = {{0, 0}, {0, 0}};  // kernels in each captured frame
    long replayed = 0;                        // kernels launched by graph replays
    WorkMarks work;                           // streams holding this session's work (destroy waits on them)
};

namespace afx {

__global__ void copy_new_nodes_kernel(float* dst, const float* src, const int* n_old, const int* n_nodes, int cap) {
    int i = *n_old + blockIdx.x * blockDim.x + threadIdx.x;
    int n = min(*n_nodes, cap);
    if (i < n) {
        dst[3 * i] = src[3 * i];
        dst[3 * i + 1] = src[3 * i + 1];
        dst[3 * i + 2] = src[3 * i + 2];
    }
}

__global__ void record_n_old_kernel(const int* n_nodes, int* n_old) { *n_old = *n_nodes; }

__global__ void frame_begin_kernel(unsigned* epoch, unsigned* ncorr, int* error, unsigned* nmverts, unsigned* nmfaces) {
    unsigned e = *epoch + 1;
    if (e >= (1u << 24)) e = 1;  // collision words are cleared by the host when this wraps
    *epoch = e;
    *ncorr = 0;
    *nmverts = 0;
    *nmfaces = 0;
}

__global__ void stats_kernel(FrameStats* s, int* frame, const int* n_nodes, const int* n_old, const unsigned* npoints,
                             const unsigned* ncorr, const GnState* gn, const unsigned* nv, const unsigned* nf,
                             const int* error, int nonrigid) {
    s->frame = *frame;
    *frame = *frame + 1;
    s->n_nodes = *n_nodes;
    s->new_nodes = nonrigid ? *n_nodes - *n_old : 0;
    s->mesh_points = *npoints;
    s->correspondences = nonrigid ? *ncorr : 0;
    s->gn_iterations_done = nonrigid ? gn->iters : 0;
    s->energy = nonrigid ? gn->e_last : 0.0;
    s->mesh_vertices = *nv;
    s->mesh_faces = *nf;
    s->error = *error;
}

static size_t al(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace afx

enum Stage { ST_PREP, ST_INTEGRATE_RIGID, ST_SORT, ST_GRAPH, ST_KNN, ST_GN_SETUP, ST_GN_LOOP, ST_SUPPORT, ST_VOXEL_WARP,
             ST_WARPED_INTEGRATE, ST_MC, ST_COUNT };

static cudaEvent_t take_event(afx_fusion* f) {
    if (!f->ev_pool.empty()) {
        cudaEvent_t e = f->ev_pool.back();
        f->ev_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

// Records an event that ends the running stage and starts `stage` (-1: no new stage).
static void stage_mark(afx_fusion* f, int stage, cudaStream_t st) {
    if (!f->timing) return;
    cudaEvent_t e = take_event(f);
    if (!e) return;
    cudaEventRecord(e, st);
    f->marks.push_back({stage, e});
}

extern "C" {

const char* afx_status_string(int s) {
    switch (s) {
        case AFX_OK: return "ok";
        case AFX_ERR_INVALID_ARGUMENT: return "invalid argument";
        case AFX_ERR_CAPACITY: return "capacity exceeded";
        case AFX_ERR_CUDA: return "CUDA error";
        case AFX_ERR_SINGULAR: return "singular Gauss-Newton block";
        case AFX_ERR_WORKSPACE: return "workspace too small";
        case AFX_ERR_UNSUPPORTED: return "unsupported input";
        case AFX_ERR_TIMEOUT: return "device wait timed out";
        case AFX_ERR_NO_MEMORY: return "out of device memory";
        case AFX_ERR_IO: return "file input/output failed";
    }
    return "unknown status";
}

int afx_version(void) { return 100; }

int afx_last_cuda_error(void) { return g_last_cuda_error; }

void afx_fusion_default_params(afx_fusion_params* p) {
    std::memset(p, 0, sizeof(*p));
    p->width = 640;
    p->height = 576;
    const float K[9] = {504.f, 0.f, 0.f, 0.f, 504.f, 0.f, 320.f, 288.f, 1.f};
    std::memcpy(p->K, K, sizeof(K));
    p->dims[0] = p->dims[1] = p->dims[2] = 256;
    p->volume_size[0] = p->volume_size[1] = p->volume_size[2] = 1.024f;
    p->delta = 0.016f;
    p->depth_threshold = 1.2f;
    p->bilateral = 1;
    p->bilateral_r = 2;
    p->sigma_i = 0.03f;
    p->sigma_s = 2.f;
    p->bilateral_thr = 0.09f;
    p->excl_angle_lo = 1.3f;
    p->excl_angle_hi = 2.1f;
    p->graph_radius = 0.025f;
    p->knn = 4;
    p->kreg = 8;
    p->update_graph = 1;
    p->icp_iterations = 1;
    p->gn_iterations = 5;
    p->lambda_depth = 1.f;
    p->lambda_reg = 14.142135623730951f;
    p->energy_min_step = 1e-4f;
    p->corr_thresh = 0.01f;
    p->solver = 1;
    p->pcg_iterations = 10;
    p->pcg_tol = 0.0;
    p->integrate = 1;
    p->extract_mesh = 1;
    p->node_capacity = 16384;
    p->mesh_capacity = 2000000;
    p->triangle_capacity = 4000000;
}

// Sizes of every buffer of a session with these parameters (no allocation).
static void session_layout(const afx_fusion_params& p, afx_fusion* f) {
    float vs[3];
    for (int c = 0; c < 3; ++c) vs[c] = p.volume_size[c] / (float)p.dims[c];
    f->vol = make_volume(p.dims, vs, p.volume_size);
    f->S = (long)p.dims[0] * p.dims[1] * p.dims[2];
    f->P = (long)p.width * p.height;
    // voxels per node cube: 2 * ((r / voxelSize).cast<int>() + 1) + 1 (src/VolumeFusion.cu:702-706)
    for (int c = 0; c < 3; ++c) f->per[c] = 2 * ((int)(p.graph_radius / vs[c]) + 1) + 1;
    const long M = p.mesh_capacity, N = p.node_capacity, S = f->S, Pp = f->P;
    const long nbricks = brick_count_total(f->vol);
    f->ws_sort_bytes = sort_unique_volume_workspace_size(M, p.dims[0] + 1);
    f->ws_graph_bytes = build_graph_ws(M);
    f->ws_corr_bytes = corr_ws(M);
    f->ws_support_bytes = support_workspace_size(f->vol, (int)N, f->per);
    f->ws_gn_bytes = gn_workspace_size(M, (int)N, p.knn, p.kreg);
    size_t sz = 0;
    auto add = [&](size_t n) { sz += al(n); };
    f->fmt = p.precision == AFX_PRECISION_FP16 ? kVoxF16 : kVoxF32;
    const long vb = (long)vox_bytes(f->fmt);
    add(S * vb); add(S * vb); add(S * 4);                // tsdf weights coll
    add(Pp * 2); add(Pp * 4); add(Pp * 12); add(Pp * 12);  // frame buffers
    add(Pp * 2); add(Pp * 2);                              // host-frame input buffers
    add(64); add(64); add(64); add(64); add(64);          // centroids acc error epoch
    add(M * 12); add(64); add(M * 12); add(64); add(64);  // point-cloud double buffer + used count
    add(N * 12); add(N * 12); add(N * 12); add(N * 4); add(N * 64); add(N * 64); add(64); add(64);
    add(M * p.knn * 4); add(M * p.knn * 4); add(M * p.knn * 4);
    add(N * p.kreg * 4); add(N * p.kreg * 4);
    add(M * 12); add(M * 8); add(64); add(M * 4);
    add(p.triangle_capacity * 36); add(p.triangle_capacity * 12); add(64); add(64);
    const long mesh_knn = p.warp_mesh ? p.triangle_capacity * 3 * p.knn * 4 : 0;  // output-mesh warp
    add(mesh_knn); add(mesh_knn); add(mesh_knn);
    add(nbricks * 512 * sizeof(WarpedVoxel)); add(nbricks * 512); add(nbricks);
    add(mc_tile_ws_words(f->vol) * 4);
    add(p.distortion.is_distorted ? Pp * 8 : 0);
    add(sizeof(FrameStats)); add(64);
    add(f->ws_sort_bytes); add(f->ws_graph_bytes); add(f->ws_corr_bytes); add(f->ws_support_bytes); add(f->ws_gn_bytes);
    f->arena_bytes = sz + 4096;
}

static bool params_valid(const afx_fusion_params& p) {
    return !(p.width < 3 || p.height < 3 || p.dims[0] < 3 || p.dims[1] < 3 || p.dims[2] < 3 || p.knn < 1 ||
             p.knn > 8 || p.kreg < 1 || p.kreg > 8 || p.node_capacity < 1 || p.mesh_capacity < 1 ||
             p.triangle_capacity < 1 || !(p.graph_radius > 0.f) || p.icp_iterations < 0 || p.gn_iterations < 0 ||
             p.pcg_iterations < 0 || (p.precision != AFX_PRECISION_FP32 && p.precision != AFX_PRECISION_FP16) ||
             (p.blend != AFX_BLEND_LBS && p.blend != AFX_BLEND_DQB));
}

size_t afx_fusion_memory_bytes(const afx_fusion_params* params) {
    if (!params || !params_valid(*params)) return 0;
    afx_fusion tmp;
    tmp.p = *params;
    session_layout(*params, &tmp);
    return tmp.arena_bytes;
}

int afx_fusion_create(const afx_fusion_params* params, afx_fusion** out) {
    if (!params || !out) return AFX_ERR_INVALID_ARGUMENT;
    const afx_fusion_params& p = *params;
    if (!params_valid(p)) return AFX_ERR_INVALID_ARGUMENT;
    afx_fusion* f = new (std::nothrow) afx_fusion();
    if (!f) return AFX_ERR_NO_MEMORY;
    f->p = p;
    session_layout(p, f);
    const long M = p.mesh_capacity, N = p.node_capacity, S = f->S, Pp = f->P;
    const long nbricks = brick_count_total(f->vol);
    cudaError_t e = cudaMalloc(&f->arena, f->arena_bytes);
    if (e != cudaSuccess) {
        note_cuda_error(e);
        delete f;
        return AFX_ERR_NO_MEMORY;
    }
    char* q = static_cast<char*>(f->arena);
    auto take = [&](size_t n) {
        char* r = q;
        q += al(n);
        return r;
    };
    f->tsdf = take(S * vox_bytes(f->fmt));
    f->weights = take(S * vox_bytes(f->fmt));
    f->coll = (unsigned*)take(S * 4);
    f->depth_mm = (uint16_t*)take(Pp * 2);
    f->in_buf[0] = (uint16_t*)take(Pp * 2);
    f->in_buf[1] = (uint16_t*)take(Pp * 2);
    f->depth = (float*)take(Pp * 4);
    f->verts = (float*)take(Pp * 12);
    f->normals = (float*)take(Pp * 12);
    f->centroid0 = (float*)take(64);
    f->centroid = (float*)take(64);
    f->acc = (unsigned long long*)take(64);
    f->error = (int*)take(64);
    f->epoch = (unsigned*)take(64);
    f->points_buf[0] = (float*)take(M * 12);
    f->npoints_buf[0] = (unsigned*)take(64);
    f->points_buf[1] = (float*)take(M * 12);
    f->npoints_buf[1] = (unsigned*)take(64);
    f->mesh_used = (unsigned*)take(64);
    f->points = f->points_buf[0];
    f->npoints = f->npoints_buf[0];
    f->nodes_host = (float*)take(N * 12);
    f->nodes_dev = (float*)take(N * 12);
    f->nodes_t = (float*)take(N * 12);
    f->radii = (float*)take(N * 4);
    f->T = (float*)take(N * 64);
    f->Tp = (float*)take(N * 64);
    f->n_nodes = (int*)take(64);
    f->n_old = (int*)take(64);
    f->midx = (uint32_t*)take(M * p.knn * 4);
    f->mdist = (float*)take(M * p.knn * 4);
    f->mw = (float*)take(M * p.knn * 4);
    f->gidx = (uint32_t*)take(N * p.kreg * 4);
    f->gdist = (float*)take(N * p.kreg * 4);
    f->warped = (float*)take(M * 12);
    f->corr = (int*)take(M * 8);
    f->ncorr = (unsigned*)take(64);
    f->corr_of_vertex = (int*)take(M * 4);
    f->mverts = (float*)take(p.triangle_capacity * 36);
    f->mfaces = (int*)take(p.triangle_capacity * 12);
    f->nmverts = (unsigned*)take(64);
    f->nmfaces = (unsigned*)take(64);
    const long mesh_knn = p.warp_mesh ? p.triangle_capacity * 3 * p.knn * 4 : 0;
    f->vidx = (uint32_t*)take(mesh_knn);
    f->vdist = (float*)take(mesh_knn);
    f->vw = (float*)take(mesh_knn);
    f->wvox = (WarpedVoxel*)take(nbricks * 512 * sizeof(WarpedVoxel));
    f->wcount = (unsigned char*)take(nbricks * 512);
    f->occ = (unsigned char*)take(nbricks);
    f->mc_tiles = (unsigned*)take(mc_tile_ws_words(f->vol) * 4);
    f->umap = p.distortion.is_distorted ? (uint32_t*)take(Pp * 8) : nullptr;
    f->stats = (FrameStats*)take(sizeof(FrameStats));
    f->frame_dev = (int*)take(64);
    f->ws_sort = take(f->ws_sort_bytes);
    f->ws_graph = take(f->ws_graph_bytes);
    f->ws_corr = take(f->ws_corr_bytes);
    f->ws_support = take(f->ws_support_bytes);
    f->ws_gn = take(f->ws_gn_bytes);
    if (!carve_support(f->ws_support, f->ws_support_bytes, f->vol, (int)N, f->per, &f->sup) ||
        !gn_carve(f->ws_gn, f->ws_gn_bytes, M, (int)N, p.knn, p.kreg, &f->gn)) {
        cudaFree(f->arena);
        delete f;
        return AFX_ERR_WORKSPACE;
    }
    f->launches_at_create = launches_total();
    // The whole arena is cleared, so no buffer starts with the bytes of an earlier allocation,
    // then the volume and counters are set; on a private non-blocking stream, so that creating a
    // session neither waits for nor holds up other sessions' work.
    cudaStream_t init = nullptr;
    e = cudaStreamCreateWithFlags(&init, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&f->side, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&f->ev_fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&f->ev_join, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&f->copy_st, cudaStreamNonBlocking);
    for (int k = 0; k < 2 && e == cudaSuccess; ++k) {
        e = cudaEventCreateWithFlags(&f->ev_in_ready[k], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&f->ev_in_free[k], cudaEventDisableTiming);
    }
    if (e == cudaSuccess) e = cudaMemsetAsync(f->arena, 0, f->arena_bytes, init);
    int rc = e == cudaSuccess ? afx_fusion_reset(f, init) : note_cuda_error(e);
    if (!rc && f->umap)  // cv::undistort's map, built once: it depends on the camera only
        rc = undistort_map_impl(f->umap, p.width, p.height, p.K, &p.distortion, AFX_UNDISTORT_LINEAR, init);
    e = init ? cudaStreamSynchronize(init) : cudaSuccess;
    if (!rc && e != cudaSuccess) rc = note_cuda_error(e);
    if (init) cudaStreamDestroy(init);
    f->work.wait_and_clear();  // the reset's mark names the private stream
    if (rc) {
        if (f->side) cudaStreamDestroy(f->side);
        if (f->ev_fork) cudaEventDestroy(f->ev_fork);
        if (f->ev_join) cudaEventDestroy(f->ev_join);
        if (f->copy_st) cudaStreamDestroy(f->copy_st);
        for (int k = 0; k < 2; ++k) {
            if (f->ev_in_ready[k]) cudaEventDestroy(f->ev_in_ready[k]);
            if (f->ev_in_free[k]) cudaEventDestroy(f->ev_in_free[k]);
        }
        cudaFree(f->arena);
        delete f;
        return rc;
    }
    *out = f;
    return AFX_OK;
}

// Forget the captured frame graphs (they are captured again on next use).
static void drop_graphs(afx_fusion* f) {
    for (int b = 0; b < 2; ++b)
        for (int c = 0; c < 2; ++c) {
            if (f->gexec[b][c]) cudaGraphExecDestroy(f->gexec[b][c]);
            if (f->graph[b][c]) cudaGraphDestroy(f->graph[b][c]);
            f->gexec[b][c] = nullptr;
            f->graph[b][c] = nullptr;
            f->glaunches[b][c] = 0;
        }
    ++f->graph_epoch;
}

int afx_fusion_destroy(afx_fusion* f) {
    if (!f) return AFX_ERR_INVALID_ARGUMENT;
    f->work.wait_and_clear();  // the session's own work on every stream it was given
    if (f->side) cudaStreamSynchronize(f->side);  // joined into those streams, unless a frame failed midway
    for (auto& m : f->marks) cudaEventDestroy(m.second);
    for (auto e : f->ev_pool) cudaEventDestroy(e);
    drop_graphs(f);
    if (f->cap_stream) cudaStreamDestroy(f->cap_stream);
    if (f->side) cudaStreamDestroy(f->side);
    if (f->ev_fork) cudaEventDestroy(f->ev_fork);
    if (f->ev_join) cudaEventDestroy(f->ev_join);
    if (f->copy_st) {
        cudaStreamSynchronize(f->copy_st);  // a host frame's copy, if the caller never ran its frame
        cudaStreamDestroy(f->copy_st);
    }
    for (int k = 0; k < 2; ++k) {
        if (f->ev_in_ready[k]) cudaEventDestroy(f->ev_in_ready[k]);
        if (f->ev_in_free[k]) cudaEventDestroy(f->ev_in_free[k]);
    }
    cudaError_t e = cudaFree(f->arena);
    delete f;
    return note_cuda_error(e);
}

__global__ void fill_kernel(float* p, long n, float v) {
    long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (i < n) p[i] = v;
}

__global__ void fill_u16_kernel(unsigned short* p, long n, unsigned short v) {
    long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (i < n) p[i] = v;
}

int afx_fusion_reset(afx_fusion* f, void* stream) {
    if (!f) return AFX_ERR_INVALID_ARGUMENT;
    cudaStream_t st = as_stream(stream);
    // DeviceTsdf::initDefault: values -1, weights 0 (0xBC00 is -1 in FP16)
    if (f->fmt == kVoxF16)
        fill_u16_kernel<<<blocks_for(f->S, 256), 256, 0, st>>>(static_cast<unsigned short*>(f->tsdf), f->S, 0xBC00);
    else
        fill_kernel<<<blocks_for(f->S, 256), 256, 0, st>>>(static_cast<float*>(f->tsdf), f->S, -1.f);
    AFX_LAUNCH_CHECK();
    AFX_CUDA(cudaMemsetAsync(f->weights, 0, f->S * vox_bytes(f->fmt), st));
    AFX_CUDA(cudaMemsetAsync(f->coll, 0, f->S * 4, st));
    AFX_CUDA(cudaMemsetAsync(f->occ, 0, brick_count_total(f->vol), st));
    AFX_CUDA(cudaMemsetAsync(f->centroid0, 0, 64, st));
    AFX_CUDA(cudaMemsetAsync(f->acc, 0, 64, st));
    AFX_CUDA(cudaMemsetAsync(f->error, 0, 64, st));
    AFX_CUDA(cudaMemsetAsync(f->epoch, 0, 64, st));
    AFX_CUDA(cudaMemsetAsync(f->npoints_buf[0], 0, 64, st));
    AFX_CUDA(cudaMemsetAsync(f->npoints_buf[1], 0, 64, st));
    AFX_CUDA(cudaMemsetAsync(f->mesh_used, 0, 64, st));
    f->cur = 0;
    f->points = f->points_buf[0];
    f->npoints = f->npoints_buf[0];
    AFX_CUDA(cudaMemsetAsync(f->frame_dev, 0, 64, st));
    AFX_CUDA(cudaMemsetAsync(f->n_nodes, 0, 64, st));
    AFX_CUDA(cudaMemsetAsync(f->n_old, 0, 64, st));
    AFX_CUDA(cudaMemsetAsync(f->ncorr, 0, 64, st));
    AFX_CUDA(cudaMemsetAsync(f->nmverts, 0, 64, st));
    AFX_CUDA(cudaMemsetAsync(f->nmfaces, 0, 64, st));
    AFX_CUDA(cudaMemsetAsync(f->stats, 0, sizeof(FrameStats), st));
    f->frame = 0;
    f->work.note(st);
    return AFX_OK;
}

// The output mesh of the frame, as the reference leaves it (src/VolumeFusion.cu:744-762): vertices
// translated by the frame-0 centroid (runTranslateKernel) and, with warp_mesh (settings.isMeshWarped,
// details::warpMeshGPU :75-110), warped into the live frame: the K nearest graph nodes of every
// vertex (getKnnData over the host node positions), skinning weights with the d < r cut-off
// (runComputeWarpWeightsKernel) and the blend of the committed transforms (runWarpKernel, in place).
static int finish_output_mesh(afx_fusion* f, bool nonrigid, cudaStream_t st) {
    const afx_fusion_params& p = f->p;
    if (!p.extract_mesh) return AFX_OK;
    const long vmax = p.triangle_capacity * 3;
    int rc = translate_dev_impl(f->mverts, f->mverts, f->nmverts, vmax, f->centroid0, 1.f, st);
    if (rc || !p.warp_mesh || !nonrigid) return rc;
    rc = knn_impl(f->vidx, f->vdist, f->nodes_host, f->n_nodes, p.node_capacity, f->mverts, f->nmverts, vmax, p.knn, 0,
                  st);
    if (!rc) rc = warp_weights_impl(f->vw, f->radii, f->vidx, f->vdist, f->nmverts, vmax, p.knn, f->n_nodes, st);
    if (!rc) rc = warp_impl(f->mverts, f->mverts, f->T, f->vidx, f->vw, f->nmverts, vmax, p.knn, st, p.blend);
    return rc;
}

static int extract_frame_mesh(afx_fusion* f, int cur, cudaStream_t st) {
    // canonical point cloud for the next frame (runMarchingCubesMeshKernel on the volume the next
    // frame starts from) and, if asked, the output mesh (runMarchingCubesFullKernel), in one pass
    const int next = cur ^ 1;
    AFX_CUDA(cudaMemsetAsync(f->npoints_buf[next], 0, 4, st));
    const bool mesh = f->p.extract_mesh != 0;
    return mc_fused_impl(f->tsdf, f->weights, f->fmt, f->vol, 0.f, f->points_buf[next], f->npoints_buf[next], f->p.mesh_capacity,
                         mesh ? f->mverts : nullptr, mesh ? f->nmverts : nullptr, f->p.triangle_capacity * 3,
                         mesh ? f->mfaces : nullptr, mesh ? f->nmfaces : nullptr, f->p.triangle_capacity, st, f->error,
                         f->mc_tile, f->occ, f->mc_tiles);
}

// Everything a frame does on the device, in stream order on `st`; host state is not changed.
// Non-rigid frames use the point-cloud buffer `cur` (the parity after the toggle) and build the
// graph when `build`.
static int enqueue_frame(afx_fusion* f, const uint16_t* depth_mm, cudaStream_t st, int cur, bool build) {
    const afx_fusion_params& p = f->p;
    int rc;
    static const float I3[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    frame_begin_kernel<<<1, 1, 0, st>>>(f->epoch, f->ncorr, f->error, f->nmverts, f->nmfaces);
    AFX_LAUNCH_CHECK();
    // af::loadProcessFrame (src/VolumeFusion.cu:151-220)
    afx_prep_params pp;
    std::memcpy(pp.K, p.K, sizeof(pp.K));
    pp.depth_threshold = p.depth_threshold;
    pp.bilateral = p.bilateral;
    pp.bilateral_r = p.bilateral_r;
    pp.sigma_i = p.sigma_i;
    pp.sigma_s = p.sigma_s;
    pp.bilateral_thr = p.bilateral_thr;
    pp.excl_angle_lo = p.excl_angle_lo;
    pp.excl_angle_hi = p.excl_angle_hi;
    stage_mark(f, ST_PREP, st);
    rc = frame_prep_impl(depth_mm, p.width, p.height, &pp, f->depth, f->verts, f->normals,
                         f->frame == 0 ? f->centroid0 : f->centroid, f->acc, f->error, st, f->umap);
    if (rc) return rc;
    if (f->frame == 0) {
        stage_mark(f, ST_INTEGRATE_RIGID, st);
        // rigid integration at the frame-0 centroid (src/VolumeFusion.cu:334-336)
        rc = integrate_rigid_impl(f->tsdf, f->weights, f->fmt, f->depth, p.width, p.height, p.delta, f->vol, I3, nullptr, p.K,
                                  st, f->centroid0, f->occ);
        if (rc) return rc;
        stage_mark(f, ST_MC, st);
        rc = extract_frame_mesh(f, cur, st);
        if (!rc) rc = finish_output_mesh(f, false, st);
        if (rc) return rc;
        stage_mark(f, -1, st);
        stats_kernel<<<1, 1, 0, st>>>(f->stats, f->frame_dev, f->n_nodes, f->n_old, f->mesh_used, f->ncorr, f->gn.state,
                                      f->nmverts, f->nmfaces, f->error, 0);
        AFX_LAUNCH_CHECK();
        return AFX_OK;
    }
    const long M = p.mesh_capacity;
    const int N = p.node_capacity;
    // canonical point cloud: sort + unique, then + frame-0 centroid (src/VolumeFusion.cu:382-389)
    stage_mark(f, ST_SORT, st);
    float* points = f->points_buf[cur];
    unsigned* npoints = f->npoints_buf[cur];
    rc = sort_unique_volume_impl(points, npoints, M, f->ws_sort, f->ws_sort_bytes, f->vol, st, f->error);
    if (rc) return rc;
    AFX_CUDA(cudaMemcpyAsync(f->mesh_used, npoints, 4, cudaMemcpyDeviceToDevice, st));
    if (rc) return rc;
    rc = translate_dev_impl(points, points, npoints, M, f->centroid0, 1.f, st);
    if (rc) return rc;
    // motion graph (src/VolumeFusion.cu:394-404)
    stage_mark(f, ST_GRAPH, st);
    record_n_old_kernel<<<1, 1, 0, st>>>(f->n_nodes, f->n_old);
    AFX_LAUNCH_CHECK();
    if (build) {
        rc = build_graph_impl(f->nodes_host, f->radii, f->T, f->n_nodes, N, points, npoints, M, p.graph_radius,
                              f->ws_graph, f->ws_graph_bytes, f->error, st);
        if (rc) return rc;
        copy_new_nodes_kernel<<<blocks_for(N, 256), 256, 0, st>>>(f->nodes_dev, f->nodes_host, f->n_old, f->n_nodes, N);
        AFX_LAUNCH_CHECK();
    }
    // Voxel support (the node -> brick lists) needs only the graph: with stage timing off it is built
    // on the side stream while the KNN and Gauss-Newton stages run (they read nodes_dev too, and
    // write none of what the support build touches); the join is before the voxel warp.
    const bool fork = !f->timing;
    if (fork) {
        AFX_CUDA(cudaEventRecord(f->ev_fork, st));
        AFX_CUDA(cudaStreamWaitEvent(f->side, f->ev_fork, 0));
        rc = translate_dev_impl(f->nodes_t, f->nodes_dev, nullptr, N, f->centroid0, -1.f, f->side);
        if (!rc) rc = build_support(f->sup, f->vol, f->per, f->nodes_t, f->radii, f->n_nodes, N, f->error, f->side);
        const cudaError_t je = cudaEventRecord(f->ev_join, f->side);  // recorded even after a failure: the join
        if (rc) return rc;
        if (je != cudaSuccess) return note_cuda_error(je);
    }
    // KNN and weights (src/VolumeFusion.cu:410-424)
    stage_mark(f, ST_KNN, st);
    rc = knn_impl(f->midx, f->mdist, f->nodes_host, f->n_nodes, N, points, npoints, M, p.knn, 0, st);
    if (rc) return rc;
    rc = knn_impl(f->gidx, f->gdist, f->nodes_host, f->n_nodes, N, f->nodes_host,
                  reinterpret_cast<const unsigned*>(f->n_nodes), N, p.kreg, 1, st);
    if (rc) return rc;
    rc = afx_filter_disconnected(f->gidx, f->gdist, f->n_nodes, N, p.kreg, f->radii, st);
    if (rc) return rc;
    rc = warp_weights_impl(f->mw, f->radii, f->midx, f->mdist, npoints, M, p.knn, f->n_nodes, st);
    if (rc) return rc;
    GnArgs g;
    std::memset(&g, 0, sizeof(g));
    g.mesh = points;
    g.mesh_count = npoints;
    g.m_max = M;
    g.midx = f->midx;
    g.mw = f->mw;
    g.k = p.knn;
    g.normals = f->normals;
    g.frame = f->verts;
    g.corr = f->corr;
    g.corr_count = f->ncorr;
    g.c_max = M;
    g.corr_of_vertex = f->corr_of_vertex;
    g.nodes = f->nodes_dev;
    g.n_nodes = f->n_nodes;
    g.n_max = N;
    g.gidx = f->gidx;
    g.kreg = p.kreg;
    g.lam_d = p.lambda_depth;
    g.lam_r = p.lambda_reg;
    g.min_step = p.energy_min_step;
    g.blend = p.blend;
    g.b = f->gn;
    g.error = f->error;
    stage_mark(f, ST_GN_SETUP, st);
    rc = gn_frame_setup(g, st);
    if (rc) return rc;
    const double tol = p.solver == 2 ? p.pcg_tol : 0.0;
    for (int icp = 0; icp < p.icp_iterations; ++icp) {
        // warp with the committed transforms, then projective correspondences (src/VolumeFusion.cu:439-447)
        rc = warp_impl(f->warped, points, f->T, f->midx, f->mw, npoints, M, p.knn, st, p.blend);
        if (rc) return rc;
        rc = correspondences_impl(f->corr, f->ncorr, M, f->warped, npoints, M, p.K, f->depth, p.height, p.width,
                                  f->verts, p.corr_thresh, f->corr_of_vertex, f->ws_corr, f->ws_corr_bytes, st);
        if (rc) return rc;
        rc = gn_icp_setup(g, f->Tp, f->T, st);
        if (rc) return rc;
        stage_mark(f, ST_GN_LOOP, st);
        rc = gn_loop(g, points, f->warped, f->T, f->Tp, p.gn_iterations, p.pcg_iterations, tol, st);
        if (rc) return rc;
    }
    // voxel support, warp, collisions and warped integration (src/VolumeFusion.cu:702-741)
    stage_mark(f, ST_SUPPORT, st);
    if (fork) {
        AFX_CUDA(cudaStreamWaitEvent(st, f->ev_join, 0));
    } else {
        rc = translate_dev_impl(f->nodes_t, f->nodes_dev, nullptr, N, f->centroid0, -1.f, st);
        if (rc) return rc;
        rc = build_support(f->sup, f->vol, f->per, f->nodes_t, f->radii, f->n_nodes, N, f->error, st);
        if (rc) return rc;
    }
    // the reference translates its device graph back in place: p = (p - c) + c (src/VolumeFusion.cu:721)
    rc = translate_dev_impl(f->nodes_dev, f->nodes_t, nullptr, N, f->centroid0, 1.f, st);
    if (rc) return rc;
    WarpArgs wa;
    std::memset(&wa, 0, sizeof(wa));
    wa.vol = f->vol;
    wa.bg = make_bricks(f->vol);
    wa.k = p.knn;
    wa.nodes_t = f->nodes_t;
    wa.radii = f->radii;
    wa.transforms = f->T;
    wa.brick_offset = f->sup.brick_offset;
    wa.brick_count = f->sup.brick_count;
    wa.brick_nodes = f->sup.brick_nodes;
    wa.active = f->sup.active;
    wa.n_active = f->sup.n_active;
    for (int c = 0; c < 3; ++c) wa.per[c] = f->per[c];
    wa.centroid_dev = f->centroid0;
    std::memcpy(wa.Rinv, I3, sizeof(I3));
    wa.blend = p.blend;
    wa.out = f->wvox;
    wa.out_count = f->wcount;
    wa.coll = f->coll;
    wa.epoch_dev = f->epoch;
    wa.error = f->error;
    stage_mark(f, ST_VOXEL_WARP, st);
    rc = launch_brick_warp(wa, wa.bg.n, st);
    if (rc) return rc;
    stage_mark(f, ST_WARPED_INTEGRATE, st);
    if (p.integrate) {
        WarpedIntegrateArgs ia;
        ia.vol = f->vol;
        ia.bg = wa.bg;
        ia.active = f->sup.active;
        ia.n_active = f->sup.n_active;
        ia.in = f->wvox;
        ia.in_count = f->wcount;
        ia.coll = f->coll;
        ia.epoch_dev = f->epoch;
        ia.tsdf = f->tsdf;
        ia.weights = f->weights;
        ia.fmt = f->fmt;
        ia.depth = f->depth;
        ia.W = p.width;
        ia.H = p.height;
        ia.delta = p.delta;
        ia.K = make_intrinsics(p.K);
        ia.occ = f->occ;
        rc = launch_brick_integrate(ia, wa.bg.n, st);
        if (rc) return rc;
    }
    stage_mark(f, ST_MC, st);
    rc = extract_frame_mesh(f, cur, st);
    if (!rc) rc = finish_output_mesh(f, true, st);
    if (rc) return rc;
    stage_mark(f, -1, st);
    stats_kernel<<<1, 1, 0, st>>>(f->stats, f->frame_dev, f->n_nodes, f->n_old, f->mesh_used, f->ncorr, f->gn.state,
                                  f->nmverts, f->nmfaces, f->error, 1);
    AFX_LAUNCH_CHECK();
    return AFX_OK;
}

// Capture the non-rigid frame for (build, cur) into a CUDA graph on a private stream.
static int capture_frame(afx_fusion* f, int cur, bool build) {
    if (!f->cap_stream) AFX_CUDA(cudaStreamCreateWithFlags(&f->cap_stream, cudaStreamNonBlocking));
    const long l0 = launches_total();
    AFX_CUDA(cudaStreamBeginCapture(f->cap_stream, cudaStreamCaptureModeThreadLocal));
    const int rc = enqueue_frame(f, f->depth_mm, f->cap_stream, cur, build);
    cudaGraph_t graph = nullptr;
    const cudaError_t e = cudaStreamEndCapture(f->cap_stream, &graph);
    if (rc || e != cudaSuccess || !graph) {
        if (graph) cudaGraphDestroy(graph);
        cudaGetLastError();
        return rc ? rc : AFX_ERR_CUDA;
    }
    cudaGraphExec_t exec = nullptr;
    const cudaError_t ie = cudaGraphInstantiate(&exec, graph, 0);
    if (ie != cudaSuccess) {
        cudaGraphDestroy(graph);
        return note_cuda_error(ie);
    }
    f->gexec[build][cur] = exec;
    f->graph[build][cur] = graph;
    f->glaunches[build][cur] = launches_total() - l0;
    return AFX_OK;
}

int afx_fusion_process(afx_fusion* f, const uint16_t* depth_mm, void* stream) {
    if (!f || !depth_mm) return AFX_ERR_INVALID_ARGUMENT;
    cudaStream_t st = as_stream(stream);
    if (f->frame == 0) {
        const int rc = enqueue_frame(f, depth_mm, st, f->cur, false);
        if (rc) return rc;
        f->frame++;
        f->work.note(st);
        return AFX_OK;
    }
    const int cur = f->cur ^ 1;
    const bool build = f->frame == 1 || f->p.update_graph;
    // frames 1 and 2 run eagerly (first-use set-up of the kernels happens there); later frames
    // replay a captured graph that reads the frame from the session's own input buffer
    bool replay = f->graphs && !f->timing && f->frame >= 3;
    if (replay && !f->gexec[build][cur] && capture_frame(f, cur, build) != AFX_OK) {
        f->graphs = false;  // capture failed: keep launching one by one
        replay = false;
    }
    if (replay) {
        if (depth_mm != f->depth_mm)
            AFX_CUDA(cudaMemcpyAsync(f->depth_mm, depth_mm, (size_t)f->P * 2, cudaMemcpyDeviceToDevice, st));
        AFX_CUDA(cudaGraphLaunch(f->gexec[build][cur], st));
        f->replayed += f->glaunches[build][cur];
    } else {
        const int rc = enqueue_frame(f, depth_mm, st, cur, build);
        if (rc) return rc;
    }
    f->cur = cur;
    f->points = f->points_buf[cur];
    f->npoints = f->npoints_buf[cur];
    f->frame++;
    f->work.note(st);
    return AFX_OK;
}

// The frame is copied into one of two input buffers on the session's copy stream (after the frame
// that last read that buffer) and the frame waits for the copy: a caller that submits the next frame
// before the current one finishes gets its copy overlapped with the current frame's kernels.
int afx_fusion_process_host(afx_fusion* f, const uint16_t* depth_mm_host, void* stream) {
    if (!f || !depth_mm_host) return AFX_ERR_INVALID_ARGUMENT;
    cudaStream_t st = as_stream(stream);
    const int k = f->frame & 1;
    AFX_CUDA(cudaStreamWaitEvent(f->copy_st, f->ev_in_free[k], 0));
    AFX_CUDA(cudaMemcpyAsync(f->in_buf[k], depth_mm_host, f->P * 2, cudaMemcpyHostToDevice, f->copy_st));
    AFX_CUDA(cudaEventRecord(f->ev_in_ready[k], f->copy_st));
    AFX_CUDA(cudaStreamWaitEvent(st, f->ev_in_ready[k], 0));
    int rc = afx_fusion_process(f, f->in_buf[k], stream);
    const cudaError_t e = cudaEventRecord(f->ev_in_free[k], st);  // the buffer is free once this frame is done
    if (!rc && e != cudaSuccess) rc = note_cuda_error(e);
    return rc;
}

static_assert(sizeof(FrameStats) == sizeof(afx_frame_stats), "statistics layouts differ");

int afx_fusion_stats_async(afx_fusion* f, afx_frame_stats* out_host, void* stream) {
    if (!f || !out_host) return AFX_ERR_INVALID_ARGUMENT;
    AFX_CUDA(cudaMemcpyAsync(out_host, f->stats, sizeof(FrameStats), cudaMemcpyDeviceToHost, as_stream(stream)));
    f->work.note(as_stream(stream));
    return AFX_OK;
}

int afx_fusion_stats(afx_fusion* f, afx_frame_stats* out, void* stream) {
    if (!f || !out) return AFX_ERR_INVALID_ARGUMENT;
    cudaStream_t st = as_stream(stream);
    FrameStats s;
    AFX_CUDA(cudaMemcpyAsync(&s, f->stats, sizeof(s), cudaMemcpyDeviceToHost, st));
    AFX_CUDA(cudaStreamSynchronize(st));
    out->frame = s.frame;
    out->n_nodes = s.n_nodes;
    out->new_nodes = s.new_nodes;
    out->mesh_points = s.mesh_points;
    out->correspondences = s.correspondences;
    out->gn_iterations_done = s.gn_iterations_done;
    out->energy = s.energy;
    out->mesh_vertices = s.mesh_vertices;
    out->mesh_faces = s.mesh_faces;
    out->error = s.error;
    if (s.error & ERRF_TIMEOUT) return AFX_ERR_TIMEOUT;
    if (s.error & ERRF_SINGULAR) return AFX_ERR_SINGULAR;
    if (s.error & ERRF_UNSUPPORTED) return AFX_ERR_UNSUPPORTED;
    if (s.error & (ERRF_CAPACITY | ERRF_INDEX)) return AFX_ERR_CAPACITY;
    return AFX_OK;
}

}  // extern "C"

namespace afx {

// Voxels of the active bricks with at least one supporting node (count slot > 0).
__global__ void support_count_kernel(const unsigned char* count, const unsigned* n_active, unsigned long long* out) {
    const long n = (long)*n_active * 512;
    unsigned long long c = 0;
    AFX_GRID_STRIDE(i, n) c += count[i] ? 1ull : 0ull;
    c = warp_sum(c);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(out, c);
}

__global__ void occ_count_kernel(const unsigned char* occ, long n, unsigned long long* out) {
    unsigned long long c = 0;
    AFX_GRID_STRIDE(i, n) c += occ[i] ? 1ull : 0ull;
    c = warp_sum(c);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(out, c);
}

}  // namespace afx

extern "C" {

int afx_fusion_occupied_bricks(afx_fusion* f, unsigned long long* bricks, unsigned long long* total, void* stream) {
    if (!f || !bricks) return AFX_ERR_INVALID_ARGUMENT;
    cudaStream_t st = as_stream(stream);
    const long n = brick_count_total(f->vol);
    unsigned long long* cnt = reinterpret_cast<unsigned long long*>(f->acc) + 5;  // spare word of acc's 64 B
    AFX_CUDA(cudaMemsetAsync(cnt, 0, sizeof(unsigned long long), st));
    occ_count_kernel<<<grid_for(n, 256), 256, 0, st>>>(f->occ, n, cnt);
    AFX_LAUNCH_CHECK();
    AFX_CUDA(cudaMemcpyAsync(bricks, cnt, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
    AFX_CUDA(cudaStreamSynchronize(st));
    if (total) *total = (unsigned long long)n;
    return AFX_OK;
}

int afx_fusion_support_size(afx_fusion* f, unsigned* active_bricks, unsigned long long* supported_voxels,
                            void* stream) {
    if (!f) return AFX_ERR_INVALID_ARGUMENT;
    cudaStream_t st = as_stream(stream);
    unsigned nb = 0;
    AFX_CUDA(cudaMemcpyAsync(&nb, f->sup.n_active, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
    AFX_CUDA(cudaStreamSynchronize(st));
    if (active_bricks) *active_bricks = nb;
    if (supported_voxels) {
        unsigned long long* cnt = reinterpret_cast<unsigned long long*>(f->acc) + 4;  // spare words of acc's 64 B
        AFX_CUDA(cudaMemsetAsync(cnt, 0, sizeof(unsigned long long), st));
        if (nb) {
            support_count_kernel<<<grid_for((long)nb * 512, 256), 256, 0, st>>>(f->wcount, f->sup.n_active, cnt);
            AFX_LAUNCH_CHECK();
        }
        AFX_CUDA(cudaMemcpyAsync(supported_voxels, cnt, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
        AFX_CUDA(cudaStreamSynchronize(st));
    }
    return AFX_OK;
}

int afx_fusion_tsdf(afx_fusion* f, float** tsdf, float** weights) {
    if (!f) return AFX_ERR_INVALID_ARGUMENT;
    if (f->fmt != kVoxF32) return AFX_ERR_UNSUPPORTED;  // FP16 sessions: afx_fusion_volume
    if (tsdf) *tsdf = static_cast<float*>(f->tsdf);
    if (weights) *weights = static_cast<float*>(f->weights);
    return AFX_OK;
}

int afx_fusion_volume(afx_fusion* f, void** tsdf, void** weights, int* precision) {
    if (!f) return AFX_ERR_INVALID_ARGUMENT;
    if (tsdf) *tsdf = f->tsdf;
    if (weights) *weights = f->weights;
    if (precision) *precision = f->fmt == kVoxF16 ? AFX_PRECISION_FP16 : AFX_PRECISION_FP32;
    return AFX_OK;
}

int afx_fusion_graph(afx_fusion* f, float** nodes, float** radii, float** transforms, int** n_nodes) {
    if (!f) return AFX_ERR_INVALID_ARGUMENT;
    if (nodes) *nodes = f->nodes_host;
    if (radii) *radii = f->radii;
    if (transforms) *transforms = f->T;
    if (n_nodes) *n_nodes = f->n_nodes;
    return AFX_OK;
}

int afx_fusion_centroid(afx_fusion* f, float** centroid) {
    if (!f || !centroid) return AFX_ERR_INVALID_ARGUMENT;
    *centroid = f->centroid0;
    return AFX_OK;
}

int afx_fusion_point_cloud(afx_fusion* f, float** points, unsigned** count) {
    if (!f) return AFX_ERR_INVALID_ARGUMENT;
    if (points) *points = f->points;
    if (count) *count = f->npoints;
    return AFX_OK;
}

int afx_fusion_mesh(afx_fusion* f, float** vertices, unsigned** vertex_count, int** faces, unsigned** face_count) {
    if (!f) return AFX_ERR_INVALID_ARGUMENT;
    if (vertices) *vertices = f->mverts;
    if (vertex_count) *vertex_count = f->nmverts;
    if (faces) *faces = f->mfaces;
    if (face_count) *face_count = f->nmfaces;
    return AFX_OK;
}

int afx_fusion_frame_views(afx_fusion* f, float** depth, float** vertices, float** normals) {
    if (!f) return AFX_ERR_INVALID_ARGUMENT;
    if (depth) *depth = f->depth;
    if (vertices) *vertices = f->verts;
    if (normals) *normals = f->normals;
    return AFX_OK;
}

int afx_fusion_set_transforms(afx_fusion* f, const float* transforms_host, int n, void* stream) {
    if (!f || !transforms_host || n < 0 || n > f->p.node_capacity) return AFX_ERR_INVALID_ARGUMENT;
    AFX_CUDA(cudaMemcpyAsync(f->T, transforms_host, (size_t)n * 64, cudaMemcpyHostToDevice, as_stream(stream)));
    f->work.note(as_stream(stream));
    return AFX_OK;
}

long afx_fusion_kernel_launches(const afx_fusion* f) {
    return f ? launches_total() - f->launches_at_create + f->replayed : 0;
}

int afx_fusion_set_graphs(afx_fusion* f, int on) {
    if (!f) return AFX_ERR_INVALID_ARGUMENT;
    f->graphs = on != 0;
    return AFX_OK;
}

int afx_fusion_graph_count(const afx_fusion* f) {
    if (!f) return 0;
    int c = 0;
    for (auto& row : f->gexec)
        for (auto& g : row) c += g != nullptr;
    return f->graphs ? c : 0;
}

int afx_fusion_set_tile(afx_fusion* f, int tile) {
    if (!f || tile < 0 || tile >= kMcTiles) return AFX_ERR_INVALID_ARGUMENT;
    if (tile != f->mc_tile) {
        AFX_CUDA(f->work.wait_and_clear());  // graphs in flight may still use the old tile
        drop_graphs(f);
        f->mc_tile = tile;
    }
    return AFX_OK;
}

int afx_fusion_get_tile(const afx_fusion* f) { return f ? f->mc_tile : -1; }

// Times every marching-cubes tile on the session's current volume (the extraction at the end of
// a frame, re-run: the next frame's raw point cloud and the current mesh are written again with the
// same contents, triangles possibly in another order) and keeps the fastest.  Blocks on `stream`.
int afx_fusion_autotune(afx_fusion* f, int* tile_out, float* ms_out, void* stream) {
    if (!f) return AFX_ERR_INVALID_ARGUMENT;
    cudaStream_t st = as_stream(stream);
    AFX_CUDA(cudaStreamSynchronize(st));
    cudaEvent_t e0, e1;
    AFX_CUDA(cudaEventCreate(&e0));
    AFX_CUDA(cudaEventCreate(&e1));
    const int saved = f->mc_tile;
    int best = saved;
    float best_ms = 1e30f;
    int rc = AFX_OK;
    for (int tile = 0; tile < kMcTiles && rc == AFX_OK; ++tile) {
        f->mc_tile = tile;
        float t_min = 1e30f;
        for (int rep = 0; rep < 4 && rc == AFX_OK; ++rep) {  // the first run of a tile also sets it up
            cudaEventRecord(e0, st);
            rc = extract_frame_mesh(f, f->cur, st);
            cudaEventRecord(e1, st);
            if (cudaEventSynchronize(e1) != cudaSuccess) rc = AFX_ERR_CUDA;
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (rep > 0 && ms < t_min) t_min = ms;
        }
        if (ms_out) ms_out[tile] = t_min;
        if (t_min < best_ms) {
            best_ms = t_min;
            best = tile;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    f->mc_tile = saved;
    if (rc) return rc;
    rc = afx_fusion_set_tile(f, best);
    if (tile_out) *tile_out = best;
    return rc;
}

int afx_fusion_set_timing(afx_fusion* f, int on) {
    if (!f) return AFX_ERR_INVALID_ARGUMENT;
    f->timing = on != 0;
    return AFX_OK;
}

int afx_fusion_stage_times(afx_fusion* f, double* ms, int n, int reset) {
    if (!f || !ms || n < 1) return AFX_ERR_INVALID_ARGUMENT;
    for (int i = 0; i < n; ++i) ms[i] = 0.0;
    if (!f->marks.empty()) cudaEventSynchronize(f->marks.back().second);
    for (size_t i = 0; i + 1 < f->marks.size(); ++i) {
        int stage = f->marks[i].first;
        if (stage < 0 || stage >= n) continue;
        float t = 0.f;
        if (cudaEventElapsedTime(&t, f->marks[i].second, f->marks[i + 1].second) == cudaSuccess) ms[stage] += t;
    }
    cudaGetLastError();
    if (reset) {
        for (auto& m : f->marks) f->ev_pool.push_back(m.second);
        f->marks.clear();
    }
    return ST_COUNT;
}

int afx_copy_device(void* dst, const void* src, size_t bytes, void* stream) {
    if ((!dst || !src) && bytes) return AFX_ERR_INVALID_ARGUMENT;
    if (!bytes) return AFX_OK;
    AFX_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, as_stream(stream)));
    return AFX_OK;
}

}  // extern "C"

// ------------------------------------------------------------------------------------
// Batched form: one frame of every session of a batch with one graph launch.
//
// Each session keeps its own buffers, kernels and reduction orders (so its results are those it
// has alone).  A session whose next frame is replayed (fourth frame of a sequence on) contributes
// its captured frame graph as a child node of one parent graph, after a copy node that brings its
// frame into the session's input buffer and before a copy node that brings its statistics to the
// batch's pinned host array.  The children have no edges between them, so their kernels overlap on
// the device.  Parent graphs are cached per pattern of (build mode, buffer parity, graph epoch)
// of the sessions -- a batch that advances in step alternates between two -- and only the copy
// sources change from call to call (executable-graph node updates, no re-instantiation).  Sessions
// in their first frames run their kernels one by one on the caller's stream first.
// ------------------------------------------------------------------------------------

struct afx_batch {
    std::vector<afx_fusion*> s;
    afx_frame_stats* stats_host = nullptr;  // pinned, one per session
    struct Exec {
        cudaGraphExec_t exec = nullptr;
        cudaGraph_t graph = nullptr;              // kept: node updates name its nodes
        std::vector<int> members;                 // session indices in the graph
        std::vector<cudaGraphNode_t> in_copy;     // frame copy node of each member
    };
    std::map<std::vector<long>, Exec> cache;
    long graph_launches = 0;
    WorkMarks work;  // streams the batch's graphs were launched on
};

namespace {

// Failure of a graph-building call: reported on stderr when AFX_VERBOSE is set; the runtime's
// last-error state is cleared so that later launches do not see it.
int batch_fail(const char* what, cudaError_t e) {
    if (std::getenv("AFX_VERBOSE")) std::fprintf(stderr, "afx_batch: %s: %s\n", what, cudaGetErrorString(e));
    cudaGetLastError();
    return note_cuda_error(e);
}

void batch_free(afx_batch* b) {
    for (auto& kv : b->cache) {
        if (kv.second.exec) cudaGraphExecDestroy(kv.second.exec);
        if (kv.second.graph) cudaGraphDestroy(kv.second.graph);
    }
    if (b->stats_host) cudaFreeHost(b->stats_host);
    delete b;
}

// The parent graph for the members' (build, cur) variants.
int batch_instantiate(afx_batch* b, const std::vector<int>& members, const std::vector<int>& build,
                      const std::vector<int>& cur, const uint16_t* const* depth, afx_batch::Exec* out) {
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaGraphCreate(&g, 0);
    if (e != cudaSuccess) return batch_fail("cudaGraphCreate", e);
    out->members = members;
    out->in_copy.assign(members.size(), nullptr);
    const char* what = nullptr;
    for (size_t k = 0; k < members.size() && e == cudaSuccess; ++k) {
        afx_fusion* f = b->s[members[k]];
        cudaGraphNode_t cp = nullptr, child = nullptr, st = nullptr;
        what = "frame copy node";
        e = cudaGraphAddMemcpyNode1D(&cp, g, nullptr, 0, f->depth_mm, depth[members[k]], (size_t)f->P * 2,
                                     cudaMemcpyDefault);
        if (e == cudaSuccess) {
            what = "child graph node";
            e = cudaGraphAddChildGraphNode(&child, g, &cp, 1, f->graph[build[k]][cur[k]]);
        }
        if (e == cudaSuccess) {
            what = "statistics copy node";
            e = cudaGraphAddMemcpyNode1D(&st, g, &child, 1, b->stats_host + members[k], f->stats, sizeof(FrameStats),
                                         cudaMemcpyDefault);
        }
        out->in_copy[k] = cp;
    }
    if (e == cudaSuccess) {
        what = "instantiate";
        e = cudaGraphInstantiate(&out->exec, g, 0);
    }
    if (e != cudaSuccess) {
        cudaGraphDestroy(g);
        out->exec = nullptr;
        return batch_fail(what, e);
    }
    out->graph = g;
    return AFX_OK;
}

}  // namespace

extern "C" {

int afx_batch_create(afx_fusion* const* sessions, int n, afx_batch** out) {
    if (!sessions || n < 1 || !out) return AFX_ERR_INVALID_ARGUMENT;
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < i; ++j)
            if (!sessions[i] || sessions[i] == sessions[j]) return AFX_ERR_INVALID_ARGUMENT;
    afx_batch* b = new (std::nothrow) afx_batch();
    if (!b) return AFX_ERR_NO_MEMORY;
    b->s.assign(sessions, sessions + n);
    const cudaError_t e = cudaHostAlloc(reinterpret_cast<void**>(&b->stats_host), sizeof(afx_frame_stats) * n,
                                        cudaHostAllocDefault);
    if (e != cudaSuccess) {
        batch_free(b);
        return note_cuda_error(e);
    }
    std::memset(b->stats_host, 0, sizeof(afx_frame_stats) * n);
    *out = b;
    return AFX_OK;
}

int afx_batch_destroy(afx_batch* b) {
    if (!b) return AFX_ERR_INVALID_ARGUMENT;
    b->work.wait_and_clear();  // the batch's graph launches
    batch_free(b);
    return AFX_OK;
}

int afx_batch_process(afx_batch* b, const uint16_t* const* depth_mm, void* stream) {
    if (!b || !depth_mm) return AFX_ERR_INVALID_ARGUMENT;
    cudaStream_t st = as_stream(stream);
    const int n = (int)b->s.size();
    for (int i = 0; i < n; ++i)
        if (!depth_mm[i] || depth_mm[i] == b->s[i]->depth_mm) return AFX_ERR_INVALID_ARGUMENT;
    std::vector<int> members, build, cur;
    std::vector<long> key;
    for (int i = 0; i < n; ++i) {
        afx_fusion* f = b->s[i];
        const int c = f->cur ^ 1;
        const bool bd = f->frame == 1 || f->p.update_graph;
        bool replay = f->graphs && !f->timing && f->frame >= 3;
        if (replay && !f->gexec[bd][c] && capture_frame(f, c, bd) != AFX_OK) {
            f->graphs = false;
            replay = false;
        }
        if (!replay) {  // first frames of a sequence (or graphs off): kernels one by one
            int rc = afx_fusion_process(f, depth_mm[i], stream);
            if (!rc) rc = afx_fusion_stats_async(f, b->stats_host + i, stream);
            if (rc) return rc;
            continue;
        }
        members.push_back(i);
        build.push_back(bd);
        cur.push_back(c);
        key.push_back(((long)i << 40) | ((long)f->graph_epoch << 2) | (bd << 1) | c);
    }
    if (members.empty()) return AFX_OK;
    auto it = b->cache.find(key);
    if (it == b->cache.end()) {
        afx_batch::Exec ex;
        const int rc = batch_instantiate(b, members, build, cur, depth_mm, &ex);
        if (rc) return rc;
        it = b->cache.emplace(key, ex).first;
    } else {
        for (size_t k = 0; k < members.size(); ++k) {
            afx_fusion* f = b->s[members[k]];
            const cudaError_t e = cudaGraphExecMemcpyNodeSetParams1D(
                it->second.exec, it->second.in_copy[k], f->depth_mm, depth_mm[members[k]], (size_t)f->P * 2,
                cudaMemcpyDefault);
            if (e != cudaSuccess) return batch_fail("frame copy update", e);
        }
    }
    const cudaError_t le = cudaGraphLaunch(it->second.exec, st);
    if (le != cudaSuccess) return batch_fail("launch", le);
    ++b->graph_launches;
    b->work.note(st);
    for (size_t k = 0; k < members.size(); ++k) {
        afx_fusion* f = b->s[members[k]];
        f->work.note(st);  // the member's frame ran inside the batch graph on st
        f->replayed += f->glaunches[build[k]][cur[k]];
        f->cur = cur[k];
        f->points = f->points_buf[cur[k]];
        f->npoints = f->npoints_buf[cur[k]];
        f->frame++;
    }
    return AFX_OK;
}

int afx_batch_stats(afx_batch* b, afx_frame_stats* out, int n) {
    if (!b || !out || n < (int)b->s.size()) return AFX_ERR_INVALID_ARGUMENT;
    std::memcpy(out, b->stats_host, sizeof(afx_frame_stats) * b->s.size());
    return AFX_OK;
}

long afx_batch_graph_launches(const afx_batch* b) { return b ? b->graph_launches : 0; }

}  // extern "C"

// ------------------------------------------------------------------------------------
// Session volume and mesh to and from the reference's file formats (afx_io.cu)
// ------------------------------------------------------------------------------------

extern "C" {

int afx_fusion_save_volume(afx_fusion* f, const char* path, void* stream) {
    if (!f || !path) return AFX_ERR_INVALID_ARGUMENT;
    cudaStream_t st = as_stream(stream);
    const size_t S = (size_t)f->S;
    std::vector<float> t(S), w(S);
    if (f->fmt == kVoxF16) {
        std::vector<__half> th(S);
        std::vector<unsigned short> wh(S);
        AFX_CUDA(cudaMemcpyAsync(th.data(), f->tsdf, 2 * S, cudaMemcpyDeviceToHost, st));
        AFX_CUDA(cudaMemcpyAsync(wh.data(), f->weights, 2 * S, cudaMemcpyDeviceToHost, st));
        AFX_CUDA(cudaStreamSynchronize(st));
        for (size_t i = 0; i < S; ++i) {
            t[i] = __half2float(th[i]);  // exact widening
            w[i] = (float)wh[i];
        }
    } else {
        AFX_CUDA(cudaMemcpyAsync(t.data(), f->tsdf, 4 * S, cudaMemcpyDeviceToHost, st));
        AFX_CUDA(cudaMemcpyAsync(w.data(), f->weights, 4 * S, cudaMemcpyDeviceToHost, st));
        AFX_CUDA(cudaStreamSynchronize(st));
    }
    return afx_tsdf_save(path, f->p.dims, f->p.volume_size, f->vol.vs, f->p.delta, t.data(), w.data());
}

}  // extern "C"

namespace afx {

// Brick occupancy of a volume read from a file: bricks holding any voxel with a weight.
template <class WT>
__global__ void occ_from_weights_kernel(const WT* weights, Volume vol, int nbx, int nby, unsigned char* occ) {
    const long S = (long)vol.dims[0] * vol.dims[1] * vol.dims[2];
    AFX_GRID_STRIDE(i, S) {
        if (!(weights[i] > (WT)0)) continue;
        const int x = (int)(i % vol.dims[0]), y = (int)((i / vol.dims[0]) % vol.dims[1]);
        const int z = (int)(i / ((long)vol.dims[0] * vol.dims[1]));
        occ[((long)(z >> 3) * nby + (y >> 3)) * nbx + (x >> 3)] = 1;
    }
}

static int rebuild_occupancy(afx_fusion* f, cudaStream_t st) {
    const BrickGrid bg = make_bricks(f->vol);
    AFX_CUDA(cudaMemsetAsync(f->occ, 0, bg.n, st));
    if (f->fmt == kVoxF16)
        occ_from_weights_kernel<<<grid_for(f->S, 256), 256, 0, st>>>(static_cast<const unsigned short*>(f->weights),
                                                                      f->vol, bg.nb[0], bg.nb[1], f->occ);
    else
        occ_from_weights_kernel<<<grid_for(f->S, 256), 256, 0, st>>>(static_cast<const float*>(f->weights), f->vol,
                                                                      bg.nb[0], bg.nb[1], f->occ);
    AFX_LAUNCH_CHECK();
    return AFX_OK;
}

}  // namespace afx

extern "C" {

int afx_fusion_volume_changed(afx_fusion* f, void* stream) {
    if (!f) return AFX_ERR_INVALID_ARGUMENT;
    return rebuild_occupancy(f, as_stream(stream));
}

int afx_fusion_load_volume(afx_fusion* f, const char* path, void* stream) {
    if (!f || !path) return AFX_ERR_INVALID_ARGUMENT;
    int dims[3];
    int rc = afx_tsdf_load_header(path, dims, nullptr, nullptr, nullptr);
    if (rc) return rc;
    if (dims[0] != f->p.dims[0] || dims[1] != f->p.dims[1] || dims[2] != f->p.dims[2]) return AFX_ERR_INVALID_ARGUMENT;
    const size_t S = (size_t)f->S;
    std::vector<float> t(S), w(S);
    rc = afx_tsdf_load(path, t.data(), w.data(), (long)S);
    if (rc) return rc;
    cudaStream_t st = as_stream(stream);
    if (f->fmt == kVoxF16) {
        std::vector<__half> th(S);
        std::vector<unsigned short> wh(S);
        for (size_t i = 0; i < S; ++i) {
            if (!(w[i] >= 0.f && w[i] <= 65535.f) || w[i] != (float)(unsigned short)w[i]) return AFX_ERR_UNSUPPORTED;
            th[i] = __float2half_rn(t[i]);
            wh[i] = (unsigned short)w[i];
        }
        AFX_CUDA(cudaMemcpyAsync(f->tsdf, th.data(), 2 * S, cudaMemcpyHostToDevice, st));
        AFX_CUDA(cudaMemcpyAsync(f->weights, wh.data(), 2 * S, cudaMemcpyHostToDevice, st));
    } else {
        AFX_CUDA(cudaMemcpyAsync(f->tsdf, t.data(), 4 * S, cudaMemcpyHostToDevice, st));
        AFX_CUDA(cudaMemcpyAsync(f->weights, w.data(), 4 * S, cudaMemcpyHostToDevice, st));
    }
    rc = rebuild_occupancy(f, st);
    if (rc) return rc;
    AFX_CUDA(cudaStreamSynchronize(st));
    return AFX_OK;
}

int afx_fusion_save_mesh_ply(afx_fusion* f, const char* path, void* stream) {
    if (!f || !path) return AFX_ERR_INVALID_ARGUMENT;
    if (!f->p.extract_mesh) return AFX_ERR_UNSUPPORTED;
    cudaStream_t st = as_stream(stream);
    unsigned nf = 0;
    AFX_CUDA(cudaMemcpyAsync(&nf, f->nmfaces, 4, cudaMemcpyDeviceToHost, st));
    AFX_CUDA(cudaStreamSynchronize(st));
    const long faces = nf < (unsigned long)f->p.triangle_capacity ? (long)nf : f->p.triangle_capacity;
    std::vector<float> v(9 * (size_t)faces);
    std::vector<int> fc(3 * (size_t)faces);
    AFX_CUDA(cudaMemcpyAsync(v.data(), f->mverts, v.size() * 4, cudaMemcpyDeviceToHost, st));
    AFX_CUDA(cudaMemcpyAsync(fc.data(), f->mfaces, fc.size() * 4, cudaMemcpyDeviceToHost, st));
    AFX_CUDA(cudaStreamSynchronize(st));
    return afx_save_ply(path, v.data(), 3 * faces, nullptr, fc.data(), faces);
}

}  // extern "C"
