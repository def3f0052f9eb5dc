// afx_serve.cu -- serving many depth streams on one GPU.
//
// A server owns up to max_sessions fusion sessions.  A session is admitted only while the
// device bytes of all admitted sessions stay within the memory budget (afx_fusion_memory_bytes);
// a refused open reports AFX_ERR_NO_MEMORY and the caller retries once others have closed.
// Every session has its own CUDA stream and a small ring of in-flight frames, so frames of
// different sessions that arrive while others are running are queued at once and overlap on the
// device (each non-rigid frame is one CUDA-graph launch after the first three frames).
// Frames of one session stay in order on its stream.  submit() copies the host depth into the
// slot's pinned buffer and enqueues the frame; poll() returns finished frames with their
// statistics and their latency from submit() to completion.  A session's results do not
// depend on what else runs: its kernels touch only its own buffers and reduce in fixed orders.
//
// A closed session is kept, idle, for reuse: a later open with equal parameters takes it back
// after afx_fusion_reset (queued on its stream), so its device arena, pinned slots, stream and
// captured frame graphs are reused -- no allocation, no device-wide synchronisation from
// cudaFree, no graph capture.  Idle sessions count against the budget; an open that needs room
// frees the oldest idle ones first.
#include <chrono>
#include <cstring>
#include <map>
#include <mutex>
#include <new>
#include <vector>

#include "afx_internal.h"

namespace {

constexpr int kSlots = 4;  // frames in flight per session

using Clock = std::chrono::steady_clock;

struct Slot {
    uint16_t* staging = nullptr;        // pinned depth, width * height
    afx_frame_stats* stats = nullptr;   // pinned statistics of the frame
    cudaEvent_t done = nullptr;
    Clock::time_point t_submit;
    uint64_t tag = 0;
};

struct Session {
    int id = 0;
    afx_fusion* f = nullptr;
    cudaStream_t st = nullptr;
    size_t bytes = 0;
    long pixels = 0;
    afx_fusion_params params{};
    Slot slots[kSlots];
    int head = 0, count = 0;  // ring of in-flight frames
    bool closing = false;
};

// Field by field (the struct has padding).
bool params_equal(const afx_fusion_params& a, const afx_fusion_params& b) {
    static_assert(sizeof(afx_fusion_params) == 248, "afx_fusion_params changed: update params_equal");
    bool eq = a.width == b.width && a.height == b.height && a.delta == b.delta &&
              a.depth_threshold == b.depth_threshold && a.bilateral == b.bilateral &&
              a.bilateral_r == b.bilateral_r && a.sigma_i == b.sigma_i && a.sigma_s == b.sigma_s &&
              a.bilateral_thr == b.bilateral_thr && a.excl_angle_lo == b.excl_angle_lo &&
              a.excl_angle_hi == b.excl_angle_hi && a.graph_radius == b.graph_radius && a.knn == b.knn &&
              a.kreg == b.kreg && a.update_graph == b.update_graph && a.icp_iterations == b.icp_iterations &&
              a.gn_iterations == b.gn_iterations && a.lambda_depth == b.lambda_depth && a.lambda_reg == b.lambda_reg &&
              a.energy_min_step == b.energy_min_step && a.corr_thresh == b.corr_thresh && a.solver == b.solver &&
              a.pcg_iterations == b.pcg_iterations && a.pcg_tol == b.pcg_tol && a.integrate == b.integrate &&
              a.extract_mesh == b.extract_mesh && a.node_capacity == b.node_capacity &&
              a.mesh_capacity == b.mesh_capacity && a.triangle_capacity == b.triangle_capacity &&
              a.precision == b.precision && a.warp_mesh == b.warp_mesh && a.blend == b.blend;
    const afx_camera_distortion &da = a.distortion, &db = b.distortion;
    eq = eq && da.is_distorted == db.is_distorted;
    if (da.is_distorted)  // the coefficients matter only to a distorted camera
        eq = eq && da.k1 == db.k1 && da.k2 == db.k2 && da.k3 == db.k3 && da.k4 == db.k4 && da.k5 == db.k5 &&
             da.k6 == db.k6 && da.codx == db.codx && da.cody == db.cody && da.p1 == db.p1 && da.p2 == db.p2;
    for (int i = 0; i < 9; ++i) eq = eq && a.K[i] == b.K[i];
    for (int i = 0; i < 3; ++i) eq = eq && a.dims[i] == b.dims[i] && a.volume_size[i] == b.volume_size[i];
    return eq;
}

double ms_since(Clock::time_point t0) {
    return std::chrono::duration<double, std::milli>(Clock::now() - t0).count();
}

void free_session(Session* s) {
    if (!s) return;
    if (s->st) cudaStreamSynchronize(s->st);
    for (Slot& sl : s->slots) {
        if (sl.staging) cudaFreeHost(sl.staging);
        if (sl.stats) cudaFreeHost(sl.stats);
        if (sl.done) cudaEventDestroy(sl.done);
    }
    if (s->f) afx_fusion_destroy(s->f);
    if (s->st) cudaStreamDestroy(s->st);
    delete s;
}

}  // namespace

struct afx_server {
    size_t budget = 0, used = 0, idle_bytes = 0;  // used: open sessions; idle_bytes: kept for reuse
    int max_sessions = 0;
    int next_id = 1;
    long denied = 0;
    std::map<int, Session*> sessions;
    std::vector<Session*> idle;  // closed sessions, oldest first
    afx_server_counters c{};
    std::mutex mu;

    // A closed session with nothing in flight leaves the open set and waits for reuse.
    void retire(std::map<int, Session*>::iterator it) {
        Session* x = it->second;
        sessions.erase(it);
        used -= x->bytes;
        idle.push_back(x);
        idle_bytes += x->bytes;
    }
};

extern "C" {

int afx_server_create(size_t memory_budget_bytes, int max_sessions, afx_server** out) {
    if (!out || max_sessions < 1) return AFX_ERR_INVALID_ARGUMENT;
    afx_server* s = new (std::nothrow) afx_server();
    if (!s) return AFX_ERR_NO_MEMORY;
    s->budget = memory_budget_bytes;
    s->max_sessions = max_sessions;
    *out = s;
    return AFX_OK;
}

int afx_server_destroy(afx_server* s) {
    if (!s) return AFX_ERR_INVALID_ARGUMENT;
    for (auto& kv : s->sessions) free_session(kv.second);
    for (Session* x : s->idle) free_session(x);
    delete s;
    return AFX_OK;
}

int afx_server_open(afx_server* s, const afx_fusion_params* params, int* session_id) {
    if (!s || !params || !session_id) return AFX_ERR_INVALID_ARGUMENT;
    const size_t need = afx_fusion_memory_bytes(params);
    if (need == 0) return AFX_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lock(s->mu);
    const Clock::time_point t0 = Clock::now();
    if ((int)s->sessions.size() >= s->max_sessions) {
        ++s->denied;
        return AFX_ERR_NO_MEMORY;
    }
    // an idle session with the same parameters: reset it and hand it out again
    for (size_t i = 0; i < s->idle.size(); ++i) {
        Session* x = s->idle[i];
        if (!params_equal(x->params, *params)) continue;
        const int rc = afx_fusion_reset(x->f, x->st);
        if (rc) return rc;
        s->idle.erase(s->idle.begin() + (long)i);
        s->idle_bytes -= x->bytes;
        x->closing = false;
        x->head = x->count = 0;
        x->id = s->next_id++;
        s->used += x->bytes;
        s->sessions[x->id] = x;
        *session_id = x->id;
        ++s->c.opens_reused;
        s->c.open_ms += ms_since(t0);
        return AFX_OK;
    }
    // room for a new one: free idle sessions, oldest first
    while (!s->idle.empty() && s->used + s->idle_bytes + need > s->budget) {
        Session* v = s->idle.front();
        s->idle.erase(s->idle.begin());
        s->idle_bytes -= v->bytes;
        free_session(v);
        ++s->c.evictions;
    }
    if (s->used + need > s->budget) {
        ++s->denied;
        return AFX_ERR_NO_MEMORY;
    }
    Session* x = new (std::nothrow) Session();
    if (!x) return AFX_ERR_NO_MEMORY;
    x->pixels = (long)params->width * params->height;
    x->params = *params;
    int rc = afx_fusion_create(params, &x->f);
    if (rc) {
        delete x;
        return rc;
    }
    cudaError_t e = cudaStreamCreateWithFlags(&x->st, cudaStreamNonBlocking);
    for (Slot& sl : x->slots) {
        if (e == cudaSuccess) e = cudaHostAlloc(reinterpret_cast<void**>(&sl.staging), x->pixels * 2, cudaHostAllocDefault);
        if (e == cudaSuccess) e = cudaHostAlloc(reinterpret_cast<void**>(&sl.stats), sizeof(afx_frame_stats),
                                                cudaHostAllocDefault);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming);
    }
    if (e != cudaSuccess) {
        free_session(x);
        return afx::note_cuda_error(e);
    }
    x->bytes = need;
    x->id = s->next_id++;
    s->used += need;
    s->sessions[x->id] = x;
    *session_id = x->id;
    ++s->c.opens_fresh;
    s->c.open_ms += ms_since(t0);
    return AFX_OK;
}

// Closes once the session's frames in flight have finished (at the next poll, or now if idle);
// its memory then returns to the budget.
int afx_server_close(afx_server* s, int session_id) {
    if (!s) return AFX_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lock(s->mu);
    auto it = s->sessions.find(session_id);
    if (it == s->sessions.end()) return AFX_ERR_INVALID_ARGUMENT;
    Session* x = it->second;
    x->closing = true;
    if (x->count == 0) s->retire(it);
    return AFX_OK;
}

// AFX_ERR_CAPACITY: the session already has kSlots frames in flight (poll, then retry).
int afx_server_submit(afx_server* s, int session_id, const uint16_t* depth_mm_host, uint64_t tag) {
    if (!s || !depth_mm_host) return AFX_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lock(s->mu);
    auto it = s->sessions.find(session_id);
    if (it == s->sessions.end() || it->second->closing) return AFX_ERR_INVALID_ARGUMENT;
    Session* x = it->second;
    if (x->count == kSlots) return AFX_ERR_CAPACITY;
    Slot& sl = x->slots[(x->head + x->count) % kSlots];
    sl.t_submit = Clock::now();
    sl.tag = tag;
    std::memcpy(sl.staging, depth_mm_host, (size_t)x->pixels * 2);
    const Clock::time_point t1 = Clock::now();
    int rc = afx_fusion_process_host(x->f, sl.staging, x->st);
    if (rc) return rc;
    rc = afx_fusion_stats_async(x->f, sl.stats, x->st);
    if (rc) return rc;
    const cudaError_t re = cudaEventRecord(sl.done, x->st);
    if (re != cudaSuccess) return afx::note_cuda_error(re);
    ++x->count;
    ++s->c.submits;
    s->c.staging_ms += std::chrono::duration<double, std::milli>(t1 - sl.t_submit).count();
    s->c.enqueue_ms += ms_since(t1);
    return AFX_OK;
}

int afx_server_poll(afx_server* s, afx_server_result* out, int max_results, int* n_results) {
    if (!s || !n_results || (max_results > 0 && !out)) return AFX_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lock(s->mu);
    int n = 0;
    const Clock::time_point now = Clock::now();
    ++s->c.polls;
    for (auto it = s->sessions.begin(); it != s->sessions.end();) {
        Session* x = it->second;
        while (x->count > 0 && n < max_results) {
            Slot& sl = x->slots[x->head];
            const cudaError_t q = cudaEventQuery(sl.done);
            if (q == cudaErrorNotReady) break;
            if (q != cudaSuccess) return afx::note_cuda_error(q);
            afx_server_result& r = out[n++];
            r.session_id = x->id;
            r.tag = sl.tag;
            r.latency_ms = std::chrono::duration<double, std::milli>(now - sl.t_submit).count();
            r.stats = *sl.stats;
            x->head = (x->head + 1) % kSlots;
            --x->count;
        }
        if (x->closing && x->count == 0) {
            s->retire(it++);
        } else {
            ++it;
        }
    }
    *n_results = n;
    s->c.results += n;
    s->c.poll_ms += ms_since(now);
    return AFX_OK;
}

// The session handle, e.g. to read its volume or graph (valid until the session is closed).
afx_fusion* afx_server_session(afx_server* s, int session_id) {
    if (!s) return nullptr;
    std::lock_guard<std::mutex> lock(s->mu);
    auto it = s->sessions.find(session_id);
    return it == s->sessions.end() ? nullptr : it->second->f;
}

int afx_server_usage(afx_server* s, size_t* used_bytes, int* sessions, long* denied) {
    if (!s) return AFX_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lock(s->mu);
    if (used_bytes) *used_bytes = s->used;
    if (sessions) *sessions = (int)s->sessions.size();
    if (denied) *denied = s->denied;
    return AFX_OK;
}

int afx_server_get_counters(afx_server* s, afx_server_counters* out) {
    if (!s || !out) return AFX_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lock(s->mu);
    *out = s->c;
    out->idle_sessions = (int)s->idle.size();
    out->idle_bytes = s->idle_bytes;
    return AFX_OK;
}

}  // extern "C"
