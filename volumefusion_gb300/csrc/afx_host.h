// afx_host.h -- host-side one-time set-up, thread-safe and per CUDA context.
//
// Function attributes (the dynamic shared-memory opt-in, non-portable cluster sizes) and the
// contents of __constant__ tables belong to a CUDA context: a second device, or the context a
// device gets after a reset, starts without them.  Set-up that must precede the first launch
// therefore runs once per (device, context), under a lock, so that host threads driving
// different sessions concurrently never see a half-done set-up.
#pragma once

#include <mutex>

#include <cuda_runtime.h>

#include "afx_common.cuh"

namespace afx {

constexpr int kMaxDevices = 64;

// Identifier of the calling thread's current CUDA context, unique for the life of the process
// (a context created after a device reset gets a new one); 0 when there is no context yet or
// the driver cannot say.
unsigned long long current_context_id();

// Record of a set-up done per device context.
struct ContextOnce {
    std::mutex mu;
    unsigned long long ctx[kMaxDevices] = {};  // context the set-up last succeeded in (0: never)
};

// Runs fn() -- an afx status-returning set-up -- unless it has already succeeded in the current
// context of the current device; concurrent callers wait for the one running it.  Where the
// driver gives no context identifier the set-up runs once per device.  Later calls cost a lock
// and two driver queries and launch nothing, so they are safe inside a stream capture.
template <class F>
int once_per_context(ContextOnce& o, F&& fn) {
    int dev = 0;
    const cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return note_cuda_error(e);
    if (dev < 0 || dev >= kMaxDevices) return AFX_ERR_UNSUPPORTED;
    unsigned long long id = current_context_id();
    if (id == 0) id = ~0ull;
    std::lock_guard<std::mutex> lock(o.mu);
    if (o.ctx[dev] == id) return AFX_OK;
    const int rc = fn(dev);
    if (rc == AFX_OK) {
        const unsigned long long now = current_context_id();  // the set-up may have created the context
        o.ctx[dev] = now ? now : ~0ull;
    }
    return rc;
}

}  // namespace afx
