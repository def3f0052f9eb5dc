"""Serving many depth streams on one GPU (afx_server_* in the C ABI).

Sessions are admitted while their device memory fits the server's budget; each has its own CUDA
stream, so frames of different sessions overlap on the device, and frames of one session run in
order.  submit() returns at once; poll() hands back finished frames with their latency.  A
closed session is kept for reuse by a later open with the same configuration.
"""
import ctypes as C

import numpy as np

from ._lib import AfxError, FrameStats, ServerCounters, ServerResult, check, lib
from .fusion import params_from_config

AFX_ERR_CAPACITY = 2
AFX_ERR_NO_MEMORY = 8


def session_bytes(cfg, extract_mesh=True):
    """Device bytes a session with this configuration allocates (its admission cost)."""
    p = params_from_config(cfg, extract_mesh=extract_mesh)
    return int(lib().afx_fusion_memory_bytes(C.byref(p)))


class Server:
    def __init__(self, memory_budget_bytes, max_sessions=256):
        h = C.c_void_p()
        check(lib().afx_server_create(int(memory_budget_bytes), int(max_sessions), C.byref(h)), "afx_server_create")
        self.h = h
        self._buf = (ServerResult * 1024)()

    def close(self):
        if getattr(self, "h", None):
            lib().afx_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def open(self, cfg, extract_mesh=True):
        """Session id, or None when the memory budget does not admit it now."""
        p = params_from_config(cfg, extract_mesh=extract_mesh)
        sid = C.c_int(0)
        st = lib().afx_server_open(self.h, C.byref(p), C.byref(sid))
        if st == AFX_ERR_NO_MEMORY:
            return None
        check(st, "afx_server_open")
        return sid.value

    def close_session(self, sid):
        check(lib().afx_server_close(self.h, int(sid)), "afx_server_close")

    def submit(self, sid, depth_mm, tag=0):
        """False when the session already has its maximum of frames in flight."""
        arr = np.ascontiguousarray(depth_mm, dtype=np.uint16)
        st = lib().afx_server_submit(self.h, int(sid), arr.ctypes.data_as(C.c_void_p), C.c_uint64(int(tag)))
        if st == AFX_ERR_CAPACITY:
            return False
        check(st, "afx_server_submit")
        return True

    def poll(self):
        """Finished frames: list of (session_id, tag, latency_ms, stats dict)."""
        n = C.c_int(0)
        check(lib().afx_server_poll(self.h, self._buf, len(self._buf), C.byref(n)), "afx_server_poll")
        out = []
        for i in range(n.value):
            r = self._buf[i]
            out.append((r.session_id, r.tag, r.latency_ms, {f[0]: getattr(r.stats, f[0]) for f in FrameStats._fields_}))
        return out

    def usage(self):
        used, n, denied = C.c_size_t(0), C.c_int(0), C.c_long(0)
        check(lib().afx_server_usage(self.h, C.byref(used), C.byref(n), C.byref(denied)), "afx_server_usage")
        return {"used_bytes": used.value, "sessions": n.value, "denied": denied.value}

    def counters(self):
        """Reuse of closed sessions and the host time spent inside the server's calls."""
        c = ServerCounters()
        check(lib().afx_server_get_counters(self.h, C.byref(c)), "afx_server_get_counters")
        return {f[0]: getattr(c, f[0]) for f in ServerCounters._fields_}

    def session_handle(self, sid):
        return lib().afx_server_session(self.h, int(sid))


__all__ = ["Server", "session_bytes", "AfxError"]
