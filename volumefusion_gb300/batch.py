"""Batched form: one frame of every session of a batch in one graph launch (afx_batch_* in the
C ABI).  Sessions keep their own state, and their results are the ones they produce alone."""
import ctypes as C

import torch

from ._lib import FrameStats, check, lib


class Batch:
    def __init__(self, sessions):
        """sessions: FusionSession objects (the batch does not own them)."""
        self.sessions = list(sessions)
        arr = (C.c_void_p * len(self.sessions))(*[s.h.value for s in self.sessions])
        h = C.c_void_p()
        check(lib().afx_batch_create(arr, len(self.sessions), C.byref(h)), "afx_batch_create")
        self.h = h
        self._ptrs = (C.c_void_p * len(self.sessions))()
        self._stats = (FrameStats * len(self.sessions))()

    def close(self):
        if getattr(self, "h", None):
            lib().afx_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def process(self, frames, stream=None):
        """frames[i]: session i's frame as a uint16/int16 CUDA tensor (H, W) or a pinned CPU tensor."""
        assert len(frames) == len(self.sessions)
        for i, f in enumerate(frames):
            assert f.is_contiguous() and f.element_size() == 2 and (f.is_cuda or f.is_pinned())
            self._ptrs[i] = f.data_ptr()
        s = stream if stream is not None else torch.cuda.current_stream()
        check(lib().afx_batch_process(self.h, self._ptrs, C.c_void_p(s.cuda_stream)), "afx_batch_process")

    def stats(self, stream=None):
        """Statistics of the last frames (synchronises the stream)."""
        s = stream if stream is not None else torch.cuda.current_stream()
        s.synchronize()
        check(lib().afx_batch_stats(self.h, C.cast(self._stats, C.c_void_p), len(self.sessions)), "afx_batch_stats")
        return [{f[0]: getattr(x, f[0]) for f in FrameStats._fields_} for x in self._stats]

    def graph_launches(self):
        return lib().afx_batch_graph_launches(self.h)


__all__ = ["Batch"]
