"""GB300 (sm_103a) implementation of VolumeFusion's per-frame non-rigid TSDF fusion hot path.

The compute lives in libafx.so (hand-written CUDA, C ABI in include/afx/afx.h).  This
package is the Python host layer: ``af`` mirrors the reference's af:: operator API over
torch CUDA tensors, ``fusion.FusionSession`` runs the whole per-frame loop on the device,
``synth`` renders the seeded synthetic depth scenes and ``configs`` names the workloads.
"""
__all__ = ["af", "fusion", "synth", "configs", "build"]
