// afx_internal.h -- functions shared between the library's translation units.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "afx_common.cuh"

namespace afx {

// Voxel storage formats (afx_store.cuh): the reference's FP32 values + FP32 weights, or the
// precision form's FP16 values + uint16 weights.
enum { kVoxF32 = 0, kVoxF16 = 1 };
inline size_t vox_bytes(int fmt) { return fmt == kVoxF16 ? 2 : 4; }  // per array and voxel

// ---- scans (afx_scan.cu) ----
// Exclusive prefix sum of n unsigned values; out may alias in.  If total != nullptr the
// sum of all n values is written there (device).  Workspace: scan_workspace_size(n).
size_t scan_workspace_size(long n);
int scan_exclusive(const unsigned* in, unsigned* out, long n, unsigned* total, void* ws, cudaStream_t st);
// Same, with the element count read from the device (n = min(*count, n_max)).
int scan_exclusive_dev(const unsigned* in, unsigned* out, const unsigned* count, long n_max, unsigned* total, void* ws,
                       cudaStream_t st);

// ---- prep (afx_prep.cu) ----
// undistort_map: a cv::undistort map of the frame (afx_undistort_map, AFX_UNDISTORT_LINEAR) to sample the
// metres through before the filter, or null.
int frame_prep_impl(const uint16_t* mm, int width, int height, const afx_prep_params* p, float* depth, float* vertices,
                    float* normals, float* centroid, unsigned long long* acc, int* error, cudaStream_t st,
                    const uint32_t* undistort_map = nullptr);
// afx_undistort_map / afx_undistort_depth (afx_undistort.cu)
int undistort_map_impl(uint32_t* map, int width, int height, const float K[9], const afx_camera_distortion* d, int mode,
                       cudaStream_t st);
int undistort_apply_impl(float* dst, const float* src, int width, int height, const uint32_t* map, int mode,
                         cudaStream_t st);

// ---- integration (afx_integrate.cu) ----
// occ (optional): one byte per 8^3 brick, set to 1 for every brick where a voxel gets a weight
int integrate_rigid_impl(void* tsdf, void* weights, int fmt, const float* depth, int W, int H, float delta,
                         const Volume& vol, const float* R, const float* t, const float* K, cudaStream_t st,
                         const float* t_dev = nullptr, unsigned char* occ = nullptr);
// initialise (-1, 0) + rigid integration in one write-only pass (FP32 volumes, X % 4 == 0, 16-byte
// aligned arrays; AFX_ERR_UNSUPPORTED otherwise)
int integrate_fresh_impl(float* tsdf, float* weights, const float* depth, int W, int H, float delta, const Volume& vol,
                         const float* R, const float* t, const float* K, cudaStream_t st);
void rotation_inverse(const float* R, float* Rinv);

// ---- marching cubes and sorting (afx_mc.cu) ----
size_t sort_unique_workspace_size(long n_max);
int sort_unique_impl(float* pts, unsigned* count, long n_max, void* ws, size_t ws_bytes, cudaStream_t st);
// The same result for a marching-cubes cloud of `vol` (x within the volume), by voxel-column buckets.
size_t sort_unique_volume_workspace_size(long n_max, int nb);
int sort_unique_volume_impl(float* pts, unsigned* count, long n_max, void* ws, size_t ws_bytes, const Volume& vol,
                            cudaStream_t st, int* error = nullptr);
int mc_fused_impl(const void* tsdf, const void* weights, int fmt, const Volume& vol, float iso, float* points,
                  unsigned* point_count, long point_cap, float* verts, unsigned* vert_count, long vert_cap, int* faces,
                  unsigned* face_count, long face_cap, cudaStream_t st, int* error = nullptr, int tile = 0,
                  const unsigned char* occ = nullptr,   // occ: brick occupancy (tiles without an occupied
                                                        // brick hold no active cube and are skipped)
                  unsigned* tile_ws = nullptr);         // mc_tile_ws_words(vol) words: with occ, the
                                                        // persistent tiles walk a list of occupied tiles
size_t mc_tile_ws_words(const Volume& vol);
// marching-cubes tiles (the session's autotuner picks one): TMA bricks of 16, 8 or 32 cubes along z,
// the column march from global memory, or a persistent grid with two stages of bricks 8 or 16 deep
enum { kMcTileTma16 = 0, kMcTileTma8 = 1, kMcTileTma32 = 2, kMcTileColumn = 3, kMcTilePipe8 = 4, kMcTilePipe16 = 5, kMcTilePipe4 = 6,
       kMcTiles = 7 };
int translate_impl(float* pts, const unsigned* count, long n_max, const float* t, cudaStream_t st);
// pts += sign * t_dev (t_dev in device memory); dst may differ from src
int translate_dev_impl(float* dst, const float* src, const unsigned* count, long n_max, const float* t_dev, float sign,
                       cudaStream_t st);

}  // namespace afx

namespace afx {
// ---- graph (afx_graph.cu) ----
size_t build_graph_ws(long mesh_max);
int build_graph_impl(float* nodes, float* radii, float* T, int* n_nodes, int cap, const float* mesh,
                     const unsigned* mesh_count, long mesh_max, float r, void* ws, size_t ws_bytes, int* error,
                     cudaStream_t st);
int knn_impl(uint32_t* idx, float* dist, const float* nodes, const int* n_nodes, int n_max, const float* pts,
             const unsigned* count, long m_max, int k, int excl, cudaStream_t st);
int warp_weights_impl(float* w, const float* radii, const uint32_t* idx, const float* dist, const unsigned* count,
                      long m_max, int k, const int* n_nodes, cudaStream_t st);
// blend: AFX_BLEND_LBS (the reference's linear blend) or AFX_BLEND_DQB (dual quaternions, afx_dqb.cuh)
int warp_impl(float* out, const float* pts, const float* T, const uint32_t* idx, const float* w, const unsigned* count,
              long m_max, int k, cudaStream_t st, int blend = AFX_BLEND_LBS);
size_t corr_ws(long m_max);
int correspondences_impl(int* corr, unsigned* corr_count, long cap, const float* warped, const unsigned* count,
                         long m_max, const float* K, const float* depth, int rows, int cols, const float* frame,
                         float thresh, int* corr_of_vertex, void* ws, size_t ws_bytes, cudaStream_t st);
}  // namespace afx
