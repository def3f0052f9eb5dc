// afx_voxel.h -- brick-sparse voxel support / warp / integration shared with the session driver.
#pragma once

#include "afx_internal.h"

namespace afx {

constexpr int kBrick = 8;
constexpr int kBrickVox = kBrick * kBrick * kBrick;
constexpr int kMaxBrickNodes = 192;  // candidate nodes per brick held in shared memory
constexpr int kMaxK = 8;

struct NodeCube {
    int lo[3], hi[3];  // inclusive voxel range of the node's support cube, clipped to the volume
};

struct BrickGrid {
    int nb[3];  // bricks per axis
    long n;
};

inline BrickGrid make_bricks(const Volume& v) {
    BrickGrid g;
    for (int c = 0; c < 3; ++c) g.nb[c] = (v.dims[c] + kBrick - 1) / kBrick;
    g.n = (long)g.nb[0] * g.nb[1] * g.nb[2];
    return g;
}

struct SupportArgs {
    Volume vol;
    BrickGrid bg;
    int per[3];
    const float* nodes;  // node positions already translated by -centroid (as the reference does)
    const float* radii;
    const int* n_nodes;
    int n_max;
    unsigned* brick_count;   // [bg.n]
    unsigned* brick_offset;  // [bg.n + 1]
    unsigned* brick_cursor;  // [bg.n]
    unsigned* brick_nodes;   // [pair capacity]
    long pair_capacity;
    int* error;
};

// Per-voxel output of the support pass, compact per active brick (slot * 512 + local).
struct WarpedVoxel {
    float p[3];       // warped voxel centre (camera space)
    int target;       // linear index of the voxel the warped centre falls into, -1 if outside
};

struct WarpArgs {
    Volume vol;
    BrickGrid bg;
    int k;
    const float* nodes_t;     // translated node positions
    const float* radii;
    const float* transforms;  // committed node transforms (column-major 4x4)
    const unsigned* brick_offset;
    const unsigned* brick_count;
    const unsigned* brick_nodes;
    const unsigned* active;
    const unsigned* n_active;
    int per[3];
    const float* centroid_dev;  // frame-0 centroid (volume translation), device
    float Rinv[9];
    int blend;                  // AFX_BLEND_LBS or AFX_BLEND_DQB
    // outputs: either compact (session) or dense per-voxel arrays (API)
    WarpedVoxel* out;          // [n_active * 512] or null
    unsigned char* out_count;  // [n_active * 512] or null
    unsigned* coll;            // collision words (epoch << 8 | count), [S] or null
    const unsigned* epoch_dev;
    uint32_t* dense_idx;       // [S*k] or null
    float* dense_dist;
    int* dense_count;
    int* error;
};

struct WarpedIntegrateArgs {
    Volume vol;
    BrickGrid bg;
    const unsigned* active;
    const unsigned* n_active;
    const WarpedVoxel* in;
    const unsigned char* in_count;
    const unsigned* coll;
    const unsigned* epoch_dev;
    void* tsdf;     // voxel storage of format fmt (kVoxF32 / kVoxF16)
    void* weights;
    int fmt;
    const float* depth;
    int W, H;
    float delta;
    Intrinsics K;
    unsigned char* occ;  // brick occupancy (brick index = active brick id), or null
};

// Workspace layout for the support gather.
struct SupportWorkspace {
    unsigned* brick_count;
    unsigned* brick_offset;
    unsigned* brick_cursor;
    unsigned* brick_nodes;
    unsigned* active;
    unsigned* n_active;
    void* scan_tmp;
    size_t scan_tmp_bytes;
    long pair_capacity;
};

size_t support_workspace_size(const Volume& vol, int n_nodes_max, const int* per);
bool carve_support(void* ws, size_t bytes, const Volume& vol, int n_nodes_max, const int* per, SupportWorkspace* s);
int build_support(const SupportWorkspace& s, const Volume& vol, const int* per, const float* nodes_t,
                  const float* radii, const int* n_nodes, int n_max, int* error, cudaStream_t st);
int launch_brick_warp(const WarpArgs& a, long max_active, cudaStream_t st);
int launch_brick_integrate(const WarpedIntegrateArgs& a, long max_active, cudaStream_t st);
long brick_count_total(const Volume& vol);

}  // namespace afx
