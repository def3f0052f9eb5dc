// afx_gn.h -- Gauss-Newton buffers and entry points shared with the session driver.
#pragma once

#include "afx_internal.h"

namespace afx {

constexpr int kMaxNbr = 64;      // neighbours per node in J^T J (both sides of the diagonal)
constexpr int kSegMax = 8192;    // vertices per node list sortable in shared memory
constexpr int kGnWarps = 4;

struct GnState {
    double e_prev;
    double e_last;
    double e_depth, e_reg;
    int done;
    int commit;
    int iters;
    int error;
};

struct GnBuffers {
    // per frame
    unsigned* lcnt;        // [N]
    unsigned* loff;        // [N+1]
    unsigned* lcur;        // [N]
    unsigned* lst;         // [M*K]  vertex*K + slot, per node, ascending
    unsigned* icnt;        // [N] incoming regularisation edges
    unsigned* ioff;        // [N+1]
    unsigned* icur;        // [N]
    unsigned* ilst;        // [N*kreg]  x*kreg + k, per node, ascending
    // per ICP iteration
    int* nbr_cnt;          // [N]
    int* nbr;              // [N*kMaxNbr] sorted neighbour ids
    int* nbr_ref;          // [N*kMaxNbr] block index (owner*kMaxNbr + slot), negative = transpose of -(ref+1)
    float* blocks;         // [N*kMaxNbr*36] upper blocks (a,b), b > a, row-major
    float* diag;           // [N*36]
    float* minv;           // [N*36] inverse diagonal blocks (FP64 Gauss-Jordan, stored FP32)
    float* jrow;           // [M*K*6] depth-row Jacobian block of each node-list entry (per ICP iteration)
    int* jc;               // [M*K]   its correspondence index, -1 if the vertex has none
    // per GN iteration
    float* jtr;            // [N*6]
    float* rdepth;         // [C_max]
    float* rreg;           // [N*kreg*3]
    float* x, *r, *z, *p, *ap;  // PCG vectors [N*6]
    void* scan_ws;
    GnState* state;
};

struct GnArgs {
    // geometry
    const float* mesh;        // canonical vertices (camera space)
    const unsigned* mesh_count;
    long m_max;
    const uint32_t* midx;
    const float* mw;
    int k;
    const float* normals;     // frame normals
    const float* frame;       // frame vertices
    const int* corr;
    const unsigned* corr_count;
    long c_max;
    const int* corr_of_vertex;
    const float* nodes;       // node positions used by the regularisation term
    const int* n_nodes;
    int n_max;
    const uint32_t* gidx;
    int kreg;
    float lam_d, lam_r;
    float min_step;
    int blend;                // AFX_BLEND_LBS or AFX_BLEND_DQB for the re-warp of the canonical vertices
    GnBuffers b;
    int* error;
};

size_t gn_workspace_size(long m_max, int n_max, int k, int kreg);
bool gn_carve(void* ws, size_t bytes, long m_max, int n_max, int k, int kreg, GnBuffers* b);
int gn_frame_setup(const GnArgs& a, cudaStream_t st);
int gn_icp_setup(const GnArgs& a, float* T_pending, const float* T_committed, cudaStream_t st);
int gn_loop(const GnArgs& a, const float* points, float* warped, float* T_committed, float* T_pending, int gn_iters,
            int pcg_iters, double tol, cudaStream_t st);

}  // namespace afx
