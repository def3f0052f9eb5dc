/*
 * vf_oracle.h -- CPU oracle for the VolumeFusion non-rigid depth-fusion hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is a plain-C++ restatement of the
 * reference algorithm (vakokako/VolumeFusion, its src/ .cu and .cpp files) used by the
 * parity tests, by __graft_entry__.smoke() and by bench.py's CPU baseline leg as the
 * checker.  The product (volumefusion_gb300, libafx.so) never links or calls it.
 *
 * Floating-point semantics: every stage evaluates the same IEEE-754 binary32
 * operations, in the same order, as the reference's Eigen expressions (measured
 * against the vendored Eigen 3.3.90: 3-term sums/dots are a0+(a1+a2), Mat4*[p;1]
 * rows are ((a0+a1)+a2)+a3), with no fused multiply-add (-ffp-contract=off).  Where
 * the reference calls exp() the oracle calls vfo_expf (Cody-Waite reduction plus a
 * degree-7 Taylor polynomial), which the CUDA library evaluates identically.
 *
 * Layouts follow the reference: Vec3f = 3 packed floats, Mat3f/Mat4f column-major,
 * per-point KNN as K contiguous slots, voxel index z*X*Y + y*X + x.
 */
#ifndef VF_ORACLE_H
#define VF_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define VFO_INVALID_IDX 0xFFFFFFFFu

/* VFO_REAL is float in liboracle.so (the binary32 restatement) and double in liboracle64.so (the
 * same algorithm evaluated in binary64: the FP64 oracle the precision form's error is stated
 * against).  vfo_params and vfo_expf / vfo_round_half stay binary32 in both. */
#ifndef VFO_REAL
#define VFO_REAL float
#endif

float vfo_expf(float x);
int vfo_f2i_rz(VFO_REAL x);

/* OpenMP threads of the oracle's parallel loops (n < 1: one), and the current count.  A launcher
 * may have set OMP_NUM_THREADS for its processes; a caller that wants every host thread sets it. */
void vfo_set_threads(int n);
int vfo_threads(void);

/* ---- frame preparation (src/VertexManipulation.cu, src/BilateralFilter.cu) ---- */
void vfo_depth_from_mm(const uint16_t* mm, long n, VFO_REAL* out);
void vfo_filter_depth(VFO_REAL* depth, long n, VFO_REAL threshold);
void vfo_bilateral(VFO_REAL* out, const VFO_REAL* in, int height, int width, int r, double sigma_i, double sigma_s, VFO_REAL thr);
void vfo_depth_to_mesh(VFO_REAL* mesh, const VFO_REAL* depth, int width, int height, const VFO_REAL K[9]);
void vfo_normals(VFO_REAL* normals, const VFO_REAL* vertices, int height, int width, VFO_REAL angle_lo, VFO_REAL angle_hi);
void vfo_remove_without_normals(const VFO_REAL* normals, VFO_REAL* vertices, VFO_REAL* depth, int height, int width);
void vfo_centroid(const VFO_REAL* vertices, long n, VFO_REAL out[3]);
void vfo_frame_prep(const uint16_t* mm, int width, int height, const VFO_REAL K[9], VFO_REAL depth_threshold, int bilateral,
                    int r, double sigma_i, double sigma_s, VFO_REAL thr, VFO_REAL angle_lo, VFO_REAL angle_hi,
                    VFO_REAL* depth, VFO_REAL* vertices, VFO_REAL* normals, VFO_REAL centroid[3]);

/* ---- TSDF integration (src/TSDFIntegration.cu) ----
 * half != 0: the precision form's storage -- each updated value is rounded to the nearest binary16
 * (ties to even) as it is stored; values read are then always binary16 values. */
float vfo_round_half(float x);
void vfo_integrate_rigid(VFO_REAL* tsdf, VFO_REAL* weights, const VFO_REAL* depth, int width, int height, VFO_REAL delta,
                         const int dims[3], const VFO_REAL voxel_size[3], const VFO_REAL volume_size[3], const VFO_REAL R[9],
                         const VFO_REAL t[3], const VFO_REAL K[9], int half);

/* ---- marching cubes (src/MarchingCubes.cu / .cpp) ---- */
long vfo_mc_pointcloud(const VFO_REAL* tsdf, const VFO_REAL* weights, const int dims[3], const VFO_REAL voxel_size[3],
                       const VFO_REAL volume_size[3], VFO_REAL iso, VFO_REAL* out, long cap);
long vfo_sort_unique_vec3(VFO_REAL* pts, long n);
long vfo_mc_full(const VFO_REAL* tsdf, const VFO_REAL* weights, const int dims[3], const VFO_REAL voxel_size[3],
                 const VFO_REAL volume_size[3], VFO_REAL iso, VFO_REAL* verts, long vcap, int* faces, long fcap, long* nfaces);
void vfo_translate(VFO_REAL* pts, long n, const VFO_REAL t[3]);
void vfo_transform_points(VFO_REAL* pts, long n, const VFO_REAL T[16]);

/* ---- motion graph (src/GraphBuilder.cpp, src/MotionGraph.cpp, include/af/GraphBuilder.h) ---- */
int vfo_build_graph(VFO_REAL* nodes, VFO_REAL* radii, VFO_REAL* transforms, int n_nodes, int cap, const VFO_REAL* mesh, long m,
                    int knn, VFO_REAL radius);
void vfo_knn(const VFO_REAL* nodes, int n_nodes, const VFO_REAL* pts, long m, int k, int exclude_closest, uint32_t* idx,
             VFO_REAL* dist);
void vfo_filter_disconnected(uint32_t* idx, VFO_REAL* dist, int n_nodes, int k, const VFO_REAL* radii);
void vfo_warp_weights(VFO_REAL* w, const VFO_REAL* radii, const uint32_t* idx, const VFO_REAL* dist, long m, int k, int n_nodes);
void vfo_warp(VFO_REAL* out, const VFO_REAL* pts, long m, const VFO_REAL* transforms, const uint32_t* idx, const VFO_REAL* w, int k);
/* The same with dual-quaternion blending (Kavan et al. 2007; the session option blend = 1). */
void vfo_warp_dqb(VFO_REAL* out, const VFO_REAL* pts, long m, const VFO_REAL* transforms, const uint32_t* idx, const VFO_REAL* w, int k);

/* ---- projective correspondences (src/ComputeCorrespondence.cu) ---- */
long vfo_correspondences(int* corr, long cap, const VFO_REAL* warped, long m, const VFO_REAL K[9], const VFO_REAL* depth,
                         int rows, int cols, const VFO_REAL* frame_mesh, VFO_REAL thr);

/* ---- Gauss-Newton (src/MotionOptimization.cu, src/VolumeFusion.cu:454-691) ---- */
void vfo_residual_depth(VFO_REAL* r, const int* corr, long c, const VFO_REAL* warped, const VFO_REAL* frame_mesh,
                        const VFO_REAL* normals, VFO_REAL lambda);
void vfo_residual_reg(VFO_REAL* r, const VFO_REAL* nodes, const VFO_REAL* transforms, int n, const uint32_t* gidx, int kreg,
                      VFO_REAL lambda);
double vfo_energy(const VFO_REAL* r, long n);
int vfo_assemble(double* jtj_dense, VFO_REAL* jtj_blocks, VFO_REAL* jtr, const int* corr, long c, const VFO_REAL* canon,
                 const uint32_t* midx, const VFO_REAL* mw, int k, const VFO_REAL* normals, VFO_REAL lambda_d, const VFO_REAL* nodes,
                 int n, const uint32_t* gidx, int kreg, VFO_REAL lambda_r, const VFO_REAL* r_depth, const VFO_REAL* r_reg);
int vfo_solve_dense(const double* A, const VFO_REAL* b, int dim, double* x);
int vfo_pcg(const double* A, const VFO_REAL* b, int n_nodes, int iters, double tol, double* x, int* iters_done);
void vfo_update_transforms(VFO_REAL* transforms, const VFO_REAL* update, int n);

/* ---- voxel warp + warped integration (src/TSDFWarp.cu, src/TSDFIntegration.cu) ---- */
void vfo_tsdf_knn(uint32_t* kidx, VFO_REAL* kdist, int* kcount, const VFO_REAL* nodes, const VFO_REAL* radii, int n,
                  const VFO_REAL voxel_size[3], const VFO_REAL volume_size[3], const int dims[3], const int per_node[3], int k);
void vfo_tsdf_weights(VFO_REAL* kw, const VFO_REAL* radii, const uint32_t* kidx, const VFO_REAL* kdist, const int* kcount,
                      long s, int k);
void vfo_tsdf_vertices(VFO_REAL* verts, const VFO_REAL voxel_size[3], const VFO_REAL volume_size[3], const int dims[3]);
void vfo_warp_tsdf(VFO_REAL* verts, const VFO_REAL* transforms, const uint32_t* kidx, const VFO_REAL* kw, const int* kcount,
                   long s, int k);
void vfo_count_collisions(int* counts, const VFO_REAL* verts, const int* kcount, const VFO_REAL voxel_size[3],
                          const VFO_REAL volume_size[3], const int dims[3], const VFO_REAL Rinv[9], const VFO_REAL t[3]);
void vfo_integrate_warped(VFO_REAL* tsdf, VFO_REAL* weights, const VFO_REAL* verts, const int* collisions, const int* kcount,
                          const VFO_REAL* depth, int width, int height, VFO_REAL delta, const VFO_REAL voxel_size[3],
                          const VFO_REAL volume_size[3], const int dims[3], const VFO_REAL Rinv[9], const VFO_REAL t[3],
                          const VFO_REAL K[9], int half);

/* ---- depth ingest: the reference's OpenCV undistortions and its Brown-Conrady unprojection ----
 * vfo_undistort_map: cv::undistort's fixed-point map (mode 0, stripes of max(1, 4096 / W) rows) or
 *   cv::initUndistortRectifyMap's float map rounded for INTER_NEAREST (mode 1); 2 words per pixel:
 *   (int16 sx | int16 sy << 16, sub-pixel index fy * 32 + fx).  K column-major (fx, fy, cx, cy, K(2,2)
 *   used), k_cv = k1 k2 p1 p2 k3 k4 k5 k6.
 * vfo_undistort_depth: cv::remap through that map, zero border.
 * vfo_xy_lookup_table / vfo_bc_unproject / vfo_bc_project: src/CameraCalibration.cpp with
 *   intr = {cx, cy, fx, fy} (af::CameraIntrinsics) and dist = {k1..k6, codx, cody, p1, p2}. */
void vfo_undistort_map(uint32_t* map, int width, int height, const float K[9], const float k_cv[8], int mode);
void vfo_undistort_depth(VFO_REAL* dst, const VFO_REAL* src, int width, int height, const uint32_t* map, int mode);
void vfo_xy_lookup_table(float* table, int width, int height, const float intr[4], const float dist[10]);
void vfo_bc_unproject(float* points, int* valid, const float* pixels, const float* depths, long n, const float intr[4],
                      const float dist[10]);
void vfo_bc_project(float* pixels, int* valid, const float* points, long n, const float intr[4], const float dist[10]);
/* vfo_frame_prep with the frame's metres sampled through a mode-0 undistortion map before the filter. */
void vfo_frame_prep_undistorted(const uint16_t* mm, int width, int height, const VFO_REAL K[9], VFO_REAL depth_threshold,
                                int bilateral, int r, double sigma_i, double sigma_s, VFO_REAL thr, VFO_REAL angle_lo,
                                VFO_REAL angle_hi, const uint32_t* map, VFO_REAL* depth, VFO_REAL* vertices,
                                VFO_REAL* normals, VFO_REAL centroid[3]);

/* ---- whole-frame driver mirroring af::runVolumeFusion's per-frame loop (src/VolumeFusion.cu:343-769) ---- */
typedef struct vfo_params {
    int width, height;
    float K[9];
    int dims[3];
    float volume_size[3];
    float delta;
    float depth_threshold;
    int bilateral, bilateral_r;
    float sigma_i, sigma_s, bilateral_thr;
    float angle_lo, angle_hi;
    float graph_radius;
    int knn, kreg;
    int update_graph;
    int icp_iterations, gn_iterations;
    float lambda_depth, lambda_reg, energy_min_step, corr_thresh;
    int solver;       /* 0 = dense FP64 direct solve, 1 = block-Jacobi PCG */
    int pcg_iterations;
    double pcg_tol;
    int integrate;
    int node_cap;
    long mesh_cap;
    int precision;    /* 0 = FP32 volume, 1 = FP16 values + integer weights (the precision form) */
    int blend;        /* 0 = linear blend (the reference's), 1 = dual-quaternion blend */
    int distorted;    /* undistort every frame as af::loadProcessFrame does (cv::undistort, linear) */
    float dist_cv[8]; /* k1 k2 p1 p2 k3 k4 k5 k6 */
} vfo_params;

typedef struct vfo_fusion vfo_fusion;
vfo_fusion* vfo_fusion_create(const vfo_params* p);
void vfo_fusion_destroy(vfo_fusion* f);
int vfo_fusion_process(vfo_fusion* f, const uint16_t* depth_mm);
int vfo_fusion_num_nodes(const vfo_fusion* f);
long vfo_fusion_mesh_size(const vfo_fusion* f);
long vfo_fusion_num_corr(const vfo_fusion* f);
int vfo_fusion_gn_done(const vfo_fusion* f);
double vfo_fusion_energy(const vfo_fusion* f);
const VFO_REAL* vfo_fusion_tsdf(const vfo_fusion* f);
const VFO_REAL* vfo_fusion_weights(const vfo_fusion* f);
const VFO_REAL* vfo_fusion_nodes(const vfo_fusion* f);
const VFO_REAL* vfo_fusion_transforms(const vfo_fusion* f);
const VFO_REAL* vfo_fusion_centroid(const vfo_fusion* f);
const VFO_REAL* vfo_fusion_mesh(const vfo_fusion* f);
/* Replace the committed node transforms (used to feed a GPU solution back for stage-wise parity). */
void vfo_fusion_set_transforms(vfo_fusion* f, const VFO_REAL* transforms, int n);
/* Replace the volume (stage-wise parity: continue from the GPU's volume). */
void vfo_fusion_set_tsdf(vfo_fusion* f, const VFO_REAL* tsdf, const VFO_REAL* weights);

#ifdef __cplusplus
}
#endif
#endif
