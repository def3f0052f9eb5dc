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

float vfo_expf(float x);
int vfo_f2i_rz(float x);

/* ---- frame preparation (src/VertexManipulation.cu, src/BilateralFilter.cu) ---- */
void vfo_depth_from_mm(const uint16_t* mm, long n, float* out);
void vfo_filter_depth(float* depth, long n, float threshold);
void vfo_bilateral(float* out, const float* in, int height, int width, int r, double sigma_i, double sigma_s, float thr);
void vfo_depth_to_mesh(float* mesh, const float* depth, int width, int height, const float K[9]);
void vfo_normals(float* normals, const float* vertices, int height, int width, float angle_lo, float angle_hi);
void vfo_remove_without_normals(const float* normals, float* vertices, float* depth, int height, int width);
void vfo_centroid(const float* vertices, long n, float out[3]);
void vfo_frame_prep(const uint16_t* mm, int width, int height, const float K[9], float depth_threshold, int bilateral,
                    int r, double sigma_i, double sigma_s, float thr, float angle_lo, float angle_hi,
                    float* depth, float* vertices, float* normals, float centroid[3]);

/* ---- TSDF integration (src/TSDFIntegration.cu) ---- */
void vfo_integrate_rigid(float* tsdf, float* weights, const float* depth, int width, int height, float delta,
                         const int dims[3], const float voxel_size[3], const float volume_size[3], const float R[9],
                         const float t[3], const float K[9]);

/* ---- marching cubes (src/MarchingCubes.cu / .cpp) ---- */
long vfo_mc_pointcloud(const float* tsdf, const float* weights, const int dims[3], const float voxel_size[3],
                       const float volume_size[3], float iso, float* out, long cap);
long vfo_sort_unique_vec3(float* pts, long n);
long vfo_mc_full(const float* tsdf, const float* weights, const int dims[3], const float voxel_size[3],
                 const float volume_size[3], float iso, float* verts, long vcap, int* faces, long fcap, long* nfaces);
void vfo_translate(float* pts, long n, const float t[3]);

/* ---- motion graph (src/GraphBuilder.cpp, src/MotionGraph.cpp, include/af/GraphBuilder.h) ---- */
int vfo_build_graph(float* nodes, float* radii, float* transforms, int n_nodes, int cap, const float* mesh, long m,
                    int knn, float radius);
void vfo_knn(const float* nodes, int n_nodes, const float* pts, long m, int k, int exclude_closest, uint32_t* idx,
             float* dist);
void vfo_filter_disconnected(uint32_t* idx, float* dist, int n_nodes, int k, const float* radii);
void vfo_warp_weights(float* w, const float* radii, const uint32_t* idx, const float* dist, long m, int k, int n_nodes);
void vfo_warp(float* out, const float* pts, long m, const float* transforms, const uint32_t* idx, const float* w, int k);

/* ---- projective correspondences (src/ComputeCorrespondence.cu) ---- */
long vfo_correspondences(int* corr, long cap, const float* warped, long m, const float K[9], const float* depth,
                         int rows, int cols, const float* frame_mesh, float thr);

/* ---- Gauss-Newton (src/MotionOptimization.cu, src/VolumeFusion.cu:454-691) ---- */
void vfo_residual_depth(float* r, const int* corr, long c, const float* warped, const float* frame_mesh,
                        const float* normals, float lambda);
void vfo_residual_reg(float* r, const float* nodes, const float* transforms, int n, const uint32_t* gidx, int kreg,
                      float lambda);
double vfo_energy(const float* r, long n);
int vfo_assemble(double* jtj_dense, float* jtj_blocks, float* jtr, const int* corr, long c, const float* canon,
                 const uint32_t* midx, const float* mw, int k, const float* normals, float lambda_d, const float* nodes,
                 int n, const uint32_t* gidx, int kreg, float lambda_r, const float* r_depth, const float* r_reg);
int vfo_solve_dense(const double* A, const float* b, int dim, double* x);
int vfo_pcg(const double* A, const float* b, int n_nodes, int iters, double tol, double* x, int* iters_done);
void vfo_update_transforms(float* transforms, const float* update, int n);

/* ---- voxel warp + warped integration (src/TSDFWarp.cu, src/TSDFIntegration.cu) ---- */
void vfo_tsdf_knn(uint32_t* kidx, float* kdist, int* kcount, const float* nodes, const float* radii, int n,
                  const float voxel_size[3], const float volume_size[3], const int dims[3], const int per_node[3], int k);
void vfo_tsdf_weights(float* kw, const float* radii, const uint32_t* kidx, const float* kdist, const int* kcount,
                      long s, int k);
void vfo_tsdf_vertices(float* verts, const float voxel_size[3], const float volume_size[3], const int dims[3]);
void vfo_warp_tsdf(float* verts, const float* transforms, const uint32_t* kidx, const float* kw, const int* kcount,
                   long s, int k);
void vfo_count_collisions(int* counts, const float* verts, const int* kcount, const float voxel_size[3],
                          const float volume_size[3], const int dims[3], const float Rinv[9], const float t[3]);
void vfo_integrate_warped(float* tsdf, float* weights, const float* verts, const int* collisions, const int* kcount,
                          const float* depth, int width, int height, float delta, const float voxel_size[3],
                          const float volume_size[3], const int dims[3], const float Rinv[9], const float t[3],
                          const float K[9]);

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
const float* vfo_fusion_tsdf(const vfo_fusion* f);
const float* vfo_fusion_weights(const vfo_fusion* f);
const float* vfo_fusion_nodes(const vfo_fusion* f);
const float* vfo_fusion_transforms(const vfo_fusion* f);
const float* vfo_fusion_centroid(const vfo_fusion* f);
const float* vfo_fusion_mesh(const vfo_fusion* f);
/* Replace the committed node transforms (used to feed a GPU solution back for stage-wise parity). */
void vfo_fusion_set_transforms(vfo_fusion* f, const float* transforms, int n);
/* Replace the volume (stage-wise parity: continue from the GPU's volume). */
void vfo_fusion_set_tsdf(vfo_fusion* f, const float* tsdf, const float* weights);

#ifdef __cplusplus
}
#endif
#endif
