/*
 * afx.h -- C ABI of the GB300 (sm_103a) implementation of VolumeFusion's per-frame
 * non-rigid TSDF depth-fusion hot path.
 *
 * Conventions (replacing the reference's af:: free functions and classes):
 *  - Plain pointers and sizes only.  Array arguments are DEVICE pointers unless the
 *    name ends in _host.  Layouts are the reference's: Vec3f = 3 packed floats,
 *    Mat3f / Mat4f = 9 / 16 floats column-major, per-point KNN = K contiguous slots,
 *    Vec2i = 2 ints, voxel index z*X*Y + y*X + x.
 *  - Every call takes an explicit stream (cudaStream_t passed as void*, NULL = legacy
 *    default stream) and is asynchronous unless stated; the reference blocked on
 *    cudaDeviceSynchronize after every launch.
 *  - Every call returns an afx_status; no C++ exception crosses the ABI (the reference
 *    threw std::runtime_error from CUDA_CHECK, src/Helper.cu:7-20).
 *  - Outputs with a data-dependent length take a capacity and a device counter; a
 *    launch that would overflow stores at most `capacity` items, keeps counting, and
 *    the overflow shows as counter > capacity (the reference wrote past the end).
 *  - Calls that need temporary device memory take (workspace, workspace_bytes); the
 *    matching *_workspace_size() returns the bytes needed.
 */
#ifndef AFX_AFX_H
#define AFX_AFX_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum afx_status {
    AFX_OK = 0,
    AFX_ERR_INVALID_ARGUMENT = 1,
    AFX_ERR_CAPACITY = 2,        /* an output or internal capacity was exceeded */
    AFX_ERR_CUDA = 3,            /* a CUDA runtime call failed */
    AFX_ERR_SINGULAR = 4,        /* the Gauss-Newton system has a singular diagonal block */
    AFX_ERR_WORKSPACE = 5,       /* workspace too small */
    AFX_ERR_UNSUPPORTED = 6,     /* input outside what this implementation supports */
    AFX_ERR_TIMEOUT = 7,         /* a bounded device-side wait gave up */
    AFX_ERR_NO_MEMORY = 8,
    AFX_ERR_IO = 9               /* a file could not be opened, read or written */
} afx_status;

#define AFX_INVALID_INDEX 0xFFFFFFFFu
#define AFX_BLEND_LBS 0
#define AFX_BLEND_DQB 1

const char* afx_status_string(int status);
int afx_version(void);
/* Last CUDA error seen by the library on this thread (cudaError_t value), 0 if none. */
int afx_last_cuda_error(void);

/* af::CameraDistortion (include/af/CameraModel.h:21-33), filled from depthDistortion.txt
 * (af::loadCameraDistortion, src/dataset.cpp:44-79: file order k1 k2 p1 p2 k3 k4 k5 k6). */
typedef struct afx_camera_distortion {
    float k1, k2, k3, k4, k5, k6;
    float codx, cody;
    float p1, p2;
    int is_distorted;
} afx_camera_distortion;

/* ------------------------------------------------------------------------------------
 * Depth pre-processing (src/VertexManipulation.cu, src/BilateralFilter.cu)
 * ------------------------------------------------------------------------------------ */

/* uint16 millimetres -> float metres (depth.convertTo(CV_32FC1, 1/1000), src/dataset.cpp:188). */
int afx_depth_from_mm(float* depth, const uint16_t* depth_mm, long n, void* stream);

/* af::runFilterDepthKernel (include/af/VertexManipulation.cuh:11, src/VertexManipulation.cu:17):
 * values > threshold, < 1e-4 or NaN become +inf. */
int afx_filter_depth(float* depth, long n, float threshold, void* stream);
/* The same with the rejected values set to `fill` (runFilterDepthKernel's fillValue argument,
 * include/af/VertexManipulation.cuh:11). */
int afx_filter_depth_fill(float* depth, long n, float threshold, float fill, void* stream);

/* dst[0..n) = value (DeviceTsdf::initDefault, include/af/DeviceTsdf.cuh:23-26: values -1, weights 0). */
int afx_fill_f32(float* dst, long n, float value, void* stream);

/* af::bilateralFilterTextureOpmShared (include/af/BilateralFilter.cuh:8,
 * src/BilateralFilter.cu:180): radius r, range sigma sigma_i (m), spatial sigma
 * sigma_s (px), hard range threshold thr (m).  out and in must not alias. */
int afx_bilateral_filter(float* out, const float* in, int height, int width, int r, double sigma_i, double sigma_s,
                         float thr, void* stream);

/* af::runDepthToMeshKernel (include/af/VertexManipulation.cuh:13, src/VertexManipulation.cu:65). */
int afx_depth_to_mesh(float* vertices, const float* depth, int width, int height, const float K[9], void* stream);

/* af::runDepthVerticesNormalsKernel (include/af/VertexManipulation.cuh:23,
 * src/VertexManipulation.cu:209).  Border pixels get a zero normal (the reference leaves
 * them unwritten). */
int afx_depth_vertices_normals(float* normals, const float* vertices, int height, int width, float excl_angle_lo,
                               float excl_angle_hi, void* stream);

/* af::runRemoveDepthWithoutNormalsKernel (include/af/VertexManipulation.cuh:30, src/VertexManipulation.cu:238). */
int afx_remove_depth_without_normals(const float* normals, float* vertices, float* depth, int height, int width,
                                     void* stream);

typedef struct afx_prep_params {
    float K[9];              /* depth intrinsics, column-major */
    float depth_threshold;   /* settings.depthThreshold */
    int bilateral;           /* settings.bilateralFiltr */
    int bilateral_r;         /* settings.bilateralD (used as the radius) */
    float sigma_i, sigma_s;  /* settings.bilateralSigmaI / SigmaS */
    float bilateral_thr;     /* settings.bilateralThreshold */
    float excl_angle_lo, excl_angle_hi;  /* settings.normExclAngleRange */
} afx_prep_params;

/* af::loadProcessFrame after the image is in memory (src/VolumeFusion.cu:184-220), fused:
 * mm -> metres, filter, bilateral, back-projection, normals, removal of pixels without a
 * normal, and the centroid of the valid vertices (written to centroid[3], device).
 * One kernel (TMA-staged tiles) plus a 1-thread finaliser. */
int afx_frame_prep(const uint16_t* depth_mm, int width, int height, const afx_prep_params* params, float* depth,
                   float* vertices, float* normals, float* centroid, void* stream);

/* ------------------------------------------------------------------------------------
 * TSDF integration (src/TSDFIntegration.cu)
 * ------------------------------------------------------------------------------------ */

/* af::runIntegrateTSDFFromFrameKernel (include/af/TSDFIntegration.cuh:8,
 * src/TSDFIntegration.cu:98); DeviceTsdf::integrate (include/af/DeviceTsdf.cuh:28). */
int afx_integrate_tsdf(float* tsdf, float* weights, const float* depth, int width, int height, float delta,
                       const int dims[3], const float voxel_size[3], const float volume_size[3], const float rotate[9],
                       const float translate[3], const float K[9], void* stream);

/* ------------------------------------------------------------------------------------
 * Voxel warp and warped integration (src/TSDFWarp.cu, src/TSDFIntegration.cu)
 * Dense per-voxel forms with the reference's layouts.  The fused session path uses
 * brick-sparse kernels instead (afx_fusion_*).
 * ------------------------------------------------------------------------------------ */

/* af::runTsdfKNNGraph (include/af/TSDFWarp.h:9, src/TSDFWarp.cu:70).  Slots hold the K
 * nearest supporting nodes ordered by (distance, node index); the reference keeps the
 * first K to arrive, so the two agree where a voxel has at most K supporting nodes.
 * knn_counts need not be zeroed. */
int afx_tsdf_knn(uint32_t* knn_idx, float* knn_dist, int* knn_counts, const float* nodes, const float* radii,
                 int n_nodes, const float voxel_size[3], const float volume_size[3], const int dims[3],
                 const int voxels_per_node[3], int k, void* workspace, size_t workspace_bytes, void* stream);
size_t afx_tsdf_knn_workspace_size(const int dims[3], int n_nodes, const int voxels_per_node[3]);

/* af::runComputeTsdfWarpWeightsKernel (include/af/TSDFWarp.h:18, src/TSDFWarp.cu:118). */
int afx_tsdf_warp_weights(float* knn_weights, const float* radii, const uint32_t* knn_idx, const float* knn_dist,
                          const int* knn_counts, long n_voxels, int k, void* stream);

/* af::runGenerateTsdfVerticesKernel (include/af/TSDFWarp.h:25, src/TSDFWarp.cu:147). */
int afx_tsdf_vertices(float* vertices, const float voxel_size[3], const float volume_size[3], const int dims[3],
                      void* stream);

/* af::runWarpTsdfKernel (include/af/TSDFWarp.h:27, src/TSDFWarp.cu:192). */
int afx_warp_tsdf(float* vertices, const float* transforms, const uint32_t* knn_idx, const float* knn_weights,
                  const int* knn_counts, long n_voxels, int k, void* stream);

/* af::runCountCollisionsPerVoxelKernel (include/af/TSDFIntegration.cuh:49,
 * src/TSDFIntegration.cu:285).  Adds to `counts` (zero it first, as the reference does). */
int afx_count_collisions(int* counts, const float* vertices, const int* knn_counts, const float voxel_size[3],
                         const float volume_size[3], const int dims[3], const float rotate[9], const float translate[3],
                         void* stream);

/* af::runIntegrateWarpedTSDFFromFrameKernel (include/af/TSDFIntegration.cuh:34, src/TSDFIntegration.cu:228). */
int afx_integrate_warped_tsdf(float* tsdf, float* weights, const float* vertices, const int* collisions,
                              const int* knn_counts, const float* depth, int width, int height, float delta,
                              const float voxel_size[3], const float volume_size[3], const int dims[3],
                              const float rotate[9], const float translate[3], const float K[9], void* stream);

/* ------------------------------------------------------------------------------------
 * Marching cubes (src/MarchingCubes.cu) and point-cloud de-duplication
 * ------------------------------------------------------------------------------------ */

/* af::runMarchingCubesMeshKernel (include/af/MarchingCubes.cuh:12, src/MarchingCubes.cu:510):
 * one vertex per cut edge of every non-trivial cube; *count (device, caller-zeroed) receives
 * the number produced.  Output order is unspecified, as in the reference. */
int afx_marching_cubes_points(float* points, unsigned* count, long capacity, const float* tsdf, const float* weights,
                              const int dims[3], const float voxel_size[3], const float volume_size[3], float iso,
                              void* stream);

/* af::runMarchingCubesFullKernel (include/af/MarchingCubes.cuh:21, src/MarchingCubes.cu:683):
 * three vertices and one face per non-degenerate triangle.  Counters are device, caller-zeroed. */
int afx_marching_cubes_mesh(float* vertices, unsigned* vertex_count, long vertex_capacity, int* faces,
                            unsigned* face_count, long face_capacity, const float* tsdf, const float* weights,
                            const int dims[3], const float voxel_size[3], const float volume_size[3], float iso,
                            void* stream);

/* thrust::sort + thrust::unique of Vec3f with the lexicographic operator<
 * (src/VolumeFusion.cu:382-384, include/af/eigen_extension.cuh:15-25).  Sorts points[0..*count)
 * in place and rewrites *count (device) with the number of distinct points.
 * n_max bounds *count. */
int afx_sort_unique_points(float* points, unsigned* count, long n_max, void* workspace, size_t workspace_bytes,
                           void* stream);
size_t afx_sort_unique_points_workspace_size(long n_max);
/* The same sort + unique for a marching-cubes point cloud of a volume (every x within the volume):
 * points are bucketed by voxel column, each column sorted in shared memory, and the unique points
 * compacted in order; a column of more than 8192 points falls back to the general sort on the
 * device.  Results are identical to afx_sort_unique_points. */
size_t afx_sort_unique_volume_points_workspace_size(long n_max, const int dims[3]);
int afx_sort_unique_volume_points(float* points, unsigned* count, long n_max, const int dims[3],
                                  const float voxel_size[3], const float volume_size[3], void* workspace,
                                  size_t workspace_bytes, void* stream);

/* DeviceTsdf::extractPointCloud (include/af/DeviceTsdf.cuh:34-42): marching-cubes points,
 * then sort + unique. */
int afx_extract_point_cloud(float* points, unsigned* count, long capacity, const float* tsdf, const float* weights,
                            const int dims[3], const float voxel_size[3], const float volume_size[3], float iso,
                            void* workspace, size_t workspace_bytes, void* stream);

/* af::runTranslateKernel (include/af/VertexManipulation.cuh:16): points += t for
 * points[0..n) where n = *count if count != NULL else n_max. */
int afx_translate(float* points, const unsigned* count, long n_max, const float t[3], void* stream);

/* ------------------------------------------------------------------------------------
 * Motion graph, KNN, skinning, correspondences
 * (src/GraphBuilder.cpp, include/af/GraphBuilder.h, src/MotionGraph.cpp, src/VertexManipulation.cu,
 *  src/ComputeCorrespondence.cu)
 * ------------------------------------------------------------------------------------ */

/* af::buildGraph (include/af/GraphBuilder.h:12, src/GraphBuilder.cpp:12), on the device.
 * mesh[0..*mesh_count) is the sorted, translated canonical point cloud.  Nodes
 * (positions, radii, transforms) are appended in place; *n_nodes (device) is read and
 * updated.  All existing radii must equal `radius` (the pipeline's case); otherwise
 * AFX_ERR_UNSUPPORTED.  Node selection equals the reference's sequential greedy order. */
int afx_build_graph(float* nodes, float* radii, float* transforms, int* n_nodes, int node_capacity,
                    const float* mesh, const unsigned* mesh_count, long mesh_max, int knn, float radius,
                    void* workspace, size_t workspace_bytes, void* stream);
size_t afx_build_graph_workspace_size(long mesh_max, int node_capacity);

/* af::getKnnData<K> (include/af/GraphBuilder.h:118): the k nearest nodes of each point
 * (exclude_closest drops the nearest one, for node-to-node neighbours), ordered by
 * nanoflann's squared distance, equal distances by node index; distances are sqrt'ed;
 * missing slots hold AFX_INVALID_INDEX / FLT_MAX.  n_points = *count if count != NULL. */
int afx_knn(uint32_t* idx, float* dist, const float* nodes, const int* n_nodes, int n_nodes_max, const float* points,
            const unsigned* count, long n_points_max, int k, int exclude_closest, void* stream);

/* af::filterDisconnected<K> (include/af/GraphBuilder.h:132). */
int afx_filter_disconnected(uint32_t* idx, float* dist, const int* n_nodes, int n_nodes_max, int k,
                            const float* radii, void* stream);

/* af::runComputeWarpWeightsKernel (include/af/VertexManipulation.cuh:18, src/VertexManipulation.cu:134). */
int afx_warp_weights(float* weights, const float* radii, const uint32_t* idx, const float* dist, const unsigned* count,
                     long n_points_max, int k, const int* n_nodes, void* stream);

/* af::runWarpKernel (include/af/ComputeCorrespondence.cuh:11, src/ComputeCorrespondence.cu:32). */
int afx_warp(float* warped, const float* points, const float* transforms, const uint32_t* idx, const float* weights,
             const unsigned* count, long n_points_max, int k, void* stream);

/* afx_warp with dual-quaternion blending (Kavan et al., "Skinning with dual quaternions", 2007) in
 * place of the linear blend: each node's rigid part (the unit quaternion of its transform's upper
 * 3x3, and its translation) as a unit dual quaternion, blended with the weights after aligning
 * hemispheres with the first valid node, normalised, applied as one rigid motion.  A point whose
 * weights are all within 1e-5 of zero keeps its position, as in warpKernel.  No counterpart in the
 * reference, which blends linearly only (src/ComputeCorrespondence.cu:5-30); the blend the session
 * option `blend = AFX_BLEND_DQB` uses. */
int afx_warp_dqb(float* warped, const float* points, const float* transforms, const uint32_t* idx,
                 const float* weights, const unsigned* count, long n_points_max, int k, void* stream);

/* af::runCorrespondencePairsKernel (include/af/ComputeCorrespondence.cuh:19,
 * src/ComputeCorrespondence.cu:83): (vertex, pixel) pairs, ordered by vertex index.
 * *corr_count (device) is overwritten. */
int afx_correspondences(int* corr, unsigned* corr_count, long capacity, const float* warped, const unsigned* count,
                        long n_points_max, const float K[9], const float* depth, int rows, int cols,
                        const float* frame_vertices, float thresh, void* workspace, size_t workspace_bytes,
                        void* stream);
size_t afx_correspondences_workspace_size(long n_points_max);

/* afx_correspondences without a workspace and without allocating: for callers that must
 * not allocate device memory during the frame (real-time loops on a preallocated memory
 * budget, code running under an allocator lock or inside a host callback).  This entry
 * point has no counterpart in the reference.  Scratch is a fixed device array of the
 * library sized for AFX_CORR_STATIC_MAX_POINTS vertices (about 3 MiB); n_points_max above
 * that returns AFX_ERR_CAPACITY before any work.  The first call on each device looks up
 * the array's address, and so does the first call after a device reset (make that first
 * call before any stream capture).  All calls on a
 * device share the one array: calls that overlap in time (other streams, other host
 * threads) race and must be ordered by the caller.  Results equal afx_correspondences. */
#define AFX_CORR_STATIC_MAX_POINTS 262144L
int afx_correspondences_static(int* corr, unsigned* corr_count, long capacity, const float* warped,
                               const unsigned* count, long n_points_max, const float K[9], const float* depth,
                               int rows, int cols, const float* frame_vertices, float thresh, void* stream);

/* ------------------------------------------------------------------------------------
 * Gauss-Newton for the motion graph, step by step (src/VolumeFusion.cu:454-691 drives these
 * kernels of src/MotionOptimization.cu with a dense J and a cuSOLVER LU).  Here J is never
 * stored: J^T J is assembled block-sparse per node (the session uses the same code).
 * ------------------------------------------------------------------------------------ */
typedef struct afx_gn afx_gn;

/* Workspace for graphs of up to n_nodes_max nodes, n_points_max canonical vertices and as many
 * correspondences, k skinning and kreg regularisation neighbours (<= 8 each). */
int afx_gn_create(long n_points_max, int n_nodes_max, int k, int kreg, afx_gn** out);
int afx_gn_destroy(afx_gn* g);

/* Residuals and system for correspondences `corr` ((vertex, pixel) pairs, *n_corr of them):
 * fill_r_DepthKernel / fill_r_MRegKernel (src/MotionOptimization.cu:163-241), fill_J_DepthKernel /
 * fill_J_MRegKernel (:29-161), computeJTJAndJTrContrib* + sort/reduce_by_key + multiply* +
 * fillJTJKernel / fillJTrKernel (:243-481, src/VolumeFusion.cu:504-646) and
 * runInitIdentityKernel (src/Helper.cu:37-50).  `warped` are the canonical vertices warped by
 * `transforms`; graph_idx is the filtered K_reg-NN of each node.  Synchronises `stream`;
 * returns AFX_ERR_SINGULAR when a diagonal block has no inverse.  The system is kept in the
 * workspace (the counters are copied); afx_gn_export and afx_gn_solve read only the workspace. */
int afx_gn_build(afx_gn* g, const float* canonical, const unsigned* n_points, const uint32_t* knn_idx,
                 const float* knn_weights, const int* corr, const unsigned* n_corr, const float* frame_vertices,
                 const float* frame_normals, const float* warped, const float* nodes, const float* transforms,
                 const int* n_nodes, const uint32_t* graph_idx, float lambda_depth, float lambda_reg, void* stream);

/* The built system in the reference's layout (any pointer may be NULL): jtj = dense
 * (6 n)^2 float, row-major (symmetric), untouched diagonal blocks the identity; jtr = 6 n;
 * r_depth = one residual per correspondence; r_reg = 3 per (node, K_reg slot).  n_nodes_host is
 * the node count (the device counter's value). */
int afx_gn_export(afx_gn* g, int n_nodes_host, float* jtj, float* jtr, float* r_depth, float* r_reg, void* stream);

/* x = (J^T J)^-1 J^T r by block-Jacobi preconditioned conjugate gradients: `iterations` steps, or
 * until |r| <= tol |b| when tol > 0 (replaces linearSolverLUStable, src/LinearSolver.cu:179-224).
 * x: 6 * n_nodes_max floats, device. */
int afx_gn_solve(afx_gn* g, float* x, int iterations, double tol, void* stream);

/* runUpdateTransformsKernel (src/MotionOptimization.cu:483-506): T -= [[x_rot]x, x_t; 0]. */
int afx_update_transforms(float* transforms, const float* x, const int* n_nodes, int n_nodes_max, void* stream);

/* The reference's dense Gauss-Newton operators, for callers that keep its dense path
 * (src/VolumeFusion.cu:454-691).  J is rows x width Vec6f (6 floats), row-major; pairs and J^T r
 * elements are Vec2i (2 ints); a product is a Mat6f (36 floats, column-major); J^T J is dense with
 * rows jtj_width floats apart.  All arrays are device arrays.
 *  afx_fill_j_depth / afx_fill_j_mreg: runFill_J_DepthKernel / runFill_J_MRegKernel
 *    (include/af/MotionOptimization.cuh:9-28); K / Kreg neighbours per vertex / node (<= 8).
 *  afx_fill_r_depth / afx_fill_r_mreg: runFill_r_DepthKernel / runFill_r_MRegKernel (:30-43).
 *  afx_jtj_contrib_depth / afx_jtj_contrib_mreg: runComputeJTJAndJTrContribJ*Kernel (:51-68): the
 *    pairs (with row numbers) and J^T r elements appended after the counters' current values
 *    (device counters, updated) -- in row order, where the reference's atomics append in a varying
 *    order.  Workspace: afx_jtj_contrib_workspace_size(rows of the call).
 *  afx_multiply_jtj_pairs / afx_multiply_jtr_elems: runMultiplyJTJContribPairsKernel /
 *    runMultiplyJTrContribElemsKernel (:70-82).
 *  afx_fill_jtj / afx_fill_jtr: runFillJTJKernel / runFillJTrKernel (:84-90).  J^T J is taken as
 *    square (jtj_width / 6 nodes); pairs naming a node outside J or J^T J are skipped.
 *  afx_lu_solve: linearSolverLUStable (include/af/LinearSolver.cuh:22, src/LinearSolver.cu:179-223):
 *    x = A^-1 b by LU with partial pivoting in binary32, A column-major with leading dimension lda
 *    (left unchanged; factorised in the workspace), ipiv the 1-based pivots; AFX_ERR_SINGULAR where
 *    getrf would report info != 0.  Synchronises `stream`. */
int afx_fill_j_depth(float* J, float weight, unsigned rows, unsigned width, const int* corr, unsigned n_corr,
                     const float* mesh, const uint32_t* knn_idx, const float* knn_w, int K, const float* normals,
                     void* stream);
int afx_fill_j_mreg(float* J, float weight, unsigned rows, unsigned width, const float* nodes, unsigned n_nodes,
                    const uint32_t* knn_idx, int Kreg, void* stream);
int afx_fill_r_depth(float* r, float weight, const int* corr, unsigned n_corr, const float* warped,
                     const float* depth_mesh, const float* normals, void* stream);
int afx_fill_r_mreg(float* r, float weight, const float* nodes, const float* transforms, unsigned n_nodes,
                    const uint32_t* knn_idx, int Kreg, void* stream);
size_t afx_jtj_contrib_workspace_size(long rows);
int afx_jtj_contrib_depth(int* pairs, unsigned* rows, unsigned* n_pairs, int* jtr_elems, unsigned* n_jtr,
                          const int* corr, unsigned n_corr, const uint32_t* knn_idx, const float* knn_w, int K,
                          void* workspace, size_t workspace_bytes, void* stream);
int afx_jtj_contrib_mreg(int* pairs, unsigned* rows, unsigned row_offset, unsigned* n_pairs, int* jtr_elems,
                         unsigned* n_jtr, unsigned n_nodes, const uint32_t* knn_idx, int Kreg, void* workspace,
                         size_t workspace_bytes, void* stream);
int afx_multiply_jtj_pairs(float* out, const int* pairs, const unsigned* rows, unsigned n_pairs, const float* J,
                           unsigned width, void* stream);
int afx_multiply_jtr_elems(float* out, const int* elems, unsigned n_elems, const float* J, const float* r,
                           unsigned width, void* stream);
int afx_fill_jtj(float* JTJ, const int* coords, const float* elems, unsigned n_elems, unsigned jtj_width,
                 void* stream);
int afx_fill_jtr(float* JTr, const int* coords, const float* elems, unsigned n_elems, void* stream);
size_t afx_lu_solve_workspace_size(int n, int lda);
int afx_lu_solve(float* x, const float* A, int n, int lda, const float* b, int* ipiv, void* workspace,
                 size_t workspace_bytes, void* stream);

/* ------------------------------------------------------------------------------------
 * Whole-frame session: af::runVolumeFusion's per-frame loop (src/VolumeFusion.cu:223-769)
 * with all state (TSDF, motion graph, solver) resident on the device.
 * ------------------------------------------------------------------------------------ */

typedef struct afx_fusion_params {
    int width, height;
    float K[9];
    int dims[3];
    float volume_size[3];
    float delta;                 /* settings.tsdfDelta */
    float depth_threshold;
    int bilateral, bilateral_r;
    float sigma_i, sigma_s, bilateral_thr;
    float excl_angle_lo, excl_angle_hi;
    float graph_radius;          /* settings.motionGraphRadius */
    int knn;                     /* skinning neighbours (reference: Constants::motionGraphKNN = 6); 1..8 */
    int kreg;                    /* regularisation neighbours (reference: Constants::energyMRegKNN = 4); 1..8 */
    int update_graph;
    int icp_iterations;
    int gn_iterations;           /* reference: 20 */
    float lambda_depth, lambda_reg, energy_min_step, corr_thresh;
    int solver;                  /* 1 = block-Jacobi PCG (fixed iterations); 2 = PCG to pcg_tol */
    int pcg_iterations;
    double pcg_tol;
    int integrate;               /* settings.integrateTsdf */
    int extract_mesh;            /* run the full marching-cubes mesh each frame */
    int node_capacity;
    long mesh_capacity;          /* canonical point cloud capacity */
    long triangle_capacity;
    int precision;               /* AFX_PRECISION_FP32 (the reference's DeviceTsdf<float>) or
                                    AFX_PRECISION_FP16: FP16 TSDF values + uint16 weights, 4 B/voxel */
    int warp_mesh;               /* settings.isMeshWarped: warp the output mesh into the live frame
                                    (details::warpMeshGPU, src/VolumeFusion.cu:75-110) */
    int blend;                   /* AFX_BLEND_LBS (the reference's linear blend of node transforms) or
                                    AFX_BLEND_DQB (dual-quaternion blending of their rigid parts) for
                                    every warp: canonical points, voxel centres, output mesh.  The
                                    Gauss-Newton Jacobian is the linear blend's in both cases. */
    afx_camera_distortion distortion;  /* the depth camera's distortion; when is_distorted, every frame
                                    is undistorted as af::loadProcessFrame does (cv::undistort of the
                                    metres before the filter, src/VolumeFusion.cu:162-180), through a
                                    map built once at create (AFX_UNDISTORT_LINEAR) */
} afx_fusion_params;

#define AFX_PRECISION_FP32 0
#define AFX_PRECISION_FP16 1

typedef struct afx_fusion afx_fusion;

/* Device bytes afx_fusion_create would allocate for these parameters (0 if they are invalid);
 * used for admission by memory budget. */
size_t afx_fusion_memory_bytes(const afx_fusion_params* params);

typedef struct afx_frame_stats {
    int frame;
    int n_nodes;
    int new_nodes;
    unsigned mesh_points;        /* canonical point cloud size after de-duplication */
    unsigned correspondences;
    int gn_iterations_done;
    double energy;               /* last evaluated energy */
    unsigned mesh_vertices, mesh_faces;
    int error;                   /* device-side error flags (0 = none) */
} afx_frame_stats;

void afx_fusion_default_params(afx_fusion_params* p);
int afx_fusion_create(const afx_fusion_params* params, afx_fusion** out);
int afx_fusion_destroy(afx_fusion* f);
/* Reset the volume and graph (af::DeviceTsdf::initDefault + MotionGraph::clear). */
int afx_fusion_reset(afx_fusion* f, void* stream);
/* Process one frame: the first frame after create/reset initialises the volume by rigid
 * integration at its centroid (src/VolumeFusion.cu:327-337); later frames run the
 * non-rigid loop.  depth_mm is a device pointer (use afx_fusion_process_host for host
 * memory).  Asynchronous on `stream`. */
int afx_fusion_process(afx_fusion* f, const uint16_t* depth_mm, void* stream);
/* Same, from host memory: the frame is copied into one of two session input buffers on the
 * session's own copy stream, and the frame on `stream` waits for that copy, so frames submitted back
 * to back overlap each copy with the frame before it.  A pinned host buffer must stay unchanged until
 * its frame has run (pageable memory is staged before the call returns). */
int afx_fusion_process_host(afx_fusion* f, const uint16_t* depth_mm_host, void* stream);
/* Enqueue a copy of the last frame's statistics into host memory (pinned for an asynchronous
 * copy); the values are there once `stream` has passed this point. */
int afx_fusion_stats_async(afx_fusion* f, afx_frame_stats* out_host, void* stream);
/* Copy the last frame's statistics to host memory (synchronises `stream`). */
int afx_fusion_stats(afx_fusion* f, afx_frame_stats* out, void* stream);
/* Device views of the session state (valid until destroy). */
int afx_fusion_tsdf(afx_fusion* f, float** tsdf, float** weights);  /* FP32 sessions; else AFX_ERR_UNSUPPORTED */
/* Device view of the volume in either storage format: FP32 values + FP32 weights, or (precision
 * form) IEEE FP16 values + uint16 weights; *precision says which. */
int afx_fusion_volume(afx_fusion* f, void** tsdf, void** weights, int* precision);
/* After writing the session's volume through these views: the session keeps, per brick of 8^3
 * voxels, whether any voxel has a weight (marching cubes skips bricks without, which hold no active
 * cube) and updates it itself when it integrates or loads a volume; this rebuilds it from the
 * weights.  No counterpart in the reference.  Asynchronous on `stream`. */
int afx_fusion_volume_changed(afx_fusion* f, void* stream);
int afx_fusion_graph(afx_fusion* f, float** nodes, float** radii, float** transforms, int** n_nodes);
int afx_fusion_centroid(afx_fusion* f, float** centroid);
int afx_fusion_point_cloud(afx_fusion* f, float** points, unsigned** count);
/* The frame's output mesh (runMarchingCubesFullKernel, src/VolumeFusion.cu:744-762): 3 vertices and
 * one face per triangle, vertices translated by the frame-0 centroid and, with warp_mesh, warped
 * into the live frame.  The canonical point cloud (afx_fusion_point_cloud) is not warped. */
int afx_fusion_mesh(afx_fusion* f, float** vertices, unsigned** vertex_count, int** faces, unsigned** face_count);
int afx_fusion_frame_views(afx_fusion* f, float** depth, float** vertices, float** normals);
/* Size of the last non-rigid frame's voxel support (no counterpart in the reference): the bricks of
 * 8^3 voxels that some node's support cube touches, and the voxels in them with at least one
 * supporting node (the reference's knnCount > 0, src/TSDFWarp.cu:61-67).  Synchronises `stream`. */
int afx_fusion_support_size(afx_fusion* f, unsigned* active_bricks, unsigned long long* supported_voxels,
                            void* stream);
/* Bricks of 8^3 voxels that hold a voxel with nonzero weight (of *total in the volume): the bricks
 * marching cubes reads (no counterpart in the reference, whose kernel reads every voxel).
 * Synchronises `stream`. */
int afx_fusion_occupied_bricks(afx_fusion* f, unsigned long long* bricks, unsigned long long* total, void* stream);
/* Overwrite the committed node transforms (host memory), e.g. to replay a trajectory. */
int afx_fusion_set_transforms(afx_fusion* f, const float* transforms_host, int n, void* stream);
/* Number of kernels the library launched since the session was created. */
long afx_fusion_kernel_launches(const afx_fusion* f);

/* Replay non-rigid frames from CUDA graphs (default on): from the fourth frame of a sequence the
 * frame's kernels are launched as one graph, captured on first use (one per buffer parity); the
 * input is copied into the session's own buffer first.  Off: every kernel is launched one by
 * one.  Results are the same either way.  Stage timing always launches one by one. */
int afx_fusion_set_graphs(afx_fusion* f, int on);
/* Number of frame graphs captured so far (0 while graphs are off or capture fell back). */
int afx_fusion_graph_count(const afx_fusion* f);

/* Marching-cubes tile of the session (no counterpart in the reference): AFX_MC_TILE_TMA16 (default:
 * a CTA's brick of 32x8x16 cubes brought into shared memory by TMA), AFX_MC_TILE_TMA8,
 * AFX_MC_TILE_TMA32 (8 or 32 cubes along z), AFX_MC_TILE_COLUMN (column march from global memory),
 * AFX_MC_TILE_PIPE8 / AFX_MC_TILE_PIPE16 / AFX_MC_TILE_PIPE4 (a persistent grid whose CTAs keep two
 * bricks of 8, 16 or 4 cubes in flight).  Results are the same with every tile (point and triangle sets; triangle order
 * may differ).  afx_fusion_autotune times each tile on the session's current volume (call it after
 * a few frames), keeps the fastest and returns it in *tile (and the best time of each tile in
 * ms[AFX_MC_TILES] if given); it re-extracts the current frame's mesh and blocks on `stream`.
 * Changing the tile drops the captured frame graphs, which are captured again on next use. */
#define AFX_MC_TILE_TMA16 0
#define AFX_MC_TILE_TMA8 1
#define AFX_MC_TILE_TMA32 2
#define AFX_MC_TILE_COLUMN 3
#define AFX_MC_TILE_PIPE8 4
#define AFX_MC_TILE_PIPE16 5
#define AFX_MC_TILE_PIPE4 6
#define AFX_MC_TILES 7
int afx_fusion_set_tile(afx_fusion* f, int tile);
int afx_fusion_get_tile(const afx_fusion* f);
int afx_fusion_autotune(afx_fusion* f, int* tile, float* ms, void* stream);

/* Per-stage GPU timing (CUDA events around each stage, like the reference's TimeMap).
 * Stages: 0 prep, 1 rigid integration, 2 point-cloud sort/unique, 3 graph build, 4 KNN +
 * weights, 5 Gauss-Newton structure, 6 Gauss-Newton iterations, 7 voxel support,
 * 8 voxel warp + collisions, 9 warped integration, 10 marching cubes.
 * afx_fusion_stage_times waits for the recorded events, adds milliseconds per stage into
 * ms[0..n) and returns the number of stages; reset != 0 starts a new accumulation. */
int afx_fusion_set_timing(afx_fusion* f, int on);
int afx_fusion_stage_times(afx_fusion* f, double* ms, int n, int reset);

/* ------------------------------------------------------------------------------------
 * Serving many depth streams on one GPU (no counterpart in the reference, which fuses one
 * recorded sequence per process).  Sessions are admitted while their device bytes
 * (afx_fusion_memory_bytes) fit the budget; each has its own stream, so frames of different
 * sessions overlap on the device; frames of one session run in order.  Not thread-safe
 * across servers sharing a session; calls on one server are serialised internally.
 * ------------------------------------------------------------------------------------ */
typedef struct afx_server afx_server;

typedef struct afx_server_result {
    int session_id;
    uint64_t tag;        /* the caller's tag from afx_server_submit */
    double latency_ms;   /* afx_server_submit to the completion seen by afx_server_poll */
    afx_frame_stats stats;
} afx_server_result;

int afx_server_create(size_t memory_budget_bytes, int max_sessions, afx_server** out);
int afx_server_destroy(afx_server* s);
/* AFX_ERR_NO_MEMORY: the budget (or max_sessions) does not admit the session now. */
int afx_server_open(afx_server* s, const afx_fusion_params* params, int* session_id);
/* Closes once the session's frames in flight are done; its memory returns to the budget. */
int afx_server_close(afx_server* s, int session_id);
/* Queue one frame (host uint16 mm, copied before return).  AFX_ERR_CAPACITY: the session has
 * 4 frames in flight; poll and retry. */
int afx_server_submit(afx_server* s, int session_id, const uint16_t* depth_mm_host, uint64_t tag);
/* Up to max_results finished frames, oldest first per session. */
int afx_server_poll(afx_server* s, afx_server_result* out, int max_results, int* n_results);
/* The session's afx_fusion (for its volume, graph, mesh); NULL if unknown. */
afx_fusion* afx_server_session(afx_server* s, int session_id);
/* used_bytes: the open sessions' device bytes (idle sessions kept for reuse are counted in
 * afx_server_counters.idle_bytes; both together stay within the budget). */
int afx_server_usage(afx_server* s, size_t* used_bytes, int* sessions, long* denied);

/* A closed session stays allocated, idle, and an open with equal parameters reuses it (reset on
 * its stream; arena, stream, pinned slots and captured frame graphs kept).  Counters since
 * creation: opens that allocated and opens that reused, idle sessions freed to make room, and the
 * host time spent inside the calls (staging: the copy into the pinned slot; enqueue: the frame's
 * launches, statistics copy and event). */
typedef struct afx_server_counters {
    long opens_fresh, opens_reused, evictions;
    int idle_sessions;
    size_t idle_bytes;
    long submits, polls, results;
    double open_ms, staging_ms, enqueue_ms, poll_ms;
} afx_server_counters;
int afx_server_get_counters(afx_server* s, afx_server_counters* out);

/* ------------------------------------------------------------------------------------
 * Batched form (no counterpart in the reference): one frame of every session of a batch in one
 * graph launch.  Sessions keep their own state and results (the same as processing them one by
 * one); from the fourth frame of a session's sequence its frame graph is a child of one parent
 * graph per pattern of the sessions' states, with the frame copies and the statistics copies as
 * graph nodes.  Sessions in their first frames run their kernels one by one on `stream` first.
 * depth_mm[i] is session i's frame (device or pinned host memory, uint16 mm, not the session's own
 * input buffer).  afx_batch_stats copies the statistics of the last processed frames (valid once
 * `stream` has passed afx_batch_process).  The batch does not own the sessions.
 * ------------------------------------------------------------------------------------ */
typedef struct afx_batch afx_batch;
int afx_batch_create(afx_fusion* const* sessions, int n, afx_batch** out);
int afx_batch_destroy(afx_batch* b);
int afx_batch_process(afx_batch* b, const uint16_t* const* depth_mm, void* stream);
int afx_batch_stats(afx_batch* b, afx_frame_stats* out, int n);
/* Parent-graph launches so far (one per afx_batch_process with a replayed session). */
long afx_batch_graph_launches(const afx_batch* b);

/* DeviceTsdf::initDefault followed by runIntegrateTSDFFromFrameKernel (include/af/DeviceTsdf.cuh:26-35),
 * in one write-only pass over the volume (8 B per voxel written): the same values and weights as
 * initialising the volume and integrating the frame.  Needs dims[0] % 4 == 0 and 16-byte aligned
 * arrays (AFX_ERR_UNSUPPORTED otherwise). */
int afx_integrate_tsdf_fresh(float* tsdf, float* weights, const float* depth, int width, int height, float delta,
                             const int dims[3], const float voxel_size[3], const float volume_size[3],
                             const float rotate[9], const float translate[3], const float K[9], void* stream);

/* ------------------------------------------------------------------------------------
 * Rigid multi-camera reconstruction stream (af::startMeshReconstructionStream,
 * src/MeshRecontructionStream.cu:115-206; settings in src/Settings.cpp).  Each frame: every
 * camera's depth (uint16 mm, device) is converted, filtered (depth_threshold), bilateral-filtered
 * when enabled, back-projected with its intrinsics and moved to world space by camera_to_world (the
 * inverse of the reference's world2camera.txt, DeviceDepthImage::backProject); the clouds are
 * concatenated in camera order (n_cameras * width * height points, invalid pixels included).  The
 * volume is re-initialised and camera 0's filtered depth alone is integrated at `center` with
 * `rotation` (the reference's DeviceTsdf::integrate of cameras[0]); the full marching-cubes mesh
 * follows (3 vertices and a face per triangle, untranslated).  Lens undistortion is not applied:
 * frames must already be undistorted.  Asynchronous on `stream`; outputs are device views.
 * ------------------------------------------------------------------------------------ */
#define AFX_MAX_CAMERAS 8
typedef struct afx_rigid_stream_params {
    int n_cameras;
    int width, height;                          /* every camera's frame size */
    float K[AFX_MAX_CAMERAS][9];                /* column-major intrinsics per camera */
    float camera_to_world[AFX_MAX_CAMERAS][16]; /* column-major 4x4 per camera */
    int dims[3];                                /* settings.tsdfDim */
    float volume_size[3];                       /* settings.tsdfSize */
    float delta;                                /* settings.tsdfDelta */
    float center[3];                            /* settings.tsdfCenter */
    float rotation[9];                          /* column-major, the rotation settings.tsdfRotation gives */
    float depth_threshold;
    int bilateral, bilateral_r;
    float sigma_i, sigma_s, bilateral_thr;
    long triangle_capacity;
    afx_camera_distortion distortion[AFX_MAX_CAMERAS]; /* per camera; when is_distorted, the camera's
                                                 depth is undistorted as CameraData::processNextFrame does
                                                 (src/MeshRecontructionStream.cu:94-101): the unfiltered
                                                 metres remapped INTER_NEAREST replace the filtered frame */
} afx_rigid_stream_params;
typedef struct afx_rigid_stream afx_rigid_stream;
void afx_rigid_stream_default_params(afx_rigid_stream_params* p);
int afx_rigid_stream_create(const afx_rigid_stream_params* params, afx_rigid_stream** out);
int afx_rigid_stream_destroy(afx_rigid_stream* s);
int afx_rigid_stream_process(afx_rigid_stream* s, const uint16_t* const* depth_mm, void* stream);
int afx_rigid_stream_outputs(afx_rigid_stream* s, float** cloud, long* cloud_points, float** vertices,
                             unsigned** vertex_count, int** faces, unsigned** face_count, float** tsdf, float** weights);

/* ------------------------------------------------------------------------------------
 * On-disk formats of the reference (host arrays; the session helpers copy device state).
 * afx_save_ply: Mesh::savePly (src/Mesh.cpp:23-64), ASCII PLY with float x y z + uchar rgb per
 *   vertex (colors may be NULL: 0 0 0) and "3 a b c" faces; refuses an empty vertex list.
 * afx_tsdf_save / afx_tsdf_load: TSDFVolume::save / load (src/TSDFVolume.cpp:315-361): int32 dims,
 *   the volume size and voxel size (the 24 bytes the reference writes from m_size), float delta,
 *   float tsdf[S], float weights[S], then colour arrays (written as 127 with colour weights 0;
 *   ignored on load).  afx_tsdf_load reads the values and weights of a volume of n_voxels voxels.
 * afx_fusion_save_volume / afx_fusion_load_volume: the session's volume in that format (FP16
 *   sessions widen on save and round to nearest binary16 on load; weights must be integers 0..65535);
 *   the loaded file must have the session's dims.  afx_fusion_save_mesh_ply: the frame's output
 *   mesh.  All three synchronise `stream`.
 * ------------------------------------------------------------------------------------ */
int afx_save_ply(const char* path, const float* vertices, long n_vertices, const unsigned char* colors,
                 const int* faces, long n_faces);
int afx_tsdf_save(const char* path, const int dims[3], const float volume_size[3], const float voxel_size[3],
                  float delta, const float* tsdf, const float* weights);
int afx_tsdf_load_header(const char* path, int dims[3], float volume_size[3], float voxel_size[3], float* delta);
int afx_tsdf_load(const char* path, float* tsdf, float* weights, long n_voxels);
int afx_fusion_save_volume(afx_fusion* f, const char* path, void* stream);
int afx_fusion_load_volume(afx_fusion* f, const char* path, void* stream);
int afx_fusion_save_mesh_ply(afx_fusion* f, const char* path, void* stream);

/* ------------------------------------------------------------------------------------
 * Depth ingest: image decoding (host) and camera undistortion (device).
 *
 * afx_decode_depth_image: cv::imread(file, IMREAD_ANYDEPTH | IMREAD_ANYCOLOR) of a depth frame
 *   (src/dataset.cpp:168-189, src/KinectReader.cpp:9-21, src/AzureReader.cpp:10-22) from the file's
 *   bytes in host memory: greyscale 8- or 16-bit PNG (any filter, Adam7 or not) or TIFF (strips;
 *   none / LZW / Deflate / PackBits; horizontal predictor), to uint16 millimetres in out[height][width]
 *   (host).  out = NULL returns the size only.  AFX_ERR_UNSUPPORTED for colour or other depths,
 *   AFX_ERR_INVALID_ARGUMENT for a corrupt file (bad CRC-32 / Adler-32, truncated data),
 *   AFX_ERR_CAPACITY when capacity < width * height.  The conversion to metres happens in the frame
 *   preparation on the device (afx_depth_from_mm, afx_frame_prep).
 * afx_decode_depth_images: n images decoded on up to `threads` host threads; status[i] per image,
 *   the first non-zero status returned.  widths / heights may be NULL.
 * afx_depth_file_name: af::insertIntoPattern (src/dataset.cpp:131-150): the run of all the
 *   pattern's '*' replaced by the zero-padded index.
 * afx_read_depth_frame: afx_depth_file_name + read + afx_decode_depth_image.
 * ------------------------------------------------------------------------------------ */
int afx_decode_depth_image(const uint8_t* data, size_t len, uint16_t* out, long capacity, int* width, int* height);
int afx_decode_depth_images(int n, const uint8_t* const* data, const size_t* lens, uint16_t* const* outs,
                            const long* capacities, int* widths, int* heights, int* status, int threads);
int afx_depth_file_name(const char* pattern, long index, char* out, size_t capacity);
int afx_read_depth_frame(const char* pattern, long index, uint16_t* out, long capacity, int* width, int* height);

/* The two undistortions of the reference, both with the intrinsics as new camera matrix and
 * constant-zero borders:
 *  AFX_UNDISTORT_LINEAR  cv::undistort of the float depth (af::loadProcessFrame,
 *                        src/VolumeFusion.cu:162-180): fixed-point maps (1/32 pixel) built in stripes
 *                        of max(1, 4096 / width) rows, bilinear sampling;
 *  AFX_UNDISTORT_NEAREST cv::initUndistortRectifyMap(..., CV_32FC1) + cv::remap(INTER_NEAREST)
 *                        (src/MeshRecontructionStream.cu:94-101, src/PointCloudStream.cu:107-116).
 * afx_undistort_map writes the per-pixel source map (2 x uint32 per pixel, device; build it once per
 * camera), afx_undistort_depth applies it to a float image (dst must not alias src). */
#define AFX_UNDISTORT_LINEAR 0
#define AFX_UNDISTORT_NEAREST 1
int afx_undistort_map(uint32_t* map, int width, int height, const float K[9], const afx_camera_distortion* d,
                      int mode, void* stream);
int afx_undistort_depth(float* dst, const float* src, int width, int height, const uint32_t* map, int mode,
                        void* stream);

/* af::create_xy_lookup_table (src/CameraCalibration.cpp:261-295): for every pixel (x, y) the ray
 * (X/Z, Y/Z) of af::transformation_unproject at unit depth -- Brown-Conrady inverse by the closed-form
 * first guess and up to 20 Gauss-Newton passes (src/CameraCalibration.cpp:106-218) -- or (0, 0) where
 * the unprojection is invalid.  intrinsics = the af::CameraIntrinsics fields {cx, cy, fx, fy} as the
 * caller filled them.  table: 2 floats per pixel, device.  AFX_ERR_INVALID_ARGUMENT unless fx, fy > 0. */
int afx_xy_lookup_table(float* table, int width, int height, const float intrinsics[4],
                        const afx_camera_distortion* d, void* stream);
/* af::transformation_unproject / transformation_project (src/CameraCalibration.cpp:220-259) over n
 * points (device arrays): pixels (2 floats) + depths -> points (3 floats) and valid flags; points ->
 * pixels and valid flags. */
int afx_unproject_points(float* points, int* valid, const float* pixels, const float* depths, long n,
                         const float intrinsics[4], const afx_camera_distortion* d, void* stream);
int afx_project_points(float* pixels, int* valid, const float* points, long n, const float intrinsics[4],
                       const afx_camera_distortion* d, void* stream);

/* Stream-ordered device-to-device copy (helper for bindings that hold raw device views). */
int afx_copy_device(void* dst, const void* src, size_t bytes, void* stream);

#ifdef __cplusplus
}
#endif
#endif
