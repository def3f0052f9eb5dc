"""The reference's af:: operator API over torch CUDA tensors, backed by libafx.so.

Names, argument order and meaning follow the reference's free functions
(include/af/*.cuh, include/af/*.h); tensors stand in for its raw device pointers and
Eigen values (Vec3f -> 3 floats, Mat3f/Mat4f -> column-major floats).  Like the
reference, every call here blocks until the GPU work is done and raises on failure
(the reference's CUDA_CHECK throws std::runtime_error, src/Helper.cu:7-20).  The C ABI
underneath is asynchronous and stream-ordered.
"""
import ctypes as C

import numpy as np
import torch

from ._lib import PrepParams, check, lib

INVALID_INDEX = 0xFFFFFFFF


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _p(t):
    if t is None:
        return None
    assert t.is_cuda and t.is_contiguous(), "expected a contiguous CUDA tensor"
    return C.c_void_p(t.data_ptr())


def _f(vals, n):
    arr = (C.c_float * n)(*[float(v) for v in np.asarray(vals, dtype=np.float64).ravel()])
    return arr


def _i(vals, n):
    return (C.c_int * n)(*[int(v) for v in np.asarray(vals).ravel()])


def kcol(M):
    """3x3 / 4x4 matrix (numpy, row-major) -> column-major float list (Eigen layout)."""
    return np.asarray(M, dtype=np.float64).T.ravel()


def _sync(status, what):
    check(status, what)
    torch.cuda.current_stream().synchronize()


def _u32(n=1):
    return torch.zeros(n, dtype=torch.int32, device="cuda")


def _workspace(nbytes):
    return torch.empty(max(int(nbytes), 1), dtype=torch.uint8, device="cuda")


# ---- include/af/VertexManipulation.cuh, include/af/BilateralFilter.cuh ----

def runFilterDepthKernel(depth, threshold):
    _sync(lib().afx_filter_depth(_p(depth), depth.numel(), threshold, _stream()), "runFilterDepthKernel")


def bilateralFilterTextureOpmShared(output, input, height, width, r, sI, sS, thr):
    _sync(lib().afx_bilateral_filter(_p(output), _p(input), height, width, r, sI, sS, thr, _stream()),
          "bilateralFilterTextureOpmShared")


def runDepthToMeshKernel(mesh, depth, width, height, K):
    _sync(lib().afx_depth_to_mesh(_p(mesh), _p(depth), width, height, _f(kcol(K), 9), _stream()),
          "runDepthToMeshKernel")


def runDepthVerticesNormalsKernel(normals, vertices, depth, h, w, normExclAngleRange):
    del depth  # unused by the reference kernel as well
    lo, hi = normExclAngleRange
    _sync(lib().afx_depth_vertices_normals(_p(normals), _p(vertices), h, w, lo, hi, _stream()),
          "runDepthVerticesNormalsKernel")


def runRemoveDepthWithoutNormalsKernel(normals, vertices, depth, h, w):
    _sync(lib().afx_remove_depth_without_normals(_p(normals), _p(vertices), _p(depth), h, w, _stream()),
          "runRemoveDepthWithoutNormalsKernel")


def loadProcessFrame(depth_mm, K, depth_threshold=1.2, bilateral=True, bilateral_r=2, sigma_i=0.03, sigma_s=2.0,
                     bilateral_thr=0.09, norm_excl_angle_range=(1.3, 2.1)):
    """af::loadProcessFrame after the image is in memory (src/VolumeFusion.cu:184-220):
    returns (depth, vertices, normals, centroid) device tensors."""
    h, w = depth_mm.shape
    p = PrepParams()
    p.K[:] = list(kcol(K))
    p.depth_threshold = depth_threshold
    p.bilateral = int(bilateral)
    p.bilateral_r = bilateral_r
    p.sigma_i = sigma_i
    p.sigma_s = sigma_s
    p.bilateral_thr = bilateral_thr
    p.excl_angle_lo, p.excl_angle_hi = norm_excl_angle_range
    mm = depth_mm.to(device="cuda", dtype=torch.int16).contiguous()
    depth = torch.empty((h, w), dtype=torch.float32, device="cuda")
    verts = torch.empty((h, w, 3), dtype=torch.float32, device="cuda")
    nrm = torch.empty((h, w, 3), dtype=torch.float32, device="cuda")
    cen = torch.empty(3, dtype=torch.float32, device="cuda")
    _sync(lib().afx_frame_prep(_p(mm), w, h, C.byref(p), _p(depth), _p(verts), _p(nrm), _p(cen), _stream()),
          "loadProcessFrame")
    return depth, verts, nrm, cen


# ---- include/af/TSDFIntegration.cuh ----

def runIntegrateTSDFFromFrameKernel(tsdf, tsdfWeights, depthFrame, frameDims, delta, dims, voxelSize, volumeSize,
                                    volumeRotate, volumeTranslate, depthIntrinsics):
    _sync(lib().afx_integrate_tsdf(_p(tsdf), _p(tsdfWeights), _p(depthFrame), int(frameDims[0]), int(frameDims[1]),
                                   delta, _i(dims, 3), _f(voxelSize, 3), _f(volumeSize, 3), _f(kcol(volumeRotate), 9),
                                   _f(volumeTranslate, 3), _f(kcol(depthIntrinsics), 9), _stream()),
          "runIntegrateTSDFFromFrameKernel")


def runCountCollisionsPerVoxelKernel(collisionCounts, tsdfVertices, knnCounts, voxelSize, volumeSize, volumeDim,
                                     volumeRotate, volumeTranslate):
    _sync(lib().afx_count_collisions(_p(collisionCounts), _p(tsdfVertices), _p(knnCounts), _f(voxelSize, 3),
                                     _f(volumeSize, 3), _i(volumeDim, 3), _f(kcol(volumeRotate), 9),
                                     _f(volumeTranslate, 3), _stream()), "runCountCollisionsPerVoxelKernel")


def runIntegrateWarpedTSDFFromFrameKernel(tsdf, tsdfWeights, tsdfVertices, collisionCounts, knnCounts, depthFrame,
                                          frameDims, delta, voxelSize, volumeSize, volumeDim, volumeRotate,
                                          volumeTranslate, depthIntrinsics):
    _sync(lib().afx_integrate_warped_tsdf(_p(tsdf), _p(tsdfWeights), _p(tsdfVertices), _p(collisionCounts),
                                          _p(knnCounts), _p(depthFrame), int(frameDims[0]), int(frameDims[1]), delta,
                                          _f(voxelSize, 3), _f(volumeSize, 3), _i(volumeDim, 3),
                                          _f(kcol(volumeRotate), 9), _f(volumeTranslate, 3),
                                          _f(kcol(depthIntrinsics), 9), _stream()),
          "runIntegrateWarpedTSDFFromFrameKernel")


# ---- include/af/TSDFWarp.h ----

def runTsdfKNNGraph(knnIdxs, knnDists, knnCounts, graph, graphRadiuses, graphSize, voxelSize, volumeSize, volumeDim,
                    voxelsPerNode):
    k = knnIdxs.shape[-1]
    ws_bytes = lib().afx_tsdf_knn_workspace_size(_i(volumeDim, 3), int(graphSize), _i(voxelsPerNode, 3))
    ws = _workspace(ws_bytes)
    _sync(lib().afx_tsdf_knn(_p(knnIdxs), _p(knnDists), _p(knnCounts), _p(graph), _p(graphRadiuses), int(graphSize),
                             _f(voxelSize, 3), _f(volumeSize, 3), _i(volumeDim, 3), _i(voxelsPerNode, 3), k, _p(ws),
                             ws.numel(), _stream()), "runTsdfKNNGraph")


def runComputeTsdfWarpWeightsKernel(knnWeights, graphRadiuses, knnIdxs, knnDists, knnCounts, gridSize):
    _sync(lib().afx_tsdf_warp_weights(_p(knnWeights), _p(graphRadiuses), _p(knnIdxs), _p(knnDists), _p(knnCounts),
                                      int(gridSize), knnIdxs.shape[-1], _stream()), "runComputeTsdfWarpWeightsKernel")


def runGenerateTsdfVerticesKernel(tsdfVertices, voxelSize, volumeSize, volumeDim):
    _sync(lib().afx_tsdf_vertices(_p(tsdfVertices), _f(voxelSize, 3), _f(volumeSize, 3), _i(volumeDim, 3), _stream()),
          "runGenerateTsdfVerticesKernel")


def runWarpTsdfKernel(tsdfVertices, motionGraph, knnIdxs, knnWeights, knnCounts, voxelSize, volumeSize, volumeDim):
    del voxelSize, volumeSize
    n = int(np.prod(volumeDim))
    _sync(lib().afx_warp_tsdf(_p(tsdfVertices), _p(motionGraph), _p(knnIdxs), _p(knnWeights), _p(knnCounts), n,
                              knnIdxs.shape[-1], _stream()), "runWarpTsdfKernel")


# ---- include/af/MarchingCubes.cuh, include/af/DeviceTsdf.cuh ----

def runMarchingCubesMeshKernel(mesh, meshSize, tsdf, tsdfWeights, dims, voxelSize, volSize, isoValue=0.0):
    _sync(lib().afx_marching_cubes_points(_p(mesh), _p(meshSize), mesh.shape[0], _p(tsdf), _p(tsdfWeights),
                                          _i(dims, 3), _f(voxelSize, 3), _f(volSize, 3), isoValue, _stream()),
          "runMarchingCubesMeshKernel")


def runMarchingCubesFullKernel(mesh, meshSize, faces, facesSize, tsdf, tsdfWeights, dims, voxelSize, volSize,
                               isoValue=0.0):
    _sync(lib().afx_marching_cubes_mesh(_p(mesh), _p(meshSize), mesh.shape[0], _p(faces), _p(facesSize),
                                        faces.shape[0], _p(tsdf), _p(tsdfWeights), _i(dims, 3), _f(voxelSize, 3),
                                        _f(volSize, 3), isoValue, _stream()), "runMarchingCubesFullKernel")


def sortUnique(points, count):
    """thrust::sort + thrust::unique of Vec3f (src/VolumeFusion.cu:382-384) in place."""
    n_max = points.shape[0]
    ws = _workspace(lib().afx_sort_unique_points_workspace_size(n_max))
    _sync(lib().afx_sort_unique_points(_p(points), _p(count), n_max, _p(ws), ws.numel(), _stream()), "sortUnique")


def runTranslateKernel(mesh, meshSize, translation):
    _sync(lib().afx_translate(_p(mesh), None, int(meshSize), _f(translation, 3), _stream()), "runTranslateKernel")


# ---- include/af/GraphBuilder.h, include/af/VertexManipulation.cuh, include/af/ComputeCorrespondence.cuh ----

def buildGraph(nodes, radii, transforms, n_nodes, mesh, mesh_count, knn, radius):
    """af::buildGraph on the device; node arrays are capacity-sized and n_nodes is a 1-element int32 tensor."""
    ws = _workspace(lib().afx_build_graph_workspace_size(mesh.shape[0], nodes.shape[0]))
    _sync(lib().afx_build_graph(_p(nodes), _p(radii), _p(transforms), _p(n_nodes), nodes.shape[0], _p(mesh),
                                _p(mesh_count), mesh.shape[0], knn, radius, _p(ws), ws.numel(), _stream()),
          "buildGraph")


def getKnnData(idx, dist, nodes, n_nodes, points, count=None, excludeClosest=False):
    _sync(lib().afx_knn(_p(idx), _p(dist), _p(nodes), _p(n_nodes), nodes.shape[0], _p(points), _p(count),
                        points.shape[0], idx.shape[-1], int(excludeClosest), _stream()), "getKnnData")


def filterDisconnected(idx, dist, n_nodes, radii):
    _sync(lib().afx_filter_disconnected(_p(idx), _p(dist), _p(n_nodes), idx.shape[0], idx.shape[-1], _p(radii),
                                        _stream()), "filterDisconnected")


def runComputeWarpWeightsKernel(knnWeights, motionGraphRadiuses, knnIdxs, knnDists, meshSize, n_nodes):
    _sync(lib().afx_warp_weights(_p(knnWeights), _p(motionGraphRadiuses), _p(knnIdxs), _p(knnDists), None,
                                 int(meshSize), knnIdxs.shape[-1], _p(n_nodes), _stream()),
          "runComputeWarpWeightsKernel")


def runWarpKernel(warpedMesh, mesh, motionGraph, knnIdxs, knnWeights, meshSize):
    _sync(lib().afx_warp(_p(warpedMesh), _p(mesh), _p(motionGraph), _p(knnIdxs), _p(knnWeights), None, int(meshSize),
                         knnIdxs.shape[-1], _stream()), "runWarpKernel")


def warpDualQuaternion(warpedMesh, mesh, motionGraph, knnIdxs, knnWeights, meshSize):
    """runWarpKernel with dual-quaternion blending of the node transforms (afx_warp_dqb; no
    counterpart in the reference)."""
    _sync(lib().afx_warp_dqb(_p(warpedMesh), _p(mesh), _p(motionGraph), _p(knnIdxs), _p(knnWeights), None,
                             int(meshSize), knnIdxs.shape[-1], _stream()), "warpDualQuaternion")


def runCorrespondencePairsKernel(corrIdxs, corrIdxsSize, warpedMesh, warpedMeshSize, K, depth, depthDim, frameMesh,
                                 thresholdDist):
    rows, cols = int(depthDim[0]), int(depthDim[1])
    ws = _workspace(lib().afx_correspondences_workspace_size(int(warpedMeshSize)))
    _sync(lib().afx_correspondences(_p(corrIdxs), _p(corrIdxsSize), corrIdxs.shape[0], _p(warpedMesh), None,
                                    int(warpedMeshSize), _f(kcol(K), 9), _p(depth), rows, cols, _p(frameMesh),
                                    thresholdDist, _p(ws), ws.numel(), _stream()), "runCorrespondencePairsKernel")


# ---- include/af/MotionOptimization.cuh, src/LinearSolver.cu (the Gauss-Newton steps) ----

class GaussNewtonSystem:
    """The Gauss-Newton system of one motion-graph solve (src/VolumeFusion.cu:454-691): residuals,
    J^T J and J^T r (block-sparse on the device; `export` gives the reference's dense layout) and
    the block-Jacobi PCG solve that replaces linearSolverLUStable."""

    def __init__(self, n_points_max, n_nodes_max, k, kreg):
        h = C.c_void_p()
        check(lib().afx_gn_create(int(n_points_max), int(n_nodes_max), int(k), int(kreg), C.byref(h)), "afx_gn_create")
        self.h = h
        self.n_nodes_max = int(n_nodes_max)
        self.kreg = int(kreg)

    def close(self):
        if getattr(self, "h", None):
            lib().afx_gn_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def build(self, canonical, n_points, knn_idx, knn_weights, corr, n_corr, frame_vertices, frame_normals, warped,
              nodes, transforms, n_nodes, graph_idx, lambda_depth, lambda_reg):
        _sync(lib().afx_gn_build(self.h, _p(canonical), _p(n_points), _p(knn_idx), _p(knn_weights), _p(corr),
                                 _p(n_corr), _p(frame_vertices), _p(frame_normals), _p(warped), _p(nodes),
                                 _p(transforms), _p(n_nodes), _p(graph_idx), float(lambda_depth), float(lambda_reg),
                                 _stream()), "afx_gn_build")

    def export(self, n_nodes, n_corr):
        """(jtj (6n, 6n), jtr (6n,), r_depth (n_corr,), r_reg (n * kreg * 3,)) as CUDA tensors."""
        dim = 6 * int(n_nodes)
        jtj = torch.empty((dim, dim), dtype=torch.float32, device="cuda")
        jtr = torch.empty(dim, dtype=torch.float32, device="cuda")
        rd = torch.empty(max(int(n_corr), 1), dtype=torch.float32, device="cuda")
        rr = torch.empty(max(int(n_nodes) * self.kreg * 3, 1), dtype=torch.float32, device="cuda")
        _sync(lib().afx_gn_export(self.h, int(n_nodes), _p(jtj), _p(jtr), _p(rd), _p(rr), _stream()), "afx_gn_export")
        return jtj, jtr, rd[:int(n_corr)], rr[:int(n_nodes) * self.kreg * 3]

    def solve(self, iterations=10, tol=0.0):
        x = torch.zeros(6 * self.n_nodes_max, dtype=torch.float32, device="cuda")
        _sync(lib().afx_gn_solve(self.h, _p(x), int(iterations), float(tol), _stream()), "afx_gn_solve")
        return x


def runUpdateTransformsKernel(transforms, x, n_nodes):
    _sync(lib().afx_update_transforms(_p(transforms), _p(x), _p(n_nodes), transforms.shape[0], _stream()),
          "runUpdateTransformsKernel")


# ---- include/af/MotionOptimization.cuh, include/af/LinearSolver.cuh: the dense Gauss-Newton path ----
# J: (rows, width, 6) float tensor; pairs / elements: (n, 2) int32; rows: (n,) int32; products:
# (n, 36) (Mat6f, column-major) or (n, 6); counters: (1,) int32 device counters appended after.

def runFill_J_DepthKernel(jDepth, energyWeight, jDepthHeight, jDepthWidth, corrIdxs, corrIdxsSize, canonMesh,
                          knnIdxs, knnWeights, depthMesh, depthMeshNormals):
    K = knnIdxs.shape[-1]
    _sync(lib().afx_fill_j_depth(_p(jDepth), float(energyWeight), int(jDepthHeight), int(jDepthWidth), _p(corrIdxs),
                                 int(corrIdxsSize), _p(canonMesh), _p(knnIdxs), _p(knnWeights), int(K),
                                 _p(depthMeshNormals), _stream()), "runFill_J_DepthKernel")


def runFill_J_MRegKernel(jMReg, energyWeight, jMRegHeight, jMRegWidth, graph, graphTransforms, graphSize, knnIdxs):
    _sync(lib().afx_fill_j_mreg(_p(jMReg), float(energyWeight), int(jMRegHeight), int(jMRegWidth), _p(graph),
                                int(graphSize), _p(knnIdxs), int(knnIdxs.shape[-1]), _stream()), "runFill_J_MRegKernel")


def runFill_r_DepthKernel(rDepth, energyWeight, corrIdxs, corrIdxsSize, canonMeshWarped, depthMesh, depthMeshNormals):
    _sync(lib().afx_fill_r_depth(_p(rDepth), float(energyWeight), _p(corrIdxs), int(corrIdxsSize),
                                 _p(canonMeshWarped), _p(depthMesh), _p(depthMeshNormals), _stream()),
          "runFill_r_DepthKernel")


def runFill_r_MRegKernel(rMReg, energyWeight, graph, graphTransforms, graphSize, knnIdxs):
    _sync(lib().afx_fill_r_mreg(_p(rMReg), float(energyWeight), _p(graph), _p(graphTransforms), int(graphSize),
                                _p(knnIdxs), int(knnIdxs.shape[-1]), _stream()), "runFill_r_MRegKernel")


def runComputeJTJAndJTrContribJDepthKernel(jTJContribPairs, rowNumbers, jTJContribPairsSize, jTrContribElems,
                                           jTrContribElemsSize, corrIdxs, corrIdxsSize, knnIdxs, knnWeights):
    ws = _workspace(lib().afx_jtj_contrib_workspace_size(int(corrIdxsSize)))
    _sync(lib().afx_jtj_contrib_depth(_p(jTJContribPairs), _p(rowNumbers), _p(jTJContribPairsSize),
                                      _p(jTrContribElems), _p(jTrContribElemsSize), _p(corrIdxs), int(corrIdxsSize),
                                      _p(knnIdxs), _p(knnWeights), int(knnIdxs.shape[-1]), _p(ws), ws.numel(),
                                      _stream()), "runComputeJTJAndJTrContribJDepthKernel")


def runComputeJTJAndJTrContribJMRegKernel(jTJContribPairs, rowNumbers, rowNumberOffset, jTJContribPairsSize,
                                          jTrContribElems, jTrContribElemsSize, graphSize, knnIdxs):
    ws = _workspace(lib().afx_jtj_contrib_workspace_size(int(graphSize)))
    _sync(lib().afx_jtj_contrib_mreg(_p(jTJContribPairs), _p(rowNumbers), int(rowNumberOffset),
                                     _p(jTJContribPairsSize), _p(jTrContribElems), _p(jTrContribElemsSize),
                                     int(graphSize), _p(knnIdxs), int(knnIdxs.shape[-1]), _p(ws), ws.numel(),
                                     _stream()), "runComputeJTJAndJTrContribJMRegKernel")


def runMultiplyJTJContribPairsKernel(multipliedContribPairs, jTJContribPairs, rowNumbers, jTJContribPairsSize, J,
                                     jWidth):
    _sync(lib().afx_multiply_jtj_pairs(_p(multipliedContribPairs), _p(jTJContribPairs), _p(rowNumbers),
                                       int(jTJContribPairsSize), _p(J), int(jWidth), _stream()),
          "runMultiplyJTJContribPairsKernel")


def runMultiplyJTrContribElemsKernel(multipliedJTrContribElems, jTrContribElems, jTrContribElemsSize, J, r, jWidth):
    _sync(lib().afx_multiply_jtr_elems(_p(multipliedJTrContribElems), _p(jTrContribElems), int(jTrContribElemsSize),
                                       _p(J), _p(r), int(jWidth), _stream()), "runMultiplyJTrContribElemsKernel")


def runFillJTJKernel(JTJ, jTJElemsCoords, jTJElems, jTJElemsSize, jTJWidth):
    _sync(lib().afx_fill_jtj(_p(JTJ), _p(jTJElemsCoords), _p(jTJElems), int(jTJElemsSize), int(jTJWidth), _stream()),
          "runFillJTJKernel")


def runFillJTrKernel(JTr, jTrElemsCoordinates, jTrElems, jTrElemsSize):
    _sync(lib().afx_fill_jtr(_p(JTr), _p(jTrElemsCoordinates), _p(jTrElems), int(jTrElemsSize), _stream()),
          "runFillJTrKernel")


def linearSolverLUStable(handle, n, Acopy, lda, b, ipiv, x):
    """x = A^-1 b (A column-major with leading dimension lda, left unchanged); False where getrf would
    fail.  `handle` stands in for the cuSOLVER handle and is not used."""
    ws = _workspace(lib().afx_lu_solve_workspace_size(int(n), int(lda)))
    st = lib().afx_lu_solve(_p(x), _p(Acopy), int(n), int(lda), _p(b), _p(ipiv), _p(ws), ws.numel(), _stream())
    if st == 4:  # AFX_ERR_SINGULAR
        return False
    _sync(st, "linearSolverLUStable")
    return True
