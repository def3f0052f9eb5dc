/*
 * af/afx_gn_dense.h -- the reference's dense Gauss-Newton operators and LU solve over the C ABI
 * (header-only C++17), with the reference's names and argument lists:
 *
 *   runFill_J_DepthKernel, runFill_J_MRegKernel, runFill_r_DepthKernel, runFill_r_MRegKernel,
 *   runComputeJTJAndJTrContribJDepthKernel, runComputeJTJAndJTrContribJMRegKernel,
 *   runMultiplyJTJContribPairsKernel, runMultiplyJTrContribElemsKernel, runFillJTJKernel,
 *   runFillJTrKernel, factorial, combinations        include/af/MotionOptimization.cuh:9-90
 *   linearSolverLU, linearSolverLUStable              include/af/LinearSolver.cuh:20-22
 *
 * Every buffer is a device buffer, as in the reference; counters (pair and element sizes) are device
 * counters the calls append after.  The contributing pairs come out in row order (the reference's
 * atomics give a varying order that its caller sorts).  The solvers take any handle type in place of
 * the cusolverDnHandle_t (it is not used) and factorise in binary32 with partial pivoting.  Calls
 * block until the GPU work has finished and throw std::runtime_error on failure.
 */
#ifndef AF_AFX_GN_DENSE_H
#define AF_AFX_GN_DENSE_H

#include "afx_containers.h"

namespace af {

constexpr unsigned int factorial(const unsigned int k) { return k == 0 ? 1 : k * factorial(k - 1); }
constexpr int combinations(const unsigned int n, const unsigned int k) {
    return factorial(n) / (factorial(k) * factorial(n - k));
}

template <class KnnIdx, class KnnW>
inline void runFill_J_DepthKernel(Vec6f* jDepth, float energyWeight, unsigned int jDepthHeight, unsigned int jDepthWidth,
                                  const Vec2i* cCorrIdxs, unsigned int corrIdxsSize, const Vec3f* cCanonMesh,
                                  const KnnIdx* cKnnIdxs, const KnnW* cKnnWeights, const Vec3f* /*cDepthMesh*/,
                                  const Vec3f* cDepthMeshNormals) {
    const int K = detail::slots<KnnIdx>(0);
    detail::afx_check(afx_fill_j_depth(detail::ff<6>(jDepth), energyWeight, jDepthHeight, jDepthWidth,
                                       detail::flat<int, 2>(cCorrIdxs), corrIdxsSize, detail::ff<3>(cCanonMesh),
                                       detail::u32(cKnnIdxs), reinterpret_cast<const float*>(cKnnWeights), K,
                                       detail::ff<3>(cDepthMeshNormals), nullptr),
                      "runFill_J_DepthKernel");
}

template <class KnnIdx>
inline void runFill_J_MRegKernel(Vec6f* jMReg, float energyWeight, unsigned int jMRegHeight, unsigned int jMRegWidth,
                                 const Vec3f* cGraph, const Mat4f* /*cGraphTransforms*/, const unsigned int cGraphSize,
                                 const KnnIdx* cKNNIdxs) {
    const int Kreg = (int)(sizeof(KnnIdx) / sizeof(unsigned int));
    detail::afx_check(afx_fill_j_mreg(detail::ff<6>(jMReg), energyWeight, jMRegHeight, jMRegWidth, detail::ff<3>(cGraph),
                                      cGraphSize, detail::u32(cKNNIdxs), Kreg, nullptr),
                      "runFill_J_MRegKernel");
}

inline void runFill_r_DepthKernel(float* rDepth, float energyWeight, const Vec2i* cCorrIdxs, unsigned int corrIdxsSize,
                                  const Vec3f* cCanonMeshWarped, const Vec3f* cDepthMesh, const Vec3f* cDepthMeshNormals) {
    detail::afx_check(afx_fill_r_depth(rDepth, energyWeight, detail::flat<int, 2>(cCorrIdxs), corrIdxsSize,
                                       detail::ff<3>(cCanonMeshWarped), detail::ff<3>(cDepthMesh),
                                       detail::ff<3>(cDepthMeshNormals), nullptr),
                      "runFill_r_DepthKernel");
}

template <class KnnIdx>
inline void runFill_r_MRegKernel(float* rMReg, float energyWeight, const Vec3f* cGraph, const Mat4f* cGraphTransforms,
                                 const unsigned int cGraphSize, const KnnIdx* cKNNIdxs) {
    const int Kreg = (int)(sizeof(KnnIdx) / sizeof(unsigned int));
    detail::afx_check(afx_fill_r_mreg(rMReg, energyWeight, detail::ff<3>(cGraph), detail::ff<16>(cGraphTransforms),
                                      cGraphSize, detail::u32(cKNNIdxs), Kreg, nullptr),
                      "runFill_r_MRegKernel");
}

template <class KnnIdx, class KnnW>
inline void runComputeJTJAndJTrContribJDepthKernel(Vec2i* jTJContribPairs, unsigned int* rowNumbers,
                                                   unsigned int* jTJContribPairsSize, Vec2i* jTrContribElems,
                                                   unsigned int* jTrContribElemsSize, const Vec2i* cCorrIdxs,
                                                   unsigned int corrIdxsSize, const KnnIdx* cKnnIdxs,
                                                   const KnnW* cKnnWeights) {
    const int K = detail::slots<KnnIdx>(0);
    const size_t ws = afx_jtj_contrib_workspace_size((long)corrIdxsSize);
    DeviceArray<unsigned char> w(ws);
    detail::afx_check(afx_jtj_contrib_depth(detail::flat<int, 2>(jTJContribPairs), rowNumbers, jTJContribPairsSize,
                                            detail::flat<int, 2>(jTrContribElems), jTrContribElemsSize,
                                            detail::flat<int, 2>(cCorrIdxs), corrIdxsSize, detail::u32(cKnnIdxs),
                                            reinterpret_cast<const float*>(cKnnWeights), K, w.get(), ws, nullptr),
                      "runComputeJTJAndJTrContribJDepthKernel");
}

template <class KnnIdx>
inline void runComputeJTJAndJTrContribJMRegKernel(Vec2i* jTJContribPairs, unsigned int* rowNumbers,
                                                  unsigned int rowNumberOffset, unsigned int* jTJContribPairsSize,
                                                  Vec2i* jTrContribElems, unsigned int* jTrContribElemsSize,
                                                  const unsigned int cGraphSize, const KnnIdx* cKNNIdxs) {
    const int Kreg = (int)(sizeof(KnnIdx) / sizeof(unsigned int));
    const size_t ws = afx_jtj_contrib_workspace_size((long)cGraphSize);
    DeviceArray<unsigned char> w(ws);
    detail::afx_check(afx_jtj_contrib_mreg(detail::flat<int, 2>(jTJContribPairs), rowNumbers, rowNumberOffset,
                                           jTJContribPairsSize, detail::flat<int, 2>(jTrContribElems),
                                           jTrContribElemsSize, cGraphSize, detail::u32(cKNNIdxs), Kreg, w.get(), ws,
                                           nullptr),
                      "runComputeJTJAndJTrContribJMRegKernel");
}

inline void runMultiplyJTJContribPairsKernel(Mat6f* multipliedContribPairs, const Vec2i* cJTJContribPairs,
                                             const unsigned int* cRowNumbers, unsigned int jTJContribPairsSize,
                                             const Vec6f* cJ, const unsigned int cJWidth) {
    detail::afx_check(afx_multiply_jtj_pairs(detail::ff<36>(multipliedContribPairs), detail::flat<int, 2>(cJTJContribPairs),
                                             cRowNumbers, jTJContribPairsSize, detail::ff<6>(cJ), cJWidth, nullptr),
                      "runMultiplyJTJContribPairsKernel");
}

inline void runMultiplyJTrContribElemsKernel(Vec6f* multipliedJTrContribElems, const Vec2i* cJTrContribElems,
                                             const unsigned int cJTrContribElemsSize, const Vec6f* cJ, const float* cr,
                                             const unsigned int cJWidth) {
    detail::afx_check(afx_multiply_jtr_elems(detail::ff<6>(multipliedJTrContribElems), detail::flat<int, 2>(cJTrContribElems),
                                             cJTrContribElemsSize, detail::ff<6>(cJ), cr, cJWidth, nullptr),
                      "runMultiplyJTrContribElemsKernel");
}

inline void runFillJTJKernel(float* JTJ, const Vec2i* cJTJElemsCoords, const Mat6f* cJTJElems, unsigned int jTJElemsSize,
                             const unsigned int cJTJWidth) {
    detail::afx_check(afx_fill_jtj(JTJ, detail::flat<int, 2>(cJTJElemsCoords), detail::ff<36>(cJTJElems), jTJElemsSize,
                                   cJTJWidth, nullptr),
                      "runFillJTJKernel");
}

inline void runFillJTrKernel(Vec6f* JTr, const Vec2i* cJTrElemsCoordinates, const Vec6f* cJTrElems,
                             const unsigned int cJTrElemsSize) {
    detail::afx_check(afx_fill_jtr(detail::ff<6>(JTr), detail::flat<int, 2>(cJTrElemsCoordinates), detail::ff<6>(cJTrElems),
                                   cJTrElemsSize, nullptr),
                      "runFillJTrKernel");
}

// linearSolverLUStable (src/LinearSolver.cu:179-223): x = A^-1 b, A (column-major, lda) unchanged,
// ipiv the pivots; false where getrf would fail.
template <class Handle>
inline bool linearSolverLUStable(Handle, int n, const float* Acopy, int lda, const float* b, int* ipiv, float* x) {
    const size_t ws = afx_lu_solve_workspace_size(n, lda);
    DeviceArray<unsigned char> w(ws);
    const int rc = afx_lu_solve(x, Acopy, n, lda, b, ipiv, w.get(), ws, nullptr);
    if (rc == AFX_ERR_SINGULAR) return false;
    detail::afx_check(rc, "linearSolverLUStable");
    return true;
}

// linearSolverLU (src/LinearSolver.cu:144-177): the same with b overwritten by x and A by its LU
// factors (unit lower part below the diagonal, as getrf leaves them).
template <class Handle>
inline bool linearSolverLU(Handle, int n, float* A, int lda, float* b, int* ipiv) {
    const size_t ws = afx_lu_solve_workspace_size(n, lda);
    DeviceArray<unsigned char> w(ws);
    DeviceArray<float> x((std::size_t)n);
    const int rc = afx_lu_solve(x.get(), A, n, lda, b, ipiv, w.get(), ws, nullptr);
    if (rc == AFX_ERR_SINGULAR) return false;
    detail::afx_check(rc, "linearSolverLU");
    detail::cuda_check(cudaMemcpy(b, x.get(), sizeof(float) * (std::size_t)n, cudaMemcpyDeviceToDevice), "linearSolverLU");
    detail::cuda_check(cudaMemcpy(A, w.get(), sizeof(float) * (std::size_t)lda * n, cudaMemcpyDeviceToDevice),
                       "linearSolverLU");
    return true;
}

}  // namespace af

#endif
