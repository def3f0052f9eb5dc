// afx_gn_dense.cu -- the reference's dense Gauss-Newton operators (src/MotionOptimization.cu:29-520)
// and its LU solve (src/LinearSolver.cu:179-223), for callers that keep the reference's dense
// Jacobian / (6N)^2 J^T J path.  The fused session does not use them: it assembles J^T J
// block-sparse and solves it with a preconditioned CG (afx_gn.cu).
//
// Layouts are the reference's: J is (rows x width) Vec6f, row-major (entry (row, node) at
// row * width + node); a contributing pair is a Vec2i (a <= b) with its row number; a 6x6 product
// is an Eigen Mat6f (column-major); J^T J is a dense (6 width)^2 float matrix whose rows are
// `jtj_width` floats apart; J^T r is width Vec6f.
//
// Where the reference appends pairs and J^T r elements with atomicAdd (in an order that varies from
// run to run, and which its caller then sorts), the entry points here append them in row order --
// row by row, and within a row in the reference's loop order -- so the lists are deterministic; they
// still append after the counters' current values, as the reference's do.
//
// The LU solve is partial-pivoting Gaussian elimination in binary32 on the column-major matrix the
// reference hands to cusolverDnSgetrf (pivot: the largest magnitude in the column, the first on
// ties), then the two triangular solves.  cuSOLVER's blocked factorisation rounds in a different
// order, so x agrees with the reference's to the conditioning of the system, not bit for bit.
#include <cfloat>
#include <cstring>

#include "afx_gn.h"
#include "afx_internal.h"

namespace afx {

namespace {

AFX_D void grad3x6(const float* p, float G[3][6]) {
    // gradOfTransfVertex (src/MotionOptimization.cu:22-27)
    G[0][0] = 0.f;   G[0][1] = p[2];  G[0][2] = -p[1]; G[0][3] = 1.f; G[0][4] = 0.f; G[0][5] = 0.f;
    G[1][0] = -p[2]; G[1][1] = 0.f;   G[1][2] = p[0];  G[1][3] = 0.f; G[1][4] = 1.f; G[1][5] = 0.f;
    G[2][0] = p[1];  G[2][1] = -p[0]; G[2][2] = 0.f;   G[2][3] = 0.f; G[2][4] = 0.f; G[2][5] = 1.f;
}

// fill_J_DepthKernel (src/MotionOptimization.cu:29-61): for every slot with weight >= 1e-4,
// J(row, node) = (n w)^T G(v) lambda.
__global__ void fill_j_depth_kernel(float* J, float lam, unsigned width, const int* corr, unsigned n_corr,
                                    const float* mesh, const uint32_t* knn_idx, const float* knn_w, int K,
                                    const float* normals) {
    AFX_GRID_STRIDE(c, (long)n_corr) {
        const long v = corr[2 * c], px = corr[2 * c + 1];
        const float* n = normals + 3 * px;
        float G[3][6];
        grad3x6(mesh + 3 * v, G);
        for (int i = 0; i < K; ++i) {
            const float w = knn_w[v * K + i];
            if (w < 1.e-4f) continue;
            const uint32_t node = knn_idx[v * K + i];
            if (node >= width) continue;  // not a column of J
            const float nw[3] = {n[0] * w, n[1] * w, n[2] * w};
            float* o = J + 6 * ((long)c * width + node);
#pragma unroll
            for (int q = 0; q < 6; ++q) o[q] = (nw[0] * G[0][q] + (nw[1] * G[1][q] + nw[2] * G[2][q])) * lam;
        }
    }
}

// fill_J_MRegKernel (src/MotionOptimization.cu:82-141): rows (node * Kreg + i) * 3 + axis get
// +lambda grad_axis(node) at the node and -lambda grad_axis(node) at its neighbour.
__global__ void fill_j_mreg_kernel(float* J, float lam, unsigned width, const float* nodes, unsigned n,
                                   const uint32_t* knn, int Kreg) {
    AFX_GRID_STRIDE(c, (long)n) {
        float G[3][6];
        grad3x6(nodes + 3 * c, G);
        for (int ax = 0; ax < 3; ++ax)
#pragma unroll
            for (int q = 0; q < 6; ++q) G[ax][q] = G[ax][q] * lam;
        for (int i = 0; i < Kreg; ++i) {
            const uint32_t nb = knn[c * Kreg + i];
            if (nb >= n) continue;
            const long row = (c * Kreg + i) * 3;
            for (int ax = 0; ax < 3; ++ax) {
                float* own = J + 6 * ((row + ax) * width + c);
                float* other = J + 6 * ((row + ax) * width + nb);
#pragma unroll
                for (int q = 0; q < 6; ++q) {
                    own[q] = G[ax][q];
                    other[q] = -G[ax][q];
                }
            }
        }
    }
}

// fill_r_DepthKernel (src/MotionOptimization.cu:163-181): lambda n . (warped - depth vertex)
__global__ void fill_r_depth_kernel(float* r, float lam, const int* corr, unsigned n_corr, const float* warped,
                                    const float* depth_mesh, const float* normals) {
    AFX_GRID_STRIDE(c, (long)n_corr) {
        const long v = corr[2 * c], px = corr[2 * c + 1];
        const float d[3] = {warped[3 * v] - depth_mesh[3 * px], warped[3 * v + 1] - depth_mesh[3 * px + 1],
                            warped[3 * v + 2] - depth_mesh[3 * px + 2]};
        r[c] = lam * dot3(normals + 3 * px, d);
    }
}

// fill_r_MRegKernel (src/MotionOptimization.cu:198-226): (T_node p - T_nb p) lambda; rows of a
// filtered neighbour are left as they are.
__global__ void fill_r_mreg_kernel(float* r, float lam, const float* nodes, const float* T, unsigned n,
                                   const uint32_t* knn, int Kreg) {
    AFX_GRID_STRIDE(c, (long)n) {
        float tc[3];
        mat4_point(T + 16 * c, nodes + 3 * c, tc);
        for (int i = 0; i < Kreg; ++i) {
            const uint32_t nb = knn[c * Kreg + i];
            if (nb >= n) continue;
            float tn[3];
            mat4_point(T + 16 * (long)nb, nodes + 3 * c, tn);
            const long row = (c * Kreg + i) * 3;
            for (int ax = 0; ax < 3; ++ax) r[row + ax] = (tc[ax] - tn[ax]) * lam;
        }
    }
}

// ---- contributing pairs (computeJTJAndJTrContrib*Kernel, src/MotionOptimization.cu:243-340) ----

__global__ void contrib_depth_count_kernel(unsigned* npairs, unsigned* njtr, const int* corr, unsigned n_corr,
                                           const float* knn_w, int K) {
    AFX_GRID_STRIDE(c, (long)n_corr) {
        const long v = corr[2 * c];
        unsigned nz = 0;
        for (int i = 0; i < K; ++i) nz += knn_w[v * K + i] != 0.f ? 1u : 0u;
        npairs[c] = nz * (nz + 1) / 2;
        njtr[c] = nz;
    }
}

__global__ void contrib_depth_write_kernel(int* pairs, unsigned* rows, const unsigned* n_pairs, int* jtr,
                                           const unsigned* n_jtr, const unsigned* poff, const unsigned* joff,
                                           const int* corr, unsigned n_corr, const uint32_t* knn_idx, const float* knn_w,
                                           int K) {
    const unsigned pbase = *n_pairs, jbase = *n_jtr;
    AFX_GRID_STRIDE(c, (long)n_corr) {
        const long v = corr[2 * c];
        unsigned p = pbase + poff[c], q = jbase + joff[c];
        for (int i = 0; i < K; ++i) {
            if (knn_w[v * K + i] == 0.f) continue;
            const int ni = (int)knn_idx[v * K + i];
            for (int j = i; j < K; ++j) {
                if (knn_w[v * K + j] == 0.f) continue;
                const int nj = (int)knn_idx[v * K + j];
                rows[p] = (unsigned)c;
                pairs[2 * p] = ni < nj ? ni : nj;
                pairs[2 * p + 1] = ni < nj ? nj : ni;
                ++p;
            }
            jtr[2 * q] = (int)c;
            jtr[2 * q + 1] = ni;
            ++q;
        }
    }
}

__global__ void contrib_mreg_count_kernel(unsigned* npairs, unsigned* njtr, unsigned n, const uint32_t* knn,
                                          int Kreg) {
    AFX_GRID_STRIDE(c, (long)n) {
        unsigned live = 0;
        for (int i = 0; i < Kreg; ++i) live += knn[c * Kreg + i] < n ? 1u : 0u;
        npairs[c] = 9 * live;
        njtr[c] = 6 * live;
    }
}

__global__ void contrib_mreg_write_kernel(int* pairs, unsigned* rows, unsigned row_offset, const unsigned* n_pairs,
                                          int* jtr, const unsigned* n_jtr, const unsigned* poff, const unsigned* joff,
                                          unsigned n, const uint32_t* knn, int Kreg) {
    const unsigned pbase = *n_pairs, jbase = *n_jtr;
    AFX_GRID_STRIDE(c, (long)n) {
        unsigned p = pbase + poff[c], q = jbase + joff[c];
        for (int i = 0; i < Kreg; ++i) {
            const uint32_t nb = knn[c * Kreg + i];
            if (nb >= n) continue;
            const unsigned row = (unsigned)(c * Kreg + i) * 3 + row_offset;
            const int a = (int)c, b = (int)nb;
            for (int j = 0; j < 3; ++j) {
                rows[p] = row + j;
                pairs[2 * p] = a < b ? a : b;
                pairs[2 * p + 1] = a < b ? b : a;
                rows[p + 1] = row + j;
                pairs[2 * (p + 1)] = a;
                pairs[2 * (p + 1) + 1] = a;
                rows[p + 2] = row + j;
                pairs[2 * (p + 2)] = b;
                pairs[2 * (p + 2) + 1] = b;
                p += 3;
                jtr[2 * q] = (int)(row + j);
                jtr[2 * q + 1] = a;
                jtr[2 * (q + 1)] = (int)(row + j);
                jtr[2 * (q + 1) + 1] = b;
                q += 2;
            }
        }
    }
}

__global__ void counters_add_kernel(unsigned* n_pairs, unsigned* n_jtr, const unsigned* tp, const unsigned* tj) {
    *n_pairs += *tp;
    *n_jtr += *tj;
}

// multiplyJTJContribPairsKernel (src/MotionOptimization.cu:342-356): J(row, a) J(row, b)^T, Mat6f
// column-major (entry (i, j) at j * 6 + i).
__global__ void multiply_pairs_kernel(float* out, const int* pairs, const unsigned* rows, unsigned n, const float* J,
                                      unsigned width) {
    AFX_GRID_STRIDE(t, (long)n * 36) {
        const long c = t / 36;
        const int e = (int)(t % 36), i = e % 6, j = e / 6;
        const long row = rows[c];
        const unsigned a = (unsigned)pairs[2 * c], b = (unsigned)pairs[2 * c + 1];
        if (a >= width || b >= width) continue;  // not a node of J: left unwritten
        const float* ja = J + 6 * (row * width + a);
        const float* jb = J + 6 * (row * width + b);
        out[c * 36 + e] = ja[i] * jb[j];
    }
}

// multiplyJTrContribElemsKernel (src/MotionOptimization.cu:371-383): J(row, node) r(row)
__global__ void multiply_jtr_kernel(float* out, const int* elems, unsigned n, const float* J, const float* r,
                                    unsigned width) {
    AFX_GRID_STRIDE(t, (long)n * 6) {
        const long c = t / 6;
        const int q = (int)(t % 6);
        const long row = elems[2 * c];
        const unsigned node = (unsigned)elems[2 * c + 1];
        if (node >= width) continue;  // not a node of J: left unwritten
        out[c * 6 + q] = J[6 * (row * width + node) + q] * r[row];
    }
}

// fillJTJKernel (src/MotionOptimization.cu:399-430): block (a, b) and, for a != b, its transpose at
// (b, a); rows jtj_width floats apart.
__global__ void fill_jtj_kernel(float* JTJ, const int* coords, const float* elems, unsigned n, unsigned ld) {
    AFX_GRID_STRIDE(t, (long)n * 36) {
        const long c = t / 36;
        const int e = (int)(t % 36), i = e % 6, j = e / 6;  // elems: Mat6f column-major
        const long a = coords[2 * c], b = coords[2 * c + 1];
        if (a < 0 || b < 0 || 6 * a + 5 >= (long)ld || 6 * b + 5 >= (long)ld) continue;  // outside the matrix
        const float v = elems[c * 36 + e];
        JTJ[(6 * a + i) * (long)ld + 6 * b + j] = v;
        if (a != b) JTJ[(6 * b + j) * (long)ld + 6 * a + i] = v;
    }
}

// fillJTrKernel (src/MotionOptimization.cu:447-456)
__global__ void fill_jtr_kernel(float* JTr, const int* coords, const float* elems, unsigned n) {
    AFX_GRID_STRIDE(t, (long)n * 6) {
        const long c = t / 6;
        const int q = (int)(t % 6);
        JTr[6 * (long)coords[2 * c + 1] + q] = elems[c * 6 + q];
    }
}

// ---- LU with partial pivoting (column-major, lda) ----

constexpr int kLuThreads = 1024;

// Column k: pivot search over rows k..n-1 (largest |a|, the first on ties), row swap, multipliers.
__global__ void __launch_bounds__(kLuThreads) lu_pivot_kernel(float* A, int n, int lda, int k, int* ipiv, int* info) {
    __shared__ float bv[kLuThreads];
    __shared__ int bi[kLuThreads];
    const int t = threadIdx.x;
    float best = -1.f;
    int arg = n;
    for (int i = k + t; i < n; i += kLuThreads) {
        const float v = fabsf(A[i + (long)k * lda]);
        if (v > best) {
            best = v;
            arg = i;
        }
    }
    bv[t] = best;
    bi[t] = arg;
    __syncthreads();
    for (int s = kLuThreads / 2; s > 0; s >>= 1) {
        if (t < s) {
            const float v = bv[t + s];
            const int i = bi[t + s];
            if (v > bv[t] || (v == bv[t] && i < bi[t])) {
                bv[t] = v;
                bi[t] = i;
            }
        }
        __syncthreads();
    }
    const int p = bi[0];
    const float piv = p < n ? A[p + (long)k * lda] : 0.f;
    if (t == 0) ipiv[k] = p + 1;  // 1-based, as getrf
    if (piv == 0.f) {             // uniform across the block
        if (t == 0 && *info == 0) *info = k + 1;
        return;
    }
    __syncthreads();  // every thread has read the pivot before the rows move
    if (p != k)
        for (int j = t; j < n; j += kLuThreads) {
            const float x = A[k + (long)j * lda];
            A[k + (long)j * lda] = A[p + (long)j * lda];
            A[p + (long)j * lda] = x;
        }
    __syncthreads();
    for (int i = k + 1 + t; i < n; i += kLuThreads) A[i + (long)k * lda] = A[i + (long)k * lda] / piv;
}

// Trailing update A[i][j] -= l[i] u[j] for i, j > k.
__global__ void lu_update_kernel(float* A, int n, int lda, int k, const int* info) {
    if (*info) return;
    const long m = n - k - 1;
    AFX_GRID_STRIDE(t, m * m) {
        const int i = k + 1 + (int)(t % m), j = k + 1 + (int)(t / m);
        A[i + (long)j * lda] = A[i + (long)j * lda] - A[i + (long)k * lda] * A[k + (long)j * lda];
    }
}

// getrs (no transpose): row interchanges, L y = P b (unit diagonal), U x = y; one block.
__global__ void __launch_bounds__(kLuThreads) lu_solve_kernel(const float* A, int n, int lda, const int* ipiv,
                                                              float* x, const int* info) {
    if (*info) return;
    const int t = threadIdx.x;
    if (t == 0)
        for (int k = 0; k < n; ++k) {
            const int p = ipiv[k] - 1;
            if (p != k) {
                const float s = x[k];
                x[k] = x[p];
                x[p] = s;
            }
        }
    __syncthreads();
    for (int k = 0; k < n; ++k) {  // forward: x[i] -= l[i][k] x[k], i > k
        const float xk = x[k];
        for (int i = k + 1 + t; i < n; i += kLuThreads) x[i] = x[i] - A[i + (long)k * lda] * xk;
        __syncthreads();
    }
    for (int k = n - 1; k >= 0; --k) {  // backward
        if (t == 0) x[k] = x[k] / A[k + (long)k * lda];
        __syncthreads();
        const float xk = x[k];
        for (int i = t; i < k; i += kLuThreads) x[i] = x[i] - A[i + (long)k * lda] * xk;
        __syncthreads();
    }
}

}  // namespace

}  // namespace afx

using namespace afx;

extern "C" {

int afx_fill_j_depth(float* J, float weight, unsigned rows, unsigned width, const int* corr, unsigned n_corr,
                     const float* mesh, const uint32_t* knn_idx, const float* knn_w, int K, const float* normals,
                     void* stream) {
    if (!J || (n_corr && (!corr || !mesh || !knn_idx || !knn_w || !normals)) || K < 1 || K > 8 || n_corr > rows)
        return AFX_ERR_INVALID_ARGUMENT;
    if (!n_corr) return AFX_OK;
    fill_j_depth_kernel<<<grid_for(n_corr, 128), 128, 0, as_stream(stream)>>>(J, weight, width, corr, n_corr, mesh,
                                                                                 knn_idx, knn_w, K, normals);
    AFX_LAUNCH_CHECK();
    return AFX_OK;
}

int afx_fill_j_mreg(float* J, float weight, unsigned rows, unsigned width, const float* nodes, unsigned n_nodes,
                    const uint32_t* knn_idx, int Kreg, void* stream) {
    if (!J || (n_nodes && (!nodes || !knn_idx)) || Kreg < 1 || Kreg > 8 || (unsigned long)n_nodes * Kreg * 3 > rows ||
        n_nodes > width)
        return AFX_ERR_INVALID_ARGUMENT;
    if (!n_nodes) return AFX_OK;
    fill_j_mreg_kernel<<<grid_for(n_nodes, 128), 128, 0, as_stream(stream)>>>(J, weight, width, nodes, n_nodes, knn_idx,
                                                                                Kreg);
    AFX_LAUNCH_CHECK();
    return AFX_OK;
}

int afx_fill_r_depth(float* r, float weight, const int* corr, unsigned n_corr, const float* warped,
                     const float* depth_mesh, const float* normals, void* stream) {
    if (!r || (n_corr && (!corr || !warped || !depth_mesh || !normals))) return AFX_ERR_INVALID_ARGUMENT;
    if (!n_corr) return AFX_OK;
    fill_r_depth_kernel<<<grid_for(n_corr, 256), 256, 0, as_stream(stream)>>>(r, weight, corr, n_corr, warped,
                                                                                depth_mesh, normals);
    AFX_LAUNCH_CHECK();
    return AFX_OK;
}

int afx_fill_r_mreg(float* r, float weight, const float* nodes, const float* transforms, unsigned n_nodes,
                    const uint32_t* knn_idx, int Kreg, void* stream) {
    if (!r || (n_nodes && (!nodes || !transforms || !knn_idx)) || Kreg < 1 || Kreg > 8) return AFX_ERR_INVALID_ARGUMENT;
    if (!n_nodes) return AFX_OK;
    fill_r_mreg_kernel<<<grid_for(n_nodes, 128), 128, 0, as_stream(stream)>>>(r, weight, nodes, transforms, n_nodes,
                                                                                knn_idx, Kreg);
    AFX_LAUNCH_CHECK();
    return AFX_OK;
}

size_t afx_jtj_contrib_workspace_size(long rows) {
    if (rows < 0) return 0;
    const size_t a = (((size_t)rows * 4 + 255) / 256) * 256;
    const size_t s = ((scan_workspace_size(rows) + 255) / 256) * 256;
    return 4 * a + 2 * s + 512;
}

static int contrib_common(long rows, void* ws, size_t ws_bytes, unsigned** cp, unsigned** cj, unsigned** op,
                          unsigned** oj, unsigned** tp, unsigned** tj, void** sp, void** sj) {
    if (ws_bytes < afx_jtj_contrib_workspace_size(rows) || !ws) return AFX_ERR_WORKSPACE;
    const size_t a = (((size_t)rows * 4 + 255) / 256) * 256;
    const size_t s = ((scan_workspace_size(rows) + 255) / 256) * 256;
    char* q = static_cast<char*>(ws);
    *cp = (unsigned*)q;
    *cj = (unsigned*)(q + a);
    *op = (unsigned*)(q + 2 * a);
    *oj = (unsigned*)(q + 3 * a);
    *sp = q + 4 * a;
    *sj = q + 4 * a + s;
    *tp = (unsigned*)(q + 4 * a + 2 * s);
    *tj = (unsigned*)(q + 4 * a + 2 * s + 256);
    return AFX_OK;
}

int afx_jtj_contrib_depth(int* pairs, unsigned* rows, unsigned* n_pairs, int* jtr_elems, unsigned* n_jtr,
                          const int* corr, unsigned n_corr, const uint32_t* knn_idx, const float* knn_w, int K,
                          void* workspace, size_t workspace_bytes, void* stream) {
    if (!pairs || !rows || !n_pairs || !jtr_elems || !n_jtr || K < 1 || K > 8 ||
        (n_corr && (!corr || !knn_idx || !knn_w)))
        return AFX_ERR_INVALID_ARGUMENT;
    if (!n_corr) return AFX_OK;
    unsigned *cp, *cj, *op, *oj, *tp, *tj;
    void *sp, *sj;
    int rc = contrib_common(n_corr, workspace, workspace_bytes, &cp, &cj, &op, &oj, &tp, &tj, &sp, &sj);
    if (rc) return rc;
    cudaStream_t st = as_stream(stream);
    contrib_depth_count_kernel<<<grid_for(n_corr, 256), 256, 0, st>>>(cp, cj, corr, n_corr, knn_w, K);
    AFX_LAUNCH_CHECK();
    rc = scan_exclusive(cp, op, n_corr, tp, sp, st);
    if (!rc) rc = scan_exclusive(cj, oj, n_corr, tj, sj, st);
    if (rc) return rc;
    contrib_depth_write_kernel<<<grid_for(n_corr, 128), 128, 0, st>>>(pairs, rows, n_pairs, jtr_elems, n_jtr, op, oj,
                                                                         corr, n_corr, knn_idx, knn_w, K);
    AFX_LAUNCH_CHECK();
    counters_add_kernel<<<1, 1, 0, st>>>(n_pairs, n_jtr, tp, tj);
    AFX_LAUNCH_CHECK();
    return AFX_OK;
}

int afx_jtj_contrib_mreg(int* pairs, unsigned* rows, unsigned row_offset, unsigned* n_pairs, int* jtr_elems,
                         unsigned* n_jtr, unsigned n_nodes, const uint32_t* knn_idx, int Kreg, void* workspace,
                         size_t workspace_bytes, void* stream) {
    if (!pairs || !rows || !n_pairs || !jtr_elems || !n_jtr || Kreg < 1 || Kreg > 8 || (n_nodes && !knn_idx))
        return AFX_ERR_INVALID_ARGUMENT;
    if (!n_nodes) return AFX_OK;
    unsigned *cp, *cj, *op, *oj, *tp, *tj;
    void *sp, *sj;
    int rc = contrib_common(n_nodes, workspace, workspace_bytes, &cp, &cj, &op, &oj, &tp, &tj, &sp, &sj);
    if (rc) return rc;
    cudaStream_t st = as_stream(stream);
    contrib_mreg_count_kernel<<<grid_for(n_nodes, 256), 256, 0, st>>>(cp, cj, n_nodes, knn_idx, Kreg);
    AFX_LAUNCH_CHECK();
    rc = scan_exclusive(cp, op, n_nodes, tp, sp, st);
    if (!rc) rc = scan_exclusive(cj, oj, n_nodes, tj, sj, st);
    if (rc) return rc;
    contrib_mreg_write_kernel<<<grid_for(n_nodes, 128), 128, 0, st>>>(pairs, rows, row_offset, n_pairs, jtr_elems,
                                                                        n_jtr, op, oj, n_nodes, knn_idx, Kreg);
    AFX_LAUNCH_CHECK();
    counters_add_kernel<<<1, 1, 0, st>>>(n_pairs, n_jtr, tp, tj);
    AFX_LAUNCH_CHECK();
    return AFX_OK;
}

int afx_multiply_jtj_pairs(float* out, const int* pairs, const unsigned* rows, unsigned n_pairs, const float* J,
                           unsigned width, void* stream) {
    if (!out || (n_pairs && (!pairs || !rows || !J))) return AFX_ERR_INVALID_ARGUMENT;
    if (!n_pairs) return AFX_OK;
    multiply_pairs_kernel<<<grid_for((long)n_pairs * 36, 256), 256, 0, as_stream(stream)>>>(out, pairs, rows, n_pairs,
                                                                                               J, width);
    AFX_LAUNCH_CHECK();
    return AFX_OK;
}

int afx_multiply_jtr_elems(float* out, const int* elems, unsigned n_elems, const float* J, const float* r,
                           unsigned width, void* stream) {
    if (!out || (n_elems && (!elems || !J || !r))) return AFX_ERR_INVALID_ARGUMENT;
    if (!n_elems) return AFX_OK;
    multiply_jtr_kernel<<<grid_for((long)n_elems * 6, 256), 256, 0, as_stream(stream)>>>(out, elems, n_elems, J, r,
                                                                                            width);
    AFX_LAUNCH_CHECK();
    return AFX_OK;
}

int afx_fill_jtj(float* JTJ, const int* coords, const float* elems, unsigned n_elems, unsigned jtj_width,
                 void* stream) {
    if (!JTJ || (n_elems && (!coords || !elems))) return AFX_ERR_INVALID_ARGUMENT;
    if (!n_elems) return AFX_OK;
    fill_jtj_kernel<<<grid_for((long)n_elems * 36, 256), 256, 0, as_stream(stream)>>>(JTJ, coords, elems, n_elems,
                                                                                         jtj_width);
    AFX_LAUNCH_CHECK();
    return AFX_OK;
}

int afx_fill_jtr(float* JTr, const int* coords, const float* elems, unsigned n_elems, void* stream) {
    if (!JTr || (n_elems && (!coords || !elems))) return AFX_ERR_INVALID_ARGUMENT;
    if (!n_elems) return AFX_OK;
    fill_jtr_kernel<<<grid_for((long)n_elems * 6, 256), 256, 0, as_stream(stream)>>>(JTr, coords, elems, n_elems);
    AFX_LAUNCH_CHECK();
    return AFX_OK;
}

size_t afx_lu_solve_workspace_size(int n, int lda) {
    if (n < 0 || lda < n) return 0;
    return (((size_t)lda * n * 4 + 255) / 256) * 256 + 256;
}

int afx_lu_solve(float* x, const float* A, int n, int lda, const float* b, int* ipiv, void* workspace,
                 size_t workspace_bytes, void* stream) {
    if (!x || !A || !b || !ipiv || n < 1 || lda < n) return AFX_ERR_INVALID_ARGUMENT;
    if (!workspace || workspace_bytes < afx_lu_solve_workspace_size(n, lda)) return AFX_ERR_WORKSPACE;
    cudaStream_t st = as_stream(stream);
    float* LU = static_cast<float*>(workspace);
    int* info = reinterpret_cast<int*>(static_cast<char*>(workspace) + (((size_t)lda * n * 4 + 255) / 256) * 256);
    AFX_CUDA(cudaMemcpyAsync(LU, A, (size_t)lda * n * 4, cudaMemcpyDeviceToDevice, st));
    AFX_CUDA(cudaMemsetAsync(info, 0, 4, st));
    for (int k = 0; k < n; ++k) {
        lu_pivot_kernel<<<1, kLuThreads, 0, st>>>(LU, n, lda, k, ipiv, info);
        AFX_LAUNCH_CHECK();
        if (k + 1 < n) {
            const long m = n - k - 1;
            lu_update_kernel<<<grid_for(m * m, 256), 256, 0, st>>>(LU, n, lda, k, info);
            AFX_LAUNCH_CHECK();
        }
    }
    AFX_CUDA(cudaMemcpyAsync(x, b, (size_t)n * 4, cudaMemcpyDeviceToDevice, st));
    lu_solve_kernel<<<1, kLuThreads, 0, st>>>(LU, n, lda, ipiv, x, info);
    AFX_LAUNCH_CHECK();
    int h_info = 0;
    AFX_CUDA(cudaMemcpyAsync(&h_info, info, 4, cudaMemcpyDeviceToHost, st));
    AFX_CUDA(cudaStreamSynchronize(st));
    return h_info ? AFX_ERR_SINGULAR : AFX_OK;
}

}  // extern "C"
