// afx_gn.cu -- Gauss-Newton for the motion graph: residuals, block-sparse J^T J / J^T r
// assembly and a block-Jacobi preconditioned conjugate-gradient solve.
//
// The reference fills a dense Jacobian ((C + 3 K_reg N) x N Vec6f), lists contributing
// node pairs with atomics, sorts and reduces them with thrust, scatters into a dense
// (6N)^2 matrix and solves it with cuSOLVER LU in FP32 (src/VolumeFusion.cu:454-691,
// src/MotionOptimization.cu).  Here J is never stored: each node's warp walks the
// vertices that reference it (ascending vertex order, which is ascending correspondence
// order) and accumulates its 6x6 blocks J_a^T J_b in binary32 in a fixed order --
// depth rows by ascending correspondence, then regularisation rows by ascending row.
// Diagonal blocks without any contribution keep the identity (runInitIdentityKernel).
// J^T J depends only on the canonical geometry, weights and correspondences, so it is
// assembled once per ICP iteration; J^T r is rebuilt every Gauss-Newton iteration.
// The solve is a block-Jacobi PCG in one cooperative kernel: FP32 block SpMV, FP64 dot
// products and FP64 6x6 block inverses.
#include <cfloat>
#include <cstring>

#include "afx_gn.h"

namespace afx {

AFX_D void grad_rows(const float* p, float G[3][6]) {
    G[0][0] = 0.f;   G[0][1] = p[2];  G[0][2] = -p[1]; G[0][3] = 1.f; G[0][4] = 0.f; G[0][5] = 0.f;
    G[1][0] = -p[2]; G[1][1] = 0.f;   G[1][2] = p[0];  G[1][3] = 0.f; G[1][4] = 1.f; G[1][5] = 0.f;
    G[2][0] = p[1];  G[2][1] = -p[0]; G[2][2] = 0.f;   G[2][3] = 0.f; G[2][4] = 0.f; G[2][5] = 1.f;
}

// Depth-row Jacobian entry block for one slot (fill_J_DepthKernel, src/MotionOptimization.cu:51-60)
AFX_D void jdepth(const float* n, float w, const float G[3][6], float lam, float* J) {
    if (w < 1.e-4f) {
#pragma unroll
        for (int q = 0; q < 6; ++q) J[q] = 0.f;
        return;
    }
    float nw[3] = {n[0] * w, n[1] * w, n[2] * w};
#pragma unroll
    for (int q = 0; q < 6; ++q) J[q] = (nw[0] * G[0][q] + (nw[1] * G[1][q] + nw[2] * G[2][q])) * lam;
}

// ---- per-frame node lists ----

__global__ void lst_count_kernel(GnArgs a) {
    long m = min((long)*a.mesh_count, a.m_max);
    long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (t >= m * a.k) return;
    if (a.mw[t] == 0.f) return;
    uint32_t node = a.midx[t];
    if (node >= (uint32_t)*a.n_nodes) return;
    atomicAdd(a.b.lcnt + node, 1u);
}

__global__ void lst_fill_kernel(GnArgs a) {
    long m = min((long)*a.mesh_count, a.m_max);
    long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (t >= m * a.k) return;
    if (a.mw[t] == 0.f) return;
    uint32_t node = a.midx[t];
    if (node >= (uint32_t)*a.n_nodes) return;
    unsigned p = a.b.loff[node] + atomicAdd(a.b.lcur + node, 1u);
    a.b.lst[p] = (unsigned)t;
}

__global__ void in_count_kernel(GnArgs a) {
    int n = min(*a.n_nodes, a.n_max);
    long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (t >= (long)n * a.kreg) return;
    uint32_t nb = a.gidx[t];
    if (nb >= (uint32_t)n) return;
    atomicAdd(a.b.icnt + nb, 1u);
}

__global__ void in_fill_kernel(GnArgs a) {
    int n = min(*a.n_nodes, a.n_max);
    long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (t >= (long)n * a.kreg) return;
    uint32_t nb = a.gidx[t];
    if (nb >= (uint32_t)n) return;
    unsigned p = a.b.ioff[nb] + atomicAdd(a.b.icur + nb, 1u);
    a.b.ilst[p] = (unsigned)t;
}

// Sort each node's list ascending (bitonic in shared memory); one CTA per node.
__global__ void __launch_bounds__(256) seg_sort_kernel(unsigned* lst, const unsigned* off, const int* n_nodes, int n_max,
                                                       int* error) {
    __shared__ unsigned s[kSegMax];
    const int a = blockIdx.x;
    if (a >= min(*n_nodes, n_max)) return;
    const unsigned o = off[a];
    const int len = (int)(off[a + 1] - o);
    if (len <= 1) return;
    if (len > kSegMax) {
        if (threadIdx.x == 0) atomicOr(error, ERRF_CAPACITY);
        return;
    }
    int P = 1;
    while (P < len) P <<= 1;
    for (int i = threadIdx.x; i < P; i += blockDim.x) s[i] = i < len ? lst[o + i] : 0xffffffffu;
    __syncthreads();
    for (int size = 2; size <= P; size <<= 1)
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            for (int pidx = threadIdx.x; pidx < P / 2; pidx += blockDim.x) {
                int i = 2 * stride * (pidx / stride) + (pidx % stride), j = i + stride;
                bool asc = (i & size) == 0;
                unsigned x = s[i], y = s[j];
                if ((y < x) == asc) {
                    s[i] = y;
                    s[j] = x;
                }
            }
            __syncthreads();
        }
    for (int i = threadIdx.x; i < len; i += blockDim.x) lst[o + i] = s[i];
}

// ---- per-ICP assembly ----

// Neighbour discovery: distinct nodes b != a sharing a corresponding vertex with a (both
// weights non-zero) or joined to a by a regularisation edge.  One warp per node, bitmap in
// shared memory, so the list comes out sorted.
__global__ void __launch_bounds__(32 * kGnWarps) nbr_discover_kernel(GnArgs a, int words) {
    extern __shared__ unsigned bm[];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int node = blockIdx.x * kGnWarps + w;
    const int n = min(*a.n_nodes, a.n_max);
    unsigned* my = bm + (long)w * words;
    for (int i = lane; i < words; i += 32) my[i] = 0u;
    __syncwarp();
    if (node < n) {
        const unsigned o = a.b.loff[node], e = a.b.loff[node + 1];
        for (unsigned t = o + lane; t < e; t += 32) {
            unsigned ent = a.b.lst[t];
            long v = ent / a.k;
            if (a.corr_of_vertex[v] < 0) continue;
            for (int s = 0; s < a.k; ++s) {
                if (a.mw[v * a.k + s] == 0.f) continue;
                uint32_t bnode = a.midx[v * a.k + s];
                if (bnode != (uint32_t)node && bnode < (uint32_t)n) atomicOr(my + (bnode >> 5), 1u << (bnode & 31));
            }
        }
        for (int kk = lane; kk < a.kreg; kk += 32) {
            uint32_t nb = a.gidx[(long)node * a.kreg + kk];
            if (nb < (uint32_t)n && nb != (uint32_t)node) atomicOr(my + (nb >> 5), 1u << (nb & 31));
        }
        for (unsigned t = a.b.ioff[node] + lane; t < a.b.ioff[node + 1]; t += 32) {
            unsigned x = a.b.ilst[t] / a.kreg;
            if (x != (unsigned)node) atomicOr(my + (x >> 5), 1u << (x & 31));
        }
    }
    __syncwarp();
    if (node >= n) return;
    // ordered extraction
    int base = 0;
    for (int w0 = 0; w0 < words; w0 += 32) {
        int wi = w0 + lane;
        unsigned bits = wi < words ? my[wi] : 0u;
        int c = __popc(bits);
        int incl = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        int pos = base + incl - c;
        while (bits) {
            int bit = __ffs(bits) - 1;
            bits &= bits - 1;
            if (pos < kMaxNbr) a.b.nbr[(long)node * kMaxNbr + pos] = wi * 32 + bit;
            ++pos;
        }
        base += __shfl_sync(0xffffffffu, incl, 31);
    }
    if (lane == 0) {
        a.b.nbr_cnt[node] = min(base, kMaxNbr);
        if (base > kMaxNbr) atomicOr(a.error, ERRF_CAPACITY);
    }
}

// For neighbour slots below the diagonal, find the owner's slot (binary search).
__global__ void nbr_ref_kernel(GnArgs a) {
    const int n = min(*a.n_nodes, a.n_max);
    long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (t >= (long)n * kMaxNbr) return;
    int node = (int)(t / kMaxNbr), u = (int)(t % kMaxNbr);
    if (u >= a.b.nbr_cnt[node]) return;
    int bnode = a.b.nbr[t];
    if (bnode > node) {
        a.b.nbr_ref[t] = (int)t;
        return;
    }
    const int* L = a.b.nbr + (long)bnode * kMaxNbr;
    int lo = 0, hi = a.b.nbr_cnt[bnode] - 1, f = -1;
    while (lo <= hi) {
        int mid = (lo + hi) >> 1;
        if (L[mid] == node) {
            f = mid;
            break;
        }
        if (L[mid] < node) lo = mid + 1;
        else hi = mid - 1;
    }
    if (f < 0) {
        atomicOr(a.error, ERRF_CAPACITY);
        a.b.nbr_ref[t] = 0;
        return;
    }
    a.b.nbr_ref[t] = -((int)((long)bnode * kMaxNbr + f) + 1);
}

AFX_D int find_slot(const int* L, int cnt, int b) {
    int lo = 0, hi = cnt - 1;
    while (lo <= hi) {
        int mid = (lo + hi) >> 1;
        if (L[mid] == b) return mid;
        if (L[mid] < b) lo = mid + 1;
        else hi = mid - 1;
    }
    return -1;
}

// J^T J: node a's warp accumulates D_a and its upper blocks (a, b > a).  Lane l owns block
// entries l and l + 32 of every block; each entry is summed in a fixed sequential order.
__global__ void __launch_bounds__(32 * kGnWarps) jtj_assemble_kernel(GnArgs a) {
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int node = blockIdx.x * kGnWarps + w;
    const int n = min(*a.n_nodes, a.n_max);
    if (node >= n) return;
    const int* L = a.b.nbr + (long)node * kMaxNbr;
    const int cnt = a.b.nbr_cnt[node];
    float* D = a.b.diag + (long)node * 36;
    float* B = a.b.blocks + (long)node * kMaxNbr * 36;
    const int e0 = lane, e1 = lane + 32;  // entries this lane owns (e1 valid for lanes 0..3)
    const int i0 = e0 / 6, j0 = e0 % 6, i1 = e1 / 6, j1 = e1 % 6;
    // zero this node's accumulators
    float d0 = 0.f, d1 = 0.f;
    for (int u = 0; u < cnt; ++u) {
        if (L[u] <= node) continue;
        B[u * 36 + e0] = 0.f;
        if (e1 < 36) B[u * 36 + e1] = 0.f;
    }
    bool touched = false;
    const unsigned o = a.b.loff[node], e = a.b.loff[node + 1];
    for (unsigned t = o; t < e; ++t) {
        unsigned ent = a.b.lst[t];
        long v = ent / a.k;
        int s = (int)(ent % a.k);
        int c = a.corr_of_vertex[v];
        if (lane == 0) a.b.jc[t] = c;
        if (c < 0) continue;
        touched = true;
        int px = a.corr[2 * (long)c + 1];
        const float* nrm = a.normals + 3 * (long)px;
        float G[3][6];
        grad_rows(a.mesh + 3 * v, G);
        float Ja[6];
        jdepth(nrm, a.mw[v * a.k + s], G, a.lam_d, Ja);
        if (lane == 0)
            for (int q = 0; q < 6; ++q) a.b.jrow[(long)t * 6 + q] = Ja[q];
        for (int tt = 0; tt < a.k; ++tt) {
            float wt = a.mw[v * a.k + tt];
            if (wt == 0.f) continue;
            uint32_t bnode = a.midx[v * a.k + tt];
            if (bnode < (uint32_t)node) continue;
            float Jb[6];
            jdepth(nrm, wt, G, a.lam_d, Jb);
            if (bnode == (uint32_t)node) {
                d0 = d0 + Ja[i0] * Jb[j0];
                if (e1 < 36) d1 = d1 + Ja[i1] * Jb[j1];
            } else {
                int u = find_slot(L, cnt, (int)bnode);
                if (u < 0) continue;
                float* blk = B + u * 36;
                blk[e0] = blk[e0] + Ja[i0] * Jb[j0];
                if (e1 < 36) blk[e1] = blk[e1] + Ja[i1] * Jb[j1];
            }
        }
    }
    // regularisation rows in ascending row order: incoming edges x -> node with x < node,
    // then node's own edges, then incoming edges with x > node (src/MotionOptimization.cu:298-340)
    const unsigned io = a.b.ioff[node], ie = a.b.ioff[node + 1];
    unsigned it = io;
    auto reg_row = [&](int src, int kk) {
        uint32_t nb = a.gidx[(long)src * a.kreg + kk];
        float G[3][6];
        grad_rows(a.nodes + 3 * (long)src, G);
        for (int ax = 0; ax < 3; ++ax) {
            float g[6], gn[6];
#pragma unroll
            for (int q = 0; q < 6; ++q) {
                g[q] = G[ax][q] * a.lam_r;
                gn[q] = -g[q];
            }
            // this node is `src` (coefficient +g) or `nb` (coefficient -g)
            const float* Jn = (src == node) ? g : gn;
            d0 = d0 + Jn[i0] * Jn[j0];
            if (e1 < 36) d1 = d1 + Jn[i1] * Jn[j1];
            int other = (src == node) ? (int)nb : src;
            if (other > node) {
                const float* Jo = (src == node) ? gn : g;
                int u = find_slot(L, cnt, other);
                if (u >= 0) {
                    float* blk = B + u * 36;
                    blk[e0] = blk[e0] + Jn[i0] * Jo[j0];
                    if (e1 < 36) blk[e1] = blk[e1] + Jn[i1] * Jo[j1];
                }
            }
        }
        touched = true;
    };
    while (it < ie && a.b.ilst[it] / a.kreg < (unsigned)node) {
        unsigned ent = a.b.ilst[it++];
        reg_row((int)(ent / a.kreg), (int)(ent % a.kreg));
    }
    for (int kk = 0; kk < a.kreg; ++kk) {
        uint32_t nb = a.gidx[(long)node * a.kreg + kk];
        if (nb >= (uint32_t)n) continue;
        reg_row(node, kk);
    }
    while (it < ie) {
        unsigned ent = a.b.ilst[it++];
        reg_row((int)(ent / a.kreg), (int)(ent % a.kreg));
    }
    if (!touched) {  // identity diagonal block (src/VolumeFusion.cu:637-640)
        d0 = (i0 == j0) ? 1.f : 0.f;
        d1 = (i1 == j1) ? 1.f : 0.f;
    }
    D[e0] = d0;
    if (e1 < 36) D[e1] = d1;
}

// FP64 inverse of each diagonal block (Gauss-Jordan with partial pivoting).
__global__ void diag_inverse_kernel(GnArgs a) {
    int node = blockIdx.x * blockDim.x + threadIdx.x;
    int n = min(*a.n_nodes, a.n_max);
    if (node >= n) return;
    double m[6][12];
    const float* D = a.b.diag + (long)node * 36;
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 12; ++j) m[i][j] = j < 6 ? (double)D[i * 6 + j] : (j - 6 == i ? 1.0 : 0.0);
    bool ok = true;
    for (int c = 0; c < 6 && ok; ++c) {
        int p = c;
        for (int r = c + 1; r < 6; ++r)
            if (fabs(m[r][c]) > fabs(m[p][c])) p = r;
        if (m[p][c] == 0.0) {
            ok = false;
            break;
        }
        if (p != c)
            for (int j = 0; j < 12; ++j) {
                double t = m[p][j];
                m[p][j] = m[c][j];
                m[c][j] = t;
            }
        double d = m[c][c];
        for (int j = 0; j < 12; ++j) m[c][j] /= d;
        for (int r = 0; r < 6; ++r)
            if (r != c) {
                double f = m[r][c];
                for (int j = 0; j < 12; ++j) m[r][j] -= f * m[c][j];
            }
    }
    double* out = a.b.minv + (long)node * 36;
    if (!ok) {
        atomicOr(a.error, ERRF_SINGULAR);
        for (int i = 0; i < 36; ++i) out[i] = 0.0;
        return;
    }
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 6; ++j) out[i * 6 + j] = m[i][j + 6];
}

// ---- per-GN-iteration kernels ----

constexpr int kEnergyBlocks = 256;

// fill_r_DepthKernel / fill_r_MRegKernel + runSquareKernel + reductions
// (src/MotionOptimization.cu:163-227, src/VolumeFusion.cu:575-588); energies in FP64.
__global__ void __launch_bounds__(256) residual_kernel(GnArgs a, const float* warped, const float* T_pending) {
    if (a.b.state->done) return;
    __shared__ double sd[8], sr[8];
    const long C = min((long)*a.corr_count, a.c_max);
    const int n = min(*a.n_nodes, a.n_max);
    const long R = (long)n * a.kreg;
    double ed = 0.0, er = 0.0;
    const long stride = (long)gridDim.x * blockDim.x;
    for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < C; c += stride) {
        long v = a.corr[2 * c], px = a.corr[2 * c + 1];
        const float* wv = warped + 3 * v;
        const float* f = a.frame + 3 * px;
        float d[3] = {wv[0] - f[0], wv[1] - f[1], wv[2] - f[2]};
        float r = a.lam_d * dot3(a.normals + 3 * px, d);
        a.b.rdepth[c] = r;
        ed += (double)(r * r);
    }
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < R; t += stride) {
        int i = (int)(t / a.kreg);
        uint32_t nb = a.gidx[t];
        float* rr = a.b.rreg + 3 * t;
        if (nb >= (uint32_t)n) {
            rr[0] = rr[1] = rr[2] = 0.f;
            continue;
        }
        float tc[3], tn[3];
        mat4_point(T_pending + 16 * (long)i, a.nodes + 3 * (long)i, tc);
        mat4_point(T_pending + 16 * (long)nb, a.nodes + 3 * (long)i, tn);
        for (int ax = 0; ax < 3; ++ax) {
            float r = (tc[ax] - tn[ax]) * a.lam_r;
            rr[ax] = r;
            er += (double)(r * r);
        }
    }
    ed = warp_sum(ed);
    er = warp_sum(er);
    if ((threadIdx.x & 31) == 0) {
        sd[threadIdx.x >> 5] = ed;
        sr[threadIdx.x >> 5] = er;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double x = 0, y = 0;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) {
            x += sd[i];
            y += sr[i];
        }
        a.b.epart[2 * blockIdx.x] = x;
        a.b.epart[2 * blockIdx.x + 1] = y;
    }
}

// Energy test and commit decision (src/VolumeFusion.cu:589-598).
__global__ void __launch_bounds__(kEnergyBlocks) energy_kernel(GnArgs a, int iter) {
    GnState* s = a.b.state;
    if (s->done) return;
    __shared__ double sd[kEnergyBlocks / 32], sr[kEnergyBlocks / 32];
    // one partial pair per thread, fixed-order tree: the same totals on every run
    double ed = warp_sum(a.b.epart[2 * threadIdx.x]);
    double er = warp_sum(a.b.epart[2 * threadIdx.x + 1]);
    if ((threadIdx.x & 31) == 0) {
        sd[threadIdx.x >> 5] = ed;
        sr[threadIdx.x >> 5] = er;
    }
    __syncthreads();
    if (threadIdx.x != 0) return;
    ed = 0;
    er = 0;
    for (int i = 0; i < kEnergyBlocks / 32; ++i) {
        ed += sd[i];
        er += sr[i];
    }
    double e = ed + er;
    s->e_last = e;
    s->e_depth = ed;
    s->e_reg = er;
    if (s->e_prev - e < (double)a.min_step) {
        s->done = 1;
        return;
    }
    s->e_prev = e;
    s->commit = iter != 0;
    s->iters = iter + 1;
}

__global__ void commit_kernel(GnArgs a, float* T_committed, const float* T_pending) {
    if (a.b.state->done || !a.b.state->commit) return;
    const int n = min(*a.n_nodes, a.n_max);
    long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (t < (long)n * 16) T_committed[t] = T_pending[t];
}

// J^T r, one warp per node: lanes 0..5 each own one entry and sum in the fixed order.
__global__ void __launch_bounds__(32 * kGnWarps) jtr_kernel(GnArgs a) {
    if (a.b.state->done) return;
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int node = blockIdx.x * kGnWarps + w;
    const int n = min(*a.n_nodes, a.n_max);
    if (node >= n) return;
    const int q = lane < 6 ? lane : 0;
    float acc = 0.f;
    const unsigned o = a.b.loff[node], e = a.b.loff[node + 1];
    // J rows were formed once per ICP iteration by jtj_assemble_kernel (same values, same order)
    for (unsigned t = o; t < e; ++t) {
        int c = a.b.jc[t];
        if (c < 0) continue;
        acc = acc + a.b.jrow[(long)t * 6 + q] * a.b.rdepth[c];
    }
    const unsigned io = a.b.ioff[node], ie = a.b.ioff[node + 1];
    unsigned it = io;
    auto reg_row = [&](int src, int kk) {
        float G[3][6];
        grad_rows(a.nodes + 3 * (long)src, G);
        for (int ax = 0; ax < 3; ++ax) {
            float g = G[ax][q] * a.lam_r;
            float jn = (src == node) ? g : -g;
            acc = acc + jn * a.b.rreg[((long)src * a.kreg + kk) * 3 + ax];
        }
    };
    while (it < ie && a.b.ilst[it] / a.kreg < (unsigned)node) {
        unsigned ent = a.b.ilst[it++];
        reg_row((int)(ent / a.kreg), (int)(ent % a.kreg));
    }
    for (int kk = 0; kk < a.kreg; ++kk) {
        uint32_t nb = a.gidx[(long)node * a.kreg + kk];
        if (nb >= (uint32_t)n) continue;
        reg_row(node, kk);
    }
    while (it < ie) {
        unsigned ent = a.b.ilst[it++];
        reg_row((int)(ent / a.kreg), (int)(ent % a.kreg));
    }
    if (lane < 6) a.b.jtr[(long)node * 6 + lane] = acc;
}

// ---- PCG (cooperative, persistent) ----
//
// Only ceil(n / kGnWarps) CTAs (at most the launched grid) take part; the others leave at once.
// Each iteration has two grid barriers: after A p (reduces p.Ap) and after the r / z update
// (reduces r.z and r.r).  The new search direction p_k = z_k + beta p_{k-1} is formed in the
// A p phase (double-buffered p, so neighbours' values are computed on the fly from z and the
// previous p without a third barrier).  Reductions are finished by the last CTA to arrive, in
// CTA order, so every CTA sees the same FP64 totals.

struct PcgArgs {
    GnArgs g;
    float* T_pending;
    int iters;
    double tol;  // <= 0: run exactly `iters` iterations
};

constexpr int kRed = 4;  // reduction slots per CTA

// Arrive at the barrier with this CTA's partials; the last CTA sums all partials (fixed order)
// into totals and releases the others.  Returns false if the bounded wait gave up.
AFX_D bool grid_reduce_sync(unsigned* bar, int active, double* partial, double* totals, const double* mine, int nslots,
                            double* out, int* err) {
    __shared__ int s_ok;
    __shared__ double s_tot[kRed];
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int i = 0; i < nslots; ++i) __stcg(partial + (long)blockIdx.x * kRed + i, mine[i]);
        volatile unsigned* gen = bar + 1;
        unsigned g = *gen;
        __threadfence();
        unsigned arrived = atomicAdd(bar, 1u) + 1;
        s_ok = 1;
        if (arrived == (unsigned)active) {
            __threadfence();
            for (int i = 0; i < nslots; ++i) {
                double t = 0;
                for (int c = 0; c < active; ++c) t += __ldcg(partial + (long)c * kRed + i);
                __stcg(totals + i, t);
            }
            bar[0] = 0;
            __threadfence();
            atomicAdd(bar + 1, 1u);
        } else {
            long k = 0;
            while (*gen == g) {
                if (++k > (1L << 24)) {
                    atomicOr(err, ERRF_TIMEOUT);
                    s_ok = 0;
                    break;
                }
                __nanosleep(32);
            }
            __threadfence();
        }
        for (int i = 0; i < nslots; ++i) s_tot[i] = __ldcg(totals + i);
    }
    __syncthreads();
    for (int i = 0; i < nslots; ++i) out[i] = s_tot[i];
    return s_ok != 0;
}

AFX_D double block_sum_d(double v, double* sh) {
    v = warp_sum(v);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    double s = 0;
    if (threadIdx.x == 0)
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += sh[i];
    __syncthreads();
    return s;  // valid in thread 0
}

// Search direction entry for this iteration: z (first iteration) or z + beta * p_prev.
AFX_D float pdir(const float* z, const float* pprev, long i, double beta, bool first) {
    float zi = __ldcg(z + i);
    return first ? zi : (float)((double)zi + beta * (double)__ldcg(pprev + i));
}

// y = A p for node `node` (one warp), p formed on the fly; returns the 6 entries in every lane.
AFX_D void spmv_row(const GnBuffers& b, int node, const float* z, const float* pprev, double beta, bool first,
                    float* y6) {
    const int lane = threadIdx.x & 31;
    const int cnt = b.nbr_cnt[node];
    float acc[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    for (int u = lane; u <= cnt; u += 32) {
        const float* blk;
        long xo;
        bool tr = false;
        if (u == 0) {
            blk = b.diag + (long)node * 36;
            xo = (long)node * 6;
        } else {
            int ref = b.nbr_ref[(long)node * kMaxNbr + u - 1];
            int other = b.nbr[(long)node * kMaxNbr + u - 1];
            xo = (long)other * 6;
            if (ref >= 0) blk = b.blocks + (long)ref * 36;
            else {
                blk = b.blocks + (long)(-ref - 1) * 36;
                tr = true;
            }
        }
        float xv[6];
#pragma unroll
        for (int j = 0; j < 6; ++j) xv[j] = pdir(z, pprev, xo + j, beta, first);
#pragma unroll
        for (int i = 0; i < 6; ++i) {
            float s = 0.f;
#pragma unroll
            for (int j = 0; j < 6; ++j) s = s + (tr ? blk[j * 6 + i] : blk[i * 6 + j]) * xv[j];
            acc[i] = acc[i] + s;
        }
    }
#pragma unroll
    for (int i = 0; i < 6; ++i) y6[i] = warp_sum(acc[i]);
}

__global__ void __launch_bounds__(32 * kGnWarps) pcg_kernel(PcgArgs P) {
    GnArgs& a = P.g;
    GnBuffers& b = a.b;
    if (b.state->done) return;
    const int n = min(*a.n_nodes, a.n_max);
    const int active = max(1, min((int)gridDim.x, (n + kGnWarps - 1) / kGnWarps));
    if ((int)blockIdx.x >= active) return;
    __shared__ double sh[kGnWarps];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int gw = blockIdx.x * kGnWarps + w, nw = active * kGnWarps;
    int* err = a.error;
    float* pbuf[2] = {b.p, b.ap + (long)a.n_max * 6};  // second direction buffer follows A p
    // x = 0, r = b, z = M^-1 r; rz = r.z, bb = b.b  (one node per warp, lanes 0..5 own one entry)
    double rz_part = 0, bb_part = 0;
    for (int node = gw; node < n; node += nw) {
        if (lane < 6) {
            const long o = (long)node * 6;
            const double* Mi = b.minv + (long)node * 36 + lane * 6;
            double s = 0;
            for (int j = 0; j < 6; ++j) s += Mi[j] * (double)b.jtr[o + j];
            float zi = (float)s, ri = b.jtr[o + lane];
            b.x[o + lane] = 0.f;
            __stcg(b.r + o + lane, ri);
            __stcg(b.z + o + lane, zi);
            rz_part += (double)ri * (double)zi;
            bb_part += (double)ri * (double)ri;
        }
    }
    double mine[kRed] = {block_sum_d(rz_part, sh), block_sum_d(bb_part, sh), 0, 0};
    double tot[kRed];
    if (!grid_reduce_sync(b.bar, active, b.partial, b.partial + 4096 * kRed, mine, 2, tot, err)) return;
    double rz = tot[0];
    const double bnorm2 = tot[1];
    double beta = 0;
    int it = 0;
    for (; it < P.iters; ++it) {
        const bool first = it == 0;
        const float* pprev = pbuf[(it + 1) & 1];
        float* pcur = pbuf[it & 1];
        // p_it = z + beta p_{it-1}; Ap = A p_it; p.Ap
        double pap = 0;
        for (int node = gw; node < n; node += nw) {
            float y[6];
            spmv_row(b, node, b.z, pprev, beta, first, y);
            if (lane < 6) {
                const long o = (long)node * 6 + lane;
                float pi = pdir(b.z, pprev, o, beta, first);
                __stcg(pcur + o, pi);
                float yi = y[0];
#pragma unroll
                for (int q = 1; q < 6; ++q)
                    if (lane == q) yi = y[q];
                __stcg(b.ap + o, yi);
                pap += (double)pi * (double)yi;
            }
        }
        mine[0] = block_sum_d(pap, sh);
        if (!grid_reduce_sync(b.bar, active, b.partial, b.partial + 4096 * kRed, mine, 1, tot, err)) return;
        pap = tot[0];
        if (pap == 0.0 || !(pap == pap)) break;
        const double alpha = rz / pap;
        // x += alpha p; r -= alpha Ap; z = M^-1 r; r.z, r.r
        double rz_p = 0, rr_p = 0;
        for (int node = gw; node < n; node += nw) {
            const long o = (long)node * 6;
            float rv = 0.f;
            if (lane < 6) {
                b.x[o + lane] = (float)((double)b.x[o + lane] + alpha * (double)__ldcg(pcur + o + lane));
                rv = (float)((double)__ldcg(b.r + o + lane) - alpha * (double)__ldcg(b.ap + o + lane));
                __stcg(b.r + o + lane, rv);
            }
            float rr6[6];
#pragma unroll
            for (int j = 0; j < 6; ++j) rr6[j] = __shfl_sync(0xffffffffu, rv, j);
            if (lane < 6) {
                const double* Mi = b.minv + (long)node * 36 + lane * 6;
                double zs = 0;
                for (int j = 0; j < 6; ++j) zs += Mi[j] * (double)rr6[j];
                float zi = (float)zs;
                __stcg(b.z + o + lane, zi);
                rz_p += (double)rv * (double)zi;
                rr_p += (double)rv * (double)rv;
            }
        }
        mine[0] = block_sum_d(rz_p, sh);
        mine[1] = block_sum_d(rr_p, sh);
        if (!grid_reduce_sync(b.bar, active, b.partial, b.partial + 4096 * kRed, mine, 2, tot, err)) return;
        beta = tot[0] / rz;
        rz = tot[0];
        if (P.tol > 0 && tot[1] <= P.tol * P.tol * bnorm2) {
            ++it;
            break;
        }
    }
    // pending transforms -= [[x_rot]x, x_t; 0] (updateTransformsKernel, src/MotionOptimization.cu:483-498)
    for (int node = gw; node < n; node += nw) {
        if (lane == 0) {
            const float* u = b.x + (long)node * 6;
            float* T = P.T_pending + (long)node * 16;
            const float U[16] = {0.f, u[2], -u[1], 0.f, -u[2], 0.f, u[0], 0.f, u[1], -u[0], 0.f, 0.f, u[3], u[4], u[5], 0.f};
            for (int e = 0; e < 16; ++e) T[e] = T[e] - U[e];
        }
    }
}

}  // namespace afx

// ------------------------------------------------------------------------------------
// Host side
// ------------------------------------------------------------------------------------

namespace afx {

struct GnSizes {
    long m_max;
    int n_max, k, kreg;
};

static size_t al(size_t x) { return (x + 255) & ~(size_t)255; }

static int pcg_grid(int n_max) {
    static int cached = -1;
    if (cached < 0) {
        int dev = 0, sms = 0, per = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, pcg_kernel, 32 * kGnWarps, 0);
        cached = sms * (per < 1 ? 1 : (per > 4 ? 4 : per));
    }
    int need = (n_max + kGnWarps - 1) / kGnWarps;
    return need < 1 ? 1 : (need < cached ? need : cached);
}

size_t gn_workspace_size(long m_max, int n_max, int k, int kreg) {
    size_t s = 0;
    s += 3 * al((n_max + 1) * 4) + al(m_max * k * 4);           // lcnt loff lcur lst
    s += 3 * al((n_max + 1) * 4) + al((size_t)n_max * kreg * 4);  // icnt ioff icur ilst
    s += al(n_max * 4) + 2 * al((size_t)n_max * kMaxNbr * 4);     // nbr_cnt nbr nbr_ref
    s += al((size_t)n_max * kMaxNbr * 36 * 4) + al((size_t)n_max * 36 * 4) + al((size_t)n_max * 36 * 8);
    s += al((size_t)m_max * k * 6 * 4) + al((size_t)m_max * k * 4);  // jrow jc
    s += al((size_t)n_max * 6 * 4) * 5 + al((size_t)n_max * 6 * 4 * 2);  // jtr x r z p, ap + p2
    s += al(m_max * 4) + al((size_t)n_max * kreg * 3 * 4);        // rdepth rreg
    s += al((size_t)(4096 + 1) * kRed * 8) + al(64) + al(kEnergyBlocks * 2 * 8) + al(sizeof(GnState));
    s += al(scan_workspace_size(m_max > n_max ? m_max : n_max));
    return s + 1024;
}

bool gn_carve(void* ws, size_t bytes, long m_max, int n_max, int k, int kreg, GnBuffers* b) {
    if (!ws || bytes < gn_workspace_size(m_max, n_max, k, kreg)) return false;
    char* p = static_cast<char*>(ws);
    auto take = [&](size_t n) {
        char* q = p;
        p += al(n);
        return q;
    };
    b->lcnt = (unsigned*)take((n_max + 1) * 4);
    b->loff = (unsigned*)take((n_max + 1) * 4);
    b->lcur = (unsigned*)take((n_max + 1) * 4);
    b->lst = (unsigned*)take(m_max * k * 4);
    b->icnt = (unsigned*)take((n_max + 1) * 4);
    b->ioff = (unsigned*)take((n_max + 1) * 4);
    b->icur = (unsigned*)take((n_max + 1) * 4);
    b->ilst = (unsigned*)take((size_t)n_max * kreg * 4);
    b->nbr_cnt = (int*)take(n_max * 4);
    b->nbr = (int*)take((size_t)n_max * kMaxNbr * 4);
    b->nbr_ref = (int*)take((size_t)n_max * kMaxNbr * 4);
    b->blocks = (float*)take((size_t)n_max * kMaxNbr * 36 * 4);
    b->diag = (float*)take((size_t)n_max * 36 * 4);
    b->minv = (double*)take((size_t)n_max * 36 * 8);
    b->jrow = (float*)take((size_t)m_max * k * 6 * 4);
    b->jc = (int*)take((size_t)m_max * k * 4);
    b->jtr = (float*)take((size_t)n_max * 6 * 4);
    b->x = (float*)take((size_t)n_max * 6 * 4);
    b->r = (float*)take((size_t)n_max * 6 * 4);
    b->z = (float*)take((size_t)n_max * 6 * 4);
    b->p = (float*)take((size_t)n_max * 6 * 4);
    b->ap = (float*)take((size_t)n_max * 6 * 4 * 2);  // A p, then the second search-direction buffer
    b->rdepth = (float*)take(m_max * 4);
    b->rreg = (float*)take((size_t)n_max * kreg * 3 * 4);
    b->partial = (double*)take((size_t)(4096 + 1) * kRed * 8);
    b->bar = (unsigned*)take(64);
    b->epart = (double*)take(kEnergyBlocks * 2 * 8);
    b->state = (GnState*)take(sizeof(GnState));
    b->scan_ws = take(scan_workspace_size(m_max > n_max ? m_max : n_max));
    return true;
}

void gn_init_barrier(const GnBuffers& b, cudaStream_t st) { cudaMemsetAsync(b.bar, 0, 64, st); }

// Per frame: node -> vertex lists and incoming regularisation edges.
int gn_frame_setup(const GnArgs& a, cudaStream_t st) {
    const GnBuffers& b = a.b;
    AFX_CUDA(cudaMemsetAsync(b.lcnt, 0, (a.n_max + 1) * 4, st));
    AFX_CUDA(cudaMemsetAsync(b.lcur, 0, (a.n_max + 1) * 4, st));
    AFX_CUDA(cudaMemsetAsync(b.icnt, 0, (a.n_max + 1) * 4, st));
    AFX_CUDA(cudaMemsetAsync(b.icur, 0, (a.n_max + 1) * 4, st));
    const long mk = a.m_max * a.k;
    if (mk > 0) {
        lst_count_kernel<<<blocks_for(mk, 256), 256, 0, st>>>(a);
        AFX_LAUNCH_CHECK();
    }
    int rc = scan_exclusive(b.lcnt, b.loff, a.n_max + 1, nullptr, b.scan_ws, st);
    if (rc) return rc;
    if (mk > 0) {
        lst_fill_kernel<<<blocks_for(mk, 256), 256, 0, st>>>(a);
        AFX_LAUNCH_CHECK();
    }
    seg_sort_kernel<<<(unsigned)a.n_max, 256, 0, st>>>(b.lst, b.loff, a.n_nodes, a.n_max, a.error);
    AFX_LAUNCH_CHECK();
    const long nk = (long)a.n_max * a.kreg;
    in_count_kernel<<<blocks_for(nk, 256), 256, 0, st>>>(a);
    AFX_LAUNCH_CHECK();
    rc = scan_exclusive(b.icnt, b.ioff, a.n_max + 1, nullptr, b.scan_ws, st);
    if (rc) return rc;
    in_fill_kernel<<<blocks_for(nk, 256), 256, 0, st>>>(a);
    AFX_LAUNCH_CHECK();
    seg_sort_kernel<<<(unsigned)a.n_max, 256, 0, st>>>(b.ilst, b.ioff, a.n_nodes, a.n_max, a.error);
    AFX_LAUNCH_CHECK();
    return AFX_OK;
}

__global__ void gn_state_reset_kernel(GnState* s) {
    s->e_prev = 3.4028234663852886e+38;  // std::numeric_limits<float>::max() (src/VolumeFusion.cu:570)
    s->e_last = 0;
    s->e_depth = s->e_reg = 0;
    s->done = 0;
    s->commit = 0;
    s->iters = 0;
}

// Per ICP iteration (after correspondences): J^T J structure, blocks and block inverses.
int gn_icp_setup(const GnArgs& a, float* T_pending, const float* T_committed, cudaStream_t st) {
    const GnBuffers& b = a.b;
    gn_state_reset_kernel<<<1, 1, 0, st>>>(b.state);
    AFX_LAUNCH_CHECK();
    AFX_CUDA(cudaMemcpyAsync(T_pending, T_committed, (size_t)a.n_max * 64, cudaMemcpyDeviceToDevice, st));
    const unsigned nb = (unsigned)((a.n_max + kGnWarps - 1) / kGnWarps);
    const int words = (a.n_max + 31) / 32;
    const size_t smem = (size_t)kGnWarps * words * 4;
    if (smem > 200 * 1024) return AFX_ERR_UNSUPPORTED;
    if (smem > 48 * 1024) cudaFuncSetAttribute(nbr_discover_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    nbr_discover_kernel<<<nb, 32 * kGnWarps, smem, st>>>(a, words);
    AFX_LAUNCH_CHECK();
    nbr_ref_kernel<<<blocks_for((long)a.n_max * kMaxNbr, 256), 256, 0, st>>>(a);
    AFX_LAUNCH_CHECK();
    jtj_assemble_kernel<<<nb, 32 * kGnWarps, 0, st>>>(a);
    AFX_LAUNCH_CHECK();
    diag_inverse_kernel<<<blocks_for(a.n_max, 128), 128, 0, st>>>(a);
    AFX_LAUNCH_CHECK();
    return AFX_OK;
}

// One Gauss-Newton iteration (src/VolumeFusion.cu:571-691); `warped` is re-warped with the
// pending transforms by the caller after this returns.
int gn_iteration(const GnArgs& a, int iter, const float* warped, float* T_committed, float* T_pending, int pcg_iters,
                 double tol, cudaStream_t st) {
    const GnBuffers& b = a.b;
    residual_kernel<<<kEnergyBlocks, 256, 0, st>>>(a, warped, T_pending);
    AFX_LAUNCH_CHECK();
    energy_kernel<<<1, kEnergyBlocks, 0, st>>>(a, iter);
    AFX_LAUNCH_CHECK();
    commit_kernel<<<blocks_for((long)a.n_max * 16, 256), 256, 0, st>>>(a, T_committed, T_pending);
    AFX_LAUNCH_CHECK();
    const unsigned nb = (unsigned)((a.n_max + kGnWarps - 1) / kGnWarps);
    jtr_kernel<<<nb, 32 * kGnWarps, 0, st>>>(a);
    AFX_LAUNCH_CHECK();
    PcgArgs P;
    P.g = a;
    P.T_pending = T_pending;
    P.iters = pcg_iters;
    P.tol = tol;
    int grid = pcg_grid(a.n_max);
    void* args[] = {&P};
    AFX_CUDA(cudaLaunchCooperativeKernel((void*)pcg_kernel, dim3(grid), dim3(32 * kGnWarps), args, 0, st));
    AFX_LAUNCH_CHECK();
    (void)b;
    return AFX_OK;
}

}  // namespace afx
