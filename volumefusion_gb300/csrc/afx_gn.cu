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
// The solve is a block-Jacobi PCG in one cooperative kernel: FP32 block SpMV, dot products in
// double-binary32 (shared-memory path) or FP64 (global-memory path), FP64 6x6 block inverses.
#include <cfloat>
#include <cstring>
#include <new>

#include "afx_dqb.cuh"
#include "afx_gn.h"
#include "afx_host.h"

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
    const long m = min((long)*a.mesh_count, a.m_max);
    const uint32_t n = (uint32_t)*a.n_nodes;
    AFX_GRID_STRIDE(t, m * a.k) {
        if (a.mw[t] == 0.f) continue;
        const uint32_t node = a.midx[t];
        if (node < n) atomicAdd(a.b.lcnt + node, 1u);
    }
}

__global__ void lst_fill_kernel(GnArgs a) {
    const long m = min((long)*a.mesh_count, a.m_max);
    const uint32_t n = (uint32_t)*a.n_nodes;
    AFX_GRID_STRIDE(t, m * a.k) {
        if (a.mw[t] == 0.f) continue;
        const uint32_t node = a.midx[t];
        if (node >= n) continue;
        const unsigned p = a.b.loff[node] + atomicAdd(a.b.lcur + node, 1u);
        a.b.lst[p] = (unsigned)t;
    }
}

__global__ void in_count_kernel(GnArgs a) {
    const int n = min(*a.n_nodes, a.n_max);
    AFX_GRID_STRIDE(t, (long)n * a.kreg) {
        const uint32_t nb = a.gidx[t];
        if (nb < (uint32_t)n) atomicAdd(a.b.icnt + nb, 1u);
    }
}

__global__ void in_fill_kernel(GnArgs a) {
    const int n = min(*a.n_nodes, a.n_max);
    AFX_GRID_STRIDE(t, (long)n * a.kreg) {
        const uint32_t nb = a.gidx[t];
        if (nb >= (uint32_t)n) continue;
        const unsigned p = a.b.ioff[nb] + atomicAdd(a.b.icur + nb, 1u);
        a.b.ilst[p] = (unsigned)t;
    }
}

// Bitonic sort of one list (len <= kSegMax) through shared memory, by the whole CTA.
AFX_D void seg_sort_one(unsigned* lst, int len, unsigned* s) {
    int P = 1;
    while (P < len) P <<= 1;
    __syncthreads();  // the previous list's write-back is done with s
    for (int i = threadIdx.x; i < P; i += blockDim.x) s[i] = i < len ? lst[i] : 0xffffffffu;
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
    for (int i = threadIdx.x; i < len; i += blockDim.x) lst[i] = s[i];
}

// Sort each node's list ascending (bitonic in shared memory); one CTA per node at a time.
__global__ void __launch_bounds__(256) seg_sort_kernel(unsigned* lst, const unsigned* off, const int* n_nodes, int n_max,
                                                       int* error) {
    __shared__ unsigned s[kSegMax];
    const int n = min(*n_nodes, n_max);
    for (int a = blockIdx.x; a < n; a += gridDim.x) {
        const unsigned o = off[a];
        const int len = (int)(off[a + 1] - o);
        if (len > kSegMax) {
            if (threadIdx.x == 0) atomicOr(error, ERRF_CAPACITY);
            continue;
        }
        if (len > 1) seg_sort_one(lst + o, len, s);
    }
}


// ---- per-ICP assembly ----

// Neighbour discovery: distinct nodes b != a sharing a corresponding vertex with a (both
// weights non-zero) or joined to a by a regularisation edge.  One warp per node, bitmap in
// shared memory, so the list comes out sorted.
__global__ void __launch_bounds__(32 * kGnWarps) nbr_discover_kernel(GnArgs a, int words) {
    extern __shared__ unsigned bm[];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int n = min(*a.n_nodes, a.n_max);
    unsigned* my = bm + (long)w * words;
    for (int node = blockIdx.x * kGnWarps + w; node < n; node += gridDim.x * kGnWarps) {
        for (int i = lane; i < words; i += 32) my[i] = 0u;
        __syncwarp();
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
        __syncwarp();
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
        __syncwarp();  // the bitmap is cleared for the warp's next node
    }
}

// For neighbour slots below the diagonal, find the owner's slot (binary search).
__global__ void nbr_ref_kernel(GnArgs a) {
    const int n = min(*a.n_nodes, a.n_max);
    AFX_GRID_STRIDE(t, (long)n * kMaxNbr) {
        const int node = (int)(t / kMaxNbr), u = (int)(t % kMaxNbr);
        if (u >= a.b.nbr_cnt[node]) continue;
        const int bnode = a.b.nbr[t];
        if (bnode > node) {
            a.b.nbr_ref[t] = (int)t;
            continue;
        }
        const int* L = a.b.nbr + (long)bnode * kMaxNbr;
        int lo = 0, hi = a.b.nbr_cnt[bnode] - 1, f = -1;
        while (lo <= hi) {
            const int mid = (lo + hi) >> 1;
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
            continue;
        }
        a.b.nbr_ref[t] = -((int)((long)bnode * kMaxNbr + f) + 1);
    }
}

// J^T J: node a's warp accumulates D_a and its upper blocks (a, b > a).  Lane l owns block
// entries l and l + 32 of every block; each entry is summed in a fixed sequential order:
// depth rows by ascending node-list entry, then regularisation rows by ascending row.  The
// rows are staged 32 at a time, one per lane, with their Jacobian blocks already formed
// (jdepth for every contributing slot, or lam_r * G for a regularisation row), so the ordered
// loop is shared-memory loads and adds only; the upper blocks accumulate in shared memory.
constexpr int kJtjWarps = 2;
constexpr int kJtjMaxK = 8;

struct JtjStage {
    float blk[kMaxNbr * 36];           // upper blocks of this node
    int L[kMaxNbr];                    // sorted neighbour ids
    float J[32][kJtjMaxK][6];          // depth rows: jdepth of each slot; reg rows: lam_r * G (3 x 6)
    signed char slot[32][kJtjMaxK];    // -1: diagonal, >= 0: upper block, -2: no contribution
    int own[32];                       // depth rows: the row's own slot, -1 without correspondence;
                                       // reg rows: 1 own edge, 0 incoming edge, -1 skipped
    unsigned qt[32];                   // depth rows with a correspondence, queued in entry order:
    unsigned qe[32];                   // node-list position, entry (vertex * k + slot)
    int qc[32];                        // and correspondence
};

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

__global__ void __launch_bounds__(32 * kJtjWarps) jtj_assemble_kernel(GnArgs a) {
    __shared__ JtjStage stage[kJtjWarps];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    JtjStage& S = stage[w];
    const int n = min(*a.n_nodes, a.n_max);
    const int k = a.k;
    const int e0 = lane, e1 = lane + 32;  // entries this lane owns (e1 valid for lanes 0..3)
    const int i0 = e0 / 6, j0 = e0 % 6, i1 = e1 / 6, j1 = e1 % 6;
    const bool has1 = e1 < 36;
    for (int node = blockIdx.x * kJtjWarps + w; node < n; node += gridDim.x * kJtjWarps) {
        const int cnt = a.b.nbr_cnt[node];
        for (int u = lane; u < cnt; u += 32) S.L[u] = a.b.nbr[(long)node * kMaxNbr + u];
        for (int x = lane; x < cnt * 36; x += 32) S.blk[x] = 0.f;
        __syncwarp();
        float d0 = 0.f, d1 = 0.f;
        bool touched = false;
        // Depth rows: the node list is read 128 entries at a time (4 per lane, their loads in
        // flight together); entries whose vertex has a correspondence are queued in entry order
        // and, 32 at a time, staged (one row per lane: the Jacobian block of every slot) and then
        // accumulated in order.  Entries without a correspondence contribute nothing.
        auto run_queue = [&](int nq) {
            if (lane < nq) {
                const unsigned t = S.qt[lane], ent = S.qe[lane];
                const long v = ent / k;
                const int s = (int)(ent % k);
                const int c = S.qc[lane];
                S.own[lane] = s;
                const int px = a.corr[2 * (long)c + 1];
                const float nrm[3] = {a.normals[3 * (long)px], a.normals[3 * (long)px + 1], a.normals[3 * (long)px + 2]};
                const float p[3] = {a.mesh[3 * v], a.mesh[3 * v + 1], a.mesh[3 * v + 2]};
                float G[3][6];
                grad_rows(p, G);
                for (int tt = 0; tt < k; ++tt) {
                    const float wt = a.mw[v * k + tt];
                    const uint32_t bnode = a.midx[v * k + tt];
                    int sl = -2;
                    if (wt != 0.f && bnode >= (uint32_t)node) {
                        if (bnode == (uint32_t)node) sl = -1;
                        else {
                            const int f = find_slot(S.L, cnt, (int)bnode);
                            if (f >= 0) sl = f;
                        }
                    }
                    S.slot[lane][tt] = (signed char)sl;
                    if (sl != -2 || tt == s) {
                        float Jt[6];
                        jdepth(nrm, wt, G, a.lam_d, Jt);
#pragma unroll
                        for (int q = 0; q < 6; ++q) S.J[lane][tt][q] = Jt[q];
                        if (tt == s)  // this row's J block, for J^T r
#pragma unroll
                            for (int q = 0; q < 6; ++q) a.b.jrow[(long)t * 6 + q] = Jt[q];
                    }
                }
            }
            __syncwarp();
            for (int r = 0; r < nq; ++r) {
                const int s = S.own[r];
                touched = true;
                const float ja0 = S.J[r][s][i0];
                const float ja1 = has1 ? S.J[r][s][i1] : 0.f;
                for (int tt = 0; tt < k; ++tt) {
                    const int sl = S.slot[r][tt];
                    if (sl == -2) continue;
                    const float jb0 = S.J[r][tt][j0];
                    const float jb1 = S.J[r][tt][j1];
                    if (sl == -1) {
                        d0 = d0 + ja0 * jb0;
                        if (has1) d1 = d1 + ja1 * jb1;
                    } else {
                        float* blk = S.blk + sl * 36;
                        blk[e0] = blk[e0] + ja0 * jb0;
                        if (has1) blk[e1] = blk[e1] + ja1 * jb1;
                    }
                }
            }
            __syncwarp();
        };
        const unsigned o = a.b.loff[node], e = a.b.loff[node + 1];
        int qn = 0;  // queued rows (warp-uniform)
        for (unsigned base = o; base < e; base += 128) {
            unsigned ent[4];
            int cj[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const unsigned t = base + (unsigned)(j * 32 + lane);
                ent[j] = t < e ? a.b.lst[t] : 0u;
            }
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const unsigned t = base + (unsigned)(j * 32 + lane);
                cj[j] = -1;
                if (t < e) {
                    cj[j] = a.corr_of_vertex[ent[j] / k];
                    a.b.jc[t] = cj[j];
                }
            }
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                unsigned bal = __ballot_sync(0xffffffffu, cj[j] >= 0);
                while (bal) {
                    unsigned take = bal;
                    for (int drop = __popc(bal) - (32 - qn); drop > 0; --drop) take &= ~(0x80000000u >> __clz(take));
                    if (take & (1u << lane)) {
                        const int pos = qn + __popc(take & ((1u << lane) - 1u));
                        S.qt[pos] = base + (unsigned)(j * 32 + lane);
                        S.qe[pos] = ent[j];
                        S.qc[pos] = cj[j];
                    }
                    qn += __popc(take);
                    bal &= ~take;
                    __syncwarp();
                    if (qn == 32) {
                        run_queue(32);
                        qn = 0;
                    }
                }
            }
        }
        if (qn) run_queue(qn);
        // regularisation rows in ascending row order: incoming edges x -> node with x < node,
        // then node's own edges, then incoming edges with x > node (src/MotionOptimization.cu:298-340)
        const unsigned io = a.b.ioff[node], nin = a.b.ioff[node + 1] - io;
        unsigned nlo = 0;  // incoming rows with source below node (ilst is ascending)
        for (unsigned x = lane; x < nin; x += 32) nlo += (a.b.ilst[io + x] / a.kreg < (unsigned)node) ? 1u : 0u;
        nlo = warp_sum(nlo);
        const unsigned nrows = nin + (unsigned)a.kreg;
        for (unsigned base = 0; base < nrows; base += 32) {
            const unsigned r = base + lane;
            if (r < nrows) {
                int src, kk;
                if (r < nlo) {
                    const unsigned ent = a.b.ilst[io + r];
                    src = (int)(ent / a.kreg);
                    kk = (int)(ent % a.kreg);
                } else if (r < nlo + (unsigned)a.kreg) {
                    src = node;
                    kk = (int)(r - nlo);
                } else {
                    const unsigned ent = a.b.ilst[io + r - a.kreg];
                    src = (int)(ent / a.kreg);
                    kk = (int)(ent % a.kreg);
                }
                const uint32_t nbk = a.gidx[(long)src * a.kreg + kk];
                const bool live = !(src == node && nbk >= (uint32_t)n);  // own edge filtered out
                S.own[lane] = live ? (src == node ? 1 : 0) : -1;
                float G[3][6];
                grad_rows(a.nodes + 3 * (long)src, G);
#pragma unroll
                for (int ax = 0; ax < 3; ++ax)
#pragma unroll
                    for (int q = 0; q < 6; ++q) S.J[lane][ax][q] = G[ax][q] * a.lam_r;
                const int other = (src == node) ? (int)nbk : src;
                int sl = -2;
                if (other > node) {
                    const int f = find_slot(S.L, cnt, other);
                    if (f >= 0) sl = f;
                }
                S.slot[lane][0] = (signed char)sl;
            }
            __syncwarp();
            const int nb = (int)min(32u, nrows - base);
            for (int rr = 0; rr < nb; ++rr) {
                const int self = S.own[rr];
                if (self < 0) continue;
                touched = true;
                const int sl = S.slot[rr][0];
#pragma unroll
                for (int ax = 0; ax < 3; ++ax) {
                    const float g_i0 = S.J[rr][ax][i0], g_j0 = S.J[rr][ax][j0];
                    const float g_i1 = has1 ? S.J[rr][ax][i1] : 0.f, g_j1 = S.J[rr][ax][j1];
                    // this node is `src` (coefficient +g) or the edge's target (coefficient -g)
                    const float n_i0 = self ? g_i0 : -g_i0, n_j0 = self ? g_j0 : -g_j0;
                    const float n_i1 = self ? g_i1 : -g_i1, n_j1 = self ? g_j1 : -g_j1;
                    d0 = d0 + n_i0 * n_j0;
                    if (has1) d1 = d1 + n_i1 * n_j1;
                    if (sl >= 0) {
                        const float o_j0 = self ? -g_j0 : g_j0, o_j1 = self ? -g_j1 : g_j1;
                        float* blk = S.blk + sl * 36;
                        blk[e0] = blk[e0] + n_i0 * o_j0;
                        if (has1) blk[e1] = blk[e1] + n_i1 * o_j1;
                    }
                }
            }
            __syncwarp();
        }
        if (!touched) {  // identity diagonal block (src/VolumeFusion.cu:637-640)
            d0 = (i0 == j0) ? 1.f : 0.f;
            d1 = (i1 == j1) ? 1.f : 0.f;
        }
        float* D = a.b.diag + (long)node * 36;
        D[e0] = d0;
        if (has1) D[e1] = d1;
        float* B = a.b.blocks + (long)node * kMaxNbr * 36;
        for (int u = 0; u < cnt; ++u) {
            if (S.L[u] <= node) continue;
            B[u * 36 + e0] = S.blk[u * 36 + e0];
            if (has1) B[u * 36 + e1] = S.blk[u * 36 + e1];
        }
        __syncwarp();
    }
}

// Inverse of each diagonal block: Gauss-Jordan with partial pivoting in FP64, one warp per
// node with lane j < 12 owning column j of [D | I]; stored rounded to FP32 (the preconditioner
// is applied in FP32).
AFX_D void diag_inverse_node(const GnArgs& a, int node) {
    const int lane = threadIdx.x & 31;
    const float* D = a.b.diag + (long)node * 36;
    const bool own = lane < 12;
    double col[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) col[i] = !own ? 0.0 : (lane < 6 ? (double)D[i * 6 + lane] : (lane - 6 == i ? 1.0 : 0.0));
    bool ok = true;
#pragma unroll
    for (int c = 0; c < 6; ++c) {
        // pivot: the largest |m[r][c]|, r >= c (first on ties), read from lane c
        int p = c;
        double best = fabs(__shfl_sync(0xffffffffu, col[c], c));
#pragma unroll
        for (int r = c + 1; r < 6; ++r) {
            double v = fabs(__shfl_sync(0xffffffffu, col[r], c));
            if (v > best) {
                best = v;
                p = r;
            }
        }
        if (best == 0.0) {
            ok = false;
            break;
        }
        if (p != c) {
#pragma unroll
            for (int r = c + 1; r < 6; ++r)
                if (r == p) {
                    double t = col[r];
                    col[r] = col[c];
                    col[c] = t;
                }
        }
        const double d = __shfl_sync(0xffffffffu, col[c], c);
        col[c] /= d;
#pragma unroll
        for (int r = 0; r < 6; ++r)
            if (r != c) {
                double f = __shfl_sync(0xffffffffu, col[r], c);
                col[r] -= f * col[c];
            }
    }
    float* out = a.b.minv + (long)node * 36;
    if (!ok) {
        if (lane == 0) atomicOr(a.error, ERRF_SINGULAR);
        if (lane < 6)
            for (int i = 0; i < 6; ++i) out[i * 6 + lane] = 0.f;
        return;
    }
    if (lane >= 6 && lane < 12)
#pragma unroll
        for (int i = 0; i < 6; ++i) out[i * 6 + lane - 6] = (float)col[i];
}

__global__ void __launch_bounds__(128) diag_inverse_kernel(GnArgs a) {
    const int n = min(*a.n_nodes, a.n_max);
    for (int node = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); node < n; node += gridDim.x * (blockDim.x >> 5))
        diag_inverse_node(a, node);
}

// ---- Gauss-Newton loop: one thread-block cluster per ICP iteration ----
//
// All Gauss-Newton iterations of one ICP iteration (src/VolumeFusion.cu:571-691) run in one
// launch of a single cluster of kGnClusterMax CTAs (16 where the device allows non-portable
// cluster sizes, else 8).  Phases are separated by the hardware cluster barrier
// (barrier.cluster.arrive.release / wait.acquire), so no CTA spins on memory.  FP64
// reductions go through distributed shared memory: each CTA writes its block sum into a slot
// of its own shared memory and, after the barrier, reads every CTA's slot in rank order, so
// all CTAs hold bit-identical totals and take identical branches.  Values exchanged between
// CTAs through global memory (residuals, pending transforms, PCG vectors, warped vertices)
// are stored with st.global.cg and loaded with ld.global.cg, i.e. always from L2.
// Per iteration:
//   residuals + energies -> energy test and commit -> J^T r -> PCG (x = 0, block-Jacobi,
//   FP32 block SpMV, double-float or FP64 dots, two cluster barriers per PCG iteration)
//   -> T_pending -= [[x_rot]x, x_t; 0] -> re-warp the canonical vertices with T_pending.

constexpr int kLoopThreads = 512;
constexpr int kLoopWarps = kLoopThreads / 32;

AFX_D unsigned cluster_rank() {
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}

AFX_D unsigned cluster_size() {
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
    return r;
}

// All threads of all CTAs of the cluster; orders every prior memory access before every later one.
AFX_D void cluster_barrier() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// Load a double from the shared memory of CTA `rank` of this cluster, at the offset of `p` here.
AFX_D double dsmem_load(const double* p, unsigned rank) {
    unsigned local = (unsigned)__cvta_generic_to_shared(p), remote;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(remote) : "r"(local), "r"(rank));
    double v;
    asm volatile("ld.shared::cluster.f64 %0, [%1];" : "=d"(v) : "r"(remote) : "memory");
    return v;
}

// Double-binary32 ("double-float") arithmetic: a value is the unevaluated sum hi + lo of two
// binary32 numbers with |lo| <= ulp(hi) / 2, about 48 significant bits.  A sum is the accurate
// double-float addition of Hida, Li and Bailey's QD library (2001): Knuth's TwoSum (the exact
// rounding error of a binary32 sum) on the high and the low parts, then Dekker's Fast2Sum to
// renormalise; a product of two binary32 values is exact as p + fma(x, y, -p).  TwoSum's error term
// is exact whatever the operand order, so df_add(a, b) and df_add(b, a) agree bit for bit and
// every lane of a butterfly ends with the same total.  On this part a dependent binary64 add takes
// ~150-200 cycles; a double-float add is a chain of ~8 binary32 operations.
struct DF {
    float hi, lo;
};

AFX_D DF two_sum(float a, float b) {
    const float s = a + b, v = s - a;
    return {s, (a - (s - v)) + (b - v)};
}

AFX_D DF fast_two_sum(float a, float b) {
    const float s = a + b;
    return {s, b - (s - a)};
}

AFX_D DF df_add(DF a, DF b) {
    DF s = two_sum(a.hi, b.hi);
    const DF t = two_sum(a.lo, b.lo);
    s = fast_two_sum(s.hi, s.lo + t.hi);
    return fast_two_sum(s.hi, s.lo + t.lo);
}

AFX_D DF df_prod(float x, float y) {
    const float p = x * y;
    return {p, fmaf(x, y, -p)};
}

AFX_D DF df_shfl_xor(DF v, int o) {
    return {__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o)};
}

// a / b rounded to binary32 (within about half an ulp): the binary32 quotient of the high parts,
// corrected once by the remainder, which fma forms exactly.
AFX_D float df_quotient(DF a, DF b) {
    const float q = a.hi / b.hi;
    if (q == 0.f || !isfinite(q)) return q;
    const float r = (fmaf(-q, b.hi, a.hi) + a.lo) - q * b.lo;
    return q + r / b.hi;
}

AFX_D bool df_zero_or_nan(DF v) { return v.hi == 0.f || v.hi != v.hi; }

struct ClusterSums {
    double slot[2][4];            // this CTA's block sums, double-buffered across calls
    double warp[kLoopWarps * 4];  // per-warp sums
    double total[4];
    int phase;
    // PCG scalars, written by lane 0 of warp 0 and read by every thread after a __syncthreads
    DF rz_df, bn_df;  // r.z of the current iterate, b.b (shared-memory path)
    float alpha, beta;
    int stop;
};

// Sums v[0..NV) over every thread of the cluster; all threads of all CTAs get identical totals.
// Fixed-shape FP64 trees: butterfly within each warp, then over the CTA's warps, then over the
// CTAs by rank.  Contains one cluster barrier.
template <int NV>
AFX_D void cluster_sum(double (&v)[NV], ClusterSums& cs) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int i = 0; i < NV; ++i) {
        double s = warp_sum(v[i]);
        if (lane == 0) cs.warp[w * 4 + i] = s;
    }
    __syncthreads();
    const int ph = cs.phase;
    if (w == 0) {
#pragma unroll
        for (int i = 0; i < NV; ++i) {
            double s = lane < kLoopWarps ? cs.warp[lane * 4 + i] : 0.0;
#pragma unroll
            for (int o = kLoopWarps / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
            if (lane == 0) cs.slot[ph][i] = s;
        }
    }
    cluster_barrier();
    if (w == 0) {
        const unsigned ncta = cluster_size();
#pragma unroll
        for (int i = 0; i < NV; ++i) {
            double t = lane < (int)ncta ? dsmem_load(&cs.slot[ph][i], lane) : 0.0;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
            if (lane == 0) cs.total[i] = t;
        }
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < NV; ++i) v[i] = cs.total[i];
    if (threadIdx.x == 0) cs.phase = ph ^ 1;
}

// Double-floats in this CTA's shared memory and in CTA `rank`'s (8-byte slots, hi first).
AFX_D void sts_df(double* local, DF v) {
    const unsigned a = (unsigned)__cvta_generic_to_shared(local);
    asm volatile("st.shared.v2.f32 [%0], {%1, %2};" ::"r"(a), "f"(v.hi), "f"(v.lo) : "memory");
}
AFX_D DF lds_df_local(const double* local) {
    const unsigned a = (unsigned)__cvta_generic_to_shared(local);
    DF v;
    asm volatile("ld.shared.v2.f32 {%0, %1}, [%2];" : "=f"(v.hi), "=f"(v.lo) : "r"(a) : "memory");
    return v;
}
AFX_D DF dsmem_load_df(const double* p, unsigned rank) {
    unsigned local = (unsigned)__cvta_generic_to_shared(p), remote;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(remote) : "r"(local), "r"(rank));
    DF v;
    asm volatile("ld.shared::cluster.v2.f32 {%0, %1}, [%2];" : "=f"(v.hi), "=f"(v.lo) : "r"(remote) : "memory");
    return v;
}

// cluster_sum in double-float arithmetic: the same fixed-shape trees (warp butterfly, the CTA's
// warps, the CTAs by rank) with df_add, so every thread of every CTA gets identical totals.
// Contains one cluster barrier.
template <int NV>
AFX_D void cluster_sum_df(DF (&v)[NV], ClusterSums& cs) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int i = 0; i < NV; ++i) {
        DF s = v[i];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s = df_add(s, df_shfl_xor(s, o));
        if (lane == 0) sts_df(&cs.warp[w * 4 + i], s);
    }
    __syncthreads();
    const int ph = cs.phase;
    if (w == 0) {
#pragma unroll
        for (int i = 0; i < NV; ++i) {
            DF s = {0.f, 0.f};
            if (lane < kLoopWarps) s = lds_df_local(&cs.warp[lane * 4 + i]);
#pragma unroll
            for (int o = kLoopWarps / 2; o > 0; o >>= 1) s = df_add(s, df_shfl_xor(s, o));
            if (lane == 0) sts_df(&cs.slot[ph][i], s);
        }
    }
    cluster_barrier();
    if (w == 0) {
        const unsigned ncta = cluster_size();
#pragma unroll
        for (int i = 0; i < NV; ++i) {
            DF t = {0.f, 0.f};
            if (lane < (int)ncta) t = dsmem_load_df(&cs.slot[ph][i], lane);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) t = df_add(t, df_shfl_xor(t, o));
            if (lane == 0) sts_df(&cs.total[i], t);
        }
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < NV; ++i) v[i] = lds_df_local(&cs.total[i]);
    if (threadIdx.x == 0) cs.phase = ph ^ 1;
}

struct LoopArgs {
    GnArgs g;
    const float* points;  // canonical vertices
    float* warped;
    float* T_committed;
    float* T_pending;
    int gn_iters, pcg_iters;
    double tol;  // <= 0: run exactly pcg_iters PCG iterations
};

// J^T r of one node, one warp: lane l sums the node-list entries l, l+32, ... (depth rows, J
// rows formed once per ICP iteration by jtj_assemble_kernel) and then the regularisation rows
// l, l+32, ... (incoming edges, then the node's own); the 32 partial sums are combined by a
// butterfly, so every lane returns the same six totals.
AFX_D void jtr_node(const GnArgs& a, int node, int n, float (&acc)[6]) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int q = 0; q < 6; ++q) acc[q] = 0.f;
    const unsigned o = a.b.loff[node], e = a.b.loff[node + 1];
#pragma unroll 4
    for (unsigned t = o + lane; t < e; t += 32) {
        const int c = a.b.jc[t];
        if (c < 0) continue;
        const float rd = __ldcg(a.b.rdepth + c);
        const float* J = a.b.jrow + (long)t * 6;
#pragma unroll
        for (int q = 0; q < 6; ++q) acc[q] = acc[q] + J[q] * rd;
    }
    const unsigned io = a.b.ioff[node], nin = a.b.ioff[node + 1] - io;
    for (unsigned u = lane; u < nin + (unsigned)a.kreg; u += 32) {
        int src, kk;
        if (u < nin) {
            const unsigned ent = a.b.ilst[io + u];
            src = (int)(ent / a.kreg);
            kk = (int)(ent % a.kreg);
        } else {
            src = node;
            kk = (int)(u - nin);
            if (a.gidx[(long)node * a.kreg + kk] >= (uint32_t)n) continue;
        }
        float G[3][6];
        grad_rows(a.nodes + 3 * (long)src, G);
#pragma unroll
        for (int ax = 0; ax < 3; ++ax) {
            const float r = __ldcg(a.b.rreg + ((long)src * a.kreg + kk) * 3 + ax);
#pragma unroll
            for (int q = 0; q < 6; ++q) {
                const float g = G[ax][q] * a.lam_r;
                const float jn = (src == node) ? g : -g;
                acc[q] = acc[q] + jn * r;
            }
        }
    }
#pragma unroll
    for (int q = 0; q < 6; ++q) acc[q] = warp_sum(acc[q]);
}

// Row `i` of A z for node `node`: the node's blocks (diagonal first, then the neighbours in
// ascending order) times z, FP32.
AFX_D float spmv_entry(const GnBuffers& b, int node, int i, const float* z) {
    const int cnt = b.nbr_cnt[node];
    float acc = 0.f;
    {
        const float* B = b.diag + (long)node * 36 + i * 6;
        const float* x = z + (long)node * 6;
        float s = 0.f;
#pragma unroll
        for (int j = 0; j < 6; ++j) s = s + B[j] * __ldcg(x + j);
        acc = acc + s;
    }
#pragma unroll 2
    for (int u = 0; u < cnt; ++u) {
        const int ref = b.nbr_ref[(long)node * kMaxNbr + u];
        const float* x = z + (long)b.nbr[(long)node * kMaxNbr + u] * 6;
        float s = 0.f;
        if (ref >= 0) {
            const float* B = b.blocks + (long)ref * 36 + i * 6;
#pragma unroll
            for (int j = 0; j < 6; ++j) s = s + B[j] * __ldcg(x + j);
        } else {
            const float* B = b.blocks + (long)(-ref - 1) * 36 + i;
#pragma unroll
            for (int j = 0; j < 6; ++j) s = s + B[j * 6] * __ldcg(x + j);
        }
        acc = acc + s;
    }
    return acc;
}

// ---- PCG with the system resident in distributed shared memory ----
//
// For graphs up to kDsNpc nodes per CTA, each CTA of the cluster owns a contiguous node range
// and keeps, in its shared memory, the rows of J^T J for its nodes (diagonal block, then the
// neighbour blocks in ascending neighbour order, lower ones stored transposed so every block
// is row-major B_ij), their block inverses, its slices of x, r, p, A p, and a full copy of z.
// After each update a CTA writes its new z slice into every CTA's copy (st.shared::cluster), so
// the SpMV reads only local shared memory.  Partial sums are written into every CTA's slot
// array and summed locally in rank order after the cluster barrier: identical totals in all
// CTAs.  J^T J does not change during the Gauss-Newton loop, so the rows are staged once.

constexpr int kDsNodes = 1024;   // node limit of this path (full z copy)
constexpr int kDsNpc = 64;       // nodes per CTA
constexpr int kDsBlocks = 1024;  // blocks per CTA (diagonal included)
constexpr int kDsMaxCta = 16;

struct DsLayout {
    float* z;       // [kDsNodes * 6] full copy
    float* pf;      // [kDsNodes * 6] full copy of the search direction (each CTA forms it)
    float* x;       // [kDsNpc * 6] own slices
    float* r;
    float* ap;      // [kDsNpc * 6] own slice of A p
    float* minv;    // [kDsNpc * 36]
    float* blk;     // [kDsBlocks * 36]
    int* col;       // [kDsBlocks] neighbour node of each block
    int* rowptr;    // [kDsNpc + 1]
    double* slot;   // [2][kDsMaxCta][4]
    int* misc;      // [4]
};

constexpr size_t kDsSmem = sizeof(float) * ((size_t)kDsNodes * 12 + 3 * kDsNpc * 6 + kDsNpc * 36 + (size_t)kDsBlocks * 36) +
                           sizeof(int) * (kDsBlocks + kDsNpc + 1 + 4) + sizeof(double) * 2 * kDsMaxCta * 4 + 64;

AFX_D DsLayout ds_layout(void* base) {
    DsLayout d;
    double* dp = static_cast<double*>(base);
    d.slot = dp;
    float* f = reinterpret_cast<float*>(dp + 2 * kDsMaxCta * 4);
    d.z = f;
    f += kDsNodes * 6;
    d.pf = f;
    f += kDsNodes * 6;
    d.x = f;
    f += kDsNpc * 6;
    d.r = f;
    f += kDsNpc * 6;
    d.ap = f;
    f += kDsNpc * 6;
    d.minv = f;
    f += kDsNpc * 36;
    d.blk = f;
    f += (size_t)kDsBlocks * 36;
    int* ip = reinterpret_cast<int*>(f);
    d.col = ip;
    ip += kDsBlocks;
    d.rowptr = ip;
    ip += kDsNpc + 1;
    d.misc = ip;
    return d;
}

// Store to the same shared-memory offset in CTA `rank` of this cluster.
AFX_D void dsmem_store_f32(float* local, unsigned rank, float v) {
    unsigned a = (unsigned)__cvta_generic_to_shared(local), ra;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(ra) : "r"(a), "r"(rank));
    asm volatile("st.shared::cluster.f32 [%0], %1;" ::"r"(ra), "f"(v) : "memory");
}
AFX_D void dsmem_store_f64(double* local, unsigned rank, double v) {
    unsigned a = (unsigned)__cvta_generic_to_shared(local), ra;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(ra) : "r"(a), "r"(rank));
    asm volatile("st.shared::cluster.f64 [%0], %1;" ::"r"(ra), "d"(v) : "memory");
}
// A double-float into an 8-byte slot of CTA `rank` (hi at the lower address).
AFX_D void dsmem_store_df(double* local, unsigned rank, DF v) {
    unsigned a = (unsigned)__cvta_generic_to_shared(local), ra;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(ra) : "r"(a), "r"(rank));
    asm volatile("st.shared::cluster.v2.f32 [%0], {%1, %2};" ::"r"(ra), "f"(v.hi), "f"(v.lo) : "memory");
}


// Cluster sum through the slot arrays: the CTA's block total is written into slot[ph][rank] of
// every CTA; after the barrier each CTA adds the slots in rank order.
// `live` (warp-uniform) is false for warps whose lanes hold only zeros: they skip the FP64
// butterfly (FP64 issue is scarce on this part) and contribute an exact 0.
template <int NV>
AFX_D void ds_sum(double (&v)[NV], const DsLayout& d, ClusterSums& cs, int& ph, bool live = true) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const unsigned rank = cluster_rank(), ncta = cluster_size();
#pragma unroll
    for (int i = 0; i < NV; ++i) {
        const double s = live ? warp_sum(v[i]) : 0.0;
        if (lane == 0) cs.warp[w * 4 + i] = s;
    }
    __syncthreads();
    if (w == 0) {
#pragma unroll
        for (int i = 0; i < NV; ++i) {
            double s = lane < kLoopWarps ? cs.warp[lane * 4 + i] : 0.0;
#pragma unroll
            for (int o = kLoopWarps / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
            // lane q < ncta sends the total to CTA q
            if (lane < (int)ncta) dsmem_store_f64(d.slot + (ph * kDsMaxCta + rank) * 4 + i, lane, s);
        }
    }
    cluster_barrier();
    if (w == 0) {
#pragma unroll
        for (int i = 0; i < NV; ++i) {
            double t = lane < (int)ncta ? d.slot[(ph * kDsMaxCta + lane) * 4 + i] : 0.0;
#pragma unroll
            for (int o = kDsMaxCta / 2; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
            if (lane == 0) cs.total[i] = t;
        }
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < NV; ++i) v[i] = cs.total[i];
    ph ^= 1;
}

// Stage this CTA's rows; returns (uniformly over the cluster) whether every CTA's rows fit.
AFX_D bool ds_stage(const GnBuffers& b, int n, const DsLayout& d, ClusterSums& cs, int& ph) {
    const unsigned rank = cluster_rank(), ncta = cluster_size();
    const int npc = (n + (int)ncta - 1) / (int)ncta;
    const int start = min(n, (int)rank * npc), own = min(n, start + npc) - start;
    if (threadIdx.x < 32) {
        // row pointers: diagonal + neighbour blocks per own node (one warp, inclusive scan)
        int carry = 0;
        for (int base = 0; base < own; base += 32) {
            const int li = base + (int)threadIdx.x;
            const int c = li < own ? 1 + b.nbr_cnt[start + li] : 0;
            int incl = c;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, incl, o);
                if ((int)threadIdx.x >= o) incl += y;
            }
            if (li < own) d.rowptr[li] = carry + incl - c;
            carry += __shfl_sync(0xffffffffu, incl, 31);
        }
        if (threadIdx.x == 0) {
            d.rowptr[own] = carry;
            d.misc[0] = carry;
        }
    }
    __syncthreads();
    double need[1] = {d.misc[0] > kDsBlocks ? 1.0 : 0.0};
    ds_sum<1>(need, d, cs, ph);
    if (need[0] != 0.0) return false;
    // copy the rows (block-major, 36 floats each) and the inverses
    for (int li = threadIdx.x >> 5; li < own; li += kLoopWarps) {
        const int node = start + li;
        const int lane = threadIdx.x & 31;
        const int r0 = d.rowptr[li], cnt = d.rowptr[li + 1] - r0 - 1;
        for (int e = lane; e < 36; e += 32) {
            d.blk[r0 * 36 + e] = b.diag[(long)node * 36 + e];
            d.minv[li * 36 + e] = b.minv[(long)node * 36 + e];
        }
        if (lane == 0) d.col[r0] = node;
        for (int u = 0; u < cnt; ++u) {
            const int ref = b.nbr_ref[(long)node * kMaxNbr + u];
            const float* src = b.blocks + (long)(ref >= 0 ? ref : -ref - 1) * 36;
            float* dst = d.blk + (r0 + 1 + u) * 36;
            for (int e = lane; e < 36; e += 32) dst[e] = ref >= 0 ? src[e] : src[(e % 6) * 6 + e / 6];
            if (lane == 0) d.col[r0 + 1 + u] = b.nbr[(long)node * kMaxNbr + u];
        }
    }
    __syncthreads();
    return true;
}

// Dot products x[i] . y[i] of the CTA's own entries (cnt floats each, in shared memory), summed
// over the cluster in double-float arithmetic (about 48 bits; each product enters exactly).  Warp 0
// alone does the work: lane l accumulates entries l, l + 32, ..., a butterfly gives the CTA's sum,
// and lane q sends it into slot [ph][rank] of CTA q.  After the cluster barrier warp 0 of every CTA
// adds the slots in one fixed tree, so all CTAs hold bit-identical totals.  Returns true in lane 0
// of warp 0 only, with the totals in t; the caller turns them into the scalars every thread reads
// after the next __syncthreads.
template <int NV>
AFX_D bool ds_dot(const float* const (&x)[NV], const float* const (&y)[NV], int cnt, const DsLayout& d, int& ph,
                  DF (&t)[NV]) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const unsigned rank = cluster_rank(), ncta = cluster_size();
    __syncthreads();  // the staged vectors are complete
    if (w == 0) {
#pragma unroll
        for (int i = 0; i < NV; ++i) {
            DF s = {0.f, 0.f};
            for (int o = lane; o < cnt; o += 32) s = df_add(s, df_prod(x[i][o], y[i][o]));
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) s = df_add(s, df_shfl_xor(s, o));
            if (lane < (int)ncta) dsmem_store_df(d.slot + (ph * kDsMaxCta + rank) * 4 + i, lane, s);
        }
    }
    cluster_barrier();
    const int p = ph;
    ph ^= 1;
    if (w != 0) return false;
#pragma unroll
    for (int i = 0; i < NV; ++i) {
        DF v = {0.f, 0.f};
        if (lane < (int)ncta) v = lds_df_local(d.slot + (p * kDsMaxCta + lane) * 4 + i);
#pragma unroll
        for (int o = kDsMaxCta / 2; o > 0; o >>= 1) v = df_add(v, df_shfl_xor(v, o));
        t[i] = v;
    }
    return lane == 0;
}

// One PCG solve (same recurrences as the global-memory path), then T_pending -= [x] for the own
// nodes.  J^T r is read from b.jtr.  Per iteration: p = z + beta p over all nodes (each CTA keeps a
// full copy of p and of z), A p of the own rows with up to 32 lanes per row (each summing a fixed
// stride of the row's blocks, then a butterfly), p.Ap (cluster dot), the own x / r / z updates with
// z sent to every CTA's copy, r.z (and r.r when a tolerance is set; cluster dot).  The step sizes
// are formed once per CTA by lane 0 (df_quotient) and read from shared memory.
AFX_D void pcg_ds(const LoopArgs& L, int n, const DsLayout& d, ClusterSums& cs, int& ph) {
    const GnBuffers& b = L.g.b;
    const unsigned rank = cluster_rank(), ncta = cluster_size();
    const int npc = (n + (int)ncta - 1) / (int)ncta;
    const int start = min(n, (int)rank * npc), own = min(n, start + npc) - start;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int grp = lane / 6, ei = lane - 6 * grp;
    const int li = w * 5 + grp;  // kLoopWarps * 5 >= kDsNpc: one own node per lane group
    const bool act = lane < 30 && li < own;
    const int o = li * 6 + ei;
    const int gnode = start + li;
    const int cnt = own * 6;
    const bool tol = L.tol > 0;
    float* zown = d.z + (long)start * 6;
    float* pown = d.pf + (long)start * 6;
    // SpMV lanes per row: the largest power of two with every own row covered in one pass
    int R = 1;
    while (R < 32 && 2 * R * cnt <= (int)blockDim.x) R <<= 1;
    // x = 0, r = b, z = M^-1 r
    {
        const float ji = act ? __ldcg(b.jtr + (long)gnode * 6 + ei) : 0.f;
        float zi = 0.f;
#pragma unroll
        for (int q = 0; q < 6; ++q) {
            const float rq = __shfl_sync(0xffffffffu, ji, lane < 30 ? grp * 6 + q : q);
            if (act) zi = zi + d.minv[li * 36 + ei * 6 + q] * rq;
        }
        if (act) {
            d.x[o] = 0.f;
            d.r[o] = ji;
            zown[o] = zi;
            for (unsigned q = 0; q < ncta; ++q)
                if (q != rank) dsmem_store_f32(d.z + (long)gnode * 6 + ei, q, zi);
        }
    }
    // tol^2 in binary32, for the stopping test of lane 0 of warp 0
    const float tol2 = (tol && threadIdx.x == 0) ? (float)(L.tol * L.tol) : 0.f;
    {
        DF t[2];
        bool lead;
        if (tol) lead = ds_dot<2>({d.r, d.r}, {zown, d.r}, cnt, d, ph, t);
        else {
            DF t1[1];
            lead = ds_dot<1>({d.r}, {zown}, cnt, d, ph, t1);
            t[0] = t1[0];
            t[1] = {0.f, 0.f};
        }
        if (lead) {
            cs.rz_df = t[0];
            cs.bn_df = t[1];
            cs.stop = 0;
        }
    }
    __syncthreads();
    float beta = 0.f;
    for (int it = 0; it < L.pcg_iters; ++it) {
        // p = z (first iteration) or z + beta p, formed for all nodes by every CTA from its copies
        for (int i = threadIdx.x; i < n * 6; i += blockDim.x) d.pf[i] = it ? d.z[i] + beta * d.pf[i] : d.z[i];
        __syncthreads();
        // A p of the own rows
        const int rows_per_pass = (int)blockDim.x / R;
        for (int base = 0; base < cnt; base += rows_per_pass) {
            const int q = base + (int)threadIdx.x / R, part = (int)threadIdx.x % R;
            float acc = 0.f;
            if (q < cnt) {
                const int l = q / 6, e = q - 6 * l;
                const int r1 = d.rowptr[l + 1];
                for (int bk = d.rowptr[l] + part; bk < r1; bk += R) {
                    const float* B = d.blk + bk * 36 + e * 6;
                    const float* xv = d.pf + d.col[bk] * 6;
                    float s = 0.f;
#pragma unroll
                    for (int j = 0; j < 6; ++j) s = s + B[j] * xv[j];
                    acc = acc + s;
                }
            }
            for (int m = R / 2; m > 0; m >>= 1) acc = acc + __shfl_xor_sync(0xffffffffu, acc, m);
            if (q < cnt && part == 0) d.ap[q] = acc;
        }
        {
            DF t[1];
            if (ds_dot<1>({pown}, {d.ap}, cnt, d, ph, t)) {
                cs.stop = df_zero_or_nan(t[0]) ? 1 : 0;
                cs.alpha = cs.stop ? 0.f : df_quotient(cs.rz_df, t[0]);
            }
        }
        __syncthreads();
        if (cs.stop) break;
        const float alpha = cs.alpha;
        float rv = 0.f;
        if (act) {
            d.x[o] = d.x[o] + alpha * pown[o];
            rv = d.r[o] - alpha * d.ap[o];
            d.r[o] = rv;
        }
        float zi = 0.f;
#pragma unroll
        for (int q = 0; q < 6; ++q) {
            const float rq = __shfl_sync(0xffffffffu, rv, lane < 30 ? grp * 6 + q : q);
            if (act) zi = zi + d.minv[li * 36 + ei * 6 + q] * rq;
        }
        // z is read (forming p) before the p.Ap barrier in every CTA, so it can be overwritten here
        if (act) {
            zown[o] = zi;
            for (unsigned q = 0; q < ncta; ++q)
                if (q != rank) dsmem_store_f32(d.z + (long)gnode * 6 + ei, q, zi);
        }
        {
            DF t[2];
            bool lead;
            if (tol) lead = ds_dot<2>({d.r, d.r}, {zown, d.r}, cnt, d, ph, t);
            else {
                DF t1[1];
                lead = ds_dot<1>({d.r}, {zown}, cnt, d, ph, t1);
                t[0] = t1[0];
                t[1] = {0.f, 0.f};
            }
            if (lead) {
                cs.beta = df_quotient(t[0], cs.rz_df);
                cs.rz_df = t[0];
                cs.stop = (tol && t[1].hi <= tol2 * cs.bn_df.hi) ? 1 : 0;
            }
        }
        __syncthreads();
        beta = cs.beta;
        if (cs.stop) break;
    }
    // T_pending -= [[x_rot]x, x_t; 0] for the own nodes (updateTransformsKernel,
    // src/MotionOptimization.cu:483-498); x also to global memory for inspection
    __syncthreads();
    for (int t = threadIdx.x; L.T_pending && t < own * 16; t += blockDim.x) {
        const int l = t >> 4, e = t & 15;
        const float* u = d.x + l * 6;
        float U;
        switch (e) {
            case 1: U = u[2]; break;
            case 2: U = -u[1]; break;
            case 4: U = -u[2]; break;
            case 6: U = u[0]; break;
            case 8: U = u[1]; break;
            case 9: U = -u[0]; break;
            case 12: U = u[3]; break;
            case 13: U = u[4]; break;
            case 14: U = u[5]; break;
            default: U = 0.f;
        }
        float* T = L.T_pending + (long)(start + l) * 16 + e;
        __stcg(T, __ldcg(T) - U);
    }
    for (int t = threadIdx.x; t < own * 6; t += blockDim.x) __stcg(b.x + (long)start * 6 + t, d.x[t]);
}

// ---- phases of the Gauss-Newton loop (all CTAs of the cluster unless stated) ----

// Residuals (fill_r_DepthKernel / fill_r_MRegKernel, src/MotionOptimization.cu:163-227) with
// the transforms T; partial FP64 energies of this thread (runSquareKernel + reductions,
// src/VolumeFusion.cu:575-588).
AFX_D void gn_residuals(const GnArgs& a, const float* warped, const float* T, int n, long ncorr, long gt, long gstride,
                        double (&e2)[2]) {
    const GnBuffers& b = a.b;
    const long nreg = (long)n * a.kreg;
    for (long c = gt; c < ncorr; c += gstride) {
        const long v = a.corr[2 * c], px = a.corr[2 * c + 1];
        const float* f = a.frame + 3 * px;
        float d[3] = {__ldcg(warped + 3 * v) - f[0], __ldcg(warped + 3 * v + 1) - f[1], __ldcg(warped + 3 * v + 2) - f[2]};
        const float r = a.lam_d * dot3(a.normals + 3 * px, d);
        __stcg(b.rdepth + c, r);
        e2[0] += (double)(r * r);
    }
    for (long t = gt; t < nreg; t += gstride) {
        const int i = (int)(t / a.kreg);
        const uint32_t nb = a.gidx[t];
        float* rr = b.rreg + 3 * t;
        if (nb >= (uint32_t)n) {
            __stcg(rr, 0.f);
            __stcg(rr + 1, 0.f);
            __stcg(rr + 2, 0.f);
            continue;
        }
        float Ti[16], Tn[16], tc[3], tn[3];
#pragma unroll
        for (int e = 0; e < 16; ++e) {
            Ti[e] = __ldcg(T + 16 * (long)i + e);
            Tn[e] = __ldcg(T + 16 * (long)nb + e);
        }
        mat4_point(Ti, a.nodes + 3 * (long)i, tc);
        mat4_point(Tn, a.nodes + 3 * (long)i, tn);
        for (int ax = 0; ax < 3; ++ax) {
            const float r = (tc[ax] - tn[ax]) * a.lam_r;
            __stcg(rr + ax, r);
            e2[1] += (double)(r * r);
        }
    }
}

// J^T r of every node into b.jtr (one node per warp).
AFX_D void gn_jtr(const GnArgs& a, int n, int gw, int nw) {
    const int lane = threadIdx.x & 31;
    for (int node = gw; node < n; node += nw) {
        float jv[6];
        jtr_node(a, node, n, jv);
        if (lane < 6) {
            float ji = jv[0];
#pragma unroll
            for (int q = 1; q < 6; ++q)
                if (lane == q) ji = jv[q];
            __stcg(a.b.jtr + (long)node * 6 + lane, ji);
        }
    }
}

// PCG with the vectors in global memory (graphs above the shared-memory limit); J^T r from
// b.jtr, solution in b.x.  Same recurrences and arithmetic as pcg_ds.
AFX_D void pcg_global(const LoopArgs& L, int n, ClusterSums& cs) {
    const GnBuffers& b = L.g.b;
    const unsigned rank = cluster_rank(), ncta = cluster_size();
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int gw = (int)rank * kLoopWarps + w, nw = (int)ncta * kLoopWarps;
    const int grp = lane / 6, ei = lane - 6 * grp;
    const bool glane = lane < 30;
    const int gstep = nw * 5;
    // x = 0, r = b, z = M^-1 r; rz = r.z, bb = b.b
    DF d2[2] = {{0.f, 0.f}, {0.f, 0.f}};
    for (int base = gw * 5; base < n; base += gstep) {  // warp-uniform trip count
        const int node = base + grp;
        const bool act = glane && node < n;
        const long o = (long)node * 6 + ei;
        const float ji = act ? __ldcg(b.jtr + o) : 0.f;
        float zi = 0.f;
        const float* Mi = b.minv + (long)(act ? node : 0) * 36 + ei * 6;
#pragma unroll
        for (int q = 0; q < 6; ++q) {
            const float rq = __shfl_sync(0xffffffffu, ji, glane ? grp * 6 + q : q);
            if (act) zi = zi + Mi[q] * rq;
        }
        if (act) {
            __stcg(b.x + o, 0.f);
            __stcg(b.r + o, ji);
            __stcg(b.z + o, zi);
            d2[0] = df_add(d2[0], df_prod(ji, zi));
            d2[1] = df_add(d2[1], df_prod(ji, ji));
        }
    }
    cluster_sum_df<2>(d2, cs);
    // six lanes per node (entry i = lane % 6 of node group lane / 6, five groups per warp)
    DF rz = d2[0];
    const DF bnorm2 = d2[1];
    const float tol2 = L.tol > 0 ? (float)(L.tol * L.tol) : 0.f;
    float beta = 0.f;
    for (int it = 0; it < L.pcg_iters; ++it) {
        // p = z (first iteration) or z + beta p for the own entries, then A p once all are written
        for (int base = gw * 5; base < n; base += gstep) {
            const int node = base + grp;
            if (glane && node < n) {
                const long o = (long)node * 6 + ei;
                const float zi = __ldcg(b.z + o);
                __stcg(b.p + o, it ? zi + beta * __ldcg(b.p + o) : zi);
            }
        }
        cluster_barrier();
        DF pap[1] = {{0.f, 0.f}};
        if (glane)
            for (int node = gw * 5 + grp; node < n; node += gstep) {
                const long o = (long)node * 6 + ei;
                const float api = spmv_entry(b, node, ei, b.p);
                __stcg(b.ap + o, api);
                pap[0] = df_add(pap[0], df_prod(__ldcg(b.p + o), api));
            }
        cluster_sum_df<1>(pap, cs);
        if (df_zero_or_nan(pap[0])) break;
        const float alpha = df_quotient(rz, pap[0]);
        // x += alpha p; r -= alpha A p; z = M^-1 r; r.z, r.r
        DF q2[2] = {{0.f, 0.f}, {0.f, 0.f}};
        for (int base = gw * 5; base < n; base += gstep) {
            const int node = base + grp;
            const bool act = glane && node < n;
            const long o = (long)node * 6 + ei;
            float rv = 0.f;
            if (act) {
                __stcg(b.x + o, __ldcg(b.x + o) + alpha * __ldcg(b.p + o));
                rv = __ldcg(b.r + o) - alpha * __ldcg(b.ap + o);
                __stcg(b.r + o, rv);
            }
            float zi = 0.f;
            const float* Mi = b.minv + (long)(act ? node : 0) * 36 + ei * 6;
#pragma unroll
            for (int q = 0; q < 6; ++q) {
                const float rq = __shfl_sync(0xffffffffu, rv, glane ? grp * 6 + q : q);
                if (act) zi = zi + Mi[q] * rq;
            }
            if (act) {
                __stcg(b.z + o, zi);
                q2[0] = df_add(q2[0], df_prod(rv, zi));
                q2[1] = df_add(q2[1], df_prod(rv, rv));
            }
        }
        cluster_sum_df<2>(q2, cs);
        beta = df_quotient(q2[0], rz);
        rz = q2[0];
        if (L.tol > 0 && q2[1].hi <= tol2 * bnorm2.hi) break;
    }
}

// T -= [[x_rot]x, x_t; 0] for nodes [lo, hi) with x in global memory (updateTransformsKernel,
// src/MotionOptimization.cu:483-498); entry e of node i by thread (i - lo) * 16 + e.
AFX_D void update_transforms_range(float* T, const float* x, int lo, int hi, long t0, long tstride) {
    for (long t = t0; t < (long)(hi - lo) * 16; t += tstride) {
        const long node = lo + t / 16;
        const int e = (int)(t & 15);
        const float* u = x + node * 6;
        float U;
        switch (e) {
            case 1: U = __ldcg(u + 2); break;
            case 2: U = -__ldcg(u + 1); break;
            case 4: U = -__ldcg(u + 2); break;
            case 6: U = __ldcg(u + 0); break;
            case 8: U = __ldcg(u + 1); break;
            case 9: U = -__ldcg(u + 0); break;
            case 12: U = __ldcg(u + 3); break;
            case 13: U = __ldcg(u + 4); break;
            case 14: U = __ldcg(u + 5); break;
            default: U = 0.f;
        }
        float* Te = T + node * 16 + e;
        __stcg(Te, __ldcg(Te) - U);
    }
}

// Canonical vertices warped by T (warpKernel, src/ComputeCorrespondence.cu:13-30, or the dual-quaternion
// blend of afx_dqb.cuh).  T is written by other CTAs of this launch: read through L2.
AFX_D void gn_rewarp(const GnArgs& a, const float* points, float* warped, const float* T, long m, long gt,
                     long gstride) {
    if (a.blend == AFX_BLEND_DQB) {
        for (long i = gt; i < m; i += gstride) {
            const float p[3] = {points[3 * i], points[3 * i + 1], points[3 * i + 2]};
            float o[3];
            dq_blend_point(
                [T](uint32_t nb, float* Tn) {
#pragma unroll
                    for (int e = 0; e < 16; ++e) Tn[e] = __ldcg(T + 16 * (long)nb + e);
                },
                a.midx + i * a.k, a.mw + i * a.k, a.k, AFX_INVALID_INDEX, p, o);
            __stcg(warped + 3 * i, o[0]);
            __stcg(warped + 3 * i + 1, o[1]);
            __stcg(warped + 3 * i + 2, o[2]);
        }
        return;
    }
    for (long i = gt; i < m; i += gstride) {
        const float p[3] = {points[3 * i], points[3 * i + 1], points[3 * i + 2]};
        bool zero = true;
        for (int j = 0; j < a.k; ++j)
            if (!(fabsf(a.mw[i * a.k + j]) <= 1e-5f)) zero = false;
        float acc[3] = {p[0], p[1], p[2]};
        if (!zero) {
            acc[0] = acc[1] = acc[2] = 0.f;
            for (int j = 0; j < a.k; ++j) {
                const uint32_t nb = a.midx[i * a.k + j];
                if (nb == AFX_INVALID_INDEX) continue;
                float Tn[16], o[3];
#pragma unroll
                for (int e = 0; e < 16; ++e) Tn[e] = __ldcg(T + 16 * (long)nb + e);
                mat4_point(Tn, p, o);
                const float wj = a.mw[i * a.k + j];
                acc[0] = acc[0] + wj * o[0];
                acc[1] = acc[1] + wj * o[1];
                acc[2] = acc[2] + wj * o[2];
            }
        }
        __stcg(warped + 3 * i, acc[0]);
        __stcg(warped + 3 * i + 1, acc[1]);
        __stcg(warped + 3 * i + 2, acc[2]);
    }
}

// One solve from b.jtr: x in b.x (and in the own slices of the shared-memory layout); with
// L.T_pending set, T_pending -= [x] as well.  Ends with a cluster barrier.
AFX_D void gn_solve(const LoopArgs& L, int n, bool ds, const DsLayout& dsl, ClusterSums& cs, int& ds_ph, long gt,
                    long gstride) {
    if (ds) {
        pcg_ds(L, n, dsl, cs, ds_ph);
    } else {
        pcg_global(L, n, cs);
        cluster_barrier();  // x complete
        if (L.T_pending) update_transforms_range(L.T_pending, L.g.b.x, 0, n, gt, gstride);
    }
    cluster_barrier();
}

__global__ void __launch_bounds__(kLoopThreads, 1) gn_loop_kernel(LoopArgs L) {
    const GnArgs& a = L.g;
    const GnBuffers& b = a.b;
    __shared__ ClusterSums cs;
    extern __shared__ double ds_smem[];
    if (threadIdx.x == 0) cs.phase = 0;
    // Every CTA of the cluster must be running before any thread touches another CTA's shared
    // memory (the first such store is in ds_stage).  Under load the CTAs of a cluster need not
    // start together; a store into a CTA that has not started is an SM fault.
    cluster_barrier();
    const unsigned rank = cluster_rank(), ncta = cluster_size();
    const int w = threadIdx.x >> 5;
    const long gt = (long)rank * kLoopThreads + threadIdx.x, gstride = (long)ncta * kLoopThreads;
    const int gw = (int)rank * kLoopWarps + w, nw = (int)ncta * kLoopWarps;
    const bool leader = rank == 0 && threadIdx.x == 0;
    const int n = min(*a.n_nodes, a.n_max);
    const long ncorr = min((long)*a.corr_count, a.c_max);
    const long m = min((long)*a.mesh_count, a.m_max);
    GnState* s = b.state;
    double e_prev = s->e_prev;
    bool done = s->done != 0;
    // small graphs: the system lives in distributed shared memory for the whole loop
    const DsLayout dsl = ds_layout(ds_smem);
    int ds_ph = 0;
    const bool ds = !done && n > 0 && (n + (int)ncta - 1) / (int)ncta <= kDsNpc && ds_stage(b, n, dsl, cs, ds_ph);
    for (int iter = 0; iter < L.gn_iters && !done; ++iter) {
        double e2[2] = {0.0, 0.0};
        gn_residuals(a, L.warped, L.T_pending, n, ncorr, gt, gstride, e2);
        cluster_sum<2>(e2, cs);
        // ---- energy test and commit decision (src/VolumeFusion.cu:589-598)
        const double e = e2[0] + e2[1];
        if (leader) {
            s->e_last = e;
            s->e_depth = e2[0];
            s->e_reg = e2[1];
        }
        if (e_prev - e < (double)a.min_step) {
            if (leader) s->done = 1;
            done = true;
            break;
        }
        e_prev = e;
        const bool commit = iter != 0;
        if (leader) {
            s->e_prev = e;
            s->commit = commit;
            s->iters = iter + 1;
        }
        if (commit)
            for (long t = gt; t < (long)n * 16; t += gstride) L.T_committed[t] = __ldcg(L.T_pending + t);
        gn_jtr(a, n, gw, nw);
        cluster_barrier();
        gn_solve(L, n, ds, dsl, cs, ds_ph, gt, gstride);
        gn_rewarp(a, L.points, L.warped, L.T_pending, m, gt, gstride);
        cluster_barrier();
    }
    // no CTA leaves while another may still read its shared memory
    cluster_barrier();
}

// One PCG solve of a system assembled by afx_gn_build (J^T J blocks, inverses and J^T r in the
// workspace); x in b.x.
__global__ void __launch_bounds__(kLoopThreads, 1) gn_solve_kernel(LoopArgs L) {
    const GnArgs& a = L.g;
    __shared__ ClusterSums cs;
    extern __shared__ double ds_smem[];
    if (threadIdx.x == 0) cs.phase = 0;
    cluster_barrier();  // every CTA running before any access to another CTA's shared memory
    const unsigned rank = cluster_rank(), ncta = cluster_size();
    const long gt = (long)rank * kLoopThreads + threadIdx.x, gstride = (long)ncta * kLoopThreads;
    const int n = min(*a.n_nodes, a.n_max);
    const DsLayout dsl = ds_layout(ds_smem);
    int ds_ph = 0;
    const bool ds = n > 0 && (n + (int)ncta - 1) / (int)ncta <= kDsNpc && ds_stage(a.b, n, dsl, cs, ds_ph);
    gn_solve(L, n, ds, dsl, cs, ds_ph, gt, gstride);
    // no CTA leaves while another may still read its shared memory
    cluster_barrier();
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

// Cluster size for gn_loop_kernel: 16 CTAs where the device runs non-portable clusters of
// that size, else the portable 8.
static int gn_cluster_size() {
    static ContextOnce once;
    static int cached_dev[kMaxDevices];
    once_per_context(once, [](int dev) {
        int cached = 0;
        cudaFuncSetAttribute(gn_loop_kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        cudaFuncSetAttribute(gn_loop_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kDsSmem);
        cudaFuncSetAttribute(gn_solve_kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        cudaFuncSetAttribute(gn_solve_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kDsSmem);
        const int sizes[2] = {16, 8};
        for (int c : sizes) {
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = dim3(c);
            cfg.blockDim = dim3(kLoopThreads);
            cfg.dynamicSmemBytes = kDsSmem;
            cudaLaunchAttribute at[1];
            at[0].id = cudaLaunchAttributeClusterDimension;
            at[0].val.clusterDim.x = c;
            at[0].val.clusterDim.y = 1;
            at[0].val.clusterDim.z = 1;
            cfg.attrs = at;
            cfg.numAttrs = 1;
            int clusters = 0;
            if (cudaOccupancyMaxActiveClusters(&clusters, gn_loop_kernel, &cfg) == cudaSuccess && clusters > 0) {
                cached = c;
                break;
            }
            cudaGetLastError();
        }
        cached_dev[dev] = cached ? cached : 8;
        return (int)AFX_OK;
    });
    int dev = 0;
    cudaGetDevice(&dev);
    return cached_dev[dev] ? cached_dev[dev] : 8;
}

size_t gn_workspace_size(long m_max, int n_max, int k, int kreg) {
    size_t s = 0;
    s += 3 * al((n_max + 1) * 4) + al(m_max * k * 4);           // lcnt loff lcur lst
    s += 3 * al((n_max + 1) * 4) + al((size_t)n_max * kreg * 4);  // icnt ioff icur ilst
    s += al(n_max * 4) + 2 * al((size_t)n_max * kMaxNbr * 4);     // nbr_cnt nbr nbr_ref
    s += al((size_t)n_max * kMaxNbr * 36 * 4) + al((size_t)n_max * 36 * 4) + al((size_t)n_max * 36 * 4);
    s += al((size_t)m_max * k * 6 * 4) + al((size_t)m_max * k * 4);  // jrow jc
    s += al((size_t)n_max * 6 * 4) * 5 + al((size_t)n_max * 6 * 4 * 2);  // jtr x r z p, ap + p2
    s += al(m_max * 4) + al((size_t)n_max * kreg * 3 * 4);        // rdepth rreg
    s += al(sizeof(GnState));
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
    b->minv = (float*)take((size_t)n_max * 36 * 4);
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
    b->state = (GnState*)take(sizeof(GnState));
    b->scan_ws = take(scan_workspace_size(m_max > n_max ? m_max : n_max));
    return true;
}

// Per frame: node -> vertex lists and incoming regularisation edges.
int gn_frame_setup(const GnArgs& a, cudaStream_t st) {
    const GnBuffers& b = a.b;
    AFX_CUDA(cudaMemsetAsync(b.lcnt, 0, (a.n_max + 1) * 4, st));
    AFX_CUDA(cudaMemsetAsync(b.lcur, 0, (a.n_max + 1) * 4, st));
    AFX_CUDA(cudaMemsetAsync(b.icnt, 0, (a.n_max + 1) * 4, st));
    AFX_CUDA(cudaMemsetAsync(b.icur, 0, (a.n_max + 1) * 4, st));
    const long mk = a.m_max * a.k;
    if (mk > 0) {
        lst_count_kernel<<<grid_for(mk, 256), 256, 0, st>>>(a);
        AFX_LAUNCH_CHECK();
    }
    int rc = scan_exclusive(b.lcnt, b.loff, a.n_max + 1, nullptr, b.scan_ws, st);
    if (rc) return rc;
    if (mk > 0) {
        lst_fill_kernel<<<grid_for(mk, 256), 256, 0, st>>>(a);
        AFX_LAUNCH_CHECK();
    }
    seg_sort_kernel<<<grid_for_nodes(a.n_max, 1), 256, 0, st>>>(b.lst, b.loff, a.n_nodes, a.n_max, a.error);
    AFX_LAUNCH_CHECK();
    const long nk = (long)a.n_max * a.kreg;
    in_count_kernel<<<grid_for(nk, 256), 256, 0, st>>>(a);
    AFX_LAUNCH_CHECK();
    rc = scan_exclusive(b.icnt, b.ioff, a.n_max + 1, nullptr, b.scan_ws, st);
    if (rc) return rc;
    in_fill_kernel<<<grid_for(nk, 256), 256, 0, st>>>(a);
    AFX_LAUNCH_CHECK();
    seg_sort_kernel<<<grid_for_nodes(a.n_max, 1), 256, 0, st>>>(b.ilst, b.ioff, a.n_nodes, a.n_max, a.error);
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
    if (T_pending)
        AFX_CUDA(cudaMemcpyAsync(T_pending, T_committed, (size_t)a.n_max * 64, cudaMemcpyDeviceToDevice, st));
    const unsigned nb = grid_for_nodes(a.n_max, kGnWarps);  // grid-stride over the live nodes
    const int words = (a.n_max + 31) / 32;
    const size_t smem = (size_t)kGnWarps * words * 4;
    if (smem > 200 * 1024) return AFX_ERR_UNSUPPORTED;
    static ContextOnce once;  // the opt-in covers every size accepted above
    if (smem > 48 * 1024) {
        const int rc = once_per_context(once, [](int) {
            return note_cuda_error(
                cudaFuncSetAttribute(nbr_discover_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
        });
        if (rc) return rc;
    }
    nbr_discover_kernel<<<nb, 32 * kGnWarps, smem, st>>>(a, words);
    AFX_LAUNCH_CHECK();
    nbr_ref_kernel<<<grid_for((long)a.n_max * kMaxNbr, 256), 256, 0, st>>>(a);
    AFX_LAUNCH_CHECK();
    jtj_assemble_kernel<<<grid_for_nodes(a.n_max, kJtjWarps), 32 * kJtjWarps, 0, st>>>(a);
    AFX_LAUNCH_CHECK();
    diag_inverse_kernel<<<grid_for_nodes(a.n_max, 4), 128, 0, st>>>(a);
    AFX_LAUNCH_CHECK();
    return AFX_OK;
}

// All Gauss-Newton iterations of one ICP iteration (src/VolumeFusion.cu:571-691): one launch
// of gn_loop_kernel.  On return (stream order) T_committed holds the last accepted transforms,
// T_pending the last update and `warped` the canonical vertices warped by T_pending.
static int launch_cluster(void (*kernel)(LoopArgs), const LoopArgs& L, cudaStream_t st) {
    const int c = gn_cluster_size();
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(c);
    cfg.blockDim = dim3(kLoopThreads);
    cfg.dynamicSmemBytes = kDsSmem;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = c;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    AFX_CUDA(cudaLaunchKernelEx(&cfg, kernel, L));
    AFX_LAUNCH_CHECK();
    return AFX_OK;
}

int gn_loop(const GnArgs& a, const float* points, float* warped, float* T_committed, float* T_pending, int gn_iters,
            int pcg_iters, double tol, cudaStream_t st) {
    if (gn_iters <= 0) return AFX_OK;
    LoopArgs L;
    L.g = a;
    L.points = points;
    L.warped = warped;
    L.T_committed = T_committed;
    L.T_pending = T_pending;
    L.gn_iters = gn_iters;
    L.pcg_iters = pcg_iters;
    L.tol = tol;
    return launch_cluster(gn_loop_kernel, L, st);
}

}  // namespace afx

// ------------------------------------------------------------------------------------
// Stand-alone Gauss-Newton operators: residuals, J^T J / J^T r (exported in the reference's dense
// layout), the PCG solve and the transform update, for callers that drive the steps themselves.
// ------------------------------------------------------------------------------------

namespace afx {

__global__ void gn_corr_of_vertex_kernel(const int* corr, const unsigned* n_corr, long c_max, int* cov) {
    const long nc = min((long)*n_corr, c_max);
    AFX_GRID_STRIDE(c, nc) cov[corr[2 * c]] = (int)c;
}

__global__ void __launch_bounds__(256) gn_residual_kernel(GnArgs a, const float* warped, const float* T) {
    const int n = min(*a.n_nodes, a.n_max);
    const long ncorr = min((long)*a.corr_count, a.c_max);
    double e2[2] = {0.0, 0.0};
    gn_residuals(a, warped, T, n, ncorr, blockIdx.x * (long)blockDim.x + threadIdx.x, (long)gridDim.x * blockDim.x, e2);
}

__global__ void __launch_bounds__(256) gn_jtr_kernel(GnArgs a) {
    const int n = min(*a.n_nodes, a.n_max);
    const int gw = (int)((blockIdx.x * (long)blockDim.x + threadIdx.x) >> 5);
    gn_jtr(a, n, gw, (int)((gridDim.x * (long)blockDim.x) >> 5));
}

// Dense (6 n_host)^2 J^T J: diagonal blocks, upper blocks and their transposes (the layout
// fillJTJKernel writes over runInitIdentityKernel's identity).
__global__ void gn_dense_kernel(GnArgs a, int n_host, float* jtj) {
    const int n = min(min(*a.n_nodes, a.n_max), n_host);
    const long ld = 6L * n_host;
    const int lane = threadIdx.x & 31;
    for (long node = (blockIdx.x * (long)blockDim.x + threadIdx.x) >> 5; node < n;
         node += (gridDim.x * (long)blockDim.x) >> 5) {
        for (int e = lane; e < 36; e += 32) {
            const int i = e / 6, j = e % 6;
            jtj[(node * 6 + i) * ld + node * 6 + j] = a.b.diag[node * 36 + e];
        }
        const int cnt = a.b.nbr_cnt[node];
        for (int u = 0; u < cnt; ++u) {
            const long other = a.b.nbr[node * kMaxNbr + u];
            if (other <= node) continue;
            const float* B = a.b.blocks + (node * kMaxNbr + u) * 36;
            for (int e = lane; e < 36; e += 32) {
                const int i = e / 6, j = e % 6;
                jtj[(node * 6 + i) * ld + other * 6 + j] = B[e];
                jtj[(other * 6 + j) * ld + node * 6 + i] = B[e];
            }
        }
    }
}

__global__ void gn_copy_residuals_kernel(GnArgs a, float* r_depth, float* r_reg) {
    const int n = min(*a.n_nodes, a.n_max);
    const long ncorr = min((long)*a.corr_count, a.c_max);
    const long nreg = (long)n * a.kreg * 3;
    AFX_GRID_STRIDE(t, ncorr + nreg) {
        if (t < ncorr) {
            if (r_depth) r_depth[t] = __ldcg(a.b.rdepth + t);
        } else if (r_reg) {
            r_reg[t - ncorr] = __ldcg(a.b.rreg + (t - ncorr));
        }
    }
}

__global__ void update_transforms_kernel(float* T, const float* x, const int* n_nodes, int n_max) {
    const int n = min(*n_nodes, n_max);
    update_transforms_range(T, x, 0, n, blockIdx.x * (long)blockDim.x + threadIdx.x, (long)gridDim.x * blockDim.x);
}

}  // namespace afx

struct afx_gn {
    long m_max;
    int n_max, k, kreg;
    void* arena;
    afx::GnBuffers b;
    int* cov;
    int* error;
    unsigned* counts;  // copies of the caller's counters at build time: points, correspondences, nodes
    afx::GnArgs last;
    bool built;
};

using namespace afx;

extern "C" {

int afx_gn_create(long n_points_max, int n_nodes_max, int k, int kreg, afx_gn** out) {
    if (!out || n_points_max < 1 || n_nodes_max < 1 || k < 1 || k > 8 || kreg < 1 || kreg > 8)
        return AFX_ERR_INVALID_ARGUMENT;
    afx_gn* g = new (std::nothrow) afx_gn();
    if (!g) return AFX_ERR_NO_MEMORY;
    g->m_max = n_points_max;
    g->n_max = n_nodes_max;
    g->k = k;
    g->kreg = kreg;
    const size_t ws = gn_workspace_size(n_points_max, n_nodes_max, k, kreg);
    const size_t bytes = ws + al((size_t)n_points_max * 4) + 512;
    if (cudaMalloc(&g->arena, bytes) != cudaSuccess) {
        cudaGetLastError();
        delete g;
        return AFX_ERR_NO_MEMORY;
    }
    gn_carve(g->arena, ws, n_points_max, n_nodes_max, k, kreg, &g->b);
    g->cov = reinterpret_cast<int*>(static_cast<char*>(g->arena) + ws);
    g->error = reinterpret_cast<int*>(static_cast<char*>(g->arena) + ws + al((size_t)n_points_max * 4));
    g->counts = reinterpret_cast<unsigned*>(static_cast<char*>(g->arena) + ws + al((size_t)n_points_max * 4) + 256);
    if (cudaMemset(g->error, 0, 4) != cudaSuccess) {
        cudaFree(g->arena);
        delete g;
        return note_cuda_error(cudaGetLastError());
    }
    g->built = false;
    *out = g;
    return AFX_OK;
}

int afx_gn_destroy(afx_gn* g) {
    if (!g) return AFX_ERR_INVALID_ARGUMENT;
    cudaDeviceSynchronize();
    cudaError_t e = cudaFree(g->arena);
    delete g;
    return note_cuda_error(e);
}

int afx_gn_build(afx_gn* g, const float* canonical, const unsigned* n_points, const uint32_t* knn_idx,
                 const float* knn_weights, const int* corr, const unsigned* n_corr, const float* frame_vertices,
                 const float* frame_normals, const float* warped, const float* nodes, const float* transforms,
                 const int* n_nodes, const uint32_t* graph_idx, float lambda_depth, float lambda_reg, void* stream) {
    if (!g || !canonical || !n_points || !knn_idx || !knn_weights || !corr || !n_corr || !frame_vertices ||
        !frame_normals || !warped || !nodes || !transforms || !n_nodes || !graph_idx)
        return AFX_ERR_INVALID_ARGUMENT;
    cudaStream_t st = as_stream(stream);
    // later calls use these copies, not the caller's counters
    AFX_CUDA(cudaMemcpyAsync(g->counts, n_points, 4, cudaMemcpyDeviceToDevice, st));
    AFX_CUDA(cudaMemcpyAsync(g->counts + 1, n_corr, 4, cudaMemcpyDeviceToDevice, st));
    AFX_CUDA(cudaMemcpyAsync(g->counts + 2, n_nodes, 4, cudaMemcpyDeviceToDevice, st));
    n_points = g->counts;
    n_corr = g->counts + 1;
    n_nodes = reinterpret_cast<const int*>(g->counts + 2);
    GnArgs a;
    std::memset(&a, 0, sizeof(a));
    a.mesh = canonical;
    a.mesh_count = n_points;
    a.m_max = g->m_max;
    a.midx = knn_idx;
    a.mw = knn_weights;
    a.k = g->k;
    a.normals = frame_normals;
    a.frame = frame_vertices;
    a.corr = corr;
    a.corr_count = n_corr;
    a.c_max = g->m_max;
    a.corr_of_vertex = g->cov;
    a.nodes = nodes;
    a.n_nodes = n_nodes;
    a.n_max = g->n_max;
    a.gidx = graph_idx;
    a.kreg = g->kreg;
    a.lam_d = lambda_depth;
    a.lam_r = lambda_reg;
    a.b = g->b;
    a.error = g->error;
    AFX_CUDA(cudaMemsetAsync(g->error, 0, 4, st));
    AFX_CUDA(cudaMemsetAsync(g->cov, 0xff, (size_t)g->m_max * 4, st));
    gn_corr_of_vertex_kernel<<<grid_for(g->m_max, 256), 256, 0, st>>>(corr, n_corr, g->m_max, g->cov);
    AFX_LAUNCH_CHECK();
    int rc = gn_frame_setup(a, st);
    if (rc) return rc;
    rc = gn_icp_setup(a, nullptr, nullptr, st);
    if (rc) return rc;
    gn_residual_kernel<<<grid_for(g->m_max + (long)g->n_max * g->kreg, 256), 256, 0, st>>>(a, warped, transforms);
    AFX_LAUNCH_CHECK();
    gn_jtr_kernel<<<grid_for((long)g->n_max * 32, 256), 256, 0, st>>>(a);
    AFX_LAUNCH_CHECK();
    g->last = a;
    g->built = true;
    int err = 0;
    AFX_CUDA(cudaMemcpyAsync(&err, g->error, 4, cudaMemcpyDeviceToHost, st));
    AFX_CUDA(cudaStreamSynchronize(st));
    if (err & ERRF_SINGULAR) return AFX_ERR_SINGULAR;
    if (err & ERRF_CAPACITY) return AFX_ERR_CAPACITY;
    return AFX_OK;
}

int afx_gn_export(afx_gn* g, int n_nodes_host, float* jtj, float* jtr, float* r_depth, float* r_reg, void* stream) {
    if (!g || !g->built || n_nodes_host < 0 || n_nodes_host > g->n_max) return AFX_ERR_INVALID_ARGUMENT;
    cudaStream_t st = as_stream(stream);
    const long dim = 6L * n_nodes_host;
    if (jtj && dim > 0) {
        AFX_CUDA(cudaMemsetAsync(jtj, 0, (size_t)dim * dim * 4, st));
        gn_dense_kernel<<<grid_for((long)n_nodes_host * 32, 256), 256, 0, st>>>(g->last, n_nodes_host, jtj);
        AFX_LAUNCH_CHECK();
    }
    if (jtr && dim > 0) AFX_CUDA(cudaMemcpyAsync(jtr, g->b.jtr, (size_t)dim * 4, cudaMemcpyDeviceToDevice, st));
    if (r_depth || r_reg) {
        gn_copy_residuals_kernel<<<grid_for(g->m_max + (long)g->n_max * g->kreg * 3, 256), 256, 0, st>>>(g->last, r_depth,
                                                                                                          r_reg);
        AFX_LAUNCH_CHECK();
    }
    return AFX_OK;
}

int afx_gn_solve(afx_gn* g, float* x, int iterations, double tol, void* stream) {
    if (!g || !g->built || !x || iterations < 0) return AFX_ERR_INVALID_ARGUMENT;
    cudaStream_t st = as_stream(stream);
    LoopArgs L;
    std::memset(&L, 0, sizeof(L));
    L.g = g->last;
    L.pcg_iters = iterations;
    L.tol = tol;
    int rc = launch_cluster(gn_solve_kernel, L, st);
    if (rc) return rc;
    AFX_CUDA(cudaMemcpyAsync(x, g->b.x, (size_t)g->n_max * 6 * 4, cudaMemcpyDeviceToDevice, st));
    return AFX_OK;
}

int afx_update_transforms(float* transforms, const float* x, const int* n_nodes, int n_nodes_max, void* stream) {
    if (!transforms || !x || !n_nodes || n_nodes_max < 0) return AFX_ERR_INVALID_ARGUMENT;
    if (n_nodes_max == 0) return AFX_OK;
    update_transforms_kernel<<<grid_for((long)n_nodes_max * 16, 256), 256, 0, as_stream(stream)>>>(transforms, x, n_nodes,
                                                                                                  n_nodes_max);
    AFX_LAUNCH_CHECK();
    return AFX_OK;
}

}  // extern "C"
