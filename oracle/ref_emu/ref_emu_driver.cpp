// ref_emu_driver.cpp -- C entry points around the reference's GPU kernels executed on the host
// (oracle pins for the stages that exist only as CUDA in the reference).  Test build only; see
// oracle/ref_emu/build_emu.py.  Pointers are host memory ("device" memory is host memory in the
// emulation).  K and K_reg are the reference's compile-time constants (motionGraphKNN = 6,
// energyMRegKNN = 4).
#include <af/BilateralFilter.cuh>
#include <af/ComputeCorrespondence.cuh>
#include <af/Helper.cuh>
#include <af/MarchingCubes.cuh>
#include <af/MotionOptimization.cuh>
#include <af/TSDFIntegration.cuh>
#include <af/TSDFWarp.h>
#include <af/VertexManipulation.cuh>

#include <algorithm>
#include <cstring>
#include <numeric>
#include <vector>

namespace {
constexpr int K = Constants::motionGraphKNN;
constexpr int KR = Constants::energyMRegKNN;
Mat3f m3(const float* cm) {
    Mat3f M;
    std::memcpy(M.data(), cm, 36);
    return M;
}
Vec3f v3(const float* p) { return Vec3f(p[0], p[1], p[2]); }
Vec3i i3(const int* p) { return Vec3i(p[0], p[1], p[2]); }
}  // namespace

extern "C" {

int emu_knn_k() { return K; }
int emu_kreg() { return KR; }

void emu_filter_depth(float* depth, unsigned n, float thr) { af::runFilterDepthKernel(depth, n, thr); }

void emu_bilateral(float* out, const float* in, int h, int w, int r, double sI, double sS, float thr) {
    af::bilateralFilterTextureOpmShared(out, in, h, w, r, sI, sS, thr);
}

void emu_depth_to_mesh(float* mesh, const float* depth, int w, int h, const float* K9) {
    af::runDepthToMeshKernel(reinterpret_cast<Vec3f*>(mesh), depth, w, h, m3(K9));
}

void emu_normals(float* normals, float* verts, const float* depth, int h, int w, float lo, float hi) {
    af::runDepthVerticesNormalsKernel(reinterpret_cast<Vec3f*>(normals), reinterpret_cast<Vec3f*>(verts), depth, h, w,
                                      {lo, hi});
}

void emu_remove(float* normals, float* verts, float* depth, int h, int w) {
    af::runRemoveDepthWithoutNormalsKernel(reinterpret_cast<Vec3f*>(normals), reinterpret_cast<Vec3f*>(verts), depth, h,
                                           w);
}

void emu_integrate_rigid(float* tsdf, float* w, const float* depth, int W, int H, float delta, const int* dims,
                         const float* vs, const float* size, const float* R, const float* t, const float* K9) {
    af::runIntegrateTSDFFromFrameKernel(tsdf, w, depth, Vec2i(W, H), delta, i3(dims), v3(vs), v3(size), m3(R), v3(t),
                                        m3(K9));
}

void emu_warp_weights(float* wts, const float* radii, const unsigned* idx, const float* dist, long m) {
    af::runComputeWarpWeightsKernel(reinterpret_cast<Vecf<K>*>(wts), radii, reinterpret_cast<const Vecui<K>*>(idx),
                                    reinterpret_cast<const Vecf<K>*>(dist), m);
}

void emu_warp(float* out, const float* pts, const float* T, const unsigned* idx, const float* wts, long m) {
    af::runWarpKernel(reinterpret_cast<Vec3f*>(out), reinterpret_cast<const Vec3f*>(pts),
                      reinterpret_cast<const Mat4f*>(T), reinterpret_cast<const Vecui<K>*>(idx),
                      reinterpret_cast<const Vecf<K>*>(wts), m);
}

long emu_correspondences(int* corr, const float* warped, long m, const float* K9, const float* depth, int rows,
                         int cols, const float* frame, float thr) {
    unsigned n = 0;
    af::runCorrespondencePairsKernel(reinterpret_cast<Vec2i*>(corr), &n, reinterpret_cast<const Vec3f*>(warped), m,
                                     m3(K9), depth, Vec2i(rows, cols), reinterpret_cast<const Vec3f*>(frame), thr);
    return n;
}

// Residuals, Jacobian, J^T J and J^T r exactly as src/VolumeFusion.cu:454-646 drives the kernels,
// with thrust::sort_by_key / reduce_by_key restated by std::stable_sort and sequential sums.
// Outputs: jtj dense (6n)^2 row-major as filled by fillJTJKernel, jtr [6n], r [C + 3*KR*n].
void emu_gn_assemble(float* jtj, float* jtr, float* r_out, const int* corr, unsigned C, const float* canon,
                     const unsigned* midx, const float* mw, const float* normals, const float* frame,
                     const float* warped, const float* nodes, const float* T, unsigned n, const unsigned* gidx,
                     float lam_d, float lam_r) {
    const size_t jDepthHeight = C, jMRegHeight = (size_t)n * KR * 3, jHeight = jDepthHeight + jMRegHeight;
    std::vector<Vec6f> J(jHeight * n, Vec6f::Zero());
    std::vector<float> r(jHeight, 0.f);
    const Vec2i* cc = reinterpret_cast<const Vec2i*>(corr);
    af::runFill_J_DepthKernel(J.data(), lam_d, jDepthHeight, n, cc, C, reinterpret_cast<const Vec3f*>(canon),
                              reinterpret_cast<const Vecui<K>*>(midx), reinterpret_cast<const Vecf<K>*>(mw),
                              reinterpret_cast<const Vec3f*>(frame), reinterpret_cast<const Vec3f*>(normals));
    af::runFill_r_DepthKernel(r.data(), lam_d, cc, C, reinterpret_cast<const Vec3f*>(warped),
                              reinterpret_cast<const Vec3f*>(frame), reinterpret_cast<const Vec3f*>(normals));
    af::runFill_r_MRegKernel(r.data() + jDepthHeight, lam_r, reinterpret_cast<const Vec3f*>(nodes),
                             reinterpret_cast<const Mat4f*>(T), n, reinterpret_cast<const Vecui<KR>*>(gidx));
    af::runFill_J_MRegKernel(J.data() + jDepthHeight * n, lam_r, jMRegHeight, n, reinterpret_cast<const Vec3f*>(nodes),
                             reinterpret_cast<const Mat4f*>(T), n, reinterpret_cast<const Vecui<KR>*>(gidx));
    const size_t maxPairs = jDepthHeight * (af::combinations(K, 2) + K) + jMRegHeight * 3;
    const size_t maxElems = jDepthHeight * K + jMRegHeight * 2;
    std::vector<Vec2i> pairs(maxPairs), elems(maxElems);
    std::vector<unsigned> rows(maxPairs);
    unsigned npairs = 0, nelems = 0;
    af::runComputeJTJAndJTrContribJDepthKernel(pairs.data(), rows.data(), &npairs, elems.data(), &nelems, cc, C,
                                               reinterpret_cast<const Vecui<K>*>(midx),
                                               reinterpret_cast<const Vecf<K>*>(mw));
    af::runComputeJTJAndJTrContribJMRegKernel(pairs.data(), rows.data(), (unsigned)jDepthHeight, &npairs, elems.data(),
                                              &nelems, n, reinterpret_cast<const Vecui<KR>*>(gidx));
    std::vector<unsigned> order(npairs);
    std::iota(order.begin(), order.end(), 0u);
    std::stable_sort(order.begin(), order.end(), [&](unsigned a, unsigned b) {
        return pairs[a][0] < pairs[b][0] || (pairs[a][0] == pairs[b][0] && pairs[a][1] < pairs[b][1]);
    });
    std::vector<Vec2i> sp(npairs);
    std::vector<unsigned> sr(npairs);
    for (unsigned i = 0; i < npairs; ++i) {
        sp[i] = pairs[order[i]];
        sr[i] = rows[order[i]];
    }
    std::vector<Mat6f> prod(npairs);
    af::runMultiplyJTJContribPairsKernel(prod.data(), sp.data(), sr.data(), npairs, J.data(), n);
    std::vector<Vec2i> coords;
    std::vector<Mat6f> sums;
    for (unsigned i = 0; i < npairs; ++i) {
        if (!coords.empty() && coords.back() == sp[i]) sums.back() += prod[i];
        else {
            coords.push_back(sp[i]);
            sums.push_back(prod[i]);
        }
    }
    std::vector<unsigned> eorder(nelems);
    std::iota(eorder.begin(), eorder.end(), 0u);
    std::stable_sort(eorder.begin(), eorder.end(), [&](unsigned a, unsigned b) { return elems[a][1] < elems[b][1]; });
    std::vector<Vec2i> se(nelems);
    for (unsigned i = 0; i < nelems; ++i) se[i] = elems[eorder[i]];
    std::vector<Vec6f> eprod(nelems);
    af::runMultiplyJTrContribElemsKernel(eprod.data(), se.data(), nelems, J.data(), r.data(), n);
    std::vector<Vec2i> ecoords;
    std::vector<Vec6f> esums;
    for (unsigned i = 0; i < nelems; ++i) {
        if (!ecoords.empty() && ecoords.back()[1] == se[i][1]) esums.back() += eprod[i];
        else {
            ecoords.push_back(se[i]);
            esums.push_back(eprod[i]);
        }
    }
    const unsigned W = n * 6;
    std::memset(jtj, 0, sizeof(float) * (size_t)W * W);
    runInitIdentityKernel(jtj, W);
    af::runFillJTJKernel(jtj, coords.data(), sums.data(), (unsigned)coords.size(), W);
    std::memset(jtr, 0, sizeof(float) * W);
    af::runFillJTrKernel(reinterpret_cast<Vec6f*>(jtr), ecoords.data(), esums.data(), (unsigned)ecoords.size());
    std::memcpy(r_out, r.data(), sizeof(float) * jHeight);
}

void emu_update_transforms(float* T, const float* x, unsigned n) {
    af::runUpdateTransformsKernel(reinterpret_cast<Mat4f*>(T), reinterpret_cast<const Vec6f*>(x), n);
}

void emu_tsdf_knn(unsigned* kidx, float* kdist, int* kcount, const float* nodes, const float* radii, unsigned n,
                  const float* vs, const float* size, const int* dims, const int* per) {
    af::runTsdfKNNGraph(reinterpret_cast<Vecui<K>*>(kidx), reinterpret_cast<Vecf<K>*>(kdist), kcount,
                        reinterpret_cast<const Vec3f*>(nodes), radii, n, v3(vs), v3(size), i3(dims), i3(per));
}

void emu_tsdf_weights(float* kw, const float* radii, const unsigned* kidx, const float* kdist, const int* kcount,
                      long S) {
    af::runComputeTsdfWarpWeightsKernel(reinterpret_cast<Vecf<K>*>(kw), radii, reinterpret_cast<const Vecui<K>*>(kidx),
                                        reinterpret_cast<const Vecf<K>*>(kdist), kcount, S);
}

void emu_tsdf_vertices(float* v, const float* vs, const float* size, const int* dims) {
    af::runGenerateTsdfVerticesKernel(reinterpret_cast<Vec3f*>(v), v3(vs), v3(size), i3(dims));
}

void emu_translate(float* pts, unsigned n, const float* t) { af::runTranslateKernel(reinterpret_cast<Vec3f*>(pts), n, v3(t)); }

void emu_warp_tsdf(float* v, const float* T, const unsigned* kidx, const float* kw, const int* kcount, const float* vs,
                   const float* size, const int* dims) {
    af::runWarpTsdfKernel(reinterpret_cast<Vec3f*>(v), reinterpret_cast<const Mat4f*>(T),
                          reinterpret_cast<const Vecui<K>*>(kidx), reinterpret_cast<const Vecf<K>*>(kw), kcount, v3(vs),
                          v3(size), i3(dims));
}

void emu_count_collisions(int* counts, const float* v, const int* kcount, const float* vs, const float* size,
                          const int* dims, const float* R, const float* t) {
    af::runCountCollisionsPerVoxelKernel(counts, reinterpret_cast<const Vec3f*>(v), kcount, v3(vs), v3(size), i3(dims),
                                         m3(R), v3(t));
}

void emu_integrate_warped(float* tsdf, float* w, const float* v, const int* coll, const int* kcount, const float* depth,
                          int W, int H, float delta, const float* vs, const float* size, const int* dims, const float* R,
                          const float* t, const float* K9) {
    af::runIntegrateWarpedTSDFFromFrameKernel(tsdf, w, reinterpret_cast<const Vec3f*>(v), coll, kcount, depth,
                                              Vec2i(W, H), delta, v3(vs), v3(size), i3(dims), m3(R), v3(t), m3(K9));
}

unsigned emu_mc_points(float* out, const float* tsdf, const float* w, const int* dims, const float* vs,
                       const float* size) {
    unsigned n = 0;
    af::runMarchingCubesMeshKernel(reinterpret_cast<Vec3f*>(out), &n, tsdf, w, i3(dims), v3(vs), v3(size), 0.f);
    return n;
}

unsigned emu_mc_full(float* verts, int* faces, unsigned* nfaces, const float* tsdf, const float* w, const int* dims,
                     const float* vs, const float* size) {
    unsigned nv = 0, nf = 0;
    af::runMarchingCubesFullKernel(reinterpret_cast<Vec3f*>(verts), &nv, reinterpret_cast<Vec3i*>(faces), &nf, tsdf, w,
                                   i3(dims), v3(vs), v3(size), 0.f);
    *nfaces = nf;
    return nv;
}

}  // extern "C"
