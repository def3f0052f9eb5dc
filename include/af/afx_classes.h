/*
 * af/afx_classes.h -- the reference's af:: classes over the C ABI (header-only C++17): include
 * this one header for the whole C++ surface.
 *
 *   containers (DeviceBuffer, DeviceKnn, DeviceMotionGraph, Settings, ...)   af/afx_containers.h
 *   DeviceTsdf, MotionGraph, buildGraph, getKnnData, ...                      af/afx_motion_graph.h
 *   WarpField                             include/af/WarpField.cuh:20-111, src/WarpField.cu:30-50
 *   TSDFVolume                            include/af/TSDFVolume.h:10-113, src/TSDFVolume.cpp
 *   GaussNewtonSystem                     the Gauss-Newton step of src/VolumeFusion.cu:454-691
 *   the run* operators                    af/afx_shims.h
 *   depth ingest (loadDepthFrame, DepthUndistorter, create_xy_lookup_table, ...)  af/afx_ingest.h
 *   the dense Gauss-Newton operators and LU solve (runFill_J_*, ..., linearSolverLUStable)  af/afx_gn_dense.h
 *
 * Every computation runs on the GPU through the afx_* entry points; calls block until the GPU
 * work has finished and throw std::runtime_error on failure.  The reference's MotionGraph,
 * TSDFVolume and Constants live in the global namespace: define AFX_GLOBAL_CLASS_NAMES before
 * including this header to bring them there as well.
 */
#ifndef AF_AFX_CLASSES_H
#define AF_AFX_CLASSES_H

#include <string>
#include <vector>

#include "afx_gn_dense.h"
#include "afx_ingest.h"
#include "afx_motion_graph.h"

namespace af {

// ---- include/af/WarpField.cuh, src/WarpField.cu ----
// The motion graph lives on the device; the graph build and every KNN query run there
// (the reference builds on the host and copies the new nodes over).
class WarpField {
public:
    WarpField(std::size_t bufferSize, const Settings& settings)
        : _motionGraph_d(bufferSize), _motionGraphknnIdxs_d((unsigned int)bufferSize),
          _graphKnnDists_d(bufferSize), _pointCloud_d(1), _settings(settings) {}

    // Snapshots the point cloud and, with settings.updateGraph, appends the nodes it needs
    // (af::buildGraph with Constants::motionGraphKNN neighbours and settings.motionGraphRadius).
    template <template <class> class Container>
    void spreadMotionGraph(const Container<Vec3f>& pointCloud_d) {
        const std::size_t m = pointCloud_d.size();
        _pointCloud_d.resizeBuffer(m ? m : 1);
        if (m)
            detail::cuda_check(cudaMemcpy(_pointCloud_d.bufferPtr(), pointCloud_d.bufferPtr(), m * sizeof(Vec3f),
                                          cudaMemcpyDeviceToDevice),
                               "WarpField::spreadMotionGraph");
        _pointCloud_d.setSize((unsigned int)m);
        if (!_settings.updateGraph || m == 0) return;
        detail::Workspace ws(afx_build_graph_workspace_size((long)m, (int)_motionGraph_d.bufferSize()));
        detail::afx_check(afx_build_graph(detail::ff<3>(_motionGraph_d.pointsPtr()), _motionGraph_d.radiusesPtr(),
                                          detail::ff<16>(_motionGraph_d.transformsPtr()), _motionGraph_d.countPtr(),
                                          (int)_motionGraph_d.bufferSize(), detail::ff<3>(_pointCloud_d.bufferPtr()),
                                          _pointCloud_d.size_dPtr(), (long)m, (int)Constants::motionGraphKNN,
                                          _settings.motionGraphRadius, ws.p, ws.bytes, nullptr),
                          "WarpField::spreadMotionGraph");
        _motionGraph_d.syncCount();
    }

    // Each node's Constants::energyMRegKNN nearest other nodes (the regularisation neighbours).
    void computeGraphKnns() {
        const std::size_t n = _motionGraph_d.count();
        if (n > _motionGraphknnIdxs_d.bufferSize()) throw std::runtime_error("WarpField::computeGraphKnns: buffer");
        if (n)
            detail::afx_check(afx_knn(detail::u32(_motionGraphknnIdxs_d.bufferPtr()),
                                      reinterpret_cast<float*>(_graphKnnDists_d.get()),
                                      detail::ff<3>(_motionGraph_d.pointsPtr()), _motionGraph_d.countPtr(),
                                      (int)_motionGraph_d.bufferSize(), detail::ff<3>(_motionGraph_d.pointsPtr()),
                                      nullptr, (long)n, (int)Constants::energyMRegKNN, 1, nullptr),
                              "WarpField::computeGraphKnns");
        _motionGraphknnIdxs_d.setSize((unsigned int)n);
    }

    // The snapshot's Constants::motionGraphKNN nearest nodes.
    void computePointCloudKnns(DeviceKnn<(int)Constants::motionGraphKNN>& knnResult_d) {
        computeKnns<(int)Constants::motionGraphKNN>(knnResult_d, _pointCloud_d);
    }

    // ... and their skinning weights (runComputeWarpWeightsKernel).
    void computePointCloudWeightedKnns(DeviceKnnWeighted<(int)Constants::motionGraphKNN>& knnResult_d) {
        computePointCloudKnns(knnResult_d);
        const int k = (int)Constants::motionGraphKNN;
        if (knnResult_d.size())
            detail::afx_check(afx_warp_weights(reinterpret_cast<float*>(knnResult_d.weightsPtr()),
                                               _motionGraph_d.radiusesPtr(), detail::u32(knnResult_d.idxsPtr()),
                                               reinterpret_cast<const float*>(knnResult_d.distsPtr()), nullptr,
                                               (long)knnResult_d.size(), k, _motionGraph_d.countPtr(), nullptr),
                              "WarpField::computePointCloudWeightedKnns");
    }

    template <int K, template <class> class Container>
    void computeKnns(DeviceKnn<K>& knnResult_d, const Container<Vec3f>& pointCloud_d) {
        const std::size_t m = pointCloud_d.size();
        if (m > knnResult_d.bufferSize()) throw std::runtime_error("WarpField::computeKnns: result buffer too small");
        if (m)
            detail::afx_check(afx_knn(detail::u32(knnResult_d.idxsPtr()), reinterpret_cast<float*>(knnResult_d.distsPtr()),
                                      detail::ff<3>(_motionGraph_d.pointsPtr()), _motionGraph_d.countPtr(),
                                      (int)_motionGraph_d.bufferSize(), detail::ff<3>(pointCloud_d.bufferPtr()),
                                      nullptr, (long)m, K, 0, nullptr),
                              "WarpField::computeKnns");
        knnResult_d.setSize(m);
    }

    template <int K>
    void warp(DeviceBuffer<Vec3f>& warpedPoints, const DeviceBuffer<Vec3f>& points,
              const DeviceKnnWeighted<K>& pointsKnn) {
        warpedPoints.setSize(points.size());
        if (points.size())
            af::runWarpKernel(warpedPoints.bufferPtr(), points.bufferPtr(), _motionGraph_d.transformsPtr(),
                              pointsKnn.idxsPtr(), pointsKnn.weightsPtr(), points.size());
    }

    DeviceMotionGraph& motionGraph_d() { return _motionGraph_d; }
    // The regularisation neighbours computeGraphKnns found (private in the reference, where
    // its Gauss-Newton code reads them directly).
    const DeviceBuffer<Vecui<(int)Constants::energyMRegKNN>>& graphKnnIdxs_d() const { return _motionGraphknnIdxs_d; }

    // The graph on the host.
    MotionGraph motionGraph() const {
        MotionGraph g;
        const std::size_t n = _motionGraph_d.count();
        std::vector<Vec3f> p(n);
        std::vector<float> r(n);
        std::vector<Mat4f> T(n);
        copyToHost(p.data(), _motionGraph_d.pointsPtr(), n);
        copyToHost(r.data(), _motionGraph_d.radiusesPtr(), n);
        copyToHost(T.data(), _motionGraph_d.transformsPtr(), n);
        for (std::size_t i = 0; i < n; ++i) g.push_back(p[i], r[i], T[i]);
        return g;
    }

private:
    DeviceMotionGraph _motionGraph_d;
    DeviceBuffer<Vecui<(int)Constants::energyMRegKNN>> _motionGraphknnIdxs_d;
    DeviceArray<Vecf<(int)Constants::energyMRegKNN>> _graphKnnDists_d;
    DeviceBufferCounted<Vec3f> _pointCloud_d;
    const Settings& _settings;
};

// ---- include/af/TSDFVolume.h, src/TSDFVolume.cpp ----
// The reference's host volume.  Values, weights and colours stay in host vectors, as there;
// integrate() runs the GPU integration (runIntegrateTSDFFromFrameKernel) on them.  That rule
// equals the CPU loop of src/TSDFVolume.cpp:55-170 on one frame to 4 ULP (the reference's own
// test bound) but saturates weights at 15 where the CPU loop lets them grow; colour is not
// integrated (the fusion path has none) and a non-empty colour image is refused.
class TSDFVolume {
public:
    TSDFVolume(const Vec3i& dimensions, const Vec3f& size, const Mat3f& K)
        : m_dim(dimensions), m_gridSize(count_of(dimensions)), m_size(size), m_voxelSize(quotient(size, dimensions)),
          m_K(K), m_delta(0.05f), m_deltaInv(1.0f / 0.05f), m_centroid(Vec3f(0.f, 0.f, 0.f)) {
        init();
    }
    ~TSDFVolume() { release(); }

    bool init() {
        m_tsdf.assign(m_gridSize, -1.0f);
        m_weights.assign(m_gridSize, 0.0f);
        m_colorR.assign(m_gridSize, (unsigned char)127);
        m_colorG.assign(m_gridSize, (unsigned char)127);
        m_colorB.assign(m_gridSize, (unsigned char)127);
        m_weightsColor.assign(m_gridSize, 0.0f);
        return true;
    }
    void release() {}

    void bbox(Vec3d& min, Vec3d& max) const {
        min = Vec3d(-m_size[0] * 0.5, -m_size[1] * 0.5, -m_size[2] * 0.5);
        max = Vec3d(m_size[0] * 0.5, m_size[1] * 0.5, m_size[2] * 0.5);
    }
    void setSize(const Vec3f& size) {
        m_size = size;
        m_voxelSize = quotient(m_size, m_dim);
    }
    Vec3f size() const { return m_size; }
    Vec3f voxelSize() const { return m_voxelSize; }
    std::size_t gridSize() const { return m_gridSize; }
    Vec3i dimensions() const { return m_dim; }

    // voxel * voxelSize - size / 2 (src/TSDFVolume.cpp:400-410)
    Vec3f voxelToWorld(const Vec3i& voxel) const {
        Vec3f p = m_size;
        for (int i = 0; i < 3; ++i) p[i] = (float)voxel[i] * m_voxelSize[i] - m_size[i] * 0.5f;
        return p;
    }
    Vec3f voxelToWorld(int i, int j, int k) const { return voxelToWorld(Vec3i(i, j, k)); }
    Vec3f voxelToWorld(const Vec3f& voxel) const {
        Vec3f p = m_size;
        for (int i = 0; i < 3; ++i) p[i] = voxel[i] * m_voxelSize[i] - m_size[i] * 0.5f;
        return p;
    }
    Vec3f worldToVoxelF(const Vec3f& pt) const {
        Vec3f v = pt;
        for (int i = 0; i < 3; ++i) v[i] = (pt[i] + 0.5f * m_size[i]) * (float)(1.0 / m_voxelSize[i]);
        return v;
    }
    Vec3i worldToVoxel(const Vec3f& pt) const {
        const Vec3f v = worldToVoxelF(pt);
        return Vec3i((int)v[0], (int)v[1], (int)v[2]);
    }
    Vec3f cameraToObject(const Vec3f& pt) const {
        Vec3f w = pt;
        for (int i = 0; i < 3; ++i) w[i] = pt[i] - m_centroid[i];
        return w;
    }
    Vec3f voxelToCamera(const Vec3i& voxel) const {
        Vec3f w = voxelToWorld(voxel);
        for (int i = 0; i < 3; ++i) w[i] = w[i] + m_centroid[i];
        return w;
    }
    Vec3i cameraToVoxel(const Vec3f& pt) const { return worldToVoxel(cameraToObject(pt)); }

    // Depth (metres, rows x cols) seen from `pose` (world to camera: R p + t).
    void integrate(const Mat4f& pose, const float* depth, int rows, int cols) {
        float R[9], t[3], K[9], vs[3], size[3];
        int dims[3];
        for (int c = 0; c < 3; ++c)
            for (int r = 0; r < 3; ++r) R[c * 3 + r] = pose.data()[c * 4 + r];
        for (int r = 0; r < 3; ++r) t[r] = pose.data()[12 + r];
        detail::to_m3(m_K, K);
        detail::to_f3(m_voxelSize, vs);
        detail::to_f3(m_size, size);
        detail::to_i3(m_dim, dims);
        m_centroid = Vec3f(t[0], t[1], t[2]);
        DeviceArray<float> T(m_gridSize), W(m_gridSize), D((std::size_t)rows * (std::size_t)cols);
        copyToDevice(T.get(), m_tsdf.data(), m_gridSize);
        copyToDevice(W.get(), m_weights.data(), m_gridSize);
        copyToDevice(D.get(), depth, D.size());
        detail::afx_check(afx_integrate_tsdf(T.get(), W.get(), D.get(), cols, rows, m_delta, dims, vs, size, R, t, K,
                                             nullptr),
                          "TSDFVolume::integrate");
        copyToHost(m_tsdf.data(), T.get(), m_gridSize);
        copyToHost(m_weights.data(), W.get(), m_gridSize);
    }
    // The reference's signature with OpenCV-style images (.empty(), .data, .rows, .cols; depth CV_32F).
    template <class Image>
    void integrate(const Mat4f& pose, const Image& color, const Image& depth, const Image& normals = Image()) {
        (void)normals;
        if (!color.empty()) throw std::invalid_argument("TSDFVolume::integrate: colour integration is not supported");
        integrate(pose, reinterpret_cast<const float*>(depth.data), depth.rows, depth.cols);
    }

    // The reference's file format (src/TSDFVolume.cpp:315-361).
    bool load(const std::string& filename) {
        int dims[3];
        float size[3], vs[3], delta = 0.f;
        if (afx_tsdf_load_header(filename.c_str(), dims, size, vs, &delta) != AFX_OK)
            throw std::runtime_error("TSDFVolume::load(" + filename + "): Couldn't open the file.");
        m_dim = Vec3i(dims[0], dims[1], dims[2]);
        m_gridSize = count_of(m_dim);
        m_size = Vec3f(size[0], size[1], size[2]);
        m_voxelSize = Vec3f(vs[0], vs[1], vs[2]);
        setDelta(delta);
        const bool ok = init();
        if (afx_tsdf_load(filename.c_str(), m_tsdf.data(), m_weights.data(), (long)m_gridSize) != AFX_OK)
            throw std::runtime_error("TSDFVolume::load(" + filename + "): short file.");
        return ok;
    }
    bool save(const std::string& filename) {
        int dims[3];
        float size[3], vs[3];
        detail::to_i3(m_dim, dims);
        detail::to_f3(m_size, size);
        detail::to_f3(m_voxelSize, vs);
        if (afx_tsdf_save(filename.c_str(), dims, size, vs, m_delta, m_tsdf.data(), m_weights.data()) != AFX_OK)
            throw std::runtime_error("TSDFVolume::save(" + filename + "): Couldn't open the file.");
        return true;
    }

    // sdf clamped to [-delta, delta], over delta (src/TSDFVolume.cpp:45-53)
    float truncate(float sdf) const {
        float v = sdf;
        if (v > m_delta)
            v = m_delta;
        else if (v < -m_delta)
            v = -m_delta;
        return v * m_deltaInv;
    }

    void setDelta(float delta) {
        m_delta = delta;
        m_deltaInv = 1.0f / m_delta;
    }
    float delta() const { return m_delta; }

    std::vector<float>& tsdf() { return m_tsdf; }
    std::vector<float>& tsdfWeights() { return m_weights; }
    std::vector<unsigned char>& colorR() { return m_colorR; }
    std::vector<unsigned char>& colorG() { return m_colorG; }
    std::vector<unsigned char>& colorB() { return m_colorB; }
    const std::vector<float>& tsdf() const { return m_tsdf; }
    const std::vector<float>& tsdfWeights() const { return m_weights; }
    const std::vector<unsigned char>& colorR() const { return m_colorR; }
    const std::vector<unsigned char>& colorG() const { return m_colorG; }
    const std::vector<unsigned char>& colorB() const { return m_colorB; }
    float* ptrTsdf() { return m_tsdf.data(); }
    float* ptrTsdfWeights() { return m_weights.data(); }
    unsigned char* ptrColorR() { return m_colorR.data(); }
    unsigned char* ptrColorG() { return m_colorG.data(); }
    unsigned char* ptrColorB() { return m_colorB.data(); }
    const float* ptrTsdf() const { return m_tsdf.data(); }
    const float* ptrTsdfWeights() const { return m_weights.data(); }
    const unsigned char* ptrColorR() const { return m_colorR.data(); }
    const unsigned char* ptrColorG() const { return m_colorG.data(); }
    const unsigned char* ptrColorB() const { return m_colorB.data(); }
    Vec3f centroid() const { return m_centroid; }

protected:
    static std::size_t count_of(const Vec3i& d) { return (std::size_t)d[0] * (std::size_t)d[1] * (std::size_t)d[2]; }
    static Vec3f quotient(const Vec3f& s, const Vec3i& d) {
        Vec3f v = s;
        for (int i = 0; i < 3; ++i) v[i] = s[i] / (float)d[i];
        return v;
    }

    Vec3i m_dim;
    std::size_t m_gridSize;
    Vec3f m_size;
    Vec3f m_voxelSize;
    std::vector<float> m_tsdf;
    std::vector<float> m_weights;
    std::vector<unsigned char> m_colorR;
    std::vector<unsigned char> m_colorG;
    std::vector<unsigned char> m_colorB;
    std::vector<float> m_weightsColor;
    Mat3f m_K;
    float m_delta;
    float m_deltaInv;
    Vec3f m_centroid;
};

// ---- the Gauss-Newton step (src/VolumeFusion.cu:454-691, src/MotionOptimization.cu, src/LinearSolver.cu) ----
// The reference fills a dense Jacobian (runFill_J_DepthKernel, runFill_J_MRegKernel), lists the
// contributing pairs (runComputeJTJAndJTrContrib*), multiplies and scatters them
// (runMultiply*, runFillJTJKernel, runFillJTrKernel) and solves with cuSOLVER LU
// (linearSolverLUStable).  This object replaces that sequence as a unit: build() assembles the
// residuals, J^T J and J^T r block-sparse on the device, exportDense() gives them in the
// reference's dense layout, and solve() runs the block-Jacobi preconditioned conjugate
// gradients that take the place of the LU solve.  Pointers are device pointers.
class GaussNewtonSystem {
public:
    GaussNewtonSystem(long nPointsMax, int nNodesMax, int k = (int)Constants::motionGraphKNN,
                      int kreg = (int)Constants::energyMRegKNN)
        : _nNodesMax(nNodesMax) {
        const int st = afx_gn_create(nPointsMax, nNodesMax, k, kreg, &_g);
        if (st != AFX_OK) throw std::runtime_error(std::string("afx_gn_create: ") + afx_status_string(st));
    }
    ~GaussNewtonSystem() { afx_gn_destroy(_g); }
    GaussNewtonSystem(const GaussNewtonSystem&) = delete;
    GaussNewtonSystem& operator=(const GaussNewtonSystem&) = delete;

    // Canonical points, their skinning neighbours and weights, the (point, pixel) correspondences
    // with the frame's vertices and normals, the warped points, the nodes with their transforms
    // and regularisation neighbours; counts are device values.
    template <class P3, class PI, class PW, class P2, class Q3, class R3, class W3, class N3, class P16, class GI>
    void build(const P3* canonical, const unsigned* nPoints, const PI* knnIdx, const PW* knnWeights, const P2* corr,
               const unsigned* nCorr, const Q3* frameVertices, const R3* frameNormals, const W3* warped,
               const N3* nodes, const P16* transforms, const int* nNodes, const GI* graphIdx, float lambdaDepth,
               float lambdaReg) {
        detail::afx_check(afx_gn_build(_g, detail::ff<3>(canonical), nPoints, detail::u32(knnIdx),
                                       reinterpret_cast<const float*>(knnWeights), detail::flat<int, 2>(corr), nCorr,
                                       detail::ff<3>(frameVertices), detail::ff<3>(frameNormals),
                                       detail::ff<3>(warped), detail::ff<3>(nodes), detail::ff<16>(transforms),
                                       nNodes, detail::u32(graphIdx), lambdaDepth, lambdaReg, nullptr),
                          "GaussNewtonSystem::build");
    }

    // jtj: (6 n)^2 row-major, jtr: 6 n, rDepth: one per correspondence, rReg: 3 per (node, slot);
    // any may be null.
    void exportDense(int nNodesHost, float* jtj, float* jtr, float* rDepth, float* rReg) {
        detail::afx_check(afx_gn_export(_g, nNodesHost, jtj, jtr, rDepth, rReg, nullptr),
                          "GaussNewtonSystem::exportDense");
    }

    // x (6 per node, nNodesMax nodes) = (J^T J)^-1 J^T r, for runUpdateTransformsKernel.
    template <class P6>
    void solve(P6* x, int iterations = 10, double tol = 0.0) {
        detail::afx_check(afx_gn_solve(_g, detail::ff<6>(x), iterations, tol, nullptr), "GaussNewtonSystem::solve");
    }

    int nodesMax() const { return _nNodesMax; }
    afx_gn* handle() { return _g; }

private:
    afx_gn* _g = nullptr;
    int _nNodesMax;
};

}  // namespace af

#ifdef AFX_GLOBAL_CLASS_NAMES
using af::Constants;
using af::MotionGraph;
using af::TSDFVolume;
using af::VertexCloud;
#endif

#endif
