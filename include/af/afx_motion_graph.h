/*
 * af/afx_motion_graph.h -- DeviceTsdf, MotionGraph and the graph builder of the af:: surface
 * (header-only C++17 over the C ABI).
 *
 *   DeviceTsdf                            include/af/DeviceTsdf.cuh:13-84
 *   VertexCloud, MotionGraph              include/af/VertexCloud.h:9-40, include/af/MotionGraph.h:7-48
 *   buildGraph, getKnnData, filterDisconnected, removeDuplicates, translate
 *                                         include/af/GraphBuilder.h:14-62
 *
 * Every computation runs on the GPU through the afx_* entry points, including the ones the
 * reference runs on the host (MotionGraph::knnSearch / warp, buildGraph, getKnnData,
 * filterDisconnected): host containers are copied to the device for the call and the results
 * copied back.  Calls block until the GPU work has finished and throw std::runtime_error on
 * failure.  af/afx_classes.h includes this header.
 */
#ifndef AF_AFX_MOTION_GRAPH_H
#define AF_AFX_MOTION_GRAPH_H

#include <cmath>
#include <cstring>
#include <limits>
#include <string>
#include <vector>

#include "afx_containers.h"

namespace af {

// ---- include/af/DeviceTsdf.cuh ----
template <class Precision = float>
class DeviceTsdf {
    static_assert(std::is_same<Precision, float>::value,
                  "the integration kernels update binary32 volumes (binary16 storage is a session option)");

public:
    DeviceTsdf() = default;
    DeviceTsdf(const Vec3f& volSize, const Vec3i& volDim, const Vec3f& center, const Mat3f& rotation,
               float delta = 0.01f)
        : _tsdf_d(count_of(volDim)), _weights_d(count_of(volDim)), _delta(delta), _volDim(volDim), _volSize(volSize),
          _center(center), _rotation(rotation) {
        initDefault();
    }
    DeviceTsdf(const Vec3f& volSize, const Vec3i& volDim, float delta = 0.01f)
        : DeviceTsdf(volSize, volDim, Vec3f::Zero(), Mat3f::Identity(), delta) {}

    // values -1, weights 0
    void initDefault() {
        detail::afx_check(afx_fill_f32(tsdfPtr(), (long)voxelCount(), -1.f, nullptr), "DeviceTsdf::initDefault");
        detail::afx_check(afx_fill_f32(weightsPtr(), (long)voxelCount(), 0.f, nullptr), "DeviceTsdf::initDefault");
    }

    // One depth frame through the volume's pose (runIntegrateTSDFFromFrameKernel).
    void integrate(const DeviceDepthImage& depthFrame_d) {
        af::runIntegrateTSDFFromFrameKernel(tsdfPtr(), weightsPtr(), depthFrame_d.dataPtr(),
                                            Vec2i((int)depthFrame_d.width(), (int)depthFrame_d.height()), _delta,
                                            _volDim, voxelSize(), _volSize, rotation(), center(),
                                            depthFrame_d.depthIntrinsics());
    }

    // Marching-cubes points of the zero level, sorted and de-duplicated.  The buffer's previous
    // contents are replaced (the reference's callers pass an empty buffer; its kernel appends).
    void extractPointCloud(DeviceBufferCounted<Vec3f>& pointCloud) {
        int dims[3];
        float vs[3], size[3];
        detail::to_i3(_volDim, dims);
        detail::to_f3(voxelSize(), vs);
        detail::to_f3(_volSize, size);
        const long cap = (long)pointCloud.bufferSize();
        detail::Workspace ws(afx_sort_unique_points_workspace_size(cap));
        detail::afx_check(afx_extract_point_cloud(detail::ff<3>(pointCloud.bufferPtr()), pointCloud.size_dPtr(), cap,
                                                  tsdfPtr(), weightsPtr(), dims, vs, size, 0.f, ws.p, ws.bytes,
                                                  nullptr),
                          "DeviceTsdf::extractPointCloud");
        pointCloud.syncHostSize();
    }

    void setDelta(float delta) { _delta = delta; }
    float delta() const { return _delta; }

    // Keeps the first voxels, as thrust's resize does; new voxels are -1 / 0.
    void setVolDim(const Vec3i& volDim) {
        _volDim = volDim;
        _tsdf_d.resize(count_of(volDim), -1.f);
        _weights_d.resize(count_of(volDim), 0.f);
    }
    Vec3i volDim() const { return _volDim; }
    void setVolSize(const Vec3f& volSize) { _volSize = volSize; }
    Vec3f volSize() const { return _volSize; }
    void setCenter(const Vec3f& center) { _center = center; }
    Vec3f center() const { return _center; }
    void setRotation(const Mat3f& rotation) { _rotation = rotation; }
    Mat3f rotation() const { return _rotation; }

    Vec3f voxelSize() const {
        Vec3f v = _volSize;
        for (int i = 0; i < 3; ++i) v[i] = _volSize[i] / (float)_volDim[i];
        return v;
    }
    std::size_t voxelCount() const { return count_of(_volDim); }

    Precision* tsdfPtr() { return _tsdf_d.get(); }
    const Precision* tsdfPtr() const { return _tsdf_d.get(); }
    Precision* weightsPtr() { return _weights_d.get(); }
    const Precision* weightsPtr() const { return _weights_d.get(); }
    const DeviceArray<Precision>& tsdf_d() const { return _tsdf_d; }
    const DeviceArray<Precision>& weights_d() const { return _weights_d; }

private:
    static std::size_t count_of(const Vec3i& d) { return (std::size_t)d[0] * (std::size_t)d[1] * (std::size_t)d[2]; }

    DeviceArray<Precision> _tsdf_d;
    DeviceArray<Precision> _weights_d;
    float _delta = 0.01f;
    Vec3i _volDim = Vec3i(0, 0, 0);
    Vec3f _volSize = Vec3f(0.f, 0.f, 0.f);
    Vec3f _center = Vec3f(0.f, 0.f, 0.f);
    Mat3f _rotation = Mat3f::Identity();
};

// ---- include/af/VertexCloud.h ----
template <class Vertex>
struct VertexCloud {
    std::vector<Vertex> vec_;

    std::size_t kdtree_get_point_count() const { return vec_.size(); }
    typename Vertex::value_type kdtree_get_pt(const std::size_t idx, const std::size_t dim) const {
        return vec_[idx][(int)dim];
    }
    template <class BBOX>
    bool kdtree_get_bbox(BBOX&) const {
        return false;
    }
    void clear() noexcept { vec_.clear(); }
    bool empty() const noexcept { return vec_.empty(); }
    std::size_t size() const noexcept { return vec_.size(); }
    void push_back(const Vertex& v) { vec_.push_back(v); }
};

// ---- include/af/MotionGraph.h, src/MotionGraph.cpp ----
class MotionGraph {
public:
    MotionGraph() = default;
    virtual ~MotionGraph() = default;

    VertexCloud<Vec3f>& graph() { return mGraph; }
    std::vector<float>& radiuses() { return mRadiuses; }
    std::vector<Mat4f>& transforms() { return mTransforms; }
    const VertexCloud<Vec3f>& graph() const { return mGraph; }
    const std::vector<float>& radiuses() const { return mRadiuses; }
    const std::vector<Mat4f>& transforms() const { return mTransforms; }

    void push_back(const Vec3f& cPos, const float cRadius, const Mat4f& cTransform) {
        if (cRadius < 0) throw std::runtime_error("MotionGraph::push_back(): warp radius cannot be <0.");
        mGraph.vec_.push_back(cPos);
        mRadiuses.push_back(cRadius);
        mTransforms.push_back(cTransform);
    }
    void updateAt(const std::size_t cIndex, const Vec3f& cPos, const float cRadius, const Mat4f& cTransform) {
        if (cRadius < 0) throw std::runtime_error("MotionGraph::updateAt(): warp radius cannot be <0.");
        mGraph.vec_[cIndex] = cPos;
        mRadiuses[cIndex] = cRadius;
        mTransforms[cIndex] = cTransform;
    }
    void eraseAt(const std::size_t cIndex) {
        mGraph.vec_.erase(mGraph.vec_.begin() + (long)cIndex);
        mRadiuses.erase(mRadiuses.begin() + (long)cIndex);
        mTransforms.erase(mTransforms.begin() + (long)cIndex);
    }
    void clear() {
        mGraph.clear();
        mRadiuses.clear();
        mTransforms.clear();
    }

    // The skinning weight of one node at one distance, in the reference's double-precision form
    // (src/MotionGraph.cpp:39-41).
    float weight(std::size_t nodeId, float distance) {
        const float r = mRadiuses[nodeId];
        return (distance >= r) ? 0.f : (float)std::exp(-(distance * distance) / (2 * std::pow((double)r, 2)));
    }

    // The KNN nearest nodes of one point, on the device (afx_knn): ordered by distance, equal
    // distances by node index, missing slots UINT_MAX / FLT_MAX.
    template <int KNN>
    void knnSearch(Vecui<KNN>& outputIndicies, Vecf<KNN>& outputDists, const Vec3f& cPoint,
                   bool excludeClosest = false) const;
    // At most resultsCount nearest nodes (fewer when the graph is smaller).
    void knnSearch(std::vector<unsigned int>& outputIndicies, std::vector<float>& outputDists, const Vec3f& cPoint,
                   std::size_t resultsCount) const;

    // Linear blend of the cKnnCount nearest nodes' transforms (src/MotionGraph.cpp:62-90), on the
    // device: afx_knn, afx_warp_weights, afx_warp.  The weights are binary32 there, so points
    // agree with the reference's double-precision weights to float rounding.
    void warp(std::vector<Vec3f>& warpedPoints, const std::vector<Vec3f>& cInputPoints,
              const std::size_t cKnnCount = Constants::motionGraphKNN);

private:
    VertexCloud<Vec3f> mGraph;
    std::vector<float> mRadiuses;
    std::vector<Mat4f> mTransforms;
};

namespace detail {

// A MotionGraph's nodes on the device, with room for `capacity` nodes.
struct DeviceGraphCopy {
    DeviceArray<Vec3f> nodes;
    DeviceArray<float> radii;
    DeviceArray<Mat4f> transforms;
    DeviceInt n;
    int capacity;

    DeviceGraphCopy(const MotionGraph& g, std::size_t cap)
        : nodes(cap ? cap : 1), radii(cap ? cap : 1), transforms(cap ? cap : 1), n((int)g.graph().size()),
          capacity((int)(cap ? cap : 1)) {
        const std::size_t m = g.graph().size();
        copyToDevice(nodes.get(), g.graph().vec_.data(), m);
        copyToDevice(radii.get(), g.radiuses().data(), m);
        copyToDevice(transforms.get(), g.transforms().data(), m);
    }
};

// The k nearest graph nodes of m host points, row-major (point i's slots at i * k), on the device.
inline void knn_on_device(const MotionGraph& g, const Vec3f* points, std::size_t m, int k, bool excludeClosest,
                          uint32_t* idx, float* dist) {
    if (m == 0) return;
    DeviceGraphCopy dg(g, g.graph().size());
    DeviceArray<Vec3f> p(m);
    copyToDevice(p.get(), points, m);
    DeviceArray<uint32_t> I(m * (std::size_t)k);
    DeviceArray<float> D(m * (std::size_t)k);
    afx_check(afx_knn(I.get(), D.get(), ff<3>(dg.nodes.get()), dg.n.p, dg.capacity, ff<3>(p.get()), nullptr, (long)m,
                      k, excludeClosest ? 1 : 0, nullptr),
              "knn");
    copyToHost(idx, I.get(), I.size());
    copyToHost(dist, D.get(), D.size());
}

}  // namespace detail

template <int KNN>
void MotionGraph::knnSearch(Vecui<KNN>& outputIndicies, Vecf<KNN>& outputDists, const Vec3f& cPoint,
                            bool excludeClosest) const {
    detail::knn_on_device(*this, &cPoint, 1, KNN, excludeClosest, reinterpret_cast<uint32_t*>(outputIndicies.data()),
                          outputDists.data());
}

inline void MotionGraph::knnSearch(std::vector<unsigned int>& outputIndicies, std::vector<float>& outputDists,
                                   const Vec3f& cPoint, std::size_t resultsCount) const {
    const std::size_t found = std::min(resultsCount, mGraph.size());
    outputIndicies.assign(resultsCount, 0u);
    outputDists.assign(resultsCount, 0.f);
    if (resultsCount)
        detail::knn_on_device(*this, &cPoint, 1, (int)resultsCount, false, outputIndicies.data(), outputDists.data());
    outputIndicies.resize(found);
    outputDists.resize(found);
}

inline void MotionGraph::warp(std::vector<Vec3f>& warpedPoints, const std::vector<Vec3f>& cInputPoints,
                              const std::size_t cKnnCount) {
    const std::size_t m = cInputPoints.size();
    warpedPoints.resize(m);
    if (m == 0) return;
    const int k = (int)cKnnCount;
    detail::DeviceGraphCopy dg(*this, mGraph.size());
    DeviceArray<Vec3f> p(m), out(m);
    copyToDevice(p.get(), cInputPoints.data(), m);
    DeviceArray<uint32_t> I(m * cKnnCount);
    DeviceArray<float> D(m * cKnnCount), W(m * cKnnCount);
    detail::afx_check(afx_knn(I.get(), D.get(), detail::ff<3>(dg.nodes.get()), dg.n.p, dg.capacity,
                              detail::ff<3>(p.get()), nullptr, (long)m, k, 0, nullptr),
                      "MotionGraph::warp (knn)");
    detail::afx_check(afx_warp_weights(W.get(), dg.radii.get(), I.get(), D.get(), nullptr, (long)m, k, dg.n.p, nullptr),
                      "MotionGraph::warp (weights)");
    detail::afx_check(afx_warp(detail::ff<3>(out.get()), detail::ff<3>(p.get()), detail::ff<16>(dg.transforms.get()),
                               I.get(), W.get(), nullptr, (long)m, k, nullptr),
                      "MotionGraph::warp");
    copyToHost(warpedPoints.data(), out.get(), m);
}

// ---- include/af/GraphBuilder.h, src/GraphBuilder.cpp ----

// Appends a node (radius cMotionGraphMinRadius, the nearest node's transform) for every point of
// `mesh`, in order, that no node covers (src/GraphBuilder.cpp:12-51), on the device (afx_build_graph).
// The device build needs one radius for all nodes: a graph holding other radii is refused.
inline void buildGraph(MotionGraph& graph, const std::vector<Vec3f>& mesh, const std::size_t cMotionGraphKnn,
                       const float cMotionGraphMinRadius) {
    if (mesh.empty()) return;
    const std::size_t n0 = graph.graph().size();
    const std::size_t cap = n0 + mesh.size();
    detail::DeviceGraphCopy dg(graph, cap);
    DeviceArray<Vec3f> m(mesh.size());
    copyToDevice(m.get(), mesh.data(), mesh.size());
    DeviceArray<unsigned> mc(1);
    const unsigned cnt = (unsigned)mesh.size();
    copyToDevice(mc.get(), &cnt, 1);
    detail::Workspace ws(afx_build_graph_workspace_size((long)mesh.size(), (int)cap));
    detail::afx_check(afx_build_graph(detail::ff<3>(dg.nodes.get()), dg.radii.get(), detail::ff<16>(dg.transforms.get()),
                                      dg.n.p, (int)cap, detail::ff<3>(m.get()), mc.get(), (long)mesh.size(),
                                      (int)cMotionGraphKnn, cMotionGraphMinRadius, ws.p, ws.bytes, nullptr),
                      "buildGraph");
    const std::size_t n1 = (std::size_t)dg.n.get();
    std::vector<Vec3f> nodes(n1 - n0);
    std::vector<float> radii(n1 - n0);
    std::vector<Mat4f> T(n1 - n0);
    copyToHost(nodes.data(), dg.nodes.get() + n0, nodes.size());
    copyToHost(radii.data(), dg.radii.get() + n0, radii.size());
    copyToHost(T.data(), dg.transforms.get() + n0, T.size());
    for (std::size_t i = 0; i < nodes.size(); ++i) graph.push_back(nodes[i], radii[i], T[i]);
}

// Per point, the KNN nearest nodes (excludeClosest drops the nearest one, for node-to-node
// neighbours); missing slots UINT_MAX / FLT_MAX (include/af/GraphBuilder.h:18-30).
template <int KNN>
void getKnnData(std::vector<Vecui<KNN>>& knnIdxs, std::vector<Vecf<KNN>>& knnDists, const MotionGraph& cGraph,
                const std::vector<Vec3f>& cMesh, bool excludeClosest = false) {
    knnIdxs.resize(cMesh.size());
    knnDists.resize(cMesh.size());
    detail::knn_on_device(cGraph, cMesh.data(), cMesh.size(), KNN, excludeClosest,
                          reinterpret_cast<uint32_t*>(knnIdxs.data()), reinterpret_cast<float*>(knnDists.data()));
}

// The same in the flat layout of src/GraphBuilder.cpp:53-78: slot k of point i at i + k * size.
inline void getKnnData(std::vector<unsigned int>& knnIdxs, std::vector<float>& knnDists, MotionGraph& cGraph,
                       const std::vector<Vec3f>& cMesh, const int cKnn, bool excludeClosest = false) {
    const std::size_t m = cMesh.size();
    std::vector<unsigned int> I(m * (std::size_t)cKnn);
    std::vector<float> D(m * (std::size_t)cKnn);
    detail::knn_on_device(cGraph, cMesh.data(), m, cKnn, excludeClosest, I.data(), D.data());
    knnIdxs.resize(I.size());
    knnDists.resize(D.size());
    for (std::size_t i = 0; i < m; ++i)
        for (int k = 0; k < cKnn; ++k) {
            knnIdxs[i + (std::size_t)k * m] = I[i * (std::size_t)cKnn + (std::size_t)k];
            knnDists[i + (std::size_t)k * m] = D[i * (std::size_t)cKnn + (std::size_t)k];
        }
}

// Row i holds node i's neighbours: those farther than 1.3 x node i's radius are cut
// (include/af/GraphBuilder.h:32-47), on the device (afx_filter_disconnected).
template <int KNN>
void filterDisconnected(std::vector<Vecui<KNN>>& knnIdxs, std::vector<Vecf<KNN>>& knnDists, const MotionGraph& cGraph) {
    const std::size_t rows = knnIdxs.size();
    if (rows == 0) return;
    if (rows > cGraph.graph().size() || knnDists.size() != rows)
        throw std::invalid_argument("filterDisconnected: one row per graph node");
    detail::DeviceGraphCopy dg(cGraph, cGraph.graph().size());
    DeviceArray<Vecui<KNN>> I(rows);
    DeviceArray<Vecf<KNN>> D(rows);
    copyToDevice(I.get(), knnIdxs.data(), rows);
    copyToDevice(D.get(), knnDists.data(), rows);
    detail::afx_check(afx_filter_disconnected(reinterpret_cast<uint32_t*>(I.get()), reinterpret_cast<float*>(D.get()),
                                              dg.n.p, (int)rows, KNN, dg.radii.get(), nullptr),
                      "filterDisconnected");
    copyToHost(knnIdxs.data(), I.get(), rows);
    copyToHost(knnDists.data(), D.get(), rows);
}

// The distinct points of cInput (the reference's unordered_set leaves their order unspecified;
// here they come out sorted), on the device (afx_sort_unique_points).
inline void removeDuplicates(std::vector<Vec3f>& output, const std::vector<Vec3f>& cInput) {
    const std::size_t m = cInput.size();
    output.clear();
    if (m == 0) return;
    DeviceArray<Vec3f> p(m);
    copyToDevice(p.get(), cInput.data(), m);
    DeviceArray<unsigned> c(1);
    const unsigned cnt = (unsigned)m;
    copyToDevice(c.get(), &cnt, 1);
    detail::Workspace ws(afx_sort_unique_points_workspace_size((long)m));
    detail::afx_check(afx_sort_unique_points(detail::ff<3>(p.get()), c.get(), (long)m, ws.p, ws.bytes, nullptr),
                      "removeDuplicates");
    unsigned n = 0;
    copyToHost(&n, c.get(), 1);
    output.resize(n);
    copyToHost(output.data(), p.get(), n);
}

inline void translate(std::vector<Vec3f>& data, const Vec3f& cTransVec) {
    if (data.empty()) return;
    DeviceArray<Vec3f> p(data.size());
    copyToDevice(p.get(), data.data(), data.size());
    af::runTranslateKernel(p.get(), (unsigned int)data.size(), cTransVec);
    copyToHost(data.data(), p.get(), data.size());
}

}  // namespace af

#endif
