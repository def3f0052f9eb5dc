// af_surface_check.cpp -- a C++ caller of the af:: surface (af/afx_classes.h) written the way the
// reference's own code calls it: DeviceTsdf -> extractPointCloud -> MotionGraph / buildGraph /
// getKnnData / filterDisconnected -> WarpField (spreadMotionGraph, weighted KNN, warp) ->
// runCorrespondencePairsKernel -> GaussNewtonSystem -> runUpdateTransformsKernel, plus TSDFVolume
// integrate / save / load, and the depth-ingest functions (loadDepthFrame, loadIntrinsics,
// loadCameraDistortion, DepthUndistorter, create_xy_lookup_table).  It reads one pair of prepared
// frames (and a PNG frame with its calibration files) from <in_dir> and writes every
// intermediate result to <out_dir> as raw arrays; tests/test_cpp_surface_gpu.py compares them
// with the CPU oracle.  Built with AFX_TEST_WITH_EIGEN, the value types are Eigen's.
#ifdef AFX_TEST_WITH_EIGEN
#include <Eigen/Core>
#endif
#include <af/afx_classes.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

namespace {

std::string g_in, g_out;

template <class T>
std::vector<T> read_raw(const std::string& name) {
    std::ifstream f(g_in + "/" + name, std::ios::binary | std::ios::ate);
    if (!f) throw std::runtime_error("cannot read " + name);
    const std::streamsize bytes = f.tellg();
    f.seekg(0);
    std::vector<T> v((std::size_t)bytes / sizeof(T));
    f.read(reinterpret_cast<char*>(v.data()), (std::streamsize)(v.size() * sizeof(T)));
    return v;
}

template <class T>
void write_raw(const std::string& name, const T* p, std::size_t n) {
    std::ofstream f(g_out + "/" + name, std::ios::binary);
    f.write(reinterpret_cast<const char*>(p), (std::streamsize)(n * sizeof(T)));
}
template <class T>
void write_raw(const std::string& name, const std::vector<T>& v) {
    write_raw(name, v.data(), v.size());
}
template <class T>
std::vector<T> download(const T* d, std::size_t n) {
    std::vector<T> v(n);
    af::copyToHost(v.data(), d, n);
    return v;
}

int run() {
    // meta: width, height, fx, fy, cx, cy, dims[3], size[3], delta, radius, corr_thresh,
    //       lambda_depth, lambda_reg, centroid[3]
    const std::vector<float> meta = read_raw<float>("meta.bin");
    const int w = (int)meta[0], h = (int)meta[1];
    af::Mat3f K = af::Mat3f::Identity();
    K(0, 0) = meta[2];
    K(1, 1) = meta[3];
    K(0, 2) = meta[4];
    K(1, 2) = meta[5];
    const af::Vec3i dims((int)meta[6], (int)meta[7], (int)meta[8]);
    const af::Vec3f size(meta[9], meta[10], meta[11]);
    const float delta = meta[12], radius = meta[13], corrThresh = meta[14], lamD = meta[15], lamR = meta[16];
    const af::Vec3f c(meta[17], meta[18], meta[19]);
    const std::size_t P = (std::size_t)w * (std::size_t)h;

    const std::vector<float> depth0 = read_raw<float>("depth0.bin");
    const std::vector<float> depth1 = read_raw<float>("depth1.bin");
    const std::vector<af::Vec3f> verts1 = read_raw<af::Vec3f>("verts1.bin");
    const std::vector<af::Vec3f> normals1 = read_raw<af::Vec3f>("normals1.bin");

    // 1. DeviceTsdf: integrate frame 0 through the volume pose (identity rotation, centre c)
    af::CameraModel camera;
    camera.width = (unsigned)w;
    camera.height = (unsigned)h;
    camera.depthIntrinsics = K;
    af::DeviceDepthImage depth_d((std::size_t)h, (std::size_t)w, camera);
    depth_d.upload(depth0.data());
    af::DeviceTsdf<float> tsdf(size, dims, c, af::Mat3f::Identity(), delta);
    tsdf.integrate(depth_d);
    write_raw("tsdf.bin", download(tsdf.tsdfPtr(), tsdf.voxelCount()));
    write_raw("weights.bin", download(tsdf.weightsPtr(), tsdf.voxelCount()));

    // 2. point cloud (marching cubes, sort, unique), then into camera space
    af::DeviceBufferCounted<af::Vec3f> cloud((unsigned)(tsdf.voxelCount() * 3 / 4));
    tsdf.extractPointCloud(cloud);
    write_raw("cloud.bin", cloud.download());
    af::runTranslateKernel(cloud.bufferPtr(), cloud.size(), c);
    const std::vector<af::Vec3f> mesh = cloud.download();
    write_raw("mesh.bin", mesh);
    const std::size_t m = mesh.size();

    // 3. host MotionGraph through buildGraph / getKnnData / filterDisconnected / warp
    af::MotionGraph graph;
    af::buildGraph(graph, mesh, af::Constants::motionGraphKNN, radius);
    const std::size_t n = graph.graph().size();
    write_raw("nodes.bin", graph.graph().vec_);
    write_raw("radii.bin", graph.radiuses());
    write_raw("transforms.bin", graph.transforms());

    std::vector<af::Vecui<6>> midx;
    std::vector<af::Vecf<6>> mdist;
    af::getKnnData(midx, mdist, graph, mesh);
    write_raw("midx.bin", midx);
    write_raw("mdist.bin", mdist);

    std::vector<unsigned int> fidx;
    std::vector<float> fdist;
    af::getKnnData(fidx, fdist, graph, graph.graph().vec_, 4, true);
    write_raw("flat_idx.bin", fidx);
    write_raw("flat_dist.bin", fdist);

    std::vector<af::Vecui<4>> gidx;
    std::vector<af::Vecf<4>> gdist;
    af::getKnnData(gidx, gdist, graph, graph.graph().vec_, true);
    af::filterDisconnected(gidx, gdist, graph);
    write_raw("gidx.bin", gidx);
    write_raw("gdist.bin", gdist);

    af::Vecui<6> one_idx;
    af::Vecf<6> one_dist;
    graph.knnSearch(one_idx, one_dist, mesh[m / 2]);
    write_raw("one_idx.bin", one_idx.data(), 6);
    write_raw("one_dist.bin", one_dist.data(), 6);

    for (std::size_t i = 0; i < n; ++i) {  // a smooth deterministic motion
        af::Mat4f& T = graph.transforms()[i];
        T.data()[12] += 0.003f * std::sin(1.3f * (float)i);
        T.data()[13] += 0.003f * std::cos(0.7f * (float)i);
        T.data()[14] += 0.002f * std::sin(0.4f * (float)i + 1.0f);
    }
    write_raw("transforms_moved.bin", graph.transforms());
    std::vector<af::Vec3f> warped_host;
    graph.warp(warped_host, mesh);
    write_raw("warped_motion_graph.bin", warped_host);

    // 4. WarpField on the device: the same graph, skinning, warp
    af::Settings settings;
    settings.motionGraphRadius = radius;
    af::WarpField field(n + 64, settings);
    field.spreadMotionGraph(cloud);
    const std::size_t nf = field.motionGraph_d().count();
    write_raw("field_nodes.bin", download(field.motionGraph_d().pointsPtr(), nf));
    af::DeviceKnnWeighted<(int)af::Constants::motionGraphKNN> knn_d(m);
    field.computePointCloudWeightedKnns(knn_d);
    write_raw("field_midx.bin", download(knn_d.idxsPtr(), m));
    write_raw("field_mw.bin", download(knn_d.weightsPtr(), m));
    field.computeGraphKnns();
    write_raw("field_gidx.bin", download(field.graphKnnIdxs_d().bufferPtr(), nf));
    af::copyToDevice(field.motionGraph_d().transformsPtr(), graph.transforms().data(), n);
    af::DeviceBuffer<af::Vec3f> warped_d((unsigned)m);
    field.warp(warped_d, cloud, knn_d);
    write_raw("warped_field.bin", warped_d.download());

    // the stand-alone weights operator on the same neighbours
    af::DeviceArray<af::Vecf<6>> w2(m);
    af::runComputeWarpWeightsKernel(w2.get(), field.motionGraph_d().radiusesPtr(), knn_d.idxsPtr(), knn_d.distsPtr(), m);
    write_raw("weights_op.bin", download(w2.get(), m));

    // 5. correspondences with frame 1
    af::DeviceArray<float> d1(P);
    af::copyToDevice(d1.get(), depth1.data(), P);
    af::DeviceArray<af::Vec3f> v1(P), n1(P);
    af::copyToDevice(v1.get(), verts1.data(), P);
    af::copyToDevice(n1.get(), normals1.data(), P);
    af::DeviceBufferCounted<af::Vec2i> corr_d((unsigned)m);
    af::runCorrespondencePairsKernel(corr_d.bufferPtr(), corr_d.size_dPtr(), warped_d.bufferPtr(), m, K, d1.get(),
                                     af::Vec2i(h, w), v1.get(), corrThresh);
    corr_d.syncHostSize();
    const std::size_t nc = corr_d.size();
    write_raw("corr.bin", corr_d.download());

    // 6. Gauss-Newton: build, dense export, 10 PCG iterations, transform update
    af::DeviceBuffer<af::Vecui<4>> gidx_d((unsigned)n);
    gidx_d.upload(gidx);
    af::DeviceArray<unsigned> npts(1);
    const unsigned mu = (unsigned)m;
    af::copyToDevice(npts.get(), &mu, 1);
    af::GaussNewtonSystem gn((long)m + 16, (int)n + 8, 6, 4);
    gn.build(cloud.bufferPtr(), npts.get(), knn_d.idxsPtr(), knn_d.weightsPtr(), corr_d.bufferPtr(), corr_d.size_dPtr(),
             v1.get(), n1.get(), warped_d.bufferPtr(), field.motionGraph_d().pointsPtr(),
             field.motionGraph_d().transformsPtr(), field.motionGraph_d().countPtr(), gidx_d.bufferPtr(), lamD, lamR);
    const std::size_t dim = 6 * n;
    af::DeviceArray<float> jtj(dim * dim), jtr(dim), rd(nc ? nc : 1), rr(n * 4 * 3);
    gn.exportDense((int)n, jtj.get(), jtr.get(), rd.get(), rr.get());
    write_raw("jtj.bin", download(jtj.get(), dim * dim));
    write_raw("jtr.bin", download(jtr.get(), dim));
    write_raw("r_depth.bin", download(rd.get(), nc));
    write_raw("r_reg.bin", download(rr.get(), n * 12));
    // 6b. the reference's dense sequence (src/VolumeFusion.cu:454-660) through the dense operators,
    // its thrust sort + reduce_by_key done on the host as a stable sort and sequential sums
    {
        const unsigned hD = (unsigned)nc, hR = (unsigned)(n * 4 * 3), rowsJ = hD + hR;
        af::DeviceArray<af::Vec6f> J((std::size_t)rowsJ * n);
        af::DeviceArray<float> r(rowsJ);
        af::detail::cuda_check(cudaMemset(J.get(), 0, sizeof(af::Vec6f) * (std::size_t)rowsJ * n), "memset");
        af::detail::cuda_check(cudaMemset(r.get(), 0, sizeof(float) * rowsJ), "memset");
        af::runFill_J_DepthKernel(J.get(), lamD, hD, (unsigned)n, corr_d.bufferPtr(), hD, cloud.bufferPtr(),
                                  knn_d.idxsPtr(), knn_d.weightsPtr(), v1.get(), n1.get());
        af::runFill_r_DepthKernel(r.get(), lamD, corr_d.bufferPtr(), hD, warped_d.bufferPtr(), v1.get(), n1.get());
        af::runFill_r_MRegKernel(r.get() + hD, lamR, field.motionGraph_d().pointsPtr(),
                                 field.motionGraph_d().transformsPtr(), (unsigned)n, gidx_d.bufferPtr());
        af::runFill_J_MRegKernel(J.get() + (std::size_t)hD * n, lamR, hR, (unsigned)n, field.motionGraph_d().pointsPtr(),
                                 field.motionGraph_d().transformsPtr(), (unsigned)n, gidx_d.bufferPtr());
        const unsigned maxPairs = hD * (af::combinations(6, 2) + 6) + hR * 3, maxElems = hD * 6 + hR * 2;
        af::DeviceArray<af::Vec2i> pairs(maxPairs), elems(maxElems);
        af::DeviceArray<unsigned> rows(maxPairs), counts(2);
        af::detail::cuda_check(cudaMemset(counts.get(), 0, 8), "memset");
        af::runComputeJTJAndJTrContribJDepthKernel(pairs.get(), rows.get(), counts.get(), elems.get(), counts.get() + 1,
                                                   corr_d.bufferPtr(), hD, knn_d.idxsPtr(), knn_d.weightsPtr());
        af::runComputeJTJAndJTrContribJMRegKernel(pairs.get(), rows.get(), hD, counts.get(), elems.get(), counts.get() + 1,
                                                  (unsigned)n, gidx_d.bufferPtr());
        const std::vector<unsigned> cnt = download(counts.get(), 2);
        std::vector<af::Vec2i> P = download(pairs.get(), cnt[0]), E = download(elems.get(), cnt[1]);
        std::vector<unsigned> R = download(rows.get(), cnt[0]);
        std::vector<unsigned> order(cnt[0]);
        for (unsigned i = 0; i < cnt[0]; ++i) order[i] = i;
        std::stable_sort(order.begin(), order.end(), [&](unsigned a, unsigned b) {
            return P[a][0] < P[b][0] || (P[a][0] == P[b][0] && P[a][1] < P[b][1]);
        });
        std::vector<af::Vec2i> sp(cnt[0]);
        std::vector<unsigned> sr(cnt[0]);
        for (unsigned i = 0; i < cnt[0]; ++i) {
            sp[i] = P[order[i]];
            sr[i] = R[order[i]];
        }
        af::DeviceArray<af::Vec2i> sp_d(cnt[0]);
        af::DeviceArray<unsigned> sr_d(cnt[0]);
        af::DeviceArray<af::Mat6f> prod_d(cnt[0]);
        af::copyToDevice(sp_d.get(), sp.data(), sp.size());
        af::copyToDevice(sr_d.get(), sr.data(), sr.size());
        af::runMultiplyJTJContribPairsKernel(prod_d.get(), sp_d.get(), sr_d.get(), cnt[0], J.get(), (unsigned)n);
        std::vector<float> prod(36 * (std::size_t)cnt[0]);
        af::copyToHost(prod.data(), reinterpret_cast<const float*>(prod_d.get()), prod.size());
        std::vector<af::Vec2i> coords;
        std::vector<float> sums;
        for (unsigned i = 0; i < cnt[0]; ++i) {
            if (!coords.empty() && coords.back()[0] == sp[i][0] && coords.back()[1] == sp[i][1]) {
                float* s = sums.data() + sums.size() - 36;
                for (int e = 0; e < 36; ++e) s[e] = s[e] + prod[36 * (std::size_t)i + e];
            } else {
                coords.push_back(sp[i]);
                sums.insert(sums.end(), prod.begin() + 36 * (std::size_t)i, prod.begin() + 36 * (std::size_t)(i + 1));
            }
        }
        std::vector<unsigned> eorder(cnt[1]);
        for (unsigned i = 0; i < cnt[1]; ++i) eorder[i] = i;
        std::stable_sort(eorder.begin(), eorder.end(), [&](unsigned a, unsigned b) { return E[a][1] < E[b][1]; });
        std::vector<af::Vec2i> se(cnt[1]);
        for (unsigned i = 0; i < cnt[1]; ++i) se[i] = E[eorder[i]];
        af::DeviceArray<af::Vec2i> se_d(cnt[1]);
        af::DeviceArray<af::Vec6f> eprod_d(cnt[1]);
        af::copyToDevice(se_d.get(), se.data(), se.size());
        af::runMultiplyJTrContribElemsKernel(eprod_d.get(), se_d.get(), cnt[1], J.get(), r.get(), (unsigned)n);
        std::vector<float> eprod(6 * (std::size_t)cnt[1]);
        af::copyToHost(eprod.data(), reinterpret_cast<const float*>(eprod_d.get()), eprod.size());
        std::vector<af::Vec2i> ecoords;
        std::vector<float> esums;
        for (unsigned i = 0; i < cnt[1]; ++i) {
            if (!ecoords.empty() && ecoords.back()[1] == se[i][1]) {
                float* s = esums.data() + esums.size() - 6;
                for (int e = 0; e < 6; ++e) s[e] = s[e] + eprod[6 * (std::size_t)i + e];
            } else {
                ecoords.push_back(se[i]);
                esums.insert(esums.end(), eprod.begin() + 6 * (std::size_t)i, eprod.begin() + 6 * (std::size_t)(i + 1));
            }
        }
        std::vector<float> eye(dim * dim, 0.f);  // runInitIdentityKernel
        for (std::size_t i = 0; i < dim; ++i) eye[i * dim + i] = 1.f;
        af::DeviceArray<float> jtj2(dim * dim), jtr2(dim), x2(dim);
        af::copyToDevice(jtj2.get(), eye.data(), eye.size());
        af::detail::cuda_check(cudaMemset(jtr2.get(), 0, sizeof(float) * dim), "memset");
        af::DeviceArray<af::Vec2i> c_d(coords.size()), ec_d(ecoords.size());
        af::DeviceArray<float> s_d(sums.size()), es_d(esums.size());
        af::copyToDevice(c_d.get(), coords.data(), coords.size());
        af::copyToDevice(s_d.get(), sums.data(), sums.size());
        af::copyToDevice(ec_d.get(), ecoords.data(), ecoords.size());
        af::copyToDevice(es_d.get(), esums.data(), esums.size());
        af::runFillJTJKernel(jtj2.get(), c_d.get(), reinterpret_cast<const af::Mat6f*>(s_d.get()), (unsigned)coords.size(),
                             (unsigned)dim);
        af::runFillJTrKernel(reinterpret_cast<af::Vec6f*>(jtr2.get()), ec_d.get(),
                             reinterpret_cast<const af::Vec6f*>(es_d.get()), (unsigned)ecoords.size());
        write_raw("jtj_dense_ops.bin", download(jtj2.get(), dim * dim));
        write_raw("jtr_dense_ops.bin", download(jtr2.get(), dim));
        write_raw("r_dense_ops.bin", download(r.get(), rowsJ));
        af::DeviceArray<int> ipiv(dim);
        const bool solved = af::linearSolverLUStable(nullptr, (int)dim, jtj2.get(), (int)dim, jtr2.get(), ipiv.get(), x2.get());
        if (!solved) throw std::runtime_error("linearSolverLUStable failed");
        write_raw("x_lu.bin", download(x2.get(), dim));
    }

    af::DeviceArray<af::Vec6f> x((std::size_t)gn.nodesMax());
    gn.solve(x.get(), 10);
    write_raw("x.bin", download(x.get(), n));
    af::runUpdateTransformsKernel(field.motionGraph_d().transformsPtr(), x.get(), (unsigned)n);
    write_raw("transforms_updated.bin", download(field.motionGraph_d().transformsPtr(), n));

    // 7. TSDFVolume: the same frame through pose [I | c], save, load
    af::TSDFVolume volume(dims, size, K);
    volume.setDelta(delta);
    af::Mat4f pose = af::Mat4f::Identity();
    pose(0, 3) = c[0];
    pose(1, 3) = c[1];
    pose(2, 3) = c[2];
    volume.integrate(pose, depth0.data(), h, w);
    write_raw("volume_tsdf.bin", volume.tsdf());
    const std::string path = g_out + "/volume.tsdf";
    volume.save(path);
    af::TSDFVolume loaded(af::Vec3i(1, 1, 1), af::Vec3f(1.f, 1.f, 1.f), K);
    loaded.load(path);
    const bool same = loaded.tsdf() == volume.tsdf() && loaded.tsdfWeights() == volume.tsdfWeights() &&
                      loaded.dimensions() == volume.dimensions() && loaded.delta() == volume.delta();

    // 8. depth filter with a fill value (DeviceImage::nullifyUpperBound fills +inf)
    af::DeviceArray<float> f0(P);
    af::copyToDevice(f0.get(), depth0.data(), P);
    af::runFilterDepthKernel(f0.get(), (unsigned)P, 0.9f, 0.0f);
    write_raw("filtered.bin", download(f0.get(), P));

    // 9. depth ingest: af::loadDepthFrame of a 16-bit PNG by pattern, the calibration files,
    // cv::undistort on the device, and create_xy_lookup_table
    af::DeviceDepthImage frame(camera);
    af::loadDepthFrame(g_in + "/frame-******.depth.png", 3, frame);
    write_raw("ingest_depth.bin", download(frame.dataPtr(), frame.size()));
    af::Mat3f Kf;
    af::loadIntrinsics(g_in + "/depthIntrinsics.txt", Kf);
    af::CameraDistortion dist;
    const bool has_dist = af::loadCameraDistortion(g_in + "/depthDistortion.txt", dist);
    af::DepthUndistorter undistort(Kf, dist, (int)frame.width(), (int)frame.height());
    undistort.apply(frame);
    write_raw("ingest_undistorted.bin", download(frame.dataPtr(), frame.size()));
    af::CameraModel lens;
    lens.width = (unsigned)frame.width();
    lens.height = (unsigned)frame.height();
    lens.intrinsics.cx = Kf(0, 2);
    lens.intrinsics.cy = Kf(1, 2);
    lens.intrinsics.fx = Kf(0, 0);
    lens.intrinsics.fy = Kf(1, 1);
    lens.distortion = dist;
    af::DeviceBuffer<af::Vec2f> table(1);
    const bool table_ok = af::create_xy_lookup_table(lens, table);
    write_raw("ingest_xy.bin", download(table.bufferPtr(), table.size()));

    std::printf("{\"points\": %zu, \"nodes\": %zu, \"field_nodes\": %zu, \"correspondences\": %zu, "
                "\"volume_roundtrip\": %s, \"ingest\": [%d, %d, %s, %s, \"%s\"]}\n",
                m, n, nf, nc, same ? "true" : "false", (int)frame.width(), (int)frame.height(),
                has_dist ? "true" : "false", table_ok ? "true" : "false",
                af::insertIntoPattern("frame-******.depth.png", 42).c_str());
    return 0;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc != 3) {
        std::fprintf(stderr, "usage: %s <in_dir> <out_dir>\n", argv[0]);
        return 2;
    }
    g_in = argv[1];
    g_out = argv[2];
    try {
        return run();
    } catch (const std::exception& e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
}
