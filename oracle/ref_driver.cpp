// ref_driver.cpp -- C entry points around the reference's own CPU classes, built with
// oracle/Makefile.ref into oracle/_ref/libvfref.so from the reference source tree.
//
// Test infrastructure only.  It lets the tests and the fixture generator run the
// reference's TSDFVolume::integrate, MarchingCubes::computeIsoSurface/computePointCloud,
// af::buildGraph, af::getKnnData, af::filterDisconnected and MotionGraph::warp on
// in-memory inputs.  Nothing here re-implements the reference; it only marshals arrays.
#include <af/CameraCalibration.h>
#include <af/GraphBuilder.h>
#include <af/MarchingCubes.h>
#include <af/Mesh.h>
#include <af/MotionGraph.h>
#include <af/TSDFVolume.h>

#include <cstring>
#include <vector>

namespace {

Mat3f mat3(const float* cm) {
    Mat3f M;
    std::memcpy(M.data(), cm, sizeof(float) * 9);
    return M;
}

void load_graph(MotionGraph& g, const float* nodes, const float* radii, const float* T, int n) {
    for (int i = 0; i < n; ++i) {
        Mat4f M;
        std::memcpy(M.data(), T + 16 * i, sizeof(float) * 16);
        g.push_back(Vec3f(nodes[3 * i], nodes[3 * i + 1], nodes[3 * i + 2]), radii[i], M);
    }
}

template <int K>
void knn_impl(const MotionGraph& g, const float* pts, long m, int exclude, unsigned* idx, float* dist) {
    std::vector<Vec3f> P(m);
    for (long i = 0; i < m; ++i) P[i] = Vec3f(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]);
    std::vector<Vecui<K>> I;
    std::vector<Vecf<K>> D;
    af::getKnnData(I, D, g, P, exclude != 0);
    for (long i = 0; i < m; ++i)
        for (int s = 0; s < K; ++s) {
            idx[i * K + s] = I[i][s];
            dist[i * K + s] = D[i][s];
        }
}

template <int K>
void filter_impl(const MotionGraph& g, unsigned* idx, float* dist, int n) {
    std::vector<Vecui<K>> I(n);
    std::vector<Vecf<K>> D(n);
    for (int i = 0; i < n; ++i)
        for (int s = 0; s < K; ++s) {
            I[i][s] = idx[i * K + s];
            D[i][s] = dist[i * K + s];
        }
    af::filterDisconnected(I, D, g);
    for (int i = 0; i < n; ++i)
        for (int s = 0; s < K; ++s) {
            idx[i * K + s] = I[i][s];
            dist[i * K + s] = D[i][s];
        }
}

af::CameraModel bc_camera(int width, int height, const float* intr, const float* dist) {
    af::CameraModel cam;
    cam.width = (unsigned)width;
    cam.height = (unsigned)height;
    cam.intrinsics.cx = intr[0];
    cam.intrinsics.cy = intr[1];
    cam.intrinsics.fx = intr[2];
    cam.intrinsics.fy = intr[3];
    af::CameraDistortion& d = cam.distortion;
    d.k1 = dist[0];
    d.k2 = dist[1];
    d.k3 = dist[2];
    d.k4 = dist[3];
    d.k5 = dist[4];
    d.k6 = dist[5];
    d.codx = dist[6];
    d.cody = dist[7];
    d.p1 = dist[8];
    d.p2 = dist[9];
    d.is_distorted = true;
    return cam;
}

}  // namespace

namespace af {
// defined with external linkage in src/CameraCalibration.cpp:220-259 (no header declares them)
bool transformation_unproject(const af::CameraModel& camera, const Eigen::Vector2f& point2d, const float depth,
                              Eigen::Vector3f& point3d, int* valid);
bool transformation_project(const af::CameraModel& camera, const Eigen::Vector3f& point3d, Eigen::Vector2f& point2d,
                            int* valid);
}  // namespace af

extern "C" {

// af::create_xy_lookup_table (src/CameraCalibration.cpp:261-295) into table[height][width][2];
// intr = {cx, cy, fx, fy}, dist = {k1..k6, codx, cody, p1, p2}.  Returns its result (0/1).
int ref_xy_lookup_table(float* table, int width, int height, const float* intr, const float* dist) {
    af::CameraModel cam = bc_camera(width, height, intr, dist);
    cv::Mat t(height, width, table);
    return af::create_xy_lookup_table(cam, t) ? 1 : 0;
}

// af::transformation_unproject over n pixels (2 floats) and depths -> points (3 floats), valid.
void ref_bc_unproject(float* pts, int* valid, const float* px, const float* depth, long n, const float* intr,
                      const float* dist) {
    af::CameraModel cam = bc_camera(1, 1, intr, dist);
    for (long i = 0; i < n; ++i) {
        Eigen::Vector3f p(0.f, 0.f, 0.f);
        int v = 0;
        af::transformation_unproject(cam, Eigen::Vector2f(px[2 * i], px[2 * i + 1]), depth[i], p, &v);
        for (int c = 0; c < 3; ++c) pts[3 * i + c] = p(c);
        valid[i] = v;
    }
}

// af::transformation_project over n points -> pixels (left as passed in where the reference leaves them).
void ref_bc_project(float* px, int* valid, const float* pts, long n, const float* intr, const float* dist) {
    af::CameraModel cam = bc_camera(1, 1, intr, dist);
    for (long i = 0; i < n; ++i) {
        Eigen::Vector2f q(px[2 * i], px[2 * i + 1]);
        int v = 0;
        af::transformation_project(cam, Eigen::Vector3f(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]), q, &v);
        px[2 * i] = q(0);
        px[2 * i + 1] = q(1);
        valid[i] = v;
    }
}


// TSDFVolume::integrate (src/TSDFVolume.cpp:55-171); pose = Mat4f column-major
void ref_integrate(float* tsdf, float* weights, const float* depth, int width, int height, const float* K,
                   const int* dims, const float* size, float delta, const float* pose) {
    TSDFVolume vol(Vec3i(dims[0], dims[1], dims[2]), Vec3f(size[0], size[1], size[2]), mat3(K));
    vol.setDelta(delta);
    std::vector<unsigned char> color((size_t)width * height * 3, 0);
    cv::Mat c(height, width, color.data());
    cv::Mat d(height, width, const_cast<float*>(depth));
    Mat4f P;
    std::memcpy(P.data(), pose, sizeof(float) * 16);
    vol.integrate(P, c, d);
    std::memcpy(tsdf, vol.tsdf().data(), sizeof(float) * vol.tsdf().size());
    std::memcpy(weights, vol.tsdfWeights().data(), sizeof(float) * vol.tsdfWeights().size());
}

// MarchingCubes::computeIsoSurface / computePointCloud (src/MarchingCubes.cpp:297, :484)
long ref_marching_cubes(const float* tsdf, const float* weights, const int* dims, const float* size, float iso,
                        int point_cloud, float* verts, long vcap, int* faces, long fcap, long* nfaces) {
    const size_t S = (size_t)dims[0] * dims[1] * dims[2];
    std::vector<float> t(tsdf, tsdf + S), w(weights, weights + S);
    std::vector<unsigned char> col(S + 2, 127);
    MarchingCubes mc(Vec3i(dims[0], dims[1], dims[2]), Vec3f(size[0], size[1], size[2]));
    Mesh mesh;
    if (point_cloud) mc.computePointCloud(mesh, t, w, col, col, col, iso);
    else mc.computeIsoSurface(mesh, t, w, col, col, col, iso);
    const auto& V = mesh.vertexCloud().vec_;
    for (size_t i = 0; i < V.size() && (long)i < vcap; ++i)
        for (int c = 0; c < 3; ++c) verts[3 * i + c] = V[i][c];
    const auto& F = mesh.faces();
    for (size_t i = 0; i < F.size() && (long)i < fcap; ++i)
        for (int c = 0; c < 3; ++c) faces[3 * i + c] = F[i][c];
    if (nfaces) *nfaces = (long)F.size();
    return (long)V.size();
}

// af::buildGraph (src/GraphBuilder.cpp:12-50)
int ref_build_graph(float* nodes, float* radii, float* T, int n, int cap, const float* mesh, long m, int knn,
                    float radius) {
    MotionGraph g;
    load_graph(g, nodes, radii, T, n);
    std::vector<Vec3f> P(m);
    for (long i = 0; i < m; ++i) P[i] = Vec3f(mesh[3 * i], mesh[3 * i + 1], mesh[3 * i + 2]);
    af::buildGraph(g, P, (std::size_t)knn, radius);
    int nn = (int)g.graph().size();
    if (nn > cap) return -1;
    for (int i = 0; i < nn; ++i) {
        for (int c = 0; c < 3; ++c) nodes[3 * i + c] = g.graph().vec_[i][c];
        radii[i] = g.radiuses()[i];
        std::memcpy(T + 16 * i, g.transforms()[i].data(), sizeof(float) * 16);
    }
    return nn;
}

// af::getKnnData<K> (include/af/GraphBuilder.h:118-130); K in {4, 6, 8}
int ref_knn(const float* nodes, const float* radii, int n, const float* pts, long m, int k, int exclude,
            unsigned* idx, float* dist) {
    MotionGraph g;
    std::vector<float> T((size_t)16 * n, 0.f);
    load_graph(g, nodes, radii, T.data(), n);
    switch (k) {
        case 4: knn_impl<4>(g, pts, m, exclude, idx, dist); return 0;
        case 6: knn_impl<6>(g, pts, m, exclude, idx, dist); return 0;
        case 8: knn_impl<8>(g, pts, m, exclude, idx, dist); return 0;
    }
    return -1;
}

// af::filterDisconnected<K> (include/af/GraphBuilder.h:132-146)
int ref_filter_disconnected(const float* nodes, const float* radii, int n, int k, unsigned* idx, float* dist) {
    MotionGraph g;
    std::vector<float> T((size_t)16 * n, 0.f);
    load_graph(g, nodes, radii, T.data(), n);
    switch (k) {
        case 4: filter_impl<4>(g, idx, dist, n); return 0;
        case 6: filter_impl<6>(g, idx, dist, n); return 0;
        case 8: filter_impl<8>(g, idx, dist, n); return 0;
    }
    return -1;
}

// MotionGraph::warp (src/MotionGraph.cpp:62-90)
void ref_warp(const float* nodes, const float* radii, const float* T, int n, const float* pts, long m, int k,
              float* out) {
    MotionGraph g;
    load_graph(g, nodes, radii, T, n);
    std::vector<Vec3f> P(m), W;
    for (long i = 0; i < m; ++i) P[i] = Vec3f(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]);
    g.warp(W, P, (size_t)k);
    for (long i = 0; i < m; ++i)
        for (int c = 0; c < 3; ++c) out[3 * i + c] = W[i][c];
}

// Mesh::savePly (src/Mesh.cpp:23-64) of the given vertices (and colours, 0 if null) and faces.
int ref_save_ply(const char* path, const float* v, long nv, const unsigned char* rgb, const int* faces, long nf) {
    Mesh mesh;
    for (long i = 0; i < nv; ++i) {
        Vec3b c(rgb ? rgb[3 * i] : 0, rgb ? rgb[3 * i + 1] : 0, rgb ? rgb[3 * i + 2] : 0);
        mesh.addVertex(Vec3f(v[3 * i], v[3 * i + 1], v[3 * i + 2]), c);
    }
    for (long i = 0; i < nf; ++i) mesh.faces().push_back(Vec3i(faces[3 * i], faces[3 * i + 1], faces[3 * i + 2]));
    return mesh.savePly(path) ? 0 : 1;
}

// TSDFVolume::save (src/TSDFVolume.cpp:343-361) of a volume holding the given values and weights.
int ref_tsdf_save(const char* path, const int* dims, const float* size, float delta, const float* tsdf,
                  const float* weights) {
    TSDFVolume vol(Vec3i(dims[0], dims[1], dims[2]), Vec3f(size[0], size[1], size[2]), Mat3f::Identity());
    vol.setDelta(delta);
    std::memcpy(vol.ptrTsdf(), tsdf, sizeof(float) * vol.gridSize());
    std::memcpy(vol.ptrTsdfWeights(), weights, sizeof(float) * vol.gridSize());
    return vol.save(path) ? 0 : 1;
}

// TSDFVolume::load (src/TSDFVolume.cpp:315-341): dims, size, voxel size and delta as loaded, and the
// values and weights (cap voxels at most).
long ref_tsdf_load(const char* path, int* dims, float* size, float* voxel_size, float* delta, float* tsdf,
                   float* weights, long cap) {
    TSDFVolume vol(Vec3i(1, 1, 1), Vec3f(1.f, 1.f, 1.f), Mat3f::Identity());
    if (!vol.load(path)) return -1;
    Vec3i d = vol.dimensions();
    Vec3f sz = vol.size(), vs = vol.voxelSize();
    for (int c = 0; c < 3; ++c) {
        dims[c] = d[c];
        size[c] = sz[c];
        voxel_size[c] = vs[c];
    }
    *delta = vol.delta();
    const long n = (long)vol.gridSize() < cap ? (long)vol.gridSize() : cap;
    std::memcpy(tsdf, vol.ptrTsdf(), sizeof(float) * n);
    std::memcpy(weights, vol.ptrTsdfWeights(), sizeof(float) * n);
    return (long)vol.gridSize();
}

}  // extern "C"
