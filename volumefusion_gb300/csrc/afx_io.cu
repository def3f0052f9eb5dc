// afx_io.cu -- on-disk formats of the reference: the ASCII PLY mesh (Mesh::savePly) and the binary
// TSDF volume (TSDFVolume::save / load).  Host code; the session helpers that copy device state in
// and out are in afx_fusion.cu.
//
// PLY (src/Mesh.cpp:23-64): header "ply / format ascii 1.0 / element vertex N / property float x y z
// / property uchar red green blue / element face F / property list uchar int vertex_indices /
// end_header", then one line "x y z r g b" per vertex and "3 a b c" per face.  Coordinates are
// printed the way a default std::ostream prints a float (6 significant digits, %g style).
//
// TSDF volume (src/TSDFVolume.cpp:315-361), little-endian, no padding:
//   int32 dims[3]
//   24 bytes written from TSDFVolume::m_size: the volume size (3 x float) followed by the member
//        after it, m_voxelSize (3 x float) -- the reference writes sizeof(double) * 3 from a Vec3f
//   float delta
//   float tsdf[S], float weights[S]
//   uint8 colorR[S], colorG[S], colorB[S], float weightsColor[S]
// The fusion path has no colour: colours are written as the reference's uninitialised default (127)
// with colour weights 0, and ignored on load.
#include <cstdio>
#include <cstring>
#include <vector>

#include "afx_internal.h"

namespace {

struct File {
    FILE* f = nullptr;
    File(const char* path, const char* mode) : f(std::fopen(path, mode)) {}
    ~File() {
        if (f) std::fclose(f);
    }
};

bool write_all(FILE* f, const void* p, size_t n) { return n == 0 || std::fwrite(p, 1, n, f) == n; }
bool read_all(FILE* f, void* p, size_t n) { return n == 0 || std::fread(p, 1, n, f) == n; }

constexpr size_t kHeaderBytes = 12 + 24 + 4;

}  // namespace

extern "C" {

int afx_save_ply(const char* path, const float* vertices, long n_vertices, const unsigned char* colors,
                 const int* faces, long n_faces) {
    if (!path || n_vertices < 0 || n_faces < 0 || (n_vertices && !vertices) || (n_faces && !faces))
        return AFX_ERR_INVALID_ARGUMENT;
    if (n_vertices == 0) return AFX_ERR_INVALID_ARGUMENT;  // savePly refuses an empty vertex cloud
    File out(path, "w");
    if (!out.f) return AFX_ERR_IO;
    std::fprintf(out.f,
                 "ply\nformat ascii 1.0\nelement vertex %ld\nproperty float x\nproperty float y\nproperty float z\n"
                 "property uchar red\nproperty uchar green\nproperty uchar blue\nelement face %d\n"
                 "property list uchar int vertex_indices\nend_header\n",
                 n_vertices, (int)n_faces);
    for (long i = 0; i < n_vertices; ++i) {
        const int r = colors ? colors[3 * i] : 0, g = colors ? colors[3 * i + 1] : 0, b = colors ? colors[3 * i + 2] : 0;
        std::fprintf(out.f, "%g %g %g %d %d %d\n", (double)vertices[3 * i], (double)vertices[3 * i + 1],
                     (double)vertices[3 * i + 2], r, g, b);
    }
    for (long i = 0; i < n_faces; ++i)
        std::fprintf(out.f, "3 %d %d %d\n", faces[3 * i], faces[3 * i + 1], faces[3 * i + 2]);
    return std::ferror(out.f) ? AFX_ERR_IO : AFX_OK;
}

int afx_tsdf_save(const char* path, const int dims[3], const float volume_size[3], const float voxel_size[3],
                  float delta, const float* tsdf, const float* weights) {
    if (!path || !dims || !volume_size || !voxel_size || !tsdf || !weights) return AFX_ERR_INVALID_ARGUMENT;
    if (dims[0] <= 0 || dims[1] <= 0 || dims[2] <= 0) return AFX_ERR_INVALID_ARGUMENT;
    const size_t S = (size_t)dims[0] * dims[1] * dims[2];
    File out(path, "wb");
    if (!out.f) return AFX_ERR_IO;
    bool ok = write_all(out.f, dims, 12) && write_all(out.f, volume_size, 12) && write_all(out.f, voxel_size, 12) &&
              write_all(out.f, &delta, 4) && write_all(out.f, tsdf, 4 * S) && write_all(out.f, weights, 4 * S);
    std::vector<unsigned char> colour(S, 127);
    for (int c = 0; c < 3 && ok; ++c) ok = write_all(out.f, colour.data(), S);
    std::vector<float> zero(S, 0.f);
    ok = ok && write_all(out.f, zero.data(), 4 * S);
    return ok ? AFX_OK : AFX_ERR_IO;
}

int afx_tsdf_load_header(const char* path, int dims[3], float volume_size[3], float voxel_size[3], float* delta) {
    if (!path || !dims) return AFX_ERR_INVALID_ARGUMENT;
    File in(path, "rb");
    if (!in.f) return AFX_ERR_IO;
    unsigned char h[kHeaderBytes];
    if (!read_all(in.f, h, sizeof h)) return AFX_ERR_IO;
    std::memcpy(dims, h, 12);
    if (volume_size) std::memcpy(volume_size, h + 12, 12);
    if (voxel_size) std::memcpy(voxel_size, h + 24, 12);
    if (delta) std::memcpy(delta, h + 36, 4);
    if (dims[0] <= 0 || dims[1] <= 0 || dims[2] <= 0) return AFX_ERR_IO;
    return AFX_OK;
}

int afx_tsdf_load(const char* path, float* tsdf, float* weights, long n_voxels) {
    if (!path || !tsdf || !weights || n_voxels <= 0) return AFX_ERR_INVALID_ARGUMENT;
    int dims[3];
    int rc = afx_tsdf_load_header(path, dims, nullptr, nullptr, nullptr);
    if (rc) return rc;
    if ((long)dims[0] * dims[1] * dims[2] != n_voxels) return AFX_ERR_INVALID_ARGUMENT;
    File in(path, "rb");
    if (!in.f || std::fseek(in.f, (long)kHeaderBytes, SEEK_SET) != 0) return AFX_ERR_IO;
    const size_t S = (size_t)n_voxels;
    return read_all(in.f, tsdf, 4 * S) && read_all(in.f, weights, 4 * S) ? AFX_OK : AFX_ERR_IO;
}

}  // extern "C"
