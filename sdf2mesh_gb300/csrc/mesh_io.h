// mesh_io.h -- ASCII STL / PLY writers with the reference's text format
// (src/mesh.rs:8-141, 167-210): Rust `{}` float text, facet normal
// (v2 - v0) x (v1 - v0) unnormalised, writer chosen by extension.
#pragma once
#include <cstddef>
#include <cstdint>

namespace s2m {
// Rust `{}` Display of an f32 into buf (>= 64 bytes); returns the length.
int format_f32(float v, char *buf);
bool write_stl(const char *path, const float *pos, const uint32_t *tris, uint64_t ntris);
// Binary STL (not in the reference, whose ASCII files run to GBs at 2048^3,
// README.md:96): same facets and normals, written from all host threads.
bool write_stl_binary(const char *path, const float *pos, const uint32_t *tris, uint64_t ntris);
bool write_ply(const char *path, const float *pos, const float *nrm, uint64_t nverts, const uint32_t *tris,
               uint64_t ntris);
// mesh.rs:182-196: "STL" / "PLY" by case-insensitive extension.
int write_mesh_file(const char *path, const float *pos, const float *nrm, uint64_t nverts, const uint32_t *tris,
                    uint64_t ntris, char *err, size_t errlen);
}  // namespace s2m
