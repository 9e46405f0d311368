// mesh_io.cpp -- parallel ASCII STL / PLY writers.  The text is the
// reference's (src/mesh.rs:8-48 STLWriter, :50-141 PLYWriter): floats as Rust
// `{}` prints them (shortest round-trip digits, never an exponent), so files
// compare byte for byte.  Chunks of the mesh are formatted on all host
// threads and written in order.
#include "mesh_io.h"

#include <fcntl.h>
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <charconv>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "../../include/sdf2mesh.h"

namespace s2m {

int format_f32(float v, char *out) {
  if (std::isnan(v)) { std::memcpy(out, "NaN", 4); return 3; }
  if (std::isinf(v)) {
    if (v < 0) { std::memcpy(out, "-inf", 5); return 4; }
    std::memcpy(out, "inf", 4);
    return 3;
  }
  char tmp[48];
  auto r = std::to_chars(tmp, tmp + sizeof tmp, std::fabs(v), std::chars_format::scientific);
  *r.ptr = 0;
  // tmp = d[.ddd]e[+-]XX
  char digits[32];
  int nd = 0;
  const char *p = tmp;
  while (*p && *p != 'e') {
    if (*p != '.') digits[nd++] = *p;
    ++p;
  }
  int ex = std::atoi(p + 1);
  int point = ex + 1;  // value = 0.d1d2.. * 10^point
  char *o = out;
  if (std::signbit(v)) *o++ = '-';
  if (nd == 1 && digits[0] == '0') {
    *o++ = '0';
  } else if (point <= 0) {
    *o++ = '0';
    *o++ = '.';
    for (int i = 0; i < -point; ++i) *o++ = '0';
    for (int i = 0; i < nd; ++i) *o++ = digits[i];
  } else if (point >= nd) {
    for (int i = 0; i < nd; ++i) *o++ = digits[i];
    for (int i = nd; i < point; ++i) *o++ = '0';
  } else {
    for (int i = 0; i < point; ++i) *o++ = digits[i];
    *o++ = '.';
    for (int i = point; i < nd; ++i) *o++ = digits[i];
  }
  *o = 0;
  return int(o - out);
}

namespace {

inline void put(std::string &s, const char *t) { s.append(t); }
inline void putf(std::string &s, float v) {
  char b[64];
  int n = format_f32(v, b);
  s.append(b, size_t(n));
}

template <class F>
bool parallel_write(FILE *fp, uint64_t n, F &&format_range) {
  unsigned nt = std::max(1u, std::min(64u, std::thread::hardware_concurrency()));
  const uint64_t chunk = 1u << 16;
  uint64_t nchunks = (n + chunk - 1) / chunk;
  for (uint64_t c0 = 0; c0 < nchunks; c0 += nt) {
    uint64_t c1 = std::min(nchunks, c0 + nt);
    std::vector<std::string> bufs(size_t(c1 - c0));
    std::vector<std::thread> th;
    for (uint64_t c = c0; c < c1; ++c)
      th.emplace_back([&, c] { format_range(bufs[size_t(c - c0)], c * chunk, std::min(n, (c + 1) * chunk)); });
    for (auto &t : th) t.join();
    for (auto &b : bufs)
      if (std::fwrite(b.data(), 1, b.size(), fp) != b.size()) return false;
  }
  return true;
}

}  // namespace

bool write_stl(const char *path, const float *pos, const uint32_t *tris, uint64_t ntris) {
  FILE *fp = std::fopen(path, "wb");
  if (!fp) return false;
  bool ok = std::fputs("solid\n", fp) >= 0;
  ok = ok && parallel_write(fp, ntris, [&](std::string &s, uint64_t a, uint64_t b) {
    s.reserve(size_t(b - a) * 160);
    for (uint64_t t = a; t < b; ++t) {
      const float *v0 = pos + 3 * size_t(tris[3 * t]);
      const float *v1 = pos + 3 * size_t(tris[3 * t + 1]);
      const float *v2 = pos + 3 * size_t(tris[3 * t + 2]);
      // lib.rs:181-185: (v2 - v0).cross(v1 - v0)
      float ux = v2[0] - v0[0], uy = v2[1] - v0[1], uz = v2[2] - v0[2];
      float wx = v1[0] - v0[0], wy = v1[1] - v0[1], wz = v1[2] - v0[2];
      float nx = uy * wz - uz * wy, ny = uz * wx - ux * wz, nz = ux * wy - uy * wx;
      put(s, "facet normal "); putf(s, nx); put(s, " "); putf(s, ny); put(s, " "); putf(s, nz);
      put(s, "\n\touter loop\n");
      for (const float *v : {v0, v1, v2}) {
        put(s, "\t\tvertex "); putf(s, v[0]); put(s, " "); putf(s, v[1]); put(s, " "); putf(s, v[2]); put(s, "\n");
      }
      put(s, "\tendloop\nendfacet\n");
    }
  });
  ok = ok && std::fputs("endsolid\n", fp) >= 0;
  return std::fclose(fp) == 0 && ok;
}

// Binary STL: an 80-byte header, the triangle count (u32), then 50 bytes per
// triangle -- the facet normal (v2 - v0) x (v1 - v0) as in lib.rs:181-185,
// the three vertices (12 little-endian f32) and a zero attribute word.  The
// file size is known up front, so every host thread formats its own ranges
// of triangles and writes them at their offsets (pwrite); nothing waits on
// another thread's text.
bool write_stl_binary(const char *path, const float *pos, const uint32_t *tris, uint64_t ntris) {
  if (ntris > 0xFFFFFFFFull) return false;
  const int fd = ::open(path, O_WRONLY | O_CREAT | O_TRUNC, 0644);
  if (fd < 0) return false;
  unsigned char head[84] = {0};
  static const char kTitle[] = "binary STL, sdf2mesh_gb300 dual contouring";
  std::memcpy(head, kTitle, sizeof kTitle - 1);
  const uint32_t n32 = uint32_t(ntris);
  for (int b = 0; b < 4; ++b) head[80 + b] = (unsigned char)((n32 >> (8 * b)) & 0xffu);
  bool ok = ::pwrite(fd, head, sizeof head, 0) == ssize_t(sizeof head);
  const uint64_t chunk = 1u << 16;
  const uint64_t nchunks = (ntris + chunk - 1) / chunk;
  std::atomic<uint64_t> next{0};
  std::atomic<bool> good{ok};
  auto put_f32 = [](unsigned char *o, float v) {
    uint32_t u;
    std::memcpy(&u, &v, 4);
    o[0] = (unsigned char)(u & 0xffu);
    o[1] = (unsigned char)((u >> 8) & 0xffu);
    o[2] = (unsigned char)((u >> 16) & 0xffu);
    o[3] = (unsigned char)(u >> 24);
  };
  auto worker = [&] {
    std::vector<unsigned char> buf(size_t(chunk) * 50);
    for (;;) {
      const uint64_t c = next.fetch_add(1);
      if (c >= nchunks || !good.load()) return;
      const uint64_t a = c * chunk, b = std::min(ntris, a + chunk);
      unsigned char *o = buf.data();
      for (uint64_t t = a; t < b; ++t, o += 50) {
        const float *v0 = pos + 3 * size_t(tris[3 * t]);
        const float *v1 = pos + 3 * size_t(tris[3 * t + 1]);
        const float *v2 = pos + 3 * size_t(tris[3 * t + 2]);
        const float ux = v2[0] - v0[0], uy = v2[1] - v0[1], uz = v2[2] - v0[2];
        const float wx = v1[0] - v0[0], wy = v1[1] - v0[1], wz = v1[2] - v0[2];
        const float n[3] = {uy * wz - uz * wy, uz * wx - ux * wz, ux * wy - uy * wx};
        for (int k = 0; k < 3; ++k) put_f32(o + 4 * k, n[k]);
        const float *vs[3] = {v0, v1, v2};
        for (int v = 0; v < 3; ++v)
          for (int k = 0; k < 3; ++k) put_f32(o + 12 + 12 * v + 4 * k, vs[v][k]);
        o[48] = o[49] = 0;
      }
      const size_t bytes = size_t(b - a) * 50;
      size_t done = 0;
      while (done < bytes) {
        const ssize_t w = ::pwrite(fd, buf.data() + done, bytes - done, off_t(84 + 50 * a + done));
        if (w <= 0) {
          good = false;
          return;
        }
        done += size_t(w);
      }
    }
  };
  const unsigned nt = std::max(1u, std::min(64u, std::thread::hardware_concurrency()));
  std::vector<std::thread> th;
  for (unsigned i = 0; i < std::min<uint64_t>(nt, std::max<uint64_t>(1, nchunks)); ++i) th.emplace_back(worker);
  for (auto &t : th) t.join();
  ok = good.load();
  return ::close(fd) == 0 && ok;
}

bool write_ply(const char *path, const float *pos, const float *nrm, uint64_t nverts, const uint32_t *tris,
               uint64_t ntris) {
  FILE *fp = std::fopen(path, "wb");
  if (!fp) return false;
  bool ok = std::fprintf(fp,
                         "ply\nformat ascii 1.0\ncomment written by rust-sdf\nelement vertex %llu\n"
                         "property float x\nproperty float y\nproperty float z\n"
                         "property float nx\nproperty float ny\nproperty float nz\n"
                         "element face %llu\nproperty list uchar int vertex_index\nend_header\n",
                         (unsigned long long)nverts, (unsigned long long)ntris) > 0;
  ok = ok && parallel_write(fp, nverts, [&](std::string &s, uint64_t a, uint64_t b) {
    s.reserve(size_t(b - a) * 80);
    for (uint64_t i = a; i < b; ++i) {
      putf(s, pos[3 * i]); put(s, " "); putf(s, pos[3 * i + 1]); put(s, " "); putf(s, pos[3 * i + 2]); put(s, " ");
      putf(s, nrm[3 * i]); put(s, " "); putf(s, nrm[3 * i + 1]); put(s, " "); putf(s, nrm[3 * i + 2]); put(s, "\n");
    }
  });
  ok = ok && parallel_write(fp, ntris, [&](std::string &s, uint64_t a, uint64_t b) {
    s.reserve(size_t(b - a) * 32);
    char num[16];
    for (uint64_t t = a; t < b; ++t) {
      put(s, "3");
      for (int k = 0; k < 3; ++k) {
        auto r = std::to_chars(num, num + sizeof num, tris[3 * t + k]);
        s.push_back(' ');
        s.append(num, size_t(r.ptr - num));
      }
      s.push_back('\n');
    }
  });
  return std::fclose(fp) == 0 && ok;
}

int write_mesh_file(const char *path, const float *pos, const float *nrm, uint64_t nverts, const uint32_t *tris,
                    uint64_t ntris, char *err, size_t errlen) {
  std::string p(path);
  size_t slash = p.find_last_of('/');
  size_t dot = p.find_last_of('.');
  std::string ext;
  if (dot != std::string::npos && (slash == std::string::npos || dot > slash + 1)) ext = p.substr(dot + 1);
  for (char &c : ext) c = char(std::toupper((unsigned char)c));
  bool ok;
  if (ext == "STL") ok = write_stl(path, pos, tris, ntris);
  else if (ext == "PLY") ok = write_ply(path, pos, nrm, nverts, tris, ntris);
  else {
    if (err && errlen) std::snprintf(err, errlen, "Unknown file extension: %s", ext.c_str());
    return S2M_E_INVALID;
  }
  if (!ok) {
    if (err && errlen) std::snprintf(err, errlen, "could not write %s", path);
    return S2M_E_IO;
  }
  return S2M_OK;
}

}  // namespace s2m
