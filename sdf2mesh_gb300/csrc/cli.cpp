// cli.cpp -- the `sdf2mesh` command line, a drop-in for the reference binary
// (src/bin/sdf2mesh/main.rs:95-137 flags, :139-175 parameters, :177-364 run),
// written over the C ABI of libsdf2mesh_gb300.so.
//
//   sdf2mesh (--sdf|-i FILE.sdf3d | --glsl FILE [--glsl-sdf NAME]) --mesh|-0 OUT.{stl,ply}
//            [--resolution|-r N (256)] [--bounds|-b B (2.0)] [--debug-wgsl FILE]
//            [--debug-cuda FILE] [--exact-resolution] [--no-slice-lag] [--fmad] [--binary-stl]
//
// As in the reference, a resolution that is not a power of two is rounded up
// (main.rs:141-148) and slices are emitted with the reference's one-slice lag
// (main.rs:324-355); --exact-resolution and --no-slice-lag turn those off.
// Errors exit non-zero where the reference panics.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <fstream>
#include <sstream>
#include <string>

#include "sdf2mesh.h"

namespace {

void log(const char *level, const std::string &msg) {
  auto now = std::chrono::system_clock::now().time_since_epoch();
  long long ns = (long long)std::chrono::duration_cast<std::chrono::nanoseconds>(now).count();
  std::time_t secs = std::time_t(ns / 1000000000LL);
  char buf[32];
  std::strftime(buf, sizeof buf, "%Y-%m-%dT%H:%M:%S", std::gmtime(&secs));
  std::fprintf(stderr, "[%s.%09lldZ %s sdf2mesh] %s\n", buf, ns % 1000000000LL, level, msg.c_str());
}

void usage() {
  std::fprintf(stderr,
               "Usage: sdf2mesh [OPTIONS] --mesh <MESH>\n\n"
               "Options:\n"
               "  -i, --sdf <SDF>                Input SDF file\n"
               "      --shadertoy-id <ID>        Input ShaderToy shader ID (unavailable: no network)\n"
               "      --shadertoy-sdf <NAME>     ShaderToy SDF name [default: sdf]\n"
               "      --shadertoy-file <FILE>    ShaderToy-style code from a file (inputs are zero)\n"
               "      --glsl <GLSL>              Input GLSL fragment shader\n"
               "      --glsl-sdf <NAME>          GLSL SDF name [default: sdf]\n"
               "  -0, --mesh <MESH>              Output mesh file (supports STL and PLY output)\n"
               "      --debug-wgsl <FILE>        Output WGSL file for debugging\n"
               "      --debug-cuda <FILE>        Output the lowered CUDA C for debugging\n"
               "      --debug-png <PREFIX>       Accepted and ignored (no per-slice images)\n"
               "  -r, --resolution <N>           Grid resolution. Default: 256\n"
               "  -b, --bounds <B>               Size of bounding box. Default: 2\n"
               "      --exact-resolution         Do not round the resolution to a power of two\n"
               "      --no-slice-lag             Emit every slice at its own index\n"
               "      --fmad                     Allow FMA contraction in the SDF (faster, not bit-exact)\n"
               "      --binary-stl               Write the STL in binary form (50 bytes per facet)\n"
               "  -h, --help                     Print help\n");
}

bool read_text(const std::string &path, std::string &out) {
  std::ifstream f(path, std::ios::binary);
  if (!f) return false;
  std::ostringstream ss;
  ss << f.rdbuf();
  out = ss.str();
  return true;
}

}  // namespace

int main(int argc, char **argv) {
  std::string sdf, glsl, glsl_sdf = "sdf", mesh, debug_wgsl, debug_cuda, shadertoy_id, shadertoy_file,
      shadertoy_sdf = "sdf";
  unsigned long resolution = 256;
  double bounds = 2.0;
  bool exact_res = false, no_lag = false, fmad = false, binary_stl = false;
  for (int i = 1; i < argc; ++i) {
    std::string a = argv[i];
    std::string v;
    auto eq = a.find('=');
    if (a.rfind("--", 0) == 0 && eq != std::string::npos) {
      v = a.substr(eq + 1);
      a = a.substr(0, eq);
    }
    auto value = [&](std::string &dst) -> bool {
      if (!v.empty()) {
        dst = v;
        return true;
      }
      if (i + 1 >= argc) {
        std::fprintf(stderr, "error: a value is required for '%s'\n", a.c_str());
        return false;
      }
      dst = argv[++i];
      return true;
    };
    std::string tmp;
    if (a == "-h" || a == "--help") {
      usage();
      return 0;
    } else if (a == "-i" || a == "--sdf") {
      if (!value(sdf)) return 2;
    } else if (a == "--glsl") {
      if (!value(glsl)) return 2;
    } else if (a == "--glsl-sdf") {
      if (!value(glsl_sdf)) return 2;
    } else if (a == "--shadertoy-id") {
      if (!value(shadertoy_id)) return 2;
    } else if (a == "--shadertoy-sdf") {
      if (!value(shadertoy_sdf)) return 2;
    } else if (a == "--shadertoy-file") {
      if (!value(shadertoy_file)) return 2;
    } else if (a == "--debug-png") {
      if (!value(tmp)) return 2;
    } else if (a == "-0" || a == "--mesh") {
      if (!value(mesh)) return 2;
    } else if (a == "--debug-wgsl") {
      if (!value(debug_wgsl)) return 2;
    } else if (a == "--debug-cuda") {
      if (!value(debug_cuda)) return 2;
    } else if (a == "-r" || a == "--resolution") {
      if (!value(tmp)) return 2;
      char *end = nullptr;
      resolution = std::strtoul(tmp.c_str(), &end, 10);
      if (!end || *end || tmp.empty() || tmp[0] == '-') {
        std::fprintf(stderr, "error: invalid value '%s' for '--resolution <N>'\n", tmp.c_str());
        return 2;
      }
    } else if (a == "-b" || a == "--bounds") {
      if (!value(tmp)) return 2;
      char *end = nullptr;
      bounds = std::strtod(tmp.c_str(), &end);
      if (!end || *end || tmp.empty()) {
        std::fprintf(stderr, "error: invalid value '%s' for '--bounds <B>'\n", tmp.c_str());
        return 2;
      }
    } else if (a == "--exact-resolution") {
      exact_res = true;
    } else if (a == "--no-slice-lag") {
      no_lag = true;
    } else if (a == "--fmad") {
      fmad = true;
    } else if (a == "--binary-stl") {
      binary_stl = true;
    } else {
      std::fprintf(stderr, "error: unexpected argument '%s'\n", a.c_str());
      usage();
      return 2;
    }
  }
  if (mesh.empty()) {
    std::fprintf(stderr, "error: the following required arguments were not provided:\n  --mesh <MESH>\n");
    return 2;
  }
  if (!shadertoy_id.empty()) {
    log("ERROR", "ShaderToy input needs network access, which this build does not use");
    return 1;
  }
  char err[16384] = {0};
  std::string source;
  int lang = S2M_LANG_WGSL;
  if (!sdf.empty()) {
    log("INFO", "Reading SDF from " + sdf + "...");
    char *pre = nullptr;
    if (s2m_preprocess_file(sdf.c_str(), &pre, err, sizeof err) != S2M_OK) {
      log("ERROR", err);
      return 1;
    }
    source = pre;
    s2m_free_string(pre);
  } else if (!shadertoy_file.empty()) {
    log("INFO", "Reading SDF from ShaderToy-style file " + shadertoy_file + "...");
    if (!read_text(shadertoy_file, source)) {
      log("ERROR", "could not read " + shadertoy_file);
      return 1;
    }
    lang = S2M_LANG_SHADERTOY;
    glsl_sdf = shadertoy_sdf;
  } else if (!glsl.empty()) {
    log("INFO", "Reading SDF from GLSL fragment shader " + glsl + "...");
    if (!read_text(glsl, source)) {
      log("ERROR", "could not read " + glsl);
      return 1;
    }
    lang = S2M_LANG_GLSL;
  } else {
    log("ERROR", "no SDF given (--sdf or --glsl)");
    return 2;
  }
  if (!debug_wgsl.empty()) {
    std::ofstream f(debug_wgsl, std::ios::binary);
    f << source;
  }

  s2m_sdf *h = nullptr;
  int rc = s2m_compile(source.c_str(), lang, glsl_sdf.c_str(), fmad ? S2M_COMPILE_FMAD : 0u, &h, err, sizeof err);
  if (rc != S2M_OK) {
    log("ERROR", std::string(s2m_status_string(rc)) + ": " + err);
    return 1;
  }
  if (!debug_cuda.empty()) {
    std::ofstream f(debug_cuda, std::ios::binary);
    f << s2m_sdf_cuda_source(h);
  }
  log("INFO", "SDF compiled for sm_103a.");

  s2m_params p;
  std::memset(&p, 0, sizeof p);
  p.resolution = uint32_t(resolution);
  p.bounds = float(bounds);
  p.eps = 1e-4f;
  p.flags = (exact_res ? 0u : S2M_JOB_POW2_ROUNDING) | (no_lag ? 0u : S2M_JOB_SLICE_LAG);
  unsigned long rounded = resolution;
  if (!exact_res && __builtin_popcountl(resolution) > 1) {
    rounded = 2ul << (63 - __builtin_clzl(resolution));
    log("WARN", "Resolution should be a power of 2 (actual resolution : " + std::to_string(rounded) + ")");
  }
  s2m_mesh *m = nullptr;
  auto t0 = std::chrono::steady_clock::now();
  rc = s2m_mesh_create(h, &p, nullptr, &m, err, sizeof err);
  if (rc != S2M_OK) {
    log("ERROR", std::string(s2m_status_string(rc)) + ": " + err);
    s2m_sdf_free(h);
    return 1;
  }
  double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  s2m_mesh_info info;
  s2m_mesh_get_info(m, &info);
  log("INFO", "Mesh has " + std::to_string(info.nverts) + " vertices.");
  if (info.invalid_quads)
    log("WARN", std::to_string(info.invalid_quads) + " invalid quads. Mesh will not be water-tight!");
  char line[256];
  std::snprintf(line, sizeof line, "Meshed %u^3 cells in %.3f s (%.2f Gvoxels/s)", info.resolution, secs,
                double(info.cells) / secs / 1e9);
  log("INFO", line);
  rc = binary_stl ? s2m_mesh_write_stl_binary(m, mesh.c_str(), err, sizeof err)
                  : s2m_mesh_write(m, mesh.c_str(), err, sizeof err);
  int status = 0;
  if (rc != S2M_OK) {
    log("ERROR", std::string("Could not write mesh to ") + mesh + ": " + err);
    status = 1;
  } else {
    log("INFO", "Mesh written to " + mesh);
  }
  s2m_mesh_free(m);
  s2m_sdf_free(h);
  return status;
}
