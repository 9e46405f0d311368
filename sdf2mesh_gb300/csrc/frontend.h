// frontend.h -- the shader front end of sdf2mesh_gb300: `.sdf3d` WGSL and
// GLSL SDF sources are preprocessed, parsed, type-checked and lowered to CUDA
// C that NVRTC compiles together with the dual-contouring kernels.
//
// It replaces, for this project, the reference's shader path:
//   src/shader.rs:44-67, 159-203   (`use` / `include` expansion of .sdf3d files)
//   src/shader.rs:73-104           (GLSL fragment shader -> sdf3d wrapper)
//   src/shadertoy.rs:169-194       (naga GLSL -> WGSL; here GLSL is parsed directly)
//   src/shadertoy.rs:196-352       (WGSL text surgery helpers)
#pragma once
#include <string>
#include <vector>

namespace s2m {

enum class Lang { WGSL = 0, GLSL = 1 };

struct FrontendResult {
  bool ok = false;
  int status = 0;                     // S2M_* status code on failure
  std::string error;                  // "line N: message"
  std::vector<std::string> warnings;
  std::string cuda;                   // lowered CUDA C (needs s2m_prelude.cuh)
  double fp32_ops = 0;                // algorithmic FP32 ops per sdf3d call
  double sfu_ops = 0;                 // sqrt / div / transcendental ops per call
  bool ops_exact = true;              // false when a loop bound was not static
  double run_fp32_ops = 0;            // per point in runs of 4 sharing x, y (0: no run form)
  double run_sfu_ops = 0;
  int prune_combinators = 0;          // combinators the tile-pruning form can skip (0: no such form)
  int prune_words = 0;                // 32-bit activity words per tile
};

// Built-in WGSL modules selected by `use <name>;` (shader.rs:12-20, 50-62).
// Returns nullptr for unknown names (which the reference drops silently).
const char *builtin_module_source(const std::string &name);

// Expand `use X;` and `include "f";` lines of a .sdf3d file
// (shader.rs:159-203).  `log` receives the messages the reference logs.
bool preprocess_sdf3d_file(const std::string &path, std::string &out, std::string &err,
                           std::vector<std::string> *log);
// The same on in-memory text; includes are resolved relative to the working
// directory as in the reference, then relative to `base_dir`.
std::string preprocess_sdf3d_text(const std::string &src, const std::string &self_path,
                                  const std::string &base_dir, std::vector<std::string> *log);

// ShaderToy-style code wrapped into a GLSL fragment shader (shadertoy.rs:154-166).
std::string shadertoy_wrap(const std::string &code);

// Parse, check and lower a complete source.  For GLSL, `sdf_name` is the
// function with signature float(vec3) (shader.rs:89-98); a wrapper `sdf3d`
// is generated when the source has none.
FrontendResult translate(const std::string &source, Lang lang, const std::string &sdf_name);

// The batch interpreter's postfix CSG program (opcodes S2M_CSG_*) of a
// preprocessed .sdf3d source whose sdf3d is one expression over the
// library's primitives and operators with constant arguments; false (and
// why) for any other source.
bool csg_from_source(const std::string &source, std::vector<float> &prog, std::string &why);

// Text helpers with the behaviour of shadertoy.rs:248-352.
bool wgsl_remove_function(const std::string &wgsl, const std::string &function_name,
                          std::string &out);
bool wgsl_has_function(const std::string &wgsl, const std::string &function_name);
bool wgsl_rename_function(const std::string &wgsl, const std::string &old_name,
                          const std::string &new_name, std::string &out);

}  // namespace s2m
