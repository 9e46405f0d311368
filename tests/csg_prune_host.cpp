// Host build of the batch engine's CSG interpreter (s2m_csg.cuh) for the
// pruning tests: the interval pass of a tile and the point interpreter, full
// and pruned, compiled by the host compiler without FMA contraction.
#include <cstdint>

#include "../sdf2mesh_gb300/csrc/s2m_prelude.cuh"
#include "../sdf2mesh_gb300/csrc/s2m_csg.cuh"

extern "C" {

int csg_code_words() { return S2_CSG_CODE_WORDS; }

// box = {x.lo, x.hi, y.lo, y.hi, z.lo, z.hi}; root = {lo, hi}
int csg_tile(const float *prog, int len, const float *box, unsigned *codes, float *root) {
  s2i X, Y, Z, r;
  X.lo = box[0]; X.hi = box[1];
  Y.lo = box[2]; Y.hi = box[3];
  Z.lo = box[4]; Z.hi = box[5];
  const int ok = s2c_tile(prog, len, X, Y, Z, codes, &r);
  root[0] = r.lo;
  root[1] = r.hi;
  return ok;
}

// Runs of 4 points (x, y, z0 .. z3): xyz holds n runs of 6 floats (x, y, z0,
// z1, z2, z3); out gets 4 values per run.  codes == nullptr: the full program.
void csg_eval4(const float *prog, int len, const float *xyz, int n, const unsigned *codes, float *out) {
  const S2CsgSdf f{prog, len};
  for (int r = 0; r < n; ++r) {
    const float *p = xyz + 6 * r;
    if (codes) f.eval_run_pruned<4>(p[0], p[1], p + 2, out + 4 * r, codes);
    else f.eval_run<4>(p[0], p[1], p + 2, out + 4 * r);
  }
}

}  // extern "C"
