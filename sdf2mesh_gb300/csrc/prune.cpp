// prune.cpp -- segment analysis and code generation for tile pruning (see
// prune.h for the idea and the soundness argument).
//
// Segments.  Operand `side` (0 = a, 1 = b) of an enabled combinator c opens
// segment (c, side).  A node belongs to the innermost segment through which
// every path from it to the result passes: the post-dominating combinator
// operand edge.  Nodes are visited from the result backwards, and a node's
// segment is the lowest common ancestor, in the segment tree, of what each
// of its uses requires.  A node in segment S is needed only when S is
// active, so the point code evaluates S's nodes inside one `if` on S's bit.
//
// Generated code:
//   s2m_user_sdf_tile(X, Y, Z, m, fp, sfu, root)   intervals of the tile's
//       coordinates -> activity bits m[] (2 per combinator: operand a needed,
//       operand b needed), the FP32 / SFU operations per point that remain,
//       and the interval of the SDF's value;
//   s2m_user_sdf_tile_in(X, Y, Z, pm, m, ...)  the same for a tile inside a
//       box whose bits pm are known: only pm's active segments are evaluated;
//   s2m_user_sdf_pruned(x, y, z, m)          the point value, evaluating only
//       the active segments; bit-identical to s2m_user_sdf.
#include "prune.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <sstream>

namespace s2m {
namespace {

// A combinator side is worth a branch when its subgraph costs at least this
// (FP32 ops + 4 per SFU op).
constexpr double kMinSkipWeight = 6.0;
constexpr int kMaxCombinators = 256;

std::string lit(float v) {
  if (std::isnan(v)) return "__int_as_float(0x7fc00000)";
  if (std::isinf(v)) return v > 0 ? "__int_as_float(0x7f800000)" : "__int_as_float(0xff800000)";
  char b[64];
  std::snprintf(b, sizeof b, "%af", double(v));
  return std::string("(") + b + ")";
}

bool is_comb(POp op) {
  return op == POp::Min || op == POp::Max || op == POp::SmoothUnion || op == POp::SmoothIntersection ||
         op == POp::SmoothSubtraction;
}

bool is_leaf(POp op) { return op == POp::X || op == POp::Y || op == POp::Z || op == POp::Const; }

struct OpCost {
  double fp = 0, sfu = 0;
  double weight() const { return fp + 4.0 * sfu; }
};

OpCost node_cost(POp op) {
  switch (op) {
    // negation is an operand modifier on the GPU, free as in the frontend's count
    case POp::X: case POp::Y: case POp::Z: case POp::Const: case POp::Neg: return {0, 0};
    case POp::Add: case POp::Sub: case POp::Mul: case POp::Abs: case POp::Floor: case POp::Ceil:
    case POp::Min: case POp::Max:
      return {1, 0};
    case POp::Clamp: case POp::Saturate: return {2, 0};
    case POp::Mix: return {4, 0};
    case POp::Div: case POp::Sqrt: case POp::Sin: case POp::Cos: case POp::Exp: case POp::Log: case POp::Pow:
    case POp::Atan2:
      return {0, 1};
    case POp::SmoothUnion: case POp::SmoothIntersection: case POp::SmoothSubtraction: return {13, 1};
  }
  return {0, 0};
}

class Pruner {
 public:
  explicit Pruner(const PruneIR &ir) : ir_(ir), n_(int(ir.nodes.size())) {}

  PruneCode run() {
    PruneCode pc;
    if (ir_.root < 0 || ir_.root >= n_) return pc;
    mark_live();
    // 1. every combinator enabled; 2. keep those with a side worth skipping
    // (With no combinator worth a branch the form is still emitted: the
    // tile's value interval alone decides the tiles far from the surface.)
    std::vector<int> cand;
    for (int v = 0; v < n_; ++v)
      if (live_[v] && is_comb(ir_.nodes[size_t(v)].op)) cand.push_back(v);
    set_enabled(cand);
    owners();
    std::vector<double> sub = subtree_weights();
    std::vector<std::pair<double, int>> keep;
    for (size_t ci = 0; ci < combs_.size(); ++ci) {
      double w = std::max(sub[size_t(seg(int(ci), 0))], sub[size_t(seg(int(ci), 1))]);
      if (w >= kMinSkipWeight) keep.push_back({w, combs_[ci]});
    }
    if (int(keep.size()) > kMaxCombinators) {
      std::stable_sort(keep.begin(), keep.end(), [](auto &x, auto &y) { return x.first > y.first; });
      keep.resize(size_t(kMaxCombinators));
    }
    std::vector<int> en;
    for (auto &k : keep) en.push_back(k.second);
    std::sort(en.begin(), en.end());
    set_enabled(en);
    owners();
    pc.combinators = int(combs_.size());
    pc.words = std::max(1, (2 * pc.combinators + 31) / 32);
    std::ostringstream o;
    o << "// tile pruning: " << pc.combinators << " combinators, " << pc.words << " words of activity bits\n";
    o << "#define S2M_HAS_PRUNE 1\n#define S2M_PRUNE_WORDS " << pc.words << "\n";
    var_.assign(size_t(n_), 0);
    for (int v = 0; v < n_; ++v) {
      const PNode &p = nd(v);
      var_[size_t(v)] = p.op == POp::Z || (p.a >= 0 && var_[size_t(p.a)]) || (p.b >= 0 && var_[size_t(p.b)]) ||
                        (p.c >= 0 && var_[size_t(p.c)]);
    }
    emit_tile(o, pc.words, false);
    emit_tile(o, pc.words, true);
    run4_ = false;
    emit_point(o);
    run4_ = true;
    emit_point(o);
    pc.cuda = o.str();
    pc.ok = true;
    return pc;
  }

 private:
  const PruneIR &ir_;
  int n_;
  std::vector<char> live_;
  std::vector<std::vector<std::pair<int, int>>> uses_;
  std::vector<int> comb_of_;  // node -> enabled combinator index, or -1
  std::vector<int> combs_;    // enabled combinator nodes, ascending
  std::vector<int> owner_;    // node -> segment
  std::vector<int> sparent_, sdepth_;
  std::vector<char> var_;  // depends on z (one value per point of a run of 4)
  bool run4_ = false;      // emitting the run-of-4 form

  static int seg(int ci, int side) { return 1 + 2 * ci + side; }
  static bool is_smooth(POp op) {
    return op == POp::SmoothUnion || op == POp::SmoothIntersection || op == POp::SmoothSubtraction;
  }
  const PNode &nd(int v) const { return ir_.nodes[size_t(v)]; }

  void mark_live() {
    live_.assign(size_t(n_), 0);
    uses_.assign(size_t(n_), {});
    live_[size_t(ir_.root)] = 1;
    for (int v = n_ - 1; v >= 0; --v) {
      if (!live_[size_t(v)]) continue;
      const PNode &p = nd(v);
      const int args[3] = {p.a, p.b, p.c};
      for (int i = 0; i < 3; ++i)
        if (args[i] >= 0) {
          live_[size_t(args[i])] = 1;
          uses_[size_t(args[i])].push_back({v, i});
        }
    }
  }

  void set_enabled(const std::vector<int> &en) {
    combs_ = en;
    comb_of_.assign(size_t(n_), -1);
    for (size_t i = 0; i < en.size(); ++i) comb_of_[size_t(en[i])] = int(i);
  }

  int lca(int a, int b) const {
    while (sdepth_[size_t(a)] > sdepth_[size_t(b)]) a = sparent_[size_t(a)];
    while (sdepth_[size_t(b)] > sdepth_[size_t(a)]) b = sparent_[size_t(b)];
    while (a != b) {
      a = sparent_[size_t(a)];
      b = sparent_[size_t(b)];
    }
    return a;
  }

  void owners() {
    const size_t ns = 1 + 2 * combs_.size();
    sparent_.assign(ns, -1);
    sdepth_.assign(ns, 0);
    owner_.assign(size_t(n_), -1);
    for (int v = n_ - 1; v >= 0; --v) {
      if (!live_[size_t(v)]) continue;
      int o = -1;
      if (v == ir_.root) o = 0;
      for (auto &[u, pos] : uses_[size_t(v)]) {
        const int cu = comb_of_[size_t(u)];
        const int want = (cu >= 0 && pos < 2) ? seg(cu, pos) : owner_[size_t(u)];
        o = o < 0 ? want : lca(o, want);
      }
      owner_[size_t(v)] = o;
      const int cv = comb_of_[size_t(v)];
      if (cv >= 0)
        for (int side = 0; side < 2; ++side) {
          sparent_[size_t(seg(cv, side))] = o;
          sdepth_[size_t(seg(cv, side))] = sdepth_[size_t(o)] + 1;
        }
    }
  }

  // Weight of every segment including the segments nested in it.
  std::vector<double> subtree_weights() const {
    const size_t ns = sparent_.size();
    std::vector<double> w(ns, 0.0);
    for (int v = 0; v < n_; ++v)
      if (live_[size_t(v)] && !is_leaf(nd(v).op)) w[size_t(owner_[size_t(v)])] += node_cost(nd(v).op).weight();
    std::vector<int> order(ns);
    for (size_t i = 0; i < ns; ++i) order[i] = int(i);
    std::sort(order.begin(), order.end(), [&](int a, int b) { return sdepth_[size_t(a)] > sdepth_[size_t(b)]; });
    for (int s : order)
      if (sparent_[size_t(s)] >= 0) w[size_t(sparent_[size_t(s)])] += w[size_t(s)];
    return w;
  }

  std::string val(int v) const {
    const PNode &p = nd(v);
    switch (p.op) {
      case POp::X: return "x";
      case POp::Y: return "y";
      case POp::Z: return "z";
      case POp::Const: return lit(p.k);
      default: return "v" + std::to_string(v);
    }
  }

  std::string ival(int v) const {
    const PNode &p = nd(v);
    switch (p.op) {
      case POp::X: return "X";
      case POp::Y: return "Y";
      case POp::Z: return "Z";
      case POp::Const: return "s2i_pt(" + lit(p.k) + ")";
      default: return "i" + std::to_string(v);
    }
  }

  // The pruned code calls the out-of-line smooth operators.
  std::string call_sfx() const { return "_call"; }

  // Point expression of a node (combinators: their full arithmetic).  In the
  // run-of-4 form a node that varies with z is an s2x4 and its builtins are
  // the lane-wise s2r_ forms (the same operations per lane).
  std::string expr(int v) const {
    const PNode &p = nd(v);
    if (run4_ && var_[size_t(v)] &&
        (p.op == POp::SmoothUnion || p.op == POp::SmoothIntersection || p.op == POp::SmoothSubtraction)) {
      const char *f = p.op == POp::SmoothUnion ? "s2r_op_smooth_union_call"
                      : p.op == POp::SmoothIntersection ? "s2r_op_smooth_intersection_call"
                                                        : "s2r_op_smooth_subtraction_call";
      return std::string(f) + "(" + as_var(p.a, true) + ", " + as_var(p.b, true) + ", " + as_var(p.c, true) + ")";
    }
    std::string e = expr_scalar(v);
    if (run4_ && var_[size_t(v)] && e.compare(0, 3, "s2_") == 0) e = "s2r_" + e.substr(3);
    return e;
  }
  std::string expr_scalar(int v) const {
    const PNode &p = nd(v);
    const std::string A = p.a >= 0 ? val(p.a) : "", B = p.b >= 0 ? val(p.b) : "", C = p.c >= 0 ? val(p.c) : "";
    switch (p.op) {
      case POp::Neg: return "(-" + A + ")";
      case POp::Add: return "(" + A + " + " + B + ")";
      case POp::Sub: return "(" + A + " - " + B + ")";
      case POp::Mul: return "(" + A + " * " + B + ")";
      case POp::Div: return "(" + A + " / " + B + ")";
      case POp::Abs: return "s2_abs(" + A + ")";
      case POp::Floor: return "s2_floor(" + A + ")";
      case POp::Ceil: return "s2_ceil(" + A + ")";
      case POp::Sqrt: return "s2_sqrt(" + A + ")";
      case POp::Min: return "s2_min(" + A + ", " + B + ")";
      case POp::Max: return "s2_max(" + A + ", " + B + ")";
      case POp::Clamp: return "s2_clamp(" + A + ", " + B + ", " + C + ")";
      case POp::Saturate: return "s2_saturate(" + A + ")";
      case POp::Mix: return "s2_mix(" + A + ", " + B + ", " + C + ")";
      case POp::Sin: return "s2_sin(" + A + ")";
      case POp::Cos: return "s2_cos(" + A + ")";
      case POp::Exp: return "s2_exp(" + A + ")";
      case POp::Log: return "s2_log(" + A + ")";
      case POp::Pow: return "s2_pow(" + A + ", " + B + ")";
      case POp::Atan2: return "s2_atan2(" + A + ", " + B + ")";
      case POp::SmoothUnion: return "s2_op_smooth_union" + call_sfx() + "(" + A + ", " + B + ", " + C + ")";
      case POp::SmoothIntersection: return "s2_op_smooth_intersection" + call_sfx() + "(" + A + ", " + B + ", " + C + ")";
      case POp::SmoothSubtraction: return "s2_op_smooth_subtraction" + call_sfx() + "(" + A + ", " + B + ", " + C + ")";
      default: return "";
    }
  }

  // Interval of a node; enabled combinators also store their decision in d<v>.
  std::string iexpr(int v) const {
    const PNode &p = nd(v);
    const std::string A = p.a >= 0 ? ival(p.a) : "", B = p.b >= 0 ? ival(p.b) : "", C = p.c >= 0 ? ival(p.c) : "";
    const std::string D = comb_of_[size_t(v)] >= 0 ? "&d" + std::to_string(v) : "nullptr";
    switch (p.op) {
      case POp::Neg: return "s2i_neg(" + A + ")";
      case POp::Add: return "s2i_add(" + A + ", " + B + ")";
      case POp::Sub: return "s2i_sub(" + A + ", " + B + ")";
      case POp::Mul: return p.a == p.b ? "s2i_sq(" + A + ")" : "s2i_mul(" + A + ", " + B + ")";
      case POp::Div: return "s2i_div(" + A + ", " + B + ")";
      case POp::Abs: return "s2i_abs(" + A + ")";
      case POp::Floor: return "s2i_floor(" + A + ")";
      case POp::Ceil: return "s2i_ceil(" + A + ")";
      case POp::Sqrt: return "s2i_sqrt(" + A + ")";
      case POp::Min: return "s2i_min_sel(" + A + ", " + B + ", " + D + ")";
      case POp::Max: return "s2i_max_sel(" + A + ", " + B + ", " + D + ")";
      case POp::Clamp: return "s2i_clamp(" + A + ", " + B + ", " + C + ")";
      case POp::Saturate: return "s2i_clamp(" + A + ", s2i_pt(0.0f), s2i_pt(1.0f))";
      case POp::Mix: return "s2i_mix(" + A + ", " + B + ", " + C + ")";
      case POp::Sin: case POp::Cos: return "s2i_unit(" + A + ")";
      case POp::Atan2: return "s2i_angle(" + A + ", " + B + ")";
      case POp::Exp: case POp::Log: case POp::Pow: return "s2i_unknown()";
      case POp::SmoothUnion: return "s2i_smooth_union_sel(" + A + ", " + B + ", " + C + ", " + D + ")";
      case POp::SmoothIntersection: return "s2i_smooth_intersection_sel(" + A + ", " + B + ", " + C + ", " + D + ")";
      case POp::SmoothSubtraction: return "s2i_smooth_subtraction_sel(" + A + ", " + B + ", " + C + ", " + D + ")";
      default: return ival(v);
    }
  }

  static std::string bit_test(int bit) {
    return "(m[" + std::to_string(bit >> 5) + "] & 0x" + [&] {
      char b[16];
      std::snprintf(b, sizeof b, "%xu", 1u << (bit & 31));
      return std::string(b);
    }() + ")";
  }

  // The tile function.  `guarded`: the form for a tile inside a larger box
  // whose activity bits pm are known.  A segment inactive there is inactive
  // in the tile, and a combinator with one operand inactive there keeps the
  // other one, so only the nodes of segments active in pm are evaluated.
  void emit_tile(std::ostringstream &o, int words, bool guarded) const {
    if (guarded)
      o << "S2I_FN void s2m_user_sdf_tile_in(const s2i X, const s2i Y, const s2i Z, const unsigned *pm, unsigned *m, "
           "float *fp, float *sfu, s2i *root)\n{\n";
    else
      o << "S2I_FN void s2m_user_sdf_tile(const s2i X, const s2i Y, const s2i Z, unsigned *m, float *fp, float *sfu, "
           "s2i *root)\n{\n";
    o << "  (void)X; (void)Y; (void)Z;\n";
    for (int v : combs_) o << "  int d" << v << " = 0;\n";
    if (!guarded) {
      for (int v = 0; v < n_; ++v) {
        if (!live_[size_t(v)] || is_leaf(nd(v).op)) continue;
        o << "  const s2i i" << v << " = " << iexpr(v) << ";\n";
      }
    } else {
      for (int v = 0; v < n_; ++v)
        if (live_[size_t(v)] && !is_leaf(nd(v).op)) o << "  s2i i" << v << ";\n";
      emit_tile_region(o, 0, regions(), "  ");
    }
    // activity: parents (larger node index) before the segments nested in them
    const size_t ns = 1 + 2 * combs_.size();
    o << "  const bool s0 = true;\n";
    for (int ci = int(combs_.size()) - 1; ci >= 0; --ci) {
      const int v = combs_[size_t(ci)];
      o << "  const bool s" << seg(ci, 0) << " = s" << owner_[size_t(v)] << " && d" << v << " != 2;\n";
      o << "  const bool s" << seg(ci, 1) << " = s" << owner_[size_t(v)] << " && d" << v << " != 1;\n";
    }
    for (int w = 0; w < words; ++w) {
      o << "  m[" << w << "] = 0u";
      for (int b = 0; b < 32; ++b) {
        const int s = 1 + 32 * w + b;
        if (size_t(s) < ns) o << " | (s" << s << " ? 0x" << std::hex << (1u << b) << std::dec << "u : 0u)";
      }
      o << ";\n";
    }
    // operations per point that remain: each active segment's own nodes, and
    // the arithmetic of every needed combinator that keeps both operands
    std::vector<OpCost> sc(ns);
    for (int v = 0; v < n_; ++v) {
      if (!live_[size_t(v)] || is_leaf(nd(v).op) || comb_of_[size_t(v)] >= 0) continue;
      OpCost c = node_cost(nd(v).op);
      sc[size_t(owner_[size_t(v)])].fp += c.fp;
      sc[size_t(owner_[size_t(v)])].sfu += c.sfu;
    }
    auto sum = [&](bool sfu) {
      std::ostringstream e;
      e << "0.0f";
      for (size_t s = 0; s < ns; ++s) {
        const double c = sfu ? sc[s].sfu : sc[s].fp;
        if (c > 0) e << " + (s" << s << " ? " << c << ".0f : 0.0f)";
      }
      for (size_t ci = 0; ci < combs_.size(); ++ci) {
        const int v = combs_[ci];
        OpCost c = node_cost(nd(v).op);
        const double x = sfu ? c.sfu : c.fp;
        if (x > 0) e << " + (s" << owner_[size_t(v)] << " && d" << v << " == 0 ? " << x << ".0f : 0.0f)";
      }
      return e.str();
    };
    o << "  *fp = " << sum(false) << ";\n";
    o << "  *sfu = " << sum(true) << ";\n";
    o << "  *root = " << ival(ir_.root) << ";\n";  // bounds the SDF's value at every point of the box
    o << "}\n";
  }

  // The guarded tile function's body, in the regions of the point code: a
  // combinator is
  //   if (b active in pm) { <region of b>; i = a active in pm ? sel(a, b) : b; }
  //   else if (a active in pm) i = a;
  // and the nodes of an operand-a segment inside a region are guarded by
  // that segment's bit in pm.
  static std::string ptest(int bit) {
    return "(pm[" + std::to_string(bit >> 5) + "] >> " + std::to_string(bit & 31) + " & 1u)";
  }
  void emit_tile_combinator(std::ostringstream &o, int v, const std::vector<std::vector<int>> &members,
                            const std::string &ind) const {
    const int ci = comb_of_[size_t(v)];
    const PNode &p = nd(v);
    const int sa = seg(ci, 0), sb = seg(ci, 1);
    const std::string keepA = p.op == POp::SmoothSubtraction ? "s2i_neg(" + ival(p.a) + ")" : ival(p.a);
    o << ind << "if " << ptest(sb - 1) << " {\n";
    emit_tile_region(o, sb, members, ind + "  ");
    o << ind << "  if " << ptest(sa - 1) << " i" << v << " = " << iexpr(v) << ";\n";
    o << ind << "  else { i" << v << " = " << ival(p.b) << "; d" << v << " = 2; }\n";
    o << ind << "} else if " << ptest(sa - 1) << " {\n";
    o << ind << "  i" << v << " = " << keepA << "; d" << v << " = 1;\n" << ind << "}\n";
  }

  // Chains as in the point code: a chunk whose operand-b bits are all clear
  // in pm keeps operand a throughout (d = 1 for each combinator; one that is
  // not needed has d unused, and d = 1 leaves its operands inactive).
  void emit_tile_region(std::ostringstream &o, int R, const std::vector<std::vector<int>> &members,
                        const std::string &ind) const {
    int open = R;
    auto close = [&]() {
      if (open != R) o << ind << "}\n";
      open = R;
    };
    const std::vector<int> &mem = members[size_t(R)];
    for (size_t idx = 0; idx < mem.size(); ++idx) {
      const int v = mem[idx];
      const int ci = comb_of_[size_t(v)];
      if (ci >= 0) {
        close();
        size_t end = idx + 1;
        if (chain_link(-1, v))
          while (end < mem.size() && chain_link(mem[end - 1], mem[end])) ++end;
        if (end - idx < 4) {
          emit_tile_combinator(o, v, members, ind);
          continue;
        }
        for (size_t c0 = idx; c0 < end; c0 += kChainChunk) {
          const size_t c1 = std::min(end, c0 + size_t(kChainChunk));
          std::ostringstream test;
          for (auto &[w, msk] : chunk_b_words(mem, c0, c1)) {
            char hx[16];
            std::snprintf(hx, sizeof hx, "%xu", msk);
            test << (test.tellp() > 0 ? " | " : "") << "(pm[" << w << "] & 0x" << hx << ")";
          }
          o << ind << "if (" << test.str() << ") {\n";
          for (size_t k = c0; k < c1; ++k) emit_tile_combinator(o, mem[k], members, ind + "  ");
          o << ind << "} else {\n";
          o << ind << "  i" << mem[c1 - 1] << " = " << ival(nd(mem[c0]).a) << ";\n";
          for (size_t k = c0; k < c1; ++k) o << ind << "  d" << mem[k] << " = 1;\n";
          o << ind << "}\n";
        }
        idx = end - 1;
        continue;
      }
      const int s = owner_[size_t(v)];
      if (s != open) {
        close();
        if (s != R) o << ind << "if " << ptest(s - 1) << " {\n";
        open = s;
      }
      o << ind << (open != R ? "  " : "") << "i" << v << " = " << iexpr(v) << ";\n";
    }
    close();
  }

  // Point code.  Every node is placed in a region: the innermost operand-b
  // segment enclosing its segment, or the top level.  A region's nodes are
  // emitted in ascending order; a node whose segment is not the region
  // itself (an operand-a segment inside it) is guarded by that segment's
  // bit, consecutive nodes of one segment sharing one `if`.  A combinator is
  // emitted where its index falls, without a guard of its own (when its
  // segment is inactive its value is simply not used), as
  //     if (b active) { <region of operand b>; v = a active ? op(a, b) : b; } else v = a;
  // so a combinator that keeps operand a costs one test.  Operand-a
  // segments are not nested blocks: a chain of combinators stays one level
  // deep.
  void emit_combinator(std::ostringstream &o, int v, const std::vector<std::vector<int>> &members,
                       const std::string &ind) const {
    const int ci = comb_of_[size_t(v)];
    const PNode &p = nd(v);
    const int sa = seg(ci, 0), sb = seg(ci, 1);
    const std::string A = as_var(p.a, var_[size_t(v)]), B = as_var(p.b, var_[size_t(v)]);
    // a decided smooth operator's result is its kept operand with -0 made +0
    // (s2_canon; the operator's arithmetic at h = 1 or 0)
    const bool smooth = is_smooth(p.op);
    const std::string keepA = smooth ? "s2_canon(" + (p.op == POp::SmoothSubtraction ? "(-" + A + ")" : A) + ")" : A;
    const std::string keepB = smooth ? "s2_canon(" + B + ")" : B;
    o << ind << "if " << bit_test(sb - 1) << " {\n";
    emit_region(o, sb, members, ind + "  ");
    o << ind << "  if " << bit_test(sa - 1) << " v" << v << " = " << expr(v) << ";\n";
    o << ind << "  else v" << v << " = " << keepB << ";\n";
    o << ind << "} else {\n" << ind << "  v" << v << " = " << keepA << ";\n" << ind << "}\n";
  }

  // A chain: consecutive members of a region, each combinator the operand a
  // of the next and used nowhere else (c = op(op(op(x, b1), b2), b3) ...).
  // Its combinators are emitted in chunks of kChainChunk under one test of
  // their operand-b bits: when none is set, every combinator of the chunk
  // keeps operand a and the chunk's result is its input.  (Not for the smooth
  // subtraction, whose "keep a" is -a.)
  static constexpr int kChainChunk = 8;
  // operand-b bits of the combinators mem[c0, c1), by word
  std::map<int, unsigned> chunk_b_words(const std::vector<int> &mem, size_t c0, size_t c1) const {
    std::map<int, unsigned> words;
    for (size_t k = c0; k < c1; ++k) {
      const int bit = seg(comb_of_[size_t(mem[k])], 1) - 1;
      words[bit >> 5] |= 1u << (bit & 31);
    }
    return words;
  }
  bool chain_link(int prev, int v) const {
    const int ci = comb_of_[size_t(v)];
    if (ci < 0 || nd(v).op == POp::SmoothSubtraction) return false;
    if (prev < 0) return true;
    return nd(v).a == prev && uses_[size_t(prev)].size() == 1;
  }

  void emit_region(std::ostringstream &o, int R, const std::vector<std::vector<int>> &members,
                   const std::string &ind) const {
    int open = R;
    auto close = [&]() {
      if (open != R) o << ind << "}\n";
      open = R;
    };
    const std::vector<int> &mem = members[size_t(R)];
    for (size_t idx = 0; idx < mem.size(); ++idx) {
      const int v = mem[idx];
      const int ci = comb_of_[size_t(v)];
      if (ci >= 0) {
        close();
        size_t end = idx + 1;  // the chain starting at v: mem[idx, end)
        if (chain_link(-1, v))
          while (end < mem.size() && chain_link(mem[end - 1], mem[end])) ++end;
        if (end - idx < 4) {
          emit_combinator(o, v, members, ind);
          continue;
        }
        for (size_t c0 = idx; c0 < end; c0 += kChainChunk) {
          const size_t c1 = std::min(end, c0 + size_t(kChainChunk));
          std::ostringstream test;
          for (auto &[w, msk] : chunk_b_words(mem, c0, c1)) {
            char hx[16];
            std::snprintf(hx, sizeof hx, "%xu", msk);
            test << (test.tellp() > 0 ? " | " : "") << "(m[" << w << "] & 0x" << hx << ")";
          }
          const int last = mem[c1 - 1];
          bool smooth = false;  // the chunk's kept input passes a smooth operator: s2_canon
          for (size_t k = c0; k < c1; ++k) smooth = smooth || is_smooth(nd(mem[k]).op);
          const std::string in = as_var(nd(mem[c0]).a, var_[size_t(last)]);
          o << ind << "if (" << test.str() << ") {\n";
          for (size_t k = c0; k < c1; ++k) emit_combinator(o, mem[k], members, ind + "  ");
          o << ind << "} else {\n";
          o << ind << "  v" << last << " = " << (smooth ? "s2_canon(" + in + ")" : in) << ";\n";
          o << ind << "}\n";
        }
        idx = end - 1;
        continue;
      }
      const int s = owner_[size_t(v)];
      if (s != open) {
        close();
        if (s != R) o << ind << "if " << bit_test(s - 1) << " {\n";
        open = s;
      }
      o << ind << (open != R ? "  " : "") << "v" << v << " = " << expr(v) << ";\n";
    }
    close();
  }

  // Region of each node: the innermost operand-b segment among its segment
  // and the segment's ancestors (0: top level).
  std::vector<std::vector<int>> regions() const {
    const size_t ns = 1 + 2 * combs_.size();
    std::vector<std::vector<int>> members(ns);
    for (int v = 0; v < n_; ++v) {
      if (!live_[size_t(v)] || is_leaf(nd(v).op)) continue;
      int r = owner_[size_t(v)];
      while (r != 0 && (r - 1) % 2 != 1) r = sparent_[size_t(r)];
      members[size_t(r)].push_back(v);
    }
    return members;
  }

  // A value as an s2x4 where one is wanted (a uniform value is splat).
  std::string as_var(int v, bool want) const {
    return run4_ && want && !var_[size_t(v)] ? "s2x4_splat(" + val(v) + ")" : val(v);
  }

  void emit_point(std::ostringstream &o) const {
    // Out of line on the device (S2M_PRUNED_FN): inlined into the lattice
    // kernel's point loop, the branchy body let the compiler keep far more
    // values live across iterations than the registers hold.
    if (run4_)
      o << "S2M_PRUNED_FN s2x4 s2m_user_sdf_pruned_run4(float x, float y, s2x4 z, const unsigned *m)\n{\n";
    else
      o << "S2M_PRUNED_FN float s2m_user_sdf_pruned(float x, float y, float z, const unsigned *m)\n{\n";
    o << "  (void)x; (void)y; (void)z;\n";
    for (int v = 0; v < n_; ++v)
      if (live_[size_t(v)] && !is_leaf(nd(v).op))
        o << (run4_ && var_[size_t(v)] ? "  s2x4 v" : "  float v") << v << ";\n";
    emit_region(o, 0, regions(), "  ");
    o << "  return " << (run4_ ? as_var(ir_.root, true) : val(ir_.root)) << ";\n}\n";
  }
};

}  // namespace

PruneCode prune_codegen(const PruneIR &ir) { return Pruner(ir).run(); }

}  // namespace s2m
