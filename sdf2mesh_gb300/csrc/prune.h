// prune.h -- tile pruning of a straight-line SDF.
//
// The frontend lowers a straight-line sdf3d (float scalars and vectors, user
// functions inlined) to a scalar expression graph.  Its combinators -- min,
// max and the library's smooth union / intersection / subtraction -- are the
// places where one operand can make the other irrelevant.  For a tile of
// lattice points, an interval evaluation of the same binary32 operations
// bounds every intermediate value; where the bounds prove that a combinator
// returns one operand bit for bit at every point of the tile, the other
// operand's exclusive subgraph is not evaluated there.
//
// Soundness: each operation used here is monotone in each argument on the
// domain where it is applied (or, for products and quotients, takes its
// extremes at the corners), and round-to-nearest is monotone.  So evaluating
// an operation on the interval endpoints with the same rounding bounds the
// value the point code computes.  Intervals with an infinite or NaN endpoint,
// or from operations without a proof (exp, log, pow, atan2), are "unknown"
// and block every decision that depends on them.  Each decision also rules
// out the signed-zero cases in which the combinator's arithmetic would not
// return the operand's exact bits.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace s2m {

enum class POp : uint8_t {
  X, Y, Z, Const,
  Neg, Add, Sub, Mul, Div,
  Abs, Floor, Ceil, Sqrt, Min, Max, Clamp, Saturate, Mix,
  Sin, Cos, Exp, Log, Pow, Atan2,
  SmoothUnion, SmoothIntersection, SmoothSubtraction  // (a, b, k) as in sdf::op
};

struct PNode {
  POp op = POp::Const;
  int a = -1, b = -1, c = -1;
  float k = 0.0f;  // Const value
};

struct PruneIR {
  std::vector<PNode> nodes;  // arguments precede their users
  int root = -1;
};

struct PruneCode {
  bool ok = false;
  std::string cuda;      // s2m_user_sdf_tile + s2m_user_sdf_pruned (+ S2M_HAS_PRUNE)
  int combinators = 0;   // combinators that can prune
  int words = 0;         // 32-bit words of activity bits per tile
};

// Analysis and code generation; ok == false when nothing can be pruned.
PruneCode prune_codegen(const PruneIR &ir);

}  // namespace s2m
