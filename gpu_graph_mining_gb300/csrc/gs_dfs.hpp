// DFS codes: the reference's 5-tuple edge representation, right-most path,
// text form, and the minimum-DFS-code (canonicality) check.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace gsgb {

constexpr int kMaxPatternVertices = 64;   // columns an embedding row may have
constexpr int kMaxPatternEdges = 128;     // edges a pattern may have

// One DFS code edge, field order of types::DFS (src/globals/dfs_code.hpp:17-23).
struct DFS {
  int32_t from, to, fromlabel, elabel, tolabel;
  bool is_forward() const { return from < to; }
  bool operator==(const DFS &o) const
  {
    return from == o.from && to == o.to && fromlabel == o.fromlabel && elabel == o.elabel && tolabel == o.tolabel;
  }
  bool operator!=(const DFS &o) const { return !(*this == o); }
};

using Code = std::vector<DFS>;

// Indices of the forward edges on the right-most path, deepest first
// (DFSCode::buildRMPath, src/globals/dfs_code.cpp:75-90).  Returns the count.
int build_rmpath(const DFS *code, int n, int *rm);

// Label conventions of emitted codes.  FULL carries every vertex label (the
// GPU reference's codes, built from extension_element_t); SEQ writes -1 for
// fromlabel after the first edge and for the tolabel of backward edges (the
// sequential miner's codes, src/gspan/gspan.cpp:254,267).
enum LabelStyle { LABELS_FULL = 0, LABELS_SEQ = 1 };
void to_style(const DFS *in, int n, LabelStyle style, DFS *out);

// "(f t fl el tl);(...)" as DFSCode::to_string(false) (dfs_code.cpp:199-216).
std::string code_to_string(const DFS *code, int n);

// Canonicality test with the exact semantics of the sequential miner's
// gSpan::is_min (src/gspan/ismin.cpp:36-143): rebuild the minimum code of
// the pattern greedily and compare position by position from the second
// edge on.  Accepts codes in either label style.
class MinChecker {
public:
  bool is_min(const DFS *code, int n);

private:
  struct Emb {
    uint8_t map[kMaxPatternVertices];  // min-code vertex -> pattern vertex
    uint8_t hist[kMaxPatternEdges];    // min-code edge   -> pattern edge id
    uint64_t vmask;
    uint64_t emask[2];
  };
  struct PAdj { int32_t to, elabel, id; };
  int nv_ = 0;
  int32_t vlab_[kMaxPatternVertices];
  std::vector<PAdj> adj_[kMaxPatternVertices];
  int32_t ef_[kMaxPatternEdges], et_[kMaxPatternEdges];
  std::vector<Emb> cur_, next_;
  DFS seq_[kMaxPatternEdges];
  DFS mc_[kMaxPatternEdges];
};

}  // namespace gsgb
