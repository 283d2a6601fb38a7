// Device-side layouts shared by the kernels (gs_kernels.cu) and the host
// engine that fills them (gs_engine.cpp).
//
// Graph database in HBM (one per resident database):
//   adj[E2]      uint64: low 32 bits = neighbour (global vertex id),
//                high 32 bits = (edge label << 16) | neighbour vertex label;
//                with adj_sorted, ascending within each vertex's entries
//   adj_off[V+1] int32 CSR offsets, vlabel[V] dense vertex labels,
//   vgraph[V]    graph id of each vertex,
//   pair_idx[VL*EL*VL]  dense index of (elabel, tolabel) among the pairs that
//                occur next to a vertex of label fl, or -1.
// Labels are compacted order-preservingly to 0..VL-1 / 0..EL-1 (< 2^16).
//
// Embedding store: one column per pattern vertex, element = int2
// {graph vertex, row in the previous column}; an embedding is the chain
// from a row of the last column back to column 0 (the reference's
// embedding_list_columns, src/globals/embedding_lists.hpp:12-60).  A forward
// child appends a column; a backward child replaces the last column with a
// filtered copy.  Each DFS-tree node also carries gord[row]: the dense rank
// of the row's graph among the graphs that contain the node's pattern
// (0..support-1), the index into the node's support bitmaps.
#pragma once
#include <cstdint>

namespace gsgb {

struct DevDB {
  const unsigned long long *adj;
  const int32_t *adj_off;
  const int32_t *vlabel;
  const int32_t *vgraph;
  const int32_t *vgbase;    // [V] first global vertex of each vertex's graph
  const int32_t *vbase;     // [G+1] first global vertex of each graph
  const int32_t *adj_pair;  // [E2] pair index of each directed entry: pair_idx(label(source), el, label(nbr))
  const int32_t *pair_idx;
  int32_t VL, EL;
  int32_t n_graphs;
  int32_t n_vertices;
  int32_t max_graph_vertices;
  int32_t adj_sorted;  // 1: each vertex's entries ascend (adj as unsigned 64-bit values)
  const int32_t *root_off;   // [VL+1] first key of each vertex label's (elabel, tolabel) pairs
  const int32_t *pair_code;  // [root_off[VL]] (elabel << 16) | tolabel of each pair
};

// Per job of a root phase (the root level of a group of jobs, one launch per
// kernel): its vertices as 32-vertex warp tiles in the group's tile space, its
// bitmaps, counter copies and keys at their offsets in the group's buffers.
struct RootJob {
  long long tile_begin;  // first warp tile of the job (its vertex 0)
  long long bm_base;     // first bitmap word of the job's key 0
  long long cnt_base;    // first counter of the job's copy 0 (copy q at cnt_base + q * R)
  int32_t db;            // index into the resident-database table
  int32_t words;         // bitmap words per key = ceil(graphs / 32)
  int32_t R;             // root keys of the job's database
  int32_t copies;        // counter copies
  int32_t key_base;      // first key of the job in the group's key space
  int32_t pad;
};

// Per DFS-tree node of a wave (a batch of nodes extended together).
struct NodeDesc {
  long long row_begin;   // first row in the wave's concatenated row space
  long long tile_begin;  // first 32-row warp tile of the node (tiles never span two nodes)
  long long bm_base;     // first support-bitmap word of the node's key 0
  const int32_t *gord;   // [nrows]
  int32_t nrows;
  int32_t k;             // columns = pattern vertices; the right-most vertex is k-1
  int32_t col_off;       // first entry in the wave's column-pointer table
  int32_t slot_off;      // first entry in the wave's slot table
  int32_t vtab_off;      // first entry in the wave's vertex table (k entries)
  int32_t nslot;         // right-most path vertices; slot nslot-1 is the right-most vertex
  int32_t minlabel;      // label of pattern vertex 0: forward targets need label >= minlabel
  int32_t words;         // bitmap words per key = ceil(support / 32)
  int32_t key_base;      // first key of the node in the wave's key space
  int32_t nkeys;
  int32_t db;            // index into the resident-database table
  int32_t minsup;        // the node's job's minimum support (candidate selection)
  int32_t code_off;      // the node's DFS code: edges code_off.. of the wave's code table
  int32_t code_len;      //   (5 int32 per edge: from, to, fromlabel, elabel, tolabel)
  int32_t nfwd;          // keys below nfwd are forward extensions
  // Lists strategy (extension by intersection): a forward child's extensions
  // from right-most-path vertices other than its new right-most vertex are
  // its parent's frequent forward extensions at the same parent row (minus
  // the child's new vertex), read from the parent's per-row lists instead of
  // the database; only the right-most vertex's adjacency is scanned.  The
  // child's right-most path up to the new edge's source u is the parent's, so
  // those slots have the parent's forward keys: a list entry's parent key lk
  // is the child's key when lk < join_hi (slots up to u) and, from u itself,
  // lk >= join_key (pairs at or after the new edge's).  csr_off == nullptr:
  // no join, every right-most-path vertex is scanned.
  const int32_t *csr_off;  // [csr_rows + 1] the parent rows' list offsets into csr_ent
  const int2 *csr_ent;     // list entries {neighbour, parent's forward key}
  int32_t csr_rows;        // parent rows
  int32_t join_lo;         // first forward key of u
  int32_t join_key;        // the new edge's key (in the parent)
  int32_t join_hi;         // one past u's forward keys
};

// One right-most-path vertex of a node.
struct SlotDesc {
  int32_t vertex;    // pattern vertex id
  int32_t vlab;      // its (dense) label
  int32_t fkey_off;  // forward keys of this slot: fkey_off + pair_idx(vlab, el, tl)
  int32_t fel, ftl;  // forward order rule from the right-most-path edge leaving this
                     // vertex: allowed iff fel < el || (fel == el && ftl <= tl); fel = -1
                     // for the right-most vertex (no rule)
  int32_t bkey_off;  // backward keys to this vertex: bkey_off + el; -1 if not a target
  int32_t bel, blab; // backward order rule: allowed iff bel < el || (bel == el && blab <= label(rightmost))
  // the same two rules as single compares against an adjacency entry's high
  // word hi = (el << 16) | nbr_label: forward allowed iff hi >= frule
  // (INT32_MIN for the right-most vertex); backward allowed iff el >= bmin
  int32_t frule;
  int32_t bmin;
};

// Output slots of a child node selected for materialisation.
struct ChildOut {
  int2 *col;      // the child's new last column
  int2 *col0;     // root children only: column 0
  int32_t *gord;  // the child's graph ranks
  int32_t kind;   // 0 forward, 1 backward, 2 root
  int32_t cap;    // rows allocated (the count pass's embedding count for the key)
};

}  // namespace gsgb
