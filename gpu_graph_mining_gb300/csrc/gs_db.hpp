// Host-side graph database: the four file formats of the reference's dbio
// layer, label compaction, and the CSR arrays the device copy is built from.
#pragma once
#include <cstdint>
#include <functional>
#include <string>
#include <vector>

namespace gsgb {

// Runs fn(begin, end, part) over [0, n) split into contiguous parts on the
// host's cores (one part when n < 2 * min_chunk).
void parallel_ranges(int64_t n, const std::function<void(int64_t, int64_t, int)> &fn, int64_t min_chunk = 4096);

// File types, numbered like dbio::FILE_TYPE (src/globals/dbio.hpp:9).
enum FileType { FT_TXT = 0, FT_BIN = 1, FT_FSG = 2, FT_CUDABIN = 3 };

// Parses "txt"/"-txt"/"bin"/... like dbio::ftype2str (src/globals/dbio.cpp:33-41);
// returns -1 for an unknown name.
int parse_filetype(const char *name);

// A database of undirected labelled simple graphs in CSR form.  Vertex ids
// are global (graph g owns [vbase[g], vbase[g+1])); each vertex's adjacency
// keeps the reference's per-vertex push order (Vertex::push,
// src/globals/graph_types.hpp:38-44), both directions of every edge stored.
struct HostDB {
  int32_t n_graphs = 0;
  std::vector<int64_t> vbase;    // [G+1]
  std::vector<int32_t> vlabel;   // [V]   labels as read
  std::vector<int64_t> aoff;     // [V+1]
  std::vector<int32_t> adj_to;   // [E2]  neighbour, global vertex id
  std::vector<int32_t> adj_el;   // [E2]  edge label as read

  int64_t n_vertices() const { return (int64_t)vlabel.size(); }
  int64_t n_adj() const { return (int64_t)adj_to.size(); }
  int32_t graph_nv(int32_t g) const { return (int32_t)(vbase[g + 1] - vbase[g]); }
};

// Order-preserving dense relabelling.  The miner only compares labels
// (<, ==), so mapping the sorted distinct labels to 0..n-1 leaves every
// pattern, code and support unchanged; output maps back through *_of.
struct LabelMap {
  std::vector<int32_t> vlabel_of;  // dense vertex label -> original
  std::vector<int32_t> elabel_of;  // dense edge label   -> original
};

// Result of a parse: empty error string on success.
struct LoadResult {
  std::string error;
  int code = 0;  // gs_status value on failure
};

// validate = false keeps self loops and parallel edges (for fix_database).
LoadResult load_database(const char *path, int filetype, HostDB &db, bool validate = true);
LoadResult db_from_cudabin_arrays(int32_t db_size, int32_t edges_sizes, int32_t max_graph_vertex_count,
                                  const int32_t *edges, const int32_t *edges_labels,
                                  const int32_t *vertex_labels, const int32_t *vertex_offsets, HostDB &db);
LoadResult write_database(const HostDB &db, const char *path, int filetype);

// Rejects self loops and parallel edges (the mining path assumes simple
// graphs, as the reference's cudabin layout does: cuda_graph_types.cpp:65-127
// sizes its edge arrays from distinct edge ids).
LoadResult validate_simple(const HostDB &db);

// The repairs of the reference's convertdb tool (fix_database,
// src/globals/fix_database.cpp:10-85, with check_graph,
// check_database.cpp:10-30), graph by graph:
//  - a graph with a self loop or a repeated neighbour at some vertex is
//    rebuilt: self loops dropped, each neighbour kept once (its first edge
//    label; a differing label on a parallel edge is an error), every
//    vertex's neighbours in ascending order;
//  - a graph in which no vertex other than 0 has vertex 0 as a neighbour
//    loses vertex 0 and its other vertices move down by one (inputs written
//    with ids from 1).
// Counts the graphs rebuilt and renumbered.
LoadResult fix_database(HostDB &db, int64_t *fixed, int64_t *renumbered);

// Builds the dense label arrays (vertex and edge) and the label maps.
void compact_labels(const HostDB &db, std::vector<int32_t> &vl_dense, std::vector<int32_t> &el_dense, LabelMap &map);

// Seeded synthetic databases standing in for the reference's datasets.
struct GenParams {
  int64_t n_graphs = 340;
  int mode = 0;                 // 0: spanning tree + ring edges; 1: seeded patterns (PAFI-like)
  int vmin = 10, vmax = 60;     // mode 0 vertex count range
  double ring_per_vertex = 0.05;
  double mean_edges = 30.0;     // mode 1: edges per graph ~ Poisson(mean)
  int n_vlabels = 5;
  double vzipf = 0.0;           // 0 = uniform, else Zipf exponent
  int n_elabels = 5;
  std::vector<double> eweights; // optional categorical edge-label weights
  int n_seeds = 50;
  double seed_mean_edges = 4.0; // Poisson mean of edges per seed pattern (min seed_min_edges)
  int seed_min_edges = 1, seed_max_edges = 0;  // max 0 = unbounded
  double seed_cover = 0.5;      // fraction of each graph's edge budget filled with seed copies
  uint64_t seed = 1;
};

void generate_database(const GenParams &p, HostDB &db);

// Canned configurations 1..5 (see the configs of the benchmark description):
// returns false for an unknown id.  `scale` multiplies the graph count.
bool config_params(int config, uint64_t seed, double scale, GenParams &p);

}  // namespace gsgb
