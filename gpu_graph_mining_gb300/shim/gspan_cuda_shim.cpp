// Drop-in for the reference's GPU miner: links the reference's mains
// (src/gspan_cuda/common_main.cpp:28,88 obtain the miner through
// get_gspan_cuda_instance()) against libgspan_gb300 instead of a gspan_cuda
// variant.  Built with the reference's own headers and flags (nvcc -x cu, its
// include directories), in place of gspan_cuda_no_sort_support.cpp.
//
// set_database (src/gspan_cuda/gspan_cuda.hpp:284-285) is not virtual: the
// base class's runs and keeps the database's host arrays in
// h_cuda_graph_database (gspan_cuda.cpp:73-104).  run() (gspan_cuda.hpp:292,
// virtual) hands those arrays to gs_db_from_arrays_device, which copies them
// to the GPU and builds the device database there, as the reference's
// copy_to_device does, then mines with the support set by set_min_support
// and emits every pattern to the graph_output set by set_graph_output.
#include <stdexcept>

#include <dfs_code.hpp>
#include <graph_output.hpp>
#include <gspan_cuda.hpp>

#include "gspan_gb300.h"

namespace {

struct gb300_miner : public gspan_cuda::gspan_cuda {
  static void emit(const int32_t *d, int32_t n, int64_t sup, void *user)
  {
    types::DFSCode code;
    for(int i = 0; i < n; i++) code.push(d[5 * i], d[5 * i + 1], d[5 * i + 2], d[5 * i + 3], d[5 * i + 4]);
    static_cast<graph_output *>(user)->output_graph(code, (size_t)sup);
  }

  void run() override
  {
    const types::graph_database_cuda &c = h_cuda_graph_database;
    gs_status st = GS_OK;
    gs_db *db = gs_db_from_arrays_device(c.db_size, c.edges_sizes, c.max_graph_vertex_count, c.vertex_count, c.edges,
                                         c.edges_labels, c.vertex_labels, c.vertex_offsets, &st);
    if(!db) throw std::runtime_error(gs_last_error());
    st = gs_mine(db, minimal_support, 0, output ? emit : nullptr, output);
    gs_db_free(db);
    // the reference reports failures as exceptions
    if(st != GS_OK) throw std::runtime_error(gs_last_error());
  }
};

}  // namespace

gspan_cuda::gspan_cuda *get_gspan_cuda_instance() { return new gb300_miner(); }
