// Link-time stand-ins for two debugging checks of the reference's GPU miner
// (defined in its gtest-based src/gspan_cuda/tests/test_embeddings.cpp and ext_test2.cpp, which
// needs Google Test).  gspan_cuda.cpp calls them only from its own
// cross-checking run (run_intern2), which the no_sort variant does not use.
// Test infrastructure only (oracle/gspan_cuda.mk).
#include <cstdio>

#include <embedding_lists.hpp>
#include <graph_types.hpp>

void check_host_db_agains_embedding(const types::graph_database_t &, types::DFS, const types::embedding_list_columns &)
{
  std::fprintf(stderr, "check_host_db_agains_embedding: not built in this harness\n");
}

void check_embedding_against_host_db(const types::graph_database_t &, types::DFS, const types::embedding_list_columns &)
{
  std::fprintf(stderr, "check_embedding_against_host_db: not built in this harness\n");
}

// the same for gspan_cuda_tests.cpp's per-embedding check (tests/ext_test2.cpp)
#include <gspan_cuda.hpp>

bool check_one_embedding(types::graph_database_t &, types::graph_database_cuda &, std::vector<int>,
                         types::embedding_list_columns, int, gspan_cuda::extension_element_t *, int)
{
  std::fprintf(stderr, "check_one_embedding: not built in this harness\n");
  return true;
}
