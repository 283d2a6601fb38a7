// Capture harness for the reference's GPU miner gspan_cuda_no_sort
// (src/gspan_cuda/gspan_cuda_no_sort.cpp), used as a second oracle.
//
// Test infrastructure only: oracle/gspan_cuda.mk compiles it with the
// reference's own sources into oracle/_ref/gspan_cuda_ref; nothing in the
// product links it.
//
// It mirrors src/gspan_cuda/main_gspan_cuda_no_sort.cpp:28-120 (same
// <filetype> <file> <abs-minsup> arguments, exit codes 1/2/3, the same
// cuda_configurator block sizes) but replaces its counting sink with one that
// writes "<code.to_string(false)>\t<support>" per reported pattern.  The GPU
// miner's codes carry every vertex label (no -1), and its order is its own
// traversal's, so a comparison with the sequential reference sorts the lines
// after normalising the labels.  Wall time of run() goes to stderr.
#include <cstdio>
#include <cstdlib>
#include <string>
#include <sys/time.h>

#include <cuda_configurator.hpp>
#include <dbio.hpp>
#include <graph_output.hpp>
#include <graph_types.hpp>
#include <gspan_cuda_no_sort.hpp>

class capture_output : public graph_output {
  FILE *out;
  double count;
public:
  explicit capture_output(FILE *f) : out(f), count(0) {}
  virtual void output_graph(const types::Graph &g, size_t support) { count += 1; }
  virtual void output_graph(const types::DFSCode &code, size_t support) {
    if(out) std::fprintf(out, "%s\t%zu\n", code.to_string(false).c_str(), support);
    count += 1;
  }
  virtual double get_count() { return count; }
  virtual std::string to_string() { return "capture_output"; }
};

int main(int argc, char **argv)
{
  if(argc != 4 && argc != 5) {
    std::fprintf(stderr, "usage: %s <filetype> <filename> <support-int-abs> [<output-filename>|-]\n", argv[0]);
    return 1;
  }
  const int minsup = std::atoi(argv[3]);
  dbio::FILE_TYPE ft = dbio::ftype2str(std::string(argv[1]));
  types::graph_database_t database;
  types::graph_database_cuda cuda_gdb(true);
  if(ft == dbio::CUDABIN) dbio::read_database_cudabin(std::string(argv[2]), cuda_gdb);
  else dbio::read_database(ft, std::string(argv[2]), database);
  const size_t n = ft == dbio::CUDABIN ? (size_t)cuda_gdb.size() : database.size();
  if(minsup >= (int)n) {
    std::fprintf(stderr, "error: user specified support %d is greater then the database size %zu\n", minsup, n);
    return 2;
  }
  if(minsup < 1) {
    std::fprintf(stderr, "error: absolute_min_support < 1\n");
    return 3;
  }
  FILE *f = 0;
  if(argc == 5 && std::string(argv[4]) != "-") f = std::fopen(argv[4], "w");
  else if(argc == 4) f = stdout;
  capture_output out(f);

  cudapp::cuda_configurator exec_config;
  exec_config.set_parameter("create_first_embeddings.valid_vertex", 128);
  exec_config.set_parameter("create_first_embeddings.store_map", 128);
  exec_config.set_parameter("create_first_embeddings.find_valid_edge", 128);
  exec_config.set_parameter("create_first_embeddings.edge_store", 128);
  exec_config.set_parameter("compute_extensions.store_validity", 128);
  exec_config.set_parameter("compute_extensions.exec_extension_op", 128);
  exec_config.set_parameter("compute_support.boundaries", 128);
  exec_config.set_parameter("filter_backward_embeddings.store_col_indices", 128);
  exec_config.set_parameter("filter_backward_embeddings.copy_rows", 128);

  int rc = 0;
  timeval t0, t1;
  try {
    gspan_cuda::gspan_cuda_no_sort g;
    if(ft == dbio::CUDABIN) g.set_database(cuda_gdb);
    else g.set_database(database, true);
    g.set_min_support(minsup);
    g.set_graph_output(&out);
    g.set_exec_configurator(&exec_config);
    gettimeofday(&t0, 0);
    g.run();
    gettimeofday(&t1, 0);
    g.delete_database_from_device();
  } catch(std::exception &e) {
    std::fprintf(stderr, "exception: %s\n", e.what());
    rc = 5;
  }
  if(f && f != stdout) std::fclose(f);
  if(rc == 0) {
    const double secs = (t1.tv_sec - t0.tv_sec) + 1e-6 * (t1.tv_usec - t0.tv_usec);
    std::fprintf(stderr, "total_time=%.6f total_frequent_graphs=%.0f\n", secs, out.get_count());
  }
  return rc;
}
