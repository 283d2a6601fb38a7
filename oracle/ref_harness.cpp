// Capture harness for the reference's sequential gSpan (src/gspan/gspan.cpp,
// Taku Kudo's algorithm as shipped in zakimjz/GPU_graph_mining).
//
// Test infrastructure only.  It is compiled by oracle/Makefile together with
// the reference's own source files, straight from the read-only reference
// tree, into oracle/_ref/gspan_ref.  Nothing in the product links it.
//
// It mirrors src/gspan/main.cpp:21-97 (same <filetype> <file> <abs-minsup>
// arguments, same exit codes 1/2/3) but replaces the graph_file_output sink
// (src/globals/graph_output.cpp:91-96, which drops the support) with one that
// writes "<code.to_string(false)>\t<support>" per reported pattern, in the
// reference's traversal order.  Wall time of gSpan::run() goes to stderr as
// "total_time=<seconds>".
#include <cstdio>
#include <cstdlib>
#include <string>
#include <sys/time.h>

#include <graph_output.hpp>
#include <graph_types.hpp>
#include <dbio.hpp>
#include <gspan.hpp>

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
  int minsup = std::atoi(argv[3]);
  types::graph_database_t database;
  dbio::FILE_TYPE ft = dbio::ftype2str(std::string(argv[1]));
  if(ft == dbio::CUDABIN) {
    types::graph_database_cuda cuda_gdb(true);
    dbio::read_database_cudabin(std::string(argv[2]), cuda_gdb);
    cuda_gdb.convert_to_host_representation(database);
  } else {
    dbio::read_database(ft, std::string(argv[2]), database);
  }
  if(minsup >= (int)database.size()) {
    std::fprintf(stderr, "error: user specified support %d is greater then the database size %zu\n", minsup, database.size());
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

  timeval t0, t1;
  gettimeofday(&t0, 0);
  GSPAN::gSpan g;
  g.set_database(database);
  g.set_min_support(minsup);
  g.set_graph_output(&out);
  g.run();
  gettimeofday(&t1, 0);
  double secs = (t1.tv_sec - t0.tv_sec) + 1e-6 * (t1.tv_usec - t0.tv_usec);
  if(f && f != stdout) std::fclose(f);
  std::fprintf(stderr, "total_time=%.6f total_frequent_graphs=%.0f\n", secs, out.get_count());
  return 0;
}
