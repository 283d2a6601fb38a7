// Command-line miner with the reference mains' interface:
//   gspan_gb300 <filetype> <filename> <support-int-abs> [<output-filename>|-]
//               [--seq-labels] [--max-edges N] [--wave-nodes N] [--stats]
// (src/gspan_cuda/common_main.cpp:26-70 and src/gspan/main.cpp:21-66: same
// positional arguments, exit code 1 for usage, 2 when the support is not
// below the database size, 3 when it is below 1).  Each frequent pattern is
// written as "<code>\t<support>", code in DFSCode::to_string(false) form.
// "total_time=<s> total_frequent_graphs=<n>" goes to stderr, like the
// reference's LOG_VALUE lines.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "../../include/gspan_gb300.h"

namespace {

struct Sink {
  FILE *f;
  long long n;
};

void emit(const int32_t *d, int32_t n, int64_t support, void *user)
{
  Sink *s = (Sink *)user;
  s->n++;
  if(!s->f) return;
  for(int32_t i = 0; i < n; i++)
    std::fprintf(s->f, "%s(%d %d %d %d %d)", i ? ";" : "", d[5 * i], d[5 * i + 1], d[5 * i + 2], d[5 * i + 3], d[5 * i + 4]);
  std::fprintf(s->f, "\t%lld\n", (long long)support);
}

}  // namespace

int main(int argc, char **argv)
{
  if(argc < 4) {
    std::fprintf(stderr,
                 "usage: \n%s <filetype> <filename> <support-int-abs> [<output-filename>|-] [--seq-labels] "
                 "[--max-edges N] [--wave-nodes N] [--stats]\n",
                 argv[0]);
    return 1;
  }
  const int32_t ft = gs_filetype_from_name(argv[1]);
  if(ft < 0) {
    std::fprintf(stderr, "unknown filetype %s\n", argv[1]);
    return 1;
  }
  const int minsup = std::atoi(argv[3]);
  const char *outpath = nullptr;
  bool stats = false;
  gs_mine_opts o;
  gs_mine_opts_default(&o);
  for(int i = 4; i < argc; i++) {
    if(!std::strcmp(argv[i], "--seq-labels")) o.label_style = GS_LABELS_SEQ;
    else if(!std::strcmp(argv[i], "--max-edges") && i + 1 < argc) o.max_edges = std::atoi(argv[++i]);
    else if(!std::strcmp(argv[i], "--wave-nodes") && i + 1 < argc) o.wave_nodes = std::atoi(argv[++i]);
    else if(!std::strcmp(argv[i], "--stats")) stats = true;
    else outpath = argv[i];
  }
  gs_status st = GS_OK;
  gs_db *db = gs_db_load(argv[2], ft, &st);
  if(!db) {
    std::fprintf(stderr, "error: %s\n", gs_last_error());
    return 4;
  }
  if(minsup >= gs_db_size(db)) {
    std::fprintf(stderr, "error: user specified support %d is greater then the database size %d\n", minsup,
                 gs_db_size(db));
    gs_db_free(db);
    return 2;
  }
  if(minsup < 1) {
    std::fprintf(stderr, "error: absolute_min_support < 1\n");
    gs_db_free(db);
    return 3;
  }
  Sink sink{ nullptr, 0 };
  if(!outpath) sink.f = stdout;
  else if(std::strcmp(outpath, "-") != 0) {
    sink.f = std::fopen(outpath, "w");
    if(!sink.f) {
      std::fprintf(stderr, "cannot open %s\n", outpath);
      gs_db_free(db);
      return 4;
    }
  }
  gs_mine_stats ms;
  std::memset(&ms, 0, sizeof(ms));
  auto t0 = std::chrono::steady_clock::now();
  st = gs_mine_ex(db, minsup, &o, emit, &sink, &ms);
  double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if(sink.f && sink.f != stdout) std::fclose(sink.f);
  gs_db_free(db);
  if(st != GS_OK) {
    std::fprintf(stderr, "error: %s\n", gs_last_error());
    return st == GS_ERR_MINSUP_TOO_LARGE ? 2 : (st == GS_ERR_MINSUP_TOO_SMALL ? 3 : 5);
  }
  std::fprintf(stderr, "total_time=%.6f total_frequent_graphs=%lld\n", secs, sink.n);
  if(stats)
    std::fprintf(stderr,
                 "waves=%lld launches=%lld nodes=%lld rows=%lld extensions=%lld candidates=%lld count_ms=%.3f "
                 "mat_ms=%.3f support_ms=%.3f root_ms=%.3f host_min_ms=%.3f count_GBps=%.1f\n",
                 (long long)ms.waves, (long long)ms.launches, (long long)ms.nodes, (long long)ms.rows,
                 (long long)ms.extensions, (long long)ms.candidates, ms.count_ms, ms.mat_ms, ms.support_ms,
                 ms.root_ms, ms.host_min_ms, ms.count_ms > 0 ? ms.count_bytes / ms.count_ms / 1e6 : 0.0);
  return 0;
}
