// gspan_gb300_convertdb: the reference's convertdb tool (src/globals/
// convertdb.cpp:28-66) over the C ABI: read a database, apply the
// fix_database repairs, write it in another format.
//
//   gspan_gb300_convertdb <filetype-in> <filename-in> <filetype-out> <filename-out>
//
// Exit codes: 0 done, 1 usage, 2 read / repair / write error.
#include <cstdio>

#include "../../include/gspan_gb300.h"

int main(int argc, char **argv)
{
  if(argc != 5) {
    std::fprintf(stderr, "usage: \n%s <filetype-in> <filename-in>  <filetype-out> <filename-out>\n", argv[0]);
    return 1;
  }
  const int32_t in = gs_filetype_from_name(argv[1]), out = gs_filetype_from_name(argv[3]);
  if(in < 0 || out < 0) {
    std::fprintf(stderr, "unknown filetype\n");
    return 1;
  }
  std::printf("reading database\n");
  gs_convert_info info;
  const gs_status st = gs_db_convert(argv[2], in, argv[4], out, &info);
  if(st != GS_OK) {
    std::fprintf(stderr, "%s\n", gs_last_error());
    return 2;
  }
  std::printf("graphs: %lld (repaired %lld, renumbered from 1: %lld); vertex labels: %d; edge labels: %d\n",
              (long long)info.graphs, (long long)info.graphs_fixed, (long long)info.graphs_renumbered,
              info.vertex_labels, info.edge_labels);
  std::printf("writing database\n");
  return 0;
}
