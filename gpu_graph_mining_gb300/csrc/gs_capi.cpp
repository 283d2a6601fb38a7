// extern "C" layer over the miner (declarations in include/gspan_gb300.h).
#include "../../include/gspan_gb300.h"

#include <cstring>
#include <set>
#include <string>
#include <vector>

#include "gs_db.hpp"
#include "gs_engine.hpp"
#include "gs_handles.hpp"

namespace {

thread_local std::string t_err;

gs_status set_err(gs_status code, const std::string &msg)
{
  t_err = msg;
  return code;
}

gs_db *finish_load(gsgb::LoadResult r, gs_db *db, gs_status *st)
{
  if(!r.error.empty()) {
    delete db;
    if(st) *st = set_err(r.code ? r.code : GS_ERR_FORMAT, r.error);
    return nullptr;
  }
  try {
    db->d.prepare();
  } catch(const gsgb::Error &e) {
    delete db;
    if(st) *st = set_err(e.code, e.what());
    return nullptr;
  }
  if(st) *st = GS_OK;
  t_err.clear();
  return db;
}

void fill_opts(const gs_mine_opts *o, gsgb::MineOptions &m)
{
  if(!o) return;
  m.max_edges = o->max_edges;
  m.label_style = o->label_style;
  if(o->wave_nodes > 0) m.wave_nodes = o->wave_nodes;
  if(o->threads > 0) m.threads = o->threads;
  if(o->wave_rows > 0) m.wave_rows = o->wave_rows;
  if(o->wave_words > 0) m.wave_words = o->wave_words;
  m.min_check = o->min_check == 1 ? 1 : 0;
  m.launch_mode = o->launch_mode == 1 ? 1 : 0;
  if(o->count_grid > 0 && o->count_grid <= 1024) m.count_grid = o->count_grid;
  m.extension = o->extension == GS_EXTENSION_LISTS ? 1 : o->extension == GS_EXTENSION_AUTO ? 2 : 0;
  if(o->deep_nodes > 0) m.deep_nodes = o->deep_nodes;
  m.serial = o->serial == 1 ? 1 : 0;
  if(o->schedulers > 0 && o->schedulers <= 64) m.schedulers = o->schedulers;
  if(o->root_parts > 1 && o->root_part >= 0 && o->root_part < o->root_parts) {
    m.root_parts = o->root_parts;
    m.root_part = o->root_part;
  }
}

void fill_stats(const gsgb::MineStats &s, gs_mine_stats *o)
{
  if(!o) return;
  o->patterns = s.patterns;
  o->waves = s.waves;
  o->launches = s.launches;
  o->nodes = s.nodes;
  o->rows = s.rows;
  o->extensions = s.extensions;
  o->candidates = s.candidates;
  o->count_bytes = s.count_bytes;
  o->mat_bytes = s.mat_bytes;
  o->count_ms = s.count_ms;
  o->mat_ms = s.mat_ms;
  o->support_ms = s.support_ms;
  o->root_ms = s.root_ms;
  o->host_min_ms = s.host_min_ms;
  o->wall_ms = s.wall_ms;
  o->peak_pool_bytes = s.peak_pool_bytes;
  o->h2d_bytes = s.h2d_bytes;
  o->d2h_bytes = s.d2h_bytes;
  o->host_build_ms = s.host_build_ms;
  o->host_wait_ms = s.host_wait_ms;
  o->host_select_ms = s.host_select_ms;
  o->host_emit_ms = s.host_emit_ms;
  o->min_host_checks = s.min_host;
  o->list_entries = s.list_entries;
  o->join_nodes = s.join_nodes;
  o->sel_bytes = s.sel_bytes;
  o->sel_ms = s.sel_ms;
  o->min_ms = s.min_ms;
}

struct BatchCtx {
  gs_batch_emit_fn fn;
  void *user;
  int32_t index;
};

void batch_trampoline(const int32_t *dfs, int32_t n, int64_t sup, void *u)
{
  BatchCtx *c = (BatchCtx *)u;
  c->fn(c->index, dfs, n, sup, c->user);
}

}  // namespace

namespace gsgb {
void capi_set_error(const char *msg) { t_err = msg ? msg : ""; }
}  // namespace gsgb

extern "C" {

const char *gs_last_error(void) { return t_err.c_str(); }

int32_t gs_filetype_from_name(const char *name) { return gsgb::parse_filetype(name); }

gs_db *gs_db_load(const char *path, int32_t filetype, gs_status *status)
{
  if(!path) {
    if(status) *status = set_err(GS_ERR_USAGE, "null path");
    return nullptr;
  }
  gs_db *db = new gs_db();
  return finish_load(gsgb::load_database(path, filetype, db->d.host), db, status);
}

gs_db *gs_db_from_arrays(int32_t db_size, int32_t edges_sizes, int32_t max_graph_vertex_count, int32_t vertex_count,
                         const int32_t *edges, const int32_t *edges_labels, const int32_t *vertex_labels,
                         const int32_t *vertex_offsets, gs_status *status)
{
  (void)vertex_count;
  if(db_size < 0 || edges_sizes < 0 || max_graph_vertex_count < 0 ||
     (edges_sizes > 0 && (!edges || !edges_labels)) ||
     ((int64_t)db_size * max_graph_vertex_count > 0 && (!vertex_labels || !vertex_offsets))) {
    if(status) *status = set_err(GS_ERR_USAGE, "invalid arrays");
    return nullptr;
  }
  gs_db *db = new gs_db();
  gsgb::LoadResult r = gsgb::db_from_cudabin_arrays(db_size, edges_sizes, max_graph_vertex_count, edges,
                                                    edges_labels, vertex_labels, vertex_offsets, db->d.host);
  if(r.error.empty()) r = gsgb::validate_simple(db->d.host);
  return finish_load(r, db, status);
}

gs_db *gs_db_from_arrays_device(int32_t db_size, int32_t edges_sizes, int32_t max_graph_vertex_count,
                                int32_t vertex_count, const int32_t *edges, const int32_t *edges_labels,
                                const int32_t *vertex_labels, const int32_t *vertex_offsets, gs_status *status)
{
  gsgb::DeviceScope device_scope;
  (void)vertex_count;
  if(db_size < 0 || edges_sizes < 0 || max_graph_vertex_count < 0 ||
     (edges_sizes > 0 && (!edges || !edges_labels)) || !vertex_offsets ||
     ((int64_t)db_size * max_graph_vertex_count > 0 && !vertex_labels)) {
    if(status) *status = set_err(GS_ERR_USAGE, "invalid arrays");
    return nullptr;
  }
  gs_db *db = new gs_db();
  try {
    gsgb::ingest_cudabin_device(db->d, db_size, edges_sizes, max_graph_vertex_count, edges, edges_labels,
                                vertex_labels, vertex_offsets);
  } catch(const gsgb::Error &e) {
    delete db;
    if(status) *status = set_err(e.code, e.what());
    return nullptr;
  }
  if(status) *status = GS_OK;
  t_err.clear();
  return db;
}

gs_db *gs_db_generate(int32_t config, uint64_t seed, double scale, gs_status *status)
{
  gsgb::GenParams p;
  if(!gsgb::config_params(config, seed, scale > 0 ? scale : 1.0, p)) {
    if(status) *status = set_err(GS_ERR_USAGE, "unknown configuration");
    return nullptr;
  }
  gs_db *db = new gs_db();
  gsgb::generate_database(p, db->d.host);
  return finish_load(gsgb::LoadResult(), db, status);
}

gs_status gs_db_write(const gs_db *db, const char *path, int32_t filetype)
{
  gsgb::DeviceScope device_scope;
  if(!db || !path) return set_err(GS_ERR_USAGE, "null argument");
  try {
    const_cast<gs_db *>(db)->d.ensure_host();
  } catch(const gsgb::Error &e) {
    return set_err(e.code, e.what());
  }
  gsgb::LoadResult r = gsgb::write_database(db->d.host, path, filetype);
  if(!r.error.empty()) return set_err(r.code ? r.code : GS_ERR_IO, r.error);
  return GS_OK;
}

int32_t gs_db_size(const gs_db *db) { return db ? db->d.host.n_graphs : -1; }

gs_status gs_db_convert(const char *in_path, int32_t in_type, const char *out_path, int32_t out_type,
                        gs_convert_info *info)
{
  if(!in_path || !out_path) return set_err(GS_ERR_USAGE, "null path");
  gsgb::HostDB db;
  gsgb::LoadResult r = gsgb::load_database(in_path, in_type, db, false);
  if(!r.error.empty()) return set_err(r.code ? r.code : GS_ERR_FORMAT, r.error);
  int64_t fixed = 0, renumbered = 0;
  r = gsgb::fix_database(db, &fixed, &renumbered);
  if(!r.error.empty()) return set_err(r.code ? r.code : GS_ERR_FORMAT, r.error);
  if(out_type == GS_BIN && db.n_graphs == 0)
    return set_err(GS_ERR_FORMAT, "Cannot save empty database.");  // write_database_bin, dbio.cpp:211
  r = gsgb::write_database(db, out_path, out_type);
  if(!r.error.empty()) return set_err(r.code ? r.code : GS_ERR_IO, r.error);
  if(info) {
    std::set<int32_t> vl(db.vlabel.begin(), db.vlabel.end()), el(db.adj_el.begin(), db.adj_el.end());
    info->graphs = db.n_graphs;
    info->graphs_fixed = fixed;
    info->graphs_renumbered = renumbered;
    info->vertex_labels = (int32_t)vl.size();
    info->edge_labels = (int32_t)el.size();
  }
  t_err.clear();
  return GS_OK;
}

gs_status gs_db_get_info(const gs_db *db, gs_db_info *info)
{
  if(!db || !info) return set_err(GS_ERR_USAGE, "null argument");
  info->graphs = db->d.host.n_graphs;
  info->vertices = db->d.n_vertices();
  info->adjacency_entries = db->d.n_adj();
  info->vertex_labels = db->d.VL;
  info->edge_labels = db->d.EL;
  info->device_bytes = db->d.resident ? (int64_t)db->d.d_bytes : 0;
  return GS_OK;
}

gs_status gs_db_upload(gs_db *db)
{
  gsgb::DeviceScope device_scope;
  if(!db) return set_err(GS_ERR_USAGE, "null database");
  try {
    db->d.upload();
  } catch(const gsgb::Error &e) {
    return set_err(e.code, e.what());
  }
  return GS_OK;
}

void gs_db_free(gs_db *db)
{
  gsgb::DeviceScope device_scope;
  delete db;
}

void gs_mine_opts_default(gs_mine_opts *o)
{
  if(!o) return;
  gsgb::MineOptions m;
  o->max_edges = m.max_edges;
  o->label_style = m.label_style;
  o->wave_nodes = m.wave_nodes;
  o->threads = m.threads;
  o->wave_rows = m.wave_rows;
  o->wave_words = m.wave_words;
  o->root_part = 0;
  o->root_parts = 1;
  o->min_check = m.min_check;
  o->launch_mode = m.launch_mode;
  o->count_grid = m.count_grid;
  o->deep_nodes = m.deep_nodes;
  o->extension = m.extension;
  o->serial = m.serial;
  o->schedulers = m.schedulers;
}

gs_status gs_mine_ex(gs_db *db, int32_t abs_minsup, const gs_mine_opts *opts, gs_emit_fn emit, void *user,
                     gs_mine_stats *stats)
{
  gsgb::DeviceScope device_scope;
  if(!db) return set_err(GS_ERR_USAGE, "null database");
  std::vector<gsgb::MineJob> jobs(1);
  gsgb::MineOptions mo;
  fill_opts(opts, mo);
  jobs[0].db = &db->d;
  jobs[0].minsup = abs_minsup;
  jobs[0].opt = mo;
  jobs[0].emit = emit;
  jobs[0].user = user;
  gsgb::MineStats st;
  std::string err;
  int rc = gsgb::run_jobs(jobs, mo, &st, err);
  fill_stats(st, stats);
  if(rc != 0) return set_err(rc, err);
  t_err.clear();
  return GS_OK;
}

gs_status gs_mine_collect(gs_db *db, int32_t abs_minsup, const gs_mine_opts *opts, gs_patterns **out,
                          gs_mine_stats *stats)
{
  if(!out) return set_err(GS_ERR_USAGE, "null output");
  *out = nullptr;
  gsgb::PatternBuf *b = new gsgb::PatternBuf();
  gs_status st = gs_mine_ex(db, abs_minsup, opts, gsgb::PatternBuf::emit, b, stats);
  if(st != GS_OK) {
    delete b;
    return st;
  }
  *out = b->publish();
  return GS_OK;
}

void gs_patterns_free(gs_patterns *p)
{
  // view is the first member of PatternBuf
  delete reinterpret_cast<gsgb::PatternBuf *>(p);
}

gs_status gs_mine(gs_db *db, int32_t abs_minsup, int32_t max_edges, gs_emit_fn emit, void *user)
{
  gs_mine_opts o;
  gs_mine_opts_default(&o);
  o.max_edges = max_edges;
  return gs_mine_ex(db, abs_minsup, &o, emit, user, nullptr);
}

gs_status gs_mine_batch(gs_db *const *dbs, int32_t n, const int32_t *abs_minsups, const gs_mine_opts *opts,
                        gs_batch_emit_fn emit, void *user, gs_mine_stats *stats)
{
  gsgb::DeviceScope device_scope;
  if(n < 0 || (n > 0 && (!dbs || !abs_minsups))) return set_err(GS_ERR_USAGE, "invalid batch");
  gsgb::MineOptions mo;
  fill_opts(opts, mo);
  std::vector<gsgb::MineJob> jobs(n);
  std::vector<BatchCtx> ctx(n);
  for(int32_t i = 0; i < n; i++) {
    if(!dbs[i]) return set_err(GS_ERR_USAGE, "null database in batch");
    ctx[i] = BatchCtx{ emit, user, i };
    jobs[i].db = &dbs[i]->d;
    jobs[i].minsup = abs_minsups[i];
    jobs[i].opt = mo;
    jobs[i].emit = emit ? batch_trampoline : nullptr;
    jobs[i].user = &ctx[i];
    jobs[i].tag = i;
  }
  gsgb::MineStats st;
  std::string err;
  int rc = gsgb::run_jobs(jobs, mo, &st, err);
  fill_stats(st, stats);
  if(rc != 0) return set_err(rc, err);
  t_err.clear();
  return GS_OK;
}

gs_status gs_autotune(gs_db *const *dbs, int32_t n, const int32_t *abs_minsups, gs_mine_opts *opts,
                      gs_tune_report *report)
{
  gsgb::DeviceScope device_scope;
  if(n <= 0 || !dbs || !abs_minsups || !opts) return set_err(GS_ERR_USAGE, "invalid autotune arguments");
  gsgb::MineOptions mo;
  fill_opts(opts, mo);
  std::vector<gsgb::MineJob> jobs(n);
  for(int32_t i = 0; i < n; i++) {
    if(!dbs[i]) return set_err(GS_ERR_USAGE, "null database");
    jobs[i].db = &dbs[i]->d;
    jobs[i].minsup = abs_minsups[i];
    jobs[i].opt = mo;
    jobs[i].tag = i;
  }
  gsgb::MineOptions best;
  std::vector<gsgb::TuneTrial> trials;
  std::string err;
  const int rc = gsgb::autotune_jobs(jobs, mo, best, trials, err);
  if(rc != 0) return set_err(rc, err);
  opts->wave_nodes = best.wave_nodes;
  opts->wave_rows = best.wave_rows;
  opts->count_grid = best.count_grid;
  opts->deep_nodes = best.deep_nodes;
  opts->schedulers = best.schedulers;
  if(report) {
    report->trials = (int32_t)trials.size();
    report->wave_nodes = best.wave_nodes;
    report->wave_rows = best.wave_rows;
    report->count_grid = best.count_grid;
    report->deep_nodes = best.deep_nodes;
    report->schedulers = best.schedulers;
    report->base_ms = trials.front().ms;
    double b = trials.front().ms;
    for(const auto &t : trials)
      if(t.wave_nodes == best.wave_nodes && t.wave_rows == best.wave_rows && t.count_grid == best.count_grid &&
         t.deep_nodes == best.deep_nodes && t.schedulers == best.schedulers)
        b = t.ms;
    report->best_ms = b;
  }
  t_err.clear();
  return GS_OK;
}

gs_status gs_support_count(const int32_t *keys, const int32_t *graph_ids, int64_t n_records, int32_t n_keys,
                           int32_t n_graphs, int32_t *support)
{
  gsgb::DeviceScope device_scope;
  std::string err;
  int rc = gsgb::support_count_host(keys, graph_ids, n_records, n_keys, n_graphs, support, err);
  if(rc != 0) return set_err(rc, err);
  return GS_OK;
}

gs_status gs_filter_backward(const int32_t *column, int64_t n_rows, const int32_t *records, int64_t n_records,
                             const int32_t *dfs, int32_t *out, int64_t *n_out)
{
  gsgb::DeviceScope device_scope;
  std::string err;
  int rc = gsgb::filter_backward_host(column, n_rows, records, n_records, dfs, out, n_out, err);
  if(rc != 0) return set_err(rc, err);
  return GS_OK;
}

gs_status gs_segmented_scan(const uint32_t *data, int64_t n, int32_t exclusive, uint32_t *out)
{
  gsgb::DeviceScope device_scope;
  std::string err;
  int rc = gsgb::segmented_scan_host(data, n, nullptr, 0, exclusive != 0, out, err);
  if(rc != 0) return set_err(rc, err);
  return GS_OK;
}

gs_status gs_segmented_reduce(const uint32_t *data, int64_t n, const uint32_t *segment_count,
                              const uint32_t *segment_sizes, int32_t groups, int32_t exclusive, uint32_t *results,
                              int64_t *n_results)
{
  gsgb::DeviceScope device_scope;
  if(groups < 0 || (groups > 0 && (!segment_count || !segment_sizes)) || !n_results)
    return set_err(GS_ERR_USAGE, "invalid arguments");
  // the last element of every segment, group by group
  std::vector<int64_t> ends;
  int64_t at = 0;
  for(int32_t gi = 0; gi < groups; gi++)
    for(uint32_t c = 0; c < segment_count[gi]; c++) {
      at += segment_sizes[gi];
      if(segment_sizes[gi] == 0 || at > n) return set_err(GS_ERR_USAGE, "the segments do not fit the array");
      ends.push_back(at - 1);
    }
  *n_results = (int64_t)ends.size();
  if(ends.empty()) return GS_OK;
  if(!results) return set_err(GS_ERR_USAGE, "null results");
  std::string err;
  int rc = gsgb::segmented_scan_host(data, n, ends.data(), (int64_t)ends.size(), exclusive != 0, results, err);
  if(rc != 0) return set_err(rc, err);
  return GS_OK;
}

int32_t gs_dfs_code_is_min(const int32_t *d, int32_t n)
{
  if(!d || n < 1 || n > gsgb::kMaxPatternEdges) return -1;
  std::vector<gsgb::DFS> code(n);
  for(int32_t i = 0; i < n; i++) {
    code[i] = gsgb::DFS{ d[5 * i], d[5 * i + 1], d[5 * i + 2], d[5 * i + 3], d[5 * i + 4] };
    if(code[i].from < 0 || code[i].to < 0 || code[i].from >= gsgb::kMaxPatternVertices ||
       code[i].to >= gsgb::kMaxPatternVertices || code[i].from == code[i].to)
      return -1;
  }
  static thread_local gsgb::MinChecker checker;
  return checker.is_min(code.data(), n) ? 1 : 0;
}

void gs_engine_reset(void)
{
  gsgb::DeviceScope device_scope;
  gsgb::engine_reset();
}

void gs_engine_set_pool_bytes(int64_t bytes) { gsgb::engine_set_pool_bytes(bytes); }

}  // extern "C"
