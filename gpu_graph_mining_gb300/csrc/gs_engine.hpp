// The mining engine: resident databases, the device memory pool, and the
// wave scheduler that extends many DFS-tree nodes per kernel launch.
#pragma once
#include <cstdint>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "gs_db.hpp"
#include "gs_device.hpp"
#include "gs_dfs.hpp"

namespace gsgb {

// Status codes shared with the C ABI (include/gspan_gb300.h).
enum Status {
  ST_OK = 0,
  ST_ERR_USAGE = 1,
  ST_ERR_IO = 2,
  ST_ERR_FORMAT = 3,
  ST_ERR_CUDA = 4,
  ST_ERR_NOMEM = 5,
  ST_ERR_MINSUP_TOO_LARGE = 6,
  ST_ERR_MINSUP_TOO_SMALL = 7,
  ST_ERR_LIMIT = 8,
  ST_ERR_TIMEOUT = 9,
  ST_ERR_CANCELLED = 10,
  ST_ERR_BUDGET = 11,
  ST_ERR_STATE = 12,
};

// The library runs its device work on device 0: one GPU per process (a
// process that wants another GPU restricts CUDA_VISIBLE_DEVICES).  Every C-ABI
// entry point that touches the device holds a DeviceScope for the call: device
// 0 is made current, and the caller's thread gets back the device it had.
struct DeviceScope {
  int prev = -1;
  DeviceScope()
  {
    if(cudaGetDevice(&prev) != cudaSuccess) {
      cudaGetLastError();
      prev = -1;
    }
    if(prev != 0) cudaSetDevice(0);
  }
  ~DeviceScope()
  {
    if(prev > 0) cudaSetDevice(prev);
  }
  DeviceScope(const DeviceScope &) = delete;
  DeviceScope &operator=(const DeviceScope &) = delete;
};

struct Error : public std::runtime_error {
  int code;
  Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

void cuda_check(cudaError_t e, const char *what);

// Host database plus, once uploaded, its device copy.
struct Database {
  HostDB host;
  LabelMap labels;
  std::vector<int32_t> vl_dense, el_dense;
  int32_t VL = 0, EL = 0;
  // pairs[a] = sorted (elabel, tolabel) pairs occurring next to label-a vertices
  std::vector<std::vector<std::pair<int32_t, int32_t>>> pairs;
  std::vector<int32_t> pair_cnt, root_off;
  int32_t root_keys = 0;
  // device copy
  void *d_block = nullptr;
  size_t d_bytes = 0;
  DevDB dev{};
  int32_t *d_root_off = nullptr;
  bool resident = false;
  // built on the device from cudabin arrays (ingest_cudabin_device): the host
  // arrays stay empty until ensure_host() downloads them
  bool device_only = false;
  bool pooled = false;   // d_block is from the ingest's pool (ingest_free_block)
  int64_t dev_vertices = 0, dev_adj = 0;
  // device-built: the packed entries in input order (dev.adj may be sorted)
  const unsigned long long *adj_in = nullptr;

  void prepare();   // label compaction and pair tables (host only)
  void upload();    // device copy (idempotent)
  void release();   // frees the device copy
  void ensure_host();  // host arrays of a device-built database (original labels)
  int64_t n_vertices() const { return device_only ? dev_vertices : host.n_vertices(); }
  int64_t n_adj() const { return device_only ? dev_adj : host.n_adj(); }
  ~Database();
};

// Builds db's device copy directly from the reference's cudabin arrays (host
// memory) on the GPU: the checks and the result of db_from_cudabin_arrays +
// validate_simple + Database::prepare/upload, without the host conversion
// (gs_ingest.cu).  Throws Error.
void ingest_cudabin_device(Database &db, int32_t db_size, int32_t edges_sizes, int32_t max_graph_vertex_count,
                           const int32_t *edges, const int32_t *edges_labels, const int32_t *vertex_labels,
                           const int32_t *vertex_offsets);

// Returns the device ingest's pooled scratch to the driver.
void ingest_release();

// Frees a database block taken from the ingest's pool (after the device is idle,
// as cudaFree would be).
void ingest_free_block(void *block);

using EmitFn = void (*)(const int32_t *dfs5xN, int32_t n_edges, int64_t support, void *user);

struct MineOptions {
  int32_t max_edges = 0;      // 0 = no cap
  int32_t label_style = 0;    // LABELS_FULL / LABELS_SEQ
  int32_t wave_nodes = 4096;  // 1 = plain one-pattern-at-a-time
  int64_t wave_rows = 1 << 24;
  int64_t wave_words = 1 << 24;  // support-bitmap words per wave
  int32_t threads = 0;        // host threads for the canonicality check (0 = hardware)
  int32_t root_part = 0;      // mine only the root subtrees with index % root_parts == root_part
  int32_t root_parts = 1;
  int32_t min_check = 0;      // canonicality: 0 on the GPU (host for oversized patterns), 1 on the host
  int32_t launch_mode = 0;    // a wave's device work: 0 replayed from a CUDA graph, 1 launched directly
  int32_t count_grid = 0;     // count-kernel grid cap in blocks per SM (0 = the built-in default)
  int32_t extension = 0;      // extension strategy: 0 every right-most-path vertex's adjacency is
                              // scanned; 1 lists: forward children join their parent's per-row
                              // lists of frequent forward extensions and scan only their new
                              // right-most vertex (the reference's gspan_cuda_lists); 2 lists for
                              // waves whose databases' adjacency does not stay in L2, else 0
  int32_t deep_nodes = 0;     // a third wave context launches while this many nodes are queued (0 = wave_nodes)
  int32_t serial = 0;         // 1: every wave context issues on the engine's stream (no kernels overlap)
  int32_t schedulers = 0;     // batches: jobs split over this many schedulers, each with its own engine and
                              // host thread (0 = one per 8 jobs from 16 jobs on, at most 4; else 1)
};

struct MineStats {
  int64_t patterns = 0;
  int64_t waves = 0;
  int64_t launches = 0;
  int64_t nodes = 0;
  int64_t rows = 0;          // embedding rows extended
  int64_t extensions = 0;    // (row, extension) pairs enumerated by the count pass
  int64_t candidates = 0;    // frequent candidates checked for canonicality
  int64_t count_bytes = 0;   // algorithmic bytes of the count kernels
  int64_t mat_bytes = 0;     // algorithmic bytes of the materialise kernels
  double count_ms = 0;       // summed kernel time of the count kernels
  double mat_ms = 0;         // summed kernel time of the materialise kernels
  double support_ms = 0;
  double root_ms = 0;
  double host_min_ms = 0;    // canonicality checks on the host
  double wall_ms = 0;
  int64_t peak_pool_bytes = 0;
  int64_t h2d_bytes = 0;     // host->device bytes copied (database upload and per-wave tables)
  int64_t d2h_bytes = 0;     // device->host bytes copied (candidate supports and counts)
  double host_build_ms = 0;  // wave layout and descriptor tables
  double host_wait_ms = 0;   // blocked on the device (stream synchronisations)
  double host_select_ms = 0; // candidate decoding, child allocation, child tables
  double host_emit_ms = 0;   // pattern-tree traversal and output
  int64_t min_host = 0;      // candidates whose canonicality was checked on the host
  int64_t list_entries = 0;  // lists strategy: per-row list entries built
  int64_t join_nodes = 0;    // lists strategy: nodes extended through a join
  int64_t sel_bytes = 0;     // algorithmic bytes of the selection kernels (screen, count listed)
  double sel_ms = 0;         // summed kernel time of the selection kernels
  double min_ms = 0;         // summed kernel time of the GPU canonicality checks
};

struct MineJob {
  Database *db = nullptr;
  int32_t minsup = 1;
  MineOptions opt;
  EmitFn emit = nullptr;
  void *user = nullptr;
  int32_t tag = 0;   // caller's index (batch position / request id)
};

// Runs a set of mining jobs to completion in shared waves and emits each
// job's patterns (in the reference's traversal order) after it finishes.
// Jobs with emit == nullptr still count their patterns in stats.
int run_jobs(std::vector<MineJob> &jobs, const MineOptions &wave_opt, MineStats *stats, std::string &err);

struct JobInfo {
  int64_t live_bytes = 0;   // embedding-store bytes held by the job's pending nodes
  int64_t peak_bytes = 0;
  int64_t patterns = 0;     // set when the job finished
  int64_t pending = 0;      // DFS-tree nodes queued or in flight
  bool done = false;
  bool cancelled = false;
};

// A long-lived mining context with its own stream, device pool and scratch.
// Jobs are added at any time and advance together, wave by wave: each step
// launches waves of pending DFS-tree nodes (oldest jobs first) and completes
// the oldest wave in flight.  A job's emit callback runs inside the step that
// finishes it.  Not thread-safe: one thread drives it.  Errors throw Error;
// after one, reset() drops every job and the device state.
class Scheduler {
public:
  Scheduler(const MineOptions &wave_opt, int64_t pool_bytes);
  ~Scheduler();
  Scheduler(const Scheduler &) = delete;
  Scheduler &operator=(const Scheduler &) = delete;
  int32_t add(const MineJob &job);   // validates, mines the root level; returns the job id
  bool idle() const;                 // no unfinished job
  void step();
  void cancel(int32_t id);
  std::vector<int32_t> take_done();  // jobs finished or cancelled since the last call
  bool job_info(int32_t id, JobInfo &out);
  void forget(int32_t id);           // drops a finished job's bookkeeping
  void sync_stats();                 // folds device counters into stats()
  MineStats &stats();
  int64_t pool_used() const;
  void reset();

private:
  struct Impl;
  std::unique_ptr<Impl> p_;
};

// support[k] = number of distinct graph ids among the records with key k
// (host arrays; records must satisfy 0 <= key < n_keys, 0 <= graph < n_graphs).
int support_count_host(const int32_t *keys, const int32_t *gids, int64_t n, int32_t n_keys, int32_t n_graphs,
                       int32_t *support, std::string &err);

// Backward child column: out = the elements ({vertex, back_link}) of column at
// the rows named by the records (8 ints each) equal to the backward edge dfs,
// in row order; *n_out their count (host arrays, GPU work).
// Segmented scan of packed uint32 values (bit 31 starts a segment): with
// n_ends == 0 the whole scanned array goes to out[n]; otherwise out[j] =
// scanned[ends[j]].
int segmented_scan_host(const uint32_t *data, int64_t n, const int64_t *ends, int64_t n_ends, int exclusive,
                        uint32_t *out, std::string &err);
int filter_backward_host(const int32_t *column, int64_t n_rows, const int32_t *records, int64_t n_records,
                         const int32_t *dfs, int32_t *out, int64_t *n_out, std::string &err);

// Autotuning of the wave options for a workload (the jobs, mined as one
// batch): coordinate descent over the work chunk (wave_nodes), the row budget
// per wave (wave_rows) and the count kernel's grid cap (count_grid); each
// trial is a complete mining pass (patterns counted, not emitted), timed on
// the host clock, best of two.  best receives the fastest options; trials
// lists (wave_nodes, wave_rows, count_grid, ms) of every trial.
struct TuneTrial {
  int32_t wave_nodes;
  int64_t wave_rows;
  int32_t count_grid;
  int32_t deep_nodes;
  int32_t schedulers;
  double ms;
};
int autotune_jobs(std::vector<MineJob> &jobs, const MineOptions &base, MineOptions &best,
                  std::vector<TuneTrial> &trials, std::string &err);

// Releases the engine's device pool and scratch (the next call re-creates them).
void engine_reset();

// Bytes the engine's pool may use (0 = 70% of free device memory at first use).
void engine_set_pool_bytes(int64_t bytes);

}  // namespace gsgb
