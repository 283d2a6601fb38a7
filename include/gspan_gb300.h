/*
 * gspan_gb300.h -- C ABI of the GB300 gSpan frequent-subgraph miner.
 *
 * Plain C types only (pointers, sizes, int32/int64).  All entry points
 * report errors through a gs_status value (never abort()); the text of the
 * last error on the calling thread is available from gs_last_error().
 *
 * Drop-in correspondence with the reference (zakimjz/GPU_graph_mining):
 * the miner class gspan_cuda::gspan_cuda (src/gspan_cuda/gspan_cuda.hpp:
 * 53,284-292) with set_database / set_min_support / set_graph_output / run,
 * the database readers of src/globals/dbio.hpp:9-37 and the output sink
 * graph_output::output_graph(const DFSCode&, size_t support)
 * (src/globals/graph_output.hpp:12).
 *
 * Device: the miner, the database uploads and ingests, gs_support_count and
 * gs_filter_backward run on CUDA device 0 of the process (one GPU per
 * process; choose the GPU with CUDA_VISIBLE_DEVICES).  Each such call makes
 * device 0 current for its duration and gives the calling thread back the
 * device it had current.  gs_support_count_noalloc runs on the device of its
 * output buffer instead.
 */
#ifndef GSPAN_GB300_H
#define GSPAN_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define GS_API __attribute__((visibility("default")))
#else
#define GS_API
#endif

typedef int32_t gs_status;

/* Status codes.  GS_ERR_MINSUP_TOO_LARGE / _TOO_SMALL correspond to the
 * reference mains' exit codes 2 and 3 (src/gspan_cuda/common_main.cpp:56-70). */
enum {
  GS_OK = 0,
  GS_ERR_USAGE = 1,
  GS_ERR_IO = 2,
  GS_ERR_FORMAT = 3,
  GS_ERR_CUDA = 4,
  GS_ERR_NOMEM = 5,
  GS_ERR_MINSUP_TOO_LARGE = 6,
  GS_ERR_MINSUP_TOO_SMALL = 7,
  GS_ERR_LIMIT = 8,
  GS_ERR_TIMEOUT = 9,
  GS_ERR_CANCELLED = 10,
  GS_ERR_BUDGET = 11,
  GS_ERR_STATE = 12
};

/* File types, numbered as dbio::FILE_TYPE (src/globals/dbio.hpp:9). */
enum { GS_TXT = 0, GS_BIN = 1, GS_FSG = 2, GS_CUDABIN = 3 };

/* Label conventions of emitted DFS codes.  GS_LABELS_FULL carries every
 * vertex label, as the GPU reference's codes do; GS_LABELS_SEQ writes -1 for
 * fromlabel after the first edge and for the tolabel of backward edges, as
 * the sequential reference (src/gspan/gspan.cpp:254,267) does. */
enum { GS_LABELS_FULL = 0, GS_LABELS_SEQ = 1 };

typedef struct gs_db gs_db;

/* Thread-local text of the last error ("" if none). */
GS_API const char *gs_last_error(void);

/* Parses "txt"/"-txt"/"bin"/"fsg"/"cudabin" like dbio::ftype2str
 * (src/globals/dbio.cpp:33-41); -1 if unknown. */
GS_API int32_t gs_filetype_from_name(const char *name);

/* Loads a database file: replaces dbio::read_database / read_database_cudabin
 * (src/globals/dbio.cpp:44-60, 381-404).  Graphs must be simple (no self
 * loops, no parallel edges).  Returns NULL on error. */
GS_API gs_db *gs_db_load(const char *path, int32_t filetype, gs_status *status);

/* Builds a database from the reference's flat cudabin arrays
 * (types::graph_database_cuda, src/globals/cuda_graph_types.hpp:16-50; the
 * layout written by dbio::write_database_cudabin, dbio.cpp:354-370):
 * edges/edges_labels[edges_sizes], vertex_labels[db_size*max_graph_vertex_count],
 * vertex_offsets[db_size*max_graph_vertex_count+1], -1 marking padding.
 * Replaces gspan_cuda::set_database(graph_database_cuda&) (gspan_cuda.cpp:73-104).
 * The arrays are copied. */
GS_API gs_db *gs_db_from_arrays(int32_t db_size, int32_t edges_sizes, int32_t max_graph_vertex_count,
                                int32_t vertex_count, const int32_t *edges, const int32_t *edges_labels,
                                const int32_t *vertex_labels, const int32_t *vertex_offsets, gs_status *status);

/* gs_db_from_arrays built on the GPU: the arrays are copied to the device
 * (as graph_database_cuda::copy_to_device, cuda_graph_types.cpp:166-196,
 * does) and converted, checked, label-compacted and indexed there, so no
 * host conversion runs.  Same arguments, checks and mining results as
 * gs_db_from_arrays; the database is resident when the call returns.  The
 * host arrays are built only if the database is written (gs_db_write).
 * Vertex label values must span at most 2^22 and the label alphabet must
 * keep |VL|*|EL|*|VL| <= 2^25, else GS_ERR_LIMIT (use gs_db_from_arrays).
 * Memory: the scratch and the database come from a stream-ordered pool that
 * keeps up to 16 GiB of device memory between ingests (gs_engine_reset
 * returns it), and such a database holds its adjacency twice (8 more bytes
 * per entry): sorted for mining and in input order for gs_db_write. */
GS_API gs_db *gs_db_from_arrays_device(int32_t db_size, int32_t edges_sizes, int32_t max_graph_vertex_count,
                                       int32_t vertex_count, const int32_t *edges, const int32_t *edges_labels,
                                       const int32_t *vertex_labels, const int32_t *vertex_offsets,
                                       gs_status *status);

/* Seeded synthetic database of benchmark configuration 1..5 with `scale`
 * times its graph count.  No counterpart in the reference: it stands in for
 * the PAFI graph generator the reference's experiments used
 * (testdata/fsg/gen_graphs.sh). */
GS_API gs_db *gs_db_generate(int32_t config, uint64_t seed, double scale, gs_status *status);

/* Writes a database as txt, bin or cudabin (dbio::write_database_bin /
 * write_database_cudabin, src/globals/dbio.cpp:209-260, 354-370). */
GS_API gs_status gs_db_write(const gs_db *db, const char *path, int32_t filetype);

/* The reference's convertdb tool (src/globals/convertdb.cpp:28-66): reads a
 * database (self loops and parallel edges allowed), applies its
 * fix_database repairs (src/globals/fix_database.cpp:10-85) graph by graph,
 * and writes it out:
 *  - a graph with a self loop or a neighbour listed twice at a vertex is
 *    rebuilt with self loops dropped, each neighbour once (a parallel edge
 *    with a different label is an error, GS_ERR_FORMAT) and every vertex's
 *    neighbours in ascending order;
 *  - a graph in which no vertex but 0 has vertex 0 as a neighbour loses
 *    vertex 0 and its other vertices move down by one (files numbered from 1).
 * bin and cudabin output are byte-identical to the reference tool's; txt
 * output (which the reference's writer refuses) is also accepted.  info may
 * be NULL. */
typedef struct gs_convert_info {
  int64_t graphs;
  int64_t graphs_fixed;       /* rebuilt: self loops dropped, parallel edges merged */
  int64_t graphs_renumbered;  /* vertex 0 dropped */
  int32_t vertex_labels;      /* distinct labels written */
  int32_t edge_labels;
} gs_convert_info;
GS_API gs_status gs_db_convert(const char *in_path, int32_t in_type, const char *out_path, int32_t out_type,
                               gs_convert_info *info);

/* Number of graphs (graph_database_cuda::size, cuda_graph_types.hpp:67). */
GS_API int32_t gs_db_size(const gs_db *db);

/* Vertex / adjacency-entry / label counts of a database. */
typedef struct gs_db_info {
  int64_t graphs;
  int64_t vertices;
  int64_t adjacency_entries; /* both directions of every edge */
  int32_t vertex_labels;
  int32_t edge_labels;
  int64_t device_bytes;      /* bytes of the device copy, 0 if not resident */
} gs_db_info;
GS_API gs_status gs_db_get_info(const gs_db *db, gs_db_info *info);

/* Copies the database to the GPU now (otherwise the first mining call does). */
GS_API gs_status gs_db_upload(gs_db *db);

/* Frees the host and device copies. */
GS_API void gs_db_free(gs_db *db);

/* Output sink, the C form of graph_output::output_graph(const DFSCode&, size_t)
 * (src/globals/graph_output.hpp:12): called on the calling thread once per
 * frequent pattern, in the sequential reference's traversal order (the GPU
 * reference, gspan_cuda_no_sort.cpp:107,416, emits the same set).  dfs5xN
 * holds n_edges tuples {from, to, fromlabel, elabel, tolabel}
 * (types::DFS, src/globals/dfs_code.hpp:17-23); it is valid during the call. */
typedef void (*gs_emit_fn)(const int32_t *dfs5xN, int32_t n_edges, int64_t support, void *user);

typedef struct gs_mine_opts {
  int32_t max_edges;   /* 0 = no cap on pattern edges */
  int32_t label_style; /* GS_LABELS_FULL or GS_LABELS_SEQ */
  int32_t wave_nodes;  /* DFS-tree nodes extended per launch; 1 = one pattern at a time */
  int32_t threads;     /* host threads for the canonicality check; 0 = all cores */
  int64_t wave_rows;   /* embedding rows per launch (soft cap; 0 = default) */
  int64_t wave_words;  /* support-bitmap words per launch (soft cap; 0 = default) */
  int32_t root_part;   /* mine only the root subtrees whose index (in the reference's root */
  int32_t root_parts;  /* order) is root_part modulo root_parts; root_parts <= 1 = all */
  int32_t min_check;   /* canonicality check: 0 = on the GPU (patterns over 32 vertices or 64 edges,
                          or with too many self-embeddings, on the host), 1 = on the host */
  int32_t launch_mode; /* a wave's device work (uploads, clears, count, selection, check, results
                          copy): 0 = replayed from a per-variant CUDA graph, 1 = launched directly */
  int32_t count_grid;  /* count-kernel grid cap in blocks per SM; 0 = built-in default (64) */
  int32_t extension;   /* extension strategy: GS_EXTENSION_RMPATH (default) scans the adjacency of every
                          right-most-path vertex of every embedding; GS_EXTENSION_LISTS is the
                          reference's lists variant (gspan_cuda_lists, main_gspan_cuda_lists.cpp):
                          a forward child takes its extensions from the right-most path's older
                          vertices by joining its parent's frequent forward extensions at the same
                          parent row (extend_embeddings.cpp:206-330, intersection_fwd_fwd) and
                          scans only its new right-most vertex; GS_EXTENSION_AUTO uses the lists
                          for the waves whose databases' adjacency is larger than three quarters of
                          the L2 (rescans from DRAM), the plain scan otherwise.  Same patterns and
                          supports. */
  int32_t deep_nodes;  /* a third wave may be in flight (besides two) while at least this many DFS-tree
                          nodes are queued; 0 = wave_nodes (default), 1 = always.  More waves in flight
                          hide more of the host's work per wave when a workload has many small nodes;
                          a short queue split three ways makes smaller waves. */
  int32_t serial;      /* 0 = each wave context issues on its own stream, so that one wave's selection and
                          materialise passes run beside another wave's count (default); 1 = all on one
                          stream: no two kernels overlap, so per-kernel times in gs_mine_stats are
                          exclusive.  Same patterns and supports. */
  int32_t schedulers;  /* gs_mine_batch: the databases split over this many schedulers, each with its own
                          device pool, wave contexts and streams, run on their own host threads (the
                          host's per-node work then uses that many cores while the GPU runs their waves
                          side by side); 0 = one per 8 databases for batches of 16 or more, at most 4,
                          else 1.  Patterns are
                          emitted on the calling thread after all are mined, database by database in batch
                          order.  For one database (gs_mine_ex, gs_mine_collect) a value above 1 splits it
                          by root subtrees (part p takes the roots whose index in the reference's order is p
                          modulo P), the patterns merged back in the reference's order; 0 = not split.
                          Same patterns, supports and order. */
} gs_mine_opts;

#define GS_EXTENSION_RMPATH 0
#define GS_EXTENSION_LISTS 1
#define GS_EXTENSION_AUTO 2

typedef struct gs_mine_stats {
  int64_t patterns;
  int64_t waves;
  int64_t launches;        /* kernels launched by the miner */
  int64_t nodes;           /* DFS-tree nodes extended */
  int64_t rows;            /* embedding rows extended */
  int64_t extensions;      /* one-edge extensions enumerated */
  int64_t candidates;      /* frequent candidates checked for canonicality */
  int64_t count_bytes;     /* algorithmic bytes of the count kernels */
  int64_t mat_bytes;       /* algorithmic bytes of the materialise kernels */
  double count_ms;         /* summed device time of the count kernels */
  double mat_ms;           /* summed device time of the materialise kernels */
  double support_ms;
  double root_ms;
  double host_min_ms;
  double wall_ms;
  int64_t peak_pool_bytes;
  int64_t h2d_bytes;       /* host->device bytes copied (database upload, per-wave tables) */
  int64_t d2h_bytes;       /* device->host bytes copied (candidate supports and counts) */
  double host_build_ms;    /* host: wave layout and descriptor tables */
  double host_wait_ms;     /* host: blocked on the device */
  double host_select_ms;   /* host: candidate decoding and child allocation */
  double host_emit_ms;     /* host: output */
  int64_t min_host_checks; /* candidates whose canonicality was checked on the host */
  int64_t list_entries;    /* GS_EXTENSION_LISTS: parent-row list entries built */
  int64_t join_nodes;      /* GS_EXTENSION_LISTS: DFS-tree nodes extended through a join */
  int64_t sel_bytes;       /* algorithmic bytes of the candidate selection kernels */
  double sel_ms;           /* summed device time of the candidate selection kernels */
  double min_ms;           /* summed device time of the GPU canonicality checks */
} gs_mine_stats;

GS_API void gs_mine_opts_default(gs_mine_opts *opts);

/* Mines all frequent connected subgraphs with support >= abs_minsup:
 * replaces set_min_support + set_graph_output + run of gspan_cuda::gspan_cuda
 * (src/gspan_cuda/gspan_cuda.hpp:284-292).  Returns GS_ERR_MINSUP_TOO_LARGE
 * when abs_minsup >= number of graphs and GS_ERR_MINSUP_TOO_SMALL when < 1.
 * Patterns have at most 64 vertices and 127 edges: when a frequent pattern
 * beyond that exists the call returns GS_ERR_LIMIT (cap max_edges), never a
 * truncated result. */
GS_API gs_status gs_mine(gs_db *db, int32_t abs_minsup, int32_t max_edges, gs_emit_fn emit, void *user);
GS_API gs_status gs_mine_ex(gs_db *db, int32_t abs_minsup, const gs_mine_opts *opts, gs_emit_fn emit, void *user,
                            gs_mine_stats *stats);

/* Bulk output: all frequent patterns in one host buffer instead of one
 * output_graph call per pattern (the reference's sink is a virtual call per
 * pattern, graph_output.cpp:91-96).  Pattern i is the tuples
 * dfs[5*offset[i] .. 5*offset[i+1]) with support[i], in traversal order.
 * Free with gs_patterns_free. */
typedef struct gs_patterns {
  int64_t count;
  int64_t n_tuples;
  const int64_t *offset;  /* [count + 1] */
  const int32_t *dfs;     /* [5 * n_tuples] {from, to, fromlabel, elabel, tolabel} */
  const int64_t *support; /* [count] */
} gs_patterns;
GS_API gs_status gs_mine_collect(gs_db *db, int32_t abs_minsup, const gs_mine_opts *opts, gs_patterns **out,
                                 gs_mine_stats *stats);
GS_API void gs_patterns_free(gs_patterns *p);

/* Batched form: n databases mined together, their DFS-tree nodes sharing
 * launches.  emit receives the database index first.  No counterpart in the
 * reference (it mines one database per process). */
typedef void (*gs_batch_emit_fn)(int32_t db_index, const int32_t *dfs5xN, int32_t n_edges, int64_t support,
                                 void *user);
GS_API gs_status gs_mine_batch(gs_db *const *dbs, int32_t n, const int32_t *abs_minsups, const gs_mine_opts *opts,
                               gs_batch_emit_fn emit, void *user, gs_mine_stats *stats);

/* ---------------------------------------------------------------- serving
 * A request loop over resident databases: mining requests (database,
 * minsup, pattern-size cap) are submitted at any time from any thread and
 * mined by one server thread with continuous batching.  Requests that arrive
 * while others are on the GPU are admitted as active slots and embedding-
 * store memory free up, and their DFS-tree nodes share launches with the
 * requests already running (oldest first).  Admission charges each request
 * an embedding-store estimate (the peak seen for the same database, minsup
 * and cap, else 20 bytes per adjacency entry) against budget_bytes; a
 * request is always admitted when nothing else runs.  No counterpart in the
 * reference, which mines one database per process (common_main.cpp:28-80).
 * A request's result is the same pattern list gs_mine_collect returns. */
typedef struct gs_server gs_server;

typedef struct gs_server_opts {
  int64_t budget_bytes; /* embedding-store bytes for admission; 0 = half the free device memory */
  int64_t pool_bytes;   /* hard cap of the server's device pool; 0 = 70% of free device memory */
  int32_t max_active;   /* requests mined at once; 0 = 64 */
  int32_t wave_nodes;   /* DFS-tree nodes per launch; 0 = default */
  int32_t threads;      /* host threads for the canonicality check; 0 = all cores */
  int32_t label_style;  /* GS_LABELS_FULL or GS_LABELS_SEQ for the results */
  int32_t extension;    /* GS_EXTENSION_RMPATH (default), GS_EXTENSION_LISTS or GS_EXTENSION_AUTO, as in
                           gs_mine_opts */
  int32_t reserved;
} gs_server_opts;

enum { GS_REQ_QUEUED = 0, GS_REQ_RUNNING = 1, GS_REQ_DONE = 2, GS_REQ_CANCELLED = 3, GS_REQ_FAILED = 4 };

typedef struct gs_request_info {
  int32_t state;       /* GS_REQ_* */
  gs_status status;    /* the error of a failed request, else GS_OK */
  int64_t patterns;    /* frequent patterns found (when done) */
  double queue_ms;     /* submission to admission */
  double latency_ms;   /* submission to completion (when done) */
  int64_t peak_bytes;  /* embedding-store bytes the request held at its peak */
} gs_request_info;

typedef struct gs_server_stats {
  int64_t submitted, completed, cancelled, failed, queued, running;
  int64_t max_running;     /* most requests mined at once so far */
  int64_t patterns;        /* over completed requests */
  double p50_ms, p99_ms, mean_ms;  /* latency of completed requests, nearest rank */
  double wall_ms;          /* since creation */
  double busy_ms;          /* time with at least one request admitted */
  int64_t budget_bytes, reserved_bytes, pool_used_bytes, peak_pool_bytes;
  int64_t waves, launches;
} gs_server_stats;

GS_API void gs_server_opts_default(gs_server_opts *opts);
/* Starts the server thread; the GPU is first touched by the first request. */
GS_API gs_status gs_server_create(const gs_server_opts *opts, gs_server **out);
/* Registers a database (borrowed: it must outlive the server).  It is made
 * resident on the device by the first request that uses it. */
GS_API gs_status gs_server_add_db(gs_server *srv, gs_db *db, int32_t *db_id);
/* Queues a request.  minsup is checked now (GS_ERR_MINSUP_TOO_SMALL /
 * GS_ERR_MINSUP_TOO_LARGE as gs_mine); max_edges 0 = no cap. */
GS_API gs_status gs_server_submit(gs_server *srv, int32_t db_id, int32_t abs_minsup, int32_t max_edges,
                                  int64_t *request_id);
/* Waits up to wait_ms (0 = do not wait, < 0 = until it ends) for the request
 * to end, then fills info.  Returns GS_ERR_TIMEOUT if it is still queued or
 * running.  Once it has ended and out is not NULL, *out receives its
 * patterns (free with gs_patterns_free; NULL unless done) and the request is
 * forgotten: later calls with its id return GS_ERR_USAGE. */
GS_API gs_status gs_server_poll(gs_server *srv, int64_t request_id, int32_t wait_ms, gs_request_info *info,
                                gs_patterns **out);
/* Cancels a queued or running request (a running one stops at its next wave). */
GS_API gs_status gs_server_cancel(gs_server *srv, int64_t request_id);
GS_API gs_status gs_server_get_stats(gs_server *srv, gs_server_stats *stats);
/* Cancels what is left, stops the thread, frees the server's device memory. */
GS_API void gs_server_destroy(gs_server *srv);

/* Autotuner: picks the wave options for a workload (the databases mined
 * together at their minsups, as gs_mine_batch would).  Coordinate descent
 * over wave_nodes (1024..16384), wave_rows (2^22..2^25), count_grid
 * (16..96 blocks per SM) and deep_nodes (1, 256, 1024); every trial is a complete mining pass with the
 * patterns counted, not emitted, best of two on the host clock, and a value
 * is taken only when it is 2% faster.  opts: in, the starting options (other
 * fields are kept); out, the tuned ones.  No counterpart in the reference,
 * whose launch shapes come from a fixed cuda_configurator. */
typedef struct gs_tune_report {
  int32_t trials;
  int32_t wave_nodes;
  int64_t wave_rows;
  int32_t count_grid;
  int32_t deep_nodes;
  double base_ms;  /* the starting options */
  double best_ms;  /* the tuned options */
  int32_t schedulers;
} gs_tune_report;
GS_API gs_status gs_autotune(gs_db *const *dbs, int32_t n, const int32_t *abs_minsups, gs_mine_opts *opts,
                             gs_tune_report *report);

/* Support of candidate DFS edges from extension records: support[k] = the
 * number of distinct graph ids among the records whose key is k, computed on
 * the GPU with one support bitmap per key.  The GPU form of
 * compute_support_remapped_db_multiple_dfs (src/gspan_cuda/compute_support.cpp:
 * 885-960), which counts records x candidates flags.  Host arrays; keys in
 * [0, n_keys), graph ids in [0, n_graphs), else GS_ERR_USAGE. */
GS_API gs_status gs_support_count(const int32_t *keys, const int32_t *graph_ids, int64_t n_records, int32_t n_keys,
                                  int32_t n_graphs, int32_t *support);

/* gs_support_count for callers that cannot allocate device memory: code that
 * runs inside another framework's memory arena or allocator (which must own
 * and account for every device allocation), processes given a fixed device
 * memory budget up front, and code paths that must not incur the implicit
 * device synchronisation cudaMalloc/cudaFree can cause.  No counterpart in
 * the reference.
 *
 * It allocates nothing.  The caller passes DEVICE pointers it owns: keys and
 * graph ids (n_records each) and support (n_keys int32, written by the call).
 * The only scratch, the support bitmaps, is a fixed 4 MiB device array inside
 * this library that every GPU which loads the library holds until the process
 * exits; it must hold n_keys * ceil(n_graphs / 32) 32-bit words, at most
 * GS_NOALLOC_MAX_BITMAP_WORDS (1,048,576), else the call returns
 * GS_ERR_LIMIT and launches nothing.  Records whose key or graph id is out of
 * range are ignored.  The work runs on the device that holds d_support (the
 * caller's current device is restored before returning); `stream` (a
 * cudaStream_t; NULL = the default stream) must belong to that device, else
 * GS_ERR_USAGE.  The call queues the work and returns without synchronising;
 * support is ready when the stream reaches that point.  A CUDA error left
 * pending by earlier work of the calling thread is reported as GS_ERR_CUDA
 * before anything is launched, and left in place for its owner.
 *
 * The first call on each device looks up the scratch's device address
 * (cudaGetSymbolAddress, which may load the module) and keeps it for the life
 * of the process: make that first call before any stream capture, and do not
 * call it again after cudaDeviceReset (the kept address is then stale).
 * Every call shares the one scratch array and clears the part it uses before
 * use, so calls that may overlap on the GPU (different streams, or threads
 * without ordering) race and give wrong results: serialise them. */
#define GS_NOALLOC_MAX_BITMAP_WORDS (1u << 20)
GS_API gs_status gs_support_count_noalloc(const int32_t *d_keys, const int32_t *d_graph_ids, int64_t n_records,
                                          int32_t n_keys, int32_t n_graphs, int32_t *d_support, void *stream);

/* Backward child column: the rows of an embedding column that carry one
 * backward extension.  The GPU form of gspan_cuda::filter_backward_embeddings
 * (src/gspan_cuda/filter_backward.cpp:288-352), which marks the rows named by
 * the matching extension records, scans the marks and copies the marked
 * elements.  Host arrays:
 *   column   n_rows elements {vertex, back_link} (2 x int32 each), the
 *            parent's last embedding column;
 *   records  n_records extension records in the reference's
 *            extension_element_t layout (cuda_datastructures.hpp:13-55),
 *            8 x int32 {from, to, fromlabel, elabel, tolabel, from_grph,
 *            to_grph, row};
 *   dfs      the backward DFS edge {from, to, fromlabel, elabel, tolabel};
 *            a record matches when all five fields are equal;
 *   out      room for n_rows elements: receives the elements of the rows
 *            named by matching records, in row order, each once;
 *   n_out    receives their count.
 * GS_ERR_USAGE for a forward edge (from < to: the reference aborts), a
 * matching record whose row is outside [0, n_rows), or a null array that
 * must be given; GS_ERR_LIMIT beyond 2^31 - 2 rows. */
GS_API gs_status gs_filter_backward(const int32_t *column, int64_t n_rows, const int32_t *records, int64_t n_records,
                                    const int32_t *dfs, int32_t *out, int64_t *n_out);

/* The reference's segmented scan over packed uint32 values
 * (cuda_segmented_scan::scan, src/reduction/cuda_segmented_scan.hpp:7-24;
 * packed layout of src/reduction/segscanpacked.cu): bit 31 of an element
 * starts a new segment (element 0 always starts one), bits 0-30 are its
 * value.  out[i] (n values, unpacked) = the sum of the values of i's segment
 * up to and including i, or before i when `exclusive` is set, modulo 2^32.
 * Computed on the GPU by two plain scans (values, flags).  Host arrays; out
 * may alias data.  GS_ERR_LIMIT beyond 2^31 - 2 elements. */
GS_API gs_status gs_segmented_scan(const uint32_t *data, int64_t n, int32_t exclusive, uint32_t *out);

/* The reference's segmented reduction (cuda_segmented_reduction::reduce,
 * src/reduction/cuda_segmented_reduction.cpp:98-134): the segments are given
 * as `groups` runs of segment_count[g] segments of segment_sizes[g] elements
 * each; results[j] = the segmented scan (inclusive or exclusive) at the last
 * element of segment j, i.e. the segment's sum (without its last value when
 * exclusive).  *n_results receives the number of segments; results must hold
 * that many.  GS_ERR_USAGE when the segments run past the array. */
GS_API gs_status gs_segmented_reduce(const uint32_t *data, int64_t n, const uint32_t *segment_count,
                                     const uint32_t *segment_sizes, int32_t groups, int32_t exclusive,
                                     uint32_t *results, int64_t *n_results);

/* Canonicality of a DFS code (n_edges tuples {from, to, fromlabel, elabel,
 * tolabel}, either label convention): 1 if minimal, 0 if not, -1 on bad
 * input.  Same semantics as the sequential reference's gSpan::is_min
 * (src/gspan/ismin.cpp:36-143), which DFSCode::dfs_code_is_min
 * (src/globals/dfs_ismin.cpp:23-160) mirrors; host-only, no GPU needed. */
GS_API int32_t gs_dfs_code_is_min(const int32_t *dfs5xN, int32_t n_edges);

/* Frees the miner's device pool and scratch buffers, and returns the
 * device ingest's cached pool memory. */
GS_API void gs_engine_reset(void);
/* Caps the device pool (bytes; 0 = 70% of free device memory). */
GS_API void gs_engine_set_pool_bytes(int64_t bytes);

#ifdef __cplusplus
}
#endif

#endif /* GSPAN_GB300_H */
