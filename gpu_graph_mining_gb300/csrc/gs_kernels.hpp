// Launchers for the mining kernels (gs_kernels.cu).  All launches go to the
// given stream; none synchronises.  `err` receives bit flags when a kernel's
// consistency checks fail (1: graph rank out of range, 2: back-link, vertex or
// label-pair index out of range, 4: more child rows than counted, 8: a key's
// embedding count past 2^31 - 1); the offending access is skipped, never
// performed.
#pragma once
#include <cstdint>
#include <cstring>
#include <cuda_runtime.h>

#include "gs_device.hpp"

namespace gsgb {

// SMs of device 0 (the library's device), read once; grid caps are per SM.
int sm_count();

// Extension records of the count pass, int4 {key field, x, y, graph rank}: the
// key field holds the wave key in bits 0-26 and the counter copy the
// extension was counted in in bits 27-30 (-1: an unused slot).  A forward
// extension has (x, y) = (new vertex, parent row), a backward one the copy of
// the parent row's last column element.
constexpr int kRecCopyShift = 27;
constexpr int kRecKeyMask = (1 << kRecCopyShift) - 1;

struct ListBuild;

// A kernel launch as data: function, shape and argument values.  run()
// launches it on a stream; params() gives the argument pointers a CUDA graph
// kernel node takes (the graph copies the values when the node is set).
struct KernelCall {
  const void *func = nullptr;
  dim3 grid, block;
  unsigned smem = 0;
  template <class T> void arg(const T &v)
  {
    used_ = (used_ + alignof(T) - 1) & ~(alignof(T) - 1);
    std::memcpy(store_ + used_, &v, sizeof(T));
    off_[n_++] = (unsigned short)used_;
    used_ += sizeof(T);
  }
  void **params()
  {
    for(int i = 0; i < n_; i++) ptr_[i] = store_ + off_[i];
    return ptr_;
  }
  cudaError_t run(cudaStream_t s) { return cudaLaunchKernel(func, grid, block, params(), smem, s); }

private:
  alignas(16) unsigned char store_[384];
  unsigned short off_[16];
  void *ptr_[16];
  int n_ = 0;
  size_t used_ = 0;
};

// Root level of a group of jobs: a warp per 32 vertices of a job walks their
// adjacency; every directed entry (v -> w) with label(v) <= label(w) is a
// 1-edge embedding (get_forward_root, src/globals/graph_types.cpp:365-375).
// Sets support-bitmap bit [key][graph] and counts embeddings per key in the
// warp's counter copy; then per key of the group: tot[key] = its embeddings,
// copy q >= 1 = the count of copies 0..q-1 and copy 0 = 0 (the materialise
// pass's cursors).  tiles = the group's warp tiles; total_keys = its keys.
void launch_root_count(const RootJob *jobs, int32_t njobs, long long tiles, const DevDB *dbs, uint32_t *bm,
                       int32_t *cnt, int32_t *tot, int32_t total_keys, unsigned long long *bytes, cudaStream_t s);
// Writes the two columns and graph ranks of every selected root key of the
// group (childmap over the group's keys), with the counter copies as cursors.
void launch_root_materialize(const RootJob *jobs, int32_t njobs, long long tiles, const DevDB *dbs,
                             const uint32_t *bm, const int32_t *bmx, int32_t *cursor, const int32_t *childmap,
                             const ChildOut *outs, unsigned int *err, cudaStream_t s);

// Wave level (gs_wave.cu): a warp per 32 embedding rows of the wave's nodes.
// kmax = the largest column count of the wave's nodes (selects the instance
// sized for 8/16/32/64 pattern vertices); collen[] parallels coltab[]: the
// length of every column.
// small_graphs: every graph of the wave's databases has <= 64 vertices.
// rule_skip: in databases with sorted adjacency (DevDB::adj_sorted), a
// right-most-path vertex's entries below its forward rule are bisected past
// instead of scanned.
KernelCall wave_count_call(const NodeDesc *nodes, int32_t nnodes, long long total_tiles, int32_t kmax,
                           bool small_graphs, const int2 *const *coltab, const int32_t *collen, const SlotDesc *slots,
                           const int32_t *vtab, const DevDB *dbs, uint32_t *bm, int32_t *cnt,
                           unsigned long long *bytes, unsigned int *err, int4 *rec, long long rec_cap,
                           unsigned long long *rec_n, int32_t grid_per_sm, int32_t cnt_copies,
                           long long cnt_stride, bool join, bool rule_skip);
void launch_wave_materialize(const NodeDesc *nodes, int32_t nnodes, long long total_tiles, int32_t kmax,
                             bool small_graphs,
                             const int2 *const *coltab, const int32_t *collen, const SlotDesc *slots,
                             const int32_t *vtab, const DevDB *dbs, const uint32_t *bm, const int32_t *bmx,
                             const int32_t *childmap, int32_t *cursor, const ChildOut *outs,
                             unsigned long long *bytes, unsigned int *err, bool join, bool rule_skip,
                             cudaStream_t s);

// Materialise from the count pass's records {wave key, x, y, graph rank}:
// children whose key is selected get column element (x, y) and their graph
// rank.  keyword[key] = the key's first support-bitmap word.
// cursor: the wave's counter copies after selection (copy q of a key starts
// at the count of copies 0..q-1), cursor_stride apart; a record's copy is in
// bits 27-30 of its key field.
// lists (may be null): also counts each list row's entries at list_cnt[row]
// (lists strategy, launch_fill_lists)
void launch_materialize_records(const int4 *rec, long long n, const int32_t *childmap, const long long *keyword,
                                const uint32_t *bm, const int32_t *bmx, int32_t *cursor, long long cursor_stride,
                                const ChildOut *outs, unsigned long long *bytes, unsigned int *err,
                                const ListBuild *lists, int32_t *list_cnt, cudaStream_t s);

// Extension records given as (key, graph id) pairs: sets bit [key][graph].
// Keys and graph ids must be in range (checked by the caller).
void launch_records_bitmap(const int32_t *keys, const int32_t *gids, long long n, int32_t words, uint32_t *bm,
                           cudaStream_t s);

// One warp per key: support = popcount of the key's bitmap words; bmx gets
// the exclusive prefix popcount of each word (for graph-rank lookups).
// Wave support with candidate selection (k_screen_keys, k_count_listed).
// counters: [0] selected keys, [1] embeddings of all keys, [2] keys listed for
// counting; listed and sel hold total_keys entries.  *err_copy = *err (the
// consistency flags after the count pass).
// lnode (lists strategy, may be null): reset to -1 for every key with extensions
KernelCall screen_keys_call(const NodeDesc *nodes, int32_t nnodes, int32_t total_keys, int32_t *cnt,
                            int32_t cnt_copies, long long cnt_stride, int32_t *childmap, int2 *listed,
                            unsigned long long *counters, unsigned int *err, unsigned long long *err_copy,
                            int32_t *lnode);
// lnode (lists strategy, may be null): lnode[key] = the key's node for every
// frequent forward key
KernelCall count_listed_call(const NodeDesc *nodes, const int2 *listed, const uint32_t *bm, int32_t *cnt,
                             int32_t *bmx, long long *keyword, int4 *sel, int32_t sel_cap,
                             unsigned long long *counters, int32_t *lnode);
// Canonicality of the selected candidates (gs_ismin.cu): the low two bits of
// sel[i].w (above them the candidate's node) = 1 minimal, 0 not minimal, 2
// left to the host.  codes = the wave's code table.
KernelCall is_min_call(const NodeDesc *nodes, int32_t nnodes, const SlotDesc *slots, const DevDB *dbs,
                       const int32_t *codes, int4 *sel, int32_t sel_cap, const unsigned long long *counters);
// childmap[pairs[i].x] = pairs[i].y, and cursor[0..ncursor) = 0
void launch_scatter_childmap(const int2 *pairs, int32_t n, int32_t *childmap, int32_t *cursor, int32_t ncursor,
                             cudaStream_t s);
void launch_support(const NodeDesc *nodes, int32_t nnodes, int32_t total_keys, const uint32_t *bm, int32_t *bmx,
                    int32_t *support, cudaStream_t s);

// Lists strategy: the per-row lists of a wave's nodes' frequent forward
// extensions, built from the count pass's records (ListBuild, gs_lists.cuh):
// the records materialise pass adds each list row's entry count at off[r + 1]
// (off zeroed before), then launch_fill_lists turns the counts into offsets
// off[0..nrows_total] and writes ent[off[r] ..], the entries {neighbour, the
// node's forward key} of list row r; entries past ent_cap set err bit 4 and
// are dropped.  scratch holds list_scan_scratch(nrows_total) ints.
// The lists of one wave: lnode[wave key] = the node of a frequent forward key
// (else -1); node n's rows are list rows rowbase[n] .. (rowbase[n] < 0: the
// node keeps no lists).
struct ListBuild {
  const int32_t *lnode;
  const NodeDesc *nodes;
  const int32_t *rowbase;
};
int64_t list_scan_scratch(int64_t n);

// The reference's packed segmented scan (cuda_segmented_scan::scan,
// src/reduction/cuda_segmented_scan.hpp): bit 31 of an element starts a new
// segment, bits 0-30 are its value; out[i] = the sum of the values of i's
// segment up to i (inclusive) or before i (exclusive), modulo 2^32.
// scratch: segmented_scan_scratch(n) ints.  out may alias x.
int64_t segmented_scan_scratch(int64_t n);
void launch_segmented_scan(const uint32_t *x, int64_t n, int exclusive, int32_t *scratch, uint32_t *out,
                           cudaStream_t s);
// res[j] = scanned[ends[j]]; an index outside [0, n) sets bit 0 of *err.
void launch_gather_ends(const uint32_t *scanned, int64_t n, const long long *ends, int64_t m, uint32_t *res,
                        unsigned int *err, cudaStream_t s);

// Backward child column on its own (gs_filter_backward; the reference's
// filter_backward_embeddings, src/gspan_cuda/filter_backward.cpp:288-352):
// out = the elements of col at the rows named by the records (8 ints each,
// {from, to, fromlabel, elabel, tolabel, from_grph, to_grph, row}) equal to
// the edge e[0..5), in row order; pos[nrows + 1] (zeroed by the caller) ends
// holding the exclusive scan of the row flags (pos[nrows] = the count).  scratch holds
// filter_backward_scratch(nrows) ints.
int64_t filter_backward_scratch(int64_t nrows);
void launch_filter_backward(const int2 *col, int64_t nrows, const int32_t *rec, int64_t nrec, const int32_t *e,
                            int32_t *pos, int32_t *scratch, int2 *out, cudaStream_t s);
void launch_fill_lists(const int4 *rec, long long nrec, const ListBuild &lb, int32_t *off, int64_t nrows_total,
                       int2 *ent, int64_t ent_cap, int32_t *scratch, unsigned int *err, cudaStream_t s);

}  // namespace gsgb
