// Device-side database ingest: the reference's cudabin arrays (host memory)
// become the miner's device database without a host conversion.  The GPU
// counterpart of graph_database_cuda::copy_to_device plus the host readers'
// conversion (src/globals/cuda_graph_types.cpp:65-127, dbio.cpp:381-404):
//
//   1. per graph: valid vertex slots (a prefix of the graph's max_vc slots)
//      and adjacency entries; exclusive scans give vertex and entry bases;
//   2. per vertex slot: CSR offsets, graph ids, neighbours as global vertex
//      ids, raw labels; the checks of the host reader (offsets tile the edge
//      array, neighbours stay in their graph) and of simple graphs (no self
//      loops, no parallel edges);
//   3. labels compacted order-preservingly through presence tables over the
//      label value range (a scan turns presence into dense ids);
//   4. the (source label, edge label, target label) presence table, scanned
//      once: every pair's dense index, each label's first root key and the
//      pair codes;
//   5. the packed adjacency entries and their pair indices.
//
// Accepts exactly what gs_db_from_arrays accepts (same checks), and the
// device database is identical to the one the host path uploads.
#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <mutex>
#include <string>
#include <vector>

#include "gs_engine.hpp"
#include "gs_kernels.hpp"

namespace gsgb {

#define CK(call) cuda_check((call), #call)

namespace {

constexpr int kThreads = 256;
// consistency flags
constexpr unsigned kBadTile = 1, kBadLeave = 2, kSelfLoop = 4, kParallel = 8;

inline unsigned blocks_for(long long n)
{
  long long b = (n + kThreads - 1) / kThreads;
  if(b < 1) b = 1;
  const long long cap = 64LL * gsgb::sm_count();
  return (unsigned)(b < cap ? b : cap);
}

// ---- exclusive scan of int64 values, three passes per level
__global__ void k_scan_blocks(const long long *in, long long *out, long long n, long long *block_sums)
{
  __shared__ long long warp_tot[kThreads / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const long long i = (long long)blockIdx.x * kThreads + threadIdx.x;
  const long long v = i < n ? in[i] : 0;
  long long incl = v;
  for(int o = 1; o < 32; o <<= 1) {
    const long long t = __shfl_up_sync(0xffffffffu, incl, o);
    if(lane >= o) incl += t;
  }
  if(lane == 31) warp_tot[w] = incl;
  __syncthreads();
  if(w == 0) {
    long long x = lane < kThreads / 32 ? warp_tot[lane] : 0;
    for(int o = 1; o < 32; o <<= 1) {
      const long long t = __shfl_up_sync(0xffffffffu, x, o);
      if(lane >= o) x += t;
    }
    if(lane < kThreads / 32) warp_tot[lane] = x;
  }
  __syncthreads();
  const long long before = w > 0 ? warp_tot[w - 1] : 0;
  if(i < n) out[i] = before + incl - v;
  if(threadIdx.x == kThreads - 1) block_sums[blockIdx.x] = before + incl;
}

__global__ void k_scan_add(long long *out, long long n, const long long *block_off)
{
  const long long i = (long long)blockIdx.x * kThreads + threadIdx.x;
  if(i < n) out[i] += block_off[blockIdx.x];
}

// Scratch of one ingest: stream-ordered allocations from a pool that keeps
// its memory between ingests (up to kKeepBytes), so that repeated ingests of
// similar databases allocate and free without driver calls.  Freed in stream
// order when the ingest returns.
struct Scratch {
  cudaStream_t s;
  cudaMemPool_t pool;
  std::vector<void *> ptrs;
  cudaEvent_t after = nullptr;  // work of another stream on the scratch, ordered before the frees
  ~Scratch()
  {
    if(after) cudaStreamWaitEvent(s, after, 0);
    for(void *p : ptrs) cudaFreeAsync(p, s);
  }
  template <class T> T *get(size_t n)
  {
    void *p = nullptr;
    if(cudaMallocFromPoolAsync(&p, sizeof(T) * std::max<size_t>(n, 1), pool, s) != cudaSuccess) {
      cudaGetLastError();
      throw Error(ST_ERR_NOMEM, "device ingest: out of device memory");
    }
    ptrs.push_back(p);
    return (T *)p;
  }
};

// out[i] = sum of in[0..i) for i in [0, n]; out must hold n + 1 values
void scan_exclusive(const long long *in, long long *out, long long n, Scratch &sc)
{
  cudaStream_t s = sc.s;
  const long long nb = (n + kThreads - 1) / kThreads;
  if(nb <= 0) {
    CK(cudaMemsetAsync(out, 0, sizeof(long long), s));
    return;
  }
  long long *sums = sc.get<long long>(nb + 1);
  k_scan_blocks<<<(unsigned)nb, kThreads, 0, s>>>(in, out, n, sums);
  if(nb == 1) {
    // one block: its sum is the total
    CK(cudaMemcpyAsync(out + n, sums, sizeof(long long), cudaMemcpyDeviceToDevice, s));
  } else {
    long long *offs = sc.get<long long>(nb + 1);
    scan_exclusive(sums, offs, nb, sc);
    k_scan_add<<<(unsigned)nb, kThreads, 0, s>>>(out, n, offs);
    // the total, after the last element
    CK(cudaMemcpyAsync(out + n, offs + nb, sizeof(long long), cudaMemcpyDeviceToDevice, s));
  }
}

// ---- 1. per graph: valid slots and adjacency entries
__global__ void k_graphs(int G, int maxv, long long slots, long long esz, const int32_t *voff, long long *gnv,
                         long long *gadj, unsigned *flags)
{
  for(long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x; g < G; g += (long long)gridDim.x * blockDim.x) {
    const long long base = g * maxv;
    int nv = 0;
    while(nv < maxv && voff[base + nv] != -1) nv++;
    gnv[g] = nv;
    gadj[g] = 0;
    if(nv > 0) {
      const long long nxt = (g + 1) * maxv <= slots ? (g + 1) * maxv : slots;
      const long long b0 = voff[base], e1 = voff[nxt];
      if(b0 < 0 || e1 < b0 || e1 > esz) atomicOr(flags, kBadTile);
      else gadj[g] = e1 - b0;
    }
  }
}

// ---- 2. per vertex slot: offsets, graph ids, neighbours, raw labels, checks
__global__ void k_vertices(int G, int maxv, long long slots, long long esz, const int32_t *voff,
                           const int32_t *vlab, const int32_t *edges, const int32_t *elab, const long long *gnv,
                           const long long *vbase, const long long *gpos, int32_t *off, int32_t *vgraph,
                           int32_t *vgbase, int32_t *vl_raw, int32_t *adj_to, int32_t *el_raw, unsigned *flags)
{
  for(long long slot = (long long)blockIdx.x * blockDim.x + threadIdx.x; slot < slots;
      slot += (long long)gridDim.x * blockDim.x) {
    const long long g = slot / maxv, v = slot - g * maxv, base = g * maxv;
    const long long nv = gnv[g];
    if(v >= nv) continue;
    long long nxt = v + 1 < nv ? slot + 1 : (g + 1) * maxv;
    if(nxt > slots) nxt = slots;
    const long long b0 = voff[slot], b1 = voff[nxt], first = voff[base];
    const long long gv = vbase[g] + v;
    const long long pos = gpos[g] + (b0 - first);
    if(b0 < 0 || b1 < b0 || b1 > esz || pos < gpos[g] || pos + (b1 - b0) > gpos[g + 1]) {
      atomicOr(flags, kBadTile);
      continue;
    }
    off[gv] = (int32_t)pos;
    vgraph[gv] = (int32_t)g;
    vgbase[gv] = (int32_t)vbase[g];
    vl_raw[gv] = vlab[slot];
    const bool small = nv <= 64;
    unsigned long long seen = 0;
    for(long long k = b0; k < b1; k++) {
      const long long t = (long long)edges[k] - base;
      if(t < 0 || t >= nv) {
        atomicOr(flags, kBadLeave);
        break;
      }
      if(t == v) atomicOr(flags, kSelfLoop);
      if(small) {
        if((seen >> t) & 1ull) atomicOr(flags, kParallel);
        seen |= 1ull << t;
      } else {
        for(long long q = b0; q < k; q++)
          if(edges[q] == edges[k]) {
            atomicOr(flags, kParallel);
            break;
          }
      }
      adj_to[pos + (k - b0)] = (int32_t)(vbase[g] + t);
      el_raw[pos + (k - b0)] = elab[k];
    }
  }
}

// ---- 3. labels
// block-reduced: one pair of atomics per block (the range is one address)
__global__ void k_minmax(const int32_t *x, long long n, int *mn, int *mx)
{
  __shared__ int slo[kThreads / 32], shi[kThreads / 32];
  int lo = INT32_MAX, hi = INT32_MIN;
  for(long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    lo = min(lo, x[i]);
    hi = max(hi, x[i]);
  }
  for(int o = 16; o > 0; o >>= 1) {
    lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if(lane == 0) {
    slo[w] = lo;
    shi[w] = hi;
  }
  __syncthreads();
  if(threadIdx.x == 0) {
    for(int k = 1; k < kThreads / 32; k++) {
      lo = min(lo, slo[k]);
      hi = max(hi, shi[k]);
    }
    atomicMin(mn, lo);
    atomicMax(mx, hi);
  }
}

__global__ void k_mark(const int32_t *x, long long n, int lo, long long *present)
{
  for(long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
  {
    // a label alphabet is small: most elements find their flag already set
    long long *f = present + ((long long)x[i] - lo);
    if(!*f) *f = 1;
  }
}

// dense[i] = rank of x[i] among the distinct values; of[rank] = value
__global__ void k_relabel(int32_t *x, long long n, int lo, const long long *rank)
{
  for(long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    x[i] = (int32_t)rank[(long long)x[i] - lo];
}

__global__ void k_label_values(const long long *present, const long long *rank, long long range, int lo, int32_t *of)
{
  for(long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < range; i += (long long)gridDim.x * blockDim.x)
    if(present[i]) of[rank[i]] = (int32_t)(lo + i);
}

// ---- 4. pair table
// A label alphabet gives a small table that every thread hits: up to
// kSmemTab entries each block marks its own copy in shared memory and merges
// it once; larger tables are marked in place (read before write).
constexpr long long kSmemTab = 32768;

__global__ void k_pairs_seen(const int32_t *off, long long V, const int32_t *vl, const int32_t *adj_to,
                             const int32_t *el, int EL, int VL, long long *seen, long long tab)
{
  extern __shared__ unsigned char flags[];
  const bool local = tab <= kSmemTab;
  if(local) {
    for(long long i = threadIdx.x; i < tab; i += blockDim.x) flags[i] = 0;
    __syncthreads();
  }
  for(long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < V; v += (long long)gridDim.x * blockDim.x) {
    const long long a = vl[v];
    for(long long k = off[v]; k < off[v + 1]; k++) {
      const long long x = (a * EL + el[k]) * VL + vl[adj_to[k]];
      if(local) {
        flags[x] = 1;
      } else if(!seen[x]) {
        seen[x] = 1;
      }
    }
  }
  if(local) {
    __syncthreads();
    for(long long i = threadIdx.x; i < tab; i += blockDim.x)
      if(flags[i] && !seen[i]) seen[i] = 1;
  }
}

// pair index within the source label's pairs, pair codes, first key of each label
__global__ void k_pairs_index(const long long *seen, const long long *rank, int EL, int VL, int32_t *pair_idx,
                              int32_t *pair_code, int32_t *root_off)
{
  const long long tab = (long long)VL * EL * VL;
  for(long long x = (long long)blockIdx.x * blockDim.x + threadIdx.x; x < tab; x += (long long)gridDim.x * blockDim.x) {
    const long long a = x / ((long long)EL * VL), r = x - a * EL * VL;
    const long long row0 = rank[a * EL * VL];
    if(r == 0) root_off[a] = (int32_t)row0;
    if(seen[x]) {
      pair_idx[x] = (int32_t)(rank[x] - row0);
      pair_code[rank[x]] = (int32_t)(((r / VL) << 16) | (r % VL));
    } else {
      pair_idx[x] = -1;
    }
  }
}

// ---- 5. packed entries: adj_in in input order (for downloads), adj with each
// vertex's entries ascending when sort (by the vertex's thread: a sorting
// network in registers up to 8 entries, else an insertion sort in place; the
// caller sorts only when no vertex has more than kSortDegree entries), and
// the pair index of every adj entry
// an insertion sort of d entries makes about d * d / 4 dependent global
// accesses: 256 bounds one thread's sort to about 16,000
constexpr int kSortDegree = 256;

__global__ void k_pack(const int32_t *off, long long V, const int32_t *vl, const int32_t *adj_to, const int32_t *el,
                       const int32_t *pair_idx, int EL, int VL, bool sort, unsigned long long *adj_in,
                       unsigned long long *adj, int32_t *adj_pair)
{
  for(long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < V; v += (long long)gridDim.x * blockDim.x) {
    const long long a = vl[v], a0 = off[v], a1 = off[v + 1];
    auto entry = [&](long long k) {
      const uint32_t w = (uint32_t)adj_to[k];
      const uint32_t hi = ((uint32_t)el[k] << 16) | (uint32_t)vl[w];
      return ((unsigned long long)hi << 32) | w;
    };
    auto emit = [&](long long k, unsigned long long x) {
      adj[k] = x;
      adj_pair[k] = pair_idx[(a * EL + (long long)(x >> 48)) * VL + (long long)((x >> 32) & 0xffffu)];
    };
    if(sort && a1 - a0 <= 8) {
      // up to 8 entries: held in registers (padded with the largest value)
      // and ordered by Batcher's odd-even merge network (19 comparators)
      unsigned long long r[8];
#pragma unroll
      for(int t = 0; t < 8; t++) {
        r[t] = a0 + t < a1 ? entry(a0 + t) : ~0ull;
        if(a0 + t < a1) adj_in[a0 + t] = r[t];
      }
      constexpr int net[19][2] = { { 0, 1 }, { 2, 3 }, { 4, 5 }, { 6, 7 }, { 0, 2 }, { 1, 3 }, { 4, 6 },
                                   { 5, 7 }, { 1, 2 }, { 5, 6 }, { 0, 4 }, { 1, 5 }, { 2, 6 }, { 3, 7 },
                                   { 2, 4 }, { 3, 5 }, { 1, 2 }, { 3, 4 }, { 5, 6 } };
#pragma unroll
      for(int c = 0; c < 19; c++) {
        const unsigned long long x = r[net[c][0]], y = r[net[c][1]];
        r[net[c][0]] = x < y ? x : y;
        r[net[c][1]] = x < y ? y : x;
      }
#pragma unroll
      for(int t = 0; t < 8; t++)
        if(a0 + t < a1) emit(a0 + t, r[t]);
      continue;
    }
    for(long long k = a0; k < a1; k++) {
      const unsigned long long x = entry(k);
      adj_in[k] = x;
      long long j = k;
      if(sort)
        for(; j > a0 && adj[j - 1] > x; --j) adj[j] = adj[j - 1];
      adj[j] = x;
    }
    for(long long k = a0; k < a1; k++) emit(k, adj[k]);
  }
}

// the largest vertex degree
__global__ void k_max_degree(const int32_t *off, long long V, int *mx)
{
  __shared__ int shi[kThreads / 32];
  int hi = 0;
  for(long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < V; v += (long long)gridDim.x * blockDim.x)
    hi = max(hi, off[v + 1] - off[v]);
  for(int o = 16; o > 0; o >>= 1) hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  if((threadIdx.x & 31) == 0) shi[threadIdx.x >> 5] = hi;
  __syncthreads();
  if(threadIdx.x == 0) {
    for(int k = 1; k < kThreads / 32; k++) hi = max(hi, shi[k]);
    atomicMax(mx, hi);
  }
}

__global__ void k_max_ll(const long long *x, long long n, int *mx)
{
  __shared__ int shi[kThreads / 32];
  int hi = 0;
  for(long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    hi = max(hi, (int)x[i]);
  for(int o = 16; o > 0; o >>= 1) hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  if((threadIdx.x & 31) == 0) shi[threadIdx.x >> 5] = hi;
  __syncthreads();
  if(threadIdx.x == 0) {
    for(int k = 1; k < kThreads / 32; k++) hi = max(hi, shi[k]);
    atomicMax(mx, hi);
  }
}

__global__ void k_narrow(const long long *x, long long n, int32_t *out)
{
  for(long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    out[i] = (int32_t)x[i];
}

// A 1,000,000-graph database (80 M adjacency entries) peaks at about 4.5 GB
// of scratch plus block; below that keep size every ingest re-mapped the
// difference, which measured tens of milliseconds on some steps.
constexpr unsigned long long kKeepBytes = 16ull << 30;

// Values read back to the host at the ingest's synchronisation points
// (pinned, so the copies are asynchronous).
struct ReadBack {
  long long v_total, e_total;
  unsigned flags, pad;
  int minmax[4];        // vertex labels min, max; edge labels min, max
  long long label_cnt[2];
  long long nkeys;
  int max_vertices, max_degree;
};

// Process-wide ingest state: the ingest stream and a copy stream, the
// scratch pool and the pinned read-back area.  Ingests are serialised by mu.
// Copies an int32 host array to the device by a kernel that reads the host
// memory in place: on a GPU that reaches pageable host memory through the
// host's page tables (address translation services, as over a Grace C2C
// link) this reads at the link's bandwidth with no driver staging through
// pinned buffers, so it neither waits on host memcpy threads nor varies
// with them.  16-byte loads when both ends are 16-byte aligned, 4-byte loads
// otherwise; four loads in flight per thread.
__global__ void __launch_bounds__(kThreads) k_pull(const int32_t *__restrict__ src, int32_t *__restrict__ dst,
                                                   long long n, int vec)
{
  const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long stride = (long long)gridDim.x * blockDim.x;
  long long done = 0;
  if(vec) {
    const long long n4 = n / 4;
    const int4 *s4 = reinterpret_cast<const int4 *>(src);
    int4 *d4 = reinterpret_cast<int4 *>(dst);
    long long i = tid;
    for(; i + 3 * stride < n4; i += 4 * stride) {
      const int4 a = s4[i], b = s4[i + stride], c = s4[i + 2 * stride], d = s4[i + 3 * stride];
      d4[i] = a;
      d4[i + stride] = b;
      d4[i + 2 * stride] = c;
      d4[i + 3 * stride] = d;
    }
    for(; i < n4; i += stride) d4[i] = s4[i];
    done = n4 * 4;
  }
  for(long long i = done + tid; i < n; i += stride) dst[i] = src[i];
}

struct IngestCtx {
  std::mutex mu;
  cudaStream_t s = nullptr, s_copy = nullptr;
  cudaEvent_t ev_alloc = nullptr, ev_copied = nullptr;
  cudaMemPool_t pool = nullptr;
  ReadBack *rb = nullptr;
  int32_t *meta = nullptr;   // pinned: label values, root offsets and pair codes read back
  size_t meta_cap = 0;
  bool direct = false;       // the GPU reads pageable host memory through the host's page tables

  void init()
  {
    if(s) return;
    CK(cudaSetDevice(0));
    {
      int pma = 0, ats = 0;
      if(cudaDeviceGetAttribute(&pma, cudaDevAttrPageableMemoryAccess, 0) != cudaSuccess ||
         cudaDeviceGetAttribute(&ats, cudaDevAttrPageableMemoryAccessUsesHostPageTables, 0) != cudaSuccess) {
        cudaGetLastError();
        pma = ats = 0;
      }
      const char *env = std::getenv("GS_INGEST_MEMCPY");  // 1: always copy through cudaMemcpyAsync
      direct = pma == 1 && ats == 1 && !(env && env[0] == '1');
    }
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = 0;
    CK(cudaMemPoolCreate(&pool, &props));
    unsigned long long keep = kKeepBytes;
    CK(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
    CK(cudaMallocHost(&rb, sizeof(ReadBack)));
    CK(cudaEventCreateWithFlags(&ev_alloc, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&ev_copied, cudaEventDisableTiming));
    CK(cudaStreamCreateWithFlags(&s_copy, cudaStreamNonBlocking));
    CK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  }
  int32_t *meta_buf(size_t n)
  {
    if(n > meta_cap) {
      if(meta) CK(cudaFreeHost(meta));
      meta = nullptr;
      meta_cap = 0;
      CK(cudaMallocHost(&meta, sizeof(int32_t) * n));
      meta_cap = n;
    }
    return meta;
  }
};

// Host array -> device: the in-place read kernel where the GPU reaches
// pageable host memory through the host's page tables, else cudaMemcpyAsync.
// In the first case the array's preferred location is set to host memory
// first: a GPU that reads the same host pages again and again (a database
// ingested repeatedly from the same arrays) may otherwise have the driver move
// them into its own memory (access-counter migration); a benchmark run that
// moved about a gigabyte of pages also had one mining pass 110 ms slower than
// the others.  The advice only keeps the pages where the caller put them; if
// the driver refuses it, the read goes ahead without it.
void pull_to_device(const IngestCtx &cx, int32_t *dst, const int32_t *src, long long n, cudaStream_t st)
{
  if(n <= 0) return;
  if(!cx.direct) {
    CK(cudaMemcpyAsync(dst, src, sizeof(int32_t) * (size_t)n, cudaMemcpyHostToDevice, st));
    return;
  }
  {
    cudaMemLocation host{};
    host.type = cudaMemLocationTypeHost;
    host.id = 0;
    if(cudaMemAdvise(src, sizeof(int32_t) * (size_t)n, cudaMemAdviseSetPreferredLocation, host) != cudaSuccess)
      cudaGetLastError();
  }
  const int vec = ((reinterpret_cast<uintptr_t>(src) | reinterpret_cast<uintptr_t>(dst)) & 15) == 0;
  const long long per = vec ? 16 : 4;  // elements per thread per pass of four loads
  long long b = (n + (long long)kThreads * per - 1) / ((long long)kThreads * per);
  b = std::max(1ll, std::min(b, 4ll * gsgb::sm_count()));
  k_pull<<<(unsigned)b, kThreads, 0, st>>>(src, dst, n, vec);
  CK(cudaGetLastError());
}

IngestCtx &ingest_ctx()
{
  static IngestCtx c;
  return c;
}

// Dense ids for the labels x[0..n) in place, order-preserving, given the
// value range [lo, hi]; *cnt receives the number of distinct values (read
// back later) and the returned device array of.  of[rank] = value.
int32_t *compact_labels(int32_t *x, long long n, int lo, int hi, long long *cnt, Scratch &sc)
{
  cudaStream_t s = sc.s;
  const long long range = (long long)hi - (long long)lo + 1;
  if(range > (1ll << 22))
    throw Error(ST_ERR_LIMIT, "device ingest: label values span more than 2^22; use gs_db_from_arrays");
  long long *present = sc.get<long long>(range);
  long long *rank = sc.get<long long>(range + 1);
  int32_t *of = sc.get<int32_t>(range);
  CK(cudaMemsetAsync(present, 0, sizeof(long long) * range, s));
  k_mark<<<blocks_for(n), kThreads, 0, s>>>(x, n, lo, present);
  scan_exclusive(present, rank, range, sc);
  k_label_values<<<blocks_for(range), kThreads, 0, s>>>(present, rank, range, lo, of);
  k_relabel<<<blocks_for(n), kThreads, 0, s>>>(x, n, lo, rank);
  CK(cudaMemcpyAsync(cnt, rank + range, sizeof(long long), cudaMemcpyDeviceToHost, s));
  return of;
}

}  // namespace

void ingest_release()
{
  IngestCtx &cx = ingest_ctx();
  std::lock_guard<std::mutex> lk(cx.mu);
  if(cx.pool) cudaMemPoolTrimTo(cx.pool, 0);
}

void ingest_free_block(void *block)
{
  IngestCtx &cx = ingest_ctx();
  std::lock_guard<std::mutex> lk(cx.mu);
  // every kernel that may still read the block has finished
  cudaDeviceSynchronize();
  cudaFreeAsync(block, cx.s);
  cudaStreamSynchronize(cx.s);
}

void ingest_cudabin_device(Database &db, int32_t G, int32_t esz, int32_t maxv, const int32_t *edges,
                           const int32_t *elab, const int32_t *vlab, const int32_t *voff)
{
  if(G < 0 || esz < 0 || maxv < 0) throw Error(ST_ERR_FORMAT, "cudabin: negative sizes");
  IngestCtx &cx = ingest_ctx();
  std::lock_guard<std::mutex> lk(cx.mu);
  cx.init();
  CK(cudaSetDevice(0));
  cudaStream_t s = cx.s;
  ReadBack &rb = *cx.rb;
  // drains the streams when the ingest returns or throws (after the
  // scratch's frees are queued), so that nothing of this ingest is in flight
  // afterwards
  struct Drain {
    cudaStream_t s, s_copy;
    ~Drain()
    {
      cudaStreamSynchronize(s_copy);
      cudaStreamSynchronize(s);
    }
  } drain{ s, cx.s_copy };
  Scratch sc{ s, cx.pool, {} };
  const long long slots = (long long)G * maxv;
  // raw arrays up (the reference's copy_to_device).  The vertex offsets go
  // first and the per-graph pass is queued behind them before the other
  // arrays are copied (on the copy stream), so the pass runs during those
  // copies: with cudaMemcpyAsync from pageable memory a copy returns only
  // when it is done; with the in-place read kernel (pull_to_device) all of
  // it is queued at once.
  int32_t *d_edges = sc.get<int32_t>(esz), *d_elab = sc.get<int32_t>(esz);
  int32_t *d_vlab = sc.get<int32_t>(slots), *d_voff = sc.get<int32_t>(slots + 1);
  CK(cudaEventRecord(cx.ev_alloc, s));
  pull_to_device(cx, d_voff, voff, slots + 1, s);
  unsigned *flags = sc.get<unsigned>(1);
  CK(cudaMemsetAsync(flags, 0, sizeof(unsigned), s));

  // 1. graphs (read back: vertex and entry totals, the tiling check)
  long long *gnv = sc.get<long long>(G + 1), *gadj = sc.get<long long>(G + 1);
  long long *vbase = sc.get<long long>(G + 1), *gpos = sc.get<long long>(G + 1);
  k_graphs<<<blocks_for(G), kThreads, 0, s>>>(G, maxv, slots, esz, d_voff, gnv, gadj, flags);
  scan_exclusive(gnv, vbase, G, sc);
  scan_exclusive(gadj, gpos, G, sc);
  CK(cudaMemcpyAsync(&rb.v_total, vbase + G, sizeof(long long), cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(&rb.e_total, gpos + G, sizeof(long long), cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(&rb.flags, flags, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamWaitEvent(cx.s_copy, cx.ev_alloc, 0));
  if(esz) {
    pull_to_device(cx, d_edges, edges, esz, cx.s_copy);
    pull_to_device(cx, d_elab, elab, esz, cx.s_copy);
  }
  if(slots) pull_to_device(cx, d_vlab, vlab, slots, cx.s_copy);
  CK(cudaEventRecord(cx.ev_copied, cx.s_copy));
  sc.after = cx.ev_copied;
  CK(cudaStreamSynchronize(s));
  if(rb.flags & kBadTile) throw Error(ST_ERR_FORMAT, "cudabin: bad vertex offsets");
  const long long V = rb.v_total, E2 = rb.e_total;
  if(V >= (long long)INT32_MAX || E2 >= (long long)INT32_MAX)
    throw Error(ST_ERR_FORMAT, "database too large for 32-bit vertex/adjacency indices");

  // 2. vertices and adjacency, raw labels, checks (read back with the label ranges)
  int32_t *off = sc.get<int32_t>(V + 1), *vgraph = sc.get<int32_t>(V + 1);
  int32_t *vgbase = sc.get<int32_t>(V + 1);
  int32_t *vl = sc.get<int32_t>(V), *adj_to = sc.get<int32_t>(E2), *el = sc.get<int32_t>(E2);
  {
    const int32_t e2 = (int32_t)E2;
    CK(cudaMemcpyAsync(off + V, &e2, sizeof(int32_t), cudaMemcpyHostToDevice, s));
  }
  CK(cudaStreamWaitEvent(s, cx.ev_copied, 0));
  k_vertices<<<blocks_for(slots), kThreads, 0, s>>>(G, maxv, slots, esz, d_voff, d_vlab, d_edges, d_elab, gnv,
                                                      vbase, gpos, off, vgraph, vgbase, vl, adj_to, el, flags);
  int *mm = sc.get<int>(4);
  {
    static const int init[4] = { INT32_MAX, INT32_MIN, INT32_MAX, INT32_MIN };
    CK(cudaMemcpyAsync(mm, init, sizeof(init), cudaMemcpyHostToDevice, s));
  }
  if(V) k_minmax<<<blocks_for(V), kThreads, 0, s>>>(vl, V, mm, mm + 1);
  if(E2) k_minmax<<<blocks_for(E2), kThreads, 0, s>>>(el, E2, mm + 2, mm + 3);
  CK(cudaMemcpyAsync(&rb.flags, flags, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(rb.minmax, mm, sizeof(rb.minmax), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if(rb.flags & kBadLeave) throw Error(ST_ERR_FORMAT, "cudabin: edge leaves its graph");
  if(rb.flags & kBadTile) throw Error(ST_ERR_FORMAT, "cudabin: vertex offsets do not tile the edge array");
  if(rb.flags & kSelfLoop) throw Error(ST_ERR_FORMAT, "self loop (only simple graphs are supported)");
  if(rb.flags & kParallel) throw Error(ST_ERR_FORMAT, "parallel edges (only simple graphs are supported)");

  // 3. labels, both alphabets compacted before one read-back of their sizes
  const int vmin = rb.minmax[0], vmax = rb.minmax[1], emin = rb.minmax[2], emax = rb.minmax[3];
  rb.label_cnt[0] = rb.label_cnt[1] = 0;
  int32_t *vof = V ? compact_labels(vl, V, vmin, vmax, &rb.label_cnt[0], sc) : nullptr;
  int32_t *eof = E2 ? compact_labels(el, E2, emin, emax, &rb.label_cnt[1], sc) : nullptr;
  CK(cudaStreamSynchronize(s));
  const long long nvl = rb.label_cnt[0], nel = rb.label_cnt[1];
  const int32_t VL = std::max<int32_t>(1, (int32_t)nvl);
  const int32_t EL = std::max<int32_t>(1, (int32_t)nel);
  if(VL > 65535 || EL > 65535) throw Error(ST_ERR_LIMIT, "more than 65535 distinct vertex or edge labels");
  const long long tab = (long long)VL * EL * VL;
  if(tab > (1ll << 25))
    throw Error(ST_ERR_LIMIT, "device ingest: label alphabet too large for its pair table; use gs_db_from_arrays");

  // 4. pair table (read back: the number of pairs and the largest graph)
  long long *seen = sc.get<long long>(tab), *prank = sc.get<long long>(tab + 1);
  CK(cudaMemsetAsync(seen, 0, sizeof(long long) * tab, s));
  {
    // few blocks when the table is block-local: each merges the whole table once
    const bool local = tab <= kSmemTab;
    const unsigned nb = local ? std::min<unsigned>(blocks_for(V), 4u * (unsigned)gsgb::sm_count()) : blocks_for(V);
    k_pairs_seen<<<nb, kThreads, local ? (size_t)tab : 0, s>>>(off, V, vl, adj_to, el, EL, VL, seen, tab);
  }
  scan_exclusive(seen, prank, tab, sc);
  int *d_mx = sc.get<int>(2);
  CK(cudaMemsetAsync(d_mx, 0, 2 * sizeof(int), s));
  k_max_ll<<<blocks_for(G), kThreads, 0, s>>>(gnv, G, d_mx);
  if(V) k_max_degree<<<blocks_for(V), kThreads, 0, s>>>(off, V, d_mx + 1);
  CK(cudaMemcpyAsync(&rb.nkeys, prank + tab, sizeof(long long), cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(&rb.max_vertices, d_mx, 2 * sizeof(int), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  const long long nkeys = rb.nkeys;
  const int mxv = rb.max_vertices;
  const bool sort_adj = rb.max_degree <= kSortDegree;

  // the database block, laid out as Database::upload lays it out
  auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
  const size_t o_adj = 0;
  const size_t o_off = o_adj + al(sizeof(unsigned long long) * (E2 + 1));
  const size_t o_vl = o_off + al(sizeof(int32_t) * (V + 1));
  const size_t o_vg = o_vl + al(sizeof(int32_t) * (V + 1));
  const size_t o_gb = o_vg + al(sizeof(int32_t) * (V + 1));
  const size_t o_pi = o_gb + al(sizeof(int32_t) * (V + 1));
  const size_t o_ro = o_pi + al(sizeof(int32_t) * tab);
  const size_t o_vb = o_ro + al(sizeof(int32_t) * (VL + 1));
  const size_t o_ap = o_vb + al(sizeof(int32_t) * (G + 1));
  const size_t o_pc = o_ap + al(sizeof(int32_t) * (E2 + 1));
  const size_t o_in = o_pc + al(sizeof(int32_t) * (nkeys + 1));
  const size_t total = o_in + al(sizeof(unsigned long long) * (E2 + 1));
  char *b = nullptr;
  if(cudaMallocFromPoolAsync((void **)&b, total, cx.pool, s) != cudaSuccess) {
    cudaGetLastError();
    throw Error(ST_ERR_NOMEM, "device ingest: out of device memory");
  }
  try {
    int32_t *pidx = (int32_t *)(b + o_pi), *ro = (int32_t *)(b + o_ro), *pc = (int32_t *)(b + o_pc);
    k_pairs_index<<<blocks_for(tab), kThreads, 0, s>>>(seen, prank, EL, VL, pidx, pc, ro);
    {
      const int32_t nk = (int32_t)nkeys;
      CK(cudaMemcpyAsync(ro + VL, &nk, sizeof(int32_t), cudaMemcpyHostToDevice, s));
    }
    // 5. packed entries and the rest of the block
    k_pack<<<blocks_for(V), kThreads, 0, s>>>(off, V, vl, adj_to, el, pidx, EL, VL, sort_adj,
                                              (unsigned long long *)(b + o_in), (unsigned long long *)(b + o_adj),
                                              (int32_t *)(b + o_ap));
    CK(cudaMemcpyAsync(b + o_off, off, sizeof(int32_t) * (V + 1), cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(b + o_vl, vl, sizeof(int32_t) * V, cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(b + o_vg, vgraph, sizeof(int32_t) * V, cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(b + o_gb, vgbase, sizeof(int32_t) * V, cudaMemcpyDeviceToDevice, s));
    k_narrow<<<blocks_for(G + 1), kThreads, 0, s>>>(vbase, G + 1, (int32_t *)(b + o_vb));
    // host metadata (label values, each label's first pair, the pair codes), one read-back
    int32_t *hm = cx.meta_buf((size_t)(nvl + nel + VL + nkeys + 1));
    int32_t *h_vof = hm, *h_eof = hm + nvl, *hro = hm + nvl + nel, *hpc = hro + VL;
    if(nvl) CK(cudaMemcpyAsync(h_vof, vof, sizeof(int32_t) * nvl, cudaMemcpyDeviceToHost, s));
    if(nel) CK(cudaMemcpyAsync(h_eof, eof, sizeof(int32_t) * nel, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(hro, ro, sizeof(int32_t) * VL, cudaMemcpyDeviceToHost, s));
    if(nkeys) CK(cudaMemcpyAsync(hpc, pc, sizeof(int32_t) * nkeys, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    CK(cudaGetLastError());
    LabelMap labels;
    labels.vlabel_of.assign(h_vof, h_vof + nvl);
    labels.elabel_of.assign(h_eof, h_eof + nel);
    if(db.d_block && db.pooled) {
      // a block of an earlier ingest into this database (the lock is held here)
      cudaDeviceSynchronize();
      cudaFreeAsync(db.d_block, s);
      db.d_block = nullptr;
      db.pooled = false;
    }
    db.release();
    db.host = HostDB();
    db.host.n_graphs = G;
    db.labels = labels;
    db.VL = VL;
    db.EL = EL;
    db.pairs.assign(VL, {});
    db.pair_cnt.assign(VL, 0);
    db.root_off.assign(hro, hro + VL);
    for(int32_t a = 0; a < VL; a++) {
      const int32_t end = a + 1 < VL ? hro[a + 1] : (int32_t)nkeys;
      for(int32_t i = hro[a]; i < end; i++) db.pairs[a].push_back({ hpc[i] >> 16, hpc[i] & 0xffff });
      db.pair_cnt[a] = end - hro[a];
    }
    db.root_keys = (int32_t)nkeys;
    db.d_block = b;
    db.pooled = true;
    db.d_bytes = total;
    db.dev = DevDB{};
    db.dev.adj = (const unsigned long long *)(b + o_adj);
    db.dev.adj_off = (const int32_t *)(b + o_off);
    db.dev.vlabel = (const int32_t *)(b + o_vl);
    db.dev.vgraph = (const int32_t *)(b + o_vg);
    db.dev.vgbase = (const int32_t *)(b + o_gb);
    db.dev.pair_idx = pidx;
    db.dev.vbase = (const int32_t *)(b + o_vb);
    db.dev.adj_pair = (const int32_t *)(b + o_ap);
    db.dev.max_graph_vertices = mxv;
    db.dev.adj_sorted = sort_adj ? 1 : 0;
    db.adj_in = (const unsigned long long *)(b + o_in);
    db.dev.VL = VL;
    db.dev.EL = EL;
    db.dev.n_graphs = G;
    db.dev.n_vertices = (int32_t)V;
    db.dev.root_off = ro;
    db.dev.pair_code = pc;
    db.d_root_off = ro;
    db.resident = true;
    db.device_only = true;
    db.dev_vertices = V;
    db.dev_adj = E2;
  } catch(...) {
    cudaFreeAsync(b, s);
    throw;
  }
}

}  // namespace gsgb
