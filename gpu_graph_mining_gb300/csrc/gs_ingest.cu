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
  const long long cap = 152LL * 64;
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

// out[i] = sum of in[0..i) for i in [0, n]; out must hold n + 1 values
void scan_exclusive(const long long *in, long long *out, long long n, cudaStream_t s)
{
  const long long nb = (n + kThreads - 1) / kThreads;
  if(nb <= 0) {
    CK(cudaMemsetAsync(out, 0, sizeof(long long), s));
    return;
  }
  long long *sums = nullptr;
  CK(cudaMallocAsync(&sums, sizeof(long long) * (nb + 1), s));
  k_scan_blocks<<<(unsigned)nb, kThreads, 0, s>>>(in, out, n, sums);
  if(nb == 1) {
    // one block: its sum is the total
    CK(cudaMemcpyAsync(out + n, sums, sizeof(long long), cudaMemcpyDeviceToDevice, s));
  } else {
    long long *offs = nullptr;
    CK(cudaMallocAsync(&offs, sizeof(long long) * (nb + 1), s));
    scan_exclusive(sums, offs, nb, s);
    k_scan_add<<<(unsigned)nb, kThreads, 0, s>>>(out, n, offs);
    // the total, after the last element
    CK(cudaMemcpyAsync(out + n, offs + nb, sizeof(long long), cudaMemcpyDeviceToDevice, s));
    CK(cudaFreeAsync(offs, s));
  }
  CK(cudaFreeAsync(sums, s));
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
__global__ void k_minmax(const int32_t *x, long long n, int *mn, int *mx)
{
  int lo = INT32_MAX, hi = INT32_MIN;
  for(long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    lo = min(lo, x[i]);
    hi = max(hi, x[i]);
  }
  for(int o = 16; o > 0; o >>= 1) {
    lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
  if((threadIdx.x & 31) == 0) {
    atomicMin(mn, lo);
    atomicMax(mx, hi);
  }
}

__global__ void k_mark(const int32_t *x, long long n, int lo, long long *present)
{
  for(long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    present[(long long)x[i] - lo] = 1;
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
__global__ void k_pairs_seen(const int32_t *off, long long V, const int32_t *vl, const int32_t *adj_to,
                             const int32_t *el, int EL, int VL, long long *seen)
{
  for(long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < V; v += (long long)gridDim.x * blockDim.x) {
    const long long a = vl[v];
    for(long long k = off[v]; k < off[v + 1]; k++) seen[(a * EL + el[k]) * VL + vl[adj_to[k]]] = 1;
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

// ---- 5. packed entries
__global__ void k_pack(const int32_t *off, long long V, const int32_t *vl, const int32_t *adj_to, const int32_t *el,
                       const int32_t *pair_idx, int EL, int VL, unsigned long long *adj, int32_t *adj_pair)
{
  for(long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < V; v += (long long)gridDim.x * blockDim.x) {
    const long long a = vl[v];
    for(long long k = off[v]; k < off[v + 1]; k++) {
      const uint32_t w = (uint32_t)adj_to[k];
      const uint32_t hi = ((uint32_t)el[k] << 16) | (uint32_t)vl[w];
      adj[k] = ((unsigned long long)hi << 32) | w;
      adj_pair[k] = pair_idx[(a * EL + el[k]) * VL + vl[w]];
    }
  }
}

__global__ void k_max_ll(const long long *x, long long n, int *mx)
{
  int hi = 0;
  for(long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    hi = max(hi, (int)x[i]);
  for(int o = 16; o > 0; o >>= 1) hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  if((threadIdx.x & 31) == 0) atomicMax(mx, hi);
}

template <class T> T *dalloc(size_t n)
{
  T *p = nullptr;
  if(cudaMalloc(&p, sizeof(T) * std::max<size_t>(n, 1)) != cudaSuccess) {
    cudaGetLastError();
    throw Error(ST_ERR_NOMEM, "device ingest: out of device memory");
  }
  return p;
}

struct Frees {
  std::vector<void *> ptrs;
  ~Frees()
  {
    for(void *p : ptrs) cudaFree(p);
  }
  template <class T> T *add(T *p)
  {
    ptrs.push_back(p);
    return p;
  }
};

// dense labels of x[0..n) in place; returns the distinct values in order
std::vector<int32_t> compact_device(int32_t *x, long long n, Frees &fr, cudaStream_t s)
{
  std::vector<int32_t> of;
  if(n == 0) return of;
  int *mm = fr.add(dalloc<int>(2));
  const int init[2] = { INT32_MAX, INT32_MIN };
  CK(cudaMemcpyAsync(mm, init, sizeof(init), cudaMemcpyHostToDevice, s));
  k_minmax<<<blocks_for(n), kThreads, 0, s>>>(x, n, mm, mm + 1);
  int h[2];
  CK(cudaMemcpyAsync(h, mm, sizeof(h), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  const long long range = (long long)h[1] - (long long)h[0] + 1;
  if(range > (1ll << 22))
    throw Error(ST_ERR_LIMIT, "device ingest: label values span more than 2^22; use gs_db_from_arrays");
  long long *present = fr.add(dalloc<long long>(range));
  long long *rank = fr.add(dalloc<long long>(range + 1));
  CK(cudaMemsetAsync(present, 0, sizeof(long long) * range, s));
  k_mark<<<blocks_for(n), kThreads, 0, s>>>(x, n, h[0], present);
  scan_exclusive(present, rank, range, s);
  long long cnt = 0;
  CK(cudaMemcpyAsync(&cnt, rank + range, sizeof(cnt), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  int32_t *ofd = fr.add(dalloc<int32_t>(cnt));
  k_label_values<<<blocks_for(range), kThreads, 0, s>>>(present, rank, range, h[0], ofd);
  k_relabel<<<blocks_for(n), kThreads, 0, s>>>(x, n, h[0], rank);
  of.resize(cnt);
  CK(cudaMemcpyAsync(of.data(), ofd, sizeof(int32_t) * cnt, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  return of;
}

}  // namespace

void ingest_cudabin_device(Database &db, int32_t G, int32_t esz, int32_t maxv, const int32_t *edges,
                           const int32_t *elab, const int32_t *vlab, const int32_t *voff)
{
  if(G < 0 || esz < 0 || maxv < 0) throw Error(ST_ERR_FORMAT, "cudabin: negative sizes");
  CK(cudaSetDevice(0));
  cudaStream_t s;
  CK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  struct StreamGuard {
    cudaStream_t s;
    ~StreamGuard()
    {
      cudaStreamSynchronize(s);
      cudaStreamDestroy(s);
    }
  } sg{ s };
  Frees fr;
  const long long slots = (long long)G * maxv;
  // raw arrays up (the reference's copy_to_device)
  int32_t *d_edges = fr.add(dalloc<int32_t>(esz)), *d_elab = fr.add(dalloc<int32_t>(esz));
  int32_t *d_vlab = fr.add(dalloc<int32_t>(slots)), *d_voff = fr.add(dalloc<int32_t>(slots + 1));
  if(esz) {
    CK(cudaMemcpyAsync(d_edges, edges, sizeof(int32_t) * esz, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(d_elab, elab, sizeof(int32_t) * esz, cudaMemcpyHostToDevice, s));
  }
  if(slots) CK(cudaMemcpyAsync(d_vlab, vlab, sizeof(int32_t) * slots, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(d_voff, voff, sizeof(int32_t) * (slots + 1), cudaMemcpyHostToDevice, s));
  unsigned *flags = fr.add(dalloc<unsigned>(1));
  CK(cudaMemsetAsync(flags, 0, sizeof(unsigned), s));

  // 1. graphs
  long long *gnv = fr.add(dalloc<long long>(G + 1)), *gadj = fr.add(dalloc<long long>(G + 1));
  long long *vbase = fr.add(dalloc<long long>(G + 1)), *gpos = fr.add(dalloc<long long>(G + 1));
  k_graphs<<<blocks_for(G), kThreads, 0, s>>>(G, maxv, slots, esz, d_voff, gnv, gadj, flags);
  scan_exclusive(gnv, vbase, G, s);
  scan_exclusive(gadj, gpos, G, s);
  long long tot[2];
  unsigned hflags = 0;
  CK(cudaMemcpyAsync(&tot[0], vbase + G, sizeof(long long), cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(&tot[1], gpos + G, sizeof(long long), cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(&hflags, flags, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if(hflags & kBadTile) throw Error(ST_ERR_FORMAT, "cudabin: bad vertex offsets");
  const long long V = tot[0], E2 = tot[1];
  if(V >= (long long)INT32_MAX || E2 >= (long long)INT32_MAX)
    throw Error(ST_ERR_FORMAT, "database too large for 32-bit vertex/adjacency indices");

  // 2. vertices and adjacency, raw labels, checks
  int32_t *off = fr.add(dalloc<int32_t>(V + 1)), *vgraph = fr.add(dalloc<int32_t>(V + 1));
  int32_t *vgbase = fr.add(dalloc<int32_t>(V + 1));
  int32_t *vl = fr.add(dalloc<int32_t>(V)), *adj_to = fr.add(dalloc<int32_t>(E2)), *el = fr.add(dalloc<int32_t>(E2));
  {
    const int32_t e2 = (int32_t)E2;
    CK(cudaMemcpyAsync(off + V, &e2, sizeof(int32_t), cudaMemcpyHostToDevice, s));
  }
  k_vertices<<<blocks_for(slots), kThreads, 0, s>>>(G, maxv, slots, esz, d_voff, d_vlab, d_edges, d_elab, gnv,
                                                      vbase, gpos, off, vgraph, vgbase, vl, adj_to, el, flags);
  CK(cudaMemcpyAsync(&hflags, flags, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if(hflags & kBadLeave) throw Error(ST_ERR_FORMAT, "cudabin: edge leaves its graph");
  if(hflags & kBadTile) throw Error(ST_ERR_FORMAT, "cudabin: vertex offsets do not tile the edge array");
  if(hflags & kSelfLoop) throw Error(ST_ERR_FORMAT, "self loop (only simple graphs are supported)");
  if(hflags & kParallel) throw Error(ST_ERR_FORMAT, "parallel edges (only simple graphs are supported)");

  // 3. labels
  LabelMap labels;
  labels.vlabel_of = compact_device(vl, V, fr, s);
  labels.elabel_of = compact_device(el, E2, fr, s);
  const int32_t VL = std::max<int32_t>(1, (int32_t)labels.vlabel_of.size());
  const int32_t EL = std::max<int32_t>(1, (int32_t)labels.elabel_of.size());
  if(VL > 65535 || EL > 65535) throw Error(ST_ERR_LIMIT, "more than 65535 distinct vertex or edge labels");
  const long long tab = (long long)VL * EL * VL;
  if(tab > (1ll << 25))
    throw Error(ST_ERR_LIMIT, "device ingest: label alphabet too large for its pair table; use gs_db_from_arrays");

  // 4. pair table
  long long *seen = fr.add(dalloc<long long>(tab)), *prank = fr.add(dalloc<long long>(tab + 1));
  CK(cudaMemsetAsync(seen, 0, sizeof(long long) * tab, s));
  k_pairs_seen<<<blocks_for(V), kThreads, 0, s>>>(off, V, vl, adj_to, el, EL, VL, seen);
  scan_exclusive(seen, prank, tab, s);
  long long nkeys = 0;
  CK(cudaMemcpyAsync(&nkeys, prank + tab, sizeof(long long), cudaMemcpyDeviceToHost, s));
  int mxv = 0;
  int *d_mx = fr.add(dalloc<int>(1));
  CK(cudaMemsetAsync(d_mx, 0, sizeof(int), s));
  k_max_ll<<<blocks_for(G), kThreads, 0, s>>>(gnv, G, d_mx);
  CK(cudaMemcpyAsync(&mxv, d_mx, sizeof(int), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));

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
  const size_t total = o_pc + al(sizeof(int32_t) * (nkeys + 1));
  char *b = nullptr;
  if(cudaMalloc(&b, total) != cudaSuccess) {
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
    k_pack<<<blocks_for(V), kThreads, 0, s>>>(off, V, vl, adj_to, el, pidx, EL, VL, (unsigned long long *)(b + o_adj),
                                              (int32_t *)(b + o_ap));
    CK(cudaMemcpyAsync(b + o_off, off, sizeof(int32_t) * (V + 1), cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(b + o_vl, vl, sizeof(int32_t) * V, cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(b + o_vg, vgraph, sizeof(int32_t) * V, cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(b + o_gb, vgbase, sizeof(int32_t) * V, cudaMemcpyDeviceToDevice, s));
    {
      // vertex bases as int32
      std::vector<long long> hv(G + 1);
      CK(cudaMemcpyAsync(hv.data(), vbase, sizeof(long long) * (G + 1), cudaMemcpyDeviceToHost, s));
      CK(cudaStreamSynchronize(s));
      std::vector<int32_t> v32(hv.begin(), hv.end());
      CK(cudaMemcpyAsync(b + o_vb, v32.data(), sizeof(int32_t) * (G + 1), cudaMemcpyHostToDevice, s));
      CK(cudaStreamSynchronize(s));
    }
    // host metadata: each label's pairs, in pair-index order
    std::vector<int32_t> hro(VL + 1), hpc(std::max<long long>(nkeys, 1));
    CK(cudaMemcpyAsync(hro.data(), ro, sizeof(int32_t) * VL, cudaMemcpyDeviceToHost, s));
    if(nkeys) CK(cudaMemcpyAsync(hpc.data(), pc, sizeof(int32_t) * nkeys, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    CK(cudaGetLastError());
    hro[VL] = (int32_t)nkeys;
    db.release();
    db.host = HostDB();
    db.host.n_graphs = G;
    db.labels = labels;
    db.VL = VL;
    db.EL = EL;
    db.pairs.assign(VL, {});
    db.pair_cnt.assign(VL, 0);
    db.root_off.assign(hro.begin(), hro.begin() + VL);
    for(int32_t a = 0; a < VL; a++) {
      for(int32_t i = hro[a]; i < hro[a + 1]; i++) db.pairs[a].push_back({ hpc[i] >> 16, hpc[i] & 0xffff });
      db.pair_cnt[a] = hro[a + 1] - hro[a];
    }
    db.root_keys = (int32_t)nkeys;
    db.d_block = b;
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
    cudaStreamSynchronize(s);
    cudaFree(b);
    throw;
  }
}

}  // namespace gsgb
