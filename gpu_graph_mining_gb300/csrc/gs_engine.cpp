// Host side of the miner: resident databases, the device pool, and the wave
// scheduler.
//
// The reference drives the DFS-code tree one node at a time from the host
// (gspan_cuda_no_sort::mainloop, src/gspan_cuda/gspan_cuda_no_sort.cpp:
// 275-489): every node costs ~15-30 kernel launches, each followed by a
// device synchronise, plus per-node cudaMalloc/cudaFree.  Here a "wave" is a
// batch of pending tree nodes (possibly of different mining jobs) extended
// together: per wave there are three kernels (count, support, materialise),
// one device->host copy of the candidate supports and one synchronise.  With
// wave_nodes = 1 the same engine runs the plain one-pattern-at-a-time form.
//
// The pattern set, codes and supports follow the sequential miner
// (src/gspan/gspan.cpp:172-351): roots (fl <= tl) in ascending label order,
// candidates keyed like its Projected maps, canonicality by gSpan::is_min
// (src/gspan/ismin.cpp), output in its pre-order traversal order.
#include "gs_engine.hpp"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <functional>
#include <map>
#include <system_error>
#include <thread>
#include <unordered_map>

#include "gs_kernels.hpp"

namespace gsgb {

void cuda_check(cudaError_t e, const char *what)
{
  if(e != cudaSuccess) throw Error(ST_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define CK(call) cuda_check((call), #call)

// ------------------------------------------------------------------ database

void Database::prepare()
{
  if(VL > 0 || host.n_graphs == 0) return;
  compact_labels(host, vl_dense, el_dense, labels);
  VL = (int32_t)labels.vlabel_of.size();
  EL = (int32_t)labels.elabel_of.size();
  if(VL == 0) VL = 1;
  if(EL == 0) EL = 1;
  if(VL > 65535 || EL > 65535) throw Error(ST_ERR_LIMIT, "more than 65535 distinct vertex or edge labels");
  const int64_t tab = (int64_t)VL * EL * VL;
  if(tab > (int64_t)1 << 28) throw Error(ST_ERR_LIMIT, "label alphabet too large for the dense pair table");
  std::vector<uint8_t> seen((size_t)tab, 0);
  {
    // per-part presence tables over the vertices, merged
    std::vector<std::vector<uint8_t>> part(32);
    parallel_ranges(host.n_vertices(), [&](int64_t v0, int64_t v1, int t) {
      std::vector<uint8_t> s((size_t)tab, 0);
      for(int64_t v = v0; v < v1; v++) {
        const int64_t a = vl_dense[v];
        for(int64_t k = host.aoff[v]; k < host.aoff[v + 1]; k++)
          s[(size_t)((a * EL + el_dense[k]) * VL + vl_dense[host.adj_to[k]])] = 1;
      }
      part[t].swap(s);
    }, tab > (1 << 20) ? INT64_MAX / 4 : 1 << 15);
    for(auto &s : part)
      for(size_t i = 0; i < s.size(); i++) seen[i] |= s[i];
  }
  pairs.assign(VL, {});
  pair_cnt.assign(VL, 0);
  root_off.assign(VL, 0);
  int32_t acc = 0;
  for(int32_t a = 0; a < VL; a++) {
    for(int32_t e = 0; e < EL; e++)
      for(int32_t t = 0; t < VL; t++)
        if(seen[(size_t)(((int64_t)a * EL + e) * VL + t)]) pairs[a].push_back({ e, t });
    pair_cnt[a] = (int32_t)pairs[a].size();
    root_off[a] = acc;
    acc += pair_cnt[a];
  }
  root_keys = acc;
}

void Database::upload()
{
  if(resident) return;
  prepare();
  const int64_t V = host.n_vertices(), E2 = host.n_adj();
  const int64_t tab = (int64_t)VL * EL * VL;
  auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
  size_t o_adj = 0;
  size_t o_off = o_adj + al(sizeof(unsigned long long) * (E2 + 1));
  size_t o_vl = o_off + al(sizeof(int32_t) * (V + 1));
  size_t o_vg = o_vl + al(sizeof(int32_t) * (V + 1));
  size_t o_gb = o_vg + al(sizeof(int32_t) * (V + 1));
  size_t o_pi = o_gb + al(sizeof(int32_t) * (V + 1));
  size_t o_ro = o_pi + al(sizeof(int32_t) * tab);
  size_t o_vb = o_ro + al(sizeof(int32_t) * (VL + 1));
  size_t o_ap = o_vb + al(sizeof(int32_t) * (host.n_graphs + 1));
  size_t o_pc = o_ap + al(sizeof(int32_t) * (E2 + 1));
  size_t total = o_pc + al(sizeof(int32_t) * (root_keys + 1));
  std::vector<unsigned long long> adj(E2 + 1, 0);
  parallel_ranges(E2, [&](int64_t b, int64_t e, int) {
    for(int64_t k = b; k < e; k++) {
      const uint32_t w = (uint32_t)host.adj_to[k];
      const uint32_t hi = ((uint32_t)el_dense[k] << 16) | (uint32_t)vl_dense[w];
      adj[k] = ((unsigned long long)hi << 32) | w;
    }
  }, 1 << 16);
  // each vertex's entries in ascending (edge label, neighbour label, neighbour)
  // order: the entries a right-most-path vertex's forward rule rejects are a
  // prefix the extension kernels skip
  parallel_ranges(V, [&](int64_t v0, int64_t v1, int) {
    for(int64_t v = v0; v < v1; v++) std::sort(adj.begin() + host.aoff[v], adj.begin() + host.aoff[v + 1]);
  }, 1 << 14);
  std::vector<int32_t> off(V + 1), vg(V + 1, 0), vgb(V + 1, 0), pidx(tab, -1);
  parallel_ranges(V + 1, [&](int64_t b, int64_t e, int) {
    for(int64_t v = b; v < e; v++) off[v] = (int32_t)host.aoff[v];
  }, 1 << 16);
  parallel_ranges(host.n_graphs, [&](int64_t g0, int64_t g1, int) {
    for(int64_t g = g0; g < g1; g++)
      for(int64_t v = host.vbase[g]; v < host.vbase[g + 1]; v++) {
        vg[v] = (int32_t)g;
        vgb[v] = (int32_t)host.vbase[g];
      }
  });
  for(int32_t a = 0; a < VL; a++)
    for(size_t i = 0; i < pairs[a].size(); i++)
      pidx[((int64_t)a * EL + pairs[a][i].first) * VL + pairs[a][i].second] = (int32_t)i;
  // per directed entry: dense index of (elabel, nbr label) among the pairs of
  // the source vertex's label (the forward key offset within a slot, and the
  // root key offset within root_off[label(source)])
  std::vector<int32_t> ap(E2 + 1, 0);
  parallel_ranges(V, [&](int64_t v0, int64_t v1, int) {
    for(int64_t v = v0; v < v1; v++) {
      const int64_t a = vl_dense[v];
      for(int64_t k = host.aoff[v]; k < host.aoff[v + 1]; k++) {
        const int64_t hi = (int64_t)(adj[k] >> 32);
        ap[k] = pidx[(size_t)((a * EL + (hi >> 16)) * VL + (hi & 0xffff))];
      }
    }
  });
  std::vector<int32_t> vb(host.n_graphs + 1);
  int32_t maxnv = 0;
  for(int32_t g = 0; g <= host.n_graphs; g++) vb[g] = (int32_t)host.vbase[g];
  for(int32_t g = 0; g < host.n_graphs; g++) maxnv = std::max(maxnv, host.graph_nv(g));
  CK(cudaMalloc(&d_block, total));
  d_bytes = total;
  char *b = (char *)d_block;
  CK(cudaMemcpy(b + o_adj, adj.data(), sizeof(unsigned long long) * (E2 + 1), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(b + o_off, off.data(), sizeof(int32_t) * (V + 1), cudaMemcpyHostToDevice));
  if(V) CK(cudaMemcpy(b + o_vl, vl_dense.data(), sizeof(int32_t) * V, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(b + o_vg, vg.data(), sizeof(int32_t) * (V + 1), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(b + o_gb, vgb.data(), sizeof(int32_t) * (V + 1), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(b + o_pi, pidx.data(), sizeof(int32_t) * tab, cudaMemcpyHostToDevice));
  std::vector<int32_t> ro(root_off);
  ro.push_back(root_keys);
  std::vector<int32_t> pc(root_keys + 1, 0);
  for(int32_t a = 0; a < VL; a++)
    for(size_t i = 0; i < pairs[a].size(); i++)
      pc[root_off[a] + i] = (pairs[a][i].first << 16) | pairs[a][i].second;
  CK(cudaMemcpy(b + o_ro, ro.data(), sizeof(int32_t) * (VL + 1), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(b + o_pc, pc.data(), sizeof(int32_t) * (root_keys + 1), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(b + o_vb, vb.data(), sizeof(int32_t) * (host.n_graphs + 1), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(b + o_ap, ap.data(), sizeof(int32_t) * (E2 + 1), cudaMemcpyHostToDevice));
  dev.adj = (const unsigned long long *)(b + o_adj);
  dev.adj_off = (const int32_t *)(b + o_off);
  dev.vlabel = (const int32_t *)(b + o_vl);
  dev.vgraph = (const int32_t *)(b + o_vg);
  dev.vgbase = (const int32_t *)(b + o_gb);
  dev.pair_idx = (const int32_t *)(b + o_pi);
  dev.vbase = (const int32_t *)(b + o_vb);
  dev.adj_pair = (const int32_t *)(b + o_ap);
  dev.max_graph_vertices = maxnv;
  dev.adj_sorted = 1;
  dev.VL = VL;
  dev.EL = EL;
  dev.n_graphs = host.n_graphs;
  dev.n_vertices = (int32_t)V;
  d_root_off = (int32_t *)(b + o_ro);
  dev.root_off = d_root_off;
  dev.pair_code = (const int32_t *)(b + o_pc);
  resident = true;
}

void Database::ensure_host()
{
  if(!device_only || (int64_t)host.vlabel.size() == dev_vertices) return;
  const int64_t V = dev_vertices, E2 = dev_adj;
  const int32_t G = host.n_graphs;
  std::vector<unsigned long long> adj(E2 + 1);
  std::vector<int32_t> off(V + 1), vl(V + 1), vb(G + 1);
  CK(cudaMemcpy(adj.data(), adj_in ? adj_in : dev.adj, sizeof(unsigned long long) * E2, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(off.data(), dev.adj_off, sizeof(int32_t) * (V + 1), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(vl.data(), dev.vlabel, sizeof(int32_t) * V, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(vb.data(), dev.vbase, sizeof(int32_t) * (G + 1), cudaMemcpyDeviceToHost));
  host.vbase.assign(vb.begin(), vb.end());
  host.aoff.assign(off.begin(), off.end());
  host.vlabel.resize(V);
  for(int64_t v = 0; v < V; v++) host.vlabel[v] = labels.vlabel_of[vl[v]];
  host.adj_to.resize(E2);
  host.adj_el.resize(E2);
  for(int64_t k = 0; k < E2; k++) {
    host.adj_to[k] = (int32_t)(adj[k] & 0xffffffffull);
    host.adj_el[k] = labels.elabel_of[(uint32_t)(adj[k] >> 48)];
  }
}

void Database::release()
{
  if(d_block) {
    if(pooled) ingest_free_block(d_block);
    else cudaFree(d_block);
  }
  d_block = nullptr;
  adj_in = nullptr;
  pooled = false;
  resident = false;
}

Database::~Database() { release(); }

namespace {

// -------------------------------------------------------------- device pool

// First-fit sub-allocator over a few large cudaMalloc chunks.  Memory freed
// here is handed out again at once: the engine returns a block only after
// the last passes that may read it have completed (Engine::reap).
class Pool {
public:
  void set_limit(int64_t b) { limit_ = b; }
  // a piece of the chunks there are, or nullptr
  void *try_alloc(size_t n)
  {
    n = (n + 255) & ~(size_t)255;
    if(n == 0) n = 256;
    for(size_t c = 0; c < chunks_.size(); c++) {
      void *p = take(c, n);
      if(p) return p;
    }
    return nullptr;
  }
  void *alloc(size_t n)
  {
    if(void *p = try_alloc(n)) return p;
    n = (n + 255) & ~(size_t)255;
    if(n == 0) n = 256;
    grow(n);
    void *p = take(chunks_.size() - 1, n);
    if(!p) throw Error(ST_ERR_NOMEM, "device pool exhausted");
    return p;
  }
  void release(void *p)
  {
    if(!p) return;
    auto it = live_.find(p);
    if(it == live_.end()) return;
    int c = it->second.first;
    size_t n = it->second.second;
    live_.erase(it);
    used_ -= n;
    Chunk &ch = chunks_[c];
    size_t off = (size_t)((char *)p - ch.base);
    auto nx = ch.free.lower_bound(off);
    if(nx != ch.free.end() && off + n == nx->first) { n += nx->second; nx = ch.free.erase(nx); }
    if(nx != ch.free.begin()) {
      auto pv = std::prev(nx);
      if(pv->first + pv->second == off) { pv->second += n; return; }
    }
    ch.free.emplace(off, n);
  }
  size_t used() const { return used_; }
  size_t peak() const { return peak_; }
  void reset_peak() { peak_ = used_; }
  void destroy()
  {
    for(auto &c : chunks_) cudaFree(c.base);
    chunks_.clear();
    live_.clear();
    used_ = peak_ = total_ = 0;
  }

private:
  struct Chunk {
    char *base;
    size_t size;
    std::map<size_t, size_t> free;
  };
  void *take(size_t c, size_t n)
  {
    Chunk &ch = chunks_[c];
    for(auto it = ch.free.begin(); it != ch.free.end(); ++it) {
      if(it->second < n) continue;
      size_t off = it->first, sz = it->second;
      ch.free.erase(it);
      if(sz > n) ch.free.emplace(off + n, sz - n);
      void *p = ch.base + off;
      live_[p] = { (int)c, n };
      used_ += n;
      peak_ = std::max(peak_, used_);
      return p;
    }
    return nullptr;
  }
  void grow(size_t n)
  {
    size_t freeb = 0, totalb = 0;
    CK(cudaMemGetInfo(&freeb, &totalb));
    size_t lim = limit_ > 0 ? (size_t)limit_ : (size_t)(0.7 * (double)(freeb + total_));
    size_t want = std::max(n, next_);
    if(total_ + want > lim) want = std::max(n, lim > total_ ? lim - total_ : 0);
    if(want < n || total_ + want > lim + n) throw Error(ST_ERR_NOMEM, "device pool limit reached");
    char *p = nullptr;
    if(cudaMalloc(&p, want) != cudaSuccess) {
      cudaGetLastError();
      throw Error(ST_ERR_NOMEM, "cudaMalloc for the device pool failed");
    }
    chunks_.push_back(Chunk{ p, want, {} });
    chunks_.back().free.emplace(0, want);
    total_ += want;
    next_ = std::min<size_t>(next_ * 2, (size_t)16 << 30);
  }
  std::vector<Chunk> chunks_;
  std::unordered_map<void *, std::pair<int, size_t>> live_;
  size_t used_ = 0, peak_ = 0, total_ = 0;
  size_t next_ = (size_t)1 << 30;
  int64_t limit_ = 0;
};

// growable device / pinned buffers
template <class T> struct DBuf {
  T *p = nullptr;
  size_t cap = 0;
  void ensure(size_t n)
  {
    if(n <= cap) return;
    if(p) cudaFree(p);
    size_t c = std::max(n, cap * 2);
    if(c < 64) c = 64;
    p = nullptr;
    CK(cudaMalloc(&p, c * sizeof(T)));
    cap = c;
  }
  void free()
  {
    if(p) cudaFree(p);
    p = nullptr;
    cap = 0;
  }
};
template <class T> struct HBuf {
  T *p = nullptr;
  size_t cap = 0;
  void ensure(size_t n)
  {
    if(n <= cap) return;
    if(p) cudaFreeHost(p);
    size_t c = std::max(n, cap * 2);
    if(c < 64) c = 64;
    p = nullptr;
    CK(cudaHostAlloc(&p, c * sizeof(T), cudaHostAllocDefault));
    cap = c;
  }
  void free()
  {
    if(p) cudaFreeHost(p);
    p = nullptr;
    cap = 0;
  }
};

// ------------------------------------------------------------- host workers

class Workers {
public:
  explicit Workers(int n)
  {
    for(int i = 0; i < n; i++) th_.emplace_back([this, i] { loop(i + 1); });
  }
  ~Workers()
  {
    {
      std::lock_guard<std::mutex> g(m_);
      stop_ = true;
    }
    cv_.notify_all();
    for(auto &t : th_) t.join();
  }
  int size() const { return (int)th_.size() + 1; }
  // fn(index, worker_id); the caller is worker 0
  void run(int64_t n, const std::function<void(int64_t, int)> &fn)
  {
    if(n <= 0) return;
    if(th_.empty() || n < 8) {
      for(int64_t i = 0; i < n; i++) fn(i, 0);
      return;
    }
    {
      std::lock_guard<std::mutex> g(m_);
      fn_ = &fn;
      n_ = n;
      next_.store(0);
      busy_ = (int)th_.size();
      gen_++;
    }
    cv_.notify_all();
    work(0);
    std::unique_lock<std::mutex> l(m_);
    done_.wait(l, [this] { return busy_ == 0; });
    fn_ = nullptr;
  }

private:
  void work(int id)
  {
    while(true) {
      int64_t i = next_.fetch_add(1);
      if(i >= n_) break;
      (*fn_)(i, id);
    }
  }
  void loop(int id)
  {
    uint64_t seen = 0;
    while(true) {
      {
        std::unique_lock<std::mutex> l(m_);
        cv_.wait(l, [&] { return stop_ || gen_ != seen; });
        if(stop_) return;
        seen = gen_;
      }
      work(id);
      {
        std::lock_guard<std::mutex> g(m_);
        if(--busy_ == 0) done_.notify_all();
      }
    }
  }
  std::vector<std::thread> th_;
  std::mutex m_;
  std::condition_variable cv_, done_;
  const std::function<void(int64_t, int)> *fn_ = nullptr;
  std::atomic<int64_t> next_{ 0 };
  int64_t n_ = 0;
  int busy_ = 0;
  uint64_t gen_ = 0;
  bool stop_ = false;
};

// ------------------------------------------------------------------ engine

// One pool allocation holding the new columns and graph ranks of every child
// made by one wave (or one root phase); returned to the pool when the last
// column or rank array carved from it is released.
struct Block {
  void *base = nullptr;
  int32_t refs = 0;
};

// A column of embedding rows.  Columns form chains: a node's columns are its
// last column and that column's ancestors (parent), and a column holds one
// reference on its parent, so that a node needs one reference (its last
// column) for all of them.
struct Column {
  int2 *ptr = nullptr;
  int64_t n = 0;
  int32_t refs = 0;
  int32_t blk = -1;
  int32_t parent = -1;
};

// A node's view of one of its columns (kept in the node, so that wave
// descriptors are filled without visiting the column table).
struct ColRef {
  const int2 *ptr;
  int64_t n;
};

// One frequent pattern of a job's output tree; children in traversal order
// as a linked list.
struct PatternRec {
  int32_t parent;
  DFS edge;
  int64_t support;
  int32_t first_child = -1, last_child = -1, next_sibling = -1;
};

// A vector with room for N elements inline; longer contents move to the
// heap.  DFS-tree nodes are created and dropped by the hundred thousand per
// second, and nearly all patterns have few edges and vertices.
template <class T, int N> class SmallVec {
public:
  SmallVec() = default;
  SmallVec(const SmallVec &o) { assign(o.data(), o.size()); }
  SmallVec(SmallVec &&o) noexcept { take(o); }
  SmallVec &operator=(const SmallVec &o)
  {
    if(this != &o) assign(o.data(), o.size());
    return *this;
  }
  SmallVec &operator=(SmallVec &&o) noexcept
  {
    if(this != &o) {
      release();
      take(o);
    }
    return *this;
  }
  ~SmallVec() { release(); }
  size_t size() const { return n_; }
  bool empty() const { return n_ == 0; }
  T *data() { return heap_ ? heap_ : inl_; }
  const T *data() const { return heap_ ? heap_ : inl_; }
  T &operator[](size_t i) { return data()[i]; }
  const T &operator[](size_t i) const { return data()[i]; }
  T *begin() { return data(); }
  T *end() { return data() + n_; }
  const T *begin() const { return data(); }
  const T *end() const { return data() + n_; }
  void reserve(size_t c)
  {
    if(c <= cap()) return;
    T *h = new T[c];
    std::copy(data(), data() + n_, h);
    delete[] heap_;
    heap_ = h;
    hcap_ = c;
  }
  void push_back(const T &v)
  {
    if(n_ == cap()) reserve(std::max<size_t>(2 * cap(), N));
    data()[n_++] = v;
  }
  void assign(const T *p, size_t n)
  {
    n_ = 0;
    reserve(n);
    std::copy(p, p + n, data());
    n_ = n;
  }

private:
  size_t cap() const { return heap_ ? hcap_ : (size_t)N; }
  void release()
  {
    delete[] heap_;
    heap_ = nullptr;
    hcap_ = 0;
    n_ = 0;
  }
  void take(SmallVec &o)
  {
    n_ = o.n_;
    if(o.heap_) {
      heap_ = o.heap_;
      hcap_ = o.hcap_;
      o.heap_ = nullptr;
      o.hcap_ = 0;
    } else {
      std::copy(o.inl_, o.inl_ + o.n_, inl_);
    }
    o.n_ = 0;
  }
  T inl_[N];
  T *heap_ = nullptr;
  size_t hcap_ = 0;
  size_t n_ = 0;
};

struct PNode {
  int32_t job;
  int32_t pattern;
  SmallVec<DFS, 12> code;
  SmallVec<ColRef, 12> cols;  // column c = pattern vertex c
  int32_t last_col = -1;      // the node's reference: its last column (the rest by parent links)
  int32_t *gord;
  int32_t gord_blk;
  int64_t nrows;
  int64_t support;
  // lists strategy (forward children whose parent kept its per-row lists):
  // the parent's lists (a pool block shared by the parent's wave) and the
  // join rule (NodeDesc::join_lo / join_key / join_hi)
  int32_t list_blk = -1;
  const int32_t *list_off = nullptr;
  const int2 *list_ent = nullptr;
  int64_t list_rows = 0;
  int32_t join_lo = 0, join_key = 0, join_hi = 0;
};

// One mining job inside a scheduler.
struct JobState {
  MineJob job;
  int32_t db_slot = 0;
  std::vector<PatternRec> pats;
  std::vector<int32_t> roots;
  std::vector<int32_t> root_keys;  // each root's key (root_off[fl] + pair): the reference's root order
  std::vector<int32_t> stack;  // DFS-tree nodes waiting for a wave (top = back), as node pool ids
  int64_t pending = 0;         // nodes on the stack or in a wave in flight
  int64_t live_bytes = 0;      // embedding-store bytes held by the job's nodes
  int64_t peak_bytes = 0;
  int64_t patterns = 0;        // emitted when the job finished
  bool cancelled = false;
  bool done = false;
};

struct Candidate {
  int32_t node;
  int32_t key;
  DFS dfs;
  int32_t support;
  int32_t cnt;
  int32_t verdict;  // canonicality from the GPU: 1 / 0, or 2 = check on the host
  bool ok;
};

struct NodeLayout {
  int32_t nrm;
  int32_t maxtoc;
  int32_t nfwd;
  std::vector<int32_t> vlab;   // per pattern vertex
  std::vector<SlotDesc> slots;
};

// The device work of one wave up to its results copy: descriptor upload,
// scratch clears, count, selection, canonicality, results download, with the
// context's events between them.
struct WaveSeq {
  void *desc_dst = nullptr;
  const void *desc_src = nullptr;
  size_t desc_bytes = 0;
  void *zero = nullptr;
  size_t zero_bytes = 0;
  void *head = nullptr;
  void *head_host = nullptr;
  size_t d2h_bytes = 0;
  KernelCall count, screen, listed, ismin;
  bool with_min = false;
};

// WaveSeq as an instantiated CUDA graph, one per count-kernel variant and
// context: each wave updates the nodes' parameters and launches the graph.
struct WaveGraph {
  const void *count_func = nullptr;
  bool with_min = false;
  cudaGraph_t g = nullptr;
  cudaGraphExec_t x = nullptr;
  cudaGraphNode_t h2d, mz, mh, count, screen, listed, ismin, d2h;
};

inline cudaMemsetParams clear_params(void *dst, size_t bytes)
{
  cudaMemsetParams m{};
  m.dst = dst;
  m.pitch = 0;
  m.value = 0;
  m.elementSize = 1;
  m.width = bytes;
  m.height = 1;
  return m;
}

inline cudaKernelNodeParams kernel_params(KernelCall &c)
{
  cudaKernelNodeParams k{};
  k.func = const_cast<void *>(c.func);
  k.gridDim = c.grid;
  k.blockDim = c.block;
  k.sharedMemBytes = c.smem;
  k.kernelParams = c.params();
  k.extra = nullptr;
  return k;
}

// Header slots of a wave's results (unsigned long long each).
constexpr int kHeadRecords = 0;   // extension records written by the count pass
constexpr int kHeadFlags = 1;     // consistency flags after the count pass
constexpr int kHeadSelected = 2;  // selected candidates   } counters of
constexpr int kHeadExt = 3;       // embeddings of all keys } the support
constexpr int kHeadListed = 4;    // keys counted          } selection
constexpr int kHeadSelBytes = 5;  // algorithmic bytes     }
constexpr size_t kHeadBytes = 64;

// Device scratch and pinned mirrors of one wave in flight.  Two of them let
// the host prepare one wave's children while the GPU counts the other's.
struct WaveCtx {
  DBuf<char> d_desc;
  DBuf<uint32_t> d_bm;
  DBuf<int32_t> d_bmx, d_cnt, d_sup, d_childmap, d_cursor;
  DBuf<ChildOut> d_outs;
  // extension records of the count pass (record-driven materialise)
  DBuf<int4> d_rec;
  DBuf<unsigned long long> d_recn;
  DBuf<long long> d_keyword;
  DBuf<int32_t> d_lnode;   // lists strategy: the node of each frequent forward key
  // A wave's results, copied back in one piece: a 64-byte header (kHead*
  // slots) followed by the selected candidates {key, support, embeddings,
  // node << 2 | verdict}.  The zeroed region holds the embedding counts and the support
  // bitmaps (one memset).  The child table holds the children's outputs and
  // (key, child) pairs (one upload).
  DBuf<char> d_head, d_zero, d_mat;
  HBuf<char> h_head, h_mat;
  DBuf<int2> d_listed;               // keys with enough embeddings to be counted
  int64_t sel_hint = 4096;           // selected entries copied back with the wave's results
  bool rec_enabled = true;
  long long wanted_rec = 0;    // record capacity to have before the next wave (after an overflow)
  // pinned host mirrors
  HBuf<char> h_desc;
  HBuf<int32_t> h_sup, h_cnt, h_childmap;
  HBuf<ChildOut> h_outs;
  HBuf<long long> h_keyword;
  HBuf<unsigned long long> h_misc;  // [0] records written, [1] consistency flags, [2..3] = d_selc
  // 0/1 count, 1/6 selection, 6/2 canonicality, 3 results copied, 4/5 materialise
  // (the root context: 0/1 a group's count and support, 3 read back, 5 first
  // embeddings)
  cudaEvent_t ev[7] = {};
  bool have_events = false;
  std::vector<WaveGraph> graphs;
  // the context's stream (wave contexts; the root context uses the engine's)
  cudaStream_t stream = nullptr;
  // records of ev[5] (materialise passes), and the records of the engine's
  // ev_main and of the other contexts' ev[5] this context's stream already waits for
  uint64_t mat_gen = 0, seen_main = 0;
  uint64_t seen_mat[8] = {};

  void init(bool own_stream)
  {
    if(!have_events) {
      for(auto &e : ev) CK(cudaEventCreate(&e));
      have_events = true;
    }
    if(own_stream && !stream) CK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    h_misc.ensure(4);
  }
  void free()
  {
    d_desc.free(); d_bm.free(); d_bmx.free(); d_cnt.free(); d_sup.free(); d_childmap.free(); d_cursor.free();
    d_outs.free(); d_rec.free(); d_recn.free(); d_keyword.free(); d_listed.free(); d_lnode.free();
    d_head.free(); d_zero.free(); d_mat.free(); h_head.free(); h_mat.free();
    h_desc.free(); h_sup.free(); h_cnt.free(); h_childmap.free(); h_outs.free(); h_keyword.free(); h_misc.free();
    sel_hint = 4096;
    for(auto &g : graphs) {
      if(g.x) cudaGraphExecDestroy(g.x);
      if(g.g) cudaGraphDestroy(g.g);
    }
    graphs.clear();
    if(have_events)
      for(auto &e : ev) cudaEventDestroy(e);
    have_events = false;
    if(stream) {
      cudaStreamSynchronize(stream);
      cudaStreamDestroy(stream);
    }
    stream = nullptr;
    rec_enabled = true;
    wanted_rec = 0;
  }
};

constexpr int kMaxDbSlots = 256;  // databases one scheduler keeps in its device table before it grows
// Waves whose databases hold at most three quarters of the L2 in adjacency
// bytes (12 per entry) skip the entries below a forward rule (sorted
// adjacency): about 97 MiB on a GB300.
int64_t rule_skip_adj_bytes()
{
  static const int64_t v = [] {
    int l2 = 0;
    if(cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, 0) != cudaSuccess || l2 <= 0) {
      cudaGetLastError();
      l2 = 128 << 20;
    }
    return (int64_t)l2 * 3 / 4;
  }();
  return v;
}
// Wave contexts in flight (compile-time tunable): while the GPU works through
// the queued waves, the host completes the oldest and launches new ones.
// Contexts beyond the first two launch only when a full wave of nodes is
// queued: more waves in flight then keep the GPU fed, while a short queue is
// still split in two rather than into many small waves.
#ifndef GS_WAVE_CTX
#define GS_WAVE_CTX 3
#endif
constexpr int kWaveCtx = GS_WAVE_CTX;
static_assert(kWaveCtx <= 8, "WaveCtx::seen_mat holds 8 contexts");

struct Engine {
  // Streams: the engine's (database table, root phases) and one per wave
  // context, so that one wave's selection and materialise passes run beside
  // another's count kernel.  A wave waits (events) for the engine's stream
  // and for every other context's last materialise pass before its count.
  cudaStream_t stream = nullptr;
  cudaStream_t aux = nullptr;   // catch-up copies that must not wait for queued waves
  cudaEvent_t ev_main = nullptr;  // the engine's stream after the last jobs joined
  Pool pool;
  std::unique_ptr<Workers> workers;
  std::vector<MinChecker> checkers;
  std::vector<Column> cols;
  std::vector<int32_t> free_cols;
  std::vector<Block> blocks;
  std::vector<int32_t> free_blocks;
  int64_t pool_limit = 0;
  DBuf<DevDB> d_dbs;
  DBuf<unsigned long long> d_bytes;   // [0] count bytes, [1] materialise bytes, [2] root bytes, [3] flags
  WaveCtx ctx[kWaveCtx];
  // root phases: the root level of a group of jobs, one launch per kernel
  WaveCtx rootx;
  static constexpr int kRootGroup = 64;                    // jobs
  static constexpr int64_t kRootGroupBytes = 1LL << 30;   // bitmap bytes (one job at least)
  bool ready = false;
  // Pool blocks whose last reference was dropped go back to the pool only
  // after every wave context's last materialise pass has completed: the
  // only passes that read a node's memory after the host dropped the node
  // are the materialise passes queued for its wave (the record-driven pass
  // reads records, the enumerating fallback the wave's columns); counts read
  // live nodes only, root phases write new blocks only.  Each context's
  // event 5 follows its latest materialise pass, so when every context's
  // event 5 has completed, every block released so far is free (a later
  // record of an event only makes the wait longer).
  std::vector<void *> released;
  uint64_t main_gen = 0;          // records of ev_main

  void init(int threads)
  {
    if(!ready) {
      CK(cudaSetDevice(0));
      CK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
      CK(cudaStreamCreateWithFlags(&aux, cudaStreamNonBlocking));
      CK(cudaEventCreateWithFlags(&ev_main, cudaEventDisableTiming));
      d_bytes.ensure(4);
      d_dbs.ensure(kMaxDbSlots);
      CK(cudaMemsetAsync(d_bytes.p, 0, sizeof(unsigned long long) * 4, stream));
      for(auto &c : ctx) c.init(true);
      rootx.init(false);
      ready = true;
    }
    pool.set_limit(pool_limit);
    int want = threads > 0 ? threads : (int)std::max(1u, std::thread::hardware_concurrency());
    if(!workers || workers->size() != want) {
      workers.reset(new Workers(want - 1));
      checkers.assign(want, MinChecker());
    }
  }
  void destroy()
  {
    if(!ready) return;
    sync_all();
    released.clear();
    if(ev_main) cudaEventDestroy(ev_main);
    ev_main = nullptr;
    pool.destroy();
    d_dbs.free();
    d_bytes.free();
    for(auto &c : ctx) c.free();
    rootx.free();
    cudaStreamSynchronize(aux);
    cudaStreamDestroy(aux);
    cudaStreamDestroy(stream);
    cols.clear();
    free_cols.clear();
    blocks.clear();
    free_blocks.clear();
    workers.reset();
    ready = false;
  }
  // a pool block of `bytes`; starts with no references
  int32_t new_block(size_t bytes)
  {
    int32_t id;
    if(!free_blocks.empty()) { id = free_blocks.back(); free_blocks.pop_back(); }
    else { id = (int32_t)blocks.size(); blocks.emplace_back(); }
    blocks[id].base = take_pool(bytes);
    blocks[id].refs = 0;
    return id;
  }
  // every stream's work done
  void sync_all()
  {
    if(stream) cudaStreamSynchronize(stream);
    for(auto &c : ctx)
      if(c.stream) cudaStreamSynchronize(c.stream);
  }
  // returns the released blocks to the pool once every context's last
  // materialise pass has completed (wait: waits for them).  Returns false
  // when nothing was released.
  bool reap(bool wait)
  {
    if(released.empty()) return false;
    for(auto &c : ctx) {
      if(!c.have_events) continue;
      const cudaError_t q = cudaEventQuery(c.ev[5]);
      if(q == cudaErrorNotReady) {
        if(!wait) return false;
        CK(cudaEventSynchronize(c.ev[5]));
      } else {
        CK(q);
      }
    }
    for(void *b : released) pool.release(b);
    released.clear();
    return true;
  }
  void *take_pool(size_t bytes)
  {
    reap(false);
    if(void *p = pool.try_alloc(bytes)) return p;
    // released blocks first, the pool grows only when none is left
    if(reap(true))
      if(void *p = pool.try_alloc(bytes)) return p;
    return pool.alloc(bytes);
  }
  void block_ref(int32_t b) { blocks[b].refs++; }
  void block_unref(int32_t b)
  {
    if(--blocks[b].refs == 0) {
      released.push_back(blocks[b].base);
      blocks[b].base = nullptr;
      free_blocks.push_back(b);
    }
  }
  // a column with one reference (its creator's); it takes a reference on its
  // parent column, unless adopt (the parent's creator hands its own over)
  int32_t new_col(int2 *p, int64_t n, int32_t blk, int32_t parent, bool adopt = false)
  {
    int32_t id;
    if(!free_cols.empty()) { id = free_cols.back(); free_cols.pop_back(); }
    else { id = (int32_t)cols.size(); cols.emplace_back(); }
    cols[id].ptr = p;
    cols[id].n = n;
    cols[id].refs = 1;
    cols[id].blk = blk;
    cols[id].parent = parent;
    block_ref(blk);
    if(parent >= 0 && !adopt) cols[parent].refs++;
    return id;
  }
  // drops one reference, and a released column's reference on its parent;
  // returns the bytes of the columns released
  int64_t unref(int32_t id)
  {
    int64_t freed = 0;
    while(id >= 0 && --cols[id].refs == 0) {
      block_unref(cols[id].blk);
      cols[id].ptr = nullptr;
      free_cols.push_back(id);
      freed += cols[id].n * (int64_t)sizeof(int2);
      id = cols[id].parent;
    }
    return freed;
  }
};


// Carves consecutive 256-byte-aligned pieces out of one block.
struct Carver {
  char *base;
  size_t off = 0;
  static size_t round(size_t x) { return (x + 255) & ~(size_t)255; }
  template <class T> T *take(size_t n)
  {
    T *p = (T *)(base + off);
    off += round(sizeof(T) * n);
    return p;
  }
};

std::mutex g_mu;
Engine g_engine;
// engines of the extra schedulers of a batch split over host threads
constexpr int kMaxSchedulers = 4;
Engine g_extra[kMaxSchedulers - 1];
int64_t g_pool_limit = 0;

inline int32_t words_for(int64_t support) { return (int32_t)((support + 31) / 32); }

// Right-most-path slots and key layout of one node (see NodeDesc/SlotDesc).
void layout_node(const PNode &n, const Database &db, NodeLayout &L)
{
  const auto &c = n.code;
  int rm[kMaxPatternEdges];
  L.nrm = build_rmpath(c.data(), (int)c.size(), rm);
  L.maxtoc = c[rm[0]].to;
  const int k = L.maxtoc + 1;
  L.vlab.assign(k, 0);
  L.vlab[0] = c[0].fromlabel;
  for(const DFS &d : c)
    if(d.is_forward()) L.vlab[d.to] = d.tolabel;
  L.slots.assign(L.nrm + 1, SlotDesc{});
  int32_t fk = 0;
  for(int s = 0; s <= L.nrm; s++) {
    SlotDesc &sd = L.slots[s];
    if(s < L.nrm) {
      const DFS &e = c[rm[L.nrm - 1 - s]];
      sd.vertex = e.from;
      sd.fel = e.elabel;
      sd.ftl = e.tolabel;
    } else {
      sd.vertex = L.maxtoc;
      sd.fel = -1;
      sd.ftl = 0;
    }
    sd.vlab = L.vlab[sd.vertex];
    sd.fkey_off = fk;
    fk += db.pair_cnt[sd.vlab];
    sd.bkey_off = -1;
    sd.bel = sd.blab = 0;
    // (fel, ftl) <= (el, tl) lexicographically <=> (fel << 16 | ftl) <= (el << 16 | tl)
    sd.frule = s < L.nrm ? (int32_t)(((uint32_t)sd.fel << 16) | (uint32_t)sd.ftl) : INT32_MIN;
    sd.bmin = INT32_MAX;
  }
  L.nfwd = fk;
  const int32_t rlab = L.vlab[L.maxtoc];
  // backward targets: from-vertices of rmpath edges other than the deepest
  // (slots 0..nrm-2), unless the code already joins them to the right-most vertex
  for(int s = 0; s + 1 < L.nrm; s++) {
    SlotDesc &sd = L.slots[s];
    const DFS &e = c[rm[L.nrm - 1 - s]];
    bool joined = false;
    for(const DFS &d : c)
      if((d.from == L.maxtoc && d.to == sd.vertex) || (d.to == L.maxtoc && d.from == sd.vertex)) joined = true;
    sd.bel = e.elabel;
    sd.blab = e.tolabel;
    sd.bkey_off = joined ? -1 : fk + s * db.EL;
    // bel < el || (bel == el && blab <= label(r))  <=>  el >= bel + (blab > label(r))
    sd.bmin = joined ? INT32_MAX : e.elabel + (e.tolabel > rlab ? 1 : 0);
  }
}

int32_t layout_nkeys(const NodeLayout &L, const Database &db) { return L.nfwd + std::max(0, L.nrm - 1) * db.EL; }

// key -> candidate DFS edge (full labels)
bool decode_key(const NodeLayout &L, const Database &db, int32_t key, DFS &d)
{
  if(key < L.nfwd) {
    for(int s = 0; s <= L.nrm; s++) {
      const SlotDesc &sd = L.slots[s];
      const int32_t cnt = db.pair_cnt[sd.vlab];
      if(key >= sd.fkey_off && key < sd.fkey_off + cnt) {
        const auto &p = db.pairs[sd.vlab][key - sd.fkey_off];
        d = DFS{ sd.vertex, L.maxtoc + 1, sd.vlab, p.first, p.second };
        return true;
      }
    }
    return false;
  }
  const int32_t b = (key - L.nfwd) / db.EL, el = (key - L.nfwd) % db.EL;
  if(b < 0 || b + 1 >= L.nrm) return false;
  const SlotDesc &sd = L.slots[b];
  if(sd.bkey_off < 0) return false;
  d = DFS{ L.maxtoc, sd.vertex, L.vlab[L.maxtoc], el, sd.vlab };
  return true;
}

// order of children in the sequential miner's traversal (gspan.cpp:250-271)
bool seq_before(const DFS &a, const DFS &b)
{
  const bool fa = a.is_forward(), fb = b.is_forward();
  if(fa != fb) return !fa;
  if(!fa) {
    if(a.to != b.to) return a.to < b.to;
    return a.elabel < b.elabel;
  }
  if(a.from != b.from) return a.from > b.from;
  if(a.elabel != b.elabel) return a.elabel < b.elabel;
  return a.tolabel < b.tolabel;
}

template <class T> T *carve(char *base, size_t &off, size_t n)
{
  off = (off + 255) & ~(size_t)255;
  T *p = (T *)(base + off);
  off += sizeof(T) * n;
  return p;
}

double ms_between(cudaEvent_t a, cudaEvent_t b)
{
  float ms = 0;
  if(cudaEventElapsedTime(&ms, a, b) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return ms;
}

// adds the wall time of a scope to a millisecond counter
struct ScopeMs {
  double &acc;
  std::chrono::steady_clock::time_point t0;
  explicit ScopeMs(double &a) : acc(a), t0(std::chrono::steady_clock::now()) {}
  ~ScopeMs() { acc += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count(); }
};

using clk = std::chrono::steady_clock;

double ms_since(clk::time_point t0) { return std::chrono::duration<double, std::milli>(clk::now() - t0).count(); }

// One wave in flight: its nodes and where their descriptors live.
struct Flight {
  bool busy = false;
  bool mat_pending = false;  // the ctx's materialise events still to be read
  uint64_t seq = 0;
  std::vector<int32_t> nodes;  // node pool ids
  std::vector<NodeLayout> lays;
  NodeDesc *hn = nullptr;    // in the ctx's pinned descriptor mirror
  const NodeDesc *dn = nullptr;
  const int2 *const *dc = nullptr;
  const SlotDesc *ds = nullptr;
  const int32_t *dv = nullptr, *dl = nullptr;
  bool join = false;         // some node joins its parent's lists (lists strategy)
  int32_t W = 0, kb = 0, kmax = 1;
  bool small = true;
  bool rule_skip = false;    // the count kernel bisects past forward-rule prefixes
  bool lists = false;        // the wave builds its children's parent-row lists (lists strategy)
  int64_t tb = 0;
  int4 *rec = nullptr;
  long long rec_cap = 0;
  int64_t sel_copied = 0;    // selected entries copied back with the results
  uint32_t *bm = nullptr;    // the wave's support bitmaps (in the zeroed region)
  int32_t *cnt = nullptr;    // its counter copies, cstride apart (cursors of the records materialise)
  long long cstride = 0;
  std::vector<int32_t> sel_at, sel_order;  // the candidates' counting sort by node
};

// The wave scheduler.  Jobs join at any time (add) and leave when their last
// DFS-tree node is done; each step launches waves into the idle contexts and
// completes the oldest wave in flight.  With two contexts the host decodes
// one wave's candidates, checks canonicality and lays out its children while
// the GPU counts the other wave.  Each context issues its waves on its own
// stream: a wave's count waits for the engine's stream (database table, root
// levels) and for every other context's last materialise pass, so that its
// nodes' columns are written before it reads them; pool memory released on
// the host is reused only after every context's last materialise pass has
// completed (Engine::reap).
class Sched {
public:
  Sched(Engine &e, const MineOptions &wo, MineStats &st) : E(e), wo_(wo), st_(st)
  {
    nctx_ = wo_.wave_nodes > 1 ? kWaveCtx : 1;
    E.pool.reset_peak();
    CK(cudaMemsetAsync(E.d_bytes.p, 0, sizeof(unsigned long long) * 4, E.stream));
  }

  // Validates the job, makes its database resident, mines its root level and
  // queues its root nodes.  Returns the job id.
  int32_t add(const MineJob &j)
  {
    const int32_t id = enter(j);
    root_phase(std::vector<int32_t>{ id });
    CK(cudaEventRecord(E.ev_main, E.stream));
    E.main_gen++;
    if(jobs_[id]->pending == 0) complete(id);
    return id;
  }

  // Several jobs at once: their root levels are counted together.
  void add_all(const std::vector<MineJob> &js) { add_all_ids(js); }
  std::vector<int32_t> add_all_ids(const std::vector<MineJob> &js)
  {
    std::vector<int32_t> ids;
    ids.reserve(js.size());
    for(const MineJob &j : js) ids.push_back(enter(j));
    root_phase(ids);
    CK(cudaEventRecord(E.ev_main, E.stream));
    E.main_gen++;
    for(int32_t id : ids)
      if(jobs_[id]->pending == 0) complete(id);
    return ids;
  }

  // A job's checks, its database resident and in the device table, its state.
  int32_t enter(const MineJob &j)
  {
    if(!j.db) throw Error(ST_ERR_USAGE, "null database");
    if(j.minsup < 1) throw Error(ST_ERR_MINSUP_TOO_SMALL, "error: absolute_min_support < 1");
    if(j.minsup >= j.db->host.n_graphs)
      throw Error(ST_ERR_MINSUP_TOO_LARGE, "error: user specified support " + std::to_string(j.minsup) +
                                               " is greater then the database size " +
                                               std::to_string(j.db->host.n_graphs));
    Database *db = j.db;
    if(!db->resident) {
      db->upload();
      st_.h2d_bytes += (int64_t)db->d_bytes;
    }
    int32_t slot = -1;
    for(size_t i = 0; i < dbs_.size(); i++)
      if(dbs_[i] == db) slot = (int32_t)i;
    if(slot < 0) {
      slot = (int32_t)dbs_.size();
      dbs_.push_back(db);
      tab_.push_back(db->dev);
      if(tab_.size() > E.d_dbs.cap) {
        // the table is read by waves in flight: let them finish before it moves
        E.sync_all();
        E.d_dbs.ensure(tab_.size());
        h2d(E.d_dbs.p, tab_.data(), sizeof(DevDB) * tab_.size());
      } else {
        h2d(E.d_dbs.p + slot, &tab_[slot], sizeof(DevDB));
      }
    }
    const int32_t id = (int32_t)jobs_.size();
    jobs_.emplace_back(new JobState());
    JobState &S = *jobs_.back();
    S.job = j;
    S.db_slot = slot;
    active_++;
    order_.push_back(id);
    return id;
  }

  bool idle() const { return active_ == 0; }

  void step()
  {
    for(int c = 0; c < nctx_; c++)
      if(!fl_[c].busy) {
        const bool deep = stacked_ >= (wo_.deep_nodes > 0 ? wo_.deep_nodes : std::max(1, wo_.wave_nodes));
        if(c >= 2 && !deep) continue;
        int idle = 0;
        for(int d = 0; d < nctx_; d++) idle += (!fl_[d].busy && (d < 2 || deep)) ? 1 : 0;
        launch(c, idle);
      }
    int pick = -1;
    for(int c = 0; c < nctx_; c++)
      if(fl_[c].busy && (pick < 0 || fl_[c].seq < fl_[pick].seq)) pick = c;
    if(pick >= 0) finish(pick);
  }

  // Stops a job: its queued nodes are dropped now, the children of its nodes
  // in flight are not made.  It completes (without output) when nothing of it
  // is in flight.
  void cancel(int32_t id)
  {
    JobState *S = job(id);
    if(!S || S->done || S->cancelled) return;
    S->cancelled = true;
    for(int32_t id : S->stack) {
      drop_node(*S, pn_[id]);
      pn_free(id);
    }
    stacked_ -= (int64_t)S->stack.size();
    S->stack.clear();
    if(S->pending == 0) complete(id);
  }

  std::vector<int32_t> take_done()
  {
    std::vector<int32_t> v;
    v.swap(done_);
    return v;
  }
  JobState *job(int32_t id) { return id >= 0 && id < (int32_t)jobs_.size() ? jobs_[id].get() : nullptr; }
  void forget(int32_t id)
  {
    if(job(id) && jobs_[id]->done) jobs_[id].reset();
  }

  // Waits for the last materialise passes and folds the device counters into
  // the statistics; checks the kernels' consistency flags.
  void sync_stats()
  {
    for(int c = 0; c < nctx_; c++) {
      if(fl_[c].mat_pending) {
        CK(cudaEventSynchronize(E.ctx[c].ev[5]));
        st_.mat_ms += ms_between(E.ctx[c].ev[4], E.ctx[c].ev[5]);
        fl_[c].mat_pending = false;
      }
    }
    // every context's passes done before the counters are read
    for(auto &c : E.ctx) CK(cudaStreamSynchronize(c.stream));
    unsigned long long bytes[4] = { 0, 0, 0, 0 };
    d2h(bytes, E.d_bytes.p, sizeof(bytes));
    CK(cudaStreamSynchronize(E.stream));
    E.reap(false);
    CK(cudaGetLastError());
    check_flags(bytes[3]);
    st_.count_bytes += (int64_t)bytes[0] - seen_bytes_[0];
    st_.mat_bytes += (int64_t)bytes[1] - seen_bytes_[1];
    seen_bytes_[0] = (int64_t)bytes[0];
    seen_bytes_[1] = (int64_t)bytes[1];
    st_.peak_pool_bytes = std::max<int64_t>(st_.peak_pool_bytes, (int64_t)E.pool.peak());
  }

  int64_t pool_used() const { return (int64_t)E.pool.used(); }

private:
  Engine &E;
  const MineOptions &wo_;
  MineStats &st_;
  int nctx_ = kWaveCtx;
  std::deque<PNode> pn_;          // DFS-tree nodes (stacks and waves hold their ids)
  std::vector<int32_t> pn_free_;
  Flight fl_[kWaveCtx];
  uint64_t seq_ = 0;
  std::vector<std::unique_ptr<JobState>> jobs_;
  std::vector<int32_t> order_;   // unfinished jobs, oldest first
  std::vector<int32_t> done_;
  std::vector<Database *> dbs_;
  std::vector<char> db_seen_;  // wave building: database slots met
  std::vector<DevDB> tab_;
  int64_t active_ = 0;
  int64_t stacked_ = 0;          // nodes on all jobs' stacks
  int64_t seen_bytes_[2] = { 0, 0 };
  bool defer_emit_ = false;
  // per-wave scratch of finish(), reused
  struct Mat { int32_t node, cand, pid; };
  std::vector<Candidate> w_cands_;
  std::vector<int32_t> w_todo_, w_made_, w_made_at_, w_acc_, w_touched_;
  std::vector<ChildOut> w_outs_;
  std::vector<int2> w_pairs_;
  std::vector<Mat> w_mats_;

  // a wave context's stream (all on the engine's with the serial option)
  cudaStream_t cs(const WaveCtx &X) const { return wo_.serial ? E.stream : X.stream; }
  void h2d(void *dst, const void *src, size_t n, cudaStream_t s = nullptr)
  {
    CK(cudaMemcpyAsync(dst, src, n, cudaMemcpyHostToDevice, s ? s : E.stream));
    st_.h2d_bytes += (int64_t)n;
  }
  void d2h(void *dst, const void *src, size_t n, cudaStream_t s = nullptr)
  {
    CK(cudaMemcpyAsync(dst, src, n, cudaMemcpyDeviceToHost, s ? s : E.stream));
    st_.d2h_bytes += (int64_t)n;
  }
  // device consistency flags (slot 3 of the counters)
  unsigned int *err_flag() { return reinterpret_cast<unsigned int *>(E.d_bytes.p + 3); }
  static void check_flags(unsigned long long v)
  {
    if(v & 8) throw Error(ST_ERR_LIMIT, "a pattern has 2^31 or more embeddings in one wave");
    if(v) throw Error(ST_ERR_STATE, "kernel consistency check failed (flags " + std::to_string(v) + ")");
  }

  // DFS-tree node pool: nodes stay in place (a deque keeps references valid
  // while it grows) and stacks and waves pass their ids around
  int32_t pn_new()
  {
    int32_t id;
    if(!pn_free_.empty()) {
      id = pn_free_.back();
      pn_free_.pop_back();
    } else {
      id = (int32_t)pn_.size();
      pn_.emplace_back();
    }
    PNode &p = pn_[id];
    p.code.assign(nullptr, 0);
    p.cols.assign(nullptr, 0);
    p.last_col = -1;
    p.list_blk = -1;
    p.list_off = nullptr;
    p.list_ent = nullptr;
    p.list_rows = 0;
    p.join_lo = p.join_key = p.join_hi = 0;
    return id;
  }
  void pn_free(int32_t id) { pn_free_.push_back(id); }

  // releases a node's columns and graph ranks
  void drop_node(JobState &S, PNode &p)
  {
    S.live_bytes -= E.unref(p.last_col);
    p.last_col = -1;
    S.live_bytes -= p.nrows * (int64_t)sizeof(int32_t);
    E.block_unref(p.gord_blk);
    if(p.list_blk >= 0) E.block_unref(p.list_blk);
    p.list_blk = -1;
    S.pending--;
  }

  void complete(int32_t id)
  {
    JobState &S = *jobs_[id];
    S.done = true;
    active_--;
    order_.erase(std::find(order_.begin(), order_.end(), id));
    done_.push_back(id);
    if(!S.cancelled) {
      S.patterns = (int64_t)S.pats.size();
      st_.patterns += S.patterns;
      if(defer_emit_) return;  // emitted later by emit_deferred, on the caller's thread
      ScopeMs t(st_.host_emit_ms);
      emit(S);
    }
    std::vector<PatternRec>().swap(S.pats);
    std::vector<int32_t>().swap(S.roots);
    std::vector<int32_t>().swap(S.root_keys);
  }

public:
  // Schedulers run on worker threads keep the finished jobs' pattern trees
  // and emit them when the caller asks (the callbacks stay on its thread).
  void set_defer_emit(bool v) { defer_emit_ = v; }
  void emit_deferred(int32_t id)
  {
    JobState &S = *jobs_[id];
    if(!S.done || S.cancelled) return;
    {
      ScopeMs t(st_.host_emit_ms);
      emit(S);
    }
    release_patterns(id);
  }
  // a job split by root subtrees: its parts' roots are merged in the
  // reference's root order (root keys), one root subtree at a time
  const std::vector<int32_t> &root_keys(int32_t id) const { return jobs_[id]->root_keys; }
  void emit_root(int32_t id, size_t r)
  {
    JobState &S = *jobs_[id];
    if(!S.done || S.cancelled) return;
    ScopeMs t(st_.host_emit_ms);
    emit(S, r, r + 1);
  }
  void release_patterns(int32_t id)
  {
    JobState &S = *jobs_[id];
    std::vector<PatternRec>().swap(S.pats);
    std::vector<int32_t>().swap(S.roots);
    std::vector<int32_t>().swap(S.root_keys);
  }

private:

  // ---- root level: all frequent 1-edge codes of one job
  // The root level of jobs, in groups: every root triple's support and
  // embedding count for all jobs of a group (one launch of each kernel), read
  // back after one host wait; the frequent roots of each job in the
  // reference's order; their first embeddings (one launch for the group).
  static int32_t root_copies(int32_t R)
  {
    // copies of the root counters: every vertex adds into a few hundred counters
    return (int32_t)std::max<int64_t>(1, std::min<int64_t>(64, ((int64_t)1 << 20) / R));
  }

  void root_phase(const std::vector<int32_t> &ids)
  {
    size_t i = 0;
    while(i < ids.size()) {
      std::vector<RootJob> rj;
      std::vector<int32_t> gid;
      int64_t bmw = 0, cntn = 0;
      int32_t keys = 0;
      long long tiles = 0;
      for(; i < ids.size() && (int)rj.size() < Engine::kRootGroup; i++) {
        JobState &S = *jobs_[ids[i]];
        Database &db = *S.job.db;
        const int32_t R = db.root_keys;
        if(R == 0) continue;
        const int32_t words = words_for(db.host.n_graphs);
        const int64_t nw = (int64_t)R * words;
        if(!rj.empty() && (bmw + nw) * 4 > Engine::kRootGroupBytes) break;
        RootJob J{};
        J.tile_begin = tiles;
        J.bm_base = bmw;
        J.cnt_base = cntn;
        J.db = S.db_slot;
        J.words = words;
        J.R = R;
        J.copies = root_copies(R);
        J.key_base = keys;
        rj.push_back(J);
        gid.push_back(ids[i]);
        tiles += ((long long)db.dev.n_vertices + 31) / 32;
        bmw += nw;
        cntn += (int64_t)R * J.copies;
        keys += R;
      }
      if(!rj.empty()) root_group(rj, gid, tiles, bmw, cntn, keys);
    }
  }

  void root_group(const std::vector<RootJob> &rj, const std::vector<int32_t> &gid, long long tiles, int64_t bmw,
                  int64_t cntn, int32_t keys)
  {
    WaveCtx &X = E.rootx;
    const int32_t n = (int32_t)rj.size();
    // the pinned mirrors below were last read by the previous group's copies
    CK(cudaEventSynchronize(X.ev[5]));
    X.d_bm.ensure(bmw);
    X.d_bmx.ensure(bmw);
    X.d_cnt.ensure(cntn);
    X.d_sup.ensure(2 * (size_t)keys);  // supports, then embeddings
    X.d_childmap.ensure(keys);
    // pseudo nodes spanning each job's root keys (for the support kernel), then the job table
    const size_t nd_bytes = sizeof(NodeDesc) * n, tab_bytes = nd_bytes + sizeof(RootJob) * n;
    X.d_desc.ensure(tab_bytes);
    X.h_desc.ensure(tab_bytes);
    NodeDesc *hn = (NodeDesc *)X.h_desc.p;
    for(int32_t q = 0; q < n; q++) {
      NodeDesc nd{};
      nd.words = rj[q].words;
      nd.nkeys = rj[q].R;
      nd.key_base = rj[q].key_base;
      nd.bm_base = rj[q].bm_base;
      hn[q] = nd;
    }
    std::memcpy(X.h_desc.p + nd_bytes, rj.data(), sizeof(RootJob) * n);
    h2d(X.d_desc.p, X.h_desc.p, tab_bytes);
    const NodeDesc *d_nd = (const NodeDesc *)X.d_desc.p;
    const RootJob *d_rj = (const RootJob *)(X.d_desc.p + nd_bytes);
    CK(cudaMemsetAsync(X.d_bm.p, 0, (size_t)bmw * 4, E.stream));
    CK(cudaMemsetAsync(X.d_cnt.p, 0, (size_t)cntn * 4, E.stream));
    CK(cudaEventRecord(X.ev[0], E.stream));
    launch_root_count(d_rj, n, tiles, E.d_dbs.p, X.d_bm.p, X.d_cnt.p, X.d_sup.p + keys, keys, E.d_bytes.p + 2,
                      E.stream);
    launch_support(d_nd, n, keys, X.d_bm.p, X.d_bmx.p, X.d_sup.p, E.stream);
    CK(cudaEventRecord(X.ev[1], E.stream));
    st_.launches += 3;
    X.h_sup.ensure(2 * (size_t)keys);
    d2h(X.h_sup.p, X.d_sup.p, (size_t)keys * 8);
    d2h(X.h_misc.p + 1, E.d_bytes.p + 3, sizeof(unsigned long long));
    CK(cudaEventRecord(X.ev[3], E.stream));
    {
      const clk::time_point t0 = clk::now();
      CK(cudaEventSynchronize(X.ev[3]));
      st_.host_wait_ms += ms_since(t0);
    }
    CK(cudaGetLastError());
    check_flags(X.h_misc.p[1]);
    st_.root_ms += ms_between(X.ev[0], X.ev[1]);

    std::vector<ChildOut> outs;
    std::vector<std::vector<int32_t>> made(n);
    X.h_childmap.ensure(keys);
    for(int32_t k = 0; k < keys; k++) X.h_childmap.p[k] = -1;
    const int32_t *hsup = X.h_sup.p, *hcnt = X.h_sup.p + keys;
    for(int32_t q = 0; q < n; q++) {
      const int32_t id = gid[q];
      JobState &S = *jobs_[id];
      Database &db = *S.job.db;
      const int32_t kb = rj[q].key_base;
      const bool extend = S.job.opt.max_edges != 1;
      // frequent roots of this job (and partition), in the reference's order
      struct Sel { int32_t key, pid; DFS d; int32_t sup; int64_t n; };
      std::vector<Sel> sel;
      int32_t root_index = 0;
      size_t bytes = 0;
      for(int32_t fl = 0; fl < db.VL; fl++) {
        for(size_t p = 0; p < db.pairs[fl].size(); p++) {
          const int32_t el = db.pairs[fl][p].first, tl = db.pairs[fl][p].second;
          if(tl < fl) continue;
          const int32_t key = kb + db.root_off[fl] + (int32_t)p;
          const int32_t sup = hsup[key];
          if(sup < S.job.minsup) continue;
          // root-subtree partition: independent subtrees, no exchange between parts
          const int32_t ri = root_index++;
          if(S.job.opt.root_parts > 1 && ri % S.job.opt.root_parts != S.job.opt.root_part) continue;
          PatternRec pr{ -1, DFS{ 0, 1, fl, el, tl }, sup };
          S.pats.push_back(pr);
          const int32_t pid = (int32_t)S.pats.size() - 1;
          S.roots.push_back(pid);
          S.root_keys.push_back(key - kb);
          if(!extend) continue;
          const int64_t rows = hcnt[key];
          sel.push_back(Sel{ key, pid, pr.edge, sup, rows });
          bytes += 2 * Carver::round((size_t)rows * 8) + Carver::round((size_t)rows * 4);
        }
      }
      if(sel.empty()) continue;
      // all root columns and ranks of the job in one pool block
      const int32_t blk = E.new_block(bytes);
      Carver cv{ (char *)E.blocks[blk].base };
      for(const Sel &s : sel) {
        int2 *c1 = cv.take<int2>(s.n);
        int2 *c0 = cv.take<int2>(s.n);
        int32_t *gord = cv.take<int32_t>(s.n);
        ChildOut o{ c1, c0, gord, 2, (int32_t)s.n };
        X.h_childmap.p[s.key] = (int32_t)outs.size();
        outs.push_back(o);
        const int32_t nid = pn_new();
        PNode &nn = pn_[nid];
        nn.job = id;
        nn.pattern = s.pid;
        nn.code.push_back(s.d);
        const int32_t id0 = E.new_col(c0, s.n, blk, -1);
        nn.last_col = E.new_col(c1, s.n, blk, id0, true);
        nn.cols.push_back(ColRef{ c0, s.n });
        nn.cols.push_back(ColRef{ c1, s.n });
        nn.gord = gord;
        nn.gord_blk = blk;
        E.block_ref(blk);
        nn.nrows = s.n;
        nn.support = s.sup;
        S.live_bytes += s.n * (int64_t)(2 * sizeof(int2) + sizeof(int32_t));
        made[q].push_back(nid);
      }
      S.peak_bytes = std::max(S.peak_bytes, S.live_bytes);
    }
    if(!outs.empty()) {
      X.d_outs.ensure(outs.size());
      X.h_outs.ensure(outs.size());
      std::memcpy(X.h_outs.p, outs.data(), sizeof(ChildOut) * outs.size());
      h2d(X.d_outs.p, X.h_outs.p, sizeof(ChildOut) * outs.size());
      h2d(X.d_childmap.p, X.h_childmap.p, (size_t)keys * 4);
      // cursors: the counter copies hold each copy's offset (copy 0 at 0)
      launch_root_materialize(d_rj, n, tiles, E.d_dbs.p, X.d_bm.p, X.d_bmx.p, X.d_cnt.p, X.d_childmap.p, X.d_outs.p,
                              err_flag(), E.stream);
      st_.launches++;
    }
    CK(cudaEventRecord(X.ev[5], E.stream));
    for(int32_t q = 0; q < n; q++) {
      JobState &S = *jobs_[gid[q]];
      S.pending += (int64_t)made[q].size();
      stacked_ += (int64_t)made[q].size();
      for(auto it = made[q].rbegin(); it != made[q].rend(); ++it) S.stack.push_back(*it);
    }
  }

  // Queues a wave's device work: replayed from the context's CUDA graph for
  // its count-kernel variant (node parameters updated), or launched directly.
  void issue(WaveCtx &X, WaveSeq &q)
  {
    const cudaStream_t st = cs(X);
    st_.h2d_bytes += (int64_t)q.desc_bytes;
    st_.d2h_bytes += (int64_t)q.d2h_bytes;
    if(wo_.launch_mode != 0) {
      CK(cudaMemcpyAsync(q.desc_dst, q.desc_src, q.desc_bytes, cudaMemcpyHostToDevice, st));
      CK(cudaMemsetAsync(q.zero, 0, q.zero_bytes, st));
      CK(cudaMemsetAsync(q.head, 0, kHeadBytes, st));
      CK(cudaEventRecord(X.ev[0], st));
      CK(q.count.run(st));
      CK(cudaEventRecord(X.ev[1], st));
      CK(q.screen.run(st));
      CK(q.listed.run(st));
      CK(cudaEventRecord(X.ev[6], st));
      if(q.with_min) CK(q.ismin.run(st));
      CK(cudaEventRecord(X.ev[2], st));
      CK(cudaMemcpyAsync(q.head_host, q.head, q.d2h_bytes, cudaMemcpyDeviceToHost, st));
      CK(cudaEventRecord(X.ev[3], st));
      return;
    }
    WaveGraph *G = nullptr;
    for(auto &g : X.graphs)
      if(g.count_func == q.count.func && g.with_min == q.with_min) G = &g;
    const cudaMemsetParams mz = clear_params(q.zero, q.zero_bytes), mh = clear_params(q.head, kHeadBytes);
    cudaKernelNodeParams kc = kernel_params(q.count), ks = kernel_params(q.screen), kl = kernel_params(q.listed);
    cudaKernelNodeParams km{};
    if(q.with_min) km = kernel_params(q.ismin);
    if(!G) {
      X.graphs.emplace_back();
      G = &X.graphs.back();
      G->count_func = q.count.func;
      G->with_min = q.with_min;
      cudaGraph_t g;
      CK(cudaGraphCreate(&g, 0));
      G->g = g;
      cudaGraphNode_t e0, e1, e2, e3, e6, last;
      CK(cudaGraphAddMemcpyNode1D(&G->h2d, g, nullptr, 0, q.desc_dst, q.desc_src, q.desc_bytes,
                                  cudaMemcpyHostToDevice));
      CK(cudaGraphAddMemsetNode(&G->mz, g, &G->h2d, 1, &mz));
      CK(cudaGraphAddMemsetNode(&G->mh, g, &G->mz, 1, &mh));
      CK(cudaGraphAddEventRecordNode(&e0, g, &G->mh, 1, X.ev[0]));
      CK(cudaGraphAddKernelNode(&G->count, g, &e0, 1, &kc));
      CK(cudaGraphAddEventRecordNode(&e1, g, &G->count, 1, X.ev[1]));
      CK(cudaGraphAddKernelNode(&G->screen, g, &e1, 1, &ks));
      CK(cudaGraphAddKernelNode(&G->listed, g, &G->screen, 1, &kl));
      CK(cudaGraphAddEventRecordNode(&e6, g, &G->listed, 1, X.ev[6]));
      last = e6;
      if(q.with_min) {
        CK(cudaGraphAddKernelNode(&G->ismin, g, &last, 1, &km));
        last = G->ismin;
      }
      CK(cudaGraphAddEventRecordNode(&e2, g, &last, 1, X.ev[2]));
      CK(cudaGraphAddMemcpyNode1D(&G->d2h, g, &e2, 1, q.head_host, q.head, q.d2h_bytes, cudaMemcpyDeviceToHost));
      CK(cudaGraphAddEventRecordNode(&e3, g, &G->d2h, 1, X.ev[3]));
      CK(cudaGraphInstantiate(&G->x, g, 0));
    } else {
      CK(cudaGraphExecMemcpyNodeSetParams1D(G->x, G->h2d, q.desc_dst, q.desc_src, q.desc_bytes,
                                            cudaMemcpyHostToDevice));
      CK(cudaGraphExecMemsetNodeSetParams(G->x, G->mz, &mz));
      CK(cudaGraphExecMemsetNodeSetParams(G->x, G->mh, &mh));
      CK(cudaGraphExecKernelNodeSetParams(G->x, G->count, &kc));
      CK(cudaGraphExecKernelNodeSetParams(G->x, G->screen, &ks));
      CK(cudaGraphExecKernelNodeSetParams(G->x, G->listed, &kl));
      if(q.with_min) CK(cudaGraphExecKernelNodeSetParams(G->x, G->ismin, &km));
      CK(cudaGraphExecMemcpyNodeSetParams1D(G->x, G->d2h, q.head_host, q.head, q.d2h_bytes, cudaMemcpyDeviceToHost));
    }
    CK(cudaGraphLaunch(G->x, st));
  }

  // ---- launch one wave into context c: descriptors, count, support, results copy
  void launch(int c, int idle)
  {
    const clk::time_point t_begin = clk::now();
    WaveCtx &X = E.ctx[c];
    Flight &f = fl_[c];
    if(stacked_ == 0) return;
    // with other contexts idle take an equal share of what is queued, so that
    // every context has work and the host's share overlaps the GPU's
    int64_t limit = std::max(1, wo_.wave_nodes);
    if(nctx_ > 1 && idle > 1) limit = std::max<int64_t>(1, std::min<int64_t>(limit, (stacked_ + idle - 1) / idle));
    std::vector<int32_t> &nodes = f.nodes;
    std::vector<NodeLayout> &lays = f.lays;  // kept between waves: layouts reuse their vectors
    nodes.clear();
    int64_t rows = 0, words = 0, wkeys = 0;
    bool full = false;
    for(size_t oi = 0; oi < order_.size() && !full; oi++) {
      JobState &S = *jobs_[order_[oi]];
      const Database &db = *S.job.db;
      while(!S.stack.empty() && (int64_t)nodes.size() < limit) {
        const PNode &top = pn_[S.stack.back()];
        if(lays.size() <= nodes.size()) lays.emplace_back();
        NodeLayout &L = lays[nodes.size()];
        layout_node(top, db, L);
        const int32_t nk = layout_nkeys(L, db);
        const int64_t w = (int64_t)nk * words_for(top.support);
        // (keys per wave stay below 2^26: records carry a wave key in 27 bits)
        if(!nodes.empty() && (rows + top.nrows > wo_.wave_rows || words + w > wo_.wave_words ||
                              wkeys + nk >= ((int64_t)1 << 26))) {
          full = true;
          break;
        }
        rows += top.nrows;
        words += w;
        wkeys += nk;
        nodes.push_back(S.stack.back());
        S.stack.pop_back();
        stacked_--;
      }
      if((int64_t)nodes.size() >= limit) full = true;
    }
    const int32_t W = (int32_t)nodes.size();
    if(W == 0) return;
    st_.waves++;
    st_.nodes += W;
    st_.rows += rows;

    // descriptors
    int32_t tot_cols = 0, tot_slots = 0, tot_edges = 0;
    bool any_join = false;
    for(int32_t n = 0; n < W; n++) {
      const PNode &p = pn_[nodes[n]];
      tot_cols += (int32_t)p.cols.size();
      tot_slots += (int32_t)lays[n].slots.size();
      tot_edges += (int32_t)p.code.size();
      any_join = any_join || p.list_off != nullptr;
    }
    size_t off = 0;
    size_t need = 256 * 7 + sizeof(NodeDesc) * W + sizeof(int2 *) * tot_cols + sizeof(SlotDesc) * tot_slots +
                  2 * sizeof(int32_t) * tot_cols + 5 * sizeof(int32_t) * tot_edges;
    X.h_desc.ensure(need);
    X.d_desc.ensure(need);
    char *hb = X.h_desc.p;
    NodeDesc *hn = carve<NodeDesc>(hb, off, W);
    const int2 **hc = carve<const int2 *>(hb, off, tot_cols);
    SlotDesc *hs = carve<SlotDesc>(hb, off, tot_slots);
    int32_t *hv = carve<int32_t>(hb, off, tot_cols);
    int32_t *hl = carve<int32_t>(hb, off, tot_cols);
    int32_t *hcode = carve<int32_t>(hb, off, 5 * (size_t)tot_edges);
    const size_t desc_bytes = off;
    int32_t eo = 0;
    int32_t co = 0, so = 0, kmax = 1;
    bool small = true;  // every database of the wave has graphs of <= 64 vertices
    // adjacency bytes (entries and pair indices) of the wave's databases
    int64_t adj_bytes = 0;
    db_seen_.assign(dbs_.size(), 0);
    int64_t rb = 0, bb = 0, tb = 0;
    int32_t kb = 0;
    for(int32_t n = 0; n < W; n++) {
      const PNode &p = pn_[nodes[n]];
      const NodeLayout &L = lays[n];
      const JobState &S = *jobs_[p.job];
      const Database &db = *S.job.db;
      NodeDesc &d = hn[n];
      d = NodeDesc{};
      d.row_begin = rb;
      d.tile_begin = tb;
      d.bm_base = bb;
      d.gord = p.gord;
      d.nrows = (int32_t)p.nrows;
      d.k = (int32_t)p.cols.size();
      d.col_off = co;
      d.slot_off = so;
      d.vtab_off = co;
      d.nslot = (int32_t)L.slots.size();
      d.minlabel = p.code[0].fromlabel;
      d.words = words_for(p.support);
      d.key_base = kb;
      d.nkeys = layout_nkeys(L, db);
      d.db = S.db_slot;
      d.minsup = S.job.minsup;
      d.code_off = eo;
      d.code_len = (int32_t)p.code.size();
      d.nfwd = L.nfwd;
      if(p.list_off) {
        // lists strategy: join the parent's per-row lists
        d.csr_off = p.list_off;
        d.csr_ent = p.list_ent;
        d.csr_rows = (int32_t)p.list_rows;
        d.join_lo = p.join_lo;
        d.join_key = p.join_key;
        d.join_hi = p.join_hi;
        st_.join_nodes++;
      }
      for(const DFS &e : p.code) {
        int32_t *c = hcode + 5 * (size_t)eo++;
        c[0] = e.from;
        c[1] = e.to;
        c[2] = e.fromlabel;
        c[3] = e.elabel;
        c[4] = e.tolabel;
      }
      for(size_t cc = 0; cc < p.cols.size(); cc++) {
        hc[co + cc] = p.cols[cc].ptr;
        hl[co + cc] = (int32_t)p.cols[cc].n;
        hv[co + cc] = -1;
      }
      for(size_t s = 0; s < L.slots.size(); s++) {
        hs[so + s] = L.slots[s];
        if(L.slots[s].bkey_off >= 0) hv[co + L.slots[s].vertex] = (int32_t)s;
      }
      co += d.k;
      so += d.nslot;
      kmax = std::max(kmax, d.k);
      small = small && db.dev.max_graph_vertices <= 64;
      if(!db_seen_[S.db_slot]) {
        db_seen_[S.db_slot] = 1;
        adj_bytes += 12 * db.n_adj();
      }
      rb += p.nrows;
      tb += (p.nrows + 31) / 32;
      bb += (int64_t)d.nkeys * d.words;
      kb += d.nkeys;
    }
    char *db_ = X.d_desc.p;
    f.hn = hn;
    f.dn = (const NodeDesc *)(db_ + ((char *)hn - hb));
    f.dc = (const int2 *const *)(db_ + ((char *)hc - hb));
    f.ds = (const SlotDesc *)(db_ + ((char *)hs - hb));
    f.dv = (const int32_t *)(db_ + ((char *)hv - hb));
    f.dl = (const int32_t *)(db_ + ((char *)hl - hb));
    const int32_t *dcode = (const int32_t *)(db_ + ((char *)hcode - hb));
    f.join = any_join;
    f.W = W;
    f.kb = kb;
    f.kmax = kmax;
    f.small = small;
    // The bisection's loads are dependent and one per lane: they pay off while
    // the adjacency stays in L2 (configuration 2, 72 MB: count kernel 3%
    // faster) and cost more than the skipped items save beyond it
    // (configuration 5, 960 MB: 10% slower)
    f.rule_skip = adj_bytes <= rule_skip_adj_bytes();
    // lists strategy: always (1), or (2) for waves whose databases do not stay
    // in L2, where the joins save rescans of adjacency from DRAM
    f.lists = wo_.extension == 1 || (wo_.extension == 2 && !f.rule_skip);
    f.tb = tb;
    // copies of the wave's counters: the warps of a large node all add into that
    // node's few counters; copies spread them over L2 slices (summed by screening)
    // (records hold a key in 27 bits next to the copy: one copy beyond that)
    const int32_t ccopies =
        kb >= (1 << 27) ? 1 : (int32_t)std::max<int64_t>(1, std::min<int64_t>(16, ((int64_t)1 << 22) / std::max(kb, 1)));
    const long long cstride = (long long)Carver::round(sizeof(int32_t) * (size_t)std::max(kb, 1)) / 4;
    const size_t cnt_bytes = sizeof(int32_t) * (size_t)cstride * ccopies;
    const size_t zero_bytes = cnt_bytes + sizeof(uint32_t) * (size_t)std::max<int64_t>(bb, 1);
    X.d_zero.ensure(zero_bytes);
    X.d_head.ensure(kHeadBytes + sizeof(int4) * (size_t)std::max(kb, 1));
    X.d_bmx.ensure(std::max<int64_t>(bb, 1));
    X.d_childmap.ensure(std::max(kb, 1));
    X.d_keyword.ensure(std::max(kb, 1));
    X.d_listed.ensure(std::max(kb, 1));
    int32_t *cnt = (int32_t *)X.d_zero.p;
    f.cnt = cnt;
    f.cstride = cstride;
    f.bm = (uint32_t *)(X.d_zero.p + cnt_bytes);
    unsigned long long *head = (unsigned long long *)X.d_head.p;
    int4 *sel = (int4 *)(X.d_head.p + kHeadBytes);
    // records: how many the wave appends is not known up front, so keep the
    // largest count seen (grown after an overflow)
    f.rec = nullptr;
    f.rec_cap = 0;
    if(X.rec_enabled && X.wanted_rec > (long long)X.d_rec.cap) {
      // past 2^28 records (4 GiB) or when the device has no room, keep the
      // enumeration-based materialise instead
      if(X.wanted_rec > (1ll << 28)) X.rec_enabled = false;
      else {
        try {
          X.d_rec.ensure((size_t)X.wanted_rec);
        } catch(const Error &) {
          cudaGetLastError();
          X.rec_enabled = false;
        }
      }
    }
    if(X.rec_enabled) {
      if(X.d_rec.cap == 0) X.d_rec.ensure((size_t)1 << 22);
      f.rec = X.d_rec.p;
      f.rec_cap = (long long)X.d_rec.cap;
    }
    // the frequent candidates come back compacted: a prefix sized from earlier
    // waves, the rest (rarely) by a second copy
    f.sel_copied = std::min<int64_t>(kb, X.sel_hint);
    X.h_head.ensure(kHeadBytes + sizeof(int4) * (size_t)std::max<int64_t>(f.sel_copied, 1));
    WaveSeq q;
    q.desc_dst = X.d_desc.p;
    q.desc_src = hb;
    q.desc_bytes = desc_bytes;
    q.zero = X.d_zero.p;
    q.zero_bytes = zero_bytes;
    q.head = X.d_head.p;
    q.head_host = X.h_head.p;
    q.d2h_bytes = kHeadBytes + sizeof(int4) * (size_t)f.sel_copied;
    q.count = wave_count_call(f.dn, W, tb, kmax, small, f.dc, f.dl, f.ds, f.dv, E.d_dbs.p, f.bm, cnt, E.d_bytes.p + 0,
                              err_flag(), f.rec, f.rec_cap, f.rec ? head + kHeadRecords : nullptr,
                              wo_.count_grid, ccopies, cstride, f.join, f.rule_skip);
    int32_t *lnode = nullptr;
    if(f.lists) {
      X.d_lnode.ensure(std::max(kb, 1));
      lnode = X.d_lnode.p;
    }
    q.screen = screen_keys_call(f.dn, W, kb, cnt, ccopies, cstride, X.d_childmap.p, X.d_listed.p,
                                head + kHeadSelected, err_flag(), head + kHeadFlags, lnode);
    q.listed = count_listed_call(f.dn, X.d_listed.p, f.bm, cnt, X.d_bmx.p, X.d_keyword.p, sel, kb,
                                 head + kHeadSelected, lnode);
    q.with_min = wo_.min_check == 0;
    if(q.with_min) q.ismin = is_min_call(f.dn, W, f.ds, E.d_dbs.p, dcode, sel, kb, head + kHeadSelected);
    // the wave's nodes were made by the root phases (engine stream) or by
    // other contexts' materialise passes (their last ones cover every node
    // made so far; this context's own are ahead on its stream)
    if(!wo_.serial) {
      if(X.seen_main != E.main_gen) {
        CK(cudaStreamWaitEvent(X.stream, E.ev_main, 0));
        X.seen_main = E.main_gen;
      }
      for(int d = 0; d < kWaveCtx; d++)
        if(d != c && X.seen_mat[d] != E.ctx[d].mat_gen) {
          CK(cudaStreamWaitEvent(X.stream, E.ctx[d].ev[5], 0));
          X.seen_mat[d] = E.ctx[d].mat_gen;
        }
    }
    issue(X, q);
    st_.launches += q.with_min ? 4 : 3;
    f.busy = true;
    f.seq = ++seq_;
    st_.host_build_ms += ms_since(t_begin);
  }

  // ---- complete the wave in context c: candidates, canonicality, children
  void finish(int c)
  {
    WaveCtx &X = E.ctx[c];
    const cudaStream_t st = cs(X);
    Flight &f = fl_[c];
    {
      const clk::time_point t0 = clk::now();
      CK(cudaEventSynchronize(X.ev[3]));
      st_.host_wait_ms += ms_since(t0);
    }
    CK(cudaGetLastError());
    const unsigned long long *hh = (const unsigned long long *)X.h_head.p;
    check_flags(hh[kHeadFlags]);
    const clk::time_point t_ready = clk::now();
    const double min_before = st_.host_min_ms;
    if(f.mat_pending) {
      // this context's previous materialise ran before the count just read
      st_.mat_ms += ms_between(X.ev[4], X.ev[5]);
      f.mat_pending = false;
    }
    st_.count_ms += ms_between(X.ev[0], X.ev[1]);
    st_.support_ms += ms_between(X.ev[1], X.ev[2]);
    st_.sel_ms += ms_between(X.ev[1], X.ev[6]);
    st_.min_ms += ms_between(X.ev[6], X.ev[2]);
    std::vector<int32_t> &nodes = f.nodes;
    std::vector<NodeLayout> &lays = f.lays;
    const NodeDesc *hn = f.hn;
    const int32_t W = f.W, kb = f.kb;

    // frequent candidates (compacted on the device)
    const int64_t nsel = (int64_t)hh[kHeadSelected];
    const long long nrec = f.rec ? (long long)hh[kHeadRecords] : -1;
    st_.extensions += (int64_t)hh[kHeadExt];
    st_.sel_bytes += (int64_t)hh[kHeadSelBytes];
    // the count kernel's bytes per extension (bitmap word and counter, and the
    // record when records are on), counted here rather than in its inner loop
    st_.count_bytes += (int64_t)hh[kHeadExt] * (8 + (f.rec ? 16 : 0));
    if(nsel > kb) throw Error(ST_ERR_STATE, "candidate selection overflow");
    if(nsel > f.sel_copied) {
      // copies the whole list again (growing the pinned buffer drops its
      // contents) on the side stream: the wave's results are complete, and the
      // main stream already holds the other context's wave
      X.h_head.ensure(kHeadBytes + sizeof(int4) * (size_t)nsel);
      CK(cudaMemcpyAsync(X.h_head.p, X.d_head.p, kHeadBytes + sizeof(int4) * (size_t)nsel, cudaMemcpyDeviceToHost,
                         E.aux));
      CK(cudaStreamSynchronize(E.aux));
      st_.d2h_bytes += (int64_t)(kHeadBytes + sizeof(int4) * nsel);
    }
    const int4 *hsel = (const int4 *)(X.h_head.p + kHeadBytes);
    X.sel_hint = std::max<int64_t>(X.sel_hint, 2 * nsel);
    // the candidates grouped by node (the selection records each one's node):
    // a counting sort, each node's in any order (children are ordered below)
    std::vector<int32_t> &at = f.sel_at;
    at.assign((size_t)W + 1, 0);
    for(int64_t i = 0; i < nsel; i++) {
      const int32_t n = hsel[i].w >> 2;
      if(n < 0 || n >= W) throw Error(ST_ERR_STATE, "selected key outside the wave's nodes");
      at[n + 1]++;
    }
    for(int32_t n = 0; n < W; n++) at[n + 1] += at[n];
    std::vector<int32_t> &order = f.sel_order;
    order.resize((size_t)nsel);
    for(int64_t i = 0; i < nsel; i++) order[at[hsel[i].w >> 2]++] = (int32_t)i;
    std::vector<Candidate> &cands = w_cands_;
    cands.clear();
    cands.reserve((size_t)nsel);
    for(int64_t oi = 0; oi < nsel; oi++) {
      const int4 e = hsel[order[oi]];
      const int32_t n = e.w >> 2;
      const JobState &S = *jobs_[pn_[nodes[n]].job];
      if(S.cancelled) continue;
      Candidate cd;
      cd.node = n;
      cd.key = e.x - hn[n].key_base;
      cd.support = e.y;
      cd.cnt = e.z;
      cd.verdict = wo_.min_check == 0 ? (e.w & 3) : 2;
      cd.ok = cd.verdict == 1;
      if(cd.key < 0 || cd.key >= hn[n].nkeys) throw Error(ST_ERR_STATE, "selected key outside its node");
      // the kernels emit keys of valid extensions only: one that does not
      // decode is an inconsistency, not a pattern to skip
      if(!decode_key(lays[n], *S.job.db, cd.key, cd.dfs))
        throw Error(ST_ERR_STATE, "selected key does not decode to an extension");
      // a frequent pattern beyond what the embedding store and the checkers
      // take (64 vertices, 127 edges) is refused, never dropped: its
      // canonical form is frequent too, so the output would need it
      if(cd.cnt < 0 || cd.cnt == INT32_MAX)
        throw Error(ST_ERR_LIMIT, "a pattern has 2^31 or more embeddings in one wave");
      const size_t pe = pn_[nodes[n]].code.size() + 1;
      if(pe >= (size_t)kMaxPatternEdges || (cd.dfs.is_forward() && cd.dfs.to + 1 > kMaxPatternVertices))
        throw Error(ST_ERR_LIMIT, "frequent pattern exceeds 64 vertices or 127 edges; cap max_edges");
      cands.push_back(cd);
    }
    st_.candidates += (int64_t)cands.size();
    // canonicality: the GPU's verdicts; the rest on the host, in parallel
    {
      const clk::time_point t0 = clk::now();
      std::vector<int32_t> &todo = w_todo_;
      todo.clear();
      for(int32_t i = 0; i < (int32_t)cands.size(); i++)
        if(cands[i].verdict != 0 && cands[i].verdict != 1) todo.push_back(i);
      st_.min_host += (int64_t)todo.size();
      E.workers->run((int64_t)todo.size(), [&](int64_t ti, int w) {
        Candidate &cd = cands[todo[ti]];
        const auto &code = pn_[nodes[cd.node]].code;
        DFS buf[kMaxPatternEdges + 1];
        const size_t n = code.size();
        if(n + 1 > (size_t)kMaxPatternEdges) { cd.ok = false; return; }
        std::copy(code.begin(), code.end(), buf);
        buf[n] = cd.dfs;
        cd.ok = E.checkers[w].is_min(buf, (int)n + 1);
      });
      st_.host_min_ms += ms_since(t0);
    }

    // accepted children: output tree, materialisation slots
    std::vector<ChildOut> &outs = w_outs_;
    std::vector<int2> &pairs = w_pairs_;
    outs.clear();
    pairs.clear();
    // children in node order (a node's children are contiguous, from made_at[n])
    std::vector<int32_t> &made = w_made_;
    std::vector<int32_t> &made_at = w_made_at_;
    made.clear();
    made_at.assign((size_t)W + 1, 0);
    // lists strategy: every node with a forward child to materialise keeps
    // per-row lists of its frequent forward extensions (built from this
    // wave's records) for those children's joins
    int32_t list_blk = -1;
    int32_t *list_off = nullptr, *list_scr = nullptr;
    int2 *list_ent = nullptr;
    int64_t list_rows = 0, list_n = 0;
    std::vector<int32_t> list_rb;  // per node: its first list row, or -1
    {
      // accepted candidates; cands is grouped by node, so each node's are contiguous
      std::vector<int32_t> &acc = w_acc_;
      acc.clear();
      acc.reserve(cands.size());
      for(int32_t i = 0; i < (int32_t)cands.size(); i++)
        if(cands[i].ok) acc.push_back(i);
      // pass 1: output tree (reference order) and which children to materialise
      std::vector<Mat> &mats = w_mats_;
      mats.clear();
      mats.reserve(acc.size());
      size_t bytes = 0;
      for(size_t a0 = 0; a0 < acc.size();) {
        const int32_t n = cands[acc[a0]].node;
        size_t a1 = a0;
        while(a1 < acc.size() && cands[acc[a1]].node == n) a1++;
        std::sort(acc.begin() + a0, acc.begin() + a1,
                  [&](int32_t a, int32_t b) { return seq_before(cands[a].dfs, cands[b].dfs); });
        PNode &p = pn_[nodes[n]];
        JobState &S = *jobs_[p.job];
        const int32_t max_edges = S.job.opt.max_edges;
        for(size_t ai = a0; ai < a1; ai++) {
          const int32_t ci = acc[ai];
          const Candidate &cd = cands[ci];
          S.pats.push_back(PatternRec{ p.pattern, cd.dfs, cd.support });
          const int32_t pid = (int32_t)S.pats.size() - 1;
          PatternRec &par = S.pats[p.pattern];
          if(par.last_child < 0) par.first_child = pid;
          else S.pats[par.last_child].next_sibling = pid;
          par.last_child = pid;
          const int32_t child_edges = (int32_t)p.code.size() + 1;
          if(max_edges > 0 && child_edges >= max_edges) continue;
          if(child_edges >= kMaxPatternEdges || (cd.dfs.is_forward() && cd.dfs.to + 1 > 64))
            throw Error(ST_ERR_LIMIT, "pattern exceeds 64 vertices or 127 edges");
          mats.push_back(Mat{ n, ci, pid });
          bytes += Carver::round((size_t)cd.cnt * 8) + Carver::round((size_t)cd.cnt * 4);
        }
        a0 = a1;
      }
      if(f.lists && f.rec && nrec >= 0 && nrec <= f.rec_cap) {
        list_rb.assign(W, -1);
        std::vector<char> need(W, 0);
        for(const Mat &m : mats)
          if(cands[m.cand].dfs.is_forward()) need[m.node] = 1;
        for(int32_t n = 0; n < W; n++)
          if(need[n]) {
            list_rb[n] = (int32_t)list_rows;
            list_rows += pn_[nodes[n]].nrows;
          }
        for(const Candidate &cd : cands)
          if(need[cd.node] && cd.key < lays[cd.node].nfwd) list_n += cd.cnt;
        if(list_rows > 0 && list_rows + 1 < INT32_MAX && list_n < INT32_MAX) {
          const size_t lb = Carver::round(sizeof(int32_t) * (size_t)(list_rows + 1)) +
                            Carver::round(sizeof(int2) * (size_t)std::max<int64_t>(list_n, 1)) +
                            Carver::round(sizeof(int32_t) * (size_t)list_scan_scratch(list_rows));
          list_blk = E.new_block(lb);
          Carver lc{ (char *)E.blocks[list_blk].base };
          list_off = lc.take<int32_t>((size_t)(list_rows + 1));
          list_ent = lc.take<int2>((size_t)std::max<int64_t>(list_n, 1));
          list_scr = lc.take<int32_t>((size_t)list_scan_scratch(list_rows));
        } else {
          list_rb.clear();
        }
      }
      // pass 2: every child's new column and graph ranks carved from one block
      if(!mats.empty()) {
        const int32_t blk = E.new_block(bytes);
        Carver cv{ (char *)E.blocks[blk].base };
        made.reserve(mats.size());
        outs.reserve(mats.size());
        pairs.reserve(mats.size());
        for(const Mat &m : mats) {
          made_at[m.node + 1]++;
          const Candidate &cd = cands[m.cand];
          PNode &p = pn_[nodes[m.node]];
          JobState &S = *jobs_[p.job];
          const int64_t rowsn = cd.cnt;
          int2 *col = cv.take<int2>(rowsn);
          int32_t *gord = cv.take<int32_t>(rowsn);
          ChildOut o{ col, nullptr, gord, cd.dfs.is_forward() ? 0 : 1, (int32_t)rowsn };
          pairs.push_back(make_int2(hn[m.node].key_base + cd.key, (int32_t)outs.size()));
          outs.push_back(o);
          const int32_t nid = pn_new();
          PNode &nn = pn_[nid];
          nn.job = p.job;
          nn.pattern = m.pid;
          nn.code.reserve(p.code.size() + 1);
          nn.code.assign(p.code.data(), p.code.size());
          nn.code.push_back(cd.dfs);
          // forward children append a column, backward children replace the last
          const size_t keep = cd.dfs.is_forward() ? p.cols.size() : p.cols.size() - 1;
          nn.cols.reserve(keep + 1);
          nn.cols.assign(p.cols.data(), keep);
          nn.cols.push_back(ColRef{ col, rowsn });
          nn.last_col = E.new_col(col, rowsn, blk, cd.dfs.is_forward() ? p.last_col : E.cols[p.last_col].parent);
          nn.gord = gord;
          nn.gord_blk = blk;
          E.block_ref(blk);
          nn.nrows = rowsn;
          nn.support = cd.support;
          if(list_blk >= 0 && cd.dfs.is_forward() && list_rb[m.node] >= 0) {
            nn.list_blk = list_blk;
            E.block_ref(list_blk);
            nn.list_off = list_off + list_rb[m.node];
            nn.list_ent = list_ent;
            nn.list_rows = p.nrows;
            // the child's right-most path up to the new edge's source u is
            // the parent's, with the same forward keys: the parent's keys
            // from u's slot and the slots before it stay keys of the child
            // (from u only those at or after the new edge's pair)
            // (gspan_cuda_lists.cpp:327-369 possible_extension, 372-443 the
            // forward-forward joins)
            const NodeLayout &Lp = lays[m.node];
            for(const SlotDesc &sd : Lp.slots) {
              const int32_t hi = sd.fkey_off + S.job.db->pair_cnt[sd.vlab];
              if(cd.key >= sd.fkey_off && cd.key < hi) {
                nn.join_lo = sd.fkey_off;
                nn.join_key = cd.key;
                nn.join_hi = hi;
              }
            }
          }
          S.live_bytes += rowsn * (int64_t)(sizeof(int2) + sizeof(int32_t));
          S.peak_bytes = std::max(S.peak_bytes, S.live_bytes);
          made.push_back(nid);
        }
      }
      for(int32_t n = 0; n < W; n++) made_at[n + 1] += made_at[n];
    }
    if(!outs.empty()) {
      // one upload: children's outputs, then the (key, child) pairs
      const size_t outs_bytes = Carver::round(sizeof(ChildOut) * outs.size());
      const size_t pairs_bytes = Carver::round(sizeof(int2) * pairs.size());
      const size_t mat_bytes = outs_bytes + pairs_bytes + (list_blk >= 0 ? sizeof(int32_t) * (size_t)W : 0);
      X.d_mat.ensure(mat_bytes);
      X.h_mat.ensure(mat_bytes);
      std::memcpy(X.h_mat.p, outs.data(), sizeof(ChildOut) * outs.size());
      std::memcpy(X.h_mat.p + outs_bytes, pairs.data(), sizeof(int2) * pairs.size());
      if(list_blk >= 0) std::memcpy(X.h_mat.p + outs_bytes + pairs_bytes, list_rb.data(), sizeof(int32_t) * W);
      h2d(X.d_mat.p, X.h_mat.p, mat_bytes, st);
      const ChildOut *douts = (const ChildOut *)X.d_mat.p;
      X.d_cursor.ensure(outs.size());
      CK(cudaEventRecord(X.ev[4], st));
      launch_scatter_childmap((const int2 *)(X.d_mat.p + outs_bytes), (int32_t)pairs.size(), X.d_childmap.p,
                              X.d_cursor.p, (int32_t)outs.size(), st);
      // lists strategy: the records pass also counts the list rows
      ListBuild lb{ X.d_lnode.p, f.dn, (const int32_t *)(X.d_mat.p + outs_bytes + pairs_bytes) };
      if(list_blk >= 0) CK(cudaMemsetAsync(list_off, 0, sizeof(int32_t) * (size_t)(list_rows + 1), st));
      if(f.rec && nrec <= f.rec_cap) {
        // record-driven: one thread per extension record, no graph access
        launch_materialize_records(f.rec, nrec, X.d_childmap.p, X.d_keyword.p, f.bm, X.d_bmx.p, f.cnt, f.cstride,
                                   douts, E.d_bytes.p + 1, err_flag(), list_blk >= 0 ? &lb : nullptr,
                                   list_off + 1, st);
      } else {
        // records overflowed (or are disabled): enumerate again
        launch_wave_materialize(f.dn, W, f.tb, f.kmax, f.small, f.dc, f.dl, f.ds, f.dv, E.d_dbs.p, f.bm, X.d_bmx.p,
                                X.d_childmap.p, X.d_cursor.p, douts, E.d_bytes.p + 1, err_flag(), f.join,
                                f.rule_skip, st);
        if(f.rec) X.wanted_rec = std::max<long long>(X.wanted_rec, nrec + nrec / 4);
      }
      if(list_blk >= 0) {
        launch_fill_lists(f.rec, nrec, lb, list_off, list_rows, list_ent, list_n, list_scr, err_flag(), st);
        st_.list_entries += list_n;
        st_.launches += 2;
      }
      CK(cudaEventRecord(X.ev[5], st));
      X.mat_gen++;
      st_.launches += 2;
      f.mat_pending = true;
    }
    // the parents are done: drop their column references and graph ranks
    // (stream order keeps the materialise kernel ahead of any reuse)
    std::vector<int32_t> &touched = w_touched_;
    touched.clear();
    for(int32_t n = W - 1; n >= 0; n--) {
      JobState &S = *jobs_[pn_[nodes[n]].job];
      for(int32_t i = made_at[n + 1] - 1; i >= made_at[n]; i--) S.stack.push_back(made[i]);
      S.pending += made_at[n + 1] - made_at[n];
      stacked_ += made_at[n + 1] - made_at[n];
    }
    for(int32_t id : nodes) {
      PNode &p = pn_[id];
      JobState &S = *jobs_[p.job];
      drop_node(S, p);
      if(touched.empty() || touched.back() != p.job) touched.push_back(p.job);
      pn_free(id);
    }
    nodes.clear();
    f.busy = false;
    st_.host_select_ms += ms_since(t_ready) - (st_.host_min_ms - min_before);
    std::sort(touched.begin(), touched.end());
    touched.erase(std::unique(touched.begin(), touched.end()), touched.end());
    for(int32_t id : touched)
      if(!jobs_[id]->done && jobs_[id]->pending == 0) complete(id);
  }

  // pre-order traversal of a job's pattern tree, codes in the caller's labels
  // the patterns of roots r0..r1-1 (all by default), each root's subtree in pre-order
  void emit(JobState &S, size_t r0 = 0, size_t r1 = SIZE_MAX)
  {
    const MineJob &j = S.job;
    if(!j.emit) return;
    r1 = std::min(r1, S.roots.size());
    const LabelMap &lm = j.db->labels;
    std::vector<DFS> path, styled, orig;
    std::vector<int32_t> flat;
    struct Frame { int32_t pat; int32_t next; };
    std::vector<Frame> st;
    auto out = [&](int32_t pid) {
      const size_t n = path.size();
      styled.resize(n);
      orig.resize(n);
      for(size_t i = 0; i < n; i++) {
        orig[i] = path[i];
        orig[i].fromlabel = lm.vlabel_of[path[i].fromlabel];
        orig[i].tolabel = lm.vlabel_of[path[i].tolabel];
        orig[i].elabel = lm.elabel_of[path[i].elabel];
      }
      to_style(orig.data(), (int)n, (LabelStyle)j.opt.label_style, styled.data());
      flat.resize(n * 5);
      for(size_t i = 0; i < n; i++) {
        flat[i * 5 + 0] = styled[i].from;
        flat[i * 5 + 1] = styled[i].to;
        flat[i * 5 + 2] = styled[i].fromlabel;
        flat[i * 5 + 3] = styled[i].elabel;
        flat[i * 5 + 4] = styled[i].tolabel;
      }
      j.emit(flat.data(), (int32_t)n, S.pats[pid].support, j.user);
    };
    for(size_t ri = r0; ri < r1; ri++) {
      const int32_t r = S.roots[ri];
      path.assign(1, S.pats[r].edge);
      out(r);
      st.assign(1, Frame{ r, S.pats[r].first_child });
      while(!st.empty()) {
        Frame &fr = st.back();
        if(fr.next >= 0) {
          const int32_t cc = fr.next;
          fr.next = S.pats[cc].next_sibling;
          path.push_back(S.pats[cc].edge);
          out(cc);
          st.push_back(Frame{ cc, S.pats[cc].first_child });
        } else {
          st.pop_back();
          path.pop_back();
        }
      }
    }
  }
};

// failure cleanup: finish queued work, drop pooled memory
void engine_fail(Engine &e)
{
  if(e.ready) {
    e.sync_all();
    cudaGetLastError();
    e.destroy();
  }
}

}  // namespace

namespace {

void add_stats(MineStats &a, const MineStats &b)
{
  a.patterns += b.patterns; a.waves += b.waves; a.launches += b.launches; a.nodes += b.nodes; a.rows += b.rows;
  a.extensions += b.extensions; a.candidates += b.candidates; a.count_bytes += b.count_bytes;
  a.mat_bytes += b.mat_bytes; a.count_ms += b.count_ms; a.mat_ms += b.mat_ms; a.support_ms += b.support_ms;
  a.root_ms += b.root_ms; a.host_min_ms += b.host_min_ms; a.peak_pool_bytes += b.peak_pool_bytes;
  a.h2d_bytes += b.h2d_bytes; a.d2h_bytes += b.d2h_bytes; a.host_build_ms += b.host_build_ms;
  a.host_wait_ms += b.host_wait_ms; a.host_select_ms += b.host_select_ms; a.host_emit_ms += b.host_emit_ms;
  a.min_host += b.min_host; a.list_entries += b.list_entries; a.join_nodes += b.join_nodes;
  a.sel_bytes += b.sel_bytes; a.sel_ms += b.sel_ms; a.min_ms += b.min_ms;
}

// A batch split over P schedulers, each with its own engine (pool, wave
// contexts, streams) on its own host thread: the host's per-node work, which
// bounds a batch of many small databases, runs on P cores while the GPU runs
// the P schedulers' waves side by side.  Jobs go to the scheduler with the
// fewest graphs so far (largest first); each scheduler mines its jobs as one
// batch.  Patterns are emitted afterwards on the calling thread, job by job
// in batch order.
int run_jobs_split(std::vector<MineJob> &batch, const MineOptions &wave_opt, MineStats &st, std::string &err,
                   int P)
{
  const clk::time_point t0 = clk::now();
  // the schedulers' jobs: a batch's jobs as they are, or one job split into P
  // parts by root subtrees (part p mines the roots whose index in the
  // reference's order is its own residue, within the job's own partition)
  std::vector<MineJob> jobs;
  if(batch.size() == 1) {
    const MineJob &j0 = batch[0];
    const int32_t RP = j0.opt.root_parts > 1 ? j0.opt.root_parts : 1, rp = RP > 1 ? j0.opt.root_part : 0;
    for(int p = 0; p < P; p++) {
      MineJob j = j0;
      j.opt.root_parts = RP * P;
      j.opt.root_part = rp + RP * p;
      jobs.push_back(j);
    }
  } else {
    jobs = batch;
  }
  // databases resident before the threads start (a database may appear twice)
  for(auto &j : jobs)
    if(!j.db->resident) {
      j.db->upload();
      st.h2d_bytes += (int64_t)j.db->d_bytes;
    }
  std::vector<int32_t> order(jobs.size());
  for(size_t i = 0; i < jobs.size(); i++) order[i] = (int32_t)i;
  std::stable_sort(order.begin(), order.end(), [&](int32_t a, int32_t b) {
    return jobs[a].db->host.n_graphs > jobs[b].db->host.n_graphs;
  });
  std::vector<std::vector<int32_t>> part(P);
  std::vector<int64_t> load(P, 0);
  if(batch.size() == 1) {
    for(int p = 0; p < P; p++) part[p].push_back(p);
  } else {
    for(int32_t i : order) {
      const int p = (int)(std::min_element(load.begin(), load.end()) - load.begin());
      part[p].push_back(i);
      load[p] += jobs[i].db->host.n_graphs;
    }
  }
  for(auto &v : part) std::sort(v.begin(), v.end());
  std::vector<MineStats> pst(P);
  std::vector<std::unique_ptr<Sched>> sch(P);
  std::vector<std::vector<int32_t>> ids(P);
  std::vector<int> prc(P, ST_OK);
  std::vector<std::string> perr(P);
  auto engine = [](int p) -> Engine & { return p == 0 ? g_engine : g_extra[p - 1]; };
  auto work = [&](int p) {
    try {
      CK(cudaSetDevice(0));
      Engine &E = engine(p);
      E.pool_limit = g_pool_limit;
      E.init(wave_opt.threads);
      sch[p].reset(new Sched(E, wave_opt, pst[p]));
      sch[p]->set_defer_emit(true);
      std::vector<MineJob> js;
      for(int32_t i : part[p]) js.push_back(jobs[i]);
      ids[p] = sch[p]->add_all_ids(js);
      while(!sch[p]->idle()) sch[p]->step();
      sch[p]->sync_stats();
    } catch(const Error &e) {
      prc[p] = e.code;
      perr[p] = e.what();
    } catch(const std::exception &e) {
      prc[p] = ST_ERR_STATE;
      perr[p] = e.what();
    }
  };
  std::vector<std::thread> th;
  std::vector<int> inline_parts;  // parts whose thread could not be started run here
  for(int p = 1; p < P; p++)
    if(!part[p].empty()) {
      try {
        th.emplace_back(work, p);
      } catch(const std::system_error &) {
        inline_parts.push_back(p);
      }
    }
  if(!part[0].empty()) work(0);
  for(int p : inline_parts) work(p);
  for(auto &t : th) t.join();
  for(int p = 0; p < P; p++)
    if(prc[p] != ST_OK) {
      err = perr[p];
      const int rc = prc[p];
      for(int q = 0; q < P; q++) {
        sch[q].reset();
        if(prc[q] != ST_OK) engine_fail(engine(q));
      }
      return rc;
    }
  // patterns in batch order, on this thread
  std::vector<std::pair<int, int32_t>> where(jobs.size());
  for(int p = 0; p < P; p++)
    for(size_t k = 0; k < part[p].size(); k++) where[part[p][k]] = { p, ids[p][k] };
  if(batch.size() == 1) {
    // one job's parts: root subtrees merged in root-key order
    std::vector<size_t> cur(jobs.size(), 0);
    for(;;) {
      int best = -1;
      int32_t bk = 0;
      for(size_t q = 0; q < jobs.size(); q++) {
        const auto &rk = sch[where[q].first]->root_keys(where[q].second);
        if(cur[q] < rk.size() && (best < 0 || rk[cur[q]] < bk)) {
          best = (int)q;
          bk = rk[cur[q]];
        }
      }
      if(best < 0) break;
      sch[where[best].first]->emit_root(where[best].second, cur[best]++);
    }
    for(size_t q = 0; q < jobs.size(); q++) sch[where[q].first]->release_patterns(where[q].second);
  } else {
    for(size_t i = 0; i < jobs.size(); i++) sch[where[i].first]->emit_deferred(where[i].second);
  }
  for(int p = 0; p < P; p++) {
    add_stats(st, pst[p]);
    sch[p].reset();
  }
  st.wall_ms += ms_since(t0);
  return ST_OK;
}

}  // namespace

int run_jobs(std::vector<MineJob> &jobs, const MineOptions &wave_opt, MineStats *stats, std::string &err)
{
  std::lock_guard<std::mutex> g(g_mu);
  MineStats local;
  MineStats &st = stats ? *stats : local;
  try {
    for(auto &j : jobs) {
      if(!j.db) throw Error(ST_ERR_USAGE, "null database");
      if(j.minsup < 1) throw Error(ST_ERR_MINSUP_TOO_SMALL, "error: absolute_min_support < 1");
      if(j.minsup >= j.db->host.n_graphs)
        throw Error(ST_ERR_MINSUP_TOO_LARGE, "error: user specified support " + std::to_string(j.minsup) +
                                                 " is greater then the database size " +
                                                 std::to_string(j.db->host.n_graphs));
    }
    // a batch: one scheduler per 8 jobs from 16 on; one job: split by root
    // subtrees only when asked
    int P = wave_opt.schedulers > 0 ? wave_opt.schedulers : (jobs.size() >= 16 ? (int)(jobs.size() / 8) : 1);
    P = std::max(1, std::min<int>({ P, kMaxSchedulers, jobs.size() == 1 ? kMaxSchedulers : (int)jobs.size() }));
    if(P > 1) return run_jobs_split(jobs, wave_opt, st, err, P);
    const clk::time_point t0 = clk::now();
    g_engine.pool_limit = g_pool_limit;
    g_engine.init(wave_opt.threads);
    Sched s(g_engine, wave_opt, st);
    s.add_all(jobs);
    while(!s.idle()) s.step();
    s.sync_stats();
    st.wall_ms += ms_since(t0);
  } catch(const Error &e) {
    err = e.what();
    engine_fail(g_engine);
    return e.code;
  } catch(const std::exception &e) {
    err = e.what();
    engine_fail(g_engine);
    return ST_ERR_STATE;
  }
  return ST_OK;
}

// ------------------------------------------------------------ public scheduler

struct Scheduler::Impl {
  Engine eng;
  MineOptions wo;
  MineStats st;
  std::unique_ptr<Sched> s;
};

Scheduler::Scheduler(const MineOptions &wave_opt, int64_t pool_bytes) : p_(new Impl())
{
  p_->wo = wave_opt;
  p_->eng.pool_limit = pool_bytes;
  reset();
}

Scheduler::~Scheduler()
{
  if(!p_) return;
  p_->s.reset();
  p_->eng.destroy();
}

void Scheduler::reset()
{
  p_->s.reset();
  engine_fail(p_->eng);
  p_->eng.init(p_->wo.threads);
  p_->s.reset(new Sched(p_->eng, p_->wo, p_->st));
}

int32_t Scheduler::add(const MineJob &job) { return p_->s->add(job); }
bool Scheduler::idle() const { return p_->s->idle(); }
void Scheduler::step() { p_->s->step(); }
void Scheduler::cancel(int32_t id) { p_->s->cancel(id); }
std::vector<int32_t> Scheduler::take_done() { return p_->s->take_done(); }
void Scheduler::forget(int32_t id) { p_->s->forget(id); }
void Scheduler::sync_stats() { p_->s->sync_stats(); }
MineStats &Scheduler::stats() { return p_->st; }
int64_t Scheduler::pool_used() const { return p_->s->pool_used(); }

bool Scheduler::job_info(int32_t id, JobInfo &out)
{
  JobState *S = p_->s->job(id);
  if(!S) return false;
  out.live_bytes = S->live_bytes;
  out.peak_bytes = S->peak_bytes;
  out.patterns = S->patterns;
  out.pending = S->pending;
  out.done = S->done;
  out.cancelled = S->cancelled;
  return true;
}

int autotune_jobs(std::vector<MineJob> &jobs, const MineOptions &base, MineOptions &best,
                  std::vector<TuneTrial> &trials, std::string &err)
{
  // trials count patterns without emitting them
  std::vector<MineJob> quiet = jobs;
  for(auto &j : quiet) {
    j.emit = nullptr;
    j.user = nullptr;
  }
  auto trial = [&](const MineOptions &o, double &ms) -> int {
    double b = 1e300;
    for(int r = 0; r < 2; r++) {
      MineStats st;
      std::string e;
      const int rc = run_jobs(quiet, o, &st, e);
      if(rc) {
        err = e;
        return rc;
      }
      b = std::min(b, st.wall_ms);
    }
    ms = b;
    trials.push_back(TuneTrial{ o.wave_nodes, o.wave_rows, o.count_grid, o.deep_nodes, o.schedulers, ms });
    return ST_OK;
  };
  MineOptions cur = base;
  double cur_ms = 0;
  int rc = trial(cur, cur_ms);
  if(rc) return rc;
  // a value replaces the current one only when it is at least 2% faster
  auto consider = [&](MineOptions o) -> int {
    double ms = 0;
    const int r = trial(o, ms);
    if(r) return r;
    if(ms < 0.98 * cur_ms) {
      cur = o;
      cur_ms = ms;
    }
    return ST_OK;
  };
  for(int32_t wn : { 1024, 2048, 4096, 8192, 16384 }) {
    if(wn == cur.wave_nodes) continue;
    MineOptions o = cur;
    o.wave_nodes = wn;
    if((rc = consider(o))) return rc;
  }
  for(int64_t wr : { (int64_t)1 << 22, (int64_t)1 << 23, (int64_t)1 << 24, (int64_t)1 << 25 }) {
    if(wr == cur.wave_rows) continue;
    MineOptions o = cur;
    o.wave_rows = wr;
    if((rc = consider(o))) return rc;
  }
  for(int32_t cg : { 16, 32, 64, 96 }) {
    if(cg == cur.count_grid || (cur.count_grid == 0 && cg == 64)) continue;
    MineOptions o = cur;
    o.count_grid = cg;
    if((rc = consider(o))) return rc;
  }
  for(int32_t dn : { 1, 256, 1024 }) {
    if(dn == cur.deep_nodes) continue;
    MineOptions o = cur;
    o.deep_nodes = dn;
    if((rc = consider(o))) return rc;
  }
  // a batch: the number of schedulers it is split over
  if(jobs.size() >= 2)
    for(int32_t sc : { 1, 2, 3, 4 }) {
      if(sc == cur.schedulers || sc > (int32_t)jobs.size()) continue;
      MineOptions o = cur;
      o.schedulers = sc;
      if((rc = consider(o))) return rc;
    }
  best = cur;
  return ST_OK;
}

int support_count_host(const int32_t *keys, const int32_t *gids, int64_t n, int32_t n_keys, int32_t n_graphs,
                       int32_t *support, std::string &err)
{
  if(n < 0 || n_keys < 0 || n_graphs < 0 || (n > 0 && (!keys || !gids)) || (n_keys > 0 && !support)) {
    err = "invalid arguments";
    return ST_ERR_USAGE;
  }
  for(int64_t i = 0; i < n; i++)
    if(keys[i] < 0 || keys[i] >= n_keys || gids[i] < 0 || gids[i] >= n_graphs) {
      err = "record " + std::to_string(i) + " has a key or graph id out of range";
      return ST_ERR_USAGE;
    }
  if(n_keys == 0) return ST_OK;
  const int32_t words = std::max(1, (n_graphs + 31) / 32);
  const size_t nw = (size_t)n_keys * words;
  std::lock_guard<std::mutex> g(g_mu);
  char *blk = nullptr;
  cudaStream_t s = nullptr;
  int rc = ST_OK;
  try {
    auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
    const size_t o_k = 0, o_g = o_k + al(4 * (size_t)std::max<int64_t>(n, 1));
    const size_t o_bm = o_g + al(4 * (size_t)std::max<int64_t>(n, 1));
    const size_t o_bmx = o_bm + al(4 * nw), o_sup = o_bmx + al(4 * nw);
    const size_t o_nd = o_sup + al(4 * (size_t)n_keys), total = o_nd + al(sizeof(NodeDesc));
    CK(cudaSetDevice(0));
    CK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    CK(cudaMalloc(&blk, total));
    NodeDesc nd{};
    nd.words = words;
    nd.nkeys = n_keys;
    if(n > 0) {
      CK(cudaMemcpyAsync(blk + o_k, keys, 4 * (size_t)n, cudaMemcpyHostToDevice, s));
      CK(cudaMemcpyAsync(blk + o_g, gids, 4 * (size_t)n, cudaMemcpyHostToDevice, s));
    }
    CK(cudaMemcpyAsync(blk + o_nd, &nd, sizeof(nd), cudaMemcpyHostToDevice, s));
    CK(cudaMemsetAsync(blk + o_bm, 0, 4 * nw, s));
    launch_records_bitmap((const int32_t *)(blk + o_k), (const int32_t *)(blk + o_g), n, words,
                          (uint32_t *)(blk + o_bm), s);
    launch_support((const NodeDesc *)(blk + o_nd), 1, n_keys, (const uint32_t *)(blk + o_bm),
                   (int32_t *)(blk + o_bmx), (int32_t *)(blk + o_sup), s);
    CK(cudaMemcpyAsync(support, blk + o_sup, 4 * (size_t)n_keys, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    CK(cudaGetLastError());
  } catch(const Error &e) {
    err = e.what();
    rc = e.code;
  }
  if(s) cudaStreamSynchronize(s);
  if(blk) cudaFree(blk);
  if(s) cudaStreamDestroy(s);
  return rc;
}

int filter_backward_host(const int32_t *column, int64_t n_rows, const int32_t *records, int64_t n_records,
                         const int32_t *dfs, int32_t *out, int64_t *n_out, std::string &err)
{
  if(n_rows < 0 || n_records < 0 || !dfs || !n_out || (n_rows > 0 && (!column || !out)) ||
     (n_records > 0 && !records)) {
    err = "invalid arguments";
    return ST_ERR_USAGE;
  }
  // the reference aborts on a forward edge (DFS::is_forward: from < to)
  if(dfs[0] <= dfs[1]) {
    err = "the edge to filter by is not backward (from > to)";
    return ST_ERR_USAGE;
  }
  if(n_rows >= (int64_t)INT32_MAX) {
    err = "more than 2^31 - 2 rows";
    return ST_ERR_LIMIT;
  }
  for(int64_t i = 0; i < n_records; i++) {
    const int32_t *x = records + 8 * i;
    if(x[0] == dfs[0] && x[1] == dfs[1] && x[2] == dfs[2] && x[3] == dfs[3] && x[4] == dfs[4] &&
       (x[7] < 0 || x[7] >= n_rows)) {
      err = "record " + std::to_string(i) + " names a row outside the column";
      return ST_ERR_USAGE;
    }
  }
  *n_out = 0;
  if(n_rows == 0) return ST_OK;
  std::lock_guard<std::mutex> g(g_mu);
  char *blk = nullptr;
  cudaStream_t s = nullptr;
  int rc = ST_OK;
  try {
    auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
    const size_t o_col = 0, o_rec = o_col + al(8 * (size_t)n_rows);
    const size_t o_pos = o_rec + al(32 * (size_t)std::max<int64_t>(n_records, 1));
    const size_t o_scr = o_pos + al(4 * (size_t)(n_rows + 1));
    const size_t o_out = o_scr + al(4 * (size_t)std::max<int64_t>(filter_backward_scratch(n_rows), 1));
    const size_t total = o_out + al(8 * (size_t)n_rows);
    CK(cudaSetDevice(0));
    CK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    CK(cudaMalloc(&blk, total));
    CK(cudaMemcpyAsync(blk + o_col, column, 8 * (size_t)n_rows, cudaMemcpyHostToDevice, s));
    if(n_records > 0) CK(cudaMemcpyAsync(blk + o_rec, records, 32 * (size_t)n_records, cudaMemcpyHostToDevice, s));
    int32_t *pos = (int32_t *)(blk + o_pos);
    CK(cudaMemsetAsync(pos, 0, 4 * (size_t)(n_rows + 1), s));
    launch_filter_backward((const int2 *)(blk + o_col), n_rows, (const int32_t *)(blk + o_rec), n_records, dfs, pos,
                           (int32_t *)(blk + o_scr), (int2 *)(blk + o_out), s);
    int32_t cnt = 0;
    CK(cudaMemcpyAsync(&cnt, pos + n_rows, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if(cnt > 0) CK(cudaMemcpyAsync(out, blk + o_out, 8 * (size_t)cnt, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    CK(cudaGetLastError());
    *n_out = cnt;
  } catch(const Error &e) {
    err = e.what();
    rc = e.code;
  }
  if(s) cudaStreamSynchronize(s);
  if(blk) cudaFree(blk);
  if(s) cudaStreamDestroy(s);
  return rc;
}

// The reference's segmented scan / reduce over packed uint32 arrays
// (cuda_segmented_scan::scan, cuda_segmented_reduction::reduce,
// src/reduction/cuda_segmented_scan.hpp, cuda_segmented_reduction.cpp:
// 98-134): one device pass each, host arrays in and out.
int segmented_scan_host(const uint32_t *data, int64_t n, const int64_t *ends, int64_t n_ends, int exclusive,
                        uint32_t *out, std::string &err)
{
  if(n < 0 || n_ends < 0 || (n > 0 && !data) || (n_ends > 0 && (!ends || !out)) || (n_ends == 0 && n > 0 && !out)) {
    err = "invalid arguments";
    return ST_ERR_USAGE;
  }
  if(n >= (int64_t)INT32_MAX) {
    err = "more than 2^31 - 2 elements";
    return ST_ERR_LIMIT;
  }
  for(int64_t j = 0; j < n_ends; j++)
    if(ends[j] < 0 || ends[j] >= n) {
      err = "segment end " + std::to_string(j) + " is outside the array";
      return ST_ERR_USAGE;
    }
  if(n == 0) return ST_OK;
  std::lock_guard<std::mutex> g(g_mu);
  char *blk = nullptr;
  cudaStream_t s = nullptr;
  int rc = ST_OK;
  try {
    auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
    const size_t o_x = 0, o_scr = o_x + al(4 * (size_t)n);
    const size_t o_ends = o_scr + al(4 * (size_t)segmented_scan_scratch(n));
    const size_t o_res = o_ends + al(8 * (size_t)std::max<int64_t>(n_ends, 1));
    const size_t o_err = o_res + al(4 * (size_t)std::max<int64_t>(n_ends, 1)), total = o_err + al(4);
    CK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    CK(cudaMalloc(&blk, total));
    uint32_t *x = (uint32_t *)(blk + o_x);
    unsigned int *derr = (unsigned int *)(blk + o_err);
    CK(cudaMemcpyAsync(x, data, 4 * (size_t)n, cudaMemcpyHostToDevice, s));
    CK(cudaMemsetAsync(derr, 0, 4, s));
    launch_segmented_scan(x, n, exclusive, (int32_t *)(blk + o_scr), x, s);
    unsigned int herr = 0;
    if(n_ends > 0) {
      CK(cudaMemcpyAsync(blk + o_ends, ends, 8 * (size_t)n_ends, cudaMemcpyHostToDevice, s));
      launch_gather_ends(x, n, (const long long *)(blk + o_ends), n_ends, (uint32_t *)(blk + o_res), derr, s);
      CK(cudaMemcpyAsync(out, blk + o_res, 4 * (size_t)n_ends, cudaMemcpyDeviceToHost, s));
    } else {
      CK(cudaMemcpyAsync(out, x, 4 * (size_t)n, cudaMemcpyDeviceToHost, s));
    }
    CK(cudaMemcpyAsync(&herr, derr, 4, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    CK(cudaGetLastError());
    if(herr) throw Error(ST_ERR_STATE, "segment end outside the array on the device");
  } catch(const Error &e) {
    err = e.what();
    rc = e.code;
  }
  if(s) cudaStreamSynchronize(s);
  if(blk) cudaFree(blk);
  if(s) cudaStreamDestroy(s);
  return rc;
}

void engine_reset()
{
  {
    std::lock_guard<std::mutex> g(g_mu);
    g_engine.destroy();
    for(auto &e : g_extra) e.destroy();
  }
  ingest_release();
}

void engine_set_pool_bytes(int64_t bytes)
{
  std::lock_guard<std::mutex> g(g_mu);
  g_pool_limit = bytes;
}

}  // namespace gsgb
