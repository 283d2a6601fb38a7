/*
 * gspan_oracle.c -- CPU restatement of the reference's sequential gSpan.
 *
 * TEST INFRASTRUCTURE ONLY.  This program is the checker for the GPU miner:
 * only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg (and
 * the `--impl reference` arm) may run it.  The product never links or calls
 * it, and there is no CPU fallback path in the product.
 *
 * Parity: pinned.  Its output is compared line-for-line (same order) against
 * the reference's own src/gspan built from its sources (oracle/Makefile `ref`
 * target, harness oracle/ref_harness.cpp) on the reference's testdata and on
 * seeded synthetic databases; the resulting golden files live in tests/golden/.
 *
 * Algorithm (Yan & Han gSpan, Taku Kudo's implementation as shipped in the
 * reference), restated in C with sorted extension arrays in place of the
 * reference's std::map trees:
 *   run_intern          src/gspan/gspan.cpp:281-351   root edges (fl<=tl), map order
 *   project             src/gspan/gspan.cpp:172-274   support, is_min, report, extend
 *   support             src/gspan/gspan.cpp:89-103    count of id changes
 *   is_min              src/gspan/ismin.cpp:36-143    greedy minimum-code rebuild
 *   get_forward_root    src/globals/graph_types.cpp:365-375
 *   get_forward_pure    src/globals/graph_types.cpp:337-357
 *   get_forward_rmpath  src/globals/graph_types.cpp:305-322
 *   get_backward        src/globals/graph_types.cpp:389-413
 *   History::build      src/globals/graph_types.cpp:258-276
 *   DFSCode::buildRMPath src/globals/dfs_code.cpp:75-90
 *   DFSCode::to_string(false) src/globals/dfs_code.cpp:199-216 (output format)
 *   Graph::read (txt)   src/globals/graph_types.cpp:66-113
 *   Graph::read_fsg     src/globals/graph_types.cpp:115-170 (per-graph label renumbering)
 *   read_database_cudabin src/globals/dbio.cpp:381-404 + convert_to_host_representation
 *                       src/globals/cuda_graph_types.cpp:268-293
 *
 *   generate            the seeded benchmark databases (configurations 1-5),
 *                       the same bytes as the GPU miner's generator writes
 *
 * Usage: gspan_oracle <txt|fsg|bin|cudabin> <file> <abs-minsup> [out|-] [--max-edges N]
 *        [--graph-limit G] [--time-limit SECONDS] [--roots i/n] [--repeat K] [--roots-once]
 *        [--intervals K S]
 *        gspan_oracle gen <config[,seed[,scale]]> <abs-minsup> [same options]
 *        gspan_oracle --write-gen <config[,seed[,scale]]> <out.txt>
 *        gspan_oracle --gen-count <config[,seed[,scale]]>
 * --time-limit stops the traversal after that many seconds (a bounded sample
 * for timing; the output is then a prefix of the full output).  --roots i/n
 * mines only the frequent root edges whose index is i modulo n (independent
 * subtrees; the union over i = 0..n-1 is the full output).  --repeat K mines
 * K times over one load (timing samples); --roots-once builds the root map
 * (one pass over every graph and a sort of its edges) before them, untimed.
 * --intervals K S mines for K consecutive windows of S seconds (the
 * traversal restarting whenever it completes) and reports the cumulative
 * pattern count at the end of each window: a throughput sample of the whole
 * traversal, not of its first seconds only.  `gen` mines a generated database
 * without a file; --write-gen writes one as txt; --gen-count prints its
 * graph count.
 * Output: one line per frequent pattern, "<code>\t<support>", in the
 * reference's traversal order; codes use the reference's sequential-miner
 * convention (fromlabel -1 after the first edge, tolabel -1 on backward edges).
 * Exit codes follow src/gspan/main.cpp:56-66: 2 when minsup >= |DB|, 3 when
 * minsup < 1.  "total_time=<s> total_frequent_graphs=<n>" goes to stderr.
 */
#define _POSIX_C_SOURCE 200809L
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <stdint.h>
#include <time.h>
#include <math.h>

/* ------------------------------------------------------------------ graphs */

typedef struct {
  int from, to, elabel, id;
} oedge;

typedef struct {
  int nv, ne;       /* vertices, undirected edges (distinct ids) */
  int *vlabel;      /* [nv] */
  int *off;         /* [nv+1] adjacency offsets */
  oedge *adj;       /* [off[nv]] directed adjacency, input order per vertex */
} ograph;

typedef struct {
  ograph *g;
  int n, cap;
} odb;

static void *xmalloc(size_t n)
{
  void *p = malloc(n ? n : 1);
  if(!p) { fprintf(stderr, "oracle: out of memory\n"); exit(9); }
  return p;
}

static void *xrealloc(void *p, size_t n)
{
  p = realloc(p, n ? n : 1);
  if(!p) { fprintf(stderr, "oracle: out of memory\n"); exit(9); }
  return p;
}

/* Builder for one graph: vertices with labels, then edge list; adjacency is
 * laid out per vertex in insertion order like Vertex::push
 * (src/globals/graph_types.hpp:38-44). */
typedef struct {
  int nv, vcap;
  int *vlabel;
  int ne, ecap;
  int *ef, *et, *el;
} gbuild;

static void gb_reset(gbuild *b) { b->nv = 0; b->ne = 0; }

static void gb_vertex(gbuild *b, int id, int label)
{
  if(id + 1 > b->vcap) {
    int nc = b->vcap ? b->vcap : 16;
    while(nc < id + 1) nc *= 2;
    b->vlabel = xrealloc(b->vlabel, sizeof(int) * nc);
    b->vcap = nc;
  }
  /* Graph::read resizes to id+1 (graph_types.cpp:93); new slots get label 0
   * from Vertex's default member, but every input in practice defines them. */
  for(int i = b->nv; i < id + 1; i++) b->vlabel[i] = 0;
  if(id + 1 > b->nv) b->nv = id + 1;
  b->vlabel[id] = label;
}

static void gb_edge(gbuild *b, int f, int t, int l)
{
  if(b->ne == b->ecap) {
    int nc = b->ecap ? b->ecap * 2 : 32;
    b->ef = xrealloc(b->ef, sizeof(int) * nc);
    b->et = xrealloc(b->et, sizeof(int) * nc);
    b->el = xrealloc(b->el, sizeof(int) * nc);
    b->ecap = nc;
  }
  b->ef[b->ne] = f; b->et[b->ne] = t; b->el[b->ne] = l; b->ne++;
}

/* Edge ids follow Graph::buildEdge (graph_types.cpp:35-60): one id per
 * distinct (min(from,to), max(from,to), elabel), numbered by first
 * appearance while walking vertices in order and each vertex's adjacency in
 * order.  The first appearance of an undirected edge {a,c} is at vertex
 * min(a,c); a later copy reuses that id. */
static void assign_edge_ids(ograph *g)
{
  int next = 0;
  for(int v = 0; v < g->nv; v++) {
    for(int k = g->off[v]; k < g->off[v + 1]; k++) {
      oedge *e = &g->adj[k];
      int found = -1;
      if(e->to < v) {
        for(int j = g->off[e->to]; j < g->off[e->to + 1]; j++)
          if(g->adj[j].to == v && g->adj[j].elabel == e->elabel) { found = g->adj[j].id; break; }
      } else {
        for(int j = g->off[v]; j < k; j++)
          if(g->adj[j].to == e->to && g->adj[j].elabel == e->elabel) { found = g->adj[j].id; break; }
      }
      e->id = found >= 0 ? found : next++;
    }
  }
  g->ne = next;
}

/* Adjacency lists are laid out per vertex in insertion order (Vertex::push), each
 * undirected input edge pushed in both directions (Graph::read). */
static void gb_finish(gbuild *b, ograph *g)
{
  g->nv = b->nv;
  g->vlabel = xmalloc(sizeof(int) * b->nv);
  memcpy(g->vlabel, b->vlabel, sizeof(int) * b->nv);
  g->off = xmalloc(sizeof(int) * (b->nv + 1));
  int *deg = calloc(b->nv + 1, sizeof(int));
  for(int i = 0; i < b->ne; i++) { deg[b->ef[i]]++; deg[b->et[i]]++; }
  g->off[0] = 0;
  for(int v = 0; v < b->nv; v++) g->off[v + 1] = g->off[v] + deg[v];
  g->adj = xmalloc(sizeof(oedge) * (g->off[b->nv] + 1));
  for(int v = 0; v < b->nv; v++) deg[v] = g->off[v];
  for(int i = 0; i < b->ne; i++) {
    oedge a = { b->ef[i], b->et[i], b->el[i], -1 };
    g->adj[deg[b->ef[i]]++] = a;
    oedge r = { b->et[i], b->ef[i], b->el[i], -1 };
    g->adj[deg[b->et[i]]++] = r;
  }
  free(deg);
  assign_edge_ids(g);
}

static void db_push(odb *db, gbuild *b)
{
  if(db->n == db->cap) {
    db->cap = db->cap ? db->cap * 2 : 64;
    db->g = xrealloc(db->g, sizeof(ograph) * db->cap);
  }
  gb_finish(b, &db->g[db->n++]);
}

/* split a line into whitespace separated tokens (utils::split) */
static int tokenize(char *line, char **tok, int maxtok)
{
  int n = 0;
  char *p = line;
  while(*p && n < maxtok) {
    while(*p == ' ' || *p == '\t' || *p == '\r' || *p == '\n') p++;
    if(!*p) break;
    tok[n++] = p;
    while(*p && *p != ' ' && *p != '\t' && *p != '\r' && *p != '\n') p++;
    if(*p) *p++ = 0;
  }
  return n;
}

/* simple string -> dense id table for the fsg reader (per graph) */
typedef struct { char **keys; int n, cap; } strtab;

static int strtab_get(strtab *t, const char *s)
{
  for(int i = 0; i < t->n; i++) if(strcmp(t->keys[i], s) == 0) return i;
  if(t->n == t->cap) {
    t->cap = t->cap ? 2 * t->cap : 16;
    t->keys = xrealloc(t->keys, sizeof(char*) * t->cap);
  }
  t->keys[t->n] = xmalloc(strlen(s) + 1);
  strcpy(t->keys[t->n], s);
  return t->n++;
}

static void strtab_clear(strtab *t)
{
  for(int i = 0; i < t->n; i++) free(t->keys[i]);
  t->n = 0;
}

static int read_text_db(const char *path, int fsg, odb *db, int graph_limit)
{
  FILE *f = fopen(path, "r");
  if(!f) return -1;
  char line[1024];
  char *tok[8];
  gbuild b;
  memset(&b, 0, sizeof(b));
  strtab vt = {0}, et = {0};
  int open = 0;
  const char *etag = fsg ? "u" : "e";
  while(fgets(line, sizeof(line), f)) {
    int n = tokenize(line, tok, 8);
    if(n == 0) continue;
    if(strcmp(tok[0], "t") == 0) {
      /* Graph::read ends a graph at the next "t" only if it is non-empty */
      if(open && b.nv > 0) {
        db_push(db, &b);
        if(graph_limit > 0 && db->n >= graph_limit) { open = 0; break; }
      }
      gb_reset(&b);
      strtab_clear(&vt); strtab_clear(&et);
      open = 1;
    } else if(strcmp(tok[0], "v") == 0 && n >= 3) {
      int id = atoi(tok[1]);
      int lab = fsg ? strtab_get(&vt, tok[2]) : atoi(tok[2]);
      gb_vertex(&b, id, lab);
      open = 1;
    } else if(strcmp(tok[0], etag) == 0 && n >= 4) {
      int fr = atoi(tok[1]), to = atoi(tok[2]);
      int lab = fsg ? strtab_get(&et, tok[3]) : atoi(tok[3]);
      if(fr >= b.nv || to >= b.nv) {
        fprintf(stderr, "Format Error:  define vertex lists before edges\n");
        fclose(f);
        return -2;
      }
      gb_edge(&b, fr, to, lab);
    }
  }
  if(open && b.nv > 0) db_push(db, &b);
  fclose(f);
  strtab_clear(&vt); strtab_clear(&et);
  free(vt.keys); free(et.keys);
  free(b.vlabel); free(b.ef); free(b.et); free(b.el);
  return 0;
}

/* cudabin: int32 header {db_size, edges_sizes, max_graph_vertex_count,
 * vertex_count}, then edges[edges_sizes], edges_labels[edges_sizes],
 * vertex_labels[db*maxv], vertex_offsets[db*maxv+1]; padding slots carry -1
 * (src/globals/dbio.cpp:359-368, cuda_graph_types.cpp:65-127). */
static int read_cudabin_db(const char *path, odb *db, int graph_limit)
{
  FILE *f = fopen(path, "rb");
  if(!f) return -1;
  int32_t hdr[4];
  if(fread(hdr, sizeof(int32_t), 4, f) != 4) { fclose(f); return -2; }
  int64_t dbsz = hdr[0], esz = hdr[1], maxv = hdr[2];
  int64_t slots = dbsz * maxv;
  int32_t *edges = xmalloc(sizeof(int32_t) * esz);
  int32_t *elab = xmalloc(sizeof(int32_t) * esz);
  int32_t *vlab = xmalloc(sizeof(int32_t) * slots);
  int32_t *voff = xmalloc(sizeof(int32_t) * (slots + 1));
  int ok = fread(edges, sizeof(int32_t), esz, f) == (size_t)esz
           && fread(elab, sizeof(int32_t), esz, f) == (size_t)esz
           && fread(vlab, sizeof(int32_t), slots, f) == (size_t)slots
           && fread(voff, sizeof(int32_t), slots + 1, f) == (size_t)(slots + 1);
  fclose(f);
  if(!ok) return -2;
  for(int64_t gi = 0; gi < dbsz; gi++) {
    if(graph_limit > 0 && db->n >= graph_limit) break;
    int64_t base = gi * maxv;
    int nv = 0;
    while(nv < maxv && voff[base + nv] != -1) nv++;
    /* convert_to_host_representation pushes each directed entry into its
     * vertex's list in file order; the end of vertex v's neighbourhood is the
     * offset of the next valid slot (get_next_valid_vertex_idx), which after
     * the last vertex of a graph is the next graph's first slot or the
     * trailing sentinel. */
    ograph g;
    g.nv = nv;
    g.vlabel = xmalloc(sizeof(int) * (nv ? nv : 1));
    g.off = xmalloc(sizeof(int) * (nv + 1));
    int64_t total = 0;
    for(int v = 0; v < nv; v++) {
      int64_t nxt = (v + 1 < nv) ? base + v + 1 : (gi + 1) * maxv;
      total += voff[nxt] - voff[base + v];
    }
    g.adj = xmalloc(sizeof(oedge) * (total + 1));
    int pos = 0;
    for(int v = 0; v < nv; v++) {
      g.vlabel[v] = vlab[base + v];
      g.off[v] = pos;
      int64_t nxt = (v + 1 < nv) ? base + v + 1 : (gi + 1) * maxv;
      for(int64_t k = voff[base + v]; k < voff[nxt]; k++) {
        oedge e = { v, (int)(edges[k] - base), elab[k], -1 };
        g.adj[pos++] = e;
      }
    }
    g.off[nv] = pos;
    assign_edge_ids(&g);
    if(db->n == db->cap) {
      db->cap = db->cap ? db->cap * 2 : 64;
      db->g = xrealloc(db->g, sizeof(ograph) * db->cap);
    }
    db->g[db->n++] = g;
  }
  free(edges); free(elab); free(vlab); free(voff);
  return 0;
}

/* BIN: size_t count, size_t offset per graph, then per graph a size_t byte
 * count and Graph::serialize's layout: int size, int edge_size, bool
 * directed, int nv, per vertex {int size, int label, int nedges, nedges x
 * {from, to, elabel, id}} (src/globals/dbio.cpp:132-191,
 * src/globals/graph_types.cpp:560-608).  Edge ids are taken from the file. */
static int read_bin_db(const char *path, odb *db, int graph_limit)
{
  FILE *f = fopen(path, "rb");
  if(!f) return -1;
  uint64_t ng = 0;
  if(fread(&ng, 8, 1, f) != 1) { fclose(f); return -2; }
  if(fseek(f, (long)(8 * (ng + 1)), SEEK_SET) != 0) { fclose(f); return -2; }
  for(uint64_t gi = 0; gi < ng; gi++) {
    if(graph_limit > 0 && db->n >= graph_limit) break;
    uint64_t gsz = 0;
    int32_t tot, esz, nv;
    unsigned char directed;
    if(fread(&gsz, 8, 1, f) != 1 || fread(&tot, 4, 1, f) != 1 || fread(&esz, 4, 1, f) != 1 ||
       fread(&directed, 1, 1, f) != 1 || fread(&nv, 4, 1, f) != 1 || nv < 0) { fclose(f); return -2; }
    ograph g;
    g.nv = nv;
    g.ne = esz;
    g.vlabel = xmalloc(sizeof(int) * (nv ? nv : 1));
    g.off = xmalloc(sizeof(int) * (nv + 1));
    int cap = 64, pos = 0;
    g.adj = xmalloc(sizeof(oedge) * cap);
    for(int v = 0; v < nv; v++) {
      int32_t vs, lab, ne;
      if(fread(&vs, 4, 1, f) != 1 || fread(&lab, 4, 1, f) != 1 || fread(&ne, 4, 1, f) != 1 || ne < 0) { fclose(f); return -2; }
      g.vlabel[v] = lab;
      g.off[v] = pos;
      for(int k = 0; k < ne; k++) {
        int32_t e4[4];
        if(fread(e4, 4, 4, f) != 4) { fclose(f); return -2; }
        if(pos == cap) { cap *= 2; g.adj = xrealloc(g.adj, sizeof(oedge) * cap); }
        oedge e = { e4[0], e4[1], e4[2], e4[3] };
        g.adj[pos++] = e;
        if(e4[3] + 1 > g.ne) g.ne = e4[3] + 1;
      }
    }
    g.off[nv] = pos;
    if(db->n == db->cap) {
      db->cap = db->cap ? db->cap * 2 : 64;
      db->g = xrealloc(db->g, sizeof(ograph) * db->cap);
    }
    db->g[db->n++] = g;
  }
  fclose(f);
  return 0;
}

/* ------------------------------------------------------- seeded generator */

/* The seeded synthetic databases of the benchmark configurations 1-5, made
 * here so that the timed CPU arm and the full-size pins read no file written
 * by the GPU miner's library.  The stream is xoshiro256** seeded through
 * splitmix64 (Blackman & Vigna), which gives the same values on every
 * platform; labels come from cumulative weight tables, Poisson draws from
 * Knuth's product of uniforms.  A graph is built in the order the txt writer
 * lists it ("v" lines by vertex, then every edge once, from its lower
 * endpoint, in the order the endpoint's adjacency holds it), so the graphs
 * equal what read_text_db makes of the same database written as txt.  A CPU
 * test checks that the txt this program writes hashes to the committed
 * checksums and to the GPU miner's generator output. */

typedef struct { uint64_t s[4]; } orng;

static uint64_t splitmix64(uint64_t *x)
{
  uint64_t z = (*x += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

static void rng_seed(orng *r, uint64_t seed)
{
  for(int i = 0; i < 4; i++) r->s[i] = splitmix64(&seed);
}

static uint64_t rotl64(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

static uint64_t rng_next(orng *r)
{
  uint64_t *s = r->s;
  uint64_t out = rotl64(s[1] * 5, 7) * 9;
  uint64_t t = s[1] << 17;
  s[2] ^= s[0]; s[3] ^= s[1]; s[1] ^= s[2]; s[0] ^= s[3];
  s[2] ^= t; s[3] = rotl64(s[3], 45);
  return out;
}

/* 53 random bits in [0, 1) */
static double rng_uniform(orng *r) { return (double)(rng_next(r) >> 11) * (1.0 / 9007199254740992.0); }

/* inclusive range */
static int64_t rng_range(orng *r, int64_t lo, int64_t hi)
{
  return lo + (int64_t)(rng_next(r) % (uint64_t)(hi - lo + 1));
}

static int rng_poisson(orng *r, double mean)
{
  double lim = exp(-mean), p = 1.0;
  int k = 0;
  do { k++; p *= rng_uniform(r); } while(p > lim);
  return k - 1;
}

typedef struct { double cdf[128]; int n; } ocat;

static void cat_set(ocat *c, const double *w, int n)
{
  double s = 0;
  c->n = n;
  for(int i = 0; i < n; i++) { s += w[i]; c->cdf[i] = s; }
  for(int i = 0; i < n; i++) c->cdf[i] /= s;
}

/* first index whose cumulative weight is >= u, clamped to the last */
static int cat_draw(const ocat *c, orng *r)
{
  double u = rng_uniform(r);
  int lo = 0, hi = c->n;
  while(lo < hi) {
    int mid = (lo + hi) / 2;
    if(c->cdf[mid] < u) lo = mid + 1; else hi = mid;
  }
  return lo < c->n ? lo : c->n - 1;
}

typedef struct {
  int64_t n_graphs;
  int mode;               /* 0: spanning tree + ring edges; 1: embedded seed patterns */
  int vmin, vmax;         /* mode 0 vertex count range */
  double ring_per_vertex;
  double mean_edges;      /* mode 1: edge budget ~ Poisson(mean) */
  int n_vlabels;
  double vzipf;           /* 0 = uniform */
  int n_elabels;
  double eweights[8];
  int n_eweights;
  int n_seeds;
  double seed_mean_edges;
  int seed_min_edges, seed_max_edges;  /* max 0 = unbounded */
  double seed_cover;
  uint64_t seed;
} ogen;

/* a small graph under construction: edges in creation order, per-vertex
 * neighbour lists for the adjacency test */
typedef struct {
  int nv, vcap, ne, ecap;
  int *vl, *ef, *et, *el;
  int **nb, *nbn, *nbcap;
} sgraph;

static void sg_clear(sgraph *s) { s->nv = 0; s->ne = 0; }

static int sg_vertex(sgraph *s, int label)
{
  if(s->nv == s->vcap) {
    int nc = s->vcap ? 2 * s->vcap : 32;
    s->vl = xrealloc(s->vl, sizeof(int) * nc);
    s->nb = xrealloc(s->nb, sizeof(int *) * nc);
    s->nbn = xrealloc(s->nbn, sizeof(int) * nc);
    s->nbcap = xrealloc(s->nbcap, sizeof(int) * nc);
    for(int i = s->vcap; i < nc; i++) { s->nb[i] = 0; s->nbcap[i] = 0; }
    s->vcap = nc;
  }
  s->vl[s->nv] = label;
  s->nbn[s->nv] = 0;
  return s->nv++;
}

static int sg_adjacent(const sgraph *s, int a, int b)
{
  for(int i = 0; i < s->nbn[a]; i++) if(s->nb[a][i] == b) return 1;
  return 0;
}

static void sg_nb_push(sgraph *s, int a, int b)
{
  if(s->nbn[a] == s->nbcap[a]) {
    s->nbcap[a] = s->nbcap[a] ? 2 * s->nbcap[a] : 8;
    s->nb[a] = xrealloc(s->nb[a], sizeof(int) * s->nbcap[a]);
  }
  s->nb[a][s->nbn[a]++] = b;
}

static void sg_edge(sgraph *s, int a, int b, int label)
{
  if(s->ne == s->ecap) {
    int nc = s->ecap ? 2 * s->ecap : 64;
    s->ef = xrealloc(s->ef, sizeof(int) * nc);
    s->et = xrealloc(s->et, sizeof(int) * nc);
    s->el = xrealloc(s->el, sizeof(int) * nc);
    s->ecap = nc;
  }
  s->ef[s->ne] = a; s->et[s->ne] = b; s->el[s->ne] = label; s->ne++;
  sg_nb_push(s, a, b);
  sg_nb_push(s, b, a);
}

/* a chord between two distinct non-adjacent vertices, 24 tries at most */
static int sg_chord(sgraph *s, orng *r, int label)
{
  int n = s->nv;
  if(n < 3) return 0;
  for(int tries = 0; tries < 24; tries++) {
    int a = (int)rng_range(r, 0, n - 1), b = (int)rng_range(r, 0, n - 1);
    if(a == b || sg_adjacent(s, a, b)) continue;
    sg_edge(s, a, b, label);
    return 1;
  }
  return 0;
}

static void sg_free(sgraph *s)
{
  for(int i = 0; i < s->vcap; i++) free(s->nb[i]);
  free(s->vl); free(s->ef); free(s->et); free(s->el); free(s->nb); free(s->nbn); free(s->nbcap);
}

/* Append a generated graph in txt order: vertices, then for every vertex v in
 * order its incident edges in creation order whose other end is above v.
 * With `txt` set, also write it as a "t/v/e" graph numbered `gid`. */
static void sg_emit(const sgraph *s, gbuild *b, odb *db, FILE *txt, int64_t gid)
{
  gb_reset(b);
  for(int v = 0; v < s->nv; v++) gb_vertex(b, v, s->vl[v]);
  if(txt) {
    fprintf(txt, "t # %lld\n", (long long)gid);
    for(int v = 0; v < s->nv; v++) fprintf(txt, "v %d %d\n", v, s->vl[v]);
  }
  /* incident edges of v in creation order: scan the edge list once per vertex
   * would be quadratic; bucket them instead */
  int *cnt = calloc((size_t)s->nv + 1, sizeof(int));
  for(int i = 0; i < s->ne; i++) { cnt[s->ef[i] + 1]++; cnt[s->et[i] + 1]++; }
  for(int v = 0; v < s->nv; v++) cnt[v + 1] += cnt[v];
  int *inc = xmalloc(sizeof(int) * (2 * (size_t)s->ne + 1));
  int *pos = xmalloc(sizeof(int) * ((size_t)s->nv + 1));
  memcpy(pos, cnt, sizeof(int) * (size_t)s->nv);
  for(int i = 0; i < s->ne; i++) { inc[pos[s->ef[i]]++] = i; inc[pos[s->et[i]]++] = i; }
  for(int v = 0; v < s->nv; v++)
    for(int k = cnt[v]; k < cnt[v + 1]; k++) {
      int i = inc[k];
      int to = s->ef[i] == v ? s->et[i] : s->ef[i];
      if(to > v) {
        gb_edge(b, v, to, s->el[i]);
        if(txt) fprintf(txt, "e %d %d %d\n", v, to, s->el[i]);
      }
    }
  free(cnt); free(inc); free(pos);
  if(db) db_push(db, b);
}

static void generate(const ogen *p, odb *db, FILE *txt)
{
  orng r;
  rng_seed(&r, p->seed);
  ocat vcat, ecat;
  {
    double w[128];
    for(int i = 0; i < p->n_vlabels; i++) w[i] = p->vzipf > 0 ? 1.0 / pow((double)(i + 1), p->vzipf) : 1.0;
    cat_set(&vcat, w, p->n_vlabels);
    double e[128];
    for(int i = 0; i < p->n_elabels; i++) e[i] = p->n_eweights == p->n_elabels ? p->eweights[i] : 1.0;
    cat_set(&ecat, e, p->n_elabels);
  }
  gbuild b;
  memset(&b, 0, sizeof(b));
  sgraph s;
  memset(&s, 0, sizeof(s));
  if(p->mode == 0) {
    for(int64_t g = 0; g < p->n_graphs; g++) {
      sg_clear(&s);
      int nv = (int)rng_range(&r, p->vmin, p->vmax);
      for(int v = 0; v < nv; v++) sg_vertex(&s, cat_draw(&vcat, &r));
      for(int v = 1; v < nv; v++) {
        /* the edge label is drawn before the parent vertex */
        int lab = cat_draw(&ecat, &r);
        int a = (int)rng_range(&r, 0, v - 1);
        sg_edge(&s, a, v, lab);
      }
      double x = nv * p->ring_per_vertex;
      int extra = (int)floor(x + rng_uniform(&r));
      for(int i = 0; i < extra; i++) { int lab = cat_draw(&ecat, &r); sg_chord(&s, &r, lab); }
      sg_emit(&s, &b, db, txt, g);
    }
  } else {
    sgraph *seeds = calloc((size_t)(p->n_seeds > 0 ? p->n_seeds : 1), sizeof(sgraph));
    for(int i = 0; i < p->n_seeds; i++) {
      int ne = rng_poisson(&r, p->seed_mean_edges);
      if(ne < p->seed_min_edges) ne = p->seed_min_edges;
      if(p->seed_max_edges > 0 && ne > p->seed_max_edges) ne = p->seed_max_edges;
      sgraph *sp = &seeds[i];
      sg_vertex(sp, cat_draw(&vcat, &r));
      for(int e = 0; e < ne; e++) {
        if(sp->nv >= 3 && rng_uniform(&r) < 0.25) {
          int lab = cat_draw(&ecat, &r);
          if(sg_chord(sp, &r, lab)) continue;
        }
        int a = (int)rng_range(&r, 0, sp->nv - 1);
        int bv = sg_vertex(sp, cat_draw(&vcat, &r));
        sg_edge(sp, a, bv, cat_draw(&ecat, &r));
      }
    }
    int *first = 0;
    int nfirst = 0, capfirst = 0;
    for(int64_t g = 0; g < p->n_graphs; g++) {
      int budget = rng_poisson(&r, p->mean_edges);
      if(budget < 1) budget = 1;
      sg_clear(&s);
      nfirst = 0;
      int covered = 0;
      while(p->n_seeds > 0 && covered < p->seed_cover * budget) {
        const sgraph *sp = &seeds[rng_range(&r, 0, p->n_seeds - 1)];
        int base = s.nv;
        if(nfirst == capfirst) { capfirst = capfirst ? 2 * capfirst : 64; first = xrealloc(first, sizeof(int) * capfirst); }
        first[nfirst++] = base;
        for(int v = 0; v < sp->nv; v++) sg_vertex(&s, sp->vl[v]);
        for(int e = 0; e < sp->ne; e++) sg_edge(&s, base + sp->ef[e], base + sp->et[e], sp->el[e]);
        covered += sp->ne;
      }
      if(s.nv == 0) {
        sg_vertex(&s, cat_draw(&vcat, &r));
        if(nfirst == capfirst) { capfirst = capfirst ? 2 * capfirst : 64; first = xrealloc(first, sizeof(int) * capfirst); }
        first[nfirst++] = 0;
      }
      int used = covered;
      /* link the copies into one connected graph */
      for(int c = 1; c < nfirst; c++) {
        int lo = first[c];
        int hi = c + 1 < nfirst ? first[c + 1] - 1 : s.nv - 1;
        int a = (int)rng_range(&r, lo, hi);
        int bv = (int)rng_range(&r, 0, lo - 1);
        sg_edge(&s, a, bv, cat_draw(&ecat, &r));
        used++;
      }
      /* the rest of the budget: new leaves and chords */
      while(used < budget) {
        int leaf = rng_uniform(&r) < 0.5;
        if(!leaf) { int lab = cat_draw(&ecat, &r); leaf = !sg_chord(&s, &r, lab); }
        if(leaf) {
          int a = (int)rng_range(&r, 0, s.nv - 1);
          int bv = sg_vertex(&s, cat_draw(&vcat, &r));
          sg_edge(&s, a, bv, cat_draw(&ecat, &r));
        }
        used++;
      }
      sg_emit(&s, &b, db, txt, g);
    }
    free(first);
    for(int i = 0; i < p->n_seeds; i++) sg_free(&seeds[i]);
    free(seeds);
  }
  sg_free(&s);
  free(b.vlabel); free(b.ef); free(b.et); free(b.el);
}

static int64_t scaled_count(int64_t n, double scale)
{
  int64_t v = llround((double)n * scale);
  return v > 1 ? v : 1;
}

/* The five benchmark configurations; seed 0 picks the configuration's
 * default seed.  Returns -1 for an unknown configuration. */
static int gen_config(int config, uint64_t seed, double scale, ogen *p)
{
  memset(p, 0, sizeof(*p));
  p->n_graphs = 340; p->vmin = 10; p->vmax = 60; p->ring_per_vertex = 0.05; p->mean_edges = 30.0;
  p->n_vlabels = 5; p->n_elabels = 5; p->n_seeds = 50; p->seed_mean_edges = 4.0; p->seed_min_edges = 1;
  p->seed_cover = 0.5; p->seed = 1;
  switch(config) {
  case 1:  /* stands in for testdata/Chemical_340 */
    p->mode = 0; p->n_graphs = scaled_count(340, scale); p->vmin = 10; p->vmax = 60; p->ring_per_vertex = 0.05;
    p->n_vlabels = 66; p->vzipf = 1.5; p->n_elabels = 4;
    p->eweights[0] = 0.6; p->eweights[1] = 0.3; p->eweights[2] = 0.08; p->eweights[3] = 0.02; p->n_eweights = 4;
    p->seed = seed ? seed : 1;
    return 0;
  case 2:  /* stands in for the PAFI T100000E5PL4P50TL30V5 database */
    p->mode = 1; p->n_graphs = scaled_count(100000, scale); p->mean_edges = 30; p->n_vlabels = 5; p->n_elabels = 5;
    p->seed = seed ? seed : 2;
    return 0;
  case 3: {  /* one database of the 64-database batch: sizes and alphabets from its seed */
    orng r;
    rng_seed(&r, seed ? seed : 1000);
    double lg = log(1000.0) + rng_uniform(&r) * (log(50000.0) - log(1000.0));
    p->mode = 1; p->n_graphs = scaled_count(llround(exp(lg)), scale);
    p->n_vlabels = (int)rng_range(&r, 2, 20); p->n_elabels = (int)rng_range(&r, 2, 20);
    p->mean_edges = 10.0 + 30.0 * rng_uniform(&r);
    p->seed = seed ? seed : 1000;
    return 0;
  }
  case 4: {  /* one of the 8 resident serving databases */
    orng r;
    rng_seed(&r, seed ? seed : 2000);
    double lg = log(10000.0) + rng_uniform(&r) * (log(200000.0) - log(10000.0));
    p->mode = 1; p->n_graphs = scaled_count(llround(exp(lg)), scale);
    p->seed = seed ? seed : 2000;
    return 0;
  }
  case 5:  /* large single database */
    p->mode = 1; p->n_graphs = scaled_count(1000000, scale); p->mean_edges = 40; p->n_vlabels = 10; p->vzipf = 1.2;
    p->n_elabels = 3; p->n_seeds = 200; p->seed_mean_edges = 5.5; p->seed_min_edges = 3; p->seed_max_edges = 8;
    p->seed = seed ? seed : 5;
    return 0;
  default:
    return -1;
  }
}

/* ---------------------------------------------------------------- DFS code */

typedef struct { int from, to, fromlabel, elabel, tolabel; } odfs;

typedef struct {
  odfs *e;
  int n, cap;
} ocode;

static void code_push(ocode *c, int from, int to, int fl, int el, int tl)
{
  if(c->n == c->cap) {
    c->cap = c->cap ? 2 * c->cap : 16;
    c->e = xrealloc(c->e, sizeof(odfs) * c->cap);
  }
  odfs d = { from, to, fl, el, tl };
  c->e[c->n++] = d;
}

/* DFSCode::buildRMPath (dfs_code.cpp:75-90): indices into the code of the
 * forward edges on the right-most path, deepest first. */
static int build_rmpath(const ocode *c, int *rm)
{
  int n = 0, old_from = -1;
  for(int i = c->n - 1; i >= 0; --i) {
    if(c->e[i].from < c->e[i].to && (n == 0 || old_from == c->e[i].to)) {
      rm[n++] = i;
      old_from = c->e[i].from;
    }
  }
  return n;
}

/* ------------------------------------------------------------- embeddings */

/* PDFS (graph_types.hpp:147-155): graph id, graph edge, previous link */
typedef struct opdfs {
  int id;
  const oedge *edge;
  const struct opdfs *prev;
} opdfs;

/* History (graph_types.hpp:162-182) with epoch stamps instead of cleared
 * vectors: hasEdge/hasVertex are "stamp == current epoch". */
typedef struct {
  const oedge **edges;   /* history[i] = graph edge of code edge i */
  int n, cap;
  uint32_t *vstamp, *estamp;
  int vcap, ecap;
  uint32_t epoch;
} ohist;

static void hist_build(ohist *h, const ograph *g, const opdfs *p)
{
  if(g->nv > h->vcap) {
    h->vstamp = xrealloc(h->vstamp, sizeof(uint32_t) * g->nv);
    memset(h->vstamp, 0, sizeof(uint32_t) * g->nv);
    h->vcap = g->nv;
  }
  if(g->ne > h->ecap) {
    h->estamp = xrealloc(h->estamp, sizeof(uint32_t) * g->ne);
    memset(h->estamp, 0, sizeof(uint32_t) * g->ne);
    h->ecap = g->ne;
  }
  if(++h->epoch == 0) {
    memset(h->vstamp, 0, sizeof(uint32_t) * h->vcap);
    memset(h->estamp, 0, sizeof(uint32_t) * h->ecap);
    h->epoch = 1;
  }
  h->n = 0;
  for(const opdfs *q = p; q; q = q->prev) {
    if(h->n == h->cap) {
      h->cap = h->cap ? 2 * h->cap : 32;
      h->edges = xrealloc(h->edges, sizeof(*h->edges) * h->cap);
    }
    h->edges[h->n++] = q->edge;
    h->estamp[q->edge->id] = h->epoch;
    h->vstamp[q->edge->from] = h->epoch;
    h->vstamp[q->edge->to] = h->epoch;
  }
  for(int i = 0, j = h->n - 1; i < j; i++, j--) {
    const oedge *t = h->edges[i]; h->edges[i] = h->edges[j]; h->edges[j] = t;
  }
}

#define HAS_V(h, v) ((h)->vstamp[(v)] == (h)->epoch)
#define HAS_E(h, e) ((h)->estamp[(e)] == (h)->epoch)

/* get_backward (graph_types.cpp:389-413) */
static const oedge *get_backward(const ograph *g, const oedge *e1, const oedge *e2, const ohist *h)
{
  if(e1 == e2) return 0;
  for(int k = g->off[e2->to]; k < g->off[e2->to + 1]; k++) {
    const oedge *it = &g->adj[k];
    if(HAS_E(h, it->id)) continue;
    if(it->to == e1->from &&
       ((e1->elabel < it->elabel) ||
        (e1->elabel == it->elabel && g->vlabel[e1->to] <= g->vlabel[e2->to])))
      return it;
  }
  return 0;
}

/* Extension candidate gathered during one project() call.  kind 0 =
 * backward keyed (to, elabel); kind 1 = forward keyed (from, elabel,
 * tolabel).  seq keeps insertion order inside a key (std::map buckets are
 * appended to in embedding order). */
typedef struct {
  int kind, a, b, c;
  int seq;
  int id;
  const oedge *edge;
  const opdfs *prev;
} oext;

typedef struct { oext *x; int n, cap; } oextv;

static void ext_push(oextv *v, int kind, int a, int b, int c, int id, const oedge *e, const opdfs *prev)
{
  if(v->n == v->cap) {
    v->cap = v->cap ? 2 * v->cap : 256;
    v->x = xrealloc(v->x, sizeof(oext) * v->cap);
  }
  oext x = { kind, a, b, c, v->n, id, e, prev };
  v->x[v->n++] = x;
}

/* order of child processing in project(): backward buckets by (to asc,
 * elabel asc) first (gspan.cpp:250-257), then forward buckets by from
 * DEScending, elabel asc, tolabel asc (gspan.cpp:259-271). */
static int ext_cmp(const void *pa, const void *pb)
{
  const oext *x = pa, *y = pb;
  if(x->kind != y->kind) return x->kind - y->kind;
  if(x->kind == 0) {
    if(x->a != y->a) return x->a < y->a ? -1 : 1;
    if(x->b != y->b) return x->b < y->b ? -1 : 1;
  } else {
    if(x->a != y->a) return x->a > y->a ? -1 : 1;
    if(x->b != y->b) return x->b < y->b ? -1 : 1;
    if(x->c != y->c) return x->c < y->c ? -1 : 1;
  }
  return x->seq < y->seq ? -1 : (x->seq > y->seq);
}

/* ------------------------------------------------------------------ is_min */

/* The pattern graph built by DFSCode::toGraph (dfs_code.cpp:245-266). */
typedef struct {
  ograph g;
  gbuild b;
} opat;

static void pattern_graph(const ocode *c, gbuild *b, ograph *g)
{
  gb_reset(b);
  int nv = 0;
  for(int i = 0; i < c->n; i++) {
    int m = c->e[i].from > c->e[i].to ? c->e[i].from : c->e[i].to;
    if(m + 1 > nv) nv = m + 1;
  }
  /* toGraph overwrites labels as it goes; -1 leaves the previous value */
  int lab[1024];
  for(int v = 0; v < nv; v++) lab[v] = 0;
  for(int i = 0; i < c->n; i++) {
    if(c->e[i].fromlabel != -1) lab[c->e[i].from] = c->e[i].fromlabel;
    if(c->e[i].tolabel != -1) lab[c->e[i].to] = c->e[i].tolabel;
  }
  for(int v = 0; v < nv; v++) gb_vertex(b, v, lab[v]);
  for(int i = 0; i < c->n; i++) gb_edge(b, c->e[i].from, c->e[i].to, c->e[i].elabel);
  gb_finish(b, g);
}

static void free_graph(ograph *g)
{
  free(g->vlabel); free(g->off); free(g->adj);
}

typedef struct {
  ohist h;
  gbuild b;
  oextv ext;
} ismin_ws;

static int is_min_rec(const ocode *code, ocode *mc, const ograph *pg, opdfs *proj, int np, ismin_ws *ws, int depth);

/* gSpan::is_min (src/gspan/ismin.cpp:36-63) */
static int is_min(const ocode *code, ismin_ws *ws)
{
  if(code->n == 1) return 1;
  ograph pg;
  pattern_graph(code, &ws->b, &pg);
  /* root: minimum (fromlabel, elabel, tolabel) over get_forward_root edges */
  int best[3] = { 0, 0, 0 }, have = 0;
  for(int v = 0; v < pg.nv; v++)
    for(int k = pg.off[v]; k < pg.off[v + 1]; k++) {
      const oedge *e = &pg.adj[k];
      if(pg.vlabel[v] > pg.vlabel[e->to]) continue;
      int t[3] = { pg.vlabel[v], e->elabel, pg.vlabel[e->to] };
      if(!have || t[0] < best[0] || (t[0] == best[0] && (t[1] < best[1] || (t[1] == best[1] && t[2] < best[2])))) {
        best[0] = t[0]; best[1] = t[1]; best[2] = t[2]; have = 1;
      }
    }
  int np = 0;
  opdfs *proj = xmalloc(sizeof(opdfs) * (pg.off[pg.nv] + 1));
  for(int v = 0; v < pg.nv; v++)
    for(int k = pg.off[v]; k < pg.off[v + 1]; k++) {
      const oedge *e = &pg.adj[k];
      if(pg.vlabel[v] > pg.vlabel[e->to]) continue;
      if(pg.vlabel[v] == best[0] && e->elabel == best[1] && pg.vlabel[e->to] == best[2]) {
        opdfs p = { 0, e, 0 };
        proj[np++] = p;
      }
    }
  ocode mc = { 0, 0, 0 };
  code_push(&mc, 0, 1, best[0], best[1], best[2]);
  int r = is_min_rec(code, &mc, &pg, proj, np, ws, 0);
  free(proj);
  free(mc.e);
  free_graph(&pg);
  return r;
}

static int dfs_neq(const odfs *a, const odfs *b)
{
  return a->from != b->from || a->to != b->to || a->fromlabel != b->fromlabel ||
         a->elabel != b->elabel || a->tolabel != b->tolabel;
}

/* gSpan::project_is_min (src/gspan/ismin.cpp:65-141) */
static int is_min_rec(const ocode *code, ocode *mc, const ograph *pg, opdfs *proj, int np, ismin_ws *ws, int depth)
{
  int rm[1024];
  int nrm = build_rmpath(mc, rm);
  int minlabel = mc->e[0].fromlabel;
  int maxtoc = mc->e[rm[0]].to;
  ohist *h = &ws->h;

  /* SUBBLOCK 1: backward edges, first rmpath index that has any */
  {
    int flg = 0, newto = 0, bestel = 0, haveel = 0;
    for(int i = nrm - 1; !flg && i >= 1; --i) {
      for(int n = 0; n < np; n++) {
        hist_build(h, pg, &proj[n]);
        const oedge *e = get_backward(pg, h->edges[rm[i]], h->edges[rm[0]], h);
        if(e) {
          if(!haveel || e->elabel < bestel) { bestel = e->elabel; haveel = 1; }
          newto = mc->e[rm[i]].from;
          flg = 1;
        }
      }
    }
    if(flg) {
      /* children of the minimum elabel bucket, in embedding order */
      opdfs *child = xmalloc(sizeof(opdfs) * (np + 1));
      int nc = 0;
      for(int i = nrm - 1; i >= 1; --i) {
        int any = 0;
        for(int n = 0; n < np; n++) {
          hist_build(h, pg, &proj[n]);
          const oedge *e = get_backward(pg, h->edges[rm[i]], h->edges[rm[0]], h);
          if(e) {
            any = 1;
            if(e->elabel == bestel) { opdfs p = { 0, e, &proj[n] }; child[nc++] = p; }
          }
        }
        if(any) break;
      }
      code_push(mc, maxtoc, newto, -1, bestel, -1);
      int r;
      if(dfs_neq(&code->e[mc->n - 1], &mc->e[mc->n - 1])) r = 0;
      else r = is_min_rec(code, mc, pg, child, nc, ws, depth + 1);
      free(child);
      return r;
    }
  }

  /* SUBBLOCK 2: pure forward from the right-most vertex, else forward from
   * the right-most path, deepest first */
  {
    int flg = 0, newfrom = 0, which = -1;  /* which: -1 pure, else rmpath index */
    int bel = 0, btl = 0, have = 0;
    for(int n = 0; n < np; n++) {
      hist_build(h, pg, &proj[n]);
      const oedge *last = h->edges[rm[0]];
      for(int k = pg->off[last->to]; k < pg->off[last->to + 1]; k++) {
        const oedge *it = &pg->adj[k];
        if(minlabel > pg->vlabel[it->to] || HAS_V(h, it->to)) continue;
        int tl = pg->vlabel[it->to];
        if(!have || it->elabel < bel || (it->elabel == bel && tl < btl)) { bel = it->elabel; btl = tl; have = 1; }
        flg = 1;
        newfrom = maxtoc;
      }
    }
    for(int i = 0; !flg && i < nrm; ++i) {
      for(int n = 0; n < np; n++) {
        hist_build(h, pg, &proj[n]);
        const oedge *e = h->edges[rm[i]];
        int tolabel = pg->vlabel[e->to];
        for(int k = pg->off[e->from]; k < pg->off[e->from + 1]; k++) {
          const oedge *it = &pg->adj[k];
          int tolabel2 = pg->vlabel[it->to];
          if(e->to == it->to || minlabel > tolabel2 || HAS_V(h, it->to)) continue;
          if(e->elabel < it->elabel || (e->elabel == it->elabel && tolabel <= tolabel2)) {
            if(!have || it->elabel < bel || (it->elabel == bel && tolabel2 < btl)) { bel = it->elabel; btl = tolabel2; have = 1; }
            flg = 1;
            newfrom = mc->e[rm[i]].from;
            which = i;
          }
        }
      }
    }
    if(flg) {
      opdfs *child = xmalloc(sizeof(opdfs) * 64);
      int nc = 0, cap = 64;
      for(int n = 0; n < np; n++) {
        hist_build(h, pg, &proj[n]);
        if(which < 0) {
          const oedge *last = h->edges[rm[0]];
          for(int k = pg->off[last->to]; k < pg->off[last->to + 1]; k++) {
            const oedge *it = &pg->adj[k];
            if(minlabel > pg->vlabel[it->to] || HAS_V(h, it->to)) continue;
            if(it->elabel == bel && pg->vlabel[it->to] == btl) {
              if(nc == cap) { cap *= 2; child = xrealloc(child, sizeof(opdfs) * cap); }
              opdfs p = { 0, it, &proj[n] }; child[nc++] = p;
            }
          }
        } else {
          const oedge *e = h->edges[rm[which]];
          int tolabel = pg->vlabel[e->to];
          for(int k = pg->off[e->from]; k < pg->off[e->from + 1]; k++) {
            const oedge *it = &pg->adj[k];
            int tolabel2 = pg->vlabel[it->to];
            if(e->to == it->to || minlabel > tolabel2 || HAS_V(h, it->to)) continue;
            if(e->elabel < it->elabel || (e->elabel == it->elabel && tolabel <= tolabel2)) {
              if(it->elabel == bel && tolabel2 == btl) {
                if(nc == cap) { cap *= 2; child = xrealloc(child, sizeof(opdfs) * cap); }
                opdfs p = { 0, it, &proj[n] }; child[nc++] = p;
              }
            }
          }
        }
      }
      code_push(mc, newfrom, maxtoc + 1, -1, bel, btl);
      int r;
      if(dfs_neq(&code->e[mc->n - 1], &mc->e[mc->n - 1])) r = 0;
      else r = is_min_rec(code, mc, pg, child, nc, ws, depth + 1);
      free(child);
      return r;
    }
  }
  return 1;
}

/* ------------------------------------------------------------------- miner */

typedef struct {
  const odb *db;
  int minsup;
  double time_limit;   /* seconds, 0 = none */
  int root_part, root_parts;  /* process root subtree r only if r % root_parts == root_part */
  struct timespec t0;
  int stopped;
  int max_edges;       /* 0 = no cap */
  FILE *out;
  double count;
  ocode code;
  ohist h;
  ismin_ws ws;
  char *line;
  size_t line_cap;
  oextv roots;         /* the root edges of every graph in root-map order, built once */
  int have_roots;
  /* interval sampling: patterns reported up to the end of each of nint
   * consecutive windows of win seconds, counted over passes that restart
   * when a traversal completes */
  double win;
  int nint, icur;
  double done;         /* patterns of completed passes */
  double *icount;
} ominer;

/* support (gspan.cpp:89-103): number of id changes along the projection */
static int support(const opdfs *p, int n)
{
  int oid = -1, s = 0;
  for(int i = 0; i < n; i++) {
    if(oid != p[i].id) s++;
    oid = p[i].id;
  }
  return s;
}

static void report(ominer *m, int sup)
{
  m->count += 1;
  if(!m->out) return;
  /* DFSCode::to_string(false): "(f t fl el tl)" joined by ';' */
  for(int i = 0; i < m->code.n; i++) {
    const odfs *d = &m->code.e[i];
    fprintf(m->out, "%s(%d %d %d %d %d)", i ? ";" : "", d->from, d->to, d->fromlabel, d->elabel, d->tolabel);
  }
  fprintf(m->out, "\t%d\n", sup);
}

/* gSpan::project (gspan.cpp:172-274) */
static int out_of_time(ominer *m)
{
  if(m->time_limit <= 0) return 0;
  if(m->stopped) return 1;
  struct timespec t;
  clock_gettime(CLOCK_MONOTONIC, &t);
  double s = (t.tv_sec - m->t0.tv_sec) + 1e-9 * (t.tv_nsec - m->t0.tv_nsec);
  /* a window ends: the patterns so far (checked as each DFS-tree node starts) */
  while(m->icur < m->nint && s >= (m->icur + 1) * m->win) m->icount[m->icur++] = m->done + m->count;
  if(s > m->time_limit) m->stopped = 1;
  return m->stopped;
}

static void project(ominer *m, opdfs *proj, int np)
{
  if(out_of_time(m)) return;
  int sup = support(proj, np);
  if(sup < m->minsup) return;
  if(!is_min(&m->code, &m->ws)) return;
  report(m, sup);
  if(m->max_edges > 0 && m->code.n >= m->max_edges) return;

  int rm[1024];
  int nrm = build_rmpath(&m->code, rm);
  int minlabel = m->code.e[0].fromlabel;
  int maxtoc = m->code.e[rm[0]].to;

  oextv ext = { 0, 0, 0 };
  for(int n = 0; n < np; n++) {
    int id = proj[n].id;
    const ograph *g = &m->db->g[id];
    opdfs *cur = &proj[n];
    hist_build(&m->h, g, cur);
    const ohist *h = &m->h;
    /* backward */
    for(int i = nrm - 1; i >= 1; --i) {
      const oedge *e = get_backward(g, h->edges[rm[i]], h->edges[rm[0]], h);
      if(e) ext_push(&ext, 0, m->code.e[rm[i]].from, e->elabel, 0, id, e, cur);
    }
    /* pure forward */
    {
      const oedge *e = h->edges[rm[0]];
      for(int k = g->off[e->to]; k < g->off[e->to + 1]; k++) {
        const oedge *it = &g->adj[k];
        if(minlabel > g->vlabel[it->to] || HAS_V(h, it->to)) continue;
        ext_push(&ext, 1, maxtoc, it->elabel, g->vlabel[it->to], id, it, cur);
      }
    }
    /* backtracked forward */
    for(int i = 0; i < nrm; ++i) {
      const oedge *e = h->edges[rm[i]];
      int tolabel = g->vlabel[e->to];
      for(int k = g->off[e->from]; k < g->off[e->from + 1]; k++) {
        const oedge *it = &g->adj[k];
        int tolabel2 = g->vlabel[it->to];
        if(e->to == it->to || minlabel > tolabel2 || HAS_V(h, it->to)) continue;
        if(e->elabel < it->elabel || (e->elabel == it->elabel && tolabel <= tolabel2))
          ext_push(&ext, 1, m->code.e[rm[i]].from, it->elabel, tolabel2, id, it, cur);
      }
    }
  }
  qsort(ext.x, ext.n, sizeof(oext), ext_cmp);
  opdfs *child = xmalloc(sizeof(opdfs) * (ext.n + 1));
  for(int s = 0; s < ext.n;) {
    int e = s + 1;
    while(e < ext.n && ext.x[e].kind == ext.x[s].kind && ext.x[e].a == ext.x[s].a &&
          ext.x[e].b == ext.x[s].b && ext.x[e].c == ext.x[s].c) e++;
    for(int i = s; i < e; i++) {
      opdfs p = { ext.x[i].id, ext.x[i].edge, ext.x[i].prev };
      child[i - s] = p;
    }
    if(ext.x[s].kind == 0) code_push(&m->code, maxtoc, ext.x[s].a, -1, ext.x[s].b, -1);
    else code_push(&m->code, ext.x[s].a, maxtoc + 1, -1, ext.x[s].b, ext.x[s].c);
    project(m, child, e - s);
    m->code.n--;
    s = e;
  }
  free(child);
  free(ext.x);
}

/* gSpan::run_intern (gspan.cpp:281-351); single-vertex patterns are counted
 * but never reported by the reference (report_single is empty). */
/* the root map of run_intern (gspan.cpp:300-322): every directed edge whose
 * source label is at most its target label, grouped by (fl, el, tl) */
static void build_roots(ominer *m)
{
  const odb *db = m->db;
  oextv roots = { 0, 0, 0 };
  for(int id = 0; id < db->n; id++) {
    const ograph *g = &db->g[id];
    for(int v = 0; v < g->nv; v++)
      for(int k = g->off[v]; k < g->off[v + 1]; k++) {
        const oedge *e = &g->adj[k];
        if(g->vlabel[v] <= g->vlabel[e->to])
          ext_push(&roots, 1, g->vlabel[v], e->elabel, g->vlabel[e->to], id, e, 0);
      }
  }
  /* root map is ascending in all three keys */
  for(int i = 0; i < roots.n; i++) roots.x[i].a = -roots.x[i].a;  /* ext_cmp sorts 'a' descending */
  qsort(roots.x, roots.n, sizeof(oext), ext_cmp);
  for(int i = 0; i < roots.n; i++) roots.x[i].a = -roots.x[i].a;
  m->roots = roots;
  m->have_roots = 1;
}

static void run(ominer *m)
{
  if(!m->have_roots) build_roots(m);
  const oextv roots = m->roots;
  opdfs *proj = xmalloc(sizeof(opdfs) * (roots.n + 1));
  int root_index = 0;
  for(int s = 0; s < roots.n;) {
    int e = s + 1;
    while(e < roots.n && roots.x[e].a == roots.x[s].a && roots.x[e].b == roots.x[s].b && roots.x[e].c == roots.x[s].c) e++;
    if(m->root_parts > 1) {
      /* partition over frequent roots only, as the GPU miner does */
      int sup = 0, oid = -1;
      for(int i = s; i < e; i++) { if(roots.x[i].id != oid) sup++; oid = roots.x[i].id; }
      if(sup >= m->minsup && (root_index++ % m->root_parts) != m->root_part) { s = e; continue; }
    }
    for(int i = s; i < e; i++) {
      opdfs p = { roots.x[i].id, roots.x[i].edge, 0 };
      proj[i - s] = p;
    }
    m->code.n = 0;
    code_push(&m->code, 0, 1, roots.x[s].a, roots.x[s].b, roots.x[s].c);
    project(m, proj, e - s);
    s = e;
  }
  free(proj);
}

/* "config[,seed[,scale]]" -> generator parameters */
static int parse_gen(const char *spec, ogen *p)
{
  int config = 0;
  unsigned long long seed = 0;
  double scale = 1.0;
  char tail;
  int n = sscanf(spec, "%d,%llu,%lf%c", &config, &seed, &scale, &tail);
  if(n < 1 || n > 3 || scale <= 0) return -1;
  return gen_config(config, (uint64_t)seed, scale, p);
}

static double elapsed_s(const struct timespec *a, const struct timespec *b)
{
  return (b->tv_sec - a->tv_sec) + 1e-9 * (b->tv_nsec - a->tv_nsec);
}

int main(int argc, char **argv)
{
  if(argc == 3 && strcmp(argv[1], "--gen-count") == 0) {
    /* the graph count of a generated database, without generating it */
    ogen p;
    if(parse_gen(argv[2], &p) != 0) { fprintf(stderr, "bad generator spec %s\n", argv[2]); return 1; }
    printf("%lld\n", (long long)p.n_graphs);
    return 0;
  }
  if(argc == 4 && strcmp(argv[1], "--write-gen") == 0) {
    /* write a generated database as txt and exit */
    ogen p;
    if(parse_gen(argv[2], &p) != 0) { fprintf(stderr, "bad generator spec %s\n", argv[2]); return 1; }
    FILE *f = fopen(argv[3], "w");
    if(!f) { fprintf(stderr, "cannot open %s\n", argv[3]); return 4; }
    generate(&p, 0, f);
    fclose(f);
    return 0;
  }
  if(argc < 4) {
    fprintf(stderr, "usage: %s <txt|fsg|bin|cudabin|gen> <file|config[,seed[,scale]]> <abs-minsup> [out|-] "
                    "[--max-edges N] [--graph-limit G] [--time-limit S] [--roots i/n] [--repeat K] [--roots-once]\n"
                    "       %s --write-gen <config[,seed[,scale]]> <out.txt>\n"
                    "       %s --gen-count <config[,seed[,scale]]>\n", argv[0], argv[0], argv[0]);
    return 1;
  }
  const char *ft = argv[1];
  if(ft[0] == '-') ft++;
  const char *outpath = 0;
  int max_edges = 0, graph_limit = 0, repeat = 1, roots_once = 0, nint = 0;
  double win = 0;
  double time_limit = 0;
  int root_part = 0, root_parts = 1;
  for(int i = 4; i < argc; i++) {
    if(strcmp(argv[i], "--max-edges") == 0 && i + 1 < argc) max_edges = atoi(argv[++i]);
    else if(strcmp(argv[i], "--graph-limit") == 0 && i + 1 < argc) graph_limit = atoi(argv[++i]);
    else if(strcmp(argv[i], "--time-limit") == 0 && i + 1 < argc) time_limit = atof(argv[++i]);
    else if(strcmp(argv[i], "--repeat") == 0 && i + 1 < argc) repeat = atoi(argv[++i]);
    else if(strcmp(argv[i], "--roots-once") == 0) roots_once = 1;
    else if(strcmp(argv[i], "--intervals") == 0 && i + 2 < argc) {
      nint = atoi(argv[++i]);
      win = atof(argv[++i]);
    }
    else if(strcmp(argv[i], "--roots") == 0 && i + 1 < argc) {
      if(sscanf(argv[++i], "%d/%d", &root_part, &root_parts) != 2 || root_parts < 1 || root_part < 0 ||
         root_part >= root_parts) { fprintf(stderr, "bad --roots i/n\n"); return 1; }
    }
    else outpath = argv[i];
  }
  if(repeat < 1) { fprintf(stderr, "bad --repeat\n"); return 1; }
  odb db = { 0, 0, 0 };
  int rc;
  struct timespec tl0, tl1;
  clock_gettime(CLOCK_MONOTONIC, &tl0);
  if(strcmp(ft, "txt") == 0) rc = read_text_db(argv[2], 0, &db, graph_limit);
  else if(strcmp(ft, "fsg") == 0) rc = read_text_db(argv[2], 1, &db, graph_limit);
  else if(strcmp(ft, "cudabin") == 0) rc = read_cudabin_db(argv[2], &db, graph_limit);
  else if(strcmp(ft, "bin") == 0) rc = read_bin_db(argv[2], &db, graph_limit);
  else if(strcmp(ft, "gen") == 0) {
    ogen p;
    if(parse_gen(argv[2], &p) != 0) { fprintf(stderr, "bad generator spec %s\n", argv[2]); return 1; }
    if(graph_limit > 0 && p.n_graphs > graph_limit) p.n_graphs = graph_limit;
    generate(&p, &db, 0);
    rc = 0;
  }
  else { fprintf(stderr, "unknown filetype\n"); return 1; }
  if(rc != 0) { fprintf(stderr, "cannot read database %s\n", argv[2]); return 4; }
  clock_gettime(CLOCK_MONOTONIC, &tl1);
  int minsup = atoi(argv[3]);
  if(minsup >= db.n) {
    fprintf(stderr, "error: user specified support %d is greater then the database size %d\n", minsup, db.n);
    return 2;
  }
  if(minsup < 1) { fprintf(stderr, "error: absolute_min_support < 1\n"); return 3; }

  ominer m;
  memset(&m, 0, sizeof(m));
  m.db = &db;
  m.minsup = minsup;
  m.max_edges = max_edges;
  m.time_limit = time_limit;
  m.root_part = root_part;
  m.root_parts = root_parts;
  if(outpath == 0) m.out = stdout;
  else if(strcmp(outpath, "-") == 0) m.out = 0;
  else {
    m.out = fopen(outpath, "w");
    if(!m.out) { fprintf(stderr, "cannot open %s\n", outpath); return 4; }
  }
  {
    long long nv = 0, na = 0;
    for(int i = 0; i < db.n; i++) { nv += db.g[i].nv; na += db.g[i].off[db.g[i].nv]; }
    fprintf(stderr, "load_time=%.6f graphs=%d vertices=%lld adjacency_entries=%lld\n", elapsed_s(&tl0, &tl1), db.n,
            nv, na);
  }
  /* --roots-once builds the root map before the passes, untimed (a pass then
   * times the traversal alone); otherwise the first pass builds it */
  if(roots_once) {
    struct timespec r0, r1;
    clock_gettime(CLOCK_MONOTONIC, &r0);
    build_roots(&m);
    clock_gettime(CLOCK_MONOTONIC, &r1);
    fprintf(stderr, "roots_time=%.6f root_edges=%d\n", elapsed_s(&r0, &r1), m.roots.n);
  }
  if(nint > 0) {
    /* --intervals K S: mine for K windows of S seconds, restarting the
     * traversal whenever it completes; report the patterns found up to the
     * end of each window ("intervals=c1,c2,...", cumulative) */
    if(win <= 0 || nint > 100000) { fprintf(stderr, "bad --intervals\n"); return 1; }
    m.win = win;
    m.nint = nint;
    m.icount = xmalloc(sizeof(double) * nint);
    m.time_limit = nint * win;
    m.out = 0;
    struct timespec t0, t1;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    m.t0 = t0;
    int passes = 0;
    while(!m.stopped) {
      m.count = 0;
      run(&m);
      if(!m.stopped) { m.done += m.count; passes++; }
      out_of_time(&m);
      if(!m.stopped && m.count == 0 && passes > 0) break;  /* nothing frequent: no work to sample */
    }
    clock_gettime(CLOCK_MONOTONIC, &t1);
    for(; m.icur < nint; m.icur++) m.icount[m.icur] = m.done + m.count;
    fprintf(stderr, "sample_time=%.6f passes_completed=%d intervals=", elapsed_s(&t0, &t1), passes);
    for(int j = 0; j < nint; j++) fprintf(stderr, "%s%.0f", j ? "," : "", m.icount[j]);
    fprintf(stderr, "\n");
    return 0;
  }
  /* --repeat K mines the database K times (one timing line each, output
   * written on the first pass only), so that timed samples share one load */
  for(int rep = 0; rep < repeat; rep++) {
    struct timespec t0, t1;
    m.count = 0;
    m.stopped = 0;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    m.t0 = t0;
    run(&m);
    clock_gettime(CLOCK_MONOTONIC, &t1);
    if(rep == 0 && m.out && m.out != stdout) { fclose(m.out); m.out = 0; }
    if(rep == 0 && m.out == stdout) { fflush(stdout); m.out = 0; }
    fprintf(stderr, "total_time=%.6f total_frequent_graphs=%.0f%s\n", elapsed_s(&t0, &t1), m.count,
            m.stopped ? " stopped=time_limit" : "");
    fflush(stderr);
  }
  return 0;
}
