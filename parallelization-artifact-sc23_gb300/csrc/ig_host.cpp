// Host-side part of the library: error reporting, the ECLgraph .egr reader
// and writer, and the deterministic synthetic graph generators used by the
// benchmarks and tests.  Nothing here touches a GPU.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <string>
#include <thread>
#include <vector>

#include "ig_internal.h"

// ---------------------------------------------------------------------------
// Errors
// ---------------------------------------------------------------------------
static thread_local char g_errbuf[512];

int ig_fail(int status, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_errbuf, sizeof(g_errbuf), fmt, ap);
  va_end(ap);
  return status;
}

void ig_clear_error() { g_errbuf[0] = 0; }

extern "C" const char* ig_last_error(void) { return g_errbuf; }

extern "C" int ig_version(void) { return IG_VERSION; }

extern "C" const char* ig_status_string(int s) {
  switch (s) {
    case IG_OK: return "ok";
    case IG_ERR_INVALID_ARG: return "invalid argument";
    case IG_ERR_CUDA: return "CUDA error";
    case IG_ERR_NOMEM: return "out of memory";
    case IG_ERR_TIMEOUT: return "device wait timed out";
    case IG_ERR_UNSORTED: return "adjacency list not sorted or contains self edge";
    case IG_ERR_NO_DEVICE: return "no CUDA device";
    case IG_ERR_OVERFLOW: return "device queue overflow";
    case IG_ERR_IO: return "I/O error";
    case IG_ERR_FORMAT: return "malformed graph";
    case IG_ERR_BUSY: return "busy";
    case IG_ERR_CANCELLED: return "cancelled";
    default: return "unknown status";
  }
}

// ---------------------------------------------------------------------------
// .egr I/O -- the binary layout of include/ECLgraph.h:52-96
// ---------------------------------------------------------------------------
extern "C" void ig_csr_free_host(ig_csr* g) {
  if (!g) return;
  free(g->nindex);
  free(g->nlist);
  free(g->eweight);
  g->nindex = g->nlist = g->eweight = nullptr;
}

extern "C" int ig_egr_read(const char* path, ig_csr* out) {
  if (!path || !out) return ig_fail(IG_ERR_INVALID_ARG, "ig_egr_read: null argument");
  memset(out, 0, sizeof(*out));
  FILE* f = fopen(path, "rb");
  if (!f) return ig_fail(IG_ERR_IO, "could not open file %s", path);
  int hdr[2];
  if (fread(hdr, sizeof(int), 2, f) != 2) {
    fclose(f);
    return ig_fail(IG_ERR_FORMAT, "failed to read nodes/edges of %s", path);
  }
  const int nodes = hdr[0], edges = hdr[1];
  if (nodes < 1 || edges < 0) {
    fclose(f);
    return ig_fail(IG_ERR_FORMAT, "node or edge count too low (%d, %d)", nodes, edges);
  }
  ig_csr g{nodes, edges, nullptr, nullptr, nullptr};
  g.nindex = (int*)malloc(((size_t)nodes + 1) * sizeof(int));
  g.nlist = (int*)malloc(std::max<size_t>(1, (size_t)edges) * sizeof(int));
  g.eweight = (int*)malloc(std::max<size_t>(1, (size_t)edges) * sizeof(int));
  if (!g.nindex || !g.nlist || !g.eweight) {
    ig_csr_free_host(&g);
    fclose(f);
    return ig_fail(IG_ERR_NOMEM, "memory allocation failed");
  }
  if (fread(g.nindex, sizeof(int), (size_t)nodes + 1, f) != (size_t)nodes + 1) {
    ig_csr_free_host(&g);
    fclose(f);
    return ig_fail(IG_ERR_FORMAT, "failed to read neighbor index list");
  }
  if (fread(g.nlist, sizeof(int), (size_t)edges, f) != (size_t)edges) {
    ig_csr_free_host(&g);
    fclose(f);
    return ig_fail(IG_ERR_FORMAT, "failed to read neighbor list");
  }
  const size_t cnt = fread(g.eweight, sizeof(int), (size_t)edges, f);
  if (cnt == 0) {
    free(g.eweight);
    g.eweight = nullptr;
  } else if (cnt != (size_t)edges) {
    ig_csr_free_host(&g);
    fclose(f);
    return ig_fail(IG_ERR_FORMAT, "failed to read edge weights");
  }
  fclose(f);
  // Structural checks the reference leaves to chance: a monotone index
  // bounded by the edge count and neighbours in range.
  if (g.nindex[0] != 0 || g.nindex[nodes] != edges) {
    ig_csr_free_host(&g);
    return ig_fail(IG_ERR_FORMAT, "nindex does not span [0, edges]");
  }
  for (int v = 0; v < nodes; v++) {
    if (g.nindex[v] > g.nindex[v + 1]) {
      ig_csr_free_host(&g);
      return ig_fail(IG_ERR_FORMAT, "nindex not monotone at %d", v);
    }
  }
  for (int e = 0; e < edges; e++) {
    if (g.nlist[e] < 0 || g.nlist[e] >= nodes) {
      ig_csr_free_host(&g);
      return ig_fail(IG_ERR_FORMAT, "neighbour out of range at edge %d", e);
    }
  }
  *out = g;
  return IG_OK;
}

extern "C" int ig_egr_write(const char* path, const ig_csr* g) {
  if (!path || !g || !g->nindex || (g->edges > 0 && !g->nlist))
    return ig_fail(IG_ERR_INVALID_ARG, "ig_egr_write: null argument");
  if (g->nodes < 1 || g->edges < 0) return ig_fail(IG_ERR_INVALID_ARG, "node or edge count too low");
  FILE* f = fopen(path, "wb");
  if (!f) return ig_fail(IG_ERR_IO, "could not open file %s", path);
  int hdr[2] = {g->nodes, g->edges};
  bool ok = fwrite(hdr, sizeof(int), 2, f) == 2;
  ok = ok && fwrite(g->nindex, sizeof(int), (size_t)g->nodes + 1, f) == (size_t)g->nodes + 1;
  ok = ok && fwrite(g->nlist, sizeof(int), (size_t)g->edges, f) == (size_t)g->edges;
  if (ok && g->eweight) ok = fwrite(g->eweight, sizeof(int), (size_t)g->edges, f) == (size_t)g->edges;
  fclose(f);
  return ok ? IG_OK : ig_fail(IG_ERR_IO, "failed to write %s", path);
}

// ---------------------------------------------------------------------------
// Counter-based random numbers (SplitMix64 finaliser): value(seed, stream, i)
// depends only on its arguments, so generation is identical for any thread
// count and on any host architecture.
// ---------------------------------------------------------------------------
static inline uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
struct Rng {
  uint64_t key;
  Rng(uint64_t seed, uint64_t stream) : key(mix64(seed ^ mix64(stream * 0xD1B54A32D192ED03ull))) {}
  inline uint64_t at(uint64_t i) const { return mix64(key + i * 0x9E3779B97F4A7C15ull); }
  inline double uniform(uint64_t i) const { return (double)(at(i) >> 11) * (1.0 / 9007199254740992.0); }
};

static int hw_threads() {
  unsigned n = std::thread::hardware_concurrency();
  if (n == 0) n = 4;
  return (int)std::min(n, 64u);
}

// Set inside per-graph workers of ig_gen_batch, which run many small graphs
// in parallel: their inner loops then stay on the calling thread.
static thread_local bool t_serial = false;

template <class F>
static void parallel_for(long long n, F&& f) {
  const int T = hw_threads();
  if (n < 65536 || T == 1 || t_serial) {
    f(0LL, n, 0);
    return;
  }
  std::vector<std::thread> th;
  for (int t = 0; t < T; t++) {
    const long long b = n * t / T, e = n * (t + 1) / T;
    th.emplace_back([&f, b, e, t] { f(b, e, t); });
  }
  for (auto& x : th) x.join();
}

// Symmetric weight of the undirected edge {u, v}: uniform in [1, maxw].
static inline int edge_weight(const Rng& wr, int u, int v, int maxw) {
  const uint64_t a = (uint64_t)(unsigned)std::min(u, v), b = (uint64_t)(unsigned)std::max(u, v);
  return 1 + (int)(wr.at((a << 32) | b) % (uint64_t)maxw);
}

// Builds a symmetric, sorted, duplicate- and self-loop-free CSR from a list
// of undirected pairs (both directions are inserted).
static int build_csr(int n, const std::vector<int>& us, const std::vector<int>& vs, int maxw,
                     uint64_t wseed, ig_csr* out) {
  const long long m = (long long)us.size();
  std::vector<std::atomic<int>> deg(n);
  for (int i = 0; i < n; i++) deg[i].store(0, std::memory_order_relaxed);
  parallel_for(m, [&](long long b, long long e, int) {
    for (long long i = b; i < e; i++) {
      const int u = us[i], v = vs[i];
      if (u == v) continue;
      deg[u].fetch_add(1, std::memory_order_relaxed);
      deg[v].fetch_add(1, std::memory_order_relaxed);
    }
  });
  std::vector<long long> off(n + 1, 0);
  for (int i = 0; i < n; i++) off[i + 1] = off[i] + deg[i].load(std::memory_order_relaxed);
  if (off[n] > (long long)INT32_MAX) return ig_fail(IG_ERR_OVERFLOW, "graph has more than 2^31-1 edges");
  std::vector<int> tmp((size_t)std::max<long long>(1, off[n]));
  std::vector<std::atomic<long long>> pos(n);
  for (int i = 0; i < n; i++) pos[i].store(off[i], std::memory_order_relaxed);
  parallel_for(m, [&](long long b, long long e, int) {
    for (long long i = b; i < e; i++) {
      const int u = us[i], v = vs[i];
      if (u == v) continue;
      tmp[pos[u].fetch_add(1, std::memory_order_relaxed)] = v;
      tmp[pos[v].fetch_add(1, std::memory_order_relaxed)] = u;
    }
  });
  // sort + dedupe each list
  std::vector<int> ndeg(n);
  parallel_for(n, [&](long long b, long long e, int) {
    for (long long v = b; v < e; v++) {
      int* s = tmp.data() + off[v];
      int* t = tmp.data() + off[v + 1];
      std::sort(s, t);
      ndeg[v] = (int)(std::unique(s, t) - s);
    }
  });
  ig_csr g{n, 0, nullptr, nullptr, nullptr};
  g.nindex = (int*)malloc(((size_t)n + 1) * sizeof(int));
  if (!g.nindex) return ig_fail(IG_ERR_NOMEM, "allocation failed");
  g.nindex[0] = 0;
  for (int v = 0; v < n; v++) g.nindex[v + 1] = g.nindex[v] + ndeg[v];
  g.edges = g.nindex[n];
  g.nlist = (int*)malloc(std::max<size_t>(1, (size_t)g.edges) * sizeof(int));
  if (maxw > 0) g.eweight = (int*)malloc(std::max<size_t>(1, (size_t)g.edges) * sizeof(int));
  if (!g.nlist || (maxw > 0 && !g.eweight)) {
    ig_csr_free_host(&g);
    return ig_fail(IG_ERR_NOMEM, "allocation failed");
  }
  const Rng wr(wseed, 0x77);
  parallel_for(n, [&](long long b, long long e, int) {
    for (long long v = b; v < e; v++) {
      memcpy(g.nlist + g.nindex[v], tmp.data() + off[v], (size_t)ndeg[v] * sizeof(int));
      if (maxw > 0)
        for (int i = g.nindex[v]; i < g.nindex[v + 1]; i++)
          g.eweight[i] = edge_weight(wr, (int)v, g.nlist[i], maxw);
    }
  });
  *out = g;
  return IG_OK;
}

extern "C" int ig_gen_grid2d(int nx, int ny, int maxw, uint64_t seed, ig_csr* out) {
  if (!out || nx < 1 || ny < 1 || (long long)nx * ny > INT32_MAX)
    return ig_fail(IG_ERR_INVALID_ARG, "ig_gen_grid2d: bad size");
  const int n = nx * ny;
  ig_csr g{n, 0, nullptr, nullptr, nullptr};
  const long long e = 2LL * (nx - 1) * ny + 2LL * nx * (ny - 1);
  if (e > INT32_MAX) return ig_fail(IG_ERR_OVERFLOW, "grid too large");
  g.edges = (int)e;
  g.nindex = (int*)malloc(((size_t)n + 1) * sizeof(int));
  g.nlist = (int*)malloc(std::max<size_t>(1, (size_t)e) * sizeof(int));
  if (maxw > 0) g.eweight = (int*)malloc(std::max<size_t>(1, (size_t)e) * sizeof(int));
  if (!g.nindex || !g.nlist || (maxw > 0 && !g.eweight)) {
    ig_csr_free_host(&g);
    return ig_fail(IG_ERR_NOMEM, "allocation failed");
  }
  // vertex id = y * nx + x; neighbours listed in ascending id order
  int k = 0;
  for (int y = 0; y < ny; y++) {
    for (int x = 0; x < nx; x++) {
      g.nindex[y * nx + x] = k;
      if (y > 0) g.nlist[k++] = (y - 1) * nx + x;
      if (x > 0) g.nlist[k++] = y * nx + x - 1;
      if (x + 1 < nx) g.nlist[k++] = y * nx + x + 1;
      if (y + 1 < ny) g.nlist[k++] = (y + 1) * nx + x;
    }
  }
  g.nindex[n] = k;
  if (maxw > 0) {
    const Rng wr(seed, 0x77);
    for (int v = 0; v < n; v++)
      for (int i = g.nindex[v]; i < g.nindex[v + 1]; i++) g.eweight[i] = edge_weight(wr, v, g.nlist[i], maxw);
  }
  *out = g;
  return IG_OK;
}

// Fisher-Yates permutation of [0, n) from the counter RNG.
static std::vector<int> random_permutation(int n, uint64_t seed) {
  std::vector<int> p(n);
  std::iota(p.begin(), p.end(), 0);
  const Rng r(seed, 0x9e3);
  for (int i = n - 1; i > 0; i--) {
    const int j = (int)(r.at((uint64_t)i) % (uint64_t)(i + 1));
    std::swap(p[i], p[j]);
  }
  return p;
}

extern "C" int ig_gen_rmat(int scale, int edge_factor, double a, double b, double c, uint64_t seed,
                           int maxw, int permute, ig_csr* out) {
  if (!out || scale < 1 || scale > 30 || edge_factor < 1 || a < 0 || b < 0 || c < 0 || a + b + c > 1.0)
    return ig_fail(IG_ERR_INVALID_ARG, "ig_gen_rmat: bad parameters");
  const int n = 1 << scale;
  const long long m = (long long)n * edge_factor;
  std::vector<int> us((size_t)m), vs((size_t)m);
  // Each level consumes 32 random bits: quadrant a (0,0), b (0,1), c (1,0), d (1,1).
  const uint32_t ta = (uint32_t)std::min(4294967295.0, a * 4294967296.0);
  const uint32_t tb = (uint32_t)std::min(4294967295.0, (a + b) * 4294967296.0);
  const uint32_t tc = (uint32_t)std::min(4294967295.0, (a + b + c) * 4294967296.0);
  const Rng r(seed, 0x5a7);
  parallel_for(m, [&](long long lo, long long hi, int) {
    for (long long k = lo; k < hi; k++) {
      int u = 0, v = 0;
      uint64_t bits = 0;
      for (int lev = 0; lev < scale; lev++) {
        if ((lev & 1) == 0) bits = r.at((uint64_t)k * 16 + (uint64_t)(lev >> 1));
        const uint32_t x = (uint32_t)(bits >> ((lev & 1) * 32));
        const int bu = (x >= tb) ? 1 : 0;
        const int bv = (x >= ta && x < tb) || (x >= tc) ? 1 : 0;
        u = (u << 1) | bu;
        v = (v << 1) | bv;
      }
      us[k] = u;
      vs[k] = v;
    }
  });
  if (permute) {
    const std::vector<int> p = random_permutation(n, seed);
    parallel_for(m, [&](long long lo, long long hi, int) {
      for (long long k = lo; k < hi; k++) {
        us[k] = p[us[k]];
        vs[k] = p[vs[k]];
      }
    });
  }
  return build_csr(n, us, vs, maxw, seed, out);
}

extern "C" int ig_gen_road(int nx, int ny, double delete_frac, double shortcut_frac, uint64_t seed, int maxw,
                           ig_csr* out) {
  if (!out || nx < 1 || ny < 1 || (long long)nx * ny > INT32_MAX || delete_frac < 0 || delete_frac > 1 ||
      shortcut_frac < 0)
    return ig_fail(IG_ERR_INVALID_ARG, "ig_gen_road: bad parameters");
  const int n = nx * ny;
  const long long horiz = (long long)(nx - 1) * ny, vert = (long long)nx * (ny - 1);
  const long long grid_edges = horiz + vert;
  const long long shortcuts = (long long)llround(shortcut_frac * (double)grid_edges);
  const Rng del(seed, 0xde1), sc(seed, 0x5c);
  std::vector<int> us, vs;
  us.reserve((size_t)(grid_edges + shortcuts));
  vs.reserve((size_t)(grid_edges + shortcuts));
  for (long long e = 0; e < grid_edges; e++) {
    if (del.uniform((uint64_t)e) < delete_frac) continue;
    int u, v;
    if (e < horiz) {
      const int y = (int)(e / (nx - 1)), x = (int)(e % (nx - 1));
      u = y * nx + x;
      v = u + 1;
    } else {
      const long long f = e - horiz;
      const int y = (int)(f / nx), x = (int)(f % nx);
      u = y * nx + x;
      v = u + nx;
    }
    us.push_back(u);
    vs.push_back(v);
  }
  for (long long s = 0; s < shortcuts; s++) {
    us.push_back((int)(sc.at((uint64_t)(2 * s)) % (uint64_t)n));
    vs.push_back((int)(sc.at((uint64_t)(2 * s + 1)) % (uint64_t)n));
  }
  return build_csr(n, us, vs, maxw, seed, out);
}

extern "C" int ig_gen_er(int n, double avg_degree, uint64_t seed, int maxw, ig_csr* out) {
  if (!out || n < 1 || avg_degree < 0) return ig_fail(IG_ERR_INVALID_ARG, "ig_gen_er: bad parameters");
  const long long m = (long long)llround((double)n * avg_degree / 2.0);
  std::vector<int> us((size_t)m), vs((size_t)m);
  const Rng r(seed, 0xe7);
  parallel_for(m, [&](long long lo, long long hi, int) {
    for (long long k = lo; k < hi; k++) {
      us[k] = (int)(r.at((uint64_t)(2 * k)) % (uint64_t)n);
      vs[k] = (int)(r.at((uint64_t)(2 * k + 1)) % (uint64_t)n);
    }
  });
  return build_csr(n, us, vs, maxw, seed, out);
}

extern "C" int ig_degree_order(const ig_csr* in, ig_csr* out) {
  if (!in || !out || !in->nindex || in->nodes < 1) return ig_fail(IG_ERR_INVALID_ARG, "ig_degree_order: bad graph");
  const int n = in->nodes;
  std::vector<int> order(n);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
    return (in->nindex[x + 1] - in->nindex[x]) < (in->nindex[y + 1] - in->nindex[y]);
  });
  std::vector<int> rank(n);
  for (int i = 0; i < n; i++) rank[order[i]] = i;
  ig_csr g{n, in->edges, nullptr, nullptr, nullptr};
  g.nindex = (int*)malloc(((size_t)n + 1) * sizeof(int));
  g.nlist = (int*)malloc(std::max<size_t>(1, (size_t)in->edges) * sizeof(int));
  if (in->eweight) g.eweight = (int*)malloc(std::max<size_t>(1, (size_t)in->edges) * sizeof(int));
  if (!g.nindex || !g.nlist || (in->eweight && !g.eweight)) {
    ig_csr_free_host(&g);
    return ig_fail(IG_ERR_NOMEM, "allocation failed");
  }
  g.nindex[0] = 0;
  for (int i = 0; i < n; i++) {
    const int v = order[i];
    g.nindex[i + 1] = g.nindex[i] + (in->nindex[v + 1] - in->nindex[v]);
  }
  parallel_for(n, [&](long long b, long long e, int) {
    std::vector<std::pair<int, int>> tmp;
    for (long long i = b; i < e; i++) {
      const int v = order[i];
      tmp.clear();
      for (int k = in->nindex[v]; k < in->nindex[v + 1]; k++)
        tmp.emplace_back(rank[in->nlist[k]], in->eweight ? in->eweight[k] : 0);
      std::sort(tmp.begin(), tmp.end());
      int k = g.nindex[i];
      for (auto& p : tmp) {
        g.nlist[k] = p.first;
        if (g.eweight) g.eweight[k] = p.second;
        k++;
      }
    }
  });
  *out = g;
  return IG_OK;
}

extern "C" int ig_pick_sources(const ig_csr* g, int k, uint64_t seed, int* out) {
  if (!g || !out || k < 0 || !g->nindex) return ig_fail(IG_ERR_INVALID_ARG, "ig_pick_sources: bad argument");
  const Rng r(seed, 0x50);
  std::vector<char> taken(g->nodes, 0);
  int got = 0;
  for (uint64_t i = 0; got < k && i < (uint64_t)g->nodes * 64 + 1024; i++) {
    const int v = (int)(r.at(i) % (uint64_t)g->nodes);
    if (taken[v] || g->nindex[v + 1] == g->nindex[v]) continue;
    taken[v] = 1;
    out[got++] = v;
  }
  if (got < k) return ig_fail(IG_ERR_INVALID_ARG, "fewer than %d vertices with degree > 0", k);
  return IG_OK;
}

extern "C" int ig_csr_check_sorted(const ig_csr* g) {
  if (!g || !g->nindex || (g->edges > 0 && !g->nlist)) return ig_fail(IG_ERR_INVALID_ARG, "null graph");
  for (int v = 0; v < g->nodes; v++)
    for (int i = g->nindex[v] + 1; i < g->nindex[v + 1]; i++)
      if (g->nlist[i - 1] >= g->nlist[i]) return ig_fail(IG_ERR_UNSORTED, "adjacency of %d not sorted", v);
  for (int v = 0; v < g->nodes; v++)
    for (int i = g->nindex[v]; i < g->nindex[v + 1]; i++)
      if (g->nlist[i] == v) return ig_fail(IG_ERR_UNSORTED, "self edge at %d", v);
  return IG_OK;
}

static inline uint64_t fnv(uint64_t h, const void* p, size_t n) {
  const unsigned char* b = (const unsigned char*)p;
  for (size_t i = 0; i < n; i++) {
    h ^= b[i];
    h *= 0x100000001b3ull;
  }
  return h;
}

extern "C" uint64_t ig_csr_digest(const ig_csr* g) {
  if (!g) return 0;
  uint64_t h = 0xcbf29ce484222325ull;
  h = fnv(h, &g->nodes, sizeof(int));
  h = fnv(h, &g->edges, sizeof(int));
  if (g->nindex) h = fnv(h, g->nindex, ((size_t)g->nodes + 1) * sizeof(int));
  if (g->nlist) h = fnv(h, g->nlist, (size_t)g->edges * sizeof(int));
  if (g->eweight) h = fnv(h, g->eweight, (size_t)g->edges * sizeof(int));
  return h;
}

// RMAT pairs on n vertices (ids drawn at the next power of two, taken mod n).
static void rmat_pairs(int n, long long m, double a, double b, double c, const Rng& r, std::vector<int>& us,
                       std::vector<int>& vs) {
  int scale = 0;
  while ((1LL << scale) < n) scale++;
  const uint32_t ta = (uint32_t)std::min(4294967295.0, a * 4294967296.0);
  const uint32_t tb = (uint32_t)std::min(4294967295.0, (a + b) * 4294967296.0);
  const uint32_t tc = (uint32_t)std::min(4294967295.0, (a + b + c) * 4294967296.0);
  us.resize((size_t)m);
  vs.resize((size_t)m);
  for (long long k = 0; k < m; k++) {
    long long u = 0, v = 0;
    uint64_t bits = 0;
    for (int lev = 0; lev < scale; lev++) {
      if ((lev & 1) == 0) bits = r.at((uint64_t)k * 16 + (uint64_t)(lev >> 1));
      const uint32_t x = (uint32_t)(bits >> ((lev & 1) * 32));
      u = (u << 1) | ((x >= tb) ? 1 : 0);
      v = (v << 1) | (((x >= ta && x < tb) || x >= tc) ? 1 : 0);
    }
    us[k] = (int)(u % n);
    vs[k] = (int)(v % n);
  }
}

extern "C" int ig_gen_batch(int graphs, int vmin, int vmax, double er_degree, int rmat_edge_factor, double a,
                            double b, double c, uint64_t seed, int maxw, ig_csr* out_union, int* out_vptr) {
  if (graphs < 1 || vmin < 2 || vmax < vmin || !out_union || !out_vptr || er_degree < 0 || rmat_edge_factor < 0)
    return ig_fail(IG_ERR_INVALID_ARG, "ig_gen_batch: bad parameters");
  std::vector<ig_csr> parts((size_t)graphs);
  std::vector<int> rcs((size_t)graphs, IG_OK);
  const Rng sizes(seed, 0xb47c);
  std::atomic<int> next{0};
  const int T = hw_threads();
  std::vector<std::thread> th;
  for (int t = 0; t < T; t++) {
    th.emplace_back([&] {
      t_serial = true;
      for (int i = next.fetch_add(1); i < graphs; i = next.fetch_add(1)) {
        const double lo = std::log((double)vmin), hi = std::log((double)vmax);
        const int n = std::max(vmin, std::min(vmax, (int)llround(std::exp(lo + (hi - lo) * sizes.uniform((uint64_t)i)))));
        const uint64_t gseed = seed * 0x9E3779B97F4A7C15ull + (uint64_t)i;
        std::vector<int> us, vs;
        if ((i & 1) == 0) {
          const long long m = (long long)llround((double)n * er_degree / 2.0);
          const Rng r(gseed, 0xe7);
          us.resize((size_t)m);
          vs.resize((size_t)m);
          for (long long k = 0; k < m; k++) {
            us[k] = (int)(r.at((uint64_t)(2 * k)) % (uint64_t)n);
            vs[k] = (int)(r.at((uint64_t)(2 * k + 1)) % (uint64_t)n);
          }
        } else {
          const Rng r(gseed, 0x5a7);
          rmat_pairs(n, (long long)n * rmat_edge_factor, a, b, c, r, us, vs);
        }
        rcs[i] = build_csr(n, us, vs, maxw, gseed, &parts[i]);
      }
    });
  }
  for (auto& x : th) x.join();
  for (int i = 0; i < graphs; i++)
    if (rcs[i] != IG_OK) {
      for (auto& p : parts) ig_csr_free_host(&p);
      return rcs[i];
    }
  long long V = 0, E = 0;
  for (int i = 0; i < graphs; i++) {
    out_vptr[i] = (int)V;
    V += parts[i].nodes;
    E += parts[i].edges;
  }
  out_vptr[graphs] = (int)V;
  if (V > INT32_MAX || E > INT32_MAX) {
    for (auto& p : parts) ig_csr_free_host(&p);
    return ig_fail(IG_ERR_OVERFLOW, "batch exceeds 2^31-1 vertices or edges");
  }
  ig_csr u{(int)V, (int)E, nullptr, nullptr, nullptr};
  u.nindex = (int*)malloc(((size_t)V + 1) * sizeof(int));
  u.nlist = (int*)malloc(std::max<size_t>(1, (size_t)E) * sizeof(int));
  if (maxw > 0) u.eweight = (int*)malloc(std::max<size_t>(1, (size_t)E) * sizeof(int));
  if (!u.nindex || !u.nlist || (maxw > 0 && !u.eweight)) {
    ig_csr_free_host(&u);
    for (auto& p : parts) ig_csr_free_host(&p);
    return ig_fail(IG_ERR_NOMEM, "allocation failed");
  }
  std::vector<long long> eoff((size_t)graphs + 1, 0);
  for (int i = 0; i < graphs; i++) eoff[i + 1] = eoff[i] + parts[i].edges;
  parallel_for(graphs, [&](long long lo, long long hi, int) {
    for (long long i = lo; i < hi; i++) {
      const ig_csr& p = parts[i];
      const int vo = out_vptr[i];
      const long long eo = eoff[i];
      for (int v = 0; v < p.nodes; v++) u.nindex[vo + v] = (int)(eo + p.nindex[v]);
      for (int e = 0; e < p.edges; e++) u.nlist[eo + e] = p.nlist[e] + vo;
      if (maxw > 0) memcpy(u.eweight + eo, p.eweight, (size_t)p.edges * sizeof(int));
    }
  });
  u.nindex[V] = (int)E;
  for (auto& p : parts) ig_csr_free_host(&p);
  *out_union = u;
  return IG_OK;
}
