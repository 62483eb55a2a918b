/*
 * workload.c -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU generator of the synthetic RMAT workload for the CPU arms of the
 * benchmark (the timed run of the reference's own C++ programs, or of the
 * oracle's threaded restatement), so that those arms load no GPU library.
 * It restates the library's host generator (counter-based SplitMix64
 * stream, RMAT quadrant draws, optional Fisher-Yates relabelling,
 * symmetrised CSR with sorted, de-duplicated, self-loop-free lists and
 * symmetric weights), its (degree, id) relabelling and its source picker;
 * tests/test_oracle_workload.py proves its arrays identical to the
 * library generator's.
 *
 * The graph recipe is the benchmark's, not the reference's: the reference
 * reads downloaded .egr files (include/ECLgraph.h:52-80), which the
 * synthetic graphs stand in for.
 */
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

/* ---------------------------------------------------------------- random */
static inline uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
static inline uint64_t rng_key(uint64_t seed, uint64_t stream) {
  return mix64(seed ^ mix64(stream * 0xD1B54A32D192ED03ull));
}
static inline uint64_t rng_at(uint64_t key, uint64_t i) { return mix64(key + i * 0x9E3779B97F4A7C15ull); }

/* --------------------------------------------------------------- threads */
typedef struct {
  long long lo, hi;
  void* ctx;
} span_t;

static int g_threads = 8;

static void par_for(long long n, void* ctx, void* (*fn)(void*)) {
  int T = g_threads < 1 ? 1 : g_threads;
  if (n < 65536) T = 1;
  pthread_t th[256];
  span_t sp[256];
  if (T > 256) T = 256;
  for (int t = 0; t < T; t++) {
    sp[t].lo = n * t / T;
    sp[t].hi = n * (t + 1) / T;
    sp[t].ctx = ctx;
  }
  if (T == 1) {
    fn(&sp[0]);
    return;
  }
  for (int t = 0; t < T; t++) pthread_create(&th[t], NULL, fn, &sp[t]);
  for (int t = 0; t < T; t++) pthread_join(th[t], NULL);
}

/* ------------------------------------------------------------ RMAT pairs */
typedef struct {
  int scale;
  uint32_t ta, tb, tc;
  uint64_t key;
  int *us, *vs;
  const int* perm;
} rmat_ctx;

static void* rmat_worker(void* p) {
  span_t* s = (span_t*)p;
  rmat_ctx* c = (rmat_ctx*)s->ctx;
  for (long long k = s->lo; k < s->hi; k++) {
    int u = 0, v = 0;
    uint64_t bits = 0;
    for (int lev = 0; lev < c->scale; lev++) {
      if ((lev & 1) == 0) bits = rng_at(c->key, (uint64_t)k * 16 + (uint64_t)(lev >> 1));
      const uint32_t x = (uint32_t)(bits >> ((lev & 1) * 32));
      u = (u << 1) | (x >= c->tb ? 1 : 0);
      v = (v << 1) | (((x >= c->ta && x < c->tb) || x >= c->tc) ? 1 : 0);
    }
    if (c->perm) {
      u = c->perm[u];
      v = c->perm[v];
    }
    c->us[k] = u;
    c->vs[k] = v;
  }
  return NULL;
}

static uint32_t threshold(double p) {
  const double x = p * 4294967296.0;
  return (uint32_t)(x < 4294967295.0 ? x : 4294967295.0);
}

/* ------------------------------------------------------------ CSR build */
typedef struct {
  int n;
  long long m;
  const int *us, *vs;
  int* deg;          /* counts (atomic) */
  long long* off;    /* n + 1 */
  long long* pos;    /* fill positions (atomic) */
  int* tmp;
  int* ndeg;
  int *nindex, *nlist, *eweight;
  int maxw;
  uint64_t wkey;
} csr_ctx;

static void* count_worker(void* p) {
  span_t* s = (span_t*)p;
  csr_ctx* c = (csr_ctx*)s->ctx;
  for (long long i = s->lo; i < s->hi; i++) {
    const int u = c->us[i], v = c->vs[i];
    if (u == v) continue;
    __atomic_fetch_add(&c->deg[u], 1, __ATOMIC_RELAXED);
    __atomic_fetch_add(&c->deg[v], 1, __ATOMIC_RELAXED);
  }
  return NULL;
}

static void* fill_worker(void* p) {
  span_t* s = (span_t*)p;
  csr_ctx* c = (csr_ctx*)s->ctx;
  for (long long i = s->lo; i < s->hi; i++) {
    const int u = c->us[i], v = c->vs[i];
    if (u == v) continue;
    c->tmp[__atomic_fetch_add(&c->pos[u], 1, __ATOMIC_RELAXED)] = v;
    c->tmp[__atomic_fetch_add(&c->pos[v], 1, __ATOMIC_RELAXED)] = u;
  }
  return NULL;
}

static int cmp_int(const void* a, const void* b) {
  const int x = *(const int*)a, y = *(const int*)b;
  return (x > y) - (x < y);
}

static void sort_ints(int* a, long long n) {
  if (n < 24) { /* insertion sort for short lists */
    for (long long i = 1; i < n; i++) {
      const int x = a[i];
      long long j = i - 1;
      while (j >= 0 && a[j] > x) {
        a[j + 1] = a[j];
        j--;
      }
      a[j + 1] = x;
    }
    return;
  }
  qsort(a, (size_t)n, sizeof(int), cmp_int);
}

static void* sort_worker(void* p) {
  span_t* s = (span_t*)p;
  csr_ctx* c = (csr_ctx*)s->ctx;
  for (long long v = s->lo; v < s->hi; v++) {
    int* a = c->tmp + c->off[v];
    const long long len = c->off[v + 1] - c->off[v];
    sort_ints(a, len);
    long long k = 0;
    for (long long i = 0; i < len; i++)
      if (k == 0 || a[i] != a[k - 1]) a[k++] = a[i];
    c->ndeg[v] = (int)k;
  }
  return NULL;
}

static inline int edge_weight(uint64_t wkey, int u, int v, int maxw) {
  const uint64_t a = (uint64_t)(unsigned)(u < v ? u : v), b = (uint64_t)(unsigned)(u < v ? v : u);
  return 1 + (int)(rng_at(wkey, (a << 32) | b) % (uint64_t)maxw);
}

static void* copy_worker(void* p) {
  span_t* s = (span_t*)p;
  csr_ctx* c = (csr_ctx*)s->ctx;
  for (long long v = s->lo; v < s->hi; v++) {
    memcpy(c->nlist + c->nindex[v], c->tmp + c->off[v], (size_t)c->ndeg[v] * sizeof(int));
    if (c->maxw > 0)
      for (int i = c->nindex[v]; i < c->nindex[v + 1]; i++)
        c->eweight[i] = edge_weight(c->wkey, (int)v, c->nlist[i], c->maxw);
  }
  return NULL;
}

/* Outputs are malloc'd; the caller frees them with or_free.  Returns the
 * edge count, or -1 on failure. */
long long or_gen_rmat(int scale, int edge_factor, double a, double b, double c, unsigned long long seed, int maxw,
                      int permute, int threads, int** out_nindex, int** out_nlist, int** out_eweight) {
  g_threads = threads;
  const int n = 1 << scale;
  const long long m = (long long)n * edge_factor;
  rmat_ctx rc;
  rc.scale = scale;
  rc.ta = threshold(a);
  rc.tb = threshold(a + b);
  rc.tc = threshold(a + b + c);
  rc.key = rng_key(seed, 0x5a7);
  rc.us = (int*)malloc((size_t)m * sizeof(int));
  rc.vs = (int*)malloc((size_t)m * sizeof(int));
  int* perm = NULL;
  if (!rc.us || !rc.vs) return -1;
  if (permute) { /* Fisher-Yates from the counter stream */
    perm = (int*)malloc((size_t)n * sizeof(int));
    if (!perm) return -1;
    for (int i = 0; i < n; i++) perm[i] = i;
    const uint64_t pk = rng_key(seed, 0x9e3);
    for (int i = n - 1; i > 0; i--) {
      const int j = (int)(rng_at(pk, (uint64_t)i) % (uint64_t)(i + 1));
      const int t = perm[i];
      perm[i] = perm[j];
      perm[j] = t;
    }
  }
  rc.perm = perm;
  par_for(m, &rc, rmat_worker);
  free(perm);

  csr_ctx cc;
  memset(&cc, 0, sizeof(cc));
  cc.n = n;
  cc.m = m;
  cc.us = rc.us;
  cc.vs = rc.vs;
  cc.maxw = maxw;
  cc.wkey = rng_key(seed, 0x77);
  cc.deg = (int*)calloc((size_t)n, sizeof(int));
  cc.off = (long long*)malloc(((size_t)n + 1) * sizeof(long long));
  cc.pos = (long long*)malloc((size_t)n * sizeof(long long));
  cc.ndeg = (int*)malloc((size_t)n * sizeof(int));
  if (!cc.deg || !cc.off || !cc.pos || !cc.ndeg) return -1;
  par_for(m, &cc, count_worker);
  cc.off[0] = 0;
  for (int i = 0; i < n; i++) cc.off[i + 1] = cc.off[i] + cc.deg[i];
  if (cc.off[n] > 2147483647LL) return -1;
  for (int i = 0; i < n; i++) cc.pos[i] = cc.off[i];
  cc.tmp = (int*)malloc((size_t)(cc.off[n] > 0 ? cc.off[n] : 1) * sizeof(int));
  if (!cc.tmp) return -1;
  par_for(m, &cc, fill_worker);
  free(rc.us);
  free(rc.vs);
  par_for(n, &cc, sort_worker);
  cc.nindex = (int*)malloc(((size_t)n + 1) * sizeof(int));
  if (!cc.nindex) return -1;
  cc.nindex[0] = 0;
  for (int v = 0; v < n; v++) cc.nindex[v + 1] = cc.nindex[v] + cc.ndeg[v];
  const int E = cc.nindex[n];
  cc.nlist = (int*)malloc((size_t)(E > 0 ? E : 1) * sizeof(int));
  cc.eweight = maxw > 0 ? (int*)malloc((size_t)(E > 0 ? E : 1) * sizeof(int)) : NULL;
  if (!cc.nlist || (maxw > 0 && !cc.eweight)) return -1;
  par_for(n, &cc, copy_worker);
  free(cc.deg);
  free(cc.off);
  free(cc.pos);
  free(cc.tmp);
  free(cc.ndeg);
  *out_nindex = cc.nindex;
  *out_nlist = cc.nlist;
  *out_eweight = cc.eweight;
  return E;
}

/* ------------------------------------------------ (degree, id) relabelling */
typedef struct {
  const int *nindex, *nlist, *eweight;
  const int *order, *rank;
  int *onindex, *onlist, *oeweight;
} dord_ctx;

static int cmp_u64(const void* a, const void* b) {
  const uint64_t x = *(const uint64_t*)a, y = *(const uint64_t*)b;
  return (x > y) - (x < y);
}

static void* dord_worker(void* p) {
  span_t* s = (span_t*)p;
  dord_ctx* c = (dord_ctx*)s->ctx;
  uint64_t* buf = NULL;
  long long cap = 0;
  for (long long i = s->lo; i < s->hi; i++) {
    const int v = c->order[i];
    const int b = c->nindex[v], len = c->nindex[v + 1] - b;
    if (len > cap) {
      cap = len * 2;
      buf = (uint64_t*)realloc(buf, (size_t)cap * sizeof(uint64_t));
    }
    /* new ids are distinct within a list: sort (rank, weight) by rank */
    for (int k = 0; k < len; k++)
      buf[k] = ((uint64_t)(unsigned)c->rank[c->nlist[b + k]] << 32) |
               (uint64_t)(unsigned)(c->eweight ? c->eweight[b + k] : 0);
    if (len < 24) {
      for (int k = 1; k < len; k++) {
        const uint64_t x = buf[k];
        int j = k - 1;
        while (j >= 0 && buf[j] > x) {
          buf[j + 1] = buf[j];
          j--;
        }
        buf[j + 1] = x;
      }
    } else {
      qsort(buf, (size_t)len, sizeof(uint64_t), cmp_u64);
    }
    const int o = c->onindex[i];
    for (int k = 0; k < len; k++) {
      c->onlist[o + k] = (int)(buf[k] >> 32);
      if (c->oeweight) c->oeweight[o + k] = (int)(uint32_t)buf[k];
    }
  }
  free(buf);
  return NULL;
}

/* Vertices renumbered in ascending degree, ties by id (a stable counting
 * sort by degree), adjacency sorted by new id, weights carried along. */
int or_degree_order(int n, const int* nindex, const int* nlist, const int* eweight, int threads, int* onindex,
                    int* onlist, int* oeweight) {
  g_threads = threads;
  int maxd = 0;
  for (int v = 0; v < n; v++) {
    const int d = nindex[v + 1] - nindex[v];
    if (d > maxd) maxd = d;
  }
  long long* start = (long long*)calloc((size_t)maxd + 2, sizeof(long long));
  int* order = (int*)malloc((size_t)n * sizeof(int));
  int* rank = (int*)malloc((size_t)n * sizeof(int));
  if (!start || !order || !rank) return -1;
  for (int v = 0; v < n; v++) start[nindex[v + 1] - nindex[v] + 1]++;
  for (int d = 0; d <= maxd; d++) start[d + 1] += start[d];
  for (int v = 0; v < n; v++) order[start[nindex[v + 1] - nindex[v]]++] = v;
  for (int i = 0; i < n; i++) rank[order[i]] = i;
  onindex[0] = 0;
  for (int i = 0; i < n; i++) onindex[i + 1] = onindex[i] + (nindex[order[i] + 1] - nindex[order[i]]);
  dord_ctx c = {nindex, nlist, eweight, order, rank, onindex, onlist, eweight ? oeweight : NULL};
  par_for(n, &c, dord_worker);
  free(start);
  free(order);
  free(rank);
  return 0;
}

/* k distinct vertices of degree > 0 from the counter stream (seed, 0x50). */
int or_pick_sources(int n, const int* nindex, int k, unsigned long long seed, int* out) {
  const uint64_t key = rng_key(seed, 0x50);
  char* taken = (char*)calloc((size_t)n, 1);
  if (!taken) return -1;
  int got = 0;
  for (uint64_t i = 0; got < k && i < (uint64_t)n * 64 + 1024; i++) {
    const int v = (int)(rng_at(key, i) % (uint64_t)n);
    if (taken[v] || nindex[v + 1] == nindex[v]) continue;
    taken[v] = 1;
    out[got++] = v;
  }
  free(taken);
  return got == k ? 0 : -1;
}

void or_free(void* p) { free(p); }
