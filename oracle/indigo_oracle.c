/*
 * indigo_oracle.c -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement of the reference (yiqianl/Parallelization-Artifact-SC23,
 * Indigo2 suite) algorithms for BFS, SSSP, CC, MIS, PageRank and triangle
 * counting over the ECLgraph CSR.  It is the checker for the GPU library's
 * parity tests and, through the threaded functions, the CPU baseline that
 * bench.py times beside the GPU.  The product never links, loads or calls
 * this code.
 *
 * Parity pins: the serial functions are checked against outputs of the
 * reference's own C++ programs compiled from its sources (oracle/_ref, see
 * oracle/build_ref.sh) through the committed fixtures in tests/golden/.
 *
 * Every function cites the reference file:line it restates.  Compile with
 * -ffp-contract=off so the FP32 PageRank rounds as on the reference's x86
 * build (no fused multiply-add) on every host architecture.
 */
#include <limits.h>
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#define OR_INF INT_MAX

static double now_s(void) {
  struct timespec t;
  clock_gettime(CLOCK_MONOTONIC, &t);
  return (double)t.tv_sec + 1e-9 * (double)t.tv_nsec;
}

/* ------------------------------------------------------------------------
 * Binary max-heap of (key, vertex) pairs ordered like std::pair<int,int>
 * inside std::priority_queue: larger key first, then larger vertex.
 * ---------------------------------------------------------------------- */
typedef struct {
  int* key;
  int* val;
  long long size, cap;
} heap_t;

static int heap_less(const heap_t* h, long long a, long long b) {
  return h->key[a] < h->key[b] || (h->key[a] == h->key[b] && h->val[a] < h->val[b]);
}
static void heap_swap(heap_t* h, long long a, long long b) {
  int k = h->key[a], v = h->val[a];
  h->key[a] = h->key[b];
  h->val[a] = h->val[b];
  h->key[b] = k;
  h->val[b] = v;
}
static int heap_push(heap_t* h, int key, int val) {
  if (h->size == h->cap) {
    long long nc = h->cap ? 2 * h->cap : 1024;
    int* nk = (int*)realloc(h->key, (size_t)nc * sizeof(int));
    if (!nk) return -1;
    h->key = nk;
    int* nv = (int*)realloc(h->val, (size_t)nc * sizeof(int));
    if (!nv) return -1;
    h->val = nv;
    h->cap = nc;
  }
  long long i = h->size++;
  h->key[i] = key;
  h->val[i] = val;
  while (i > 0) {
    long long p = (i - 1) / 2;
    if (!heap_less(h, p, i)) break;
    heap_swap(h, p, i);
    i = p;
  }
  return 0;
}
static int heap_pop(heap_t* h) {
  int top = h->val[0];
  h->size--;
  if (h->size > 0) {
    h->key[0] = h->key[h->size];
    h->val[0] = h->val[h->size];
    long long i = 0;
    for (;;) {
      long long l = 2 * i + 1, r = l + 1, m = i;
      if (l < h->size && heap_less(h, m, l)) m = l;
      if (r < h->size && heap_less(h, m, r)) m = r;
      if (m == i) break;
      heap_swap(h, i, m);
      i = m;
    }
  }
  return top;
}

/* Label-correcting Dijkstra exactly as CPUserialDijkstra
 * (include/sssp_vertex_cpp.h:88-113; unit weights in include/bfs_vertex_cpp.h:52-77):
 * dist = maxval except src = 0, a max-heap of (-d, n) seeded with (0, src);
 * pop, relax every neighbour with the current dist of the popped vertex. */
static int dijkstra(int n, const int* nindex, const int* nlist, const int* w, int src, int* dist) {
  for (int i = 0; i < n; i++) dist[i] = OR_INF;
  dist[src] = 0;
  heap_t h = {0, 0, 0, 0};
  if (heap_push(&h, 0, src)) return -1;
  while (h.size > 0) {
    const int v = heap_pop(&h);
    const int dv = dist[v];
    for (int i = nindex[v]; i < nindex[v + 1]; i++) {
      const int nb = nlist[i];
      const int d = dv + (w ? w[i] : 1);
      if (d < dist[nb]) {
        dist[nb] = d;
        if (heap_push(&h, -d, nb)) {
          free(h.key);
          free(h.val);
          return -1;
        }
      }
    }
  }
  free(h.key);
  free(h.val);
  return 0;
}

int or_bfs_serial(int n, const int* nindex, const int* nlist, int src, int* dist) {
  return dijkstra(n, nindex, nlist, NULL, src, dist);
}

int or_sssp_serial(int n, const int* nindex, const int* nlist, const int* eweight, int src, int* dist) {
  return dijkstra(n, nindex, nlist, eweight, src, dist);
}

/* Min-label propagation to its fixed point, the topology-driven push of
 * codes/cpp/cc-cpp/CC_CPP_V_Topo_Push_IntType_ReadWrite_NonDeterm_NoBoundsBug_Block_Atomic.cpp:41-104
 * (label[v] = v, then a neighbour with a larger label takes v's label, until
 * no label changes).  Returns the number of rounds. */
int or_cc_serial(int n, const int* nindex, const int* nlist, int* label) {
  for (int v = 0; v < n; v++) label[v] = v;
  int iter = 0, goagain;
  do {
    iter++;
    goagain = 0;
    for (int v = 0; v < n; v++) {
      const int lv = label[v];
      for (int i = nindex[v]; i < nindex[v + 1]; i++) {
        const int d = nlist[i];
        if (label[d] > lv) {
          label[d] = lv;
          goagain = 1;
        }
      }
    }
  } while (goagain);
  return iter;
}

/* The reference priority hash (include/mis_vertex_cpp.h:135-140). */
unsigned int or_mis_hash(unsigned int val) {
  val = ((val >> 16) ^ val) * 0x45d9f3bu;
  val = ((val >> 16) ^ val) * 0x45d9f3bu;
  return (val >> 16) ^ val;
}

/* MIS rounds of codes/cpp/mis-cpp/MIS_CPP_V_Topo_Push_IntType_Atomic_CopyDeterm_Block.cpp:41-117:
 * priority[v] = hash(v + 712313887) (unsigned); an undecided v whose every
 * neighbour is excluded (previous round) or smaller in (priority, id) joins
 * the set in status_n and excludes its neighbours in status_n; status_n is
 * copied to status after each round.  status: 0 undecided, 1 in, 2 out.
 * Returns the number of rounds. */
int or_mis_serial(int n, const int* nindex, const int* nlist, unsigned char* status) {
  unsigned int* prio = (unsigned int*)malloc((size_t)n * sizeof(unsigned int));
  unsigned char* status_n = (unsigned char*)malloc((size_t)n);
  if (!prio || !status_n) {
    free(prio);
    free(status_n);
    return -1;
  }
  for (int v = 0; v < n; v++) {
    prio[v] = or_mis_hash((unsigned int)(v + 712313887));
    status[v] = 0;
    status_n[v] = 0;
  }
  int iter = 0, goagain;
  do {
    iter++;
    goagain = 0;
    for (int v = 0; v < n; v++) {
      if (status[v] != 0) continue;
      int i = nindex[v];
      while (i < nindex[v + 1] &&
             (status[nlist[i]] == 2 || prio[v] > prio[nlist[i]] || (prio[v] == prio[nlist[i]] && v > nlist[i])))
        i++;
      if (i < nindex[v + 1]) {
        goagain = 1;
      } else {
        status_n[v] = 1;
        for (int k = nindex[v]; k < nindex[v + 1]; k++) status_n[nlist[k]] = 2;
      }
    }
    memcpy(status, status_n, (size_t)n);
  } while (goagain);
  free(prio);
  free(status_n);
  return iter;
}

/* FP32 pull PageRank of codes/cpp/pr-cpp/PR_CPP_Pull_FloatType_Reduction_Block_Determin.cpp:41-89
 * with include/pr_cpp.h:45-47 constants as parameters: each iteration
 * contrib = score / degree, then score[i] = base + d * sum(contrib[nbr]) in
 * adjacency order (float), error += fabs(new - old) in double; stop when
 * error < epsilon or after max_iter iterations.  Returns the iteration count
 * as printed by the reference (:85-86). */
int or_pr_f32(int n, const int* nindex, const int* nlist, const int* degree, float* scores, float epsilon,
              int max_iter, float damp, double* residual) {
  const float base = (1.0f - damp) / (float)n;
  float* contrib = (float*)malloc((size_t)n * sizeof(float));
  if (!contrib) return -1;
  int iter;
  double error = 0;
  for (iter = 0; iter < max_iter; iter++) {
    error = 0;
    for (int i = 0; i < n; i++) contrib[i] = scores[i] / degree[i];
    for (int i = 0; i < n; i++) {
      float incoming = 0;
      for (int j = nindex[i]; j < nindex[i + 1]; j++) incoming += contrib[nlist[j]];
      const float old = scores[i];
      scores[i] = base + damp * incoming;
      error += fabs(scores[i] - old);
    }
    if (error < epsilon) break;
  }
  if (iter < max_iter) iter++;
  if (residual) *residual = error;
  free(contrib);
  return iter;
}

/* The same Jacobi iteration in FP64 (the accuracy reference): runs exactly
 * `iters` iterations when iters > 0, else until the L1 change < epsilon or
 * max_iter.  Returns the iterations run. */
int or_pr_f64(int n, const int* nindex, const int* nlist, const int* degree, double* scores, int iters,
              double epsilon, int max_iter, double damp, double* residual) {
  const double base = (1.0 - damp) / (double)n;
  double* contrib = (double*)malloc((size_t)n * sizeof(double));
  if (!contrib) return -1;
  const int limit = iters > 0 ? iters : max_iter;
  int it = 0;
  double error = 0;
  while (it < limit) {
    it++;
    error = 0;
    for (int i = 0; i < n; i++) contrib[i] = scores[i] / (double)degree[i];
    for (int i = 0; i < n; i++) {
      double incoming = 0;
      for (int j = nindex[i]; j < nindex[i + 1]; j++) incoming += contrib[nlist[j]];
      const double nw = base + damp * incoming;
      error += fabs(nw - scores[i]);
      scores[i] = nw;
    }
    if (iters <= 0 && error < epsilon) break;
  }
  if (residual) *residual = error;
  free(contrib);
  return it;
}

/* h_triCounting (include/tc_vertex_cpp.h:88-107) with h_common (:67-86) and a
 * 64-bit count: for v, every neighbour u > v, the common neighbours w > u. */
static long long common_count(int beg1, int end1, int beg2, int end2, const int* nlist) {
  long long common = 0;
  int pos1 = beg1, pos2 = beg2;
  while (pos1 < end1 && pos2 < end2) {
    while (pos1 < end1 && nlist[pos1] < nlist[pos2]) pos1++;
    if (pos1 < end1) {
      while (pos2 < end2 && nlist[pos2] < nlist[pos1]) pos2++;
      if (pos2 < end2 && nlist[pos1] == nlist[pos2]) {
        pos1++;
        pos2++;
        common++;
      } else {
        pos1++;
      }
    }
  }
  return common;
}

static long long tc_range(int v0, int v1, int stride, const int* nindex, const int* nlist) {
  long long count = 0;
  for (int v = v0; v < v1; v += stride) {
    const int beg1 = nindex[v], end1 = nindex[v + 1];
    int start1 = end1;
    while (beg1 < start1 && v < nlist[start1 - 1]) start1--;
    for (int j = start1; j < end1; j++) {
      const int u = nlist[j];
      const int beg2 = nindex[u], end2 = nindex[u + 1];
      int start2 = end2;
      while (beg2 < start2 && u < nlist[start2 - 1]) start2--;
      count += common_count(j + 1, end1, start2, end2, nlist);
    }
  }
  return count;
}

long long or_tc_serial(int n, const int* nindex, const int* nlist) { return tc_range(0, n, 1, nindex, nlist); }

/* TC precondition of include/tc_vertex_cpp.h (sorted, no self edge):
 * returns 1 when every list is strictly increasing. */
int or_check_sorted(int n, const int* nindex, const int* nlist) {
  for (int v = 0; v < n; v++)
    for (int i = nindex[v] + 1; i < nindex[v + 1]; i++)
      if (nlist[i - 1] >= nlist[i]) return 0;
  return 1;
}

/* ========================================================================
 * Threaded restatements of the best published C++ variants (the CPU
 * baseline).  Like the reference they spawn and join their threads every
 * iteration and split vertices in contiguous blocks (Block) or round robin
 * (Cyclic).  Each returns the seconds of its timed loop, as the reference's
 * gettimeofday pair does.
 * ====================================================================== */

typedef struct {
  int tid, nthreads;
  int n;
  const int* nindex;
  const int* nlist;
  const int* w;
  int* ia;
  int iter;
  int* goagain;
  unsigned char* st;
  const unsigned int* prio;
  const float* contrib;
  float* scores;
  float base, damp;
  double local_err;
  long long local_count;
} work_t;

static void run_threads(int T, work_t* ws, void* (*fn)(void*)) {
  pthread_t th[256];
  for (int t = 0; t < T; t++) pthread_create(&th[t], NULL, fn, &ws[t]);
  for (int t = 0; t < T; t++) pthread_join(th[t], NULL);
}

static void block_range(const work_t* w, int n, int* b, int* e) {
  *b = (int)((long long)w->tid * n / w->nthreads);
  *e = (int)((long long)(w->tid + 1) * n / w->nthreads);
}

/* codes/cpp/bfs-cpp/BFS_CPP_V_Topo_Push_IntType_ReadWrite_NoFieldBug_Block_Atomic_Determ_NoBoundsBug_NoRangeBug.cpp:41-106 */
static void* bfs_worker(void* p) {
  work_t* w = (work_t*)p;
  int b, e;
  block_range(w, w->n, &b, &e);
  for (int v = b; v < e; v++) {
    const int s = __atomic_load_n(&w->ia[v], __ATOMIC_RELAXED);
    if (s == w->iter) {
      int updated = 0;
      for (int i = w->nindex[v]; i < w->nindex[v + 1]; i++) {
        const int dst = w->nlist[i];
        const int nd = s + 1;
        if (__atomic_load_n(&w->ia[dst], __ATOMIC_RELAXED) > nd) {
          __atomic_store_n(&w->ia[dst], nd, __ATOMIC_RELAXED);
          updated = 1;
        }
      }
      if (updated) __atomic_store_n(w->goagain, 1, __ATOMIC_RELAXED);
    }
  }
  return NULL;
}

double or_bfs_threads(int n, const int* nindex, const int* nlist, int src, int* dist, int T) {
  if (T < 1 || T > 256) T = 1;
  for (int v = 0; v < n; v++) dist[v] = (v == src) ? 0 : OR_INF;
  work_t ws[256];
  int goagain;
  const double t0 = now_s();
  int iter = 0;
  do {
    goagain = 0;
    for (int t = 0; t < T; t++) {
      memset(&ws[t], 0, sizeof(work_t));
      ws[t].tid = t;
      ws[t].nthreads = T;
      ws[t].n = n;
      ws[t].nindex = nindex;
      ws[t].nlist = nlist;
      ws[t].ia = dist;
      ws[t].iter = iter;
      ws[t].goagain = &goagain;
    }
    run_threads(T, ws, bfs_worker);
    iter++;
  } while (goagain);
  return now_s() - t0;
}

static int atomic_min_int(int* addr, int val) {
  int old = __atomic_load_n(addr, __ATOMIC_RELAXED);
  while (old > val && !__atomic_compare_exchange_n(addr, &old, val, 1, __ATOMIC_RELAXED, __ATOMIC_RELAXED)) {
  }
  return old;
}

/* codes/cpp/sssp-cpp/SSSP_CPP_V_Topo_Push_IntType_ReadModifyWrite_NonDeterm_NoBoundsBug_Block_Atomic_NoRangeBug.cpp:41-105 */
static void* sssp_worker(void* p) {
  work_t* w = (work_t*)p;
  int b, e;
  block_range(w, w->n, &b, &e);
  for (int v = b; v < e; v++) {
    const int s = __atomic_load_n(&w->ia[v], __ATOMIC_RELAXED);
    if (s != OR_INF) {
      int updated = 0;
      for (int i = w->nindex[v]; i < w->nindex[v + 1]; i++) {
        const int nd = s + w->w[i];
        if (atomic_min_int(&w->ia[w->nlist[i]], nd) > nd) updated = 1;
      }
      if (updated) __atomic_store_n(w->goagain, 1, __ATOMIC_RELAXED);
    }
  }
  return NULL;
}

double or_sssp_threads(int n, const int* nindex, const int* nlist, const int* eweight, int src, int* dist, int T) {
  if (T < 1 || T > 256) T = 1;
  for (int v = 0; v < n; v++) dist[v] = (v == src) ? 0 : OR_INF;
  work_t ws[256];
  int goagain;
  const double t0 = now_s();
  do {
    goagain = 0;
    for (int t = 0; t < T; t++) {
      memset(&ws[t], 0, sizeof(work_t));
      ws[t].tid = t;
      ws[t].nthreads = T;
      ws[t].n = n;
      ws[t].nindex = nindex;
      ws[t].nlist = nlist;
      ws[t].w = eweight;
      ws[t].ia = dist;
      ws[t].goagain = &goagain;
    }
    run_threads(T, ws, sssp_worker);
  } while (goagain);
  return now_s() - t0;
}

/* codes/cpp/cc-cpp/CC_CPP_V_Topo_Push_IntType_ReadWrite_NonDeterm_NoBoundsBug_Block_Atomic.cpp:41-104 */
static void* cc_worker(void* p) {
  work_t* w = (work_t*)p;
  int b, e;
  block_range(w, w->n, &b, &e);
  for (int v = b; v < e; v++) {
    const int nl = __atomic_load_n(&w->ia[v], __ATOMIC_RELAXED);
    int updated = 0;
    for (int i = w->nindex[v]; i < w->nindex[v + 1]; i++) {
      const int dst = w->nlist[i];
      if (__atomic_load_n(&w->ia[dst], __ATOMIC_RELAXED) > nl) {
        __atomic_store_n(&w->ia[dst], nl, __ATOMIC_RELAXED);
        updated = 1;
      }
    }
    if (updated) __atomic_store_n(w->goagain, 1, __ATOMIC_RELAXED);
  }
  return NULL;
}

double or_cc_threads(int n, const int* nindex, const int* nlist, int* label, int T) {
  if (T < 1 || T > 256) T = 1;
  for (int v = 0; v < n; v++) label[v] = v;
  work_t ws[256];
  int goagain;
  const double t0 = now_s();
  do {
    goagain = 0;
    for (int t = 0; t < T; t++) {
      memset(&ws[t], 0, sizeof(work_t));
      ws[t].tid = t;
      ws[t].nthreads = T;
      ws[t].n = n;
      ws[t].nindex = nindex;
      ws[t].nlist = nlist;
      ws[t].ia = label;
      ws[t].goagain = &goagain;
    }
    run_threads(T, ws, cc_worker);
  } while (goagain);
  return now_s() - t0;
}

/* codes/cpp/mis-cpp/MIS_CPP_V_Topo_Push_IntType_Atomic_NonDeterm_Block.cpp:41-113 (in-place statuses) */
static void* mis_worker(void* p) {
  work_t* w = (work_t*)p;
  int b, e;
  block_range(w, w->n, &b, &e);
  const unsigned int* pr = w->prio;
  for (int v = b; v < e; v++) {
    if (__atomic_load_n(&w->st[v], __ATOMIC_RELAXED) == 0) {
      int i = w->nindex[v];
      while (i < w->nindex[v + 1] &&
             (__atomic_load_n(&w->st[w->nlist[i]], __ATOMIC_RELAXED) == 2 || pr[v] > pr[w->nlist[i]] ||
              (pr[v] == pr[w->nlist[i]] && v > w->nlist[i])))
        i++;
      if (i < w->nindex[v + 1]) {
        __atomic_store_n(w->goagain, 1, __ATOMIC_RELAXED);
      } else {
        __atomic_store_n(&w->st[v], (unsigned char)1, __ATOMIC_RELAXED);
        for (int k = w->nindex[v]; k < w->nindex[v + 1]; k++)
          __atomic_store_n(&w->st[w->nlist[k]], (unsigned char)2, __ATOMIC_RELAXED);
      }
    }
  }
  return NULL;
}

double or_mis_threads(int n, const int* nindex, const int* nlist, unsigned char* status, int T) {
  if (T < 1 || T > 256) T = 1;
  unsigned int* prio = (unsigned int*)malloc((size_t)n * sizeof(unsigned int));
  if (!prio) return -1;
  for (int v = 0; v < n; v++) {
    prio[v] = or_mis_hash((unsigned int)(v + 712313887));
    status[v] = 0;
  }
  work_t ws[256];
  int goagain;
  const double t0 = now_s();
  do {
    goagain = 0;
    for (int t = 0; t < T; t++) {
      memset(&ws[t], 0, sizeof(work_t));
      ws[t].tid = t;
      ws[t].nthreads = T;
      ws[t].n = n;
      ws[t].nindex = nindex;
      ws[t].nlist = nlist;
      ws[t].st = status;
      ws[t].prio = prio;
      ws[t].goagain = &goagain;
    }
    run_threads(T, ws, mis_worker);
  } while (goagain);
  const double el = now_s() - t0;
  free(prio);
  return el;
}

/* codes/cpp/pr-cpp/PR_CPP_Pull_FloatType_AtomicAdd_Block_Determin.cpp:41-87: contributions
 * computed on the calling thread, the pull sums by T threads over vertex
 * blocks, per-thread double errors added to the total. */
static void* pr_worker(void* p) {
  work_t* w = (work_t*)p;
  int b, e;
  block_range(w, w->n, &b, &e);
  double le = 0;
  for (int i = b; i < e; i++) {
    float incoming = 0;
    for (int j = w->nindex[i]; j < w->nindex[i + 1]; j++) incoming += w->contrib[w->nlist[j]];
    const float old = w->scores[i];
    w->scores[i] = w->base + w->damp * incoming;
    le += fabs(w->scores[i] - old);
  }
  w->local_err = le;
  return NULL;
}

double or_pr_threads(int n, const int* nindex, const int* nlist, const int* degree, float* scores, float epsilon,
                     int max_iter, float damp, int T, int* iterations) {
  if (T < 1 || T > 256) T = 1;
  const float base = (1.0f - damp) / (float)n;
  float* contrib = (float*)malloc((size_t)n * sizeof(float));
  if (!contrib) return -1;
  work_t ws[256];
  const double t0 = now_s();
  int iter;
  for (iter = 0; iter < max_iter; iter++) {
    double error = 0;
    for (int i = 0; i < n; i++) contrib[i] = scores[i] / degree[i];
    for (int t = 0; t < T; t++) {
      memset(&ws[t], 0, sizeof(work_t));
      ws[t].tid = t;
      ws[t].nthreads = T;
      ws[t].n = n;
      ws[t].nindex = nindex;
      ws[t].nlist = nlist;
      ws[t].contrib = contrib;
      ws[t].scores = scores;
      ws[t].base = base;
      ws[t].damp = damp;
    }
    run_threads(T, ws, pr_worker);
    for (int t = 0; t < T; t++) error += ws[t].local_err;
    if (error < epsilon) break;
  }
  const double el = now_s() - t0;
  if (iter < max_iter) iter++;
  if (iterations) *iterations = iter;
  free(contrib);
  return el;
}

/* codes/cpp/tc-cpp/TC_CPP_V_IntType_Critical_Cyclic.cpp:44-87 with a 64-bit count: vertices
 * dealt round robin, per-thread counts added under a lock. */
static pthread_mutex_t tc_mu = PTHREAD_MUTEX_INITIALIZER;
static long long tc_total;
static void* tc_worker(void* p) {
  work_t* w = (work_t*)p;
  const long long c = tc_range(w->tid, w->n, w->nthreads, w->nindex, w->nlist);
  pthread_mutex_lock(&tc_mu);
  tc_total += c;
  pthread_mutex_unlock(&tc_mu);
  return NULL;
}

double or_tc_threads(int n, const int* nindex, const int* nlist, long long* count, int T) {
  if (T < 1 || T > 256) T = 1;
  work_t ws[256];
  for (int t = 0; t < T; t++) {
    memset(&ws[t], 0, sizeof(work_t));
    ws[t].tid = t;
    ws[t].nthreads = T;
    ws[t].n = n;
    ws[t].nindex = nindex;
    ws[t].nlist = nlist;
  }
  tc_total = 0;
  const double t0 = now_s();
  run_threads(T, ws, tc_worker);
  const double el = now_s() - t0;
  *count = tc_total;
  return el;
}

/* or_pr_f64 with the pull sums spread over T threads (vertex blocks).  Each
 * vertex's sum runs in adjacency order as in or_pr_f64, so with iters > 0
 * the scores are the same bits; only the residual is summed per thread
 * first.  For checks at large sizes. */
typedef struct {
  int b, e;
  const int *nindex, *nlist;
  const double* contrib;
  double* scores;
  double base, damp, err;
} pr64_work_t;

static void* pr64_worker(void* p) {
  pr64_work_t* w = (pr64_work_t*)p;
  double le = 0;
  for (int i = w->b; i < w->e; i++) {
    double incoming = 0;
    for (int j = w->nindex[i]; j < w->nindex[i + 1]; j++) incoming += w->contrib[w->nlist[j]];
    const double nw = w->base + w->damp * incoming;
    le += fabs(nw - w->scores[i]);
    w->scores[i] = nw;
  }
  w->err = le;
  return NULL;
}

int or_pr_f64_threads(int n, const int* nindex, const int* nlist, const int* degree, double* scores, int iters,
                      double epsilon, int max_iter, double damp, int T, double* residual) {
  if (T < 1 || T > 256) T = 1;
  const double base = (1.0 - damp) / (double)n;
  double* contrib = (double*)malloc((size_t)n * sizeof(double));
  if (!contrib) return -1;
  pr64_work_t ws[256];
  pthread_t th[256];
  const int limit = iters > 0 ? iters : max_iter;
  int it = 0;
  double error = 0;
  while (it < limit) {
    it++;
    for (int i = 0; i < n; i++) contrib[i] = scores[i] / (double)degree[i];
    for (int t = 0; t < T; t++) {
      ws[t].b = (int)((long long)t * n / T);
      ws[t].e = (int)((long long)(t + 1) * n / T);
      ws[t].nindex = nindex;
      ws[t].nlist = nlist;
      ws[t].contrib = contrib;
      ws[t].scores = scores;
      ws[t].base = base;
      ws[t].damp = damp;
      pthread_create(&th[t], NULL, pr64_worker, &ws[t]);
    }
    error = 0;
    for (int t = 0; t < T; t++) {
      pthread_join(th[t], NULL);
      error += ws[t].err;
    }
    if (iters <= 0 && error < epsilon) break;
  }
  if (residual) *residual = error;
  free(contrib);
  return it;
}
