// Served form: single-source BFS and SSSP queries against a resident graph,
// answered by 64-lane multi-source traversals with continuous batching.
//
// Engines (one per query kind), each with 64 lanes; a lane holds one query:
//   BFS : per vertex a 64-bit visited mask and a 64-bit frontier mask.  One
//         step expands every vertex whose frontier mask is non-zero (all its
//         lanes at once) with 64-bit atomicOr into `next` (vertices above the
//         hub degree edge-balanced over the grid), then a finalize pass moves
//         the new bits into `visited`, counts them per lane, adds their
//         distance to the lane's sum and records target hits.  A lane's BFS
//         levels count from the step it was admitted in.
//   SSSP: per vertex 64 int32 distances (lane-contiguous rows) and a 64-bit
//         changed mask.  One round relaxes the out-edges of every vertex with
//         changed lanes, for those lanes only (Bellman-Ford rounds); a warp
//         step takes 32 independent (edge, changed lane) pairs.
// A lane retires when a step adds nothing for it; its results are read, its
// state cleared, and the lane admits the next pending query at the following
// step boundary, while the other lanes keep going (continuous batching).
// A worker thread owns the device work; clients submit and wait.
//
// Admission by device memory: an engine's state is allocated when a query of
// its kind is pending and the device's free memory (less an eighth kept in
// reserve) and the server's budget (ig_server_set_memory_budget) both cover
// it.  Otherwise the query stays pending -- deferred, not failed -- and is
// admitted when memory frees up: when the other engine falls idle it is
// released to make room, and the worker retries each millisecond.  A query
// whose engine can never fit the budget or the device fails with
// IG_ERR_NOMEM.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "ig_device.cuh"
#include "ig_options.h"

namespace {

constexpr int kLanes = 64;
constexpr int kMaxTargets = 16;
constexpr int kThreads = 256;
typedef unsigned long long u64;

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// ---------------------------------------------------------------- BFS kernels
struct BfsLaneState {
  int target[kLanes][kMaxTargets];   // -1 unused
  int tdist[kLanes][kMaxTargets];    // INT_MAX until hit
  int start[kLanes];                 // step at which the lane was admitted
  unsigned long long cnt[kLanes];    // vertices added by the current step
  unsigned long long sum[kLanes];    // sum of distances
  unsigned long long reach[kLanes];  // vertices reached (source excluded)
};

__device__ __forceinline__ void record_targets(BfsLaneState* st, const u64* is_target, int w, u64 nw, int dist_of_lane_base) {
  u64 h = nw & is_target[w];
  while (h) {
    const int q = __ffsll((long long)h) - 1;
    h &= h - 1;
    for (int t = 0; t < kMaxTargets; t++)
      if (st->target[q][t] == w) st->tdist[q][t] = dist_of_lane_base - st->start[q];
  }
}

// top-down expansion of the frontier list
__global__ void __launch_bounds__(kThreads) msbfs_expand(const int* __restrict__ nindex, const int* __restrict__ nlist,
                                                         int n, const int* flist, int fsize, const u64* fmask,
                                                         const u64* visited, u64* next, int* tlist, int* tsize,
                                                         int* hubs, int* nhub, int hub_degree, IgCtl* ctl) {
  using namespace ig;
  const int lane = lane_id();
  const long long gtid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long gthreads = (long long)gridDim.x * blockDim.x;
  auto visit = [&](bool act, int e, u64 f) {
    bool push = false;
    int w = 0;
    if (act && f) {
      w = __ldg(&nlist[e]);
      const u64 nv = f & ~visited[w];
      if (nv) push = atomicOr(&next[w], nv) == 0ull;
    }
    warp_append(push, w, tlist, tsize, n, ctl);
  };
  for (long long base = gtid & ~31LL; base < fsize; base += gthreads) {
    const long long i = base + lane;
    int u = 0, beg = 0, deg = 0;
    u64 f = 0;
    if (i < fsize) {
      u = flist[i];
      f = fmask[u];
      beg = __ldg(&nindex[u]);
      deg = __ldg(&nindex[u + 1]) - beg;
    }
    const bool hub = deg > hub_degree;
    warp_append(hub, u, hubs, nhub, n, ctl);
    warp_expand(beg, hub ? 0 : deg, [&](bool act, int e, int j) {
      const u64 fj = __shfl_sync(IG_FULL, f, j);
      visit(act, e, fj);
    });
  }
}

__global__ void __launch_bounds__(kThreads) msbfs_expand_hubs(const int* __restrict__ nindex,
                                                              const int* __restrict__ nlist, int n, const u64* fmask,
                                                              const u64* visited, u64* next, int* tlist, int* tsize,
                                                              const int* hubs, const int* nhub, IgCtl* ctl) {
  using namespace ig;
  const int nh = *nhub;
  if (nh == 0) return;
  grid_expand_hubs(nindex, hubs, nh, [&](bool act, int e, int hv) {
    bool push = false;
    int w = 0;
    if (act) {
      const u64 f = fmask[hv];
      w = __ldg(&nlist[e]);
      const u64 nv = f & ~visited[w];
      if (nv) push = atomicOr(&next[w], nv) == 0ull;
    }
    warp_append(push, w, tlist, tsize, n, ctl);
  });
}

// Clears the frontier masks of the expanded list (before the new ones are set).
__global__ void msbfs_clear_frontier(const int* flist, int fsize, u64* fmask) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < fsize; i += gridDim.x * blockDim.x) fmask[flist[i]] = 0;
}

// New bits become visited and the next frontier; per-lane counts and sums.
__global__ void __launch_bounds__(kThreads) msbfs_finalize(const int* tlist, int tsize, u64* next, u64* visited,
                                                           u64* fmask, const u64* is_target, BfsLaneState* st,
                                                           int step) {
  __shared__ unsigned s_cnt[kLanes];
  for (int q = threadIdx.x; q < kLanes; q += blockDim.x) s_cnt[q] = 0;
  __syncthreads();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < tsize; i += gridDim.x * blockDim.x) {
    const int w = tlist[i];
    const u64 nw = next[w] & ~visited[w];
    next[w] = 0;
    if (!nw) continue;
    visited[w] |= nw;
    fmask[w] = nw;
    u64 m = nw;
    while (m) {
      const int q = __ffsll((long long)m) - 1;
      m &= m - 1;
      atomicAdd(&s_cnt[q], 1u);
    }
    record_targets(st, is_target, w, nw, step + 1);
  }
  __syncthreads();
  for (int q = threadIdx.x; q < kLanes; q += blockDim.x) {
    if (s_cnt[q]) {
      atomicAdd(&st->cnt[q], (u64)s_cnt[q]);
      atomicAdd(&st->reach[q], (u64)s_cnt[q]);
      atomicAdd(&st->sum[q], (u64)s_cnt[q] * (u64)(step + 1 - st->start[q]));
    }
  }
}

// Admission: sources get their lane bit in visited and frontier; they are
// appended to the frontier list if not already in it.
__global__ void msbfs_admit(const int* srcs, const int* lanes, int count, u64* visited, u64* fmask, int* flist,
                            int* fsize, u64* is_target, BfsLaneState* st, int step) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  for (int k = 0; k < count; k++) {
    const int s = srcs[k], q = lanes[k];
    const u64 bit = 1ull << q;
    st->start[q] = step;
    if (fmask[s] == 0) flist[(*fsize)++] = s;
    visited[s] |= bit;
    fmask[s] |= bit;
    for (int t = 0; t < kMaxTargets; t++) {
      const int w = st->target[q][t];
      if (w >= 0) {
        is_target[w] |= bit;
        if (w == s) st->tdist[q][t] = 0;
      }
    }
  }
}

// Retirement: clear the lanes' bits everywhere.
__global__ void msbfs_retire(int n, u64 lanes, u64* visited, u64* fmask, u64* is_target) {
  const u64 keep = ~lanes;
  for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (long long)gridDim.x * blockDim.x) {
    visited[v] &= keep;
    fmask[v] &= keep;
    is_target[v] &= keep;
  }
}

// --------------------------------------------------------------- SSSP kernels
struct SsspLaneState {
  int target[kLanes][kMaxTargets];
  unsigned long long reached[kLanes];
  unsigned long long sum[kLanes];
  long long maxd[kLanes];
  unsigned long long cnt[kLanes];  // non-zero if the lane improved a distance in the last round
};

// Position of the r-th set bit (r counted from 0) of a 64-bit mask.
__device__ __forceinline__ int nth_set_bit(u64 m, int r) {
  unsigned x = (unsigned)m;
  int pos = 0;
  const int c0 = __popc(x);
  if (r >= c0) {
    r -= c0;
    x = (unsigned)(m >> 32);
    pos = 32;
  }
#pragma unroll
  for (int width = 16; width >= 1; width >>= 1) {
    const int c = __popc(x & ((1u << width) - 1u));
    if (r >= c) {
      r -= c;
      x >>= width;
      pos += width;
    }
  }
  return pos;
}

// One round: for every vertex u with changed lanes, relax its out-edges for
// those lanes.  The work is the (edge, changed lane) pairs: a vertex with k
// changed lanes gives each warp step 32 / k of its edges, so a vertex that
// changed in one or two lanes does not leave the warp idle, and the 32 pairs
// of a step are independent (their loads and atomics overlap).  Frontier
// vertices are dealt to warps in edge-balanced chunks: a warp owns
// `kEdgeChunk` consecutive edges of the concatenated frontier lists (prefix in
// eoff).  A vertex first changed in this round is appended to tlist through
// the warp's shared-memory buffer.
constexpr int kEdgeChunk = 64;

__global__ void __launch_bounds__(kThreads) msssp_round(const int* __restrict__ nindex, const int* __restrict__ nlist,
                                                        const int* __restrict__ eweight, int n, const int* flist,
                                                        int fsize, const int* eoff, const u64* changed,
                                                        u64* changed_next, int* dist, int* tlist, int* tsize,
                                                        SsspLaneState* st, IgCtl* ctl) {
  using namespace ig;
  __shared__ int s_buf[kThreads / 32][kWarpBuf];
  int* buf = s_buf[threadIdx.x >> 5];
  int nbuf = 0;
  const int lane = lane_id();
  const int warp_g = (int)(((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int nwarps = (int)(((long long)gridDim.x * blockDim.x) >> 5);
  const long long total = eoff[fsize];
  u64 imp_lanes = 0;  // source lanes this thread improved
  for (long long c0 = (long long)warp_g * kEdgeChunk; c0 < total; c0 += (long long)nwarps * kEdgeChunk) {
    const long long c1 = min(c0 + kEdgeChunk, total);
    // owner of c0: largest i with eoff[i] <= c0
    int lo = 0, hi = fsize - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (eoff[mid] <= c0) lo = mid;
      else hi = mid - 1;
    }
    int fi = lo;
    long long k = c0;
    while (k < c1) {  // one frontier vertex's part of the chunk at a time (warp-uniform)
      while (k >= eoff[fi + 1]) fi++;
      const int u = flist[fi];
      const long long s1 = min(c1, (long long)eoff[fi + 1]);
      const int ubeg = __ldg(&nindex[u]) + (int)(k - eoff[fi]);
      const u64 cm = changed[u];
      const int kl = __popcll(cm);
      const int pairs = (int)(s1 - k) * kl;
      for (int pb = 0; pb < pairs; pb += 32) {
        const int p = pb + lane;
        int item[1] = {0};
        int na = 0;
        if (p < pairs) {
          const int eo = p / kl;
          const int q = nth_set_bit(cm, p - eo * kl);
          const int du = dist[(long long)u * kLanes + q];
          if (du != kInf) {
            const int e = ubeg + eo;
            const int v = __ldg(&nlist[e]);
            const long long nd = (long long)du + __ldg(&eweight[e]);
            int* pv = &dist[(long long)v * kLanes + q];
            if (nd < *pv && atomicMin(pv, (int)nd) > (int)nd) {
              imp_lanes |= 1ull << q;
              if (atomicOr(&changed_next[v], 1ull << q) == 0ull) {
                item[0] = v;
                na = 1;
              }
            }
          }
        }
        warp_buf_append<1>(na, item, buf, nbuf, tlist, tsize, n, ctl);
      }
      k = s1;
    }
  }
  warp_buf_flush(buf, nbuf, tlist, tsize, n, ctl);
  // a lane that improved nothing this round is finished
  const unsigned lo_m = __reduce_or_sync(IG_FULL, (unsigned)imp_lanes);
  const unsigned hi_m = __reduce_or_sync(IG_FULL, (unsigned)(imp_lanes >> 32));
  if ((lo_m >> lane) & 1u) atomicAdd(&st->cnt[lane], 1ull);
  if ((hi_m >> lane) & 1u) atomicAdd(&st->cnt[32 + lane], 1ull);
}

// Degree prefix of the frontier (for the edge-balanced round).
__global__ void msssp_degrees(const int* __restrict__ nindex, const int* flist, int fsize, int* deg) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < fsize; i += gridDim.x * blockDim.x) {
    const int u = flist[i];
    deg[i] = __ldg(&nindex[u + 1]) - __ldg(&nindex[u]);
  }
}
// After a round: the next changed masks become current (vertices of tlist);
// the old frontier's masks are cleared first.
__global__ void msssp_clear(const int* flist, int fsize, u64* changed) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < fsize; i += gridDim.x * blockDim.x) changed[flist[i]] = 0;
}
__global__ void msssp_promote(const int* tlist, int tsize, u64* changed_next, u64* changed) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < tsize; i += gridDim.x * blockDim.x) {
    const int v = tlist[i];
    changed[v] = changed_next[v];
    changed_next[v] = 0;
  }
}

__global__ void msssp_admit(const int* srcs, const int* lanes, int count, int* dist, u64* changed, int* flist,
                            int* fsize) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  for (int k = 0; k < count; k++) {
    const int s = srcs[k], q = lanes[k];
    dist[(long long)s * kLanes + q] = 0;
    if (changed[s] == 0) flist[(*fsize)++] = s;
    changed[s] |= 1ull << q;
  }
}

// Retirement of a set of lanes: reached count, max and sum of the finite
// distances, target distances; then the lanes' distances are reset to INF.
__global__ void __launch_bounds__(kThreads) msssp_retire(int n, u64 lanes, int* dist, SsspLaneState* st,
                                                         int* tdist /* [64][16] */) {
  __shared__ unsigned long long s_reach[kLanes], s_sum[kLanes];
  __shared__ long long s_max[kLanes];
  for (int q = threadIdx.x; q < kLanes; q += blockDim.x) {
    s_reach[q] = 0;
    s_sum[q] = 0;
    s_max[q] = 0;
  }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const long long wg = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
  unsigned long long r0 = 0, r1 = 0, s0 = 0, s1 = 0;
  long long m0 = 0, m1 = 0;
  const bool on0 = (lanes >> lane) & 1ull, on1 = (lanes >> (32 + lane)) & 1ull;
  for (long long v = wg; v < n; v += nw) {
    int* row = dist + v * kLanes;
    if (on0) {
      const int d = row[lane];
      if (d != ig::kInf) {
        r0++;
        s0 += (unsigned long long)d;
        m0 = max(m0, (long long)d);
        row[lane] = ig::kInf;
      }
    }
    if (on1) {
      const int d = row[32 + lane];
      if (d != ig::kInf) {
        r1++;
        s1 += (unsigned long long)d;
        m1 = max(m1, (long long)d);
        row[32 + lane] = ig::kInf;
      }
    }
  }
  if (on0) {
    atomicAdd(&s_reach[lane], r0);
    atomicAdd(&s_sum[lane], s0);
    atomicMax(&s_max[lane], m0);
  }
  if (on1) {
    atomicAdd(&s_reach[32 + lane], r1);
    atomicAdd(&s_sum[32 + lane], s1);
    atomicMax(&s_max[32 + lane], m1);
  }
  __syncthreads();
  for (int q = threadIdx.x; q < kLanes; q += blockDim.x) {
    if ((lanes >> q) & 1ull) {
      atomicAdd(&st->reached[q], s_reach[q]);
      atomicAdd(&st->sum[q], s_sum[q]);
      atomicMax(&st->maxd[q], s_max[q]);
    }
  }
}

// Target distances are read before the reset (one thread per lane/target).
__global__ void msssp_targets(const int* dist, u64 lanes, const SsspLaneState* st, int* tdist) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= kLanes * kMaxTargets) return;
  const int q = i / kMaxTargets, t = i % kMaxTargets;
  if (!((lanes >> q) & 1ull)) return;
  const int w = st->target[q][t];
  tdist[i] = w >= 0 ? dist[(long long)w * kLanes + q] : ig::kInf;
}

__global__ void fill_int(int* p, long long n, int v) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    p[i] = v;
}

}  // namespace

// ============================================================ host runtime
struct Request {
  long long ticket;
  int kind, source, ntargets;
  int targets[kMaxTargets];
  double submit_t, admit_t = 0;
  bool cancelled = false;
};

struct Engine {
  int kind;                       // 0 BFS, 1 SSSP
  bool live = false;              // state allocated
  Request* lane_req[kLanes] = {};
  u64 busy = 0;                   // lanes holding a query
  int step = 0;
  int fsize = 0;                  // host copy of the frontier size
  // device buffers
  int *flist = nullptr, *tlist = nullptr, *hubs = nullptr, *d_small = nullptr;  // d_small: [0]=tsize [1]=nhub [2]=fsize
  int* d_admit = nullptr;         // [2 * 64]: sources then lanes
  u64 *a = nullptr, *b = nullptr, *c = nullptr;  // BFS: visited, fmask, next / SSSP: changed, changed_next, -
  u64* is_target = nullptr;
  int* dist = nullptr;            // SSSP rows
  int* deg = nullptr;
  int* eoff = nullptr;
  void* lane_state = nullptr;     // BfsLaneState / SsspLaneState
  int* tdist = nullptr;           // SSSP [64][16]
};

struct ig_server {
  ig_csr g;
  int device = 0, sms = 0;
  int max_pending = 0;
  cudaStream_t stream = nullptr;
  IgCtl* d_ctl = nullptr;
  IgScratch scratch;   // device-wide scan tiles
  IgExec ex;
  Engine eng[2];
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Request*> pending[2];
  std::unordered_map<long long, std::pair<Request*, ig_query_result>> done;
  long long next_ticket = 1;
  long long completed = 0, steps = 0;
  bool stop = false;
  int worker_rc = IG_OK;
  std::thread worker;
  long long budget = -1;          // bytes the engines may hold together (-1: no cap)
  long long deferrals = 0;        // admission attempts that found too little memory
  long long engines_created = 0;
};

// Device bytes of one engine's state (engine_alloc's allocations).
static long long engine_bytes(const ig_server* s, int kind) {
  const long long n = s->g.nodes, vb = n * (long long)sizeof(int), mb = n * (long long)sizeof(u64);
  long long b = 3 * vb + 64 + 2 * kLanes * sizeof(int) + 2 * mb;
  if (kind == 0) b += 2 * mb + (long long)sizeof(BfsLaneState);
  else b += n * kLanes * (long long)sizeof(int) + vb + vb + sizeof(int) + (long long)sizeof(SsspLaneState) +
            kLanes * kMaxTargets * (long long)sizeof(int);
  return b;
}

static int scuda(int e, const char* what) { return ig_cuda_check(e, what); }

static int engine_alloc(ig_server* s, Engine& E, int kind) {
  E.live = true;
  const int n = s->g.nodes;
  const size_t vb = (size_t)n * sizeof(int), mb = (size_t)n * sizeof(u64);
  E.kind = kind;
  int rc = IG_OK;
  auto al = [&](void** p, size_t bytes) {
    if (!rc) rc = scuda(cudaMalloc(p, std::max<size_t>(bytes, 256)), "server allocation");
  };
  al((void**)&E.flist, vb);
  al((void**)&E.tlist, vb);
  al((void**)&E.hubs, vb);
  al((void**)&E.d_small, 64);
  al((void**)&E.d_admit, 2 * kLanes * sizeof(int));
  al((void**)&E.a, mb);
  al((void**)&E.b, mb);
  if (kind == 0) {
    al((void**)&E.c, mb);
    al((void**)&E.is_target, mb);
    al(&E.lane_state, sizeof(BfsLaneState));
  } else {
    al((void**)&E.dist, (size_t)n * kLanes * sizeof(int));
    al((void**)&E.deg, vb);
    al((void**)&E.eoff, ((size_t)n + 1) * sizeof(int));
    al(&E.lane_state, sizeof(SsspLaneState));
    al((void**)&E.tdist, kLanes * kMaxTargets * sizeof(int));
  }
  if (rc) return rc;
  if (!rc) rc = scuda(cudaMemsetAsync(E.a, 0, mb, s->stream), "memset");
  if (!rc) rc = scuda(cudaMemsetAsync(E.b, 0, mb, s->stream), "memset");
  if (!rc) rc = scuda(cudaMemsetAsync(E.d_small, 0, 64, s->stream), "memset");
  if (kind == 0) {
    if (!rc) rc = scuda(cudaMemsetAsync(E.c, 0, mb, s->stream), "memset");
    if (!rc) rc = scuda(cudaMemsetAsync(E.is_target, 0, mb, s->stream), "memset");
    if (!rc) rc = scuda(cudaMemsetAsync(E.lane_state, 0, sizeof(BfsLaneState), s->stream), "memset");
  } else {
    fill_int<<<s->sms * 8, kThreads, 0, s->stream>>>(E.dist, (long long)n * kLanes, ig::kInf);
    if (!rc) rc = scuda(cudaMemsetAsync(E.lane_state, 0, sizeof(SsspLaneState), s->stream), "memset");
  }
  return rc;
}

static void engine_free(Engine& E) {
  void* ps[] = {E.flist, E.tlist, E.hubs, E.d_small, E.d_admit, E.a, E.b, E.c, E.is_target, E.dist,
                E.deg, E.eoff, E.lane_state, E.tdist};
  for (void* p : ps)
    if (p) cudaFree(p);
  const int kind = E.kind;
  E = Engine();
  E.kind = kind;
}

static void complete(ig_server* s, Request* r, const ig_query_result& res);

// Makes engine k's state resident for its pending queries.  Returns IG_OK
// when it is (or became) resident, IG_ERR_BUSY when the memory is short for
// now (the queries stay pending), another status on a CUDA error.  Queries
// whose engine can never fit fail with IG_ERR_NOMEM.
static int engine_ensure(ig_server* s, int k) {
  Engine& E = s->eng[k];
  if (E.live) return IG_OK;
  const long long need = engine_bytes(s, k);
  size_t free_b = 0, total_b = 0;
  int rc = scuda(cudaMemGetInfo(&free_b, &total_b), "cudaMemGetInfo");
  if (rc) return rc;
  long long budget;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    budget = s->budget;
  }
  const long long cap = budget >= 0 ? std::min<long long>(budget, (long long)total_b) : (long long)total_b;
  if (need + (need >> 3) > cap) {  // never fits: fail this kind's pending queries
    std::vector<Request*> drop;
    {
      std::lock_guard<std::mutex> lk(s->mu);
      drop.assign(s->pending[k].begin(), s->pending[k].end());
      s->pending[k].clear();
    }
    for (Request* r : drop) {
      ig_query_result res;
      memset(&res, 0, sizeof(res));
      res.status = IG_ERR_NOMEM;
      res.kind = r->kind;
      res.source = r->source;
      res.submit_time = r->submit_t;
      res.done_time = now_s();
      complete(s, r, res);
    }
    return IG_ERR_BUSY;
  }
  Engine& O = s->eng[1 - k];
  auto fits = [&](long long free_now) {
    const long long held = O.live ? engine_bytes(s, 1 - k) : 0;
    return need + (need >> 3) <= free_now && (budget < 0 || held + need <= budget);
  };
  if (!fits((long long)free_b)) {
    bool other_idle;
    {
      std::lock_guard<std::mutex> lk(s->mu);
      other_idle = O.live && O.busy == 0 && s->pending[1 - k].empty();
    }
    if (other_idle) {  // release the idle engine to make room
      if ((rc = scuda(cudaStreamSynchronize(s->stream), "sync"))) return rc;
      engine_free(O);
      if ((rc = scuda(cudaMemGetInfo(&free_b, &total_b), "cudaMemGetInfo"))) return rc;
    }
    if (!fits((long long)free_b)) {
      std::lock_guard<std::mutex> lk(s->mu);
      s->deferrals++;
      return IG_ERR_BUSY;
    }
  }
  if ((rc = engine_alloc(s, E, k))) {
    engine_free(E);
    return rc;
  }
  std::lock_guard<std::mutex> lk(s->mu);
  s->engines_created++;
  return IG_OK;
}

static void complete(ig_server* s, Request* r, const ig_query_result& res) {
  std::lock_guard<std::mutex> lk(s->mu);
  s->done[r->ticket] = {r, res};
  s->completed++;
  s->cv_done.notify_all();
}

// Admits pending queries of kind E.kind into free lanes (host side chooses,
// a one-thread kernel applies).
static int engine_admit(ig_server* s, Engine& E) {
  std::vector<Request*> in;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    auto& q = s->pending[E.kind];
    while (!q.empty() && E.busy != ~0ull) {
      Request* r = q.front();
      q.pop_front();
      if (r->cancelled) continue;
      int lane = __builtin_ctzll(~E.busy);
      E.busy |= 1ull << lane;
      E.lane_req[lane] = r;
      in.push_back(r);
    }
  }
  if (in.empty()) return IG_OK;
  int host[2 * kLanes];
  const double t = now_s();
  const int cnt = (int)in.size();
  for (int k = 0; k < cnt; k++) {
    Request* r = in[k];
    r->admit_t = t;
    int lane = -1;
    for (int q = 0; q < kLanes; q++)
      if (E.lane_req[q] == r) lane = q;
    host[k] = r->source;
    host[kLanes + k] = lane;
    // per-lane targets
    int tg[kMaxTargets];
    for (int j = 0; j < kMaxTargets; j++) tg[j] = j < r->ntargets ? r->targets[j] : -1;
    const size_t off = E.kind == 0 ? offsetof(BfsLaneState, target) : offsetof(SsspLaneState, target);
    int rc = scuda(cudaMemcpy((char*)E.lane_state + off + (size_t)lane * kMaxTargets * sizeof(int), tg, sizeof(tg),
                              cudaMemcpyHostToDevice),
                   "targets");
    if (rc) return rc;
    if (E.kind == 0) {
      int inf[kMaxTargets];
      for (int j = 0; j < kMaxTargets; j++) inf[j] = ig::kInf;
      rc = scuda(cudaMemcpy((char*)E.lane_state + offsetof(BfsLaneState, tdist) +
                                (size_t)lane * kMaxTargets * sizeof(int),
                            inf, sizeof(inf), cudaMemcpyHostToDevice),
                 "tdist");
      if (rc) return rc;
    }
    // copy to device before the host array goes out of scope: synchronous copies per admission batch
  }
  int rc = scuda(cudaMemcpyAsync(E.d_admit, host, sizeof(host), cudaMemcpyHostToDevice, s->stream), "admit copy");
  if (rc) return rc;
  // the frontier size lives in d_small[2]
  if (E.kind == 0)
    msbfs_admit<<<1, 32, 0, s->stream>>>(E.d_admit, E.d_admit + kLanes, cnt, E.a, E.b, E.flist, E.d_small + 2,
                                         E.is_target, (BfsLaneState*)E.lane_state, E.step);
  else
    msssp_admit<<<1, 32, 0, s->stream>>>(E.d_admit, E.d_admit + kLanes, cnt, E.dist, E.a, E.flist, E.d_small + 2);
  ig_count_launches(1);
  // the host stack arrays above are consumed by the copies before returning
  return scuda(cudaStreamSynchronize(s->stream), "admit sync");
}

// One BFS step for all busy lanes; retires lanes whose frontier emptied.
static int bfs_step(ig_server* s, Engine& E) {
  const int n = s->g.nodes;
  int small[3];
  int rc = scuda(cudaMemcpyAsync(small, E.d_small, sizeof(small), cudaMemcpyDeviceToHost, s->stream), "read");
  if (!rc) rc = scuda(cudaStreamSynchronize(s->stream), "sync");
  if (rc) return rc;
  const int fsize = small[2];
  // reset tsize / nhub, zero per-step counts
  if ((rc = scuda(cudaMemsetAsync(E.d_small, 0, 2 * sizeof(int), s->stream), "memset"))) return rc;
  if ((rc = scuda(cudaMemsetAsync((char*)E.lane_state + offsetof(BfsLaneState, cnt), 0, kLanes * sizeof(u64),
                                  s->stream),
                  "memset")))
    return rc;
  const int grid = s->sms * 8;
  msbfs_expand<<<grid, kThreads, 0, s->stream>>>(s->g.nindex, s->g.nlist, n, E.flist, fsize, E.b, E.a, E.c, E.tlist,
                                                 E.d_small, E.hubs, E.d_small + 1, ig_options().hub_degree, s->d_ctl);
  msbfs_expand_hubs<<<grid, kThreads, 0, s->stream>>>(s->g.nindex, s->g.nlist, n, E.b, E.a, E.c, E.tlist, E.d_small,
                                                      E.hubs, E.d_small + 1, s->d_ctl);
  msbfs_clear_frontier<<<grid, kThreads, 0, s->stream>>>(E.flist, fsize, E.b);
  // tsize is only known on the device: finalize over the worst case with a guard read
  int tsize = 0;
  if ((rc = scuda(cudaMemcpyAsync(&tsize, E.d_small, sizeof(int), cudaMemcpyDeviceToHost, s->stream), "read")) ||
      (rc = scuda(cudaStreamSynchronize(s->stream), "sync")))
    return rc;
  msbfs_finalize<<<std::max(1, std::min(grid, (tsize + kThreads - 1) / kThreads)), kThreads, 0, s->stream>>>(
      E.tlist, tsize, E.c, E.a, E.b, E.is_target, (BfsLaneState*)E.lane_state, E.step);
  ig_count_launches(4);
  std::swap(E.flist, E.tlist);
  const int nf = tsize;
  if ((rc = scuda(cudaMemcpyAsync(E.d_small + 2, &nf, sizeof(int), cudaMemcpyHostToDevice, s->stream), "write")))
    return rc;
  E.step++;
  // read per-lane counts; lanes that added nothing are finished
  BfsLaneState h;
  if ((rc = scuda(cudaMemcpyAsync(&h, E.lane_state, sizeof(h), cudaMemcpyDeviceToHost, s->stream), "read")) ||
      (rc = scuda(cudaStreamSynchronize(s->stream), "sync")))
    return rc;
  int err = 0;
  cudaMemcpy(&err, &s->d_ctl->err, sizeof(int), cudaMemcpyDeviceToHost);
  if (err) return ig_fail(err, "serving BFS step failed (%d)", err);
  u64 retire = 0;
  for (int q = 0; q < kLanes; q++)
    if (((E.busy >> q) & 1ull) && h.cnt[q] == 0) retire |= 1ull << q;
  if (retire) {
    const double t = now_s();
    for (int q = 0; q < kLanes; q++) {
      if (!((retire >> q) & 1ull)) continue;
      Request* r = E.lane_req[q];
      ig_query_result res;
      memset(&res, 0, sizeof(res));
      res.status = IG_OK;
      res.kind = 0;
      res.source = r->source;
      // the step that added nothing was E.step - 1; the deepest level is one less
      res.reached = 1 + (long long)h.reach[q];
      res.max_dist = res.reached > 1 ? (long long)(E.step - 1 - h.start[q]) : 0;
      res.levels = (int)res.max_dist + 1;
      res.sum_dist = (long long)h.sum[q];
      res.ntargets = r->ntargets;
      for (int j = 0; j < r->ntargets; j++) {
        res.targets[j] = r->targets[j];
        res.target_dist[j] = h.tdist[q][j];
      }
      res.submit_time = r->submit_t;
      res.admit_time = r->admit_t;
      res.done_time = t;
      complete(s, r, res);
      E.lane_req[q] = nullptr;
    }
    msbfs_retire<<<s->sms * 8, kThreads, 0, s->stream>>>(n, retire, E.a, E.b, E.is_target);
    ig_count_launches(1);
    // reset the lanes' sums and reach counts
    static const u64 zero = 0;
    for (int q = 0; q < kLanes; q++) {
      if (!((retire >> q) & 1ull)) continue;
      if ((rc = scuda(cudaMemcpyAsync((char*)E.lane_state + offsetof(BfsLaneState, sum) + q * sizeof(u64), &zero,
                                      sizeof(u64), cudaMemcpyHostToDevice, s->stream),
                      "reset")) ||
          (rc = scuda(cudaMemcpyAsync((char*)E.lane_state + offsetof(BfsLaneState, reach) + q * sizeof(u64), &zero,
                                      sizeof(u64), cudaMemcpyHostToDevice, s->stream),
                      "reset")))
        return rc;
    }
    if ((rc = scuda(cudaStreamSynchronize(s->stream), "sync"))) return rc;
    E.busy &= ~retire;
  }
  return IG_OK;
}

// One SSSP round for all busy lanes; retires lanes that improved nothing.
static int sssp_step(ig_server* s, Engine& E) {
  const int n = s->g.nodes;
  int small[3];
  int rc = scuda(cudaMemcpyAsync(small, E.d_small, sizeof(small), cudaMemcpyDeviceToHost, s->stream), "read");
  if (!rc) rc = scuda(cudaStreamSynchronize(s->stream), "sync");
  if (rc) return rc;
  const int fsize = small[2];
  if ((rc = scuda(cudaMemsetAsync(E.d_small, 0, 2 * sizeof(int), s->stream), "memset"))) return rc;
  if ((rc = scuda(cudaMemsetAsync((char*)E.lane_state + offsetof(SsspLaneState, cnt), 0, kLanes * sizeof(u64),
                                  s->stream),
                  "memset")))
    return rc;
  const int grid = s->sms * 8;
  if (fsize > 0) {
    msssp_degrees<<<grid, kThreads, 0, s->stream>>>(s->g.nindex, E.flist, fsize, E.deg);
    if ((rc = igk_exclusive_scan(&s->ex, E.deg, E.eoff, fsize, nullptr))) return rc;
    msssp_round<<<grid, kThreads, 0, s->stream>>>(s->g.nindex, s->g.nlist, s->g.eweight, n, E.flist, fsize,
                                                  (const int*)E.eoff,
                                                  E.a, E.b, E.dist, E.tlist, E.d_small, (SsspLaneState*)E.lane_state,
                                                  s->d_ctl);
    msssp_clear<<<grid, kThreads, 0, s->stream>>>(E.flist, fsize, E.a);
    ig_count_launches(3);
  }
  int tsize = 0;
  if ((rc = scuda(cudaMemcpyAsync(&tsize, E.d_small, sizeof(int), cudaMemcpyDeviceToHost, s->stream), "read")) ||
      (rc = scuda(cudaStreamSynchronize(s->stream), "sync")))
    return rc;
  if (tsize > 0) {
    msssp_promote<<<std::max(1, std::min(grid, (tsize + kThreads - 1) / kThreads)), kThreads, 0, s->stream>>>(
        E.tlist, tsize, E.b, E.a);
    ig_count_launches(1);
  }
  std::swap(E.flist, E.tlist);
  if ((rc = scuda(cudaMemcpyAsync(E.d_small + 2, &tsize, sizeof(int), cudaMemcpyHostToDevice, s->stream), "write")))
    return rc;
  E.step++;
  u64 cnt[kLanes];
  if ((rc = scuda(cudaMemcpyAsync(cnt, (char*)E.lane_state + offsetof(SsspLaneState, cnt), sizeof(cnt),
                                  cudaMemcpyDeviceToHost, s->stream),
                  "read")) ||
      (rc = scuda(cudaStreamSynchronize(s->stream), "sync")))
    return rc;
  int err = 0;
  cudaMemcpy(&err, &s->d_ctl->err, sizeof(int), cudaMemcpyDeviceToHost);
  if (err) return ig_fail(err, "serving SSSP round failed (%d)", err);
  u64 retire = 0;
  for (int q = 0; q < kLanes; q++)
    if (((E.busy >> q) & 1ull) && cnt[q] == 0) retire |= 1ull << q;
  if (!retire) return IG_OK;
  // a lane that improved nothing this round has no changed vertex left
  msssp_targets<<<(kLanes * kMaxTargets + 255) / 256, 256, 0, s->stream>>>(E.dist, retire,
                                                                            (const SsspLaneState*)E.lane_state, E.tdist);
  msssp_retire<<<grid, kThreads, 0, s->stream>>>(n, retire, E.dist, (SsspLaneState*)E.lane_state, E.tdist);
  ig_count_launches(2);
  SsspLaneState h;
  int td[kLanes * kMaxTargets];
  if ((rc = scuda(cudaMemcpyAsync(&h, E.lane_state, sizeof(h), cudaMemcpyDeviceToHost, s->stream), "read")) ||
      (rc = scuda(cudaMemcpyAsync(td, E.tdist, sizeof(td), cudaMemcpyDeviceToHost, s->stream), "read")) ||
      (rc = scuda(cudaStreamSynchronize(s->stream), "sync")))
    return rc;
  const double t = now_s();
  static const u64 zero = 0;
  static const long long zerol = 0;
  for (int q = 0; q < kLanes; q++) {
    if (!((retire >> q) & 1ull)) continue;
    Request* r = E.lane_req[q];
    ig_query_result res;
    memset(&res, 0, sizeof(res));
    res.status = IG_OK;
    res.kind = 1;
    res.source = r->source;
    res.levels = E.step;
    res.reached = (long long)h.reached[q];
    res.max_dist = h.maxd[q];
    res.sum_dist = (long long)h.sum[q];
    res.ntargets = r->ntargets;
    for (int j = 0; j < r->ntargets; j++) {
      res.targets[j] = r->targets[j];
      res.target_dist[j] = td[q * kMaxTargets + j];
    }
    res.submit_time = r->submit_t;
    res.admit_time = r->admit_t;
    res.done_time = t;
    complete(s, r, res);
    E.lane_req[q] = nullptr;
    if ((rc = scuda(cudaMemcpyAsync((char*)E.lane_state + offsetof(SsspLaneState, reached) + q * sizeof(u64), &zero,
                                    sizeof(u64), cudaMemcpyHostToDevice, s->stream),
                    "reset")) ||
        (rc = scuda(cudaMemcpyAsync((char*)E.lane_state + offsetof(SsspLaneState, sum) + q * sizeof(u64), &zero,
                                    sizeof(u64), cudaMemcpyHostToDevice, s->stream),
                    "reset")) ||
        (rc = scuda(cudaMemcpyAsync((char*)E.lane_state + offsetof(SsspLaneState, maxd) + q * sizeof(long long),
                                    &zerol, sizeof(long long), cudaMemcpyHostToDevice, s->stream),
                    "reset")))
      return rc;
  }
  if ((rc = scuda(cudaStreamSynchronize(s->stream), "sync"))) return rc;
  E.busy &= ~retire;
  return IG_OK;
}

static void worker_main(ig_server* s) {
  cudaSetDevice(s->device);
  while (true) {
    {
      std::unique_lock<std::mutex> lk(s->mu);
      s->cv_work.wait(lk, [&] {
        return s->stop || !s->pending[0].empty() || !s->pending[1].empty() || s->eng[0].busy || s->eng[1].busy;
      });
      if (s->stop) break;
    }
    int rc = IG_OK;
    bool progressed = false;
    for (int k = 0; k < 2 && rc == IG_OK; k++) {
      Engine& E = s->eng[k];
      bool want;
      {
        std::lock_guard<std::mutex> lk(s->mu);
        want = !s->pending[k].empty();
      }
      if (want && !E.live) {
        rc = engine_ensure(s, k);
        if (rc == IG_ERR_BUSY) {  // deferred: too little memory for now
          rc = IG_OK;
          continue;
        }
      }
      if (rc == IG_OK && E.live) rc = engine_admit(s, E);
      if (rc == IG_OK && E.busy) {
        rc = (k == 0) ? bfs_step(s, E) : sssp_step(s, E);
        progressed = true;
      }
    }
    if (rc == IG_OK && !progressed) {  // only deferred queries: wait for memory, then retry
      std::unique_lock<std::mutex> lk(s->mu);
      s->cv_work.wait_for(lk, std::chrono::milliseconds(1), [&] { return s->stop; });
    }
    std::lock_guard<std::mutex> lk(s->mu);
    s->steps++;
    if (rc != IG_OK) {
      s->worker_rc = rc;
      s->stop = true;
      s->cv_done.notify_all();
      break;
    }
  }
}

extern "C" int ig_server_create(const ig_csr* d_g, int max_pending, ig_server** out) {
  if (!d_g || !out || d_g->nodes < 1 || d_g->edges < 0 || !d_g->nindex || (d_g->edges > 0 && !d_g->nlist) ||
      max_pending < 1)
    return ig_fail(IG_ERR_INVALID_ARG, "ig_server_create: bad argument");
  std::unique_ptr<ig_server> s(new ig_server());
  s->g = *d_g;
  s->max_pending = max_pending;
  int rc;
  if ((rc = scuda(cudaGetDevice(&s->device), "cudaGetDevice"))) return rc;
  if ((rc = scuda(cudaDeviceGetAttribute(&s->sms, cudaDevAttrMultiProcessorCount, s->device), "SM count"))) return rc;
  // The engines' state is allocated when queries need it (engine_ensure);
  // the smaller engine must at least fit the device now.
  size_t free_b = 0, total_b = 0;
  if ((rc = scuda(cudaMemGetInfo(&free_b, &total_b), "cudaMemGetInfo"))) return rc;
  const long long need = engine_bytes(s.get(), 0);
  if (need + (need >> 3) > (long long)free_b)
    return ig_fail(IG_ERR_NOMEM, "serving state needs %lld bytes, %zu free", need, free_b);
  s->eng[0].kind = 0;
  s->eng[1].kind = 1;
  if ((rc = scuda(cudaStreamCreate(&s->stream), "stream"))) return rc;
  s->scratch.device = s->device;
  if ((rc = ig_exec_init(&s->ex, s->stream, &s->scratch, nullptr, s->device, s->sms))) return rc;
  s->d_ctl = s->ex.d_ctl;
  if ((rc = scuda(cudaMemsetAsync(s->d_ctl, 0, sizeof(IgCtl), s->stream), "memset"))) return rc;
  if ((rc = scuda(cudaStreamSynchronize(s->stream), "sync"))) return rc;
  ig_server* raw = s.release();
  raw->worker = std::thread(worker_main, raw);
  *out = raw;
  return IG_OK;
}

extern "C" int ig_server_submit(ig_server* s, int kind, int source, const int* targets, int ntargets,
                                long long* ticket) {
  if (!s || !ticket || (kind != 0 && kind != 1) || source < 0 || source >= s->g.nodes || ntargets < 0 ||
      ntargets > kMaxTargets || (ntargets > 0 && !targets))
    return ig_fail(IG_ERR_INVALID_ARG, "ig_server_submit: bad argument");
  if (kind == 1 && !s->g.eweight) return ig_fail(IG_ERR_INVALID_ARG, "graph has no weights for SSSP queries");
  for (int j = 0; j < ntargets; j++)
    if (targets[j] < 0 || targets[j] >= s->g.nodes) return ig_fail(IG_ERR_INVALID_ARG, "target out of range");
  std::lock_guard<std::mutex> lk(s->mu);
  if (s->stop) return ig_fail(s->worker_rc ? s->worker_rc : IG_ERR_CANCELLED, "server stopped");
  if ((int)(s->pending[0].size() + s->pending[1].size()) >= s->max_pending)
    return ig_fail(IG_ERR_BUSY, "serving queue full (%d pending)", s->max_pending);
  Request* r = new Request();
  r->ticket = s->next_ticket++;
  r->kind = kind;
  r->source = source;
  r->ntargets = ntargets;
  for (int j = 0; j < ntargets; j++) r->targets[j] = targets[j];
  r->submit_t = now_s();
  s->pending[kind].push_back(r);
  *ticket = r->ticket;
  s->cv_work.notify_one();
  return IG_OK;
}

extern "C" int ig_server_wait(ig_server* s, long long ticket, int timeout_ms, ig_query_result* out) {
  if (!s || !out) return ig_fail(IG_ERR_INVALID_ARG, "null argument");
  std::unique_lock<std::mutex> lk(s->mu);
  const bool ok = s->cv_done.wait_for(lk, std::chrono::milliseconds(std::max(0, timeout_ms)),
                                      [&] { return s->done.count(ticket) > 0 || s->stop; });
  auto it = s->done.find(ticket);
  if (it == s->done.end()) {
    if (s->stop) return ig_fail(s->worker_rc ? s->worker_rc : IG_ERR_CANCELLED, "server stopped");
    return ig_fail(IG_ERR_TIMEOUT, ok ? "no such ticket" : "query not finished within %d ms", timeout_ms);
  }
  *out = it->second.second;
  delete it->second.first;
  s->done.erase(it);
  return IG_OK;
}

extern "C" int ig_server_stats(ig_server* s, long long* completed, long long* steps) {
  if (!s) return ig_fail(IG_ERR_INVALID_ARG, "null");
  std::lock_guard<std::mutex> lk(s->mu);
  if (completed) *completed = s->completed;
  if (steps) *steps = s->steps;
  return s->worker_rc;
}

extern "C" int ig_server_set_memory_budget(ig_server* s, long long bytes) {
  if (!s || bytes < -1) return ig_fail(IG_ERR_INVALID_ARG, "ig_server_set_memory_budget: bad argument");
  std::lock_guard<std::mutex> lk(s->mu);
  s->budget = bytes;
  s->cv_work.notify_all();
  return IG_OK;
}

extern "C" int ig_server_memory(ig_server* s, long long* held_bytes, long long* deferrals, long long* engines_created) {
  if (!s) return ig_fail(IG_ERR_INVALID_ARG, "null");
  std::lock_guard<std::mutex> lk(s->mu);
  if (held_bytes)
    *held_bytes = (s->eng[0].live ? engine_bytes(s, 0) : 0) + (s->eng[1].live ? engine_bytes(s, 1) : 0);
  if (deferrals) *deferrals = s->deferrals;
  if (engines_created) *engines_created = s->engines_created;
  return s->worker_rc;
}

extern "C" int ig_server_destroy(ig_server* s) {
  if (!s) return IG_OK;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
    s->cv_work.notify_all();
    s->cv_done.notify_all();
  }
  if (s->worker.joinable()) s->worker.join();
  for (int k = 0; k < 2; k++) {
    for (Request* r : s->pending[k]) delete r;
    for (Request* r : s->eng[k].lane_req)
      if (r) delete r;
    engine_free(s->eng[k]);
  }
  for (auto& kv : s->done) delete kv.second.first;
  ig_scratch_release(&s->scratch);
  cudaStreamDestroy(s->stream);
  delete s;
  return IG_OK;
}
