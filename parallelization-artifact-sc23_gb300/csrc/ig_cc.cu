// Connected components by union-find hooking and pointer jumping.
//
// The reference computes labels by min-label propagation until no label
// changes (codes/cpp/cc-cpp/CC_CPP_V_Topo_Push_IntType_ReadModifyWrite_Determ_
// NoBoundsBug_Block_Atomic.cpp; CUDA: codes/cuda/cc-cuda/CC_CUDA_V_Topo_Push_
// Determ_IntType_ReadModifyWrite_NonPersist_CudaAtomic_Thread_NoBoundsBug2_
// NoBoundsBug1.cu:57-77), whose fixed point is label[v] = the smallest vertex
// id in v's component; rounds grow with the graph diameter.  Here every
// undirected edge is visited once and the two trees are linked by always
// hooking the larger root under the smaller one with atomicCAS, so a root is
// the minimum of its tree; a final pass points every vertex at its root.
// The result is the same min-id labelling in a number of passes independent
// of the diameter.  Most edges of a skewed graph never need a union: after
// linking every vertex to its first kSample neighbours (neighbour sampling,
// as in Afforest, Sutton et al. 2018) the largest component is already
// connected, and only vertices outside it link their other edges (all of
// them: the other end may be a skipped vertex; the graph is symmetric).
// Every parent pointer goes to a smaller or equal id (init, larger-under-
// smaller hooks, path halving), so each final root is its component's minimum.
//
// Default form (option cc_bfs_seed): the component of the vertex of largest
// degree -- the giant component of a skewed graph -- is found by the
// direction-optimising BFS kernel from that vertex (its source read on the
// device) and labelled with its smallest reached id; every other vertex
// starts as its own root and links all its edges by the hooking below (its
// component never touches the giant one).  On RMAT-22 this takes 0.35 ms
// against 1.0 ms for the sampling form.
//
//   init    : parent[v] = min(v, first neighbour)   (adjacency is sorted)
//   sample  : union(v, neighbour r) for r = 0 .. kSample-1
//   compress: parent[v] = root(v)
//   giant   : the most frequent root among a fixed sample of vertices
//   hook    : vertices whose root is not the giant one: union(v, w) for their
//             neighbours from position kSample on (only w < v when there is
//             no giant component); vertices above the hub degree are
//             deferred to an edge-balanced grid-wide pass
//   compress: label[v] = root(v)
#include "ig_device.cuh"
#include "ig_options.h"

namespace {

constexpr int kThreads = 256;
constexpr int kSample = 2;      // neighbours linked before the giant component is picked
constexpr int kGiantSamples = 1024;

__device__ __forceinline__ int load_parent(const int* parent, int x) {
  return *((const volatile int*)parent + x);
}

// Root of x with path halving (writes only ever point a vertex at one of its
// ancestors, so they are safe under concurrent hooking).
__device__ __forceinline__ int find_root(int* parent, int x) {
  while (true) {
    const int p = load_parent(parent, x);
    if (p == x) return x;
    const int gp = load_parent(parent, p);
    if (gp == p) return p;
    parent[x] = gp;
    x = gp;
  }
}

__device__ __forceinline__ void unite(int* parent, int u, int v) {
  int ru = find_root(parent, u);
  int rv = find_root(parent, v);
  while (ru != rv) {
    if (ru < rv) {
      const int t = ru;
      ru = rv;
      rv = t;
    }
    // ru > rv: hook the larger root under the smaller
    const int old = atomicCAS(&parent[ru], ru, rv);
    if (old == ru) return;
    ru = find_root(parent, old);
    rv = find_root(parent, rv);
  }
}

__global__ void cc_init(const int* __restrict__ nindex, const int* __restrict__ nlist, int n, int* parent) {
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
    const int b = __ldg(&nindex[v]), e = __ldg(&nindex[v + 1]);
    int p = v;
    if (b < e) {
      const int m = __ldg(&nlist[b]);
      if (m < v) p = m;
    }
    parent[v] = p;
  }
}

// Root of x without writes (for passes where many threads walk the same
// paths: path-halving writes would make them contend for the same lines).
__device__ __forceinline__ int find_root_ro(const int* parent, int x) {
  while (true) {
    const int p = load_parent(parent, x);
    if (p == x) return x;
    x = p;
  }
}

// union(v, neighbour r) for every vertex, with read-only root searches; a
// compression pass follows each round, so the trees stay flat.
__global__ void cc_link_round(const int* __restrict__ nindex, const int* __restrict__ nlist, int n, int* parent,
                              int r) {
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
    const int b = __ldg(&nindex[v]), e = __ldg(&nindex[v + 1]);
    if (b + r >= e) continue;
    int ru = find_root_ro(parent, v);
    int rv = find_root_ro(parent, __ldg(&nlist[b + r]));
    while (ru != rv) {
      if (ru < rv) {
        const int t = ru;
        ru = rv;
        rv = t;
      }
      const int old = atomicCAS(&parent[ru], ru, rv);
      if (old == ru) break;
      ru = find_root_ro(parent, old);
      rv = find_root_ro(parent, rv);
    }
  }
}

__global__ void cc_sample(const int* __restrict__ nindex, const int* __restrict__ nlist, int n, int* parent) {
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
    const int b = __ldg(&nindex[v]), e = __ldg(&nindex[v + 1]);
    // position 0 too: init linked it only when the neighbour's id is smaller
    for (int r = 0; r < kSample && b + r < e; r++) unite(parent, v, __ldg(&nlist[b + r]));
  }
}

// The most frequent root among kGiantSamples evenly spaced vertices (parent
// is compressed, so parent[x] is x's root); one block.  Written to ctl->i32[1],
// or -1 when it covers less than 1/8 of the samples (no giant component, as in
// a union of many small graphs): then no vertex is skipped and every
// undirected edge is linked once, from its larger end.
__global__ void __launch_bounds__(kThreads) cc_giant(const int* parent, int n, IgCtl* ctl) {
  __shared__ int s_root[kGiantSamples];
  __shared__ unsigned long long s_best;
  const int m = n < kGiantSamples ? n : kGiantSamples;
  for (int i = threadIdx.x; i < m; i += blockDim.x) s_root[i] = parent[(long long)i * n / m];
  if (threadIdx.x == 0) s_best = 0;
  __syncthreads();
  for (int i = threadIdx.x; i < m; i += blockDim.x) {
    int c = 0;
    for (int j = 0; j < m; j++) c += s_root[j] == s_root[i];
    // count in the high word, the smaller root wins ties (deterministic)
    atomicMax(&s_best, ((unsigned long long)c << 32) | (unsigned)(0x7fffffff - s_root[i]));
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const int count = (int)(s_best >> 32);
    ctl->i32[1] = count * 8 >= m ? 0x7fffffff - (int)(s_best & 0xffffffffu) : -1;
  }
}

__global__ void __launch_bounds__(kThreads) cc_hook(const int* __restrict__ nindex, const int* __restrict__ nlist,
                                                    int n, int* parent, int* hubs, IgCtl* ctl, int hub_degree,
                                                    int first) {
  using namespace ig;
  const int lane = lane_id();
  const long long gtid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long gthreads = (long long)gridDim.x * blockDim.x;
  const int giant = ctl->i32[1];
  const bool half = giant < 0;  // no giant component: each edge once, from its larger end
  for (long long base = gtid & ~31LL; base < n; base += gthreads) {
    const long long v = base + lane;
    int beg = 0, deg = 0;
    // a vertex still pointing at the giant root is in the giant component:
    // its edges to other components are linked from their other ends
    if (v < n && load_parent(parent, (int)v) != giant) {
      beg = __ldg(&nindex[v]) + first;  // positions below `first` were linked by the sampling
      deg = max(0, __ldg(&nindex[v + 1]) - beg);
    }
    const bool hub = deg > hub_degree;
    warp_append(hub, (int)v, hubs, &ctl->i32[0], n, ctl);
    const int vv = (int)v;
    warp_expand(beg, hub ? 0 : deg, [&](bool act, int e, int j) {
      const int u = __shfl_sync(IG_FULL, vv, j);
      if (act) {
        const int w = __ldg(&nlist[e]);
        if (!half || w < u) unite(parent, u, w);
      }
    });
  }
}

__global__ void __launch_bounds__(kThreads) cc_hook_hubs(const int* __restrict__ nindex,
                                                         const int* __restrict__ nlist, int* parent,
                                                         const int* hubs, const IgCtl* ctl) {
  using namespace ig;
  const int nh = ctl->i32[0];
  if (nh == 0) return;
  const bool half = ctl->i32[1] < 0;
  grid_expand_hubs(nindex, hubs, nh, [&](bool act, int e, int hv) {
    if (act) {
      const int w = __ldg(&nlist[e]);
      if (!half || w < hv) unite(parent, hv, w);
    }
  });
}

__global__ void cc_compress(int* parent, int n) {
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
    int r = parent[v];
    while (true) {
      const int p = parent[r];
      if (p == r) break;
      r = p;
    }
    parent[v] = r;
  }
}

// BFS-seeded form.  The seed is the vertex of largest degree (ties: the
// smaller id), packed as (degree << 32) | (0xffffffff - id) and reduced with
// one 64-bit atomicMax per warp.
__global__ void cc_seed(const int* __restrict__ nindex, int n, unsigned long long* key) {
  unsigned long long best = 0;
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
    const unsigned long long d = (unsigned)(__ldg(&nindex[v + 1]) - __ldg(&nindex[v]));
    const unsigned long long k = (d << 32) | (0xffffffffu - (unsigned)v);
    best = k > best ? k : best;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long t = __shfl_xor_sync(IG_FULL, best, o);
    best = t > best ? t : best;
  }
  if ((threadIdx.x & 31) == 0) atomicMax(key, best);
}

// After a BFS from the seed wrote levels into `label`: the smallest reached
// id (the seed's component's minimum) into *giant.
__global__ void cc_reached_min(const int* label, int n, int* giant) {
  int m = ig::kInf;
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x)
    if (label[v] != ig::kInf) m = min(m, v);
  m = __reduce_min_sync(IG_FULL, m);
  if ((threadIdx.x & 31) == 0 && m != ig::kInf) atomicMin(giant, m);
}

// Reached vertices point at that minimum (one finished tree); the others
// start as their own roots for the hooking of their edges.
__global__ void cc_from_levels(int* label, int n, const int* giant) {
  const int m = *giant;
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x)
    label[v] = label[v] != ig::kInf ? m : v;
}

// Disjoint union of graphs: the global min-id label minus the graph's first
// vertex is the graph's own min-id label.  One block per graph.
__global__ void cc_localize(int* label, const int* __restrict__ graph_vptr, int graphs) {
  for (int g = blockIdx.x; g < graphs; g += gridDim.x) {
    const int b = __ldg(&graph_vptr[g]), e = __ldg(&graph_vptr[g + 1]);
    for (int v = b + threadIdx.x; v < e; v += blockDim.x) label[v] -= b;
  }
}

}  // namespace

int igk_cc_localize(IgExec* ex, int* d_label, const int* d_graph_vptr, int graphs) {
  cc_localize<<<std::min(graphs, ex->sms * 16), kThreads, 0, ex->stream>>>(d_label, d_graph_vptr, graphs);
  ig_count_launches(1);
  return ig_cuda_check((int)cudaGetLastError(), "cc localize launch");
}

int igk_cc(IgExec* ex, const ig_csr* dg, int* d_label, bool sample) {
  const int n = dg->nodes;
  void* hubs;
  int rc;
  const IgOptions& o = ig_exec_options(ex);
  const int grid_v = std::min((n + kThreads - 1) / kThreads, ex->sms * 16);
  const int grid_w = std::max(1, std::min((n + kThreads - 1) / kThreads, ex->sms * 8));
  if (sample && o.cc_bfs_seed) {
    // The component of the largest-degree vertex (the giant one of a skewed
    // graph) is labelled by a BFS from it with its smallest reached id; the
    // other vertices link all their edges by union-find (they never touch
    // that component), skipping the reached ones.
    void* key;
    if ((rc = ig_scratch_get(ex->scratch, IG_SLOT_V2, 64, &key))) return rc;
    if ((rc = ig_cuda_check((int)cudaMemsetAsync(key, 0, 64, ex->stream), "memset"))) return rc;
    cc_seed<<<grid_v, kThreads, 0, ex->stream>>>(dg->nindex, n, (unsigned long long*)key);
    ig_count_launches(1);
    // at most cc_bfs_levels levels: on a high-diameter graph the BFS labels
    // only the seed's neighbourhood and union-find links the rest
    if ((rc = igk_bfs_keyed(ex, dg, (const unsigned long long*)key, d_label, o.cc_bfs_levels)))
      return rc;  // resets the control block
    if ((rc = ig_scratch_get(ex->scratch, IG_SLOT_Q2, (size_t)n * sizeof(int), &hubs))) return rc;
    if ((rc = ig_cuda_check((int)cudaMemsetAsync(&ex->d_ctl->i32[1], 0x7f, sizeof(int), ex->stream), "memset")))
      return rc;
    cc_reached_min<<<grid_v, kThreads, 0, ex->stream>>>(d_label, n, &ex->d_ctl->i32[1]);
    cc_from_levels<<<grid_v, kThreads, 0, ex->stream>>>(d_label, n, &ex->d_ctl->i32[1]);
    cc_hook<<<grid_w, kThreads, 0, ex->stream>>>(dg->nindex, dg->nlist, n, d_label, (int*)hubs, ex->d_ctl,
                                                 o.hub_degree, 0);
    cc_hook_hubs<<<ex->sms * 4, kThreads, 0, ex->stream>>>(dg->nindex, dg->nlist, d_label, (int*)hubs, ex->d_ctl);
    cc_compress<<<grid_v, kThreads, 0, ex->stream>>>(d_label, n);
    ig_count_launches(5);
    return ig_cuda_check((int)cudaGetLastError(), "cc launch");
  }
  if ((rc = ig_scratch_get(ex->scratch, IG_SLOT_Q2, (size_t)n * sizeof(int), &hubs))) return rc;
  if ((rc = ig_exec_reset(ex))) return rc;
  cc_init<<<grid_v, kThreads, 0, ex->stream>>>(dg->nindex, dg->nlist, n, d_label);
  if (sample && o.cc_rounds == 2) {  // the init forest flattened before the sampled unions
    cc_compress<<<grid_v, kThreads, 0, ex->stream>>>(d_label, n);
    ig_count_launches(1);
  }
  if (sample && o.cc_rounds == 1) {
    // neighbour r of every vertex linked in its own round, trees flattened after each
    for (int r = 0; r < kSample; r++) {
      cc_link_round<<<grid_v, kThreads, 0, ex->stream>>>(dg->nindex, dg->nlist, n, d_label, r);
      cc_compress<<<grid_v, kThreads, 0, ex->stream>>>(d_label, n);
    }
    cc_giant<<<1, kThreads, 0, ex->stream>>>(d_label, n, ex->d_ctl);
    ig_count_launches(2 * kSample + 1);
  } else if (sample) {
    cc_sample<<<grid_v, kThreads, 0, ex->stream>>>(dg->nindex, dg->nlist, n, d_label);
    cc_compress<<<grid_v, kThreads, 0, ex->stream>>>(d_label, n);
    cc_giant<<<1, kThreads, 0, ex->stream>>>(d_label, n, ex->d_ctl);
    ig_count_launches(3);
  } else if ((rc = ig_cuda_check((int)cudaMemsetAsync(&ex->d_ctl->i32[1], 0xff, sizeof(int), ex->stream),
                                 "memset"))) {
    return rc;  // i32[1] = -1: no giant component, every edge linked once from its larger end
  }
  cc_hook<<<grid_w, kThreads, 0, ex->stream>>>(dg->nindex, dg->nlist, n, d_label, (int*)hubs, ex->d_ctl,
                                               o.hub_degree, sample ? kSample : 0);
  cc_hook_hubs<<<ex->sms * 4, kThreads, 0, ex->stream>>>(dg->nindex, dg->nlist, d_label, (int*)hubs, ex->d_ctl);
  cc_compress<<<grid_v, kThreads, 0, ex->stream>>>(d_label, n);
  ig_count_launches(4);
  return ig_cuda_check((int)cudaGetLastError(), "cc launch");
}
