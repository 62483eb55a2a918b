// PageRank, pull formulation: one persistent, cooperatively launched kernel
// runs every iteration and tests convergence on the device.
//
// Reference semantics (include/pr_cuda.h:42-46, 113-135 and the pull variants,
// e.g. codes/cuda/pr-cuda/PR_CUDA_Pull_FloatType_Persist_Warp_Determ_
// Reduction.cu:41-83; C++ codes/cpp/pr-cpp/PR_CPP_Pull_FloatType_Reduction_
// Block_Determin.cpp:40-89): a Jacobi step
//     contrib[u] = score[u] / degree[u]
//     score[v]   = (1 - d) / V + d * sum_{u in N(v)} contrib[u],   d = 0.85
// with the FP32 L1 change sum |score_new - score_old| accumulated in double;
// iterations stop when that change is below epsilon or after max_iter.  The
// reference issues two kernels and two small copies per iteration; here the
// whole loop runs on the device and the host learns the iteration count.
//
// Accuracy: each vertex's incoming sum is accumulated in FP32 with Kahan
// compensation (lanes of a warp combine their partial sums exactly with
// TwoSum); each vertex's |change| is rounded once to a 64-bit fixed-point
// integer (units of 2^-60) and the residual is their integer sum, exact in
// any order, so every run of the same input gives bit-identical scores and
// the same iteration count however the vertices were dealt to warps.  (A
// batched run stops each graph on its own FP64 residual.)
//
// Work split: groups of 32 consecutive vertices, the first static_pct
// percent of them dealt round-robin to the warps and the rest taken from a
// per-iteration counter, a group (or a unit of groups on a graph with many)
// per claim, claimed one ahead, so the claim's round trip and the next
// group's list loads overlap the current group's sums; a list's cost varies
// with its degree, so the counter evens out the end of the iteration.  A
// vertex with <= kLight neighbours is summed by its own lane, one with more
// by an 8-lane sub-warp (subwarp) or the whole warp; a vertex above the hub
// degree is cut into fixed chunks of edges spread over all warps, and its
// chunk sums are combined in chunk order after a grid barrier.
#include <type_traits>

#include "ig_device.cuh"
#include "ig_options.h"

namespace {

constexpr int kThreads = 256;
constexpr int kLight = 16;

struct PrArgs {
  const int* __restrict__ nindex;
  const int* __restrict__ nlist;
  const int* degree;  // may be null: nindex difference
  int nodes;
  long long edges;
  float* scores;
  float* ca;          // contributions (alternating)
  float* cb;
  int* hubs;          // hub vertices in increasing id order
  int* chunk_base;    // first chunk of each hub (hubs + 1 entries)
  int* chunk_hub;     // hub index of each chunk
  float2* partial;    // per-chunk (hi, lo) sums
  int* blk;           // per-block counts for the deterministic hub compaction (2 * grid)
  unsigned long long* blkerr;  // per-block residual partials, fixed point (2 * grid)
  IgCtl* ctl;
  float eps;
  int max_iter;
  float base;
  float damp;
  unsigned long long timeout_ns;
  int hub_degree;
  int chunk;
  int prefetch;  // 1: each warp prefetches its next vertex group's lists into L2
  int subwarp;   // 1: medium lists summed four at a time by 8-lane sub-warps (else two by the warp)
  float* vals;   // two-pass form: vals[k] = contributions[nlist[k]], gathered each iteration (else null)
  // batched form (disjoint union of graphs): first vertex of each graph,
  // per-graph residuals (3 rotating slots) and per-graph iteration counts
  const int* graph_vptr;
  int graphs;
  double* gres;
  int* giters;
  int* vgraph;  // graph of every vertex (filled by the kernel before the first iteration)
  int static_pct;  // percent of the vertex groups dealt round-robin (the rest from a counter)
};

constexpr double kFix = 1152921504606846976.0;  // 2^60: residual fixed-point scale
constexpr int kPrGrab = 0;                       // hot counters kPrGrab + it % 3: groups claimed in iteration it

// |change| of one score in fixed point: a graph's scores sum to at most 1,
// so its changes sum to at most 2 and the total stays below 2^61.  (The
// batched form, whose graphs stop on their own residuals, keeps the total in
// double: it is only reported.)
__device__ __forceinline__ unsigned long long pr_fixed(double x) { return __double2ull_rn(x * kFix); }

// Adds each lane's x into gres[g_lane] with one atomic per distinct graph of the warp.
__device__ __forceinline__ void warp_add_by_graph(double* gres, int g, double x, bool valid) {
  unsigned rem = __ballot_sync(IG_FULL, valid);
  while (rem) {
    const int leader = __ffs(rem) - 1;
    const int gl = __shfl_sync(IG_FULL, g, leader);
    const bool in = valid && g == gl;
    double v = in ? x : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(IG_FULL, v, o);
    if (ig::lane_id() == leader && v != 0.0) atomicAdd(&gres[gl], v);
    rem &= ~__ballot_sync(IG_FULL, in);
  }
}

__device__ __forceinline__ void kahan_add(float& s, float& c, float x) {
  const float y = __fsub_rn(x, c);
  const float t = __fadd_rn(s, y);
  c = __fsub_rn(__fsub_rn(t, s), y);
  s = t;
}
// (hi, lo) += (h2, l2) with an exact TwoSum of the leading parts.
__device__ __forceinline__ void pair_add(float& hi, float& lo, float h2, float l2) {
  const float s = __fadd_rn(hi, h2);
  const float bb = __fsub_rn(s, hi);
  const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(h2, bb));
  const float l = __fadd_rn(e, __fadd_rn(lo, l2));
  const float t = __fadd_rn(s, l);
  lo = __fsub_rn(l, __fsub_rn(t, s));
  hi = t;
}
__device__ __forceinline__ void warp_pair_reduce(float& hi, float& lo) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float h2 = __shfl_xor_sync(IG_FULL, hi, o);
    const float l2 = __shfl_xor_sync(IG_FULL, lo, o);
    pair_add(hi, lo, h2, l2);
  }
}

// The value of edge slot k: contrib[nlist[k]], or, in the two-pass form,
// vals[k], gathered for every edge by the iteration's first pass.  The
// kTwo forms below read vals (written in this kernel: plain loads) and
// skip the index loads; the order of the adds is the same either way.
//
// Kahan sum of the values of k = b + lane, b + lane + 32, ... < e, returned
// as a (hi, lo) pair reduced over the warp (same value in all lanes).  Each
// lane keeps 8 gathers in flight and loads the next 8 indices while the
// current values arrive; the adds stay in the order k, k + 32, k + 64, ...
template <bool kTwo>
__device__ __forceinline__ void warp_gather_sum(const int* __restrict__ nlist, const float* contrib, int b, int e,
                                                float& hi, float& lo) {
  constexpr int kDepth = 8;
  float s = 0.f, c = 0.f;
  int k = b + ig::lane_id();
  int n[kDepth];
#pragma unroll
  for (int t = 0; t < kDepth; t++) n[t] = (!kTwo && k + 32 * t < e) ? __ldg(&nlist[k + 32 * t]) : 0;
  while (k < e) {
    float x[kDepth];
#pragma unroll
    for (int t = 0; t < kDepth; t++) x[t] = k + 32 * t < e ? contrib[kTwo ? k + 32 * t : n[t]] : 0.f;
    const int kn = k + 32 * kDepth;
#pragma unroll
    for (int t = 0; t < kDepth; t++) n[t] = (!kTwo && kn + 32 * t < e) ? __ldg(&nlist[kn + 32 * t]) : 0;
#pragma unroll
    for (int t = 0; t < kDepth; t++)
      if (k + 32 * t < e) kahan_add(s, c, x[t]);
    k = kn;
  }
  hi = s;
  lo = -c;
  warp_pair_reduce(hi, lo);
}

// warp_gather_sum for two vertices at once ([b1, e1) and [b2, e2)): their
// gathers are issued together (4 in flight per lane for each), each with its
// own Kahan sum in the same per-lane order as warp_gather_sum, so the results
// are the same bits.
template <bool kTwo>
__device__ __forceinline__ void warp_gather_sum2(const int* __restrict__ nlist, const float* contrib, int b1, int e1,
                                                 int b2, int e2, float& hi1, float& lo1, float& hi2, float& lo2) {
  constexpr int kDepth = 4;
  float s1 = 0.f, c1 = 0.f, s2 = 0.f, c2 = 0.f;
  int k1 = b1 + ig::lane_id(), k2 = b2 + ig::lane_id();
  while (k1 < e1 || k2 < e2) {
    int n1[kDepth], n2[kDepth];
#pragma unroll
    for (int t = 0; t < kDepth; t++) {
      n1[t] = (!kTwo && k1 + 32 * t < e1) ? __ldg(&nlist[k1 + 32 * t]) : 0;
      n2[t] = (!kTwo && k2 + 32 * t < e2) ? __ldg(&nlist[k2 + 32 * t]) : 0;
    }
    float x1[kDepth], x2[kDepth];
#pragma unroll
    for (int t = 0; t < kDepth; t++) {
      x1[t] = k1 + 32 * t < e1 ? contrib[kTwo ? k1 + 32 * t : n1[t]] : 0.f;
      x2[t] = k2 + 32 * t < e2 ? contrib[kTwo ? k2 + 32 * t : n2[t]] : 0.f;
    }
#pragma unroll
    for (int t = 0; t < kDepth; t++) {
      if (k1 + 32 * t < e1) kahan_add(s1, c1, x1[t]);
      if (k2 + 32 * t < e2) kahan_add(s2, c2, x2[t]);
    }
    k1 += 32 * kDepth;
    k2 += 32 * kDepth;
  }
  hi1 = s1;
  lo1 = -c1;
  hi2 = s2;
  lo2 = -c2;
  warp_pair_reduce(hi1, lo1);
  warp_pair_reduce(hi2, lo2);
}

// Asks L2 to fetch list[b, e) of a per-edge array (nlist, or the gathered
// values of the two-pass form) ahead of its use (cp.async.bulk.prefetch,
// 16-byte granules inside the array; no register holds the data, nothing
// waits on it).
__device__ __forceinline__ void prefetch_list(const PrArgs& a, const void* list, int b, int e) {
  const int* p = (const int*)list;
  const unsigned long long lo = (unsigned long long)(p + b) & ~15ull;
  const unsigned long long end = (unsigned long long)(p + a.edges) & ~15ull;
  unsigned long long hi = ((unsigned long long)(p + e) + 15ull) & ~15ull;
  if (hi > end) hi = end;
  if (e > b && hi > lo)
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(lo), "r"((unsigned)(hi - lo)) : "memory");
}

// Kahan sum of contrib[nlist[k]] over k = b + sub, b + sub + 8, ... < e by
// the 8 lanes of one sub-warp (sub = lane % 8), returned as a (hi, lo) pair
// reduced over those lanes (same value in all 8).  Each lane keeps 8 gathers
// in flight and loads the next 8 indices while the current values arrive.
// The order depends only on [b, e), so a vertex's sum is the same wherever
// its list lies.
template <bool kTwo>
__device__ __forceinline__ void subwarp8_gather_sum(const int* __restrict__ nlist, const float* contrib, int b, int e,
                                                    float& hi, float& lo) {
  constexpr int kDepth = 8, kW = 8;
  float s = 0.f, c = 0.f;
  int k = b + (ig::lane_id() & (kW - 1));
  int n[kDepth];
#pragma unroll
  for (int t = 0; t < kDepth; t++) n[t] = (!kTwo && k + kW * t < e) ? __ldg(&nlist[k + kW * t]) : 0;
  while (k < e) {  // lanes of a sub-warp may leave at different steps: no collectives inside
    float x[kDepth];
#pragma unroll
    for (int t = 0; t < kDepth; t++) x[t] = k + kW * t < e ? contrib[kTwo ? k + kW * t : n[t]] : 0.f;
    const int kn = k + kW * kDepth;
#pragma unroll
    for (int t = 0; t < kDepth; t++) n[t] = (!kTwo && kn + kW * t < e) ? __ldg(&nlist[kn + kW * t]) : 0;
#pragma unroll
    for (int t = 0; t < kDepth; t++)
      if (k + kW * t < e) kahan_add(s, c, x[t]);
    k = kn;
  }
  hi = s;
  lo = -c;
#pragma unroll
  for (int o = kW / 2; o > 0; o >>= 1) {
    const float h2 = __shfl_xor_sync(IG_FULL, hi, o);
    const float l2 = __shfl_xor_sync(IG_FULL, lo, o);
    pair_add(hi, lo, h2, l2);
  }
}

__device__ __forceinline__ int vdegree(const PrArgs& a, int v) {
  return a.degree ? a.degree[v] : (__ldg(&a.nindex[v + 1]) - __ldg(&a.nindex[v]));
}

template <bool kBatched, bool kTwo>
__global__ void __launch_bounds__(kThreads, 4) pr_persistent(PrArgs a) {
  using namespace ig;
  __shared__ int s_scan[33];
  __shared__ unsigned long long s_red[32];
  using Err = typename std::conditional<kBatched, double, unsigned long long>::type;
  auto fix = [](double x) -> Err {
    if constexpr (kBatched) return x;
    else return pr_fixed(x);
  };
  IgCtl* ctl = a.ctl;
  GridBar gb;  // this block's view of the barrier generation
  const int lane = lane_id();
  const int G = gridDim.x;
  const long long gtid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long gthreads = (long long)gridDim.x * blockDim.x;
  const int warp_g = (int)(gtid >> 5);
  const int nwarps = (int)(gthreads >> 5);

  // ---- initial contributions, hub census per contiguous block range
  for (long long v = gtid; v < a.nodes; v += gthreads)
    a.ca[v] = __fdiv_rn(a.scores[v], (float)vdegree(a, (int)v));
  if (kBatched)  // vertex -> graph, one block per graph (read after the next barrier)
    for (int g = blockIdx.x; g < a.graphs; g += G)
      for (int v = __ldg(&a.graph_vptr[g]) + threadIdx.x; v < __ldg(&a.graph_vptr[g + 1]); v += blockDim.x)
        a.vgraph[v] = g;
  const long long r0 = (long long)a.nodes * blockIdx.x / G, r1 = (long long)a.nodes * (blockIdx.x + 1) / G;
  {
    int nh = 0, nc = 0;
    for (long long v = r0 + threadIdx.x; v < r1; v += blockDim.x) {
      const int d = __ldg(&a.nindex[v + 1]) - __ldg(&a.nindex[v]);
      if (d > a.hub_degree) {
        nh++;
        nc += (d + a.chunk - 1) / a.chunk;
      }
    }
    int th, tc;
    block_scan_int(nh, s_scan, &th);
    block_scan_int(nc, s_scan, &tc);
    if (threadIdx.x == 0) {
      a.blk[blockIdx.x] = th;
      a.blk[G + blockIdx.x] = tc;
    }
  }
  if (!grid_sync(ctl, a.timeout_ns, gb)) return;
  // ---- deterministic compaction of the hubs (in vertex order)
  {
    int hoff = 0, coff = 0, htot = 0, ctot = 0;
    for (int b = 0; b < G; b++) {
      const int h = ld_relaxed(&a.blk[b]), c = ld_relaxed(&a.blk[G + b]);
      if (b < (int)blockIdx.x) {
        hoff += h;
        coff += c;
      }
      htot += h;
      ctot += c;
    }
    for (long long t0 = r0; t0 < r1; t0 += blockDim.x) {
      const long long v = t0 + threadIdx.x;
      int d = 0;
      if (v < r1) d = __ldg(&a.nindex[v + 1]) - __ldg(&a.nindex[v]);
      const bool hub = d > a.hub_degree;
      const int nc = hub ? (d + a.chunk - 1) / a.chunk : 0;
      int th, tc;
      const int ph = block_scan_int(hub ? 1 : 0, s_scan, &th);
      const int pc = block_scan_int(nc, s_scan, &tc);
      if (hub) {
        a.hubs[hoff + ph] = (int)v;
        a.chunk_base[hoff + ph] = coff + pc;
      }
      hoff += th;
      coff += tc;
    }
    if (gtid == 0) {
      ctl->i32[10] = htot;
      ctl->i32[11] = ctot;
      a.chunk_base[htot] = ctot;
    }
  }
  if (!grid_sync(ctl, a.timeout_ns, gb)) return;
  const int nh = ld_relaxed(&ctl->i32[10]);
  const int nchunks = ld_relaxed(&ctl->i32[11]);
  // chunk -> hub map, so a chunk finds its hub with one load every iteration
  for (int h = warp_g; h < nh; h += nwarps)
    for (int c = a.chunk_base[h] + lane; c < a.chunk_base[h + 1]; c += 32) a.chunk_hub[c] = h;
  if (!grid_sync(ctl, a.timeout_ns, gb)) return;

  float* cur = a.ca;
  float* nxt = a.cb;
  int it = 0;
  double residual = 0;
  while (it < a.max_iter) {
    it++;
    Err err = 0;  // this thread's |changes| (fixed point, but for the batched form)
    // groups claimed in this iteration; the counter of the next one is reset here
    unsigned long long* grab = hot64(ctl, kPrGrab + it % 3);
    if (gtid == 0) *hot64(ctl, kPrGrab + (it + 1) % 3) = 0;
    // batched: a graph whose residual fell below epsilon stops changing (its
    // scores are final after that iteration, as for a single-graph run)
    double* gcur = kBatched ? a.gres + (it % 3) * a.graphs : nullptr;
    const double* gprev = kBatched ? a.gres + ((it + 2) % 3) * a.graphs : nullptr;
    if (kBatched) {
      double* gnext = a.gres + ((it + 1) % 3) * a.graphs;
      for (long long g = gtid; g < a.graphs; g += gthreads) gnext[g] = 0.0;
    }
    auto frozen = [&](int g) { return kBatched && it > 1 && ld_relaxed(&gprev[g]) < (double)a.eps; };
    if (kTwo) {
      // ---- first pass: the contribution of every edge slot, vals[k] =
      // cur[nlist[k]], through 128-bit index loads and 128-bit stores (both
      // arrays 16-byte aligned, checked at launch), four quads per thread in
      // flight: the gathers of the iteration issued as one dense stream
      const long long nq = a.edges >> 2;
      const int4* nl4 = reinterpret_cast<const int4*>(a.nlist);
      float4* v4 = reinterpret_cast<float4*>(a.vals);
      for (long long q0 = gtid; q0 < nq; q0 += 4 * gthreads) {
        int4 ix[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
          const long long q = q0 + u * gthreads;
          ix[u] = q < nq ? __ldg(&nl4[q]) : make_int4(0, 0, 0, 0);
        }
        float4 x[4];
#pragma unroll
        for (int u = 0; u < 4; u++) x[u] = make_float4(cur[ix[u].x], cur[ix[u].y], cur[ix[u].z], cur[ix[u].w]);
#pragma unroll
        for (int u = 0; u < 4; u++) {
          const long long q = q0 + u * gthreads;
          if (q < nq) v4[q] = x[u];
        }
      }
      for (long long k = (nq << 2) + gtid; k < a.edges; k += gthreads) a.vals[k] = cur[__ldg(&a.nlist[k])];
      if (!grid_sync(ctl, a.timeout_ns, gb)) return;
    }
    // ---- phase A: hub chunks (partial sums) and regular vertices
    for (int c = warp_g; c < nchunks; c += nwarps) {
      const int lo = a.chunk_hub[c];  // owning hub
      const int hv = a.hubs[lo];
      if (kBatched && frozen(a.vgraph[hv])) continue;
      const int hb = __ldg(&a.nindex[hv]), he = __ldg(&a.nindex[hv + 1]);
      const int b = hb + (c - a.chunk_base[lo]) * a.chunk;
      const int e = min(b + a.chunk, he);
      float shi, slo;
      warp_gather_sum<kTwo>(a.nlist, kTwo ? a.vals : cur, b, e, shi, slo);
      if (lane == 0) a.partial[c] = make_float2(shi, slo);
    }
    // Vertex groups: this warp's sequence is warp_g, warp_g + nwarps, ...
    // below nstatic, then units of `unit` consecutive groups claimed from the
    // counter (a unit of one group unless the graph has more than 32 groups
    // per warp, as a batched pack does, so the counter takes about 32 claims
    // per warp).  Each lane's list range of the warp's next group is loaded
    // (and its list prefetched into L2), and the unit after it claimed, while
    // the current group is summed.
    const long long ngroups = ((long long)a.nodes + 31) >> 5;
    const long long nstatic = max(min(ngroups, (long long)nwarps), ngroups * a.static_pct / 100);
    const long long unit = max(1LL, (ngroups - nstatic) / (32LL * nwarps));
    auto load_ranges = [&](long long grp, int& rb, int& re) {
      const long long vn = grp * 32 + lane;
      rb = re = 0;
      if (grp < ngroups && vn < a.nodes) {
        rb = __ldg(&a.nindex[vn]);
        re = __ldg(&a.nindex[vn + 1]);
        if (a.prefetch && re - rb <= a.hub_degree) prefetch_list(a, kTwo ? (const void*)a.vals : a.nlist, rb, re);
      }
    };
    // first group of claimed unit c, and the end of the unit
    auto unit_first = [&](unsigned long long c) { return nstatic + (long long)c * unit; };
    long long grp = warp_g, gnext, uend = 0;  // uend: end of the claimed unit that holds gnext
    if (grp + nwarps < nstatic) {
      gnext = grp + nwarps;
    } else {
      unsigned long long c = 0;
      if (lane == 0) c = atomicAdd(grab, 1ull);
      gnext = unit_first(__shfl_sync(IG_FULL, c, 0));
      uend = min(gnext + unit, ngroups);
    }
    int nb = 0, ne = 0;
    load_ranges(grp, nb, ne);
    while (grp < ngroups) {
      const long long vi = grp * 32 + lane;
      int v = (int)vi;
      const int b = nb, e = ne;
      // the group after gnext: the next static one, the next in its unit,
      // or the first of a unit claimed now (used at the end)
      const bool dyn = gnext >= nstatic;
      const bool claim = gnext < ngroups && (dyn ? gnext + 1 >= uend : gnext + nwarps >= nstatic);
      unsigned long long claimed = 0;
      if (claim && lane == 0) claimed = atomicAdd(grab, 1ull);
      load_ranges(gnext, nb, ne);
      int d = e - b;
      float sum = 0.f;
      int vg = 0;
      float vbase = a.base;
      bool skip = false;
      if (kBatched && vi < a.nodes) {
        vg = a.vgraph[v];
        skip = frozen(vg);
        vbase = __fdiv_rn(__fsub_rn(1.0f, a.damp),
                          (float)(__ldg(&a.graph_vptr[vg + 1]) - __ldg(&a.graph_vptr[vg])));
      }
      if (skip) d = a.hub_degree + 1;  // handled by nobody: frozen
      const bool light = vi < a.nodes && !skip && d <= kLight;
      if (light) {
        // loads issued eight at a time so each lane keeps several gathers in
        // flight (at most two rounds for 16 neighbours); the adds stay in
        // adjacency order
        float s = 0.f, c = 0.f;
        for (int k = b; k < e; k += 8) {
          int nb[8];
#pragma unroll
          for (int t = 0; t < 8; t++) nb[t] = k + t < e ? (kTwo ? k + t : __ldg(&a.nlist[k + t])) : -1;
          float x[8];
#pragma unroll
          for (int t = 0; t < 8; t++) x[t] = nb[t] >= 0 ? (kTwo ? a.vals : cur)[nb[t]] : 0.f;
#pragma unroll
          for (int t = 0; t < 8; t++)
            if (nb[t] >= 0) kahan_add(s, c, x[t]);
        }
        sum = __fsub_rn(s, c);
      }
      unsigned med = __ballot_sync(IG_FULL, vi < a.nodes && !skip && d > kLight && d <= a.hub_degree);
      // four medium vertices at a time, one per sub-warp of 8 lanes
      while (a.subwarp && med) {
        int o[4];
#pragma unroll
        for (int q = 0; q < 4; q++) {
          o[q] = med ? __ffs(med) - 1 : -1;
          if (med) med &= med - 1;
        }
        const int q = lane >> 3;
        const int mine = q == 0 ? o[0] : q == 1 ? o[1] : q == 2 ? o[2] : o[3];
        const int mb = __shfl_sync(IG_FULL, b, mine < 0 ? 0 : mine);
        const int me = __shfl_sync(IG_FULL, e, mine < 0 ? 0 : mine);
        float h, l;
        subwarp8_gather_sum<kTwo>(a.nlist, kTwo ? a.vals : cur, mb, mine < 0 ? mb : me, h, l);
        const float tot = __fadd_rn(h, l);
#pragma unroll
        for (int r = 0; r < 4; r++) {
          const float t = __shfl_sync(IG_FULL, tot, r * 8);
          if (lane == o[r]) sum = t;
        }
      }
      // two medium vertices at a time, so short ones do not each pay a full
      // gather latency in turn
      while (med) {
        const int l1 = __ffs(med) - 1;
        med &= med - 1;
        const int l2 = med ? __ffs(med) - 1 : l1;
        if (med) med &= med - 1;
        const int mb1 = __shfl_sync(IG_FULL, b, l1), me1 = __shfl_sync(IG_FULL, e, l1);
        int mb2 = __shfl_sync(IG_FULL, b, l2), me2 = __shfl_sync(IG_FULL, e, l2);
        if (l2 == l1) me2 = mb2;  // no second vertex
        float h1, o1, h2, o2;
        warp_gather_sum2<kTwo>(a.nlist, kTwo ? a.vals : cur, mb1, me1, mb2, me2, h1, o1, h2, o2);
        if (lane == l1) sum = __fadd_rn(h1, o1);
        if (l2 != l1 && lane == l2) sum = __fadd_rn(h2, o2);
      }
      double verr = 0.0;
      const bool upd = vi < a.nodes && !skip && d <= a.hub_degree;
      if (upd) {
        const float old = a.scores[v];
        const float nw = __fadd_rn(vbase, __fmul_rn(a.damp, sum));
        a.scores[v] = nw;
        nxt[v] = __fdiv_rn(nw, (float)vdegree(a, v));
        verr = (double)fabsf(__fsub_rn(nw, old));
        err += fix(verr);
      }
      if (kBatched) warp_add_by_graph(gcur, vg, verr, upd);
      grp = gnext;
      if (claim) {
        gnext = unit_first(__shfl_sync(IG_FULL, claimed, 0));
        uend = min(gnext + unit, ngroups);
      } else {
        gnext = dyn ? gnext + 1 : gnext + nwarps;
      }
    }
    // ---- phase B: combine hub chunks in chunk order
    if (nh > 0) {
      if (!grid_sync(ctl, a.timeout_ns, gb)) return;
      for (int h = warp_g; h < nh; h += nwarps) {
        const int c0 = a.chunk_base[h], c1 = a.chunk_base[h + 1];
        float hi = 0.f, lo = 0.f;
        for (int c = c0 + lane; c < c1; c += 32) {
          const float2 p = a.partial[c];
          pair_add(hi, lo, p.x, p.y);
        }
        warp_pair_reduce(hi, lo);
        const int v = a.hubs[h];
        int hg = 0;
        float hbase = a.base;
        if (kBatched) {
          hg = a.vgraph[v];
          if (frozen(hg)) continue;
          hbase = __fdiv_rn(__fsub_rn(1.0f, a.damp),
                            (float)(__ldg(&a.graph_vptr[hg + 1]) - __ldg(&a.graph_vptr[hg])));
        }
        if (lane == 0) {
          const float sum = __fadd_rn(hi, lo);
          const float old = a.scores[v];
          const float nw = __fadd_rn(hbase, __fmul_rn(a.damp, sum));
          a.scores[v] = nw;
          nxt[v] = __fdiv_rn(nw, (float)vdegree(a, v));
          const double herr = (double)fabsf(__fsub_rn(nw, old));
          err += fix(herr);
          if (kBatched && herr != 0.0) atomicAdd(&gcur[hg], herr);
        }
      }
    }
    // block partial: integer (or the batched form's double, as bits)
    unsigned long long berr;
    if constexpr (kBatched) berr = (unsigned long long)__double_as_longlong(block_sum_double(err, (double*)s_red));
    else berr = block_sum_u64(err, s_red);
    unsigned long long* slot = a.blkerr + (it & 1) * G;
    if (threadIdx.x == 0) slot[blockIdx.x] = berr;
    if (!grid_sync(ctl, a.timeout_ns, gb)) return;
    // the grid's residual: warp 0 of every block sums the block partials
    // (integers: the same total in every block, whatever the order)
    __shared__ double s_res;
    if (threadIdx.x < 32) {
      Err r = 0;
      for (int b = threadIdx.x; b < G; b += 32) {
        const unsigned long long x = ld_relaxed(&slot[b]);
        if constexpr (kBatched) r += __longlong_as_double((long long)x);
        else r += x;
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) r += __shfl_xor_sync(IG_FULL, r, o);
      if (threadIdx.x == 0) {
        if constexpr (kBatched) s_res = r;
        else s_res = (double)r / kFix;
      }
    }
    __syncthreads();
    residual = s_res;
    float* t = cur;
    cur = nxt;
    nxt = t;
    if (!kBatched) {
      if (residual < (double)a.eps) break;
    } else {
      // record each graph's iteration count when it converges; stop when all did
      __shared__ int s_active;
      if (threadIdx.x == 0) s_active = 0;
      __syncthreads();
      int active = 0;
      for (int g = threadIdx.x; g < a.graphs; g += blockDim.x) {
        const bool conv = ld_relaxed(&gcur[g]) < (double)a.eps;
        if (!conv) active = 1;
        if (blockIdx.x == 0 && conv && a.giters[g] == 0) a.giters[g] = it;
      }
      if (active) s_active = 1;
      __syncthreads();
      if (s_active == 0) break;
    }
  }
  if (kBatched && blockIdx.x == 0)
    for (int g = threadIdx.x; g < a.graphs; g += blockDim.x)
      if (a.giters[g] == 0) a.giters[g] = it;
  if (gtid == 0) {
    ctl->iterations = it;
    ctl->residual = residual;
  }
}

}  // namespace

static int pr_launch(IgExec* ex, const ig_csr* dg, const int* d_degree, float* d_scores, float epsilon,
                     int max_iter, const int* d_graph_vptr, int graphs, int* d_iters) {
  const IgOptions& o = ig_exec_options(ex);
  const int n = dg->nodes;
  const int hub_degree = std::max(o.pr_hub_degree, 32);
  const int chunk = std::max(o.pr_chunk, 32);
  const long long max_hubs = (long long)dg->edges / (hub_degree + 1) + 1;
  const long long max_chunks = (long long)dg->edges / chunk + max_hubs + 1;
  const int max_blocks = ex->sms * 32;
  void *ca, *cb, *hubs, *cbase, *chub, *part, *blk, *blkerr, *gres = nullptr, *vgraph = nullptr;
  int rc;
  if ((rc = ig_scratch_get(ex->scratch, IG_SLOT_F0, (size_t)n * sizeof(float), &ca))) return rc;
  if ((rc = ig_scratch_get(ex->scratch, IG_SLOT_F1, (size_t)n * sizeof(float), &cb))) return rc;
  if ((rc = ig_scratch_get(ex->scratch, IG_SLOT_Q0, (size_t)max_hubs * sizeof(int), &hubs))) return rc;
  if ((rc = ig_scratch_get(ex->scratch, IG_SLOT_Q1, (size_t)(max_hubs + 1) * sizeof(int), &cbase))) return rc;
  if ((rc = ig_scratch_get(ex->scratch, IG_SLOT_Q2, (size_t)max_chunks * sizeof(float2), &part))) return rc;
  if ((rc = ig_scratch_get(ex->scratch, IG_SLOT_Q3, (size_t)max_chunks * sizeof(int), &chub))) return rc;
  if ((rc = ig_scratch_get(ex->scratch, IG_SLOT_V0, (size_t)2 * max_blocks * sizeof(int), &blk))) return rc;
  if ((rc = ig_scratch_get(ex->scratch, IG_SLOT_BLK, (size_t)2 * max_blocks * sizeof(double), &blkerr))) return rc;
  // two-pass form: edge values gathered in one dense pass (needs a 16-byte aligned nlist)
  void* vals = nullptr;
  const bool two = o.pr_two_pass && dg->edges > 0 && ((uintptr_t)dg->nlist & 15) == 0;
  if (two && (rc = ig_scratch_get(ex->scratch, IG_SLOT_E0, (size_t)dg->edges * sizeof(float), &vals))) return rc;
  if (d_graph_vptr) {
    if ((rc = ig_scratch_get(ex->scratch, IG_SLOT_V1, (size_t)3 * graphs * sizeof(double), &gres))) return rc;
    if ((rc = ig_scratch_get(ex->scratch, IG_SLOT_G2, (size_t)n * sizeof(int), &vgraph))) return rc;
    if ((rc = ig_cuda_check((int)cudaMemsetAsync(gres, 0, (size_t)3 * graphs * sizeof(double), ex->stream), "memset")))
      return rc;
    if ((rc = ig_cuda_check((int)cudaMemsetAsync(d_iters, 0, (size_t)graphs * sizeof(int), ex->stream), "memset")))
      return rc;
  }
  if ((rc = ig_exec_reset(ex))) return rc;
  const float damp = 0.85f;
  const float base = (1.0f - damp) / (float)n;
  PrArgs a{dg->nindex, dg->nlist, d_degree, n, dg->edges, d_scores, (float*)ca, (float*)cb, (int*)hubs,
           (int*)cbase, (int*)chub, (float2*)part, (int*)blk, (unsigned long long*)blkerr, ex->d_ctl, epsilon, max_iter, base, damp,
           ex->timeout_ns, hub_degree, chunk, o.pr_prefetch, o.pr_subwarp, (float*)vals, d_graph_vptr, graphs,
           (double*)gres, d_iters, (int*)vgraph, o.pr_static_pct};
  void* args[] = {&a};
  const int bps = o.pr_blocks_per_sm > 0 ? o.pr_blocks_per_sm : o.blocks_per_sm;
  const int cap = bps > 0 ? std::min(bps, 32) : 32;
  const void* fn = d_graph_vptr ? (two ? (const void*)pr_persistent<true, true> : (const void*)pr_persistent<true, false>)
                                : (two ? (const void*)pr_persistent<false, true> : (const void*)pr_persistent<false, false>);
  return ig_launch_coop(ex, fn, kThreads, 0, cap, args, nullptr);
}

int igk_pr(IgExec* ex, const ig_csr* dg, const int* d_degree, float* d_scores, float epsilon, int max_iter) {
  return pr_launch(ex, dg, d_degree, d_scores, epsilon, max_iter, nullptr, 0, nullptr);
}

int igk_pr_batched(IgExec* ex, const ig_csr* dg, const int* d_graph_vptr, int graphs, float* d_scores,
                   float epsilon, int max_iter, int* d_iters) {
  return pr_launch(ex, dg, nullptr, d_scores, epsilon, max_iter, d_graph_vptr, graphs, d_iters);
}
