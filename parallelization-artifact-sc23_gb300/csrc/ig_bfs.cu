// Breadth-first search: one persistent, cooperatively launched kernel per
// call.  Replaces the per-level host loop of the reference CUDA variants
// (e.g. codes/cuda/bfs-cuda/BFS_CUDA_V_Topo_Push_Determ_IntType_ReadWrite_
// NonPersist_Atomic_Thread_NoBoundsBug2_NoBoundsBug1.cu:56-108, one launch
// plus a 4-byte device-to-host copy per level) by grid barriers on the device.
//
// Output semantics follow include/bfs_vertex_cuda.h: dist[v] = number of
// edges on a shortest path from src, INT_MAX (`maxval`, :46) if unreachable.
//
// Each level is either
//   top-down : the frontier queue is expanded 32 vertices per warp with the
//              load-balanced warp expansion; a vertex is claimed with one
//              atomicCAS on dist (INT_MAX -> level+1) and appended to the next
//              queue with one atomic per warp (the worklist idiom of the
//              reference's *_Data_*_NonDup variants, warp-aggregated);
//              vertices above the hub degree are expanded by the whole grid;
//   bottom-up: every unvisited vertex scans its neighbours for one at the
//              current level and stops at the first (Beamer's direction
//              optimisation; the graph is symmetric as in the reference).
// The direction is chosen from the frontier's edge count and vertex count,
// identically in every block after the level's barrier.
#include "ig_device.cuh"
#include "ig_options.h"

namespace {

constexpr int kThreads = 256;

struct BfsArgs {
  const int* __restrict__ nindex;
  const int* __restrict__ nlist;
  int nodes;
  long long edges;
  int src;
  int* dist;
  int* qa;
  int* qb;
  int* hubs;
  IgCtl* ctl;
  unsigned long long timeout_ns;
  int hub_degree;
  int alpha;
  int beta;
  const int* sources;  // batched form: one source per graph of a disjoint union (else null)
  int nsources;
  // level bitmaps (three of ceil(nodes / 32) words, by level % 3): the
  // bottom-up scan tests a neighbour's bit instead of reading its distance.
  // Null: the scan reads distances (the allocation-free entry point).
  unsigned* bits;
  // when set, the source is read from the device: the vertex encoded in the
  // low word of *src_key as 0xffffffff - id (connected components' seed)
  const unsigned long long* src_key;
  // bottom-up levels: 0 = every warp scans its fixed share of 32-vertex
  // chunks (grid stride); g > 0 = after a first group by warp index, warps
  // take groups of g chunks from a per-level counter, each claimed while the
  // previous group is scanned, so the level's end is even
  int bu_claim;
  // > 0: stop after this many levels (vertices farther away stay INT_MAX);
  // connected components use it to label only the near part of the giant
  // component by BFS on a high-diameter graph
  int max_level;
};

// Hot counters of the control block, slot s = level % 3: hot32(s) size of the
// queue built during the level, hot32(3 + s) its hub count, hot64(6 + s) the
// sum of degrees of the queued vertices, hot32(9 + s) bottom-up groups claimed.

__global__ void __launch_bounds__(kThreads) bfs_persistent(BfsArgs a_in) {
  BfsArgs a = a_in;
  using namespace ig;
  IgCtl* ctl = a.ctl;
  GridBar gb;  // this block's view of the barrier generation
  const int lane = lane_id();
  const long long gtid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long gthreads = (long long)gridDim.x * blockDim.x;
  const int warp_g = (int)(gtid >> 5);
  const int nwarps = (int)(gthreads >> 5);
  if (a.src_key) a.src = (int)(0xffffffffu - (unsigned)(*a.src_key & 0xffffffffull));
  const long long nwords = ((long long)a.nodes + 31) >> 5;
  if (a.bits)  // all three level bitmaps start empty but for a single source's bit
    for (long long i = gtid; i < 3 * nwords; i += gthreads)
      a.bits[i] = (a.sources == nullptr && i == (a.src >> 5)) ? 1u << (a.src & 31) : 0u;

  long long src_deg = 0;
  int cur_size = 1;
  if (a.sources == nullptr) {
    for (long long v = gtid; v < a.nodes; v += gthreads) a.dist[v] = (v == a.src) ? 0 : kInf;
    if (gtid == 0) a.qa[0] = a.src;
    src_deg = __ldg(&a.nindex[a.src + 1]) - __ldg(&a.nindex[a.src]);
  } else {
    // several sources (one per graph of a disjoint union): all start at level 0
    for (long long v = gtid; v < a.nodes; v += gthreads) a.dist[v] = kInf;
    if (!grid_sync(ctl, a.timeout_ns, gb)) return;
    for (long long i = gtid; i < a.nsources; i += gthreads) {
      a.dist[a.sources[i]] = 0;
      a.qa[i] = a.sources[i];
      if (a.bits) atomicOr(&a.bits[a.sources[i] >> 5], 1u << (a.sources[i] & 31));
    }
    cur_size = a.nsources;
    src_deg = a.edges / 2;  // start top-down; the switch rule takes over after level 0
  }
  if (!grid_sync(ctl, a.timeout_ns, gb)) return;

  int* cur = a.qa;
  int* nxt = a.qb;
  bool bottom_up = false;
  long long unexplored = a.edges - src_deg;
  int level = 0;

  while (cur_size > 0 && (a.max_level <= 0 || level < a.max_level)) {
    const int slot = level % 3;
    if (gtid == 0) {
      const int ns = (level + 1) % 3;
      *hot32(ctl, ns) = 0;
      *hot32(ctl, 3 + ns) = 0;
      *hot64(ctl, 6 + ns) = 0;
      *hot32(ctl, 9 + ns) = 0;
    }
    int* qsize = hot32(ctl, slot);
    int* nhub = hot32(ctl, 3 + slot);
    unsigned long long* fedges = hot64(ctl, 6 + slot);
    const int next_level = level + 1;
    // this level's bits (read), the next level's (written; cleared during the
    // previous level), and the previous level's, cleared now for level + 2
    const unsigned* cbits = a.bits ? a.bits + (long long)(level % 3) * nwords : nullptr;
    unsigned* nbits = a.bits ? a.bits + (long long)((level + 1) % 3) * nwords : nullptr;
    if (a.bits && level > 0) {
      unsigned* obits = a.bits + (long long)((level + 2) % 3) * nwords;
      for (long long i = gtid; i < nwords; i += gthreads) obits[i] = 0u;
    }

    if (!bottom_up) {
      auto visit = [&](bool act, int e, int) {
        bool claim = false;
        int w = 0;
        long long wdeg = 0;
        if (act) {
          w = __ldg(&a.nlist[e]);
          if (a.dist[w] == kInf && atomicCAS(&a.dist[w], kInf, next_level) == kInf) {
            claim = true;
            wdeg = __ldg(&a.nindex[w + 1]) - __ldg(&a.nindex[w]);
            if (nbits) atomicOr(&nbits[w >> 5], 1u << (w & 31));
          }
        }
        warp_append_w(claim, w, wdeg, nxt, qsize, fedges, a.nodes, ctl);
      };
      for (int base = warp_g * 32; base < cur_size; base += nwarps * 32) {
        const int i = base + lane;
        int v = 0, beg = 0, deg = 0;
        if (i < cur_size) {
          v = cur[i];
          beg = __ldg(&a.nindex[v]);
          deg = __ldg(&a.nindex[v + 1]) - beg;
        }
        const bool hub = deg > a.hub_degree;
        warp_append(hub, v, a.hubs, nhub, a.nodes, ctl);
        warp_expand(beg, hub ? 0 : deg, visit);
      }
      if (!grid_sync(ctl, a.timeout_ns, gb)) return;
      const int nh = ld_relaxed(nhub);
      if (nh > 0) {
        grid_expand_hubs(a.nindex, a.hubs, nh, [&](bool act, int e, int) { visit(act, e, 0); });
        if (!grid_sync(ctl, a.timeout_ns, gb)) return;
      }
    } else {
      // one 32-vertex chunk starting at `base` (a multiple of 32)
      auto scan_chunk = [&](long long base) {
        const long long v = base + lane;
        bool found = false;
        long long deg = 0;
        if (v < a.nodes && a.dist[v] == kInf) {
          const int b = __ldg(&a.nindex[v]), e = __ldg(&a.nindex[v + 1]);
          deg = e - b;
          if (cbits) {
            // four neighbours per step: their index loads and bit tests are
            // independent, so they are issued together (plain loads: the bits
            // were written by this kernel during the previous level)
            for (int k = b; k < e && !found; k += 4) {
              int w[4];
#pragma unroll
              for (int t = 0; t < 4; t++) w[t] = k + t < e ? __ldg(&a.nlist[k + t]) : -1;
#pragma unroll
              for (int t = 0; t < 4; t++) found |= w[t] >= 0 && ((cbits[w[t] >> 5] >> (w[t] & 31)) & 1u);
            }
          } else {
            for (int k = b; k < e; k++) {
              if (a.dist[__ldg(&a.nlist[k])] == level) {
                found = true;
                break;
              }
            }
          }
          if (found) a.dist[v] = next_level;
        }
        if (nbits) {  // the warp's 32 consecutive vertices fill one word of the next bitmap, its only writer
          const unsigned m = __ballot_sync(IG_FULL, found);
          if (lane == 0 && (base >> 5) < nwords) nbits[base >> 5] = m;
        }
        warp_append_w(found, (int)v, deg, nxt, qsize, fedges, a.nodes, ctl);
      };
      if (a.bu_claim <= 0) {
        for (long long base = gtid & ~31LL; base < a.nodes; base += gthreads) scan_chunk(base);
      } else {
        const long long nchunks = ((long long)a.nodes + 31) >> 5;
        const long long G = a.bu_claim;
        int* bgrab = hot32(ctl, 9 + slot);
        long long q = warp_g;  // group index: chunks [q * G, q * G + G)
        while (q * G < nchunks) {
          int ahead = 0;
          if (lane == 0) ahead = atomicAdd(bgrab, 1);
          for (long long c = q * G; c < min(q * G + G, nchunks); c++) scan_chunk(c << 5);
          q = nwarps + (long long)__shfl_sync(IG_FULL, ahead, 0);
        }
      }
      if (!grid_sync(ctl, a.timeout_ns, gb)) return;
    }

    const int nf = ld_relaxed(qsize);
    const long long mf = (long long)ld_relaxed(fedges);
    unexplored -= mf;
    level = next_level;
    if (!bottom_up) {
      if (a.alpha > 0 && mf > unexplored / a.alpha) bottom_up = true;  // alpha 0: top-down only
    } else {
      if ((long long)nf * a.beta < a.nodes) bottom_up = false;
    }
    cur_size = nf;
    int* t = cur;
    cur = nxt;
    nxt = t;
  }
  if (gtid == 0) ctl->iterations = level;
}

}  // namespace

int igk_bfs(IgExec* ex, const ig_csr* dg, int src, int* d_dist) {
  const size_t vb = (size_t)dg->nodes * sizeof(int);
  void *qa, *qb, *hubs;
  int rc;
  if ((rc = ig_scratch_get(ex->scratch, IG_SLOT_Q0, vb, &qa))) return rc;
  if ((rc = ig_scratch_get(ex->scratch, IG_SLOT_Q1, vb, &qb))) return rc;
  if ((rc = ig_scratch_get(ex->scratch, IG_SLOT_Q2, vb, &hubs))) return rc;
  void* bits;
  if ((rc = ig_scratch_get(ex->scratch, IG_SLOT_V0, 3 * (((size_t)dg->nodes + 31) / 32) * 4, &bits))) return rc;
  if ((rc = ig_exec_reset(ex))) return rc;
  const IgOptions& o = ig_exec_options(ex);
  BfsArgs a{dg->nindex, dg->nlist, dg->nodes, dg->edges, src, d_dist, (int*)qa, (int*)qb, (int*)hubs,
            ex->d_ctl, ex->timeout_ns, o.bfs_hub_degree, o.bfs_alpha, o.bfs_beta, nullptr, 0,
            o.bfs_bitmap ? (unsigned*)bits : nullptr, nullptr, o.bfs_bu_claim};
  void* args[] = {&a};
  return ig_launch_coop(ex, (const void*)bfs_persistent, kThreads, 0, o.blocks_per_sm, args, nullptr);
}

// As igk_bfs, the source read on the device from *d_src_key (see BfsArgs),
// stopping after max_level levels when max_level > 0.
int igk_bfs_keyed(IgExec* ex, const ig_csr* dg, const unsigned long long* d_src_key, int* d_dist, int max_level) {
  const int src = 0;
  const size_t vb = (size_t)dg->nodes * sizeof(int);
  void *qa, *qb, *hubs;
  int rc;
  if ((rc = ig_scratch_get(ex->scratch, IG_SLOT_Q0, vb, &qa))) return rc;
  if ((rc = ig_scratch_get(ex->scratch, IG_SLOT_Q1, vb, &qb))) return rc;
  if ((rc = ig_scratch_get(ex->scratch, IG_SLOT_Q2, vb, &hubs))) return rc;
  void* bits;
  if ((rc = ig_scratch_get(ex->scratch, IG_SLOT_V0, 3 * (((size_t)dg->nodes + 31) / 32) * 4, &bits))) return rc;
  if ((rc = ig_exec_reset(ex))) return rc;
  const IgOptions& o = ig_exec_options(ex);
  BfsArgs a{dg->nindex, dg->nlist, dg->nodes, dg->edges, src, d_dist, (int*)qa, (int*)qb, (int*)hubs,
            ex->d_ctl, ex->timeout_ns, o.bfs_hub_degree, o.bfs_alpha, o.bfs_beta, nullptr, 0,
            o.bfs_bitmap ? (unsigned*)bits : nullptr, d_src_key, o.bfs_bu_claim, max_level};
  void* args[] = {&a};
  return ig_launch_coop(ex, (const void*)bfs_persistent, kThreads, 0, o.blocks_per_sm, args, nullptr);
}

// Multi-source form for a disjoint union of graphs: d_sources[i] (global ids,
// one per graph) all start at level 0, so each graph gets its own BFS levels.
int igk_bfs_multi(IgExec* ex, const ig_csr* dg, const int* d_sources, int nsources, int* d_dist) {
  const size_t vb = (size_t)dg->nodes * sizeof(int);
  void *qa, *qb, *hubs;
  int rc;
  if ((rc = ig_scratch_get(ex->scratch, IG_SLOT_Q0, vb, &qa))) return rc;
  if ((rc = ig_scratch_get(ex->scratch, IG_SLOT_Q1, vb, &qb))) return rc;
  if ((rc = ig_scratch_get(ex->scratch, IG_SLOT_Q2, vb, &hubs))) return rc;
  void* bits;
  if ((rc = ig_scratch_get(ex->scratch, IG_SLOT_V0, 3 * (((size_t)dg->nodes + 31) / 32) * 4, &bits))) return rc;
  if ((rc = ig_exec_reset(ex))) return rc;
  const IgOptions& o = ig_exec_options(ex);
  BfsArgs a{dg->nindex, dg->nlist, dg->nodes, dg->edges, 0, d_dist, (int*)qa, (int*)qb, (int*)hubs,
            ex->d_ctl, ex->timeout_ns, o.hub_degree, o.bfs_alpha, o.bfs_beta, d_sources, nsources,
            o.bfs_bitmap ? (unsigned*)bits : nullptr, nullptr, o.bfs_bu_claim};
  void* args[] = {&a};
  return ig_launch_coop(ex, (const void*)bfs_persistent, kThreads, 0, o.blocks_per_sm, args, nullptr);
}

// Launch on caller-provided scratch (two queues and a hub list of `nodes`
// ints each, and the control block already in ex->d_ctl).  Allocates nothing
// and keeps no host-side cache: the occupancy query and the cooperative
// launch are the only runtime calls.
int igk_bfs_launch_prealloc(IgExec* ex, const ig_csr* dg, int src, int* d_dist, int* qa, int* qb, int* hubs) {
  int per_sm = 0;
  int rc = ig_cuda_check((int)cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, bfs_persistent, kThreads, 0),
                         "occupancy");
  if (rc) return rc;
  const IgOptions& o = ig_exec_options(ex);
  if (o.blocks_per_sm > 0) per_sm = std::min(per_sm, o.blocks_per_sm);
  if (per_sm < 1) return ig_fail(IG_ERR_CUDA, "persistent kernel cannot be resident (occupancy 0)");
  BfsArgs a{dg->nindex, dg->nlist, dg->nodes, dg->edges, src, d_dist, qa, qb, hubs,
            ex->d_ctl, ex->timeout_ns, o.hub_degree, o.bfs_alpha, o.bfs_beta, nullptr, 0, nullptr, nullptr};
  void* args[] = {&a};
  rc = ig_cuda_check((int)cudaLaunchCooperativeKernel((const void*)bfs_persistent, dim3(per_sm * ex->sms),
                                                      dim3(kThreads), args, 0, ex->stream),
                     "cooperative launch");
  if (rc == IG_OK) ig_count_launches(1);
  return rc;
}
