// Maximal independent set by priority rounds: one persistent, cooperatively
// launched kernel per call.
//
// Reference rule (codes/cpp/mis-cpp/MIS_CPP_V_Topo_Push_IntType_Atomic_
// CopyDeterm_Block.cpp:50-73, priorities from include/mis_vertex_cpp.h:135-140
// applied to v + 712313887 and compared as UNSIGNED int): an undecided vertex
// joins the set when no non-excluded neighbour has a larger (priority, id);
// it then excludes all its neighbours; rounds repeat until nothing is
// undecided.  With fixed priorities that process has exactly one outcome --
// the greedy set taken in decreasing (priority, id) order: v is in the set iff
// no larger neighbour is in the set.  Any schedule that (1) includes v only
// once every larger neighbour is excluded and (2) excludes v only once a
// neighbour is included reaches that same set, because statuses only ever
// move from undecided to decided.  This kernel is such a schedule:
//   - an undecided vertex scans only its LARGER neighbours, starting where its
//     previous scan stopped (excluded vertices stay excluded): an included one
//     excludes it, an undecided one blocks it until a later round, and
//     reaching the end includes it and pushes "excluded" to all neighbours;
//   - statuses are updated in place (no per-round copy, unlike :89-103);
//   - the undecided vertices are compacted into a worklist each round
//     (staged per warp in shared memory, one atomic per 32 entries), so
//     later rounds touch only what is left;
//   - vertices with more than 32 neighbours are scanned 32 at a time by the
//     whole warp with ballots;
//   - groups of 32-entry chunks (up to 8 chunks, sized so every warp takes
//     about 8 groups): the first static_pct percent dealt round-robin (no
//     atomics), the rest taken one at a time from a per-round counter, so a
//     run of high-degree vertices in consecutive ids (degree-ordered input)
//     does not sit on a few warps and the counter is not hit by every
//     group of the round.
// The result equals the reference C++ CopyDeterm set bit for bit.  (The CUDA
// variants compare priorities as signed int and reach a different set.)
#include "ig_device.cuh"
#include "ig_options.h"

namespace {

constexpr int kThreads = 256;
constexpr int kUndecided = 0, kIncluded = 1, kExcluded = 2;

struct MisArgs {
  const int* __restrict__ nindex;
  const int* __restrict__ nlist;
  int nodes;
  int* status;
  int* resume;
  int* wa;
  int* wb;
  IgCtl* ctl;
  unsigned long long timeout_ns;
  int static_pct;  // percent of a round's groups dealt round-robin
};

__device__ __forceinline__ int load_status(const int* s, int v) { return *((const volatile int*)s + v); }

// (pn, n) > (pv, v) in the reference's order
__device__ __forceinline__ bool larger(unsigned pn, int n, unsigned pv, int v) {
  return pn > pv || (pn == pv && n > v);
}

__global__ void __launch_bounds__(kThreads) mis_persistent(MisArgs a) {
  using namespace ig;
  IgCtl* ctl = a.ctl;
  GridBar gb;  // this block's view of the barrier generation
  const int lane = lane_id();
  const long long gtid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long gthreads = (long long)gridDim.x * blockDim.x;
  const long long warp_g = gtid >> 5, nwarps = gthreads >> 5;
  __shared__ int s_wbuf[kThreads / 32][kWarpBuf];  // per-warp staging of worklist appends
  int* wbuf = s_wbuf[threadIdx.x >> 5];
  int wbuf_n = 0;

  for (long long v = gtid; v < a.nodes; v += gthreads) {
    a.status[v] = kUndecided;
    a.resume[v] = __ldg(&a.nindex[v]);
  }
  if (!grid_sync(ctl, a.timeout_ns, gb)) return;

  int* cur = a.wa;
  int* nxt = a.wb;
  int cur_size = a.nodes;  // round 0 walks all vertices directly
  int round = 0;
  while (cur_size > 0) {
    const int slot = round % 3;
    if (gtid == 0) {
      *hot32(ctl, (round + 1) % 3) = 0;      // worklist size of the next round
      *hot32(ctl, 3 + (round + 1) % 3) = 0;  // its chunks taken
    }
    int* wsize = hot32(ctl, slot);
    int* grab = hot32(ctl, 3 + slot);
    const int gch = (int)max(1LL, min(8LL, (long long)cur_size / (nwarps * 256)));  // chunks per group
    const long long ngroups = ((long long)cur_size + 32 * gch - 1) / (32 * gch);
    const long long nstatic = max(min(ngroups, nwarps), ngroups * a.static_pct / 100);
    long long grp = warp_g;
    if (grp >= nstatic) {
      long long nb = 0;
      if (lane == 0) nb = nstatic + atomicAdd(grab, 1);
      grp = __shfl_sync(IG_FULL, nb, 0);
    }
    for (long long base0 = grp * 32 * gch; grp < ngroups; base0 = grp * 32 * gch) {
      for (int sc = 0; sc < gch && base0 + 32 * sc < cur_size; sc++) {
        const long long base = base0 + 32 * sc;
        const long long i = base + lane;
        int v = 0, beg = 0, end = 0;
        bool live = false;
        if (i < cur_size) {
          v = (round == 0) ? (int)i : cur[i];
          live = load_status(a.status, v) == kUndecided;
          beg = a.resume[v];
          end = __ldg(&a.nindex[v + 1]);
        }
        const unsigned pv = mis_priority(v);
        bool blocked = false;
        // light vertices: sequential scan by the owning lane
        const bool light = live && (end - beg) <= 32;
        if (light) {
          // four neighbours per step: their ids, then the statuses of the
          // larger ones, loaded together; the first blocking one in list
          // order decides, as in a one-by-one scan
          int outcome = kIncluded;
          int k = beg;
          for (; k < end; k += 4) {
            int n[4], st[4];
            bool big[4];
#pragma unroll
            for (int t = 0; t < 4; t++) n[t] = k + t < end ? __ldg(&a.nlist[k + t]) : 0;
#pragma unroll
            for (int t = 0; t < 4; t++) {
              big[t] = k + t < end && larger(mis_priority(n[t]), n[t], pv, v);
              st[t] = big[t] ? load_status(a.status, n[t]) : kExcluded;
            }
            int stop = -1;
#pragma unroll
            for (int t = 3; t >= 0; t--)
              if (st[t] != kExcluded) stop = t;
            if (stop >= 0) {
              const int s = stop == 0 ? st[0] : stop == 1 ? st[1] : stop == 2 ? st[2] : st[3];
              outcome = s == kIncluded ? kExcluded : kUndecided;
              k += stop;
              break;
            }
          }
          if (outcome == kIncluded) {
            a.status[v] = kIncluded;
            for (int q = __ldg(&a.nindex[v]); q < end; q++) a.status[__ldg(&a.nlist[q])] = kExcluded;
          } else if (outcome == kExcluded) {
            a.status[v] = kExcluded;
          } else {
            a.resume[v] = k;
            blocked = true;
          }
        }
        // heavy vertices: one at a time, the warp scans 32 neighbours per step
        unsigned heavy = __ballot_sync(IG_FULL, live && !light);
        while (heavy) {
          const int src_lane = __ffs(heavy) - 1;
          heavy &= heavy - 1;
          const int hv = __shfl_sync(IG_FULL, v, src_lane);
          const int hb = __shfl_sync(IG_FULL, beg, src_lane);
          const int he = __shfl_sync(IG_FULL, end, src_lane);
          const unsigned ph = mis_priority(hv);
          int outcome = kIncluded, stop = he;
          for (int k0 = hb; k0 < he; k0 += 32) {
            const int k = k0 + lane;
            bool inc = false, und = false;
            if (k < he) {
              const int n = __ldg(&a.nlist[k]);
              if (larger(mis_priority(n), n, ph, hv)) {
                const int s = load_status(a.status, n);
                inc = s == kIncluded;
                und = s == kUndecided;
              }
            }
            const unsigned mi = __ballot_sync(IG_FULL, inc);
            const unsigned mu = __ballot_sync(IG_FULL, und);
            if (mi) { outcome = kExcluded; break; }
            if (mu) { outcome = kUndecided; stop = k0 + __ffs(mu) - 1; break; }
          }
          if (outcome == kIncluded) {
            if (lane == 0) a.status[hv] = kIncluded;
            const int b0 = __ldg(&a.nindex[hv]);
            for (int q = b0 + lane; q < he; q += 32) a.status[__ldg(&a.nlist[q])] = kExcluded;
          } else if (outcome == kExcluded) {
            if (lane == 0) a.status[hv] = kExcluded;
          } else {
            if (lane == 0) a.resume[hv] = stop;
            if (lane == src_lane) blocked = true;
          }
        }
        const int bv[1] = {v};
        warp_buf_append<1>(blocked ? 1 : 0, bv, wbuf, wbuf_n, nxt, wsize, a.nodes, ctl);
      }
      if (grp + nwarps < nstatic) {
        grp += nwarps;
      } else {
        long long nb = 0;
        if (lane == 0) nb = nstatic + atomicAdd(grab, 1);
        grp = __shfl_sync(IG_FULL, nb, 0);
      }
    }
    warp_buf_flush(wbuf, wbuf_n, nxt, wsize, a.nodes, ctl);
    if (!grid_sync(ctl, a.timeout_ns, gb)) return;
    cur_size = ld_relaxed(wsize);
    round++;
    int* t = cur;
    cur = nxt;
    nxt = t;
  }
  if (gtid == 0) ctl->iterations = round;
}

}  // namespace

int igk_mis(IgExec* ex, const ig_csr* dg, int* d_status, unsigned int* d_prio) {
  (void)d_prio;
  const size_t vb = (size_t)dg->nodes * sizeof(int);
  void *resume, *wa, *wb;
  int rc;
  if ((rc = ig_scratch_get(ex->scratch, IG_SLOT_V0, vb, &resume))) return rc;
  if ((rc = ig_scratch_get(ex->scratch, IG_SLOT_Q0, vb, &wa))) return rc;
  if ((rc = ig_scratch_get(ex->scratch, IG_SLOT_Q1, vb, &wb))) return rc;
  if ((rc = ig_exec_reset(ex))) return rc;
  const IgOptions& o = ig_exec_options(ex);
  MisArgs a{dg->nindex, dg->nlist,   dg->nodes,    d_status,       (int*)resume,
            (int*)wa,   (int*)wb,    ex->d_ctl,    ex->timeout_ns, o.mis_static_pct};
  void* args[] = {&a};
  return ig_launch_coop(ex, (const void*)mis_persistent, kThreads, 0, o.blocks_per_sm, args, nullptr);
}
