// Single-source shortest paths with int32 weights: one persistent,
// cooperatively launched kernel per call running a near/far worklist
// (two-bucket delta stepping).  Replaces the per-round host loop of the
// reference's worklist variants (e.g. codes/cuda/sssp-cuda/SSSP_CUDA_V_Data_
// Push_Determ_IntType_ReadModifyWrite_NonPersist_CudaAtomic_Thread_
// NoBoundsBug2_NoBoundsBug1_NonDup.cu:62-126), whose relaxation is
// `atomicMin(&dist[dst], dist[src] + eweight[i])` and whose worklist is
// de-duplicated with a per-vertex iteration stamp (atomicMax(&time[dst], iter)).
//
// Output semantics follow include/sssp_vertex_cuda.h: shortest distance,
// INT_MAX if unreachable (checked there against CPUserialDijkstra, :74-99).
//
// Near phase: the near queue is expanded in chunks of 32 vertices per warp
// (the first static_pct percent of a round's chunks dealt round-robin, the
// rest taken from a per-round counter); a vertex with more than warp_degree
// neighbours instead becomes work items of item_edges edges, expanded after
// the round's grid barrier in 128-edge slices, one whole warp per slice, in
// groups dealt the same way, so no warp holds the round up with a long list
// (with merge_below, a round with a small frontier has its first items taken
// by the warps that have finished their chunks, one barrier per round).
// Improved vertices are staged per warp and their queue flags settled 32 at
// a time (stage_flags).  An
// improved vertex with distance < T joins the next near queue
// (once per iteration, by stamp) and otherwise the far pile (once per epoch,
// by flag).  With expanded_check, a queued vertex is expanded only if its
// distance is below the one it was last expanded with (off by default: it
// skips about 1% of the entries for a random read and write per entry).
// A vertex of degree d above window_degree is expanded only once its
// distance is below m + C / d (m: the smallest distance queued for the
// round, C: the window constant) and is otherwise queued again for the next
// round: a list is expensive to expand with a distance that later improves,
// so the longer the list, the closer to Dijkstra order it is expanded, while
// short lists keep the parallelism of expanding everything queued.  When the
// near queue runs dry the far pile is split: the minimum
// pending distance mf is found, T becomes max(T, mf) + delta, entries below the
// old T are stale (already settled through the near queue) and dropped,
// entries below the new T form the next near queue, the rest stay far.
#include <type_traits>

#include "ig_device.cuh"
#include "ig_options.h"

namespace {

constexpr int kThreads = 256;
constexpr int kDeltaSamples = 4096;
static_assert(kDeltaSamples % 32 == 0, "delta samples are taken by whole warps");
constexpr int kSlice = 128;  // edges of a work-item slice: four per lane of one warp
constexpr int kQBuf = 32 + 32 * 8;  // warp staging: 32 + the most one step adds (two slices, 8 per lane)
static_assert(kSlice == 4 * 32, "a slice is one relax4 step of a warp");

struct SsspArgs {
  const int* __restrict__ nindex;
  const int* __restrict__ nlist;
  const int* __restrict__ eweight;
  int nodes;
  long long edges;
  int src;
  int* dist;
  int* qa;       // near queues
  int* qb;
  int* fa;       // far piles (alternating by epoch)
  int* fb;
  int* stamp;    // near-queue membership stamp
  int* farflag;  // far-pile membership (epoch + 1)
  // work items of a round, (vertex << 32) | index of its `item_edges`-edge
  // chunk: `items` holds those expanded after the round's barrier; in a
  // round whose frontier is below merge_below the first kSmallItems go to a
  // small list (alternating by round, kNoItem marking a free slot) and are
  // expanded by warps that have finished their frontier chunks
  unsigned long long* items;
  unsigned long long* small0;
  unsigned long long* small1;
  int mcap;       // item capacity of `items`
  int* expanded;  // distance each vertex was last expanded with (INT_MAX: never)
  int* members;   // vertices light-expanded since the last heavy pass
  int* inmember;  // 1 while a vertex sits in members
  IgCtl* ctl;
  unsigned long long timeout_ns;
  int item_edges;        // edges per work item
  int warp_degree;       // vertices with more neighbours than this become work items
  long long delta;       // > 0: fixed bucket width
  int delta_scale;
  int heavy_split;       // 1: light/heavy edge split (heavy edges relaxed once per bucket)
  int window_scale;      // window constant C = mean weight * window_scale (0: no window)
  int window_degree;     // vertices of at most this degree are never deferred
  int merge_below;       // rounds with a smaller frontier expand their items without a second barrier
  int spin_ns;           // pause between polls of a warp waiting for work items
  int stage_flags;       // 1: improved vertices staged per warp, their queue flags settled 32 at a time
  int chunk;             // frontier entries per warp chunk (at most 32)
  int item_group;        // most work-item slices a warp takes at a time
  int static_pct;        // share (percent) of a pass's chunks / slice groups dealt to warps without atomics
  int tail_split;        // chunks / slice groups taken from the counter are this many times smaller
  int claim_ahead;       // 1: a warp claims its next chunk from the counter when it starts the current one
  int expanded_check;    // 1: a queued vertex is skipped when its distance has not dropped since its last
                         // expansion (one more random read and write per queue entry)
};

// Per-round counters: hot counters of the control block (every warp updates
// them with atomics).  Slot s = k % 3 for near iteration k, f = epoch % 3 for
// far epochs.
enum SsspCounter : int {
  kCQueue = 0,     // [3] size of the near queue processed by near iteration k
  kCFar = 3,       // [3] far-pile size of epoch f
  kCGrab = 6,      // [3] frontier chunks taken beyond the first one per warp
  kCItems = 9,     // [3] work-item count of near iteration k
  kCMin = 12,      // [3] smallest distance queued for near iteration k
  kCMembers = 15,  // [2] member count (light/heavy split), slot mpass % 2
  kCSlices = 17,   // [3] (64-bit) work-item slices taken
  kCFarMin = 20,   // [3] (64-bit) minimum pending distance of epoch f's pile
  kCDone = 23,     // [3] warps done with the frontier part of near iteration k
  kCSlices2 = 26,  // [3] (64-bit) slices taken after the barrier of a merged round
  kCCount = 29
};
constexpr unsigned long long kNoItem = ~0ull;
constexpr int kSmallItems = 1 << 16;  // items a round expands without a second barrier
static_assert(kCCount <= kCtlHot, "SSSP counters must fit the control block's hot counters");
// ctl->u64[0..1]   weight-sample sum / count, ctl->u64[2] bucket width
// ctl->work        relaxations that improved a distance

// Lowers *slot to the warp's smallest `v` (one atomic per warp) and resets v.
__device__ __forceinline__ void publish_min(int& v, int* slot) {
  const int m = __reduce_min_sync(IG_FULL, v);
  if (ig::lane_id() == 0 && m != ig::kInf) atomicMin(slot, m);
  v = ig::kInf;
}

template <int kMinBlocks, bool kPair>
__global__ void __launch_bounds__(kThreads, kMinBlocks) sssp_persistent(SsspArgs a) {
  using namespace ig;
  IgCtl* ctl = a.ctl;
  GridBar gb;  // this block's view of the barrier generation
  auto ci = [&](int k) { return hot32(ctl, k); };
  auto cu = [&](int k) { return hot64(ctl, k); };
  const int lane = lane_id();
  const long long gtid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long gthreads = (long long)gridDim.x * blockDim.x;
  const int warp_g = (int)(gtid >> 5);
  const int nwarps = (int)(gthreads >> 5);
  __shared__ int s_qbuf[kThreads / 32][2][kPair ? kQBuf : kWarpBuf];  // per-warp staging of near / far appends
  // per-warp staging of improved vertices (vertex, new distance) whose queue
  // flags are not settled yet: fewer than 32 between steps, plus one step's
  __shared__ int2 s_cand[kThreads / 32][kPair ? kQBuf : kWarpBuf];
  int* nbuf = s_qbuf[threadIdx.x >> 5][0];
  int* fbuf = s_qbuf[threadIdx.x >> 5][1];
  int2* cbuf = s_cand[threadIdx.x >> 5];
  int nbuf_n = 0, fbuf_n = 0, cbuf_n = 0;

  for (long long v = gtid; v < a.nodes; v += gthreads) {
    a.dist[v] = (v == a.src) ? 0 : kInf;
    a.stamp[v] = 0;
    a.farflag[v] = 0;
    if (a.expanded_check) a.expanded[v] = kInf;
    if (a.heavy_split) a.inmember[v] = 0;  // read only by the light/heavy split
  }
  if (gtid < kDeltaSamples && a.edges > 0) {  // whole warps (kDeltaSamples is a multiple of 32)
    const long long e = gtid * a.edges / kDeltaSamples;
    unsigned long long w = (unsigned long long)max(0, __ldg(&a.eweight[e]));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) w += __shfl_xor_sync(IG_FULL, w, o);
    if (lane == 0) {
      atomicAdd(&ctl->u64[0], w);
      atomicAdd(&ctl->u64[1], 32ull);
    }
  }
  for (long long i = gtid; i < kSmallItems; i += gthreads) {
    a.small0[i] = kNoItem;
    a.small1[i] = kNoItem;
  }
  if (gtid == 0) a.qa[0] = a.src;
  if (gtid < kCCount) {
    const int k = (int)gtid;
    if ((k >= kCSlices && k < kCDone) || k >= kCSlices2)  // the 64-bit counters
      *cu(k) = (k >= kCFarMin && k < kCDone) ? ~0ull : 0ull;
    else *ci(k) = (k >= kCMin && k < kCMin + 3) ? kInf : 0;
  }
  if (!grid_sync(ctl, a.timeout_ns, gb)) return;

  const unsigned long long wcnt = ld_relaxed(&ctl->u64[1]);
  const double mean_w = wcnt ? (double)ld_relaxed(&ctl->u64[0]) / (double)wcnt : 1.0;
  // window constant: 0 disables the deferral
  const long long wc = a.window_scale > 0 ? max(1LL, (long long)(mean_w * a.window_scale)) : 0;
  long long delta = a.delta;
  if (delta <= 0) {
    const double mean_deg = a.nodes ? (double)a.edges / (double)a.nodes : 1.0;
    delta = (long long)(mean_w * a.delta_scale / (mean_deg > 1.0 ? mean_deg : 1.0));
    if (delta < 1) delta = 1;
  }
  if (gtid == 0) ctl->u64[2] = (unsigned long long)delta;

  int* cur = a.qa;
  int* nxt = a.qb;
  int cur_size = 1;
  long long T = delta;  // distances < T are near
  int it = 0;           // near iteration index (stamp it+1 marks the next queue)
  int mq = 0;           // smallest distance queued for iteration it (exact or below the true one)
  int slog = 0;         // log2 of the slices per work item
  while ((kSlice << slog) < a.item_edges) slog++;
  int nmin = kInf;      // this thread's smallest distance queued for the next iteration
  int epoch = 0;
  int mpass = 0;        // heavy passes done
  long long improved = 0, frontier_v = 0, frontier_e = 0;

  while (true) {
    // ------------------------------------------------------------ near phase
    // Light passes expand the near queue and relax only edges lighter than
    // delta (all edges when the split is off); every expanded vertex joins the
    // member list.  When the near queue is empty, a heavy pass relaxes the
    // heavy edges of the members once, with their settled distances (a heavy
    // edge cannot improve a vertex of the same bucket).  Member count: slot
    // 9 + mpass % 2; a heavy pass clears the other slot.
    int nmem = 0;
    while (cur_size > 0 || nmem > 0) {
      const bool heavy = cur_size == 0;
      if (gtid == 0) {
        *ci(kCQueue + (it + 2) % 3) = 0;
        *ci(kCGrab + (it + 1) % 3) = 0;
        *ci(kCItems + (it + 1) % 3) = 0;
        *cu(kCSlices + (it + 1) % 3) = 0;
        *cu(kCSlices2 + (it + 1) % 3) = 0;
        *ci(kCDone + (it + 1) % 3) = 0;
        *ci(kCMin + (it + 2) % 3) = kInf;
        if (heavy) *ci(kCMembers + (mpass + 1) % 2) = 0;
      }
      int* qsize = ci(kCQueue + (it + 1) % 3);
      int* nmembers = ci(kCMembers + mpass % 2);
      int* far = (epoch & 1) ? a.fb : a.fa;
      int* fsize = ci(kCFar + epoch % 3);
      const int next_stamp = it + 1;
      const int far_mark = epoch + 1;
      const int* frontier = heavy ? a.members : cur;
      const int fcount = heavy ? nmem : cur_size;
      // this round's work items go to list it % 2; the other list held the
      // previous round's, all consumed before the barrier that began this
      // round: free its used slots for the next round
      // one barrier (merged round) or two; uniform over the grid
      const bool merged = fcount < a.merge_below;
      const int nsmall = merged ? kSmallItems : 0;  // items that go to the small list
      unsigned long long* small = (it & 1) ? a.small1 : a.small0;
      {
        // the other small list held the previous round's items, all consumed
        // before the barrier that began this round: free its used slots
        unsigned long long* old_small = (it & 1) ? a.small0 : a.small1;
        const int nprev = min(ld_relaxed(ci(kCItems + (it + 2) % 3)), kSmallItems);
        for (long long i = gtid; i < nprev; i += gthreads) old_small[i] = kNoItem;
      }
      // Queue flags of one improved vertex per lane (lanes < cnt): a distance
      // below T joins the next near queue once per iteration (stamp), any
      // other the far pile once per epoch (flag).
      auto settle = [&](int cnt, int v, int nd) {
        bool tn = false, tf = false;
        if (ig::lane_id() < cnt) {
          if (nd < T) {
            nmin = min(nmin, nd);
            tn = a.stamp[v] != next_stamp && atomicExch(&a.stamp[v], next_stamp) != next_stamp;
          } else {
            tf = a.farflag[v] != far_mark && atomicExch(&a.farflag[v], far_mark) != far_mark;
          }
        }
        const int vv[1] = {v};
        const bool fn[1] = {tn}, ff[1] = {tf};
        warp_buf_append2_flags<1>(vv, fn, nbuf, nbuf_n, nxt, qsize, ff, fbuf, fbuf_n, far, fsize, a.nodes, ctl);
      };
      // Settles staged improved vertices 32 at a time (all of them if `all`).
      auto settle_staged = [&](bool all) {
        __syncwarp();
        while (cbuf_n >= 32 || (all && cbuf_n > 0)) {
          const int take = min(cbuf_n, 32);
          cbuf_n -= take;
          int2 c = make_int2(0, 0);
          if (lane < take) c = cbuf[cbuf_n + lane];
          __syncwarp();
          settle(take, c.x, c.y);
        }
      };
      // Four edges per lane at a time: their loads and atomics are
      // independent, so they are issued together.  The distance update is a
      // reduction (atomicMin without a result): an edge whose candidate beats
      // the distance it read counts as an improvement without waiting for the
      // atomic.  Another edge may have lowered the distance further in the
      // meantime; the vertex is then queued once more than needed (the stamp
      // keeps it to one entry per queue, the expanded-distance check skips it).
      // With stage_flags the improved vertices go to the warp's staging
      // buffer and their flags are settled once 32 have gathered, so a step
      // waits for two dependent reads (list, then distances) instead of four
      // (and the flag exchanges); otherwise each step settles its own.
      auto relax4 = [&](const auto& act, const auto& e, const auto& du) {
        constexpr int N = std::extent<std::remove_reference_t<decltype(act)>>::value;  // 4, or 8 for two slices
        int v[N], w[N], dv[N], sv[N];
        bool cand[N];
#pragma unroll
        for (int k = 0; k < N; k++) {
          v[k] = 0;
          w[k] = 0;
          if (act[k] && du[k] != kInf) {
            v[k] = __ldg(&a.nlist[e[k]]);
            w[k] = __ldg(&a.eweight[e[k]]);
          }
        }
#pragma unroll
        for (int k = 0; k < N; k++) dv[k] = (act[k] && du[k] != kInf) ? a.dist[v[k]] : 0;
#pragma unroll
        for (int k = 0; k < N; k++) {
          const bool light = !a.heavy_split || (long long)w[k] < delta;
          cand[k] = act[k] && du[k] != kInf && light != heavy && (long long)du[k] + w[k] < (long long)dv[k];
          if (cand[k]) atomicMin(&a.dist[v[k]], du[k] + w[k]);
        }
        if (a.stage_flags) {
#pragma unroll
          for (int k = 0; k < N; k++) {
            const unsigned m = __ballot_sync(IG_FULL, cand[k]);
            if (cand[k]) {
              improved++;
              cbuf[cbuf_n + __popc(m & lanemask_lt())] = make_int2(v[k], du[k] + w[k]);
            }
            cbuf_n += __popc(m);
          }
          if (cbuf_n >= 32) settle_staged(false);
          return;
        }
#pragma unroll
        for (int k = 0; k < N; k++) sv[k] = cand[k] ? a.stamp[v[k]] : 0;
        bool tn[N], tf[N];
#pragma unroll
        for (int k = 0; k < N; k++) {
          tn[k] = tf[k] = false;
          if (cand[k]) {
            improved++;
            const long long nd = (long long)du[k] + w[k];
            if (nd < T) {
              nmin = min(nmin, (int)nd);
              tn[k] = sv[k] != next_stamp && atomicExch(&a.stamp[v[k]], next_stamp) != next_stamp;
            } else {
              tf[k] = a.farflag[v[k]] != far_mark && atomicExch(&a.farflag[v[k]], far_mark) != far_mark;
            }
          }
        }
        warp_buf_append2_flags<N>(v, tn, nbuf, nbuf_n, nxt, qsize, tf, fbuf, fbuf_n, far, fsize, a.nodes, ctl);
      };
      // Frontier chunks: a chunk is 32 queue entries, fewer when the queue
      // has less than 32 per warp, so a small round's lists are spread over
      // the whole grid.  The first `nstatic` chunks are dealt round-robin
      // (warp w takes w, w + nwarps, ...); the rest of the queue is taken
      // from the round's counter in chunks of cs / tail_split entries, so
      // warps that drew light chunks take more and the pass ends evenly (the
      // round ends at the grid barrier, so the slowest warp sets its length).
      // A claim from the counter is a round trip on the warp's critical
      // path; with claim_ahead the next chunk is claimed when the current
      // one starts.
      int* grab = ci(kCGrab + it % 3);
      const int cs = fcount >= nwarps * a.chunk ? a.chunk : max(1, (fcount + nwarps - 1) / nwarps);
      const int nchunks = (fcount + cs - 1) / cs;
      const int nstatic = max(min(nchunks, nwarps), (int)((long long)nchunks * a.static_pct / 100));
      const int dyn_base = min(fcount, nstatic * cs);  // first entry of the counter's part
      const int csd = max(1, cs / a.tail_split);       // entries per claimed chunk
      auto dyn_chunk = [&](int k, int& start, int& len) {
        start = dyn_base + k * csd;
        len = max(0, min(csd, fcount - start));
      };
      int sc = warp_g;  // static chunk index; -1 once in the counter's part
      int start = 0, len = 0;
      if (sc < nstatic) {
        start = sc * cs;
        len = min(cs, fcount - start);
      } else {
        sc = -1;
        int k = 0;
        if (lane == 0) k = atomicAdd(grab, 1);
        dyn_chunk(__shfl_sync(IG_FULL, k, 0), start, len);
      }
      while (len > 0) {
        const bool next_static = sc >= 0 && sc + nwarps < nstatic;
        int ahead = 0;
        if (!next_static && a.claim_ahead && lane == 0) ahead = atomicAdd(grab, 1);
        const int base = start;
        const int i = base + lane;
        int u = 0, beg = 0, deg = 0, du = kInf;
        bool expand = false, defer = false;
        if (lane < len) {
          u = frontier[i];
          // every per-vertex read depends only on u, so they are issued together
          du = a.dist[u];
          const int ex = (heavy || !a.expanded_check) ? kInf : a.expanded[u];
          beg = __ldg(&a.nindex[u]);
          const int end = __ldg(&a.nindex[u + 1]);
          if (heavy) {
            a.inmember[u] = 0;
            expand = true;
          } else {
            // a vertex improved while already queued is queued again; expand
            // it only if its distance dropped since its last expansion
            expand = du < ex;
          }
          if (expand) {
            deg = end - beg;
            if (!heavy) {
              // (du - mq) * deg >= C: outside the window, queued again
              if (wc > 0 && deg > a.window_degree && (long long)(du - mq) * deg >= wc) {
                expand = false;
                deg = 0;
                if (a.stage_flags) {
                  defer = true;  // staged below with its distance (below T: it is in the near queue)
                } else {
                  nmin = min(nmin, du);
                  defer = a.stamp[u] != next_stamp && atomicExch(&a.stamp[u], next_stamp) != next_stamp;
                }
              } else {
                if (a.expanded_check) a.expanded[u] = du;
              }
            }

          }
        }
        if (a.stage_flags) {
          // a deferred vertex is queued again through the staged settling
          // (stamp, smallest queued distance), off this chunk's critical path
          const unsigned m = __ballot_sync(IG_FULL, defer);
          if (m) {
            if (defer) cbuf[cbuf_n + __popc(m & lanemask_lt())] = make_int2(u, du);
            cbuf_n += __popc(m);
            if (cbuf_n >= 32) settle_staged(false);
          }
        } else {
          const int dq[1] = {u};
          warp_buf_append<1>(defer ? 1 : 0, dq, nbuf, nbuf_n, nxt, qsize, a.nodes, ctl);
        }
        if (a.heavy_split && !heavy)
          warp_append(expand && atomicExch(&a.inmember[u], 1) == 0, u, a.members, nmembers, a.nodes, ctl);
        // a list longer than warp_degree becomes work items of item_edges
        // edges each, expanded after the barrier; the slots are reserved here
        // and written after the chunk's short lists, so the reservation's
        // round trip overlaps them
        const bool listed = deg > a.warp_degree;
        const int cnt = listed ? (deg + a.item_edges - 1) / a.item_edges : 0;
        int incl = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int t = __shfl_up_sync(IG_FULL, incl, o);
          if (lane >= o) incl += t;
        }
        const int itotal = __shfl_sync(IG_FULL, incl, 31);
        int ibase = 0;
        // reserved by lane 0, the lane that later reports the warp done, so
        // the report orders after the reservation
        if (itotal > 0 && lane == 0) ibase = atomicAdd(ci(kCItems + it % 3), itotal);
        if (expand) {
          frontier_v++;
          frontier_e += deg;
        }
        // the chunk's short lists here: at most 32 * warp_degree edges per warp
        warp_expand4(beg, listed ? 0 : deg, [&](const bool (&act)[4], const int (&e)[4], const int (&j)[4]) {
          int duj[4];
#pragma unroll
          for (int k = 0; k < 4; k++) duj[k] = __shfl_sync(IG_FULL, du, j[k]);
          relax4(act, e, duj);
        });
        if (itotal > 0) {
          // the warp writes the chunk's items together: slot idx belongs to
          // the last lane whose exclusive count is <= idx
          ibase = __shfl_sync(IG_FULL, ibase, 0);
          const int excl = incl - cnt;
          for (int i0 = 0; i0 < itotal; i0 += 32) {
            const int idx = i0 + lane;
            int j = 0;
#pragma unroll
            for (int step = 16; step >= 1; step >>= 1) {
              const int ej = __shfl_sync(IG_FULL, excl, j + step);
              if (ej <= idx) j += step;
            }
            const int uj = __shfl_sync(IG_FULL, u, j);
            const int c = idx - __shfl_sync(IG_FULL, excl, j);
            if (idx < itotal) {
              const unsigned long long w = ((unsigned long long)(unsigned)uj << 32) | (unsigned)c;
              const int slot = ibase + idx;
              if (slot < nsmall)
                st_relaxed(&small[slot], w);
              else if (slot - nsmall < a.mcap)
                a.items[slot - nsmall] = w;
              else
                raise(ctl, IG_ERR_OVERFLOW);
            }
          }
        }
        if (next_static) {
          sc += nwarps;
          start = sc * cs;
          len = min(cs, fcount - start);
        } else {
          sc = -1;
          if (!a.claim_ahead && lane == 0) ahead = atomicAdd(grab, 1);
          dyn_chunk(__shfl_sync(IG_FULL, ahead, 0), start, len);
        }
      }
      // Work items (vertex, chunk of item_edges edges) are cut in slices of
      // kSlice edges, 2^slog slices per item (the last ones of a short chunk
      // are empty), each expanded by one whole warp over a contiguous range
      // (no owner search); expand_slices runs slices j0..j1-1 of the items
      // whose headers lanes 0.. hold (item mfirst + t in lane t).
      auto expand_slices = [&](long long j0, long long j1, int mfirst, int hdu, int hb, int hd) {
        // slice j's four edges per lane into act/e/duk[o, o + 4)
        auto slice_edges = [&](long long j, bool* act, int* e, int* duk) {
          const int t = (int)(j >> slog) - mfirst;
          const int du = __shfl_sync(IG_FULL, hdu, t);
          const int b = __shfl_sync(IG_FULL, hb, t);
          const int d = __shfl_sync(IG_FULL, hd, t);
          const int s0 = (int)(j & ((1LL << slog) - 1)) * kSlice;
#pragma unroll
          for (int k = 0; k < 4; k++) {
            const int off = s0 + k * 32 + lane;
            act[k] = off < d;
            e[k] = b + (act[k] ? off : 0);
            duk[k] = du;
          }
        };
        long long j = j0;
        if (kPair)  // two slices per step: eight edges per lane, their loads issued together
          for (; j + 1 < j1; j += 2) {
            bool act[8];
            int e[8], duk[8];
            slice_edges(j, act, e, duk);
            slice_edges(j + 1, act + 4, e + 4, duk + 4);
            relax4(act, e, duk);
          }
        for (; j < j1; j++) {
          bool act[4];
          int e[4], duk[4];
          slice_edges(j, act, e, duk);
          relax4(act, e, duk);
        }
      };
      // Items expanded after a barrier (every item written, the count final):
      // g slices at a time, the first g by warp index, the rest taken from
      // the 64-bit counter `cnt`.
      auto barrier_items = [&](const unsigned long long* list, int nm, unsigned long long* cnt) {
        const long long units = (long long)nm << slog;
        const int g = (int)min((long long)a.item_group, max(1LL, units / (4LL * nwarps)));
        // group q holds slices [q * g, (q + 1) * g): the first nsg dealt
        // round-robin, the rest taken from the counter in groups of
        // g / tail_split slices (as the frontier chunks)
        const long long ngroups = (units + g - 1) / g;
        const long long nsg = max(min(ngroups, (long long)nwarps), ngroups * a.static_pct / 100);
        const long long dbase = min(units, nsg * g);
        const int gd = max(1, g / a.tail_split);
        long long q = warp_g, j0 = 0, j1 = 0;
        if (q < nsg) {
          j0 = q * g;
          j1 = min(j0 + g, units);
        } else {
          q = -1;
          unsigned long long k = 0;
          if (lane == 0) k = atomicAdd(cnt, 1ull);
          j0 = dbase + (long long)__shfl_sync(IG_FULL, k, 0) * gd;
          j1 = min(j0 + gd, units);
        }
        while (j0 < j1) {
          const bool next_static = q >= 0 && q + nwarps < nsg;
          unsigned long long ahead = 0;
          if (!next_static && a.claim_ahead && lane == 0) ahead = atomicAdd(cnt, 1ull);
          const int mfirst = (int)(j0 >> slog);
          const int ni = (int)((j1 - 1) >> slog) - mfirst + 1;
          int hdu = kInf, hb = 0, hd = 0;
          if (lane < ni) {
            const unsigned long long w = list[mfirst + lane];
            const int u = (int)(w >> 32);
            hdu = a.dist[u];
            const int b0 = __ldg(&a.nindex[u]), d0 = __ldg(&a.nindex[u + 1]) - b0;
            const int off0 = (int)(unsigned)w * a.item_edges;
            hb = b0 + off0;
            hd = min(a.item_edges, d0 - off0);
          }
          expand_slices(j0, j1, mfirst, hdu, hb, hd);
          if (next_static) {
            q += nwarps;
            j0 = q * g;
            j1 = min(j0 + g, units);
          } else {
            q = -1;
            if (!a.claim_ahead && lane == 0) ahead = atomicAdd(cnt, 1ull);
            j0 = dbase + (long long)__shfl_sync(IG_FULL, ahead, 0) * gd;
            j1 = min(j0 + gd, units);
          }
        }
      };
      auto end_pass = [&]() {
        settle_staged(true);
        warp_buf_flush2(nbuf, nbuf_n, nxt, qsize, fbuf, fbuf_n, far, fsize, a.nodes, ctl);
        publish_min(nmin, ci(kCMin + (it + 1) % 3));
        return grid_sync(ctl, a.timeout_ns, gb);
      };
      const int* icount = ci(kCItems + it % 3);
      bool end_barrier;  // the item pass needs a barrier of its own
      if (merged) {
        // A warp done with its frontier chunks reports it and takes slices of
        // the small list while other warps still expand theirs and add
        // items.  Slices are claimed 4 at a time from a counter; a claim
        // beyond the items reserved so far waits for more items or for every
        // warp's report (then the count is final and the claim past it is
        // dropped); a reserved item not yet written is waited for.  Every
        // wait is bounded and watches the error word.  Items beyond the small
        // list are expanded after the barrier.
        __syncwarp();
        int* done = ci(kCDone + it % 3);
        if (lane == 0) red_add_release(done, 1);
        unsigned long long* mgrab = cu(kCSlices + it % 3);
        long long seen = 0;  // slices known to exist (lane 0's view, broadcast)
        while (true) {
          long long j0 = 0, j1 = 0;
          if (lane == 0) {
            j0 = (long long)atomicAdd(mgrab, 4ull);
            j1 = j0 + 4;
            if (j1 > seen) {
              const unsigned long long t0 = globaltimer();
              unsigned spins = 0;
              while (true) {
                const bool fin = ld_acquire(done) == nwarps;  // then every reservation is visible
                seen = (long long)min(ld_relaxed(icount), kSmallItems) << slog;
                if (fin) {
                  j1 = min(j1, seen);
                  break;
                }
                if (j1 <= seen) break;
                if ((++spins & 15u) == 0 &&
                    (ld_relaxed(&ctl->err) != 0 || globaltimer() - t0 > a.timeout_ns)) {
                  if (ld_relaxed(&ctl->err) == 0) raise(ctl, IG_ERR_TIMEOUT);
                  j1 = j0;
                  break;
                }
                __nanosleep(a.spin_ns);
              }
            }
          }
          j0 = __shfl_sync(IG_FULL, j0, 0);
          j1 = __shfl_sync(IG_FULL, j1, 0);
          seen = __shfl_sync(IG_FULL, seen, 0);
          if (j0 >= j1) break;
          // the claim's items (at most 4): lane t reads item mfirst + t
          const int mfirst = (int)(j0 >> slog);
          const int ni = (int)((j1 - 1) >> slog) - mfirst + 1;
          int hdu = kInf, hb = 0, hd = 0;
          bool ok = true;
          if (lane < ni) {
            const unsigned long long* slot = &small[mfirst + lane];
            unsigned long long w = ld_relaxed(slot);
            if (w == kNoItem) {
              const unsigned long long t0 = globaltimer();
              unsigned spins = 0;
              while ((w = ld_relaxed(slot)) == kNoItem) {
                if ((++spins & 15u) == 0 &&
                    (ld_relaxed(&ctl->err) != 0 || globaltimer() - t0 > a.timeout_ns)) {
                  if (ld_relaxed(&ctl->err) == 0) raise(ctl, IG_ERR_TIMEOUT);
                  ok = false;
                  break;
                }
                __nanosleep(64);
              }
            }
            if (ok) {
              const int u = (int)(w >> 32);
              hdu = a.dist[u];
              const int b0 = __ldg(&a.nindex[u]), d0 = __ldg(&a.nindex[u + 1]) - b0;
              const int off0 = (int)(unsigned)w * a.item_edges;
              hb = b0 + off0;
              hd = min(a.item_edges, d0 - off0);
            }
          }
          if (__ballot_sync(IG_FULL, !ok)) break;
          expand_slices(j0, j1, mfirst, hdu, hb, hd);
        }
        if (!end_pass()) return;
        const int nbig = min(ld_relaxed(icount) - kSmallItems, a.mcap);
        end_barrier = nbig > 0;
        if (nbig > 0) barrier_items(a.items, nbig, cu(kCSlices2 + it % 3));
      } else {
        if (!end_pass()) return;
        const int nm = min(ld_relaxed(icount), a.mcap);
        end_barrier = nm > 0;
        if (nm > 0) barrier_items(a.items, nm, cu(kCSlices + it % 3));
      }
      if (end_barrier && !end_pass()) return;
      if (heavy) mpass++;
      cur_size = ld_relaxed(qsize);
      mq = ld_relaxed(ci(kCMin + (it + 1) % 3));
      nmem = a.heavy_split ? ld_relaxed(ci(kCMembers + mpass % 2)) : 0;
      it++;
      int* t = cur;
      cur = nxt;
      nxt = t;
    }
    // ------------------------------------------------------------ far split
    // The near queue for iteration `it` is built in `cur` with counter slot
    // it % 3 (iteration it-1 appended nothing to it) and stamp `it`.
    bool done = false;
    while (cur_size == 0) {
      const int f = epoch % 3;
      const int fsz = ld_relaxed(ci(kCFar + f));
      if (fsz == 0) {
        done = true;
        break;
      }
      int* far = (epoch & 1) ? a.fb : a.fa;
      int* far_next = (epoch & 1) ? a.fa : a.fb;
      if (gtid == 0) {
        *ci(kCFar + (epoch + 1) % 3) = 0;
        *cu(kCFarMin + (epoch + 1) % 3) = ~0ull;
      }
      for (long long i = gtid; i < fsz; i += gthreads) {
        const int d = a.dist[far[i]];
        if ((long long)d >= T) atomicMin(cu(kCFarMin + f), (unsigned long long)d);
      }
      if (!grid_sync(ctl, a.timeout_ns, gb)) return;
      const unsigned long long mfar = ld_relaxed(cu(kCFarMin + f));
      const long long T_old = T;
      if (mfar != ~0ull) T = ((long long)mfar > T ? (long long)mfar : T) + delta;
      else T = T + delta;
      // the next near queue holds distances in [T_old, T): its minimum is mfar
      mq = mfar != ~0ull ? (int)mfar : kInf;
      int* qsize = ci(kCQueue + it % 3);
      int* fsize_next = ci(kCFar + (epoch + 1) % 3);
      for (long long base = gtid & ~31LL; base < fsz; base += gthreads) {
        const long long i = base + lane;
        bool to_near = false, to_far = false;
        int v = 0;
        if (i < fsz) {
          v = far[i];
          const long long d = a.dist[v];
          if (d >= T_old) {
            if (d < T) to_near = atomicExch(&a.stamp[v], it) != it;
            else {
              to_far = true;
              a.farflag[v] = epoch + 2;
            }
          }
        }
        warp_append(to_near, v, cur, qsize, a.nodes, ctl);
        warp_append(to_far, v, far_next, fsize_next, a.nodes, ctl);
      }
      if (!grid_sync(ctl, a.timeout_ns, gb)) return;
      epoch++;
      cur_size = ld_relaxed(qsize);
    }
    if (done) break;
  }
  if (improved) atomicAdd((unsigned long long*)&ctl->work, (unsigned long long)improved);
  if (frontier_v) atomicAdd(&ctl->u64[13], (unsigned long long)frontier_v);
  if (frontier_e) atomicAdd(&ctl->u64[14], (unsigned long long)frontier_e);
  if (gtid == 0) {
    ctl->iterations = it;
    ctl->u64[12] = (unsigned long long)epoch;
  }
}

}  // namespace

int igk_sssp(IgExec* ex, const ig_csr* dg, int src, int* d_dist) {
  const size_t vb = (size_t)dg->nodes * sizeof(int);
  void *qa, *qb, *fa, *fb, *stamp, *farflag, *items, *smalls;
  int rc;
  if ((rc = ig_scratch_get(ex->scratch, IG_SLOT_Q0, vb, &qa))) return rc;
  if ((rc = ig_scratch_get(ex->scratch, IG_SLOT_Q1, vb, &qb))) return rc;
  if ((rc = ig_scratch_get(ex->scratch, IG_SLOT_Q2, vb, &fa))) return rc;
  if ((rc = ig_scratch_get(ex->scratch, IG_SLOT_Q3, vb, &fb))) return rc;
  if ((rc = ig_scratch_get(ex->scratch, IG_SLOT_V0, vb, &stamp))) return rc;
  if ((rc = ig_scratch_get(ex->scratch, IG_SLOT_V1, vb, &farflag))) return rc;
  // items: sum over a round's vertices of ceil(deg / item edges) <= nodes + edges / item edges
  const IgOptions& op = ig_exec_options(ex);
  const long long mcap_l = (long long)dg->nodes + dg->edges / std::max(1, op.sssp_item_edges) + 1;
  const int mcap = (int)std::min<long long>(mcap_l, 0x7fffffffLL - kSmallItems);
  if ((rc = ig_scratch_get(ex->scratch, IG_SLOT_G0, (size_t)mcap * sizeof(unsigned long long), &items)))
    return rc;
  if ((rc = ig_scratch_get(ex->scratch, IG_SLOT_G1, 2 * (size_t)kSmallItems * sizeof(unsigned long long),
                           &smalls)))
    return rc;
  void *expanded, *members, *inmember;
  expanded = nullptr;  // only with the expanded-distance check
  if (ig_exec_options(ex).sssp_expanded_check && (rc = ig_scratch_get(ex->scratch, IG_SLOT_F0, vb, &expanded)))
    return rc;
  if ((rc = ig_scratch_get(ex->scratch, IG_SLOT_F1, vb, &members))) return rc;
  if ((rc = ig_scratch_get(ex->scratch, IG_SLOT_E0, vb, &inmember))) return rc;
  if ((rc = ig_exec_reset(ex))) return rc;
  const IgOptions& o = ig_exec_options(ex);
  SsspArgs a{dg->nindex, dg->nlist, dg->eweight, dg->nodes, dg->edges, src, d_dist,
             (int*)qa, (int*)qb, (int*)fa, (int*)fb, (int*)stamp, (int*)farflag,
             (unsigned long long*)items, (unsigned long long*)smalls, (unsigned long long*)smalls + kSmallItems,
             mcap,
             (int*)expanded, (int*)members, (int*)inmember, ex->d_ctl, ex->timeout_ns, o.sssp_item_edges,
             o.sssp_warp_degree,
             o.sssp_delta, o.sssp_delta_scale, o.sssp_heavy_split, o.sssp_window_scale,
             o.sssp_window_degree, o.sssp_merge_below, o.sssp_spin_ns, o.sssp_stage_flags, o.sssp_chunk, o.sssp_item_group, o.sssp_static_pct, o.sssp_tail_split, o.sssp_claim_ahead, o.sssp_expanded_check};
  void* args[] = {&a};
  // the register budget follows the residency cap (4, 5 or 6 blocks of 256 threads per SM)
  // (the paired-slice form holds more registers: 3 blocks per SM, or 4 with spills)
  const void* kern = o.sssp_pair_slices == 2                        ? (const void*)sssp_persistent<4, true>
                     : o.sssp_pair_slices                          ? (const void*)sssp_persistent<3, true>
                     : o.blocks_per_sm >= 6 || o.blocks_per_sm == 0 ? (const void*)sssp_persistent<6, false>
                     : o.blocks_per_sm == 5                        ? (const void*)sssp_persistent<5, false>
                                                                   : (const void*)sssp_persistent<4, false>;
  return ig_launch_coop(ex, kern, kThreads, 0, o.blocks_per_sm, args, nullptr);
}
