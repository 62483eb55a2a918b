// Triangle counting on sorted, self-loop-free adjacency.
//
// Reference: include/tc_vertex_cuda.h:42-63 and 98-117 (h_triCounting): for
// every vertex v and neighbour u > v, count the common neighbours w > u with
// a two-pointer merge, so each triangle is counted once; the count type is
// int there and overflows on large graphs, here it is 64-bit.  The driver
// refuses unsorted input (include/tc_vertex_cuda.h:157-165); this code
// returns IG_ERR_UNSORTED for it.
//
// GB300 formulation (same count, far less work on skewed graphs):
//   1. check  : adjacency strictly increasing and no self loop
//   2. orient : edge u->w iff (deg u, u) < (deg w, w), so every vertex keeps
//               O(sqrt E) out-neighbours N+; each list is split into its out
//               part (id order) and its in part N-; counted, scanned, filled
//   3. count  : work item = (middle vertex v, a chunk of its in-neighbours
//               u).  N+(v) is hashed into shared memory (a 2048-slot table
//               and an 8192-bit filter shared by a whole block when N+(v)
//               has more than 64 entries -- more than 128 when no exact
//               bitmap applies --, a 256-slot table per warp otherwise) and
//               every w of the out-lists N+(u) is probed (a list of at least
//               tc_warp_list probes walked by the whole warp 128 at a time,
//               shorter ones through a load-balanced warp expansion, four
//               probes per lane in flight); a hit is the triangle u -> v ->
//               w, counted once (at its middle vertex).  When the ids are in
//               (degree, id) order every w of N+(v) is above v, and a middle
//               vertex with a long N+(v) sits near the top of the id range:
//               if its bitmap from v + 1's 32-id word up to id V - 1 fits 2^17
//               bits, N+(v) is an exact bitmap in the block's shared memory
//               instead (one shared load and bit test per probe, no filter
//               and no hash walk).  Work: sum over u of |N+(u)|^2 probes,
//               halved when the ids are already in (degree, id) order (the
//               degree-ordered input of the benchmark): then only the part
//               of N+(u) after v is scanned.  The filter rejects most misses
//               before the hash probe.  Blocks take their work items in runs
//               of consecutive items from a counter, so the items of one
//               middle vertex usually share a block and its table or bitmap
//               is built once.
#include "ig_device.cuh"
#include "ig_options.h"

namespace {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kOrientHub = 256;   // lists longer than this are split by one block each
constexpr int kBlockOut = 64;     // middle vertices with more out-neighbours are counted by whole blocks
constexpr int kWarpOut = 128;     // ... unless no exact bitmap applies and they have at most this many
constexpr int kChunk = 64;        // in-neighbours per warp work item
constexpr int kHashCap = 2048;    // block table slots (out-degree <= 1024 is hashed)
constexpr int kBitWords = 256;    // block filter: 8192 bits, bit (w mod 8192) set for w in N+(v)
constexpr int kWarpCap = 256;     // warp table slots (out-degree <= kWarpOut)
constexpr int kWarpBitWords = 64; // warp filter: 2048 bits
constexpr int kSpanWords = 4096;  // block bitmap: 131072 bits over the 32-id words from v + 1's up
static_assert(kSpanWords >= kHashCap + kBitWords, "the bitmap shares its memory with the table and filter");

// Work items of middle vertex v with `out` out-neighbours and `in`
// in-neighbours: warp items of kChunk in-neighbours for a short N+(v), block
// items of `block_chunk` for a long one (the block shares one table of N+(v)).
// `exact`: N+(v) fits the block's exact bitmap (ids in (degree, id) order,
// fewer than kSpanWords * 32 ids above v); without it a list of up to
// kWarpOut stays with a warp (its own hash table, no block barrier per item:
// such vertices have few in-neighbours in the skewed graphs this serves).
__device__ __forceinline__ void tc_items(int out, int in, bool exact, int block_chunk, int* warp_items,
                                         int* block_items) {
  const bool block = out > kBlockOut && (exact || out > kWarpOut);
  *warp_items = (out > 0 && !block) ? (in + kChunk - 1) / kChunk : 0;
  *block_items = block ? (in + block_chunk - 1) / block_chunk : 0;
}
// Words of the exact bitmap of middle vertex v: word k holds ids
// [32 (k + wb), 32 (k + wb + 1)) for wb = (v + 1) / 32, so the ids above v
// need the words up to that of id n - 1.
__device__ __forceinline__ int tc_span_words(int n, int v) { return v + 1 < n ? ((n - 1) >> 5) - ((v + 1) >> 5) + 1 : 0; }
__device__ __forceinline__ bool tc_exact(bool ranked, int n, int v) { return ranked && tc_span_words(n, v) <= kSpanWords; }

__device__ __forceinline__ bool before(int du, int u, int dw, int w) { return du < dw || (du == dw && u < w); }

// ctl->i32[1] = 1 unless the ids are in (degree, id) order (degrees
// non-decreasing in id).  In that order before(u, w) is w > u, so the
// orientation needs no degree lookups and a sorted list splits into its in
// part (the prefix below u) and its out part (the suffix above u).
__global__ void tc_rank_check(const int* __restrict__ nindex, int n, IgCtl* ctl) {
  for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v + 1 < n;
       v += (long long)gridDim.x * blockDim.x)
    if (__ldg(&nindex[v + 2]) - __ldg(&nindex[v + 1]) < __ldg(&nindex[v + 1]) - __ldg(&nindex[v])) ctl->i32[1] = 1;
}

__global__ void __launch_bounds__(kThreads) tc_orient_count(const int* __restrict__ nindex,
                                                            const int* __restrict__ nlist, int n, int* out_cnt,
                                                            int* item_cnt, int* item_cnt_b, int* hubs,
                                                            int block_chunk, IgCtl* ctl) {
  using namespace ig;
  __shared__ int s_cnt[kWarps][32];
  const int lane = lane_id(), wib = threadIdx.x >> 5;
  const long long gtid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long gthreads = (long long)gridDim.x * blockDim.x;
  const bool ranked = ctl->i32[1] == 0;
  for (long long base = gtid & ~31LL; base < n; base += gthreads) {
    const long long v = base + lane;
    int beg = 0, deg = 0;
    if (v < n) {
      beg = __ldg(&nindex[v]);
      deg = __ldg(&nindex[v + 1]) - beg;
    }
    s_cnt[wib][lane] = 0;
    __syncwarp();
    const int vv = (int)v;
    const bool hub = deg > kOrientHub;  // counted by one block each in tc_orient_hubs
    warp_append(hub, vv, hubs, &ctl->i32[0], n, ctl);
    bool bad = false;
    warp_expand(beg, hub ? 0 : deg, [&](bool act, int e, int j) {
      const int u = __shfl_sync(IG_FULL, vv, j);
      const int du = __shfl_sync(IG_FULL, deg, j);
      const int ub = __shfl_sync(IG_FULL, beg, j);
      if (act) {
        const int w = __ldg(&nlist[e]);
        if (w == u || (e > ub && __ldg(&nlist[e - 1]) >= w) || w < 0 || w >= n) bad = true;
        else if (ranked ? w > u : before(du, u, __ldg(&nindex[w + 1]) - __ldg(&nindex[w]), w))
          atomicAdd(&s_cnt[wib][j], 1);
      }
    });
    __syncwarp();
    if (bad) raise(ctl, IG_ERR_UNSORTED);
    if (v < n && !hub) {
      const int oc = s_cnt[wib][lane];
      out_cnt[v] = oc;
      tc_items(oc, deg - oc, tc_exact(ranked, n, vv), block_chunk, &item_cnt[v], &item_cnt_b[v]);
    }
    __syncwarp();
  }
}

// Splits every adjacency list into its out part (kept in id order) and its
// in part (in_off[v] = nindex[v] - out_off[v]).
__global__ void __launch_bounds__(kThreads) tc_orient_fill(const int* __restrict__ nindex,
                                                           const int* __restrict__ nlist, int n,
                                                           const int* __restrict__ out_off, int* out_list,
                                                           int* in_list, const IgCtl* ctl) {
  using namespace ig;
  __shared__ int s_pos[kWarps][32];
  __shared__ int s_ipos[kWarps][32];
  if (ctl->err) return;
  const bool ranked = ctl->i32[1] == 0;
  const int lane = lane_id(), wib = threadIdx.x >> 5;
  const long long gtid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long gthreads = (long long)gridDim.x * blockDim.x;
  for (long long base = gtid & ~31LL; base < n; base += gthreads) {
    const long long v = base + lane;
    int beg = 0, deg = 0;
    if (v < n) {
      beg = __ldg(&nindex[v]);
      deg = __ldg(&nindex[v + 1]) - beg;
      const int oo = out_off[v];
      s_pos[wib][lane] = oo;
      s_ipos[wib][lane] = beg - oo;
    }
    __syncwarp();
    const int vv = (int)v;
    if (ranked) {
      // sorted list in (degree, id) order: the in part is the prefix below v
      // (in_list from in_off[v] = nindex[v] - out_off[v]), the out part the
      // suffix from split = nindex[v + 1] - |N+(v)|; each element goes
      // straight to its place
      int oo = 0, split = 0;
      if (v < n) {
        oo = out_off[v];
        split = beg + deg - (out_off[v + 1] - oo);
      }
      warp_expand(beg, deg > kOrientHub ? 0 : deg, [&](bool act, int e, int j) {
        const int ooj = __shfl_sync(IG_FULL, oo, j);
        const int spj = __shfl_sync(IG_FULL, split, j);
        if (act) {
          const int w = __ldg(&nlist[e]);
          if (e >= spj) out_list[ooj + (e - spj)] = w;
          else in_list[e - ooj] = w;
        }
      });
      continue;
    }
    warp_expand(beg, deg > kOrientHub ? 0 : deg, [&](bool act, int e, int j) {
      const int u = __shfl_sync(IG_FULL, vv, j);
      const int du = __shfl_sync(IG_FULL, deg, j);
      bool keep = false;
      int w = 0;
      if (act) {
        w = __ldg(&nlist[e]);
        const int dw = __ldg(&nindex[w + 1]) - __ldg(&nindex[w]);
        keep = before(du, u, dw, w);
      }
      // order-preserving compaction among lanes with the same owner
      const unsigned same = __match_any_sync(IG_FULL, act ? j : -1);
      const unsigned km = __ballot_sync(IG_FULL, keep) & same;
      const unsigned im = __ballot_sync(IG_FULL, act && !keep) & same;
      if (keep) out_list[s_pos[wib][j] + __popc(km & lanemask_lt())] = w;
      else if (act) in_list[s_ipos[wib][j] + __popc(im & lanemask_lt())] = w;
      __syncwarp();
      const int leader = 31 - __clz(same);  // highest lane of the group advances the cursors
      if (act && lane == leader) {
        s_pos[wib][j] += __popc(km);
        s_ipos[wib][j] += __popc(im);
      }
      __syncwarp();
    });
    __syncwarp();
  }
}

// Vertices above kOrientHub neighbours, one block each: count (and check)
// their out-neighbours.  With ids in (degree, id) order a hub's out part is
// the suffix above it, found by one thread with a binary search (the fill
// checks the list).
__global__ void __launch_bounds__(kThreads) tc_orient_hubs_count(const int* __restrict__ nindex,
                                                                 const int* __restrict__ nlist, int n,
                                                                 const int* hubs, int* out_cnt, int* item_cnt,
                                                                 int* item_cnt_b, int block_chunk, IgCtl* ctl) {
  using namespace ig;
  __shared__ int s_tmp[33];
  const int nh = ctl->i32[0];
  const bool ranked = ctl->i32[1] == 0;
  if (ranked) {
    for (long long h = (long long)blockIdx.x * blockDim.x + threadIdx.x; h < nh;
         h += (long long)gridDim.x * blockDim.x) {
      const int u = hubs[h];
      const int b = __ldg(&nindex[u]), e = __ldg(&nindex[u + 1]);
      int lo = b, hi = e;  // first entry above u
      while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(&nlist[mid]) <= u) lo = mid + 1;
        else hi = mid;
      }
      const int total = e - lo;
      out_cnt[u] = total;
      tc_items(total, e - b - total, tc_exact(true, n, u), block_chunk, &item_cnt[u], &item_cnt_b[u]);
    }
    return;
  }
  for (int h = blockIdx.x; h < nh; h += gridDim.x) {
    const int u = hubs[h];
    const int b = __ldg(&nindex[u]), e = __ldg(&nindex[u + 1]), du = e - b;
    int keep = 0;
    bool bad = false;
    for (int k = b + threadIdx.x; k < e; k += blockDim.x) {
      const int w = __ldg(&nlist[k]);
      if (w == u || (k > b && __ldg(&nlist[k - 1]) >= w) || w < 0 || w >= n) bad = true;
      else if (ranked ? w > u : before(du, u, __ldg(&nindex[w + 1]) - __ldg(&nindex[w]), w)) keep++;
    }
    if (bad) raise(ctl, IG_ERR_UNSORTED);
    int total;
    block_scan_int(keep, s_tmp, &total);
    if (threadIdx.x == 0) {
      out_cnt[u] = total;
      tc_items(total, du - total, tc_exact(ranked, n, u), block_chunk, &item_cnt[u], &item_cnt_b[u]);
    }
    __syncthreads();
  }
}

// Order-preserving split of the hub lists into out and in parts, one block
// per hub.  With ids in (degree, id) order the hubs are the last nh ids and
// their lists one contiguous range of nlist, copied in 256-entry chunks
// spread over all blocks (a chunk spans at most two hub lists, each longer
// than kOrientHub), each entry checked (sorted, no self loop, in range).
__global__ void __launch_bounds__(kThreads) tc_orient_hubs_fill(const int* __restrict__ nindex,
                                                                const int* __restrict__ nlist, int n,
                                                                const int* hubs,
                                                                const int* __restrict__ out_off, int* out_list,
                                                                int* in_list, IgCtl* ctl) {
  using namespace ig;
  __shared__ int s_tmp[33];
  __shared__ int s_u0;
  if (ctl->err) return;
  const int nh = ctl->i32[0];
  const bool ranked = ctl->i32[1] == 0;
  static_assert(kThreads <= kOrientHub, "a chunk must span at most two hub lists");
  if (ranked) {
    if (nh == 0) return;
    const int h0 = n - nh;  // first hub id
    const long long k0 = __ldg(&nindex[h0]), k1 = __ldg(&nindex[n]);
    bool bad = false;
    for (long long c0 = k0 + (long long)blockIdx.x * blockDim.x; c0 < k1; c0 += (long long)gridDim.x * blockDim.x) {
      __syncthreads();
      if (threadIdx.x == 0) {  // hub holding entry c0: last u in [h0, n) with nindex[u] <= c0
        int lo = h0, hi = n - 1;
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (__ldg(&nindex[mid]) <= c0) lo = mid;
          else hi = mid - 1;
        }
        s_u0 = lo;
      }
      __syncthreads();
      const long long k = c0 + threadIdx.x;
      if (k < k1) {
        const int u0 = s_u0;
        const int u = (u0 + 1 < n && k >= __ldg(&nindex[u0 + 1])) ? u0 + 1 : u0;
        const int b = __ldg(&nindex[u]), e = __ldg(&nindex[u + 1]);
        const int op = out_off[u];
        const int split = e - (out_off[u + 1] - op);
        const int w = __ldg(&nlist[k]);
        if (w == u || (k > b && __ldg(&nlist[k - 1]) >= w) || w < 0 || w >= n) bad = true;
        else if (k >= split) out_list[op + (k - split)] = w;
        else in_list[(b - op) + (k - b)] = w;
      }
    }
    if (bad) raise(ctl, IG_ERR_UNSORTED);
    return;
  }
  for (int h = blockIdx.x; h < nh; h += gridDim.x) {
    const int u = hubs[h];
    const int b = __ldg(&nindex[u]), e = __ldg(&nindex[u + 1]), du = e - b;
    int op = out_off[u], ip = b - op;
    for (int t = b; t < e; t += blockDim.x) {
      const int k = t + threadIdx.x;
      int w = 0;
      bool act = k < e, keep = false;
      if (act) {
        w = __ldg(&nlist[k]);
        keep = before(du, u, __ldg(&nindex[w + 1]) - __ldg(&nindex[w]), w);
      }
      int tk, ti;
      const int pk = block_scan_int(keep ? 1 : 0, s_tmp, &tk);
      const int pi = block_scan_int(act && !keep ? 1 : 0, s_tmp, &ti);
      if (keep) out_list[op + pk] = w;
      else if (act) in_list[ip + pi] = w;
      op += tk;
      ip += ti;
    }
    __syncthreads();
  }
}

__device__ __forceinline__ bool contains(const int* list, int len, int x) {
  int lo = 0, hi = len;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    const int y = list[mid];
    if (y < x) lo = mid + 1;
    else hi = mid;
  }
  return lo < len && list[lo] == x;
}

__device__ __forceinline__ unsigned hash_slot(int w, unsigned mask) { return ((unsigned)w * 0x9E3779B1u >> 7) & mask; }

// item_v[k] = middle vertex of work item k (items of v: [item_off[v], item_off[v+1])).
__global__ void __launch_bounds__(kThreads) tc_item_owner(const int* __restrict__ item_off, int n, int* item_v) {
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
    const int b = item_off[v], e = item_off[v + 1];
    for (int k = b; k < e; k++) item_v[k] = v;
  }
}

// Expansion of the 32 lanes' lists [beg, beg + deg) in steps of 128 slots,
// each lane taking four consecutive slots: one owner search per lane and
// step (five shuffles) for its first slot, then a walk forward over the list
// ends held in the warp's shared scratch `own` (65 ints), instead of one
// owner search per slot.  visit4(act[4], edge[4]) is called warp-uniformly.
template <class Visit4>
__device__ __forceinline__ void warp_expand_runs4(int beg, int deg, int* own, Visit4&& visit4) {
  const int lane = ig::lane_id();
  int incl = deg;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(IG_FULL, incl, o);
    if (lane >= o) incl += t;
  }
  const int total = __shfl_sync(IG_FULL, incl, 31);
  if (total == 0) return;
  const int excl = incl - deg;
  int* s_excl = own;       // [33]: list starts in slot numbering, then the total
  int* s_beg = own + 33;   // [32]: list starts in the edge array
  __syncwarp();
  s_excl[lane] = excl;
  s_beg[lane] = beg;
  if (lane == 31) s_excl[32] = total;
  __syncwarp();
  for (int base = 0; base < total; base += 128) {
    const int s0 = base + 4 * lane;
    int j = 0;  // last list starting at or before s0 (a non-empty one when s0 < total)
#pragma unroll
    for (int step = 16; step >= 1; step >>= 1) {
      const int ex = __shfl_sync(IG_FULL, excl, j + step);
      if (ex <= s0) j += step;
    }
    bool act[4];
    int e[4];
    int jn = s_excl[j + 1], jb = s_beg[j] - s_excl[j];
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const int sl = s0 + k;
      act[k] = sl < total;
      if (act[k]) {
        while (sl >= jn) {  // ends within the total: list 31 ends at s_excl[32]
          j++;
          jn = s_excl[j + 1];
          jb = s_beg[j] - s_excl[j];
        }
      }
      e[k] = act[k] ? jb + sl : 0;
    }
    visit4(act, e);
  }
  __syncwarp();
}

// Probes of one group of <= 32 in-neighbours u of middle vertex v, one per
// lane (in_list[g .. gend)): every w of N+(u) (only the part after v when ids
// are in (degree, id) order) is looked up in N+(v): with kExact in the bitmap
// `bits` over ids v+1 ..; otherwise filter bit first, then the hash table (or
// a binary search of N+(v) when it was too long to hash).  A hit closes the
// triangle u -> v -> w, counted once at v.  Returns this lane's hits.  All
// lanes of the warp call it.
template <int kBits, bool kExact = false>
__device__ __forceinline__ unsigned long long probe_group(const int* __restrict__ out_off,
                                                          const int* __restrict__ out_list,
                                                          const int* __restrict__ in_list, int g, int gend, int v,
                                                          int vb, int vd, bool ranked, const int* tab,
                                                          const unsigned* bits, unsigned mask, bool hashed,
                                                          int warp_list, int* own) {
  using namespace ig;
  const int lane = lane_id();
  unsigned hits = 0;  // this lane's, within one group
  int ub = 0, ud = 0;
  if (g + lane < gend) {
    const int u = __ldg(&in_list[g + lane]);
    ub = __ldg(&out_off[u]);
    const int ue = __ldg(&out_off[u + 1]);
    if (ranked) {
      // rank order = id order: only w > v in N+(u) can close u -> v -> w
      int lo2 = ub, hi2 = ue;
      while (lo2 < hi2) {
        const int mid = (lo2 + hi2) >> 1;
        if (__ldg(&out_list[mid]) <= v) lo2 = mid + 1;
        else hi2 = mid;
      }
      ub = lo2;
    }
    ud = ue - ub;
  }
  // membership of w in N+(v): filter bit first (rejects most misses with one
  // shared load), then the hash table or a binary search of N+(v)
  // exact bitmap: the word of id w is at the shared address sh0 + 4 (w / 32)
  // (sh0 folds the bitmap's first word in), so a probe is a shift, one
  // shared load and a bit test (w > v: only the part of N+(u) after v is scanned)
  const unsigned sh0 = kExact ? (unsigned)__cvta_generic_to_shared(bits) - 4u * (unsigned)((v + 1) >> 5) : 0u;
  auto probe = [&](int w) -> int {
    if (kExact) {
      unsigned word;
      asm volatile("ld.shared.u32 %0, [%1];" : "=r"(word) : "r"(sh0 + ((unsigned)(w >> 5) << 2)));
      return (word >> (w & 31)) & 1u;
    }
    if (hashed) {
      if (((bits[(w >> 5) & (kBits - 1)] >> (w & 31)) & 1u) == 0) return 0;
      unsigned h = hash_slot(w, mask);
      while (true) {
        const int t = tab[h];
        if (t == w) return 1;
        if (t == -1) return 0;
        h = (h + 1) & mask;
      }
    }
    return contains(out_list + vb, vd, w) ? 1 : 0;
  };
  // lists of at least warp_list probes: the whole warp walks one list at a
  // time (no per-slot owner search), 128 probes per step with no bounds
  // tests while 128 remain, then 32 per step for the rest
  unsigned longs = __ballot_sync(IG_FULL, ud >= warp_list);
  while (longs) {
    const int l = __ffs(longs) - 1;
    longs &= longs - 1;
    const int lb = __shfl_sync(IG_FULL, ub, l), le = lb + __shfl_sync(IG_FULL, ud, l);
    int base = lb;
    for (; le - base >= 128; base += 128) {
      int w[4];
#pragma unroll
      for (int k = 0; k < 4; k++) w[k] = __ldg(&out_list[base + k * 32 + lane]);
#pragma unroll
      for (int k = 0; k < 4; k++) hits += probe(w[k]);
    }
    for (; base < le; base += 32)
      if (base + lane < le) hits += probe(__ldg(&out_list[base + lane]));
  }
  if (ud >= warp_list) ud = 0;
  // short lists: 128 probe slots per step, load-balanced over the lanes
  // (four consecutive slots per lane with `own`, else four 32-slot columns,
  // each with its own owner search)
  auto visit = [&](const bool (&act)[4], const int (&e)[4]) {
    int w[4];
#pragma unroll
    for (int k = 0; k < 4; k++) w[k] = act[k] ? __ldg(&out_list[e[k]]) : -1;
#pragma unroll
    for (int k = 0; k < 4; k++)
      if (act[k]) hits += probe(w[k]);
  };
  if (own)
    warp_expand_runs4(ub, ud, own, visit);
  else
    warp_expand4(ub, ud, [&](const bool (&act)[4], const int (&e)[4], const int (&)[4]) { visit(act, e); });
  return hits;
}

// graph of vertex v in a batch: largest g with graph_vptr[g] <= v
__device__ __forceinline__ int tc_graph_of(const int* __restrict__ graph_vptr, int graphs, int v) {
  int lo = 0, hi = graphs - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(&graph_vptr[mid]) <= v) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// Adds the warp's hits since `before` to the count of v's graph (batched form).
__device__ __forceinline__ void tc_add_graph(unsigned long long mine, unsigned long long* count,
                                             const int* graph_vptr, int graphs, int v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mine += __shfl_xor_sync(IG_FULL, mine, o);
  if (ig::lane_id() == 0 && mine) atomicAdd(&count[tc_graph_of(graph_vptr, graphs, v)], mine);
}

// Warp work items: (middle vertex v with out-degree <= kBlockOut, or <= kWarpOut without an exact bitmap, kChunk of
// its in-neighbours).  The warp hashes N+(v) into its own small table.
// kBatched: the graph is a disjoint union; triangles are added to the count of
// the graph that holds their middle vertex (graph_vptr: first vertex of each graph).
template <bool kBatched>
__global__ void __launch_bounds__(kThreads) tc_count_warp(const int* __restrict__ out_off,
                                                          const int* __restrict__ out_list,
                                                          const int* __restrict__ nindex,
                                                          const int* __restrict__ in_list,
                                                          const int* __restrict__ item_off,
                                                          const int* __restrict__ item_v, int n,
                                                          unsigned long long* count, const IgCtl* ctl,
                                                          const int* __restrict__ graph_vptr, int graphs,
                                                          int warp_list, int runs) {
  using namespace ig;
  __shared__ int s_tab[kWarps][kWarpCap + kWarpBitWords];
  __shared__ int s_own[kWarps][65];
  if (ctl->err) return;
  const int lane = lane_id(), wib = threadIdx.x >> 5;
  int* tab = s_tab[wib];
  unsigned* bits = (unsigned*)(tab + kWarpCap);
  const int warp_g = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  const int items = __ldg(&item_off[n]);
  const bool ranked = ctl->i32[1] == 0;
  unsigned long long local = 0;
  int cur_v = -1;
  unsigned mask = 0;
  bool hashed = false;
  for (int it = warp_g; it < items; it += nwarps) {
    const int v = __ldg(&item_v[it]);  // middle vertex
    const int vb = __ldg(&out_off[v]);
    const int vd = __ldg(&out_off[v + 1]) - vb;
    if (v != cur_v) {
      cur_v = v;
      hashed = 2 * vd <= kWarpCap;
      if (hashed) {
        int cap = 32;
        while (cap < 2 * vd) cap <<= 1;
        mask = (unsigned)cap - 1;
        __syncwarp();
        for (int k = lane; k < cap; k += 32) tab[k] = -1;
        for (int k = lane; k < kWarpBitWords; k += 32) bits[k] = 0u;
        __syncwarp();
        for (int k = lane; k < vd; k += 32) {
          const int w = __ldg(&out_list[vb + k]);
          atomicOr(&bits[(w >> 5) & (kWarpBitWords - 1)], 1u << (w & 31));
          unsigned h = hash_slot(w, mask);
          while (atomicCAS(&tab[h], -1, w) != -1) h = (h + 1) & mask;
        }
        __syncwarp();
      }
    }
    const int ib = __ldg(&nindex[v]) - vb;  // in_off[v]
    const int iend = __ldg(&nindex[v + 1]) - __ldg(&out_off[v + 1]);
    const int c0 = ib + (it - __ldg(&item_off[v])) * kChunk;
    const int c1 = min(c0 + kChunk, iend);
    const unsigned long long before_item = local;
    for (int g = c0; g < c1; g += 32)
      local += probe_group<kWarpBitWords>(out_off, out_list, in_list, g, c1, v, vb, vd, ranked, tab, bits, mask,
                                          hashed, warp_list, runs ? s_own[wib] : nullptr);
    if (kBatched) tc_add_graph(local - before_item, count, graph_vptr, graphs, v);
  }
  if constexpr (!kBatched) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) local += __shfl_xor_sync(IG_FULL, local, o);
    if (lane == 0 && local) atomicAdd(count, local);
  }
}
// Block work items: (middle vertex v with out-degree > kBlockOut, up to
// block_chunk of its in-neighbours).  The block hashes N+(v) once into one
// shared table (9 KB instead of a 9 KB table per warp, so eight blocks fit
// on an SM) and its warps take groups of 32 in-neighbours from a shared
// counter until the item is done.  kExact: this launch takes the items whose
// N+(v) fits the exact bitmap (ids in (degree, id) order and fewer than 2^17
// ids above v) and the other launch the rest, so each path gets its own
// register allocation.
template <bool kBatched, bool kExact>
__global__ void __launch_bounds__(kThreads, 8) tc_count_block(const int* __restrict__ out_off,
                                                              const int* __restrict__ out_list,
                                                              const int* __restrict__ nindex,
                                                              const int* __restrict__ in_list,
                                                              const int* __restrict__ item_off,
                                                              const int* __restrict__ item_v, int n,
                                                              unsigned long long* count, const IgCtl* ctl,
                                                              const int* __restrict__ graph_vptr, int graphs,
                                                              int block_chunk, int grab, int* grab_ctr,
                                                              int warp_list, int runs) {
  using namespace ig;
  // the exact bitmap, or the hash table followed by the filter
  __shared__ unsigned s_mem[kExact ? kSpanWords : kHashCap + kBitWords];
  __shared__ int s_next;
  __shared__ int s_run;
  __shared__ int s_own[kWarps][65];
  int* own = runs ? s_own[threadIdx.x >> 5] : nullptr;
  int* tab = (int*)s_mem;
  unsigned* bits = s_mem + kHashCap;
  if (ctl->err) return;
  const int lane = lane_id();
  const int items = __ldg(&item_off[n]);
  const bool ranked = ctl->i32[1] == 0;
  unsigned long long local = 0;
  int cur_v = -1;
  unsigned mask = 0;
  bool hashed = false;
  // Items are taken one per block in a grid stride, or (grab > 0) in runs of
  // `grab` consecutive items from a counter, so that the items of one middle
  // vertex mostly stay in one block and its table is built once.
  auto next_run = [&](int cur) {
    if (grab <= 0) return cur < 0 ? (int)blockIdx.x : cur + (int)gridDim.x;
    __syncthreads();
    if (threadIdx.x == 0) s_run = atomicAdd(grab_ctr, grab);
    __syncthreads();
    return s_run;
  };
  for (int run = next_run(-1); run < items; run = next_run(run))
  for (int it = run; it < (grab > 0 ? min(run + grab, items) : run + 1); it++) {
    const int v = __ldg(&item_v[it]);  // middle vertex (block-uniform)
    if (tc_exact(ranked, n, v) != kExact) continue;  // the other launch's item
    const int vb = __ldg(&out_off[v]);
    const int vd = __ldg(&out_off[v + 1]) - vb;
    __syncthreads();  // the previous item's probes are done with the table and the counter
    if (v != cur_v) {
      cur_v = v;
      hashed = !kExact && 2 * vd <= kHashCap;
      if (kExact) {
        const int words = tc_span_words(n, v);
        const int wb = (v + 1) >> 5;
        for (int k = threadIdx.x; k < words; k += blockDim.x) s_mem[k] = 0u;
        __syncthreads();
        for (int k = threadIdx.x; k < vd; k += blockDim.x) {
          const int w = __ldg(&out_list[vb + k]);
          atomicOr(&s_mem[(w >> 5) - wb], 1u << (w & 31));
        }
      } else if (hashed) {
        int cap = 32;
        while (cap < 2 * vd) cap <<= 1;
        mask = (unsigned)cap - 1;
        for (int k = threadIdx.x; k < cap; k += blockDim.x) tab[k] = -1;
        for (int k = threadIdx.x; k < kBitWords; k += blockDim.x) bits[k] = 0u;
        __syncthreads();
        for (int k = threadIdx.x; k < vd; k += blockDim.x) {
          const int w = __ldg(&out_list[vb + k]);
          atomicOr(&bits[(w >> 5) & (kBitWords - 1)], 1u << (w & 31));
          unsigned h = hash_slot(w, mask);
          while (atomicCAS(&tab[h], -1, w) != -1) h = (h + 1) & mask;
        }
      }
    }
    if (threadIdx.x == 0) s_next = 0;
    __syncthreads();
    const int ib = __ldg(&nindex[v]) - vb;  // in_off[v]
    const int iend = __ldg(&nindex[v + 1]) - __ldg(&out_off[v + 1]);
    const int c0 = ib + (it - __ldg(&item_off[v])) * block_chunk;
    const int c1 = min(c0 + block_chunk, iend);
    const unsigned long long before_item = local;
    // groups of up to 32 in-neighbours per warp; an item with few takes
    // smaller groups (at least 4), about two per warp, so they spread over
    // the block's warps instead of leaving most of them at the next barrier
    const int gsz = min(32, max(4, (c1 - c0 + 2 * kWarps - 1) / (2 * kWarps)));
    while (true) {
      int g = 0;
      if (lane == 0) g = atomicAdd(&s_next, gsz);
      g = c0 + __shfl_sync(IG_FULL, g, 0);
      if (g >= c1) break;
      const int ge = min(g + gsz, c1);
      if constexpr (kExact)
        local += probe_group<kBitWords, true>(out_off, out_list, in_list, g, ge, v, vb, vd, true, tab, s_mem, mask,
                                              false, warp_list, own);
      else
        local += probe_group<kBitWords>(out_off, out_list, in_list, g, ge, v, vb, vd, ranked, tab, bits, mask,
                                        hashed, warp_list, own);
    }
    if (kBatched) tc_add_graph(local - before_item, count, graph_vptr, graphs, v);
  }
  if constexpr (!kBatched) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) local += __shfl_xor_sync(IG_FULL, local, o);
    if (lane == 0 && local) atomicAdd(count, local);
  }
}

}  // namespace

static int tc_run(IgExec* ex, int nodes, int edges, const int* d_nindex, const int* d_nlist, unsigned long long* d_count,
                  const int* d_graph_vptr, int graphs);

int igk_tc(IgExec* ex, int nodes, int edges, const int* d_nindex, const int* d_nlist, unsigned long long* d_count) {
  return tc_run(ex, nodes, edges, d_nindex, d_nlist, d_count, nullptr, 0);
}

int igk_tc_batched(IgExec* ex, int nodes, int edges, const int* d_nindex, const int* d_nlist,
                   const int* d_graph_vptr, int graphs, unsigned long long* d_counts) {
  return tc_run(ex, nodes, edges, d_nindex, d_nlist, d_counts, d_graph_vptr, graphs);
}

static int tc_run(IgExec* ex, int nodes, int edges, const int* d_nindex, const int* d_nlist, unsigned long long* d_count,
                  const int* d_graph_vptr, int graphs) {
  const size_t vb = ((size_t)nodes + 1) * sizeof(int);
  const int block_chunk = ig_exec_options(ex).tc_block_chunk;
  const int grab = ig_exec_options(ex).tc_grab;
  const int wl = ig_exec_options(ex).tc_warp_list;
  const int runs = ig_exec_options(ex).tc_runs;
  void *cnt, *off, *icnt, *ioff, *icnt_b, *ioff_b, *list, *inl, *hubs, *itemv, *itemv_b;
  int rc;
  if ((rc = ig_scratch_get(ex->scratch, IG_SLOT_V0, vb, &cnt))) return rc;
  if ((rc = ig_scratch_get(ex->scratch, IG_SLOT_V1, vb, &off))) return rc;
  if ((rc = ig_scratch_get(ex->scratch, IG_SLOT_V2, vb, &icnt))) return rc;
  if ((rc = ig_scratch_get(ex->scratch, IG_SLOT_Q0, vb, &ioff))) return rc;
  if ((rc = ig_scratch_get(ex->scratch, IG_SLOT_F0, vb, &icnt_b))) return rc;
  if ((rc = ig_scratch_get(ex->scratch, IG_SLOT_F1, vb, &ioff_b))) return rc;
  if ((rc = ig_scratch_get(ex->scratch, IG_SLOT_Q1, vb, &hubs))) return rc;
  // items: sum over v of ceil(|N-(v)| / chunk) <= edges / chunk + nodes
  if ((rc = ig_scratch_get(ex->scratch, IG_SLOT_Q2, ((size_t)edges / kChunk + (size_t)nodes + 1) * sizeof(int),
                           &itemv)))
    return rc;
  if ((rc = ig_scratch_get(ex->scratch, IG_SLOT_Q3,
                           ((size_t)edges / block_chunk + (size_t)nodes + 1) * sizeof(int), &itemv_b)))
    return rc;
  if ((rc = ig_scratch_get(ex->scratch, IG_SLOT_E0, std::max<size_t>(1, (size_t)edges) * sizeof(int), &list)))
    return rc;
  if ((rc = ig_scratch_get(ex->scratch, IG_SLOT_G1, std::max<size_t>(1, (size_t)edges) * sizeof(int), &inl)))
    return rc;
  if ((rc = ig_exec_reset(ex))) return rc;
  const size_t ncount = d_graph_vptr ? (size_t)graphs : 1;
  if ((rc = ig_cuda_check((int)cudaMemsetAsync(d_count, 0, ncount * sizeof(unsigned long long), ex->stream),
                          "memset")))
    return rc;
  const int grid = std::max(1, std::min((nodes + kThreads - 1) / kThreads, ex->sms * 8));
  tc_rank_check<<<grid, kThreads, 0, ex->stream>>>(d_nindex, nodes, ex->d_ctl);
  tc_orient_count<<<grid, kThreads, 0, ex->stream>>>(d_nindex, d_nlist, nodes, (int*)cnt, (int*)icnt, (int*)icnt_b,
                                                      (int*)hubs, block_chunk, ex->d_ctl);
  tc_orient_hubs_count<<<ex->sms * 8, kThreads, 0, ex->stream>>>(d_nindex, d_nlist, nodes, (const int*)hubs,
                                                                 (int*)cnt, (int*)icnt, (int*)icnt_b, block_chunk,
                                                                 ex->d_ctl);
  if ((rc = igk_exclusive_scan(ex, (const int*)cnt, (int*)off, nodes, nullptr))) return rc;
  if ((rc = igk_exclusive_scan(ex, (const int*)icnt, (int*)ioff, nodes, nullptr))) return rc;
  if ((rc = igk_exclusive_scan(ex, (const int*)icnt_b, (int*)ioff_b, nodes, nullptr))) return rc;
  tc_orient_fill<<<grid, kThreads, 0, ex->stream>>>(d_nindex, d_nlist, nodes, (const int*)off, (int*)list,
                                                     (int*)inl, ex->d_ctl);
  tc_orient_hubs_fill<<<ex->sms * 8, kThreads, 0, ex->stream>>>(d_nindex, d_nlist, nodes, (const int*)hubs,
                                                                (const int*)off, (int*)list, (int*)inl, ex->d_ctl);
  tc_item_owner<<<grid, kThreads, 0, ex->stream>>>((const int*)ioff, nodes, (int*)itemv);
  tc_item_owner<<<grid, kThreads, 0, ex->stream>>>((const int*)ioff_b, nodes, (int*)itemv_b);
  const int cgrid = ex->sms * 8;
  if (d_graph_vptr) {
    tc_count_block<true, true><<<cgrid, kThreads, 0, ex->stream>>>(
        (const int*)off, (const int*)list, d_nindex, (const int*)inl, (const int*)ioff_b, (const int*)itemv_b, nodes,
        d_count, ex->d_ctl, d_graph_vptr, graphs, block_chunk, grab, &ex->d_ctl->hot[0], wl, runs);
    tc_count_block<true, false><<<cgrid, kThreads, 0, ex->stream>>>(
        (const int*)off, (const int*)list, d_nindex, (const int*)inl, (const int*)ioff_b, (const int*)itemv_b, nodes,
        d_count, ex->d_ctl, d_graph_vptr, graphs, block_chunk, grab, &ex->d_ctl->hot[kCtlSpread], wl, runs);
    tc_count_warp<true><<<cgrid, kThreads, 0, ex->stream>>>((const int*)off, (const int*)list, d_nindex,
                                                            (const int*)inl, (const int*)ioff, (const int*)itemv,
                                                            nodes, d_count, ex->d_ctl, d_graph_vptr, graphs, wl, runs);
  } else {
    tc_count_block<false, true><<<cgrid, kThreads, 0, ex->stream>>>(
        (const int*)off, (const int*)list, d_nindex, (const int*)inl, (const int*)ioff_b, (const int*)itemv_b, nodes,
        d_count, ex->d_ctl, nullptr, 0, block_chunk, grab, &ex->d_ctl->hot[0], wl, runs);
    tc_count_block<false, false><<<cgrid, kThreads, 0, ex->stream>>>(
        (const int*)off, (const int*)list, d_nindex, (const int*)inl, (const int*)ioff_b, (const int*)itemv_b, nodes,
        d_count, ex->d_ctl, nullptr, 0, block_chunk, grab, &ex->d_ctl->hot[kCtlSpread], wl, runs);
    tc_count_warp<false><<<cgrid, kThreads, 0, ex->stream>>>((const int*)off, (const int*)list, d_nindex,
                                                             (const int*)inl, (const int*)ioff, (const int*)itemv,
                                                             nodes, d_count, ex->d_ctl, nullptr, 0, wl, runs);
  }
  ig_count_launches(10);
  return ig_cuda_check((int)cudaGetLastError(), "tc launch");
}
