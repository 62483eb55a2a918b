// Device-side building blocks shared by the graph kernels:
//   - relaxed / acquire / release accessors (hand-written PTX),
//   - a grid barrier for cooperatively launched persistent kernels whose
//     wait is bounded by %globaltimer and reports IG_ERR_TIMEOUT,
//   - warp-aggregated queue append (one atomic per warp),
//   - load-balanced expansion of the adjacency lists of 32 vertices held one
//     per lane (the warp walks their concatenated edge ranges 32 at a time).
#pragma once

#include <cuda_runtime.h>
#include <climits>
#include <cstdint>

#include "ig_internal.h"

#define IG_FULL 0xffffffffu

namespace ig {

constexpr int kInf = INT_MAX;

__device__ __forceinline__ int lane_id() { return threadIdx.x & 31; }
__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

__device__ __forceinline__ unsigned long long globaltimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release(unsigned* p, unsigned v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned atom_add_acqrel(unsigned* p, unsigned v) {
  unsigned old;
  asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], %2;"
               : "=r"(old)
               : "l"(p), "r"(v)
               : "memory");
  return old;
}
__device__ __forceinline__ int ld_relaxed(const int* p) {
  int v;
  asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ unsigned long long ld_relaxed(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ long long ld_relaxed(const long long* p) {
  long long v;
  asm volatile("ld.relaxed.gpu.global.s64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ double ld_relaxed(const double* p) {
  double v;
  asm volatile("ld.relaxed.gpu.global.f64 %0, [%1];" : "=d"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void st_relaxed(unsigned long long* p, unsigned long long v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ int ld_acquire(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void red_add_release(int* p, int v) {
  asm volatile("red.release.gpu.global.add.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Hot counter k of the control block (see IgCtl::hot), as int or 64-bit.
__device__ __forceinline__ int* hot32(IgCtl* ctl, int k) { return &ctl->hot[k * kCtlSpread]; }
__device__ __forceinline__ unsigned long long* hot64(IgCtl* ctl, int k) {
  return (unsigned long long*)&ctl->hot[k * kCtlSpread];
}

// Top bit of the grid barrier's arrival count: set by every raise, so the
// last block to arrive learns of an error from its own arrival (see grid_sync).
constexpr unsigned kArriveErr = 0x80000000u;

// Records the first device-side error (and flags it to the grid barrier).
__device__ __forceinline__ void raise(IgCtl* ctl, int code) {
  atomicCAS(&ctl->err, 0, code);
  atomicOr(&ctl->sync.arrive, kArriveErr);
}

// Grid-wide barrier for a cooperative launch.  Returns false (in every
// thread of the block) when the barrier failed: a block raised an error
// before arriving, or the wait exceeded `timeout_ns`; the caller must then
// return.  Pattern: block barrier, one thread publishes its block's writes
// with a gpu-scope fence and arrives; the last arriver resets the count and
// bumps the generation with release semantics, its top bit set when the
// arrival count carried the error flag (every raise flags it, so a raise
// before any block's arrival is seen by the last arriver's own atomic); the
// others spin on an acquire load of the generation (bounded, watching the
// error word), then fence and release their block.
// `GridBar` keeps the block's view of the generation between barriers, so a
// barrier costs one atomic round trip and the wait (the generation is read
// once per kernel, at its first barrier; blocks cannot pass a barrier before
// every block has arrived, so all read the same value).
constexpr unsigned kGenErr = 0x80000000u;
struct GridBar {
  unsigned gen = 0;
  bool known = false;
};

__device__ __forceinline__ bool grid_sync(IgCtl* ctl, unsigned long long timeout_ns, GridBar& gb) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    IgSync* s = &ctl->sync;
    if (!gb.known) {
      gb.gen = ld_acquire(&s->gen) & ~kGenErr;
      gb.known = true;
    }
    const unsigned next = (gb.gen + 1) & ~kGenErr;
    __threadfence();
    const unsigned old = atom_add_acqrel(&s->arrive, 1u);
    if ((old & ~kArriveErr) == gridDim.x - 1) {
      atomicExch(&s->arrive, 0u);
      const unsigned e = (old & kArriveErr) ? kGenErr : 0u;
      st_release(&s->gen, next | e);
      ok = e == 0;
    } else {
      const unsigned long long t0 = globaltimer();
      unsigned spins = 0, g;
      while (((g = ld_acquire(&s->gen)) & ~kGenErr) == gb.gen) {
        if ((++spins & 63u) == 0) {
          if (ld_relaxed(&ctl->err) != 0) { ok = 0; break; }
          if (globaltimer() - t0 > timeout_ns) {
            raise(ctl, IG_ERR_TIMEOUT);
            ok = 0;
            break;
          }
        }
        __nanosleep(32);
      }
      if (ok && (g & kGenErr)) ok = 0;
    }
    gb.gen = next;
    __threadfence();
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// The same barrier for a kernel that keeps no GridBar (the generation is
// read at every call).
__device__ __forceinline__ bool grid_sync(IgCtl* ctl, unsigned long long timeout_ns) {
  GridBar gb;
  return grid_sync(ctl, timeout_ns, gb);
}

// Warp-aggregated append: every lane of a converged warp calls it; lanes with
// pred append `v` to q.  One atomicAdd per warp.  Returns the number appended.
__device__ __forceinline__ int warp_append(bool pred, int v, int* q, int* qsize, int cap,
                                           IgCtl* ctl) {
  const unsigned m = __ballot_sync(IG_FULL, pred);
  if (m == 0) return 0;
  const int lane = lane_id();
  const int leader = __ffs(m) - 1;
  int base = 0;
  if (lane == leader) base = atomicAdd(qsize, __popc(m));
  base = __shfl_sync(IG_FULL, base, leader);
  if (pred) {
    const int pos = base + __popc(m & lanemask_lt());
    if (pos < cap) q[pos] = v;
    else raise(ctl, IG_ERR_OVERFLOW);
  }
  return __popc(m);
}

// Same as warp_append, also adding the 64-bit sum of `w` over appending lanes
// to *wsum (used for the frontier edge count of direction-optimising BFS).
__device__ __forceinline__ void warp_append_w(bool pred, int v, long long w, int* q, int* qsize,
                                              unsigned long long* wsum, int cap, IgCtl* ctl) {
  const unsigned m = __ballot_sync(IG_FULL, pred);
  if (m == 0) return;
  long long x = pred ? w : 0;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(IG_FULL, x, o);
  const int lane = lane_id();
  const int leader = __ffs(m) - 1;
  int base = 0;
  if (lane == leader) {
    base = atomicAdd(qsize, __popc(m));
    atomicAdd(wsum, (unsigned long long)x);
  }
  base = __shfl_sync(IG_FULL, base, leader);
  if (pred) {
    const int pos = base + __popc(m & lanemask_lt());
    if (pos < cap) q[pos] = v;
    else raise(ctl, IG_ERR_OVERFLOW);
  }
}

// Load-balanced expansion.  Each lane holds one vertex's edge range
// [beg, beg+deg) (deg may be 0).  The warp walks the concatenation of the 32
// ranges, 32 edges per step; for edge slot e the owning lane j is found by a
// 5-step binary search over the exclusive prefix of the degrees.
// visit(active, edge_index, owner_lane) is called by all 32 lanes every step
// (warp-uniform), so it may use warp collectives.
template <class Visit>
__device__ __forceinline__ void warp_expand(int beg, int deg, Visit&& visit) {
  const int lane = lane_id();
  int incl = deg;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(IG_FULL, incl, o);
    if (lane >= o) incl += t;
  }
  const int total = __shfl_sync(IG_FULL, incl, 31);
  const int excl = incl - deg;
  for (int base = 0; base < total; base += 32) {
    const int e = base + lane;
    int j = 0;
#pragma unroll
    for (int step = 16; step >= 1; step >>= 1) {
      const int ex = __shfl_sync(IG_FULL, excl, j + step);
      if (ex <= e) j += step;
    }
    const int jb = __shfl_sync(IG_FULL, beg, j);
    const int je = __shfl_sync(IG_FULL, excl, j);
    visit(e < total, jb + (e - je), j);
  }
}

// Block-wide exclusive scan of `n <= blockDim.x * 4` 64-bit values held in
// shared memory `vals` (in place; vals[n] receives the total).  Requires all
// threads of the block; `warp_tmp` must hold blockDim.x/32 entries.
__device__ __forceinline__ void block_exclusive_scan64(long long* vals, int n, long long* warp_tmp) {
  const int tid = threadIdx.x;
  const int per = (n + blockDim.x - 1) / blockDim.x;  // <= 4
  long long local[4];
  long long sum = 0;
  for (int k = 0; k < per && k < 4; k++) {
    const int i = tid * per + k;
    local[k] = (i < n) ? vals[i] : 0;
    sum += local[k];
  }
  // inclusive scan of per-thread sums
  const int lane = tid & 31, warp = tid >> 5;
  long long x = sum;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const long long t = __shfl_up_sync(IG_FULL, x, o);
    if (lane >= o) x += t;
  }
  if (lane == 31) warp_tmp[warp] = x;
  __syncthreads();
  if (warp == 0) {
    const int nw = blockDim.x >> 5;
    long long w = (lane < nw) ? warp_tmp[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const long long t = __shfl_up_sync(IG_FULL, w, o);
      if (lane >= o) w += t;
    }
    if (lane < nw) warp_tmp[lane] = w;  // inclusive warp totals
  }
  __syncthreads();
  long long run = x - sum + (warp > 0 ? warp_tmp[warp - 1] : 0);
  for (int k = 0; k < per && k < 4; k++) {
    const int i = tid * per + k;
    if (i < n) vals[i] = run;
    run += local[k];
  }
  if (tid == blockDim.x - 1) vals[n] = run;
  __syncthreads();
}

// The reference MIS priority hash (include/mis_vertex_cpp.h:135-140),
// applied to v + 712313887 with unsigned arithmetic.
__device__ __forceinline__ unsigned mis_hash(unsigned val) {
  val = ((val >> 16) ^ val) * 0x45d9f3bu;
  val = ((val >> 16) ^ val) * 0x45d9f3bu;
  return (val >> 16) ^ val;
}
__device__ __forceinline__ unsigned mis_priority(int v) { return mis_hash((unsigned)v + 712313887u); }

}  // namespace ig

namespace ig {

// Vertices with more neighbours than this are expanded by the whole grid.
constexpr int kHubBatch = 1024;  // hubs staged per shared-memory pass

// Expands the adjacency lists of the `nh` vertices in `hubs` across every
// thread of the grid (edge-balanced).  visit(active, edge_index, hub_vertex)
// is called warp-uniformly.  Requires blockDim.x * 4 >= kHubBatch and all
// threads of every block.
template <class Visit>
__device__ __forceinline__ void grid_expand_hubs(const int* __restrict__ nindex, const int* hubs, int nh,
                                                 Visit&& visit) {
  __shared__ long long s_pref[kHubBatch + 1];
  __shared__ int s_beg[kHubBatch];
  __shared__ int s_v[kHubBatch];
  __shared__ long long s_warp[32];
  const long long gthreads = (long long)gridDim.x * blockDim.x;
  for (int hb = 0; hb < nh; hb += kHubBatch) {
    const int cnt = min(kHubBatch, nh - hb);
    __syncthreads();
    for (int i = threadIdx.x; i < cnt; i += blockDim.x) {
      const int v = hubs[hb + i];
      const int b = __ldg(&nindex[v]);
      s_v[i] = v;
      s_beg[i] = b;
      s_pref[i] = __ldg(&nindex[v + 1]) - b;
    }
    __syncthreads();
    block_exclusive_scan64(s_pref, cnt, s_warp);
    const long long total = s_pref[cnt];
    const long long wbase = (long long)blockIdx.x * blockDim.x + (threadIdx.x & ~31);
    for (long long base = wbase; base < total; base += gthreads) {
      const long long e = base + lane_id();
      const bool act = e < total;
      int h = 0;
      if (act) {
        int lo = 0, hi = cnt - 1;  // largest h with s_pref[h] <= e
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (s_pref[mid] <= e) lo = mid;
          else hi = mid - 1;
        }
        h = lo;
      }
      visit(act, act ? s_beg[h] + (int)(e - s_pref[h]) : 0, act ? s_v[h] : 0);
    }
  }
  __syncthreads();
}

}  // namespace ig

namespace ig {

// Block-wide exclusive scan of one int per thread; returns the thread's
// exclusive prefix and writes the block total to *total (all threads).
// `tmp` must hold 33 ints of shared memory.
__device__ __forceinline__ int block_scan_int(int x, int* tmp, int* total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  int incl = x;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(IG_FULL, incl, o);
    if (lane >= o) incl += t;
  }
  __syncthreads();
  if (lane == 31) tmp[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    int w = (lane < nw) ? tmp[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(IG_FULL, w, o);
      if (lane >= o) w += t;
    }
    if (lane < nw) tmp[lane] = w;
    if (lane == nw - 1) tmp[32] = w;
  }
  __syncthreads();
  const int res = incl - x + (warp > 0 ? tmp[warp - 1] : 0);
  *total = tmp[32];
  return res;
}

// Block-wide sum of 64-bit integers (exact); the result is valid in thread 0.
// `tmp` must hold 32 values.
__device__ __forceinline__ unsigned long long block_sum_u64(unsigned long long x, unsigned long long* tmp) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(IG_FULL, x, o);
  __syncthreads();
  if (lane == 0) tmp[warp] = x;
  __syncthreads();
  unsigned long long r = 0;
  if (warp == 0) {
    r = (lane < nw) ? tmp[lane] : 0ull;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) r += __shfl_down_sync(IG_FULL, r, o);
  }
  return r;
}

// Block-wide sum of a double with a fixed reduction tree (deterministic);
// the result is valid in thread 0.  `tmp` must hold 32 doubles.
__device__ __forceinline__ double block_sum_double(double x, double* tmp) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(IG_FULL, x, o);
  __syncthreads();
  if (lane == 0) tmp[warp] = x;
  __syncthreads();
  double r = 0;
  if (warp == 0) {
    r = (lane < nw) ? tmp[lane] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) r += __shfl_down_sync(IG_FULL, r, o);
  }
  return r;
}

}  // namespace ig

namespace ig {

// Warp-aggregated append of up to kMax items per lane (items[0..cnt)): one
// atomicAdd per warp.  All lanes of a converged warp call it.
template <int kMax>
__device__ __forceinline__ void warp_append_n(int cnt, const int (&items)[kMax], int* q, int* qsize, int cap,
                                              IgCtl* ctl) {
  const int lane = lane_id();
  int incl = cnt;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(IG_FULL, incl, o);
    if (lane >= o) incl += t;
  }
  const int total = __shfl_sync(IG_FULL, incl, 31);
  if (total == 0) return;
  int base = 0;
  if (lane == 31) base = atomicAdd(qsize, total);
  base = __shfl_sync(IG_FULL, base, 31) + incl - cnt;
#pragma unroll
  for (int k = 0; k < kMax; k++) {
    if (k < cnt) {
      if (base + k < cap) q[base + k] = items[k];
      else raise(ctl, IG_ERR_OVERFLOW);
    }
  }
}

// Load-balanced expansion like warp_expand, four 32-edge steps at a time:
// visit4(act[4], edge[4], owner_lane[4]) is called warp-uniformly with the
// four slots of each lane, so the callee can issue their memory operations
// together (more loads in flight per lane than one step at a time).
template <class Visit4>
__device__ __forceinline__ void warp_expand4(int beg, int deg, Visit4&& visit4) {
  const int lane = lane_id();
  int incl = deg;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(IG_FULL, incl, o);
    if (lane >= o) incl += t;
  }
  const int total = __shfl_sync(IG_FULL, incl, 31);
  const int excl = incl - deg;
  for (int base = 0; base < total; base += 128) {
    bool act[4];
    int edge[4], own[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const int e = base + k * 32 + lane;
      int j = 0;
#pragma unroll
      for (int step = 16; step >= 1; step >>= 1) {
        const int ex = __shfl_sync(IG_FULL, excl, j + step);
        if (ex <= e) j += step;
      }
      const int jb = __shfl_sync(IG_FULL, beg, j);
      const int je = __shfl_sync(IG_FULL, excl, j);
      act[k] = e < total;
      edge[k] = jb + (e - je);
      own[k] = j;
    }
    visit4(act, edge, own);
  }
}

}  // namespace ig

namespace ig {

// Per-warp staging of worklist appends in shared memory.  A warp gathers the
// items it appends in its own buffer and writes them to the global queue 32
// at a time (one atomicAdd on the queue counter and one coalesced 128-byte
// store per 32 items) instead of one atomicAdd per warp step on a counter that
// every warp of the grid hits.  `n` is the warp-uniform number of buffered
// items; warp_buf_flush must run before the items are needed (the grid
// barrier that ends the phase).
constexpr int kWarpBuf = 160;  // 32 + the most items one step adds (32 lanes x 4)

template <int kMax>
__device__ __forceinline__ void warp_buf_append(int cnt, const int (&items)[kMax], int* buf, int& n, int* q,
                                                int* qsize, int cap, IgCtl* ctl) {
  const int lane = lane_id();
  int incl = cnt;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(IG_FULL, incl, o);
    if (lane >= o) incl += t;
  }
  const int total = __shfl_sync(IG_FULL, incl, 31);
  if (total == 0) return;
  const int pos = n + incl - cnt;
#pragma unroll
  for (int k = 0; k < kMax; k++)
    if (k < cnt) buf[pos + k] = items[k];
  n += total;
  __syncwarp();
  while (n >= 32) {
    int base = 0;
    if (lane == 0) base = atomicAdd(qsize, 32);
    base = __shfl_sync(IG_FULL, base, 0);
    const int v = buf[lane];
    if (base + lane < cap) q[base + lane] = v;
    else raise(ctl, IG_ERR_OVERFLOW);
    __syncwarp();
    // move the rest down by 32: lane l reads index i and writes i - 32, and
    // index i - 32 was read by the same lane one pass earlier
    for (int i = 32 + lane; i < n; i += 32) buf[i - 32] = buf[i];
    __syncwarp();
    n -= 32;
  }
}

// Writes out full groups of 32 buffered items (warp-uniform n).
__device__ __forceinline__ void warp_buf_drain(int* buf, int& n, int* q, int* qsize, int cap, IgCtl* ctl) {
  const int lane = lane_id();
  while (n >= 32) {
    int base = 0;
    if (lane == 0) base = atomicAdd(qsize, 32);
    base = __shfl_sync(IG_FULL, base, 0);
    const int v = buf[lane];
    if (base + lane < cap) q[base + lane] = v;
    else raise(ctl, IG_ERR_OVERFLOW);
    __syncwarp();
    for (int i = 32 + lane; i < n; i += 32) buf[i - 32] = buf[i];
    __syncwarp();
    n -= 32;
  }
}

// Two warp_buf_append calls for two queues in one: slot k of this lane holds
// v[k], appended to the first queue if f1[k] and to the second if f2[k].  The
// per-lane counts of both (at most kMax each, so a warp's total fits in 16
// bits) are scanned together, and a warp with nothing to append returns after
// one ballot.  Flags rather than compacted arrays keep every register array
// statically indexed, so nothing goes to local memory.
template <int kMax>
__device__ __forceinline__ void warp_buf_append2_flags(const int (&v)[kMax], const bool (&f1)[kMax], int* b1, int& n1,
                                                       int* q1, int* s1, const bool (&f2)[kMax], int* b2, int& n2,
                                                       int* q2, int* s2, int cap, IgCtl* ctl) {
  int c1 = 0, c2 = 0;
#pragma unroll
  for (int k = 0; k < kMax; k++) {
    c1 += f1[k];
    c2 += f2[k];
  }
  if (__ballot_sync(IG_FULL, (c1 | c2) != 0) == 0) return;
  const int lane = lane_id();
  const int packed = c1 | (c2 << 16);
  int incl = packed;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(IG_FULL, incl, o);
    if (lane >= o) incl += t;
  }
  const int total = __shfl_sync(IG_FULL, incl, 31);
  const int ex = incl - packed;
  int p1 = n1 + (ex & 0xffff), p2 = n2 + (ex >> 16);
#pragma unroll
  for (int k = 0; k < kMax; k++) {
    if (f1[k]) b1[p1++] = v[k];
    if (f2[k]) b2[p2++] = v[k];
  }
  n1 += total & 0xffff;
  n2 += total >> 16;
  __syncwarp();
  warp_buf_drain(b1, n1, q1, s1, cap, ctl);
  warp_buf_drain(b2, n2, q2, s2, cap, ctl);
}

// warp_buf_flush of two buffers (fewer than 32 items each) with both queue
// reservations in flight together.
__device__ __forceinline__ void warp_buf_flush2(int* b1, int& n1, int* q1, int* s1, int* b2, int& n2, int* q2,
                                                int* s2, int cap, IgCtl* ctl) {
  if ((n1 | n2) == 0) return;  // warp-uniform
  const int lane = lane_id();
  int base = 0;
  if (lane == 0 && n1) base = atomicAdd(s1, n1);
  if (lane == 1 && n2) base = atomicAdd(s2, n2);
  const int p1 = __shfl_sync(IG_FULL, base, 0), p2 = __shfl_sync(IG_FULL, base, 1);
  if (lane < n1) {
    if (p1 + lane < cap) q1[p1 + lane] = b1[lane];
    else raise(ctl, IG_ERR_OVERFLOW);
  }
  if (lane < n2) {
    if (p2 + lane < cap) q2[p2 + lane] = b2[lane];
    else raise(ctl, IG_ERR_OVERFLOW);
  }
  __syncwarp();
  n1 = n2 = 0;
}

__device__ __forceinline__ void warp_buf_flush(int* buf, int& n, int* q, int* qsize, int cap, IgCtl* ctl) {
  if (n == 0) return;  // warp-uniform
  const int lane = lane_id();
  int base = 0;
  if (lane == 0) base = atomicAdd(qsize, n);
  base = __shfl_sync(IG_FULL, base, 0);
  if (lane < n) {
    if (base + lane < cap) q[base + lane] = buf[lane];
    else raise(ctl, IG_ERR_OVERFLOW);
  }
  __syncwarp();
  n = 0;
}

}  // namespace ig
