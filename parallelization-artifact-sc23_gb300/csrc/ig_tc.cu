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
//   2. orient : keep edge u->w iff (deg u, u) < (deg w, w), so every vertex
//               keeps at most O(sqrt E) out-neighbours; the kept lists stay
//               sorted by id; counted per vertex, scanned, then filled
//   3. count  : for every u, the warp stages N+(u) in shared memory (when it
//               fits) and, with the load-balanced warp expansion over the
//               lists N+(v) of u's out-neighbours v, binary-searches every
//               w in N+(v) inside N+(u); a hit is the triangle {u, v, w}.
#include "ig_device.cuh"
#include "ig_options.h"

namespace {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kStage = 1024;  // out-neighbours of u staged per warp

__device__ __forceinline__ bool before(int du, int u, int dw, int w) { return du < dw || (du == dw && u < w); }

__global__ void __launch_bounds__(kThreads) tc_orient_count(const int* __restrict__ nindex,
                                                            const int* __restrict__ nlist, int n, int* out_cnt,
                                                            IgCtl* ctl) {
  using namespace ig;
  __shared__ int s_cnt[kWarps][32];
  const int lane = lane_id(), wib = threadIdx.x >> 5;
  const long long gtid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long gthreads = (long long)gridDim.x * blockDim.x;
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
    bool bad = false;
    warp_expand(beg, deg, [&](bool act, int e, int j) {
      const int u = __shfl_sync(IG_FULL, vv, j);
      const int du = __shfl_sync(IG_FULL, deg, j);
      const int ub = __shfl_sync(IG_FULL, beg, j);
      if (act) {
        const int w = __ldg(&nlist[e]);
        if (w == u || (e > ub && __ldg(&nlist[e - 1]) >= w) || w < 0 || w >= n) bad = true;
        else {
          const int dw = __ldg(&nindex[w + 1]) - __ldg(&nindex[w]);
          if (before(du, u, dw, w)) atomicAdd(&s_cnt[wib][j], 1);
        }
      }
    });
    __syncwarp();
    if (bad) raise(ctl, IG_ERR_UNSORTED);
    if (v < n) out_cnt[v] = s_cnt[wib][lane];
    __syncwarp();
  }
}

__global__ void __launch_bounds__(kThreads) tc_orient_fill(const int* __restrict__ nindex,
                                                           const int* __restrict__ nlist, int n,
                                                           const int* __restrict__ out_off, int* out_list,
                                                           const IgCtl* ctl) {
  using namespace ig;
  __shared__ int s_pos[kWarps][32];
  if (ctl->err) return;
  const int lane = lane_id(), wib = threadIdx.x >> 5;
  const long long gtid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long gthreads = (long long)gridDim.x * blockDim.x;
  for (long long base = gtid & ~31LL; base < n; base += gthreads) {
    const long long v = base + lane;
    int beg = 0, deg = 0;
    if (v < n) {
      beg = __ldg(&nindex[v]);
      deg = __ldg(&nindex[v + 1]) - beg;
      s_pos[wib][lane] = out_off[v];
    }
    __syncwarp();
    const int vv = (int)v;
    warp_expand(beg, deg, [&](bool act, int e, int j) {
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
      if (keep) out_list[s_pos[wib][j] + __popc(km & lanemask_lt())] = w;
      __syncwarp();
      const int leader = 31 - __clz(same);  // highest lane of the group updates the cursor
      if (act && lane == leader) s_pos[wib][j] += __popc(km);
      __syncwarp();
    });
    __syncwarp();
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

__global__ void __launch_bounds__(kThreads) tc_count(const int* __restrict__ out_off, const int* __restrict__ out_list,
                                                     int n, unsigned long long* count, const IgCtl* ctl) {
  using namespace ig;
  __shared__ int s_list[kWarps][kStage];
  if (ctl->err) return;
  const int lane = lane_id(), wib = threadIdx.x >> 5;
  const int warp_g = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  unsigned long long local = 0;
  for (int u = warp_g; u < n; u += nwarps) {
    const int ub = __ldg(&out_off[u]), ue = __ldg(&out_off[u + 1]);
    const int ulen = ue - ub;
    if (ulen < 2) continue;
    const int* ulist = out_list + ub;
    const bool staged = ulen <= kStage;
    if (staged) {
      for (int k = lane; k < ulen; k += 32) s_list[wib][k] = __ldg(&out_list[ub + k]);
      __syncwarp();
      ulist = s_list[wib];
    }
    for (int g = 0; g < ulen; g += 32) {
      int vb = 0, vd = 0;
      if (g + lane < ulen) {
        const int v = staged ? s_list[wib][g + lane] : __ldg(&out_list[ub + g + lane]);
        vb = __ldg(&out_off[v]);
        vd = __ldg(&out_off[v + 1]) - vb;
      }
      warp_expand(vb, vd, [&](bool act, int e, int) {
        if (act && contains(ulist, ulen, __ldg(&out_list[e]))) local++;
      });
    }
    __syncwarp();
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) local += __shfl_xor_sync(IG_FULL, local, o);
  if (lane == 0 && local) atomicAdd(count, local);
}

}  // namespace

int igk_tc(IgExec* ex, int nodes, int edges, const int* d_nindex, const int* d_nlist, unsigned long long* d_count) {
  const size_t vb = ((size_t)nodes + 1) * sizeof(int);
  void *cnt, *off, *list;
  int rc;
  if ((rc = ig_scratch_get(ex->scratch, IG_SLOT_V0, vb, &cnt))) return rc;
  if ((rc = ig_scratch_get(ex->scratch, IG_SLOT_V1, vb, &off))) return rc;
  if ((rc = ig_scratch_get(ex->scratch, IG_SLOT_E0, std::max<size_t>(1, (size_t)edges) * sizeof(int), &list)))
    return rc;
  if ((rc = ig_exec_reset(ex))) return rc;
  if ((rc = ig_cuda_check((int)cudaMemsetAsync(d_count, 0, sizeof(unsigned long long), ex->stream), "memset")))
    return rc;
  const int grid = std::max(1, std::min((nodes + kThreads - 1) / kThreads, ex->sms * 8));
  tc_orient_count<<<grid, kThreads, 0, ex->stream>>>(d_nindex, d_nlist, nodes, (int*)cnt, ex->d_ctl);
  if ((rc = igk_exclusive_scan(ex, (const int*)cnt, (int*)off, nodes, nullptr))) return rc;
  tc_orient_fill<<<grid, kThreads, 0, ex->stream>>>(d_nindex, d_nlist, nodes, (const int*)off, (int*)list, ex->d_ctl);
  tc_count<<<ex->sms * 8, kThreads, 0, ex->stream>>>((const int*)off, (const int*)list, nodes, d_count, ex->d_ctl);
  ig_count_launches(3);
  return ig_cuda_check((int)cudaGetLastError(), "tc launch");
}
