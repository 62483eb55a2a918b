// Device-wide exclusive scan of int counts (three short kernels: tile sums,
// scan of the tile sums in one block, tile scans with their offsets).
#include "ig_device.cuh"

namespace {

constexpr int kThreads = 256;
constexpr int kPer = 8;
constexpr int kTile = kThreads * kPer;

__global__ void __launch_bounds__(kThreads) scan_tile_sums(const int* __restrict__ in, int n, long long* tile_sum) {
  __shared__ int s_tmp[33];
  const long long t0 = (long long)blockIdx.x * kTile;
  int s = 0;
  for (int k = 0; k < kPer; k++) {
    const long long i = t0 + (long long)threadIdx.x * kPer + k;
    if (i < n) s += in[i];
  }
  int total;
  ig::block_scan_int(s, s_tmp, &total);
  if (threadIdx.x == 0) tile_sum[blockIdx.x] = total;
}

__global__ void __launch_bounds__(1024) scan_tile_offsets(long long* tile_sum, int tiles) {
  __shared__ long long s_warp[32];
  __shared__ long long s_carry;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) s_carry = 0;
  __syncthreads();
  for (int b0 = 0; b0 < tiles; b0 += blockDim.x) {
    const int i = b0 + threadIdx.x;
    const long long x = i < tiles ? tile_sum[i] : 0;
    long long incl = x;
    for (int o = 1; o < 32; o <<= 1) {
      const long long t = __shfl_up_sync(IG_FULL, incl, o);
      if (lane >= o) incl += t;
    }
    if (lane == 31) s_warp[warp] = incl;
    __syncthreads();
    if (warp == 0) {
      long long w = s_warp[lane];
      for (int o = 1; o < 32; o <<= 1) {
        const long long t = __shfl_up_sync(IG_FULL, w, o);
        if (lane >= o) w += t;
      }
      s_warp[lane] = w;
    }
    __syncthreads();
    const long long excl = incl - x + (warp > 0 ? s_warp[warp - 1] : 0) + s_carry;
    if (i < tiles) tile_sum[i] = excl;
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) s_carry = excl + x;
    __syncthreads();
  }
  if (threadIdx.x == 0) tile_sum[tiles] = s_carry;
}

__global__ void __launch_bounds__(kThreads) scan_tiles(const int* __restrict__ in, int n, const long long* tile_off,
                                                       int* out, int tiles) {
  __shared__ int s_tmp[33];
  const long long t0 = (long long)blockIdx.x * kTile;
  int v[kPer];
  int s = 0;
  for (int k = 0; k < kPer; k++) {
    const long long i = t0 + (long long)threadIdx.x * kPer + k;
    v[k] = i < n ? in[i] : 0;
    s += v[k];
  }
  int total;
  int run = ig::block_scan_int(s, s_tmp, &total) + (int)tile_off[blockIdx.x];
  for (int k = 0; k < kPer; k++) {
    const long long i = t0 + (long long)threadIdx.x * kPer + k;
    if (i < n) out[i] = run;
    run += v[k];
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) out[n] = (int)tile_off[tiles];
}

}  // namespace

int igk_exclusive_scan(IgExec* ex, const int* in, int* out, int n, long long* total_host) {
  const int tiles = std::max(1, (n + kTile - 1) / kTile);
  void* ts;
  int rc;
  if ((rc = ig_scratch_get(ex->scratch, IG_SLOT_BLK, ((size_t)tiles + 1) * sizeof(long long), &ts))) return rc;
  scan_tile_sums<<<tiles, kThreads, 0, ex->stream>>>(in, n, (long long*)ts);
  scan_tile_offsets<<<1, 1024, 0, ex->stream>>>((long long*)ts, tiles);
  scan_tiles<<<tiles, kThreads, 0, ex->stream>>>(in, n, (const long long*)ts, out, tiles);
  ig_count_launches(3);
  rc = ig_cuda_check((int)cudaGetLastError(), "scan launch");
  if (rc || !total_host) return rc;
  return ig_cuda_check((int)cudaMemcpyAsync(total_host, (long long*)ts + tiles, sizeof(long long),
                                            cudaMemcpyDeviceToHost, ex->stream),
                       "scan total");
}
