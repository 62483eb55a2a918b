// Calibration: the device's rate of random 4-byte gathers.
//
// The graph kernels here spend their time on data-dependent reads of
// per-vertex arrays (distances, contributions, labels) at random positions;
// each such read moves a 32-byte sector, so their ceiling is the rate of
// random sector accesses, not the copy bandwidth.  This kernel measures that
// rate: every thread reads 8 independent hashed positions of a table per step
// (no index array is streamed) and keeps a sum so the reads are not removed.
// With the table the size of a per-vertex array (e.g. 16.8 MB at 4.2M
// vertices) the reads hit the L2; with a table larger than L2 they go to HBM.
#include "ig_device.cuh"

namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ unsigned long long mix64(unsigned long long x) {
  // SplitMix64 finaliser (Steele, Lea, Flood 2014)
  x ^= x >> 30;
  x *= 0xbf58476d1ce4e5b9ull;
  x ^= x >> 27;
  x *= 0x94d049bb133111ebull;
  x ^= x >> 31;
  return x;
}

__global__ void __launch_bounds__(kThreads) gather_probe(const float* __restrict__ table, long long n,
                                                         long long per_thread, unsigned long long salt,
                                                         float* sink) {
  const long long gtid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  float acc = 0.f;
  unsigned long long key = mix64(((unsigned long long)gtid << 20) ^ salt);
  for (long long i = 0; i < per_thread; i += 8) {
    long long pos[8];
#pragma unroll
    for (int k = 0; k < 8; k++) {
      key = mix64(key + 0x9e3779b97f4a7c15ull);
      // uniform in [0, n) with one multiply-high (n < 2^32 here)
      pos[k] = (long long)__umulhi((unsigned)(key >> 32), (unsigned)n);
    }
    float x[8];
#pragma unroll
    for (int k = 0; k < 8; k++) x[k] = table[pos[k]];
#pragma unroll
    for (int k = 0; k < 8; k++) acc += x[k];
  }
  sink[gtid] = acc;
}

__global__ void fill_table(float* t, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    t[i] = (float)(i & 1023);
}

}  // namespace

extern "C" int ig_probe_random_gather(long long table_elems, long long gathers, int reps, double* gathers_per_s) {
  if (table_elems < 1 || table_elems > 0xffffffffLL || gathers < 1 || reps < 1 || !gathers_per_s)
    return ig_fail(IG_ERR_INVALID_ARG, "ig_probe_random_gather: bad argument");
  int dev = 0, sms = 0;
  int rc = ig_cuda_check((int)cudaGetDevice(&dev), "cudaGetDevice");
  if (!rc) rc = ig_cuda_check((int)cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "SM count");
  if (rc) return rc;
  const int blocks = sms * 8;
  const long long threads = (long long)blocks * kThreads;
  const long long per_thread = ((gathers + threads - 1) / threads + 7) / 8 * 8;
  float *table = nullptr, *sink = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  rc = ig_cuda_check((int)cudaMalloc(&table, (size_t)table_elems * sizeof(float)), "probe table");
  if (!rc) rc = ig_cuda_check((int)cudaMalloc(&sink, (size_t)threads * sizeof(float)), "probe sink");
  if (!rc) rc = ig_cuda_check((int)cudaEventCreate(&e0), "event");
  if (!rc) rc = ig_cuda_check((int)cudaEventCreate(&e1), "event");
  float best = -1.f;
  if (!rc) {
    fill_table<<<sms * 4, kThreads>>>(table, table_elems);
    gather_probe<<<blocks, kThreads>>>(table, table_elems, per_thread, 1, sink);  // warm-up
    ig_count_launches(2);
    for (int r = 0; r < reps && !rc; r++) {
      cudaEventRecord(e0);
      gather_probe<<<blocks, kThreads>>>(table, table_elems, per_thread, 2 + r, sink);
      cudaEventRecord(e1);
      ig_count_launches(1);
      rc = ig_cuda_check((int)cudaEventSynchronize(e1), "probe");
      float ms = 0.f;
      if (!rc) rc = ig_cuda_check((int)cudaEventElapsedTime(&ms, e0, e1), "probe time");
      if (!rc && (best < 0.f || ms < best)) best = ms;
    }
  }
  if (!rc) rc = ig_cuda_check((int)cudaGetLastError(), "probe launch");
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(table);
  cudaFree(sink);
  if (rc) return rc;
  *gathers_per_s = (double)per_thread * (double)threads / (best * 1e-3);
  return IG_OK;
}
