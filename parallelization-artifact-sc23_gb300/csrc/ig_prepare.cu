// Device-side preparation of a CSR graph: the input contract of the suite's
// programs (symmetric, no self loops, no duplicate edges, sorted adjacency;
// include/ECLgraph.h describes the format, and the triangle-counting driver
// refuses unsorted lists, include/tc_vertex_cuda.h:157-165), plus the
// (degree, id) relabelling the triangle-counting benchmark runs on.  The
// reference prepares its inputs offline; here a graph already on the device
// (for example one uploaded from an edge list) is prepared there.
//
//   1. edges as 64-bit keys src << 32 | dst (and dst << 32 | src when
//      symmetrising); a self loop becomes a key that sorts last
//   2. radix sort of (key, weight) pairs, then reduce by key keeping the
//      smallest weight: merges duplicates, leaves each list sorted
//   3. optional relabelling: vertices sorted by the key degree << 32 | id, the
//      edges renamed and sorted again
//   4. nindex by an exclusive sum of the per-vertex counts
//
// The sorts, reductions and scans are CUB's device primitives (a plain
// library sort, as cuBLAS is for a plain GEMM); none of the six algorithms
// uses this file.
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_reduce.cuh>
#include <cub/device/device_scan.cuh>
#include <cuda/functional>

#include <algorithm>
#include <utility>
#include <vector>

#include "ig_device.cuh"

namespace {

constexpr int kThreads = 256;
constexpr unsigned long long kDropKey = ~0ull;  // self loops sort last and are cut

// row_start[nindex[v]] = v for every vertex with edges (max-scanned later
// into the source vertex of every edge)
__global__ void prep_mark_rows(const int* __restrict__ nindex, int n, int* row_of) {
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
    const int b = __ldg(&nindex[v]), e = __ldg(&nindex[v + 1]);
    if (b < e) row_of[b] = v;
  }
}

__global__ void prep_edges(const int* __restrict__ nlist, const int* __restrict__ eweight, const int* row_of,
                           long long edges, bool symmetrize, unsigned long long* keys, int* weights) {
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < edges;
       k += (long long)gridDim.x * blockDim.x) {
    const unsigned u = (unsigned)row_of[k], v = (unsigned)__ldg(&nlist[k]);
    const int w = eweight ? __ldg(&eweight[k]) : 0;
    const bool loop = u == v;
    keys[k] = loop ? kDropKey : ((unsigned long long)u << 32 | v);
    weights[k] = w;
    if (symmetrize) {
      keys[edges + k] = loop ? kDropKey : ((unsigned long long)v << 32 | u);
      weights[edges + k] = w;
    }
  }
}

__global__ void prep_count(const unsigned long long* keys, long long m, int* count) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (long long)gridDim.x * blockDim.x)
    atomicAdd(&count[keys[i] >> 32], 1);
}

__global__ void prep_order_keys(const int* count, int n, unsigned long long* keys) {
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x)
    keys[v] = (unsigned long long)(unsigned)count[v] << 32 | (unsigned)v;
}

__global__ void prep_rank(const unsigned long long* sorted, int n, int* rank) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    rank[(unsigned)sorted[i]] = i;
}

__global__ void prep_rename(unsigned long long* keys, long long m, const int* rank) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (long long)gridDim.x * blockDim.x) {
    const unsigned long long k = keys[i];
    keys[i] = (unsigned long long)(unsigned)rank[k >> 32] << 32 | (unsigned)rank[(unsigned)k];
  }
}

__global__ void prep_split(const unsigned long long* keys, long long m, int* nlist) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (long long)gridDim.x * blockDim.x)
    nlist[i] = (int)(unsigned)keys[i];
}

int bits_for(long long n) {
  int b = 1;
  while ((1ll << b) < n) b++;
  return b;
}

// Owns the call's temporary device memory.
struct Temp {
  std::vector<void*> ptrs;
  ~Temp() {
    for (void* p : ptrs) cudaFree(p);
  }
  template <class T>
  int get(T** p, size_t count) {
    void* q = nullptr;
    const int rc = ig_cuda_check((int)cudaMalloc(&q, std::max<size_t>(1, count) * sizeof(T)), "prepare buffer");
    if (rc) return rc;
    ptrs.push_back(q);
    *p = (T*)q;
    return IG_OK;
  }
};

}  // namespace

extern "C" int ig_csr_prepare(const ig_csr* d_in, int flags, ig_csr* d_out) {
  if (!d_in || !d_out || d_in->nodes < 1 || d_in->edges < 0 || !d_in->nindex || (d_in->edges > 0 && !d_in->nlist) ||
      (flags & ~(IG_PREP_SYMMETRIZE | IG_PREP_DEGREE_ORDER)))
    return ig_fail(IG_ERR_INVALID_ARG, "ig_csr_prepare: bad argument");
  const int n = d_in->nodes;
  const bool sym = (flags & IG_PREP_SYMMETRIZE) != 0;
  const long long e_in = d_in->edges;
  const long long m = sym ? 2 * e_in : e_in;
  const bool weighted = d_in->eweight != nullptr;
  cudaStream_t st = 0;
  int sms = 0, dev = 0;
  int rc = ig_cuda_check((int)cudaGetDevice(&dev), "cudaGetDevice");
  if (!rc) rc = ig_cuda_check((int)cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "SM count");
  if (rc) return rc;
  const int grid = sms * 8;
  Temp t;
  unsigned long long *ka, *kb;
  int *wa, *wb, *row_of, *count, *d_runs;
  if ((rc = t.get(&ka, m)) || (rc = t.get(&kb, m)) || (rc = t.get(&wa, m)) || (rc = t.get(&wb, m)) ||
      (rc = t.get(&row_of, e_in)) || (rc = t.get(&count, (size_t)n + 1)) || (rc = t.get(&d_runs, 1)))
    return rc;
  void* tmp = nullptr;
  size_t tmp_bytes = 0;
  auto temp = [&](size_t need) -> int {  // grow-only CUB temporary storage
    if (need <= tmp_bytes) return IG_OK;
    void* q = nullptr;
    const int r = ig_cuda_check((int)cudaMalloc(&q, need), "prepare temporary");
    if (r) return r;
    t.ptrs.push_back(q);
    tmp = q;
    tmp_bytes = need;
    return IG_OK;
  };
  long long unique = 0;
  if (e_in > 0) {
    // 1. edge keys (source of each edge by a max-scan of the row starts)
    if ((rc = ig_cuda_check((int)cudaMemsetAsync(row_of, 0, (size_t)e_in * sizeof(int), st), "memset"))) return rc;
    prep_mark_rows<<<grid, kThreads, 0, st>>>(d_in->nindex, n, row_of);
    size_t need = 0;
    if ((rc = ig_cuda_check((int)cub::DeviceScan::InclusiveScan(nullptr, need, row_of, row_of, cuda::maximum<int>{}, e_in, st), "CUB"))) return rc;
    if ((rc = temp(need))) return rc;
    need = tmp_bytes;
    if ((rc = ig_cuda_check((int)cub::DeviceScan::InclusiveScan(tmp, need, row_of, row_of, cuda::maximum<int>{}, e_in, st), "CUB"))) return rc;
    prep_edges<<<grid, kThreads, 0, st>>>(d_in->nlist, d_in->eweight, row_of, e_in, sym, ka, wa);
    // 2. sort, then merge duplicates keeping the smallest weight
    need = 0;
    if ((rc = ig_cuda_check((int)cub::DeviceRadixSort::SortPairs(nullptr, need, ka, kb, wa, wb, m, 0, 64, st), "CUB"))) return rc;
    if ((rc = temp(need))) return rc;
    need = tmp_bytes;
    if ((rc = ig_cuda_check((int)cub::DeviceRadixSort::SortPairs(tmp, need, ka, kb, wa, wb, m, 0, 64, st), "CUB"))) return rc;
    need = 0;
    if ((rc = ig_cuda_check((int)cub::DeviceReduce::ReduceByKey(nullptr, need, kb, ka, wb, wa, d_runs, cuda::minimum<int>{}, m, st), "CUB"))) return rc;
    if ((rc = temp(need))) return rc;
    need = tmp_bytes;
    if ((rc = ig_cuda_check((int)cub::DeviceReduce::ReduceByKey(tmp, need, kb, ka, wb, wa, d_runs, cuda::minimum<int>{}, m, st), "CUB"))) return rc;
    int runs = 0;
    unsigned long long last = 0;
    if ((rc = ig_cuda_check((int)cudaMemcpy(&runs, d_runs, sizeof(int), cudaMemcpyDeviceToHost), "read runs")))
      return rc;
    if (runs > 0 &&
        (rc = ig_cuda_check((int)cudaMemcpy(&last, ka + runs - 1, sizeof(last), cudaMemcpyDeviceToHost), "read key")))
      return rc;
    unique = runs - ((runs > 0 && last == kDropKey) ? 1 : 0);  // the self loops' run, if any
  }
  if (unique > 0x7fffffffLL) return ig_fail(IG_ERR_INVALID_ARG, "ig_csr_prepare: more than 2^31-1 edges");
  // per-vertex counts of the prepared edges (ka[0 .. unique) sorted by source)
  if ((rc = ig_cuda_check((int)cudaMemsetAsync(count, 0, ((size_t)n + 1) * sizeof(int), st), "memset"))) return rc;
  if (unique > 0) prep_count<<<grid, kThreads, 0, st>>>(ka, unique, count);
  if (flags & IG_PREP_DEGREE_ORDER) {
    // 3. vertices in (degree, id) order; edges renamed and sorted again
    unsigned long long *oa, *ob;
    int* rank;
    if ((rc = t.get(&oa, n)) || (rc = t.get(&ob, n)) || (rc = t.get(&rank, n))) return rc;
    prep_order_keys<<<grid, kThreads, 0, st>>>(count, n, oa);
    size_t need = 0;
    if ((rc = ig_cuda_check((int)cub::DeviceRadixSort::SortKeys(nullptr, need, oa, ob, n, 0, 64, st), "CUB"))) return rc;
    if ((rc = temp(need))) return rc;
    need = tmp_bytes;
    if ((rc = ig_cuda_check((int)cub::DeviceRadixSort::SortKeys(tmp, need, oa, ob, n, 0, 64, st), "CUB"))) return rc;
    prep_rank<<<grid, kThreads, 0, st>>>(ob, n, rank);
    if (unique > 0) {
      prep_rename<<<grid, kThreads, 0, st>>>(ka, unique, rank);
      const int vb = bits_for(n);
      need = 0;
      if ((rc = ig_cuda_check((int)cub::DeviceRadixSort::SortPairs(nullptr, need, ka, kb, wa, wb, unique, 0, 32 + vb, st), "CUB"))) return rc;
      if ((rc = temp(need))) return rc;
      need = tmp_bytes;
      if ((rc = ig_cuda_check((int)cub::DeviceRadixSort::SortPairs(tmp, need, ka, kb, wa, wb, unique, 0, 32 + vb, st), "CUB"))) return rc;
      std::swap(ka, kb);
      std::swap(wa, wb);
    }
    if ((rc = ig_cuda_check((int)cudaMemsetAsync(count, 0, ((size_t)n + 1) * sizeof(int), st), "memset"))) return rc;
    if (unique > 0) prep_count<<<grid, kThreads, 0, st>>>(ka, unique, count);
  }
  // 4. output arrays
  ig_csr out{n, (int)unique, nullptr, nullptr, nullptr};
  rc = ig_cuda_check((int)cudaMalloc(&out.nindex, ((size_t)n + 1) * sizeof(int)), "output nindex");
  if (!rc) rc = ig_cuda_check((int)cudaMalloc(&out.nlist, std::max<size_t>(1, (size_t)unique) * sizeof(int)),
                              "output nlist");
  if (!rc && weighted)
    rc = ig_cuda_check((int)cudaMalloc(&out.eweight, std::max<size_t>(1, (size_t)unique) * sizeof(int)),
                       "output eweight");
  if (!rc) {
    size_t need = 0;
    if ((rc = ig_cuda_check((int)cub::DeviceScan::ExclusiveSum(nullptr, need, count, out.nindex, n + 1, st), "CUB"))) return rc;
    rc = temp(need);
    if (!rc) {
      need = tmp_bytes;
      if ((rc = ig_cuda_check((int)cub::DeviceScan::ExclusiveSum(tmp, need, count, out.nindex, n + 1, st), "CUB"))) return rc;
    }
  }
  if (!rc && unique > 0) {
    prep_split<<<grid, kThreads, 0, st>>>(ka, unique, out.nlist);
    if (weighted)
      rc = ig_cuda_check((int)cudaMemcpyAsync(out.eweight, wa, (size_t)unique * sizeof(int),
                                              cudaMemcpyDeviceToDevice, st),
                         "copy weights");
  }
  ig_count_launches(6);
  if (!rc) rc = ig_cuda_check((int)cudaGetLastError(), "prepare launch");
  if (!rc) rc = ig_cuda_check((int)cudaStreamSynchronize(st), "prepare");
  if (rc) {
    cudaFree(out.nindex);
    cudaFree(out.nlist);
    cudaFree(out.eweight);
    return rc;
  }
  *d_out = out;
  return IG_OK;
}
