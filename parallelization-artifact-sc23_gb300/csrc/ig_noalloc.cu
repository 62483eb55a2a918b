// BFS for callers that cannot allocate device memory.
//
// Some callers of a graph library cannot call cudaMalloc at the point where
// they need a traversal: code running inside a stream-ordered region that
// must not synchronise with the allocator, processes whose device memory is
// capped or pre-partitioned by a host framework, or plugins that may only use
// the buffers their host hands them.  ig_bfs_vertex_noalloc serves them: the
// caller passes the device graph and the device output, and every scratch
// buffer the BFS kernel needs (two frontier queues, the hub list and the
// control block) lives in one file-scope __device__ array of fixed size,
// g_bfs_scratch below.  That array is part of the library's device image, so
// every GPU that loads the library holds it (12 MiB plus the control block,
// about 9 KB) until exit.
//
// Limits and rules of use:
//   * graphs of at most kNoallocMaxNodes (1,048,576) vertices; larger ones are
//     rejected with IG_ERR_INVALID_ARG before any device work;
//   * the array is shared by every call on a device and keeps the previous
//     call's contents; the control block is cleared at the start of each call
//     and the queues need no clearing (the kernel writes before it reads);
//   * calls whose GPU work overlaps (two host threads, two streams) race on the
//     array: the caller must order them;
//   * the first call on each device looks up the array's device address with
//     cudaGetSymbolAddress (once per device, that device current).  The
//     address is kept for the life of the process: after cudaDeviceReset the
//     library's device image is loaded again and the kept address is no
//     longer valid, so a process that resets a device must not call this
//     entry point on it afterwards;
//   * every call copies the device's status word back and synchronizes
//     `stream` before it returns, so no call may be made on a stream that is
//     being captured.
#include "ig_device.cuh"

namespace {

constexpr int kNoallocMaxNodes = 1 << 20;
constexpr size_t kCtlBytes = 256 * ((sizeof(IgCtl) + 255) / 256);
constexpr size_t kScratchBytes = kCtlBytes + 3ull * kNoallocMaxNodes * sizeof(int);

static __device__ __align__(256) unsigned char g_bfs_scratch[kScratchBytes];

std::mutex g_noalloc_mu;
void* g_noalloc_addr[64];  // device address of g_bfs_scratch, per device

}  // namespace

extern "C" int ig_bfs_vertex_noalloc(int src, const ig_csr* d_g, int* d_dist, void* stream) {
  if (!d_g || !d_dist) return ig_fail(IG_ERR_INVALID_ARG, "ig_bfs_vertex_noalloc: null argument");
  if (d_g->nodes < 1 || d_g->edges < 0 || !d_g->nindex || (d_g->edges > 0 && !d_g->nlist))
    return ig_fail(IG_ERR_INVALID_ARG, "ig_bfs_vertex_noalloc: bad graph");
  if (d_g->nodes > kNoallocMaxNodes)
    return ig_fail(IG_ERR_INVALID_ARG,
                   "ig_bfs_vertex_noalloc: %d vertices exceed the static scratch limit of %d vertices; "
                   "use ig_bfs_vertex",
                   d_g->nodes, kNoallocMaxNodes);
  if (src < 0 || src >= d_g->nodes) return ig_fail(IG_ERR_INVALID_ARG, "source %d out of range", src);

  int dev = 0;
  int rc = ig_cuda_check((int)cudaGetDevice(&dev), "cudaGetDevice");
  if (rc) return rc;
  if (dev < 0 || dev >= 64) return ig_fail(IG_ERR_NO_DEVICE, "device id %d out of range", dev);
  void* base = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_addr[dev]) {
      void* p = nullptr;
      rc = ig_cuda_check((int)cudaGetSymbolAddress(&p, g_bfs_scratch), "cudaGetSymbolAddress(g_bfs_scratch)");
      if (rc) return rc;
      g_noalloc_addr[dev] = p;
    }
    base = g_noalloc_addr[dev];
  }
  int sms = 0;
  rc = ig_cuda_check((int)cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "SM count");
  if (rc) return rc;

  IgExec ex;
  ex.stream = (cudaStream_t)stream;
  ex.scratch = nullptr;
  ex.d_ctl = (IgCtl*)base;
  ex.h_ctl = nullptr;
  ex.device = dev;
  ex.sms = sms;
  ex.timeout_ns = ig_timeout_ns();
  int* qa = (int*)((unsigned char*)base + kCtlBytes);
  int* qb = qa + kNoallocMaxNodes;
  int* hubs = qb + kNoallocMaxNodes;

  if ((rc = ig_exec_reset(&ex))) return rc;  // clears the control block (a kernel, no allocation)
  if ((rc = igk_bfs_launch_prealloc(&ex, d_g, src, d_dist, qa, qb, hubs))) return rc;
  int err = 0;
  rc = ig_cuda_check((int)cudaMemcpyAsync(&err, &ex.d_ctl->err, sizeof(int), cudaMemcpyDeviceToHost, ex.stream),
                     "status copy");
  if (!rc) rc = ig_cuda_check((int)cudaStreamSynchronize(ex.stream), "stream synchronize");
  if (rc) return rc;
  return ig_device_status(err);
}
