// Batched form: thousands of graphs packed as one disjoint union (global
// vertex ids, graph_vptr[g] = first vertex of graph g) and processed by one
// launch sequence per algorithm, captured once into a CUDA graph and replayed.
//
// The union needs no per-graph loop: BFS from every graph's source is one
// multi-source BFS (levels never cross graphs), CC on the union gives each
// graph's min-id labels after subtracting the graph's first vertex, TC adds a
// triangle to the graph of its middle vertex, and PageRank keeps a base score,
// a residual and a stop iteration per graph.  Results equal the plain
// single-graph calls (bit for bit for BFS, CC and TC).
#include <cuda_runtime.h>

#include <cstring>
#include <memory>

#include "ig_internal.h"

namespace {

enum BatchAlgo { kBfs = 0, kCc = 1, kTc = 2, kPr = 3, kAlgos = 4 };

struct Captured {
  cudaGraphExec_t exec = nullptr;
  long long kernels = 0;  // kernels launched by one replay
  const void* key[3] = {nullptr, nullptr, nullptr};
  float f = 0.f;
  int i = 0;
};

}  // namespace

struct ig_batch {
  ig_csr g;
  const int* vptr = nullptr;  // device int[graphs + 1]
  int graphs = 0;
  int device = 0, sms = 0;
  cudaStream_t stream = nullptr;
  IgScratch scratch;
  IgCtl* h_ctl = nullptr;
  IgExec ex;
  Captured cap[kAlgos];
  int warm[kAlgos] = {0, 0, 0, 0};  // direct runs so far (scratch is sized by the first)
  bool use_graphs = true;
  bool pending = false;
  int last_rc = IG_OK;
};

static int batch_cuda(int e, const char* what) { return ig_cuda_check(e, what); }

extern "C" int ig_batch_create(const ig_csr* d_union, const int* d_graph_vptr, int graphs, ig_batch** out) {
  if (!d_union || !d_graph_vptr || !out || graphs < 1 || d_union->nodes < graphs || d_union->edges < 0 ||
      !d_union->nindex || (d_union->edges > 0 && !d_union->nlist))
    return ig_fail(IG_ERR_INVALID_ARG, "ig_batch_create: bad argument");
  std::unique_ptr<ig_batch> b(new ig_batch());
  b->g = *d_union;
  b->vptr = d_graph_vptr;
  b->graphs = graphs;
  int rc;
  if ((rc = batch_cuda(cudaGetDevice(&b->device), "cudaGetDevice"))) return rc;
  if ((rc = batch_cuda(cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, b->device), "SM count")))
    return rc;
  if ((rc = batch_cuda(cudaStreamCreate(&b->stream), "stream"))) return rc;
  if ((rc = batch_cuda(cudaMallocHost((void**)&b->h_ctl, sizeof(IgCtl)), "pinned control block"))) return rc;
  memset(b->h_ctl, 0, sizeof(IgCtl));
  b->scratch.device = b->device;
  if ((rc = ig_exec_init(&b->ex, b->stream, &b->scratch, b->h_ctl, b->device, b->sms))) return rc;
  *out = b.release();
  return IG_OK;
}

extern "C" int ig_batch_destroy(ig_batch* b) {
  if (!b) return IG_OK;
  cudaStreamSynchronize(b->stream);
  for (auto& c : b->cap)
    if (c.exec) cudaGraphExecDestroy(c.exec);
  ig_scratch_release(&b->scratch);
  cudaFreeHost(b->h_ctl);
  cudaStreamDestroy(b->stream);
  delete b;
  return IG_OK;
}

extern "C" int ig_batch_stream(ig_batch* b, void** stream) {
  if (!b || !stream) return ig_fail(IG_ERR_INVALID_ARG, "null");
  *stream = (void*)b->stream;
  return IG_OK;
}

extern "C" int ig_batch_use_graphs(ig_batch* b, int enable) {
  if (!b) return ig_fail(IG_ERR_INVALID_ARG, "null");
  b->use_graphs = enable != 0;
  return IG_OK;
}

extern "C" int ig_batch_last_run(ig_batch* b, ig_run_info* info) {
  if (!b || !info) return ig_fail(IG_ERR_INVALID_ARG, "null");
  int rc = b->last_rc;
  if (b->pending) {
    rc = ig_exec_finish(&b->ex);
    b->pending = false;
    b->last_rc = rc;
  }
  if (rc == IG_OK && b->h_ctl->sticky_err != 0) rc = b->h_ctl->sticky_err;
  if (b->h_ctl->sticky_err != 0) {
    const int zero = 0;
    int r2 = batch_cuda(cudaMemcpyAsync(&b->ex.d_ctl->sticky_err, &zero, sizeof(int), cudaMemcpyHostToDevice,
                                        b->stream),
                        "clear sticky");
    if (!r2) r2 = batch_cuda(cudaStreamSynchronize(b->stream), "sync");
    if (r2) return r2;
  }
  memset(info, 0, sizeof(*info));
  info->status = rc;
  info->iterations = b->h_ctl->iterations;
  info->residual = b->h_ctl->residual;
  return IG_OK;
}

// Runs `body` directly for the first call of an algorithm (so every scratch
// buffer exists), then captures it once into a CUDA graph keyed by the
// arguments and replays the graph on later calls.
template <class Body>
static int batch_run(ig_batch* b, int algo, const void* k0, const void* k1, float f, int i, Body&& body) {
  if (!b) return ig_fail(IG_ERR_INVALID_ARG, "null batch");
  b->ex.timeout_ns = ig_timeout_ns();
  int rc;
  Captured& c = b->cap[algo];
  const bool same = c.exec && c.key[0] == k0 && c.key[1] == k1 && c.f == f && c.i == i;
  if (b->use_graphs && (same || b->warm[algo] > 0)) {
    if (!same) {
      if (c.exec) {
        cudaGraphExecDestroy(c.exec);
        c.exec = nullptr;
      }
      if ((rc = batch_cuda(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal), "begin capture")))
        return rc;
      long long k0n = 0, k1n = 0;
      ig_kernel_launches(&k0n);
      const int brc = body(&b->ex);
      ig_kernel_launches(&k1n);
      c.kernels = k1n - k0n;
      ig_count_launches((int)-c.kernels);  // captured, not launched: counted at each replay
      cudaGraph_t graph = nullptr;
      rc = batch_cuda(cudaStreamEndCapture(b->stream, &graph), "end capture");
      if (brc) {
        if (graph) cudaGraphDestroy(graph);
        return brc;
      }
      if (rc) return rc;
      rc = batch_cuda(cudaGraphInstantiate(&c.exec, graph, 0), "graph instantiate");
      cudaGraphDestroy(graph);
      if (rc) return rc;
      c.key[0] = k0;
      c.key[1] = k1;
      c.f = f;
      c.i = i;
    }
    rc = batch_cuda(cudaGraphLaunch(c.exec, b->stream), "graph launch");
    if (rc == IG_OK) ig_count_launches((int)c.kernels);
  } else {
    rc = body(&b->ex);
    b->warm[algo]++;
  }
  b->last_rc = rc;
  b->pending = (rc == IG_OK);
  return rc;
}

extern "C" int ig_batch_bfs(ig_batch* b, const int* d_sources, int* d_dist) {
  if (!b || !d_dist) return ig_fail(IG_ERR_INVALID_ARG, "null argument");
  // default sources: local vertex 0 of every graph = graph_vptr[0 .. graphs)
  const int* src = d_sources ? d_sources : b->vptr;
  return batch_run(b, kBfs, d_dist, src, 0.f, 0,
                   [&](IgExec* ex) { return igk_bfs_multi(ex, &b->g, src, b->graphs, d_dist); });
}

extern "C" int ig_batch_cc(ig_batch* b, int* d_label) {
  if (!b || !d_label) return ig_fail(IG_ERR_INVALID_ARG, "null argument");
  return batch_run(b, kCc, d_label, nullptr, 0.f, 0, [&](IgExec* ex) {
    int rc = igk_cc(ex, &b->g, d_label);
    if (rc) return rc;
    return igk_cc_localize(ex, d_label, b->vptr, b->graphs);
  });
}

extern "C" int ig_batch_tc(ig_batch* b, unsigned long long* d_counts) {
  if (!b || !d_counts) return ig_fail(IG_ERR_INVALID_ARG, "null argument");
  return batch_run(b, kTc, d_counts, nullptr, 0.f, 0, [&](IgExec* ex) {
    return igk_tc_batched(ex, b->g.nodes, b->g.edges, b->g.nindex, b->g.nlist, b->vptr, b->graphs, d_counts);
  });
}

extern "C" int ig_batch_pagerank(ig_batch* b, float* d_scores, float epsilon, int max_iter, int* d_iters) {
  if (!b || !d_scores || !d_iters || max_iter < 1) return ig_fail(IG_ERR_INVALID_ARG, "bad PageRank argument");
  return batch_run(b, kPr, d_scores, d_iters, epsilon, max_iter, [&](IgExec* ex) {
    return igk_pr_batched(ex, &b->g, b->vptr, b->graphs, d_scores, epsilon, max_iter, d_iters);
  });
}
