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
#include <vector>

#include "ig_internal.h"

namespace {

enum BatchAlgo { kBfs = 0, kCc = 1, kTc = 2, kPr = 3, kAlgos = 4 };

struct Captured {
  cudaGraphExec_t exec = nullptr;
  long long kernels = 0;  // kernels launched by one replay
  const void* key[3] = {nullptr, nullptr, nullptr};
  unsigned long long generation = 0;  // scratch generation the graph was captured with
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
  IgOptions opts[kAlgos];           // per-algorithm options chosen by ig_batch_autotune
  bool tuned[kAlgos] = {false, false, false, false};
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
  b->ex.opts = b->tuned[algo] ? &b->opts[algo] : nullptr;
  int rc;
  Captured& c = b->cap[algo];
  // a captured graph holds scratch addresses: reuse it only with the same
  // arguments and while no scratch slot has been reallocated since (another
  // algorithm's first run may grow a slot this one uses)
  const bool same = c.exec && c.key[0] == k0 && c.key[1] == k1 && c.f == f && c.i == i &&
                    c.generation == b->scratch.generation;
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
      c.generation = b->scratch.generation;
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

// The launch sequence of each algorithm on the union (shared by the calls
// below and by the autotuner).
static int bfs_body(ig_batch* b, IgExec* ex, const int* src, int* d_dist) {
  return igk_bfs_multi(ex, &b->g, src, b->graphs, d_dist);
}
static int cc_body(ig_batch* b, IgExec* ex, int* d_label) {
  int rc = igk_cc(ex, &b->g, d_label, false);  // many small components: no giant one to skip
  if (rc) return rc;
  return igk_cc_localize(ex, d_label, b->vptr, b->graphs);
}
static int tc_body(ig_batch* b, IgExec* ex, unsigned long long* d_counts) {
  return igk_tc_batched(ex, b->g.nodes, b->g.edges, b->g.nindex, b->g.nlist, b->vptr, b->graphs, d_counts);
}
static int pr_body(ig_batch* b, IgExec* ex, float* d_scores, float epsilon, int max_iter, int* d_iters) {
  return igk_pr_batched(ex, &b->g, b->vptr, b->graphs, d_scores, epsilon, max_iter, d_iters);
}

extern "C" int ig_batch_bfs(ig_batch* b, const int* d_sources, int* d_dist) {
  if (!b || !d_dist) return ig_fail(IG_ERR_INVALID_ARG, "null argument");
  // default sources: local vertex 0 of every graph = graph_vptr[0 .. graphs)
  const int* src = d_sources ? d_sources : b->vptr;
  return batch_run(b, kBfs, d_dist, src, 0.f, 0, [&](IgExec* ex) { return bfs_body(b, ex, src, d_dist); });
}

extern "C" int ig_batch_cc(ig_batch* b, int* d_label) {
  if (!b || !d_label) return ig_fail(IG_ERR_INVALID_ARG, "null argument");
  return batch_run(b, kCc, d_label, nullptr, 0.f, 0, [&](IgExec* ex) { return cc_body(b, ex, d_label); });
}

extern "C" int ig_batch_tc(ig_batch* b, unsigned long long* d_counts) {
  if (!b || !d_counts) return ig_fail(IG_ERR_INVALID_ARG, "null argument");
  return batch_run(b, kTc, d_counts, nullptr, 0.f, 0, [&](IgExec* ex) { return tc_body(b, ex, d_counts); });
}

extern "C" int ig_batch_pagerank(ig_batch* b, float* d_scores, float epsilon, int max_iter, int* d_iters) {
  if (!b || !d_scores || !d_iters || max_iter < 1) return ig_fail(IG_ERR_INVALID_ARG, "bad PageRank argument");
  return batch_run(b, kPr, d_scores, d_iters, epsilon, max_iter,
                   [&](IgExec* ex) { return pr_body(b, ex, d_scores, epsilon, max_iter, d_iters); });
}

// ---------------------------------------------------------------------------
// Autotuning: for each requested algorithm, time a small set of launch
// variants on this batch (direct runs, CUDA events, best of `reps`) and keep
// the fastest for the batch's later calls (its CUDA graph is re-captured).
// Variants differ only in launch shape and work-splitting thresholds, never
// in results.

namespace {

__global__ void batch_pr_init(float* s, const int* __restrict__ vptr, int graphs, int n) {
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
    int lo = 0, hi = graphs - 1;  // graph of v
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (__ldg(&vptr[mid]) <= v) lo = mid;
      else hi = mid - 1;
    }
    s[v] = 1.0f / (float)(__ldg(&vptr[lo + 1]) - __ldg(&vptr[lo]));
  }
}

std::vector<IgOptions> batch_variants(int algo, const IgOptions& base) {
  std::vector<IgOptions> out;
  auto add = [&](int bps, int hub, int pr_hub) {
    IgOptions o = base;
    if (bps >= 0) {
      if (algo == kPr) o.pr_blocks_per_sm = bps;  // PageRank has its own block count
      else o.blocks_per_sm = bps;
    }
    if (hub > 0) o.hub_degree = hub;
    if (pr_hub > 0) o.pr_hub_degree = pr_hub;
    out.push_back(o);
  };
  add(-1, 0, 0);  // the process-wide options first
  // Besides residency and hub thresholds (thread / warp / grid granularity),
  // the style axes: BFS push-pull (direction-optimising) against push only
  // (data-driven worklist levels) and bitmap against distance tests in the
  // bottom-up (pull, topology-driven) levels; CC sampled linking in one pass
  // or one round per neighbour; PageRank medium lists by the warp or by
  // 8-lane sub-warps, with or without the L2 prefetch of the next lists.
  if (algo == kBfs) {
    for (int bps : {4, 8})
      for (int hub : {256, 1024})
        for (int alpha : {14, 0})
          for (int bitmap : {1, 0}) {
            add(bps, hub, 0);
            out.back().bfs_alpha = alpha;
            out.back().bfs_bitmap = bitmap;
          }
  } else if (algo == kCc) {
    for (int hub : {64, 256, 1024, 4096})
      for (int rounds : {0, 1}) {
        add(-1, hub, 0);
        out.back().cc_rounds = rounds;
      }
  } else if (algo == kPr) {
    for (int bps : {3, 4})
      for (int ph : {1024, 4096})
        for (int sub : {0, 1})
          for (int pf : {1, 0}) {
            add(bps, 0, ph);
            out.back().pr_subwarp = sub;
            out.back().pr_prefetch = pf;
          }
  }
  return out;  // TC: its launch shape follows the shared-memory tables; nothing to tune
}

}  // namespace

extern "C" int ig_batch_autotune(ig_batch* b, int algo_mask, int reps, float* best_ms) {
  if (!b || reps < 1 || (algo_mask & ~0xF)) return ig_fail(IG_ERR_INVALID_ARG, "ig_batch_autotune: bad argument");
  int rc = IG_OK;
  const int n = b->g.nodes;
  void *d_out = nullptr, *d_aux = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if ((rc = batch_cuda(cudaMalloc(&d_out, (size_t)n * sizeof(int)), "tuning buffer"))) return rc;
  if ((rc = batch_cuda(cudaMalloc(&d_aux, (size_t)b->graphs * sizeof(unsigned long long)), "tuning buffer"))) {
    cudaFree(d_out);
    return rc;
  }
  if (!rc) rc = batch_cuda(cudaEventCreate(&e0), "event");
  if (!rc) rc = batch_cuda(cudaEventCreate(&e1), "event");
  b->ex.timeout_ns = ig_timeout_ns();
  for (int algo = 0; algo < kAlgos && !rc; algo++) {
    if (best_ms) best_ms[algo] = -1.f;
    if (!(algo_mask & (1 << algo))) continue;
    const std::vector<IgOptions> vars = batch_variants(algo, ig_options());
    float best = -1.f;
    size_t best_i = 0;
    for (size_t vi = 0; vi < vars.size() && !rc; vi++) {
      b->ex.opts = &vars[vi];
      float vbest = -1.f;
      for (int r = 0; r <= reps && !rc; r++) {  // run 0 warms up (sizes scratch)
        if (algo == kPr) {
          batch_pr_init<<<b->sms * 4, 256, 0, b->stream>>>((float*)d_out, b->vptr, b->graphs, n);
          ig_count_launches(1);
        }
        rc = batch_cuda(cudaEventRecord(e0, b->stream), "event");
        if (!rc) {
          if (algo == kBfs) rc = bfs_body(b, &b->ex, b->vptr, (int*)d_out);
          else if (algo == kCc) rc = cc_body(b, &b->ex, (int*)d_out);
          else if (algo == kTc) rc = tc_body(b, &b->ex, (unsigned long long*)d_aux);
          else rc = pr_body(b, &b->ex, (float*)d_out, 1e-6f, 100, (int*)d_aux);
        }
        if (!rc) rc = batch_cuda(cudaEventRecord(e1, b->stream), "event");
        if (!rc) rc = ig_exec_finish(&b->ex);
        float ms = 0.f;
        if (!rc) rc = batch_cuda(cudaEventElapsedTime(&ms, e0, e1), "event time");
        if (!rc && r > 0 && (vbest < 0.f || ms < vbest)) vbest = ms;
      }
      if (!rc && (best < 0.f || vbest < best)) {
        best = vbest;
        best_i = vi;
      }
    }
    if (rc) break;
    b->opts[algo] = vars[best_i];
    b->tuned[algo] = true;
    b->warm[algo] = 1;  // scratch is sized; the next call is captured with the chosen options
    if (b->cap[algo].exec) {
      cudaGraphExecDestroy(b->cap[algo].exec);
      b->cap[algo].exec = nullptr;
    }
    if (best_ms) best_ms[algo] = best;
  }
  b->ex.opts = nullptr;
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(d_out);
  cudaFree(d_aux);
  b->pending = false;
  b->last_rc = rc;
  return rc;
}

extern "C" int ig_batch_set_option(ig_batch* b, int algo, const char* name, long long value) {
  if (!b || algo < 0 || algo >= kAlgos) return ig_fail(IG_ERR_INVALID_ARG, "ig_batch_set_option: bad argument");
  IgOptions o = b->tuned[algo] ? b->opts[algo] : ig_options();
  const int rc = ig_options_set(o, name, value);
  if (rc) return rc;
  b->opts[algo] = o;
  b->tuned[algo] = true;
  if (b->cap[algo].exec) {  // captured with the old options: capture again
    cudaGraphExecDestroy(b->cap[algo].exec);
    b->cap[algo].exec = nullptr;
  }
  return IG_OK;
}

extern "C" int ig_batch_get_option(ig_batch* b, int algo, const char* name, long long* value) {
  if (!b || algo < 0 || algo >= kAlgos) return ig_fail(IG_ERR_INVALID_ARG, "ig_batch_get_option: bad argument");
  return ig_options_get(b->tuned[algo] ? b->opts[algo] : ig_options(), name, value);
}
