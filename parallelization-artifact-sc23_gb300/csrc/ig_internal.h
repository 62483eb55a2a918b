// Internal host-side declarations shared by the library's translation units.
#pragma once

#include <cstddef>
#include <cstdint>
#include <mutex>

#include "../../include/indigo_gb300.h"
#include "ig_options.h"

#ifdef __CUDACC__
#include <cuda_runtime.h>
#else
struct CUstream_st;
typedef CUstream_st* cudaStream_t;
struct CUevent_st;
typedef CUevent_st* cudaEvent_t;
#endif

// Records a formatted message for ig_last_error() and returns `status`.
int ig_fail(int status, const char* fmt, ...);
void ig_clear_error();

// ---------------------------------------------------------------------------
// Device control block: one per execution context, zeroed before every run.
// The kernels record their first error in `err` and their counters here.
// ---------------------------------------------------------------------------
struct IgSync {
  unsigned int arrive;
  unsigned int gen;
};

// Counters that every warp of a persistent kernel updates with atomics
// (queue sizes, work grabs, round minima) sit 256 bytes apart: packed into one
// line they all queue in one L2 slice, together with the grid barrier's flag
// that every block polls.
constexpr int kCtlHot = 32;     // hot counters
constexpr int kCtlSpread = 64;  // ints from one hot counter to the next

struct IgCtl {
  int sticky_err;              // first error of any run since last reported (not reset per run)
  int pad_;
  int err;                     // first ig_status raised on the device
  int iterations;              // levels / rounds / iterations executed
  long long work;              // algorithm-specific work counter
  double residual;             // PageRank residual of the last iteration
  int i32[32];                 // per-algorithm integer counters (set a few times per call)
  unsigned long long u64[16];  // per-algorithm 64-bit counters
  double f64[8];
  alignas(256) IgSync sync;    // grid barrier state, on a line of its own
  alignas(256) int hot[kCtlHot * kCtlSpread];  // hot counter k at hot[k * kCtlSpread]
};
// The part of the control block the host reads back after a run.
constexpr size_t kCtlHostBytes = offsetof(IgCtl, sync);

// Scratch slots: each algorithm names the buffers it needs; the pool grows a
// slot on demand and keeps it for later calls.
enum IgSlot {
  IG_SLOT_CTL = 0,
  IG_SLOT_OUT,      // drop-in result buffer
  IG_SLOT_Q0,
  IG_SLOT_Q1,
  IG_SLOT_Q2,
  IG_SLOT_Q3,
  IG_SLOT_V0,       // per-vertex int arrays
  IG_SLOT_V1,
  IG_SLOT_V2,
  IG_SLOT_F0,       // per-vertex float arrays
  IG_SLOT_F1,
  IG_SLOT_E0,       // per-edge int arrays
  IG_SLOT_BLK,      // per-block partials
  IG_SLOT_G0,       // graph copies (PR upload)
  IG_SLOT_G1,
  IG_SLOT_G2,
  IG_SLOT_COUNT
};

struct IgScratch {
  void* ptr[IG_SLOT_COUNT] = {};
  size_t cap[IG_SLOT_COUNT] = {};
  int device = -1;
  // bumped whenever a slot is reallocated: launches captured into a CUDA
  // graph hold slot addresses and must be captured again after a change
  unsigned long long generation = 0;
};

int ig_scratch_get(IgScratch* s, int slot, size_t bytes, void** out);
void ig_scratch_release(IgScratch* s);

// Everything a kernel launcher needs.
struct IgExec {
  cudaStream_t stream = nullptr;
  IgScratch* scratch = nullptr;
  IgCtl* d_ctl = nullptr;      // device control block
  IgCtl* h_ctl = nullptr;      // pinned host mirror
  int device = 0;
  int sms = 0;
  unsigned long long timeout_ns = 0;
  const IgOptions* opts = nullptr;  // per-handle options (batch autotuning); null = process-wide
};

// Options a launcher uses for this execution context.
inline const IgOptions& ig_exec_options(const IgExec* ex) { return ex->opts ? *ex->opts : ig_options(); }
// Reads option `name` of `o` (same names as ig_get_option).
int ig_options_get(const IgOptions& o, const char* name, long long* value);
int ig_options_set(IgOptions& o, const char* name, long long value);

// Per-device state used by the drop-in entry points.
struct IgDevice {
  int id = -1;
  int sms = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  IgScratch scratch;
  IgCtl* h_ctl = nullptr;
  std::mutex mu;
};

// Returns the state of the current device (creating it on first use).
int ig_current_device(IgDevice** out);
// Builds an execution context on the device's stream and scratch.
int ig_exec_init(IgExec* ex, cudaStream_t stream, IgScratch* scratch, IgCtl* h_ctl,
                 int device, int sms);
// Zeroes the control block on the exec's stream, first folding the previous
// run's error into sticky_err (so asynchronous callers cannot lose it).
int ig_exec_reset(IgExec* ex);
// Synchronises the stream and copies the control block back; returns the
// device-side status.
int ig_exec_finish(IgExec* ex);
// Turns a device-side status word into the call's status and message.
int ig_device_status(int err);
unsigned long long ig_timeout_ns();

// Cooperative launch of a persistent kernel with all blocks co-resident.
// `blocks_per_sm_cap` limits the grid; the block count used is returned.
int ig_launch_coop(IgExec* ex, const void* kernel, int threads, size_t smem,
                   int blocks_per_sm_cap, void** args, int* blocks_out);
int ig_cuda_check(int cuda_err, const char* what);
// Adds n to the process-wide count of kernels this library launched.
void ig_count_launches(int n);

// ---------------------------------------------------------------------------
// Algorithm launchers (enqueue on ex->stream; errors surface in ig_exec_finish)
// ---------------------------------------------------------------------------
int igk_bfs(IgExec* ex, const ig_csr* dg, int src, int* d_dist);
int igk_bfs_keyed(IgExec* ex, const ig_csr* dg, const unsigned long long* d_src_key, int* d_dist, int max_level);
int igk_bfs_launch_prealloc(IgExec* ex, const ig_csr* dg, int src, int* d_dist, int* qa, int* qb, int* hubs);
int igk_sssp(IgExec* ex, const ig_csr* dg, int src, int* d_dist);
// sample: link the first neighbours and skip the largest component's vertices
// (skewed single graphs); off for unions of many small graphs
int igk_cc(IgExec* ex, const ig_csr* dg, int* d_label, bool sample = true);
int igk_mis(IgExec* ex, const ig_csr* dg, int* d_status, unsigned int* d_prio);
int igk_pr(IgExec* ex, const ig_csr* dg, const int* d_degree, float* d_scores,
           float epsilon, int max_iter);
int igk_tc(IgExec* ex, int nodes, int edges, const int* d_nindex, const int* d_nlist,
           unsigned long long* d_count);
// Batched (disjoint union) forms
int igk_bfs_multi(IgExec* ex, const ig_csr* dg, const int* d_sources, int nsources, int* d_dist);
int igk_cc_localize(IgExec* ex, int* d_label, const int* d_graph_vptr, int graphs);
int igk_tc_batched(IgExec* ex, int nodes, int edges, const int* d_nindex, const int* d_nlist,
                   const int* d_graph_vptr, int graphs, unsigned long long* d_counts);
int igk_pr_batched(IgExec* ex, const ig_csr* dg, const int* d_graph_vptr, int graphs, float* d_scores,
                   float epsilon, int max_iter, int* d_iters);
// Device-wide exclusive scan of n ints (n+1 outputs, out[n] = total) into out.
int igk_exclusive_scan(IgExec* ex, const int* in, int* out, int n, long long* total_host);
