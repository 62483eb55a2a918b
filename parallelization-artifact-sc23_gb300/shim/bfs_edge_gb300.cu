// Drop-in variant for include/bfs_edge_cuda.h (GPUbfs_edge, :61; sp = host COO sources).
typedef int basic_t;
#include "bfs_edge_cuda.h"
#include "shim_common.h"

static double GPUbfs_edge(const int src, const ECLgraph& g, basic_t* const dist, const int* const sp) {
  const ig_csr d = ig_shim_csr(g);
  double seconds = 0;
  ig_shim_check(ig_bfs_edge(src, &d, dist, sp, &seconds), "GPUbfs_edge");
  return seconds;
}
