// Drop-in variant for include/sssp_edge_cuda.h (GPUsssp_edge, :60).
typedef int basic_t;
#include <cuda/atomic>
#include "sssp_edge_cuda.h"
#include "shim_common.h"

static double GPUsssp_edge(const int src, const ECLgraph& g, basic_t* const dist, const int* const sp) {
  const ig_csr d = ig_shim_csr(g);
  double seconds = 0;
  ig_shim_check(ig_sssp_edge(src, &d, dist, sp, &seconds), "GPUsssp_edge");
  return seconds;
}
