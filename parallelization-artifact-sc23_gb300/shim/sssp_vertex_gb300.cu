// Drop-in variant for include/sssp_vertex_cuda.h (GPUsssp_vertex, :60).
typedef int basic_t;
#include <cuda/atomic>
#include "sssp_vertex_cuda.h"
#include "shim_common.h"

static double GPUsssp_vertex(const int src, const ECLgraph& g, basic_t* const dist) {
  const ig_csr d = ig_shim_csr(g);
  double seconds = 0;
  ig_shim_check(ig_sssp_vertex(src, &d, dist, &seconds), "GPUsssp_vertex");
  return seconds;
}
