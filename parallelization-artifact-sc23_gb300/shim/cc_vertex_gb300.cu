// Drop-in variant for include/cc_vertex_cuda.h (GPUcc_vertex, :57).
typedef int basic_t;
#include <cuda/atomic>
#include "cc_vertex_cuda.h"
#include "shim_common.h"

static double GPUcc_vertex(const ECLgraph& g, basic_t* const label) {
  const ig_csr d = ig_shim_csr(g);
  double seconds = 0;
  ig_shim_check(ig_cc_vertex(&d, label, &seconds), "GPUcc_vertex");
  return seconds;
}
