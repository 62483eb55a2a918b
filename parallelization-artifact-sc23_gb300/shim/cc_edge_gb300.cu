// Drop-in variant for include/cc_edge_cuda.h (GPUcc_edge, :57).
typedef int basic_t;
#include <cuda/atomic>
#include "cc_edge_cuda.h"
#include "shim_common.h"

static double GPUcc_edge(const ECLgraph& g, basic_t* const label, const int* const sp) {
  const ig_csr d = ig_shim_csr(g);
  double seconds = 0;
  ig_shim_check(ig_cc_edge(&d, label, sp, &seconds), "GPUcc_edge");
  return seconds;
}
