// Drop-in variant for include/mis_edge_cuda.h (GPUmis_edge, :54; sp on the device).
typedef int data_type;
#include <cuda/atomic>
#include "mis_edge_cuda.h"
#include "shim_common.h"

static double GPUmis_edge(const ECLgraph& g, const int* const sp, data_type* const priority, int* const status) {
  (void)priority;
  const ig_csr d = ig_shim_csr(g);
  double seconds = 0;
  ig_shim_check(ig_mis_edge(&d, sp, nullptr, status, &seconds), "GPUmis_edge");
  return seconds;
}
