// Drop-in variant for include/mis_vertex_cuda.h (GPUmis_vertex, :54).  The
// set is the reference C++ one (unsigned priority compare); `priority` is
// left untouched, as the reference CUDA variants leave the host array.
typedef int data_type;
#include <cuda/atomic>
#include "mis_vertex_cuda.h"
#include "shim_common.h"

static double GPUmis_vertex(const ECLgraph& g, data_type* const priority, int* const status) {
  (void)priority;
  const ig_csr d = ig_shim_csr(g);
  double seconds = 0;
  ig_shim_check(ig_mis_vertex(&d, nullptr, status, &seconds), "GPUmis_vertex");
  return seconds;
}
