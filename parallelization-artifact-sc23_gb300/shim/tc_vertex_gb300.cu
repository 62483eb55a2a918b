// Drop-in variant for include/tc_vertex_cuda.h (GPUtc_vertex, :42).  basic_t
// is 64-bit here so large counts do not overflow; the driver's verifier
// h_triCounting (:98-117) is compiled with the same type.
typedef long long basic_t;
#include "tc_vertex_cuda.h"
#include "shim_common.h"

static double GPUtc_vertex(basic_t& count, const int nodes, const int* const nindex, const int* const nlist) {
  long long c = 0;
  double seconds = 0;
  ig_shim_check(ig_tc_vertex(&c, nodes, nindex, nlist, &seconds), "GPUtc_vertex");
  count = c;
  return seconds;
}
