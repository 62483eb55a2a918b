// Drop-in variant for include/tc_edge_cuda.h (GPUtc_edge, :42; all arrays on the device).
typedef long long basic_t;
#include "tc_edge_cuda.h"
#include "shim_common.h"

static double GPUtc_edge(basic_t& count, const int edges, const int* const nindex, const int* const nlist,
                         const int* const sp) {
  long long c = 0;
  double seconds = 0;
  ig_shim_check(ig_tc_edge(&c, edges, nindex, nlist, sp, &seconds), "GPUtc_edge");
  count = c;
  return seconds;
}
