// TEST INFRASTRUCTURE ONLY: the reference's serial triangle counter
// h_triCounting (include/tc_vertex_cpp.h:88-107) compiled with a 64-bit
// basic_t (the variants fix basic_t to int, which overflows on large graphs).
// The driver declares CPUtc_vertex (:44); this wrapper supplies it as a call
// of h_triCounting, which is the function whose count is dumped and timed.
// usage: ref_tc graph.egr out.bin threads(ignored)
#include "ref_common.h"
typedef long long basic_t;
#define main indigo_reference_unused_main
#include "tc_vertex_cpp.h"
#undef main
static double CPUtc_vertex(basic_t& count, const int nodes, const int* const nindex, const int* const nlist,
                           const int) {
  timeval start, end;
  gettimeofday(&start, NULL);
  count = h_triCounting(nodes, nindex, nlist);
  gettimeofday(&end, NULL);
  return end.tv_sec + end.tv_usec / 1000000.0 - start.tv_sec - start.tv_usec / 1000000.0;
}
int main(int argc, char* argv[]) {
  if (argc != 4) return 1;
  ECLgraph g = readECLgraph(argv[1]);
  for (int v = 0; v < g.nodes; v++)
    for (int i = g.nindex[v] + 1; i < g.nindex[v + 1]; i++)
      if (g.nlist[i - 1] >= g.nlist[i]) { fprintf(stderr, "ERROR: adjacency list not sorted\n"); return 4; }
  basic_t count = 0;
  const double t = CPUtc_vertex(count, g.nodes, g.nindex, g.nlist, 1);
  ig_ref_dump(argv[2], &count, sizeof(count));
  printf("runtime: %.6f\n", t);
  return 0;
}
