// TEST INFRASTRUCTURE ONLY: times the reference's best-published C++
// triangle-counting variant (codes/cpp/tc-cpp/, data/tc_cpp.csv) through
// CPUtc_vertex on a graph with sorted adjacency.  Its count type is the
// variant's own (int).  check = the count.
// usage: time_tc graph.egr threads  (requests on stdin, see time_common.h)
#include "time_common.h"
#define main indigo_reference_unused_main
#include "tc-cpp/TC_CPP_V_IntType_Critical_Cyclic.cpp"
#undef main
int main(int argc, char* argv[]) {
  if (argc != 3) return 1;
  ECLgraph g = readECLgraph(argv[1]);
  const int threads = atoi(argv[2]);
  return ig_time_loop([&](int, long long& check) {
    basic_t count = 0;
    const double t = CPUtc_vertex(count, g.nodes, g.nindex, g.nlist, threads);
    check = (long long)count;
    return t;
  });
}
