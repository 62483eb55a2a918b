// TEST INFRASTRUCTURE ONLY: times the reference's best-published C++ CC
// variant (codes/cpp/cc-cpp/, data/cc_cpp.csv) through CPUcc_vertex.
// check = number of components (vertices labelled with their own id).
// usage: time_cc graph.egr threads  (requests on stdin, see time_common.h)
#include "time_common.h"
#define main indigo_reference_unused_main
#include "cc-cpp/CC_CPP_V_Topo_Push_IntType_ReadWrite_NonDeterm_NoBoundsBug_Block_Atomic.cpp"
#undef main
int main(int argc, char* argv[]) {
  if (argc != 3) return 1;
  ECLgraph g = readECLgraph(argv[1]);
  const int threads = atoi(argv[2]);
  data_type* label = new data_type[g.nodes];
  return ig_time_loop([&](int, long long& check) {
    const double t = CPUcc_vertex(g, label, threads);
    for (int v = 0; v < g.nodes; v++) check += (label[v] == v);
    return t;
  });
}
