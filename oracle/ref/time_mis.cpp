// TEST INFRASTRUCTURE ONLY: times the reference's best-published C++ MIS
// variant (codes/cpp/mis-cpp/, data/mis_cpp.csv) through CPPmis_vertex.
// check = size of the set.
// usage: time_mis graph.egr threads  (requests on stdin, see time_common.h)
#include "time_common.h"
#define main indigo_reference_unused_main
#include "mis-cpp/MIS_CPP_V_Topo_Push_IntType_Atomic_NonDeterm_Block.cpp"
#undef main
int main(int argc, char* argv[]) {
  if (argc != 3) return 1;
  ECLgraph g = readECLgraph(argv[1]);
  const int threads = atoi(argv[2]);
  data_type* priority = new data_type[g.nodes];
  unsigned char* status = new unsigned char[g.nodes];
  return ig_time_loop([&](int, long long& check) {
    const double t = CPPmis_vertex(g, priority, status, threads);
    for (int v = 0; v < g.nodes; v++) check += (status[v] == included);
    return t;
  });
}
