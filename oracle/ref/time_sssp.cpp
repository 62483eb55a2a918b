// TEST INFRASTRUCTURE ONLY: times the reference's best-published C++ SSSP
// variant (codes/cpp/sssp-cpp/, data/sssp_cpp.csv) through CPUsssp_vertex.
// check = sum of the finite distances.
// usage: time_sssp graph.egr threads  (requests on stdin, see time_common.h)
#include "time_common.h"
#define main indigo_reference_unused_main
#include "sssp-cpp/SSSP_CPP_V_Topo_Push_IntType_ReadModifyWrite_NonDeterm_NoBoundsBug_Block_Atomic_NoRangeBug.cpp"
#undef main
int main(int argc, char* argv[]) {
  if (argc != 3) return 1;
  ECLgraph g = readECLgraph(argv[1]);
  if (g.eweight == NULL) return 4;
  const int threads = atoi(argv[2]);
  data_type* dist = new data_type[g.nodes];
  return ig_time_loop([&](int src, long long& check) {
    const double t = CPUsssp_vertex(src, g, dist, threads);
    for (int v = 0; v < g.nodes; v++)
      if (dist[v] != maxval) check += dist[v];
    return t;
  });
}
