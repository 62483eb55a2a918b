// TEST INFRASTRUCTURE ONLY: runs the reference's C++ CC (codes/cpp/cc-cpp/
// CC_CPP_V_Topo_Push_IntType_ReadModifyWrite_Determ_NoBoundsBug_Block_Atomic.cpp)
// and the driver's adjacency check (include/cc_vertex_cpp.h).
// usage: ref_cc graph.egr out.bin threads
#include "ref_common.h"
#define main indigo_reference_unused_main
#include "cc-cpp/CC_CPP_V_Topo_Push_IntType_ReadModifyWrite_Determ_NoBoundsBug_Block_Atomic.cpp"
#undef main
int main(int argc, char* argv[]) {
  if (argc != 4) return 1;
  ECLgraph g = readECLgraph(argv[1]);
  data_type* label = new data_type[g.nodes];
  const double t = CPUcc_vertex(g, label, atoi(argv[3]));
  for (int v = 0; v < g.nodes; v++)
    for (int i = g.nindex[v]; i < g.nindex[v + 1]; i++)
      if (label[g.nlist[i]] != label[v]) { fprintf(stderr, "ERROR: adjacent vertices in different components\n"); return 3; }
  ig_ref_dump(argv[2], label, sizeof(data_type) * g.nodes);
  printf("runtime: %.6f\n", t);
  return 0;
}
