// TEST INFRASTRUCTURE ONLY: runs the reference's deterministic C++ MIS
// (codes/cpp/mis-cpp/MIS_CPP_V_Topo_Push_IntType_Atomic_CopyDeterm_Block.cpp,
// unsigned priorities) and the driver's verifier (include/mis_vertex_cpp.h:56-75).
// usage: ref_mis graph.egr out.bin threads
#include "ref_common.h"
#define main indigo_reference_unused_main
#include "mis-cpp/MIS_CPP_V_Topo_Push_IntType_Atomic_CopyDeterm_Block.cpp"
#undef main
int main(int argc, char* argv[]) {
  if (argc != 4) return 1;
  ECLgraph g = readECLgraph(argv[1]);
  data_type* priority = new data_type[g.nodes];
  unsigned char* status = new unsigned char[g.nodes];
  const double t = CPPmis_vertex(g, priority, status, atoi(argv[3]));
  verify(g, status);
  ig_ref_dump(argv[2], status, g.nodes);
  printf("runtime: %.6f\n", t);
  return 0;
}
