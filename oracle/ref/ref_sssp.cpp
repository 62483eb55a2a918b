// TEST INFRASTRUCTURE ONLY: runs the reference's C++ SSSP (threads variant of
// codes/cpp/sssp-cpp/) and CPUserialDijkstra (include/sssp_vertex_cpp.h:88-113).
// usage: ref_sssp graph.egr source out.bin threads
#include "ref_common.h"
#define main indigo_reference_unused_main
#include "sssp-cpp/SSSP_CPP_V_Topo_Push_IntType_ReadModifyWrite_NonDeterm_NoBoundsBug_Block_Atomic_NoRangeBug.cpp"
#undef main
int main(int argc, char* argv[]) {
  if (argc != 5) return 1;
  ECLgraph g = readECLgraph(argv[1]);
  if (g.eweight == NULL) { fprintf(stderr, "ERROR: graph has no weights\n"); return 4; }
  const int src = atoi(argv[2]);
  data_type* dist = new data_type[g.nodes];
  data_type* ver = new data_type[g.nodes];
  const double t = CPUsssp_vertex(src, g, dist, atoi(argv[4]));
  CPUserialDijkstra(src, g, ver);
  for (int v = 0; v < g.nodes; v++)
    if (dist[v] != ver[v]) { fprintf(stderr, "ERROR: variant and verifier differ at %d\n", v); return 3; }
  ig_ref_dump(argv[3], dist, sizeof(data_type) * g.nodes);
  printf("runtime: %.6f\n", t);
  return 0;
}
