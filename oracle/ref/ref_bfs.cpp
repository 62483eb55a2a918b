// TEST INFRASTRUCTURE ONLY: runs the reference's C++ BFS (threads variant of
// codes/cpp/bfs-cpp/) and its serial verifier CPUserialDijkstra
// (include/bfs_vertex_cpp.h:52-77) on an .egr graph.
// usage: ref_bfs graph.egr source out.bin threads
#include "ref_common.h"
#define main indigo_reference_unused_main
#include "bfs-cpp/BFS_CPP_V_Topo_Push_IntType_ReadWrite_NoFieldBug_Block_Atomic_Determ_NoBoundsBug_NoRangeBug.cpp"
#undef main
int main(int argc, char* argv[]) {
  if (argc != 5) return 1;
  ECLgraph g = readECLgraph(argv[1]);
  const int src = atoi(argv[2]);
  data_type* dist = new data_type[g.nodes];
  data_type* ver = new data_type[g.nodes];
  const double t = CPPbfs_vertex(src, g, dist, atoi(argv[4]));
  CPUserialDijkstra(src, g, ver);
  for (int v = 0; v < g.nodes; v++)
    if (dist[v] != ver[v]) { fprintf(stderr, "ERROR: variant and verifier differ at %d\n", v); return 3; }
  ig_ref_dump(argv[3], dist, sizeof(data_type) * g.nodes);
  printf("runtime: %.6f\n", t);
  return 0;
}
