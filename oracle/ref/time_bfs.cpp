// TEST INFRASTRUCTURE ONLY: times the reference's best-published C++ BFS
// variant (codes/cpp/bfs-cpp/, fastest C++ BFS on RMAT-22 in data/bfs_cpp.csv)
// through its entry function CPPbfs_vertex.  check = vertices reached.
// usage: time_bfs graph.egr threads  (requests on stdin, see time_common.h)
#include "time_common.h"
#define main indigo_reference_unused_main
#include "bfs-cpp/BFS_CPP_V_Topo_Push_IntType_ReadWrite_NoFieldBug_Block_Atomic_Determ_NoBoundsBug_NoRangeBug.cpp"
#undef main
int main(int argc, char* argv[]) {
  if (argc != 3) return 1;
  ECLgraph g = readECLgraph(argv[1]);
  const int threads = atoi(argv[2]);
  data_type* dist = new data_type[g.nodes];
  return ig_time_loop([&](int src, long long& check) {
    const double t = CPPbfs_vertex(src, g, dist, threads);
    for (int v = 0; v < g.nodes; v++) check += (dist[v] != maxval);
    return t;
  });
}
