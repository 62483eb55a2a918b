// Drop-in variant for the reference BFS driver include/bfs_vertex_cuda.h: the
// driver's main() reads the graph, uploads it and calls GPUbfs_vertex three
// times; this translation unit supplies that entry function from the GB300
// library.  Build: nvcc with the reference's include/ directory and this
// repository's include/ on the include path, linked against libindigo_gb300.so.
typedef int basic_t;
#include "bfs_vertex_cuda.h"
#include "shim_common.h"

static double GPUbfs_vertex(const int src, const ECLgraph& g, basic_t* const dist) {
  const ig_csr d = ig_shim_csr(g);  // device nindex/nlist, as uploaded by main()
  double seconds = 0;
  ig_shim_check(ig_bfs_vertex(src, &d, dist, &seconds), "GPUbfs_vertex");
  return seconds;
}
