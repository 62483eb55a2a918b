// TEST INFRASTRUCTURE ONLY: runs the reference's C++ pull PageRank
// (codes/cpp/pr-cpp/PR_CPP_Pull_FloatType_Reduction_Block_Determin.cpp with the
// constants of include/pr_cpp.h:45-47) from scores 1/V and dumps the scores.
// usage: ref_pr graph.egr out.bin threads
#include "ref_common.h"
#define main indigo_reference_unused_main
#include "pr-cpp/PR_CPP_Pull_FloatType_Reduction_Block_Determin.cpp"
#undef main
int main(int argc, char* argv[]) {
  if (argc != 4) return 1;
  ECLgraph g = readECLgraph(argv[1]);
  int* degree = (int*)malloc(g.nodes * sizeof(int));
  for (int i = 0; i < g.nodes; i++) degree[i] = g.nindex[i + 1] - g.nindex[i];
  const score_type init_score = 1.0f / (score_type)g.nodes;
  score_type* scores = (score_type*)malloc(g.nodes * sizeof(score_type));
  std::fill(scores, scores + g.nodes, init_score);
  const double t = PR_CPU(g, scores, degree, atoi(argv[3]));
  ig_ref_dump(argv[2], scores, sizeof(score_type) * g.nodes);
  printf("runtime: %.6f\n", t);
  return 0;
}
