// TEST INFRASTRUCTURE ONLY: times the reference's best-published C++
// PageRank variant (codes/cpp/pr-cpp/, data/pr_cpp.csv) through PR_CPU, from
// scores 1/V as the driver sets them (include/pr_cpp.h:93-96), with the
// driver's own constants (EPSILON 1e-4, MAX_ITER 100, include/pr_cpp.h:45-47).
// check = 1e9 x the sum of the scores.
// usage: time_pr graph.egr threads  (requests on stdin, see time_common.h)
#include "time_common.h"
#define main indigo_reference_unused_main
#include "pr-cpp/PR_CPP_Pull_FloatType_AtomicAdd_Block_Determin.cpp"
#undef main
int main(int argc, char* argv[]) {
  if (argc != 3) return 1;
  ECLgraph g = readECLgraph(argv[1]);
  const int threads = atoi(argv[2]);
  int* degree = (int*)malloc(g.nodes * sizeof(int));
  for (int i = 0; i < g.nodes; i++) degree[i] = g.nindex[i + 1] - g.nindex[i];
  score_type* scores = (score_type*)malloc(g.nodes * sizeof(score_type));
  return ig_time_loop([&](int, long long& check) {
    std::fill(scores, scores + g.nodes, 1.0f / (score_type)g.nodes);
    const double t = PR_CPU(g, scores, degree, threads);
    double sum = 0;
    for (int v = 0; v < g.nodes; v++) sum += scores[v];
    check = (long long)(sum * 1e9);
    return t;
  });
}
