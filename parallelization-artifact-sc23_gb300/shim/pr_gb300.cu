// Drop-in variant for include/pr_cuda.h: PR_GPU (:48) has external linkage
// and takes the HOST graph; it prints its iterations and throughput like the
// reference variants do (e.g. codes/cuda/pr-cuda/PR_CUDA_Pull_FloatType_
// Persist_Warp_Determ_Reduction.cu:125-129).
typedef float score_type;
#include "pr_cuda.h"
#include "shim_common.h"

void PR_GPU(const ECLgraph g, score_type* scores, int* degree) {
  const ig_csr h = ig_shim_csr(g);
  int iterations = 0;
  double seconds = 0;
  ig_shim_check(ig_pr(&h, scores, degree, EPSILON, MAX_ITER, &iterations, &seconds), "PR_GPU");
  printf("GPU iterations = %d.\n", iterations);
  printf("GPU runtime: %.6fs\n\n", seconds);
  printf("Throughput: %.6f gigaedges/s\n", 0.000000001 * g.edges / seconds);
}
