// TEST INFRASTRUCTURE ONLY.  Request loop of the timing programs (time_*.cpp),
// which run the reference's own best-published C++ variants for the CPU arm
// of the benchmark.  A program loads its graph once, prints "ready", then
// answers one request per stdin line: the line holds the source vertex (or
// any integer for algorithms without one), and the answer is one line
// "runtime: <seconds> check: <integer>", where the seconds are what the
// variant's own timer returns (the figure the reference's drivers print)
// and the check is a result summary.  A line starting with 'q' ends it.
#pragma once
#include <cstdio>
#include <cstdlib>

template <class F>
static int ig_time_loop(F&& run) {
  printf("ready\n");
  fflush(stdout);
  char line[64];
  while (fgets(line, sizeof line, stdin)) {
    if (line[0] == 'q') break;
    long long check = 0;
    const double t = run(atoi(line), check);
    printf("runtime: %.9f check: %lld\n", t, check);
    fflush(stdout);
  }
  return 0;
}
