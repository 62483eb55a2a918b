// TEST INFRASTRUCTURE ONLY.  Shared helpers of the wrapper programs that run
// the reference's own C++ entry functions (compiled from its sources, never
// copied) and dump their results as raw little-endian arrays for the golden
// fixtures.  Each wrapper renames the reference driver's main() before
// including the variant file, then defines its own main.
#pragma once
#include <cstdio>
#include <cstdlib>

static inline void ig_ref_dump(const char* path, const void* data, size_t bytes) {
  FILE* f = fopen(path, "wb");
  if (!f || fwrite(data, 1, bytes, f) != bytes) {
    fprintf(stderr, "ERROR: cannot write %s\n", path);
    exit(2);
  }
  fclose(f);
}
