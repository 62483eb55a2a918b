// Shared by the drop-in translation units: turns a library status into the
// reference drivers' error behaviour (print, exit(-1); include/*_cuda.h CheckCuda).
#pragma once
#include <cstdio>
#include <cstdlib>
#include "indigo_gb300.h"

static inline void ig_shim_check(int status, const char* what) {
  if (status != IG_OK) {
    fprintf(stderr, "ERROR: %s: %s (%s)\n", what, ig_status_string(status), ig_last_error());
    exit(-1);
  }
}

template <class G>
static inline ig_csr ig_shim_csr(const G& g) {
  ig_csr c;
  c.nodes = g.nodes;
  c.edges = g.edges;
  c.nindex = g.nindex;
  c.nlist = g.nlist;
  c.eweight = g.eweight;
  return c;
}
