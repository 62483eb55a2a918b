// Tunable knobs of the kernels (set through ig_set_option; read by launchers).
#pragma once

struct IgOptions {
  int blocks_per_sm;      // cap on resident blocks per SM for persistent kernels (0 = occupancy)
  int bfs_alpha;          // top-down -> bottom-up switch: frontier edges > unexplored / alpha (0: never)
  int bfs_beta;           // bottom-up -> top-down switch: frontier vertices < V / beta
  int bfs_bitmap;         // 1: bottom-up levels test level bitmaps instead of neighbour distances
  int bfs_bu_claim;       // bottom-up levels: 32-vertex chunks per group claimed from a counter (0: grid stride)
  int hub_degree;         // degree above which a vertex is expanded by the whole grid
  int bfs_hub_degree;     // the same for the single-source BFS (and the connected-components seed BFS)
  long long sssp_delta;   // near/far bucket width (0 = derived from sampled weights)
  int sssp_delta_scale;   // derived width = mean weight * scale / mean degree
  int sssp_heavy_split;   // 1: heavy edges (w >= delta) relaxed once per bucket
  int sssp_item_edges;    // SSSP: edges per work item of a list longer than sssp_warp_degree
  int sssp_warp_degree;   // SSSP: lists longer than this become work items expanded one warp each
  int sssp_window_scale;  // SSSP: expansion window C = mean weight * scale (0 = off); a queued vertex
                          // of degree d is expanded once its distance is below round minimum + C / d
  int sssp_window_degree; // SSSP: vertices of at most this degree are never deferred by the window
  int sssp_merge_below;   // SSSP: a round whose frontier is below this expands (up to 65,536 of) its
                          // work items without a second grid barrier (0 = never)
  int sssp_spin_ns;       // SSSP: pause between polls of a warp waiting for work items (merged rounds)
  int sssp_pair_slices;   // SSSP: work-item slices expanded two at a time (eight edges per lane):
                          // 1 = at 3 blocks per SM, 2 = at 4 (register spills); 0 = one at a time
  int sssp_stage_flags;   // SSSP: 1 = improved vertices staged per warp in shared memory and their
                          // queue flags settled 32 at a time; 0 = settled by the step that found them
  int sssp_chunk;         // SSSP: frontier entries per warp chunk (1..32)
  int sssp_item_group;    // SSSP: most work-item slices a warp claims at a time (1..32)
  int sssp_static_pct;    // SSSP: percent of a pass's frontier chunks and slice groups dealt round-robin
                          // (no atomics); the rest are taken from a counter
  int sssp_tail_split;    // SSSP: chunks / slice groups taken from the counter are this many times smaller
  int sssp_claim_ahead;   // SSSP: 1 = a warp claims its next chunk from the counter as it starts the current
  int sssp_expanded_check;// SSSP: 1 = skip a queued vertex whose distance has not dropped since it was expanded
  int mis_static_pct;     // MIS: percent of a round's worklist groups dealt round-robin (no atomics)
  int pr_hub_degree;      // PageRank: degree above which a vertex is split in chunks
  int pr_chunk;           // PageRank: edges per hub chunk
  int pr_blocks_per_sm;   // PageRank: resident blocks per SM (0 = blocks_per_sm)
  int pr_prefetch;        // PageRank: 1 = a warp prefetches its next lists into L2 while summing
  int pr_subwarp;         // PageRank: 1 = medium lists summed four at a time by 8-lane sub-warps
  int pr_static_pct;      // PageRank: percent of the vertex groups dealt round-robin, the rest from a counter
  int pr_two_pass;        // PageRank: 1 = each iteration first gathers every edge's contribution in one
                          // dense pass (128-bit loads and stores), then sums the lists from it
  int tc_block_chunk;     // TC: in-neighbours per block work item
  int tc_grab;            // TC: block work items taken in runs of this many from a counter, so a middle
                          // vertex's items mostly share one block and its table (0: grid stride)
  int tc_warp_list;       // TC: probe lists at least this long are walked by the whole warp, shorter ones
                          // share the warp's slots through an owner search
  int tc_runs;            // TC: 1 = short probe lists expanded four consecutive slots per lane (one owner
                          // search per lane and step), 0 = an owner search per slot
  int cc_bfs_seed;        // CC: 1 = the largest-degree vertex's component labelled by a BFS from it,
                          // union-find for the rest (0 = neighbour sampling, then union-find;
                          // cc_rounds chooses the sampling form)
  int cc_bfs_levels;      // CC: the seed BFS stops after this many levels (0: runs to the end); vertices
                          // beyond are linked by union-find
  int cc_rounds;          // CC: 1 = sampled neighbours linked one round at a time (read-only root
                          // searches, a compression after each), 0 = both in one pass with path
                          // halving, 2 = as 0 after flattening the initial forest
};

IgOptions& ig_options();
