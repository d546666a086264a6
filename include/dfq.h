/*
 * dfq.h - C ABI of libdfq, a GB300 (sm_103a) decentralized-frontier-queue BFS.
 *
 * This is the drop-in boundary for the reference `bfs` programs of DFQ-BFS.
 * Each reference program is one CUDA file with a host main() and one
 * cooperative kernel; the canonical one is
 *   design/shared-q/atomic-sa/our-sep/upper-bound/bfs.cu   (called "DFQ" below)
 * Every entry point below says which part of that file it replaces.
 *
 * Conventions
 *   - Plain C types only: int32_t vertex ids, int64_t edge counts, caller-owned
 *     buffers.  No exceptions cross the ABI; every function returns an int status
 *     (DFQ_OK or a negative DFQ_E* code) and dfq_last_error() gives a message
 *     (thread-local).
 *   - Levels are int32 with -1 for unreached vertices: the same bit pattern as the
 *     reference's `short cost[]` (-1 = unvisited, DFQ:192,216) widened so that
 *     depth is not capped at 32767.
 *   - One call in flight per dfq_graph handle (each handle owns a CUDA stream);
 *     calls on different handles may come from different host threads.
 */
#ifndef DFQ_H
#define DFQ_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
#define DFQ_OK          0
#define DFQ_EINVAL     (-1)  /* bad argument (null pointer, source out of range, ...) */
#define DFQ_ENOMEM     (-2)  /* host or device allocation failed / over budget */
#define DFQ_ECUDA      (-3)  /* a CUDA runtime call failed */
#define DFQ_ETIMEOUT   (-4)  /* a bounded device-side wait expired; the kernel returned */
#define DFQ_EFORMAT    (-5)  /* malformed graph file or inconsistent CSR */
#define DFQ_EIO        (-6)  /* file could not be opened / read / written */
#define DFQ_EDEVICE    (-7)  /* device-side consistency check failed (queue capacity, ...) */
#define DFQ_EBUSY      (-8)  /* no free slot / memory budget for the request */

/* Message for the last failing call on this host thread ("" if none). */
const char* dfq_last_error(void);

/* Host threads used by the loaders, the CSR builder and the generators
 * (0 = the DFQ_HOST_THREADS environment variable, else every hardware
 * thread, at most 64).  Results never depend on it.  No reference
 * counterpart: the reference's loader is one fscanf loop (DFQ:184-200). */
int dfq_set_host_threads(int32_t threads);
int32_t dfq_host_threads(void);

/* ------------------------------------------------------------- host CSR */
/*
 * Compressed sparse rows: offsets[n+1], cols[e].  Arrays are owned by the
 * library (malloc) and released with dfq_csr_free().  `source` is the source
 * vertex named by the file (the reference's .dat header, DFQ:188), else 0.
 *
 * Replaces the reference's `Node{int start; int length}` AoS plus `int edge[]`
 * (DFQ:38-42,190-199): SoA offsets are half the bytes per frontier vertex and
 * need no second array to be kept consistent.
 */
typedef struct dfq_csr {
    int32_t  n;        /* vertices */
    int32_t  source;   /* source named by the input, or 0 */
    int64_t  e;        /* directed edges (< 2^31) */
    int32_t* offsets;  /* n+1 entries, offsets[0]=0, non-decreasing */
    int32_t* cols;     /* e entries, each in [0,n) */
} dfq_csr;

/* dfq_csr_from_edges / dfq_csr_load flags */
#define DFQ_CSR_SYMMETRIZE     1  /* add v->u for every u->v */
#define DFQ_CSR_DEDUP          2  /* sort each row and drop repeated neighbours */
#define DFQ_CSR_NO_SELF_LOOPS  4  /* drop u->u */

/* file formats */
#define DFQ_FMT_AUTO  0  /* sniff: '#' first -> SNAP, "DFQCSR01" magic -> BIN, else DAT */
#define DFQ_FMT_SNAP  1  /* "# Nodes: N Edges: E" / "# FromNodeId ToNodeId" / "u v" lines */
#define DFQ_FMT_DAT   2  /* reference input: "N E SOURCE", N x "start length", E x "dst x" */
#define DFQ_FMT_BIN   3  /* binary CSR cache written by dfq_csr_save */

/* Read a graph file.  Replaces the reference loader (DFQ:184-200) and adds the
 * SNAP edge list that the reference README documents (README.md:19-32) but no
 * reference binary reads.  SNAP edges are kept as given (directed) unless
 * flags ask otherwise; ids >= the header's N grow N to max id + 1.  Text is
 * parsed by all host threads over line- or token-aligned pieces; the result
 * and any error message are those of a serial reader. */
int dfq_csr_load(const char* path, int32_t format, int32_t flags, dfq_csr* out);

/* Write a graph as SNAP text, reference .dat text, or binary CSR. */
int dfq_csr_save(const char* path, const dfq_csr* g, int32_t format);

/* Build CSR from an edge list (stable counting sort by source; file order of
 * neighbours is kept unless DFQ_CSR_DEDUP sorts rows). */
int dfq_csr_from_edges(const int32_t* src, const int32_t* dst, int64_t m,
                       int32_t n, int32_t flags, dfq_csr* out);

/* Release arrays owned by a dfq_csr and zero it. */
void dfq_csr_free(dfq_csr* g);

/* ------------------------------------------------------ seeded generators */
/* All generators are deterministic in their seed and independent of the
 * number of host threads used.  No reference counterpart: the reference's
 * SNAP datasets are not in its repository, these stand in for them. */

/* Directed graph: out-degree ~ Geometric(mean mean_deg) on {0,1,...},
 * destinations ~ Zipf(alpha) over a seeded permutation of the ids, self-loops
 * and repeats redrawn (so the edge count keeps its expectation). */
int dfq_gen_zipf_geometric(int32_t n, double mean_deg, double alpha, uint64_t seed,
                           dfq_csr* out);

/* R-MAT (Chakrabarti et al. 2004): 2^scale vertices, edge_factor * 2^scale
 * generated edges, quadrant probabilities a, b, c (d = 1-a-b-c), random vertex
 * relabelling; flags as for dfq_csr_from_edges (usually SYMMETRIZE|DEDUP|NO_SELF_LOOPS). */
int dfq_gen_rmat(int32_t scale, int32_t edge_factor, double a, double b, double c,
                 uint64_t seed, int32_t flags, dfq_csr* out);

/* side x side 4-neighbour grid, a seeded fraction of undirected edges deleted;
 * if keep_lcc, only the largest connected component is kept, relabelled
 * compactly in row-major order (orig_ids, if non-null, receives for each new
 * vertex its row-major id in the full grid; caller frees with dfq_free). */
int dfq_gen_grid(int32_t side, double delete_frac, uint64_t seed, int32_t keep_lcc,
                 dfq_csr* out, int32_t** orig_ids);

/* k sources drawn uniformly (seeded) from vertices with out-degree > 0. */
int dfq_pick_sources(const dfq_csr* g, int32_t k, uint64_t seed, int32_t* out);

/* free() for arrays returned by this library. */
void dfq_free(void* p);

/* ------------------------------------------------------------- device BFS */
typedef struct dfq_opts {
    int32_t block_threads;      /* threads per block: 256, 512 or 1024; 0 (the default) = by
                                   graph: 1024 when the average degree is below 8 (high-diameter
                                   graphs: fewer, larger blocks end each small level sooner),
                                   else 512; pools and servers: 1024 where the shared-memory
                                   layout fits, else 512 */
    int32_t blocks_per_sm;      /* 0 = the occupancy limit (cooperative launch) */
    int32_t medium_min_degree;  /* deg >= this leaves the small bin (block-gathered edges)
                                   for the medium bin (one warp per vertex, int4 loads) */
    int32_t large_min_degree;   /* deg >= this goes to the grid-wide large bin */
    int32_t local_queue_cap;    /* per-block shared-memory frontier slots (0 = default) */
    int32_t local_edge_budget;  /* edges a block may keep in its shared-memory queue per
                                   level; the rest overflows to the global queue (0 = default) */
    int32_t piece_edges;        /* large-bin piece: edges one warp stages and expands
                                   (multiple of 64) */
    int32_t probe_first;        /* 1: read the visited bitmap before the atomic claim;
                                   0: claim at once and fetch row bounds alongside;
                                   2: choose per level by frontier size (every level
                                   probes on a graph stored hub-first) */
    int32_t l2_persist;         /* 1: visited bitmap in an L2 persisting access window */
    int32_t use_tma;            /* 1: stage large-bin pieces into smem with cp.async.bulk */
    int32_t timeout_ms;         /* bound on every device-side wait (0 = 5000) */
    int32_t wide_min_edges;     /* pools: a graph runs on the whole grid when it has at least */
    int32_t wide_min_degree;    /*   this many edges and this average degree (0 = defaults) */
    int32_t hot_cache;          /* K in 1..32: on levels that probe, keep the visited bits of the
                                   first K x 8192 vertex ids in K KB of shared memory per block
                                   (K rounded down to 4 KB; hub-first ids put the most-probed
                                   vertices there); 0 or -1: no cache (the default) */
    int32_t vertex_order;       /* read by dfq_graph_create only: 0 = hub-first ids (by
                                   descending degree) when the degrees are skewed, 1 = keep the
                                   input ids, 2 = hub-first always.  Results are always reported
                                   in the input ids. */
    int32_t profile;            /* 1: also record when each block finished each level (the
                                   spread and barrier times of dfq_bfs_last_levels); k > 1 in the
                                   profiling build (DFQ_CLAIM_PROBES=1): the same, for the 64
                                   levels from level k on (the product build traces levels 0-63) */
    int32_t direction;          /* 0: top-down levels only (the reference's algorithm);
                                   1: direction-optimising - levels whose frontier holds many
                                   edges run bottom-up (each unvisited vertex looks for a parent
                                   among its neighbours).  Needs an undirected graph: give 1 to
                                   dfq_graph_create, which checks that every row is sorted and
                                   every edge u->v has its v->u (else DFQ_EINVAL).  Same levels;
                                   parents may differ (still a BFS tree); E_R still reported. */
    int32_t stall_test_level;   /* failure-path test hook, 0 = off (the default).  k > 0: at the
                                   end of level k-1 the launch's last block does not arrive at the
                                   grid barrier, so every block's bounded wait runs out after
                                   timeout_ms and the call returns DFQ_ETIMEOUT; the graph stays
                                   usable.  Single-source launches (dfq_bfs, dfq_bfs_launch) only. */
    int32_t cluster_blocks;     /* single-source launches: 0 (the default) = the whole GPU, one
                                   cooperative grid with a grid barrier between levels; C in
                                   {2, 4, 8, 16} = one thread-block cluster of C blocks runs the
                                   BFS, its levels ending on a cluster barrier in distributed
                                   shared memory.  For graphs whose levels stay small (grids,
                                   meshes, road networks: thousands of levels of a few thousand
                                   vertices); a level with millions of vertices runs on C SMs
                                   only.  DFQ_EINVAL at launch if such a cluster does not fit. */
} dfq_opts;

typedef struct dfq_stats {
    float   kernel_ms;   /* device time of the BFS launch (CUDA events, launch included:
                            the reference's "- Time" definition, DFQ:279-288) */
    int32_t depth;       /* largest level reached (reference "- Dist", DFQ:290-297) */
    int32_t levels;      /* level iterations the kernel ran */
    int64_t reached;     /* vertices with level >= 0 (reference "- Touch" numerator) */
    int64_t edges;       /* E_R: sum of out-degrees over reached vertices */
    int64_t overflow;    /* frontier entries that overflowed the shared-memory queues */
    int64_t large;       /* vertices expanded through the large bin */
} dfq_stats;

typedef struct dfq_graph dfq_graph;

/* Defaults for every dfq_opts field. */
void dfq_opts_default(dfq_opts* o);

/* Copy a CSR (host or device pointers) into a device-resident graph with its
 * per-query workspace.  Replaces DFQ:194-199 + DFQ:273-277 (managed allocation
 * and prefetch of node/edge/cost) and the static __device__ queues DFQ:96-97.
 * opts may be null (defaults). */
int dfq_graph_create(const int32_t* offsets, const int32_t* cols, int32_t n, int64_t e,
                     const dfq_opts* opts, dfq_graph** out);

/* Release a graph and its workspace.  Replaces DFQ:312-316. */
int dfq_graph_destroy(dfq_graph* g);

/* Options in force on a graph / replace them (validated). */
int dfq_graph_get_opts(const dfq_graph* g, dfq_opts* o);
int dfq_graph_set_opts(dfq_graph* g, const dfq_opts* o);

/* The CUDA stream a graph's launches are queued on (as void*). */
void* dfq_graph_stream(dfq_graph* g);

/* Vertex / edge counts of a graph (-1 for a null handle).  The reference
 * keeps them in *NUM_NODES / NUM_EDGES (DFQ:185-188). */
int32_t dfq_graph_num_vertices(const dfq_graph* g);
int64_t dfq_graph_num_edges(const dfq_graph* g);

/* Single-source BFS, synchronous.  Replaces the kernel launch and its timing
 * (DFQ:255-288: occupancy-sized cooperative launch of CUDA_BFS_KERNEL_CG_NEW,
 * events around launch + synchronize).  levels[n] (required) and parents[n]
 * (nullable) may be host or device pointers; parents[src] = src, parents of
 * unreached vertices = -1.  stats may be null.  Page-locked host buffers
 * mapped into the device (cudaHostAlloc, cudaHostRegister) are written by the
 * kernel itself at the end of the run; other host buffers are copied from
 * device scratch after it. */
int dfq_bfs(dfq_graph* g, int32_t src, int32_t* levels, int32_t* parents, dfq_stats* stats);

/* Queue the same BFS on the graph's stream and return at once (device
 * pointers only).  For timing loops and CUDA-graph capture; read the outcome
 * later with dfq_graph_sync + dfq_bfs_last_stats. */
int dfq_bfs_launch(dfq_graph* g, int32_t src, int32_t* levels_dev, int32_t* parents_dev);

/* Wait for the graph's stream; returns the device status of the last launch. */
int dfq_graph_sync(dfq_graph* g);

/* Counters of the last completed launch on this graph (kernel_ms = 0 here). */
int dfq_bfs_last_stats(dfq_graph* g, dfq_stats* stats);

/* Per-level trace of the last completed launch: for the first min(levels,
 * max_levels, 64) levels, the device clock (ns) when the level started and the
 * number of frontier entries it expanded.  Returns the number of levels
 * written (>= 0) or a negative status.  Replaces the reference's per-level
 * frontier profiler (design/shared-q/atomic-sa/our-sep/upper-bound/
 * bfs_ftr_prof.cu:98-144, printed from the device at :206-208). */
int dfq_bfs_last_trace(dfq_graph* g, int64_t* start_ns, int32_t* frontier, int32_t max_levels);

/* Per-level profile of the last completed launch (first 64 levels): what the
 * level scanned and how it ended.  start_ns..last_done_ns are device clock
 * readings: last_done - first_done is the spread of block finish times (load
 * imbalance) and the next level's start_ns - last_done_ns the barrier's cost.
 * Replaces the reference's device-printf profilers (bfs_ftr_prof.cu:98-144 and
 * design/shared-q/atomic-sa/sup-sep/upper-bound/profile/workload.cuh), which print
 * per-bin frontier sizes and visit counts from inside the kernel. */
typedef struct dfq_level_info {
    int64_t start_ns;       /* %globaltimer when the level began (block 0, after the barrier) */
    int64_t first_done_ns;  /* earliest block to finish the level's work */
    int64_t last_done_ns;   /* latest block to finish it */
    int32_t frontier;       /* frontier entries expanded (local + overflow + large) */
    int32_t edges;          /* their degree sum: adjacency entries the level scans */
    int32_t overflow;       /* entries read from the global overflow queue */
    int32_t pieces;         /* large-list pieces */
    int32_t probe;          /* 1: probe-then-claim level, 0: claim at once, 2: bottom-up */
    int32_t level;          /* the level's index (the traced window starts at level 0, or in
                               the profiling build at dfq_opts.profile when that is > 1) */
    /* with profile: over all warps, the latest time (ns after the warp began the level) a warp
     * finished its block's own queue, the large-list pieces, the overflow queue, and its claims */
    int32_t phase_ns[4];
    /* profiling build only (library built with DFQ_CLAIM_PROBES=1), with profile: the latest
     * time (ns after the warp began the level) a claim batch had its neighbours in hand, had
     * their row bounds, had its claim atomics answered, and had pushed its winners; else 0 */
    int32_t claim_ns[4];
    /* profiling build only, with profile: sums over all warps of the staged large-list pieces
     * expanded on a probe level, the ns spent waiting for their bulk copies, the ns spent
     * expanding them (claims included), and the ns spent in candidate claim drains anywhere */
    int64_t piece_stats[4];
} dfq_level_info;
int dfq_bfs_last_levels(dfq_graph* g, dfq_level_info* out, int32_t max_levels);

/* Idle-lane profile of the reference's binned expansion for one BFS,
 * computed exactly on the host from its levels (identical to the
 * reference's) and the degrees.  Replaces the device counters of
 * design/shared-q/atomic-sa/our-sep/upper-bound/bfs_ftr_prof.cu:98-144 (its
 * "L: a b c e f" lines, printed at :206-208).  A frontier vertex of level L
 * with degree d > 0 falls in the first bin whose range holds d (d <=
 * tiles[0], tiles[1], tiles[2], tiles[3], else the fifth, whole-grid bin);
 * count[L][bin] += 1 and idle[L][bin] += tile - (d & (tile - 1)) for the
 * four tiled bins, threads - (d % threads) for the fifth - the reference's
 * formula, which also charges a whole tile when d is a multiple of it.
 * tiles: four increasing powers of two (the reference's TILE_SIZ_A/B/C/E,
 * bfs_ftr_prof.cu:18-35, e.g. 16, 128, 1024, 8192); threads: its
 * gridDim.x * blockDim.x.  idle and count hold max_levels x 5 entries (either
 * may be null).  Returns the number of levels filled (depth + 1, at most
 * max_levels) or a negative status. */
int dfq_frontier_profile(const dfq_csr* g, const int32_t* levels, const int32_t tiles[4], int64_t threads,
                         int32_t max_levels, int64_t* idle, int64_t* count);

/* Choose opts for this graph by timing candidate settings on a few sources;
 * writes the winner to *best and installs it on the graph. */
int dfq_autotune(dfq_graph* g, const int32_t* sources, int32_t nsrc, dfq_opts* best);

/* 1 if the graph is stored in hub-first ids (chosen at create), 0 if in its
 * input ids, -1 for a null graph. */
int32_t dfq_graph_is_hub_first(const dfq_graph* g);

/* The graph's class for tuned-option reuse: "skewed" (stored hub-first) or
 * "even", then n and the average degree rounded to powers of two, e.g.
 * "skewed-n2^22-d2^5".  Writes a NUL-terminated string into buf[len] and
 * returns its length, or a negative status. */
int dfq_graph_class(const dfq_graph* g, char* buf, int32_t len);

/* dfq_autotune with a persistent cache of tuned options: the JSON file at
 * cache_path holds one entry per (GPU, graph class), the GPU named by its
 * device name, SM count and compute capability.  A hit installs the stored
 * options without timing anything (*hit = 1); a miss tunes and adds the
 * winner to the file (*hit = 0; the file is rewritten through a temporary
 * and a rename).  The reference tuned its bins by hand per program and
 * compared settings offline (design/shared-q/atomic-sa/our-sep/upper-bound/
 * com-orkut_8-64-1024-16384-all and its siblings). */
int dfq_autotune_cached(dfq_graph* g, const int32_t* sources, int32_t nsrc, const char* cache_path,
                        dfq_opts* best, int32_t* hit);

/* ------------------------------------------- graph pools and batched BFS */
/* No reference counterpart: the reference runs one source per process launch
 * (its '$' mode re-queries one source at a time, DFQ:202-214,302-308).
 *
 * A pool holds many graphs resident on the device (their CSR arrays packed in
 * two allocations) plus the BFS workspaces.  A batch runs many queries
 * (graph, source) in ONE persistent cooperative launch: "wide" queries (graphs
 * with at least wide_min_edges edges and average degree >= wide_min_degree)
 * run one after another on the whole grid, then every block pulls "narrow"
 * queries (small or high-diameter graphs) and runs each alone with its block
 * barrier as the level barrier.  Narrow queries on large high-diameter
 * graphs (>= 65,536 vertices, average degree < 8) run on "gangs" of 2 to 16
 * blocks from the launch's start when half the grid leaves at least two
 * blocks for each of them. */
typedef struct dfq_pool dfq_pool;

typedef struct dfq_query {
    int32_t  graph;     /* index into the pool */
    int32_t  source;
    int32_t* levels;    /* device array of the graph's n entries (required) */
    int32_t* parents;   /* device array or null; all queries of a batch or none */
} dfq_query;

typedef struct dfq_query_result {
    int32_t status;     /* DFQ_OK or a DFQ_E* code of this query */
    int32_t wide;       /* 1: ran on the whole grid, 0: on one block */
    int32_t depth;
    int32_t levels;
    int64_t reached;
    int64_t edges;      /* E_R */
    double  start_us;   /* device clock, from the start of the batch launch */
    double  end_us;
} dfq_query_result;

#define DFQ_BATCH_GRAPH  1  /* capture table upload + reset + launch in a CUDA graph and replay it */

/* Upload graphs (host CSR) into a device pool.  opts may be null; its
 * wide_* fields choose how queries are split.  Replaces, for many graphs at
 * once, DFQ:194-199,273-277. */
int dfq_pool_create(const dfq_csr* graphs, int32_t ngraphs, const dfq_opts* opts, dfq_pool** out);
int dfq_pool_destroy(dfq_pool* p);
int32_t dfq_pool_num_graphs(const dfq_pool* p);
int dfq_pool_graph_info(const dfq_pool* p, int32_t graph, int32_t* n, int64_t* e, int32_t* wide);

/* The pool's options.  set_opts changes the kernel options of later
 * launches (a captured batch is re-captured); wide_min_edges,
 * wide_min_degree and vertex_order are fixed at creation (DFQ_EINVAL). */
int dfq_pool_get_opts(const dfq_pool* p, dfq_opts* o);
int dfq_pool_set_opts(dfq_pool* p, const dfq_opts* o);

/* Choose the pool's kernel options by timing dfq_pool_batch on the given
 * queries (coordinate descent over block size, bin thresholds, piece size,
 * local queue capacity, probe mode and bulk-copy staging); installs and
 * returns the winner.  The reference fixed these per program with #defines
 * (design/shared-q/atomic-sa/our-sep/upper-bound/bfs.cu:16-36). */
int dfq_pool_autotune(dfq_pool* p, const dfq_query* q, int32_t nq, dfq_opts* best);

/* One query as one plain cooperative launch on the whole grid (synchronous):
 * the per-query baseline batches are compared with. */
int dfq_pool_bfs(dfq_pool* p, int32_t graph, int32_t src, int32_t* levels_dev, int32_t* parents_dev,
                 dfq_stats* stats);

/* Run nq queries in one persistent launch (flags: DFQ_BATCH_GRAPH).  Fills
 * results[nq] (nullable) and *total_ms (device time of the batch, nullable).
 * Returns DFQ_OK if every query succeeded. */
int dfq_pool_batch(dfq_pool* p, const dfq_query* q, int32_t nq, int32_t flags, dfq_query_result* results,
                   float* total_ms);

/* ------------------------------------------------------------- serving */
/* No reference counterpart.  A server keeps a pool resident and serves a
 * stream of single-source requests with continuous batching on the device:
 * one persistent serving kernel claims requests as they are published (block
 * by block for narrow graphs; the whole grid, between its blocks' own
 * requests, for wide graphs), so requests that arrive while others run join
 * the device work at once.  Each request gets its level array (and parents)
 * from an HBM arena; a request is admitted when its arrays fit the arena's
 * budget and a ring slot is free, else it waits in FIFO order.  The kernel
 * leaves after idle_ms without work and is relaunched on the next request. */
typedef struct dfq_server dfq_server;

typedef struct dfq_server_opts {
    int64_t hbm_budget_bytes;  /* arena for per-request outputs (0 = 1/4 of free HBM) */
    int32_t ring_capacity;     /* requests on the device at once, power of two (0 = 4096) */
    int32_t idle_ms;           /* serving kernel exits after this long without work (0 = 20) */
    int32_t with_parents;      /* also produce parent arrays */
    int32_t narrow_queue_cap;  /* per-block frontier capacity for narrow requests (0 = 1 << 20);
                                  a request that outgrows it is rerun on the whole grid */
} dfq_server_opts;

typedef struct dfq_server_result {
    int64_t id;
    int64_t tag;
    int32_t status;     /* DFQ_OK or DFQ_E* */
    int32_t wide;       /* 1: ran on the whole grid */
    int32_t depth;
    int32_t retried;    /* 1: outgrew a block's queues and was rerun on the whole grid */
    int64_t reached;
    int64_t edges;
    double  submit_us;  /* host clock, microseconds since the server was created */
    double  done_us;    /* host clock when the completion was observed */
    double  device_us;  /* device time of the BFS itself */
} dfq_server_result;

int dfq_server_create(dfq_pool* pool, const dfq_server_opts* opts, dfq_server** out);
/* Queue a request (never blocks); *id identifies it in results. */
int dfq_server_submit(dfq_server* s, int32_t graph, int32_t source, int64_t tag, int64_t* id);
/* Admit what fits, (re)launch the serving kernel if needed, and return up to
 * max completed results in *count. */
int dfq_server_poll(dfq_server* s, dfq_server_result* out, int32_t max, int32_t* count);
/* Copy a completed request's levels (and parents) to host memory. */
int dfq_server_levels(dfq_server* s, int64_t id, int32_t* levels, int32_t* parents);
/* Return a completed request's arrays to the arena. */
int dfq_server_release(dfq_server* s, int64_t id);
/* Requests submitted but not yet completed. */
int64_t dfq_server_pending(const dfq_server* s);

/* Replay a request trace: request i (graph[i], source[i]) is submitted at
 * arrival_us[i] microseconds after the call starts (non-decreasing), the
 * server is polled in between, and results[i] receives its result with
 * submit_us = its scheduled arrival and done_us = when its completion was
 * observed (both on the call's clock).  Results are released as they arrive
 * unless keep (nullable) is non-zero for them; kept ones are released by the
 * caller (dfq_server_levels / dfq_server_release with results[i].id).
 * Returns after every request completed. */
int dfq_server_replay(dfq_server* s, const int32_t* graph, const int32_t* source, const double* arrival_us,
                      int32_t n, const int32_t* keep, dfq_server_result* results);
int dfq_server_destroy(dfq_server* s);

/* -------------------------------------------------- allocation-free BFS */
/* No counterpart in the reference (its kernel uses static __device__ queues
 * plus managed allocations made by main()).
 *
 * For callers that cannot call cudaMalloc: a host framework that owns the
 * GPU's memory through its own pool, a serving process that reserves its HBM
 * budget at start-up and forbids later allocation, or code that cannot accept
 * cudaMalloc/cudaFree stalling every stream on the device.  dfq_graph_create
 * allocates a workspace per graph; this entry point allocates nothing.  The
 * caller passes the CSR (offsets[n+1], cols[e]) and levels[n] (parents[n]
 * nullable) in device memory it owns; the kernel's scratch (visited bitmap,
 * frontier queues, control block) is one fixed array of
 * DFQ_NOALLOC_SCRATCH_BYTES inside libdfq that every GPU loading the library
 * holds until the process exits.  That bounds the graph to roughly
 * 24 * n + e / 5 bytes of scratch (about 1.2 million vertices at average
 * degree 16); larger graphs are rejected with DFQ_ENOMEM and a message naming
 * the bytes needed.  cols must be 16-byte aligned.  The CSR is checked on the
 * device first (DFQ_EFORMAT if malformed); that check reads every offset and
 * column once more per call, so a call moves up to twice the bytes of
 * dfq_bfs on a graph handle, which checks its CSR once at creation.
 *
 * Runs on `stream` (null = the legacy default stream) with the default
 * dfq_opts and returns after the BFS has finished; stats (nullable) gets the
 * counters, kernel_ms = 0 (no events are created).  The first call on a device
 * looks up the scratch array's device address and caches it: make it before
 * any stream capture.  All calls share the one array: calls that overlap on
 * the GPU (other streams, other host threads) race and must be serialised by
 * the caller. */
#define DFQ_NOALLOC_SCRATCH_BYTES (32u << 20)
int dfq_bfs_noalloc(const int32_t* offsets_dev, const int32_t* cols_dev, int32_t n, int64_t e,
                    int32_t src, int32_t* levels_dev, int32_t* parents_dev, void* stream,
                    dfq_stats* stats);

#ifdef __cplusplus
}
#endif
#endif /* DFQ_H */
