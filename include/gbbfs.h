/*
 * gbbfs — direction-optimizing BFS on one GB300 GPU, behind a plain C ABI.
 *
 * This is the drop-in boundary for the BFS hot path of DMM-GAPBS.  The
 * reference has no FFI layer: its boundary is the kernel functor
 * `pvector<NodeID> DOBFS(const Graph&, NodeID source, ...)` that `main` hands
 * to BenchmarkKernel (src/bfs.cc:142, :268, :273; src/benchmark.h:118-145),
 * the graph that Builder::MakeGraph constructs (src/builder.h:314-338,
 * gapbs-verify/builder.h:231-252), the SourcePicker sequence
 * (src/benchmark.h:49-88) and the bfs_output.txt file that BFSVerifier writes
 * (src/bfs.cc:213-235).  Each entry point below names the reference interface
 * it replaces.
 *
 * Conventions: every call returns a gbbfs status (GBBFS_OK == 0).  No C++
 * exception crosses this boundary.  A graph handle owns one CUDA stream and
 * its per-search device state; calls on one handle must not run concurrently
 * (one handle per host thread).  Host arrays stay owned by the caller.
 * NodeID is int32_t and edge offsets int64_t, as in the reference
 * (src/benchmark.h:31, src/graph.h SGOffset).
 */
#ifndef GBBFS_H_
#define GBBFS_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. */
#define GBBFS_OK 0
#define GBBFS_ERR_ARG 1     /* bad argument (NULL handle, source out of range, ...) */
#define GBBFS_ERR_NOMEM 2   /* not enough free HBM (checked before allocating)      */
#define GBBFS_ERR_CUDA 3    /* a CUDA runtime call failed                            */
#define GBBFS_ERR_TIMEOUT 4 /* a bounded device-side wait gave up                    */
#define GBBFS_ERR_BOUNDS 5  /* a device-side bounds check fired                      */
#define GBBFS_ERR_STATE 6   /* call out of order (e.g. results before a search)      */
#define GBBFS_ERR_IO 7      /* file could not be read or written                     */

/* Step kinds of the per-search trace, in the order the reference prints them
 * with PrintStep (gapbs-verify/bfs.cc:124-165, src/bfs.cc:144-184). */
#define GBBFS_STEP_TD 1 /* "td <next frontier size>"              */
#define GBBFS_STEP_E 2  /* "e"  QueueToBitmap (top-down -> bottom-up) */
#define GBBFS_STEP_BU 3 /* "bu <awake count>"                     */
#define GBBFS_STEP_C 4  /* "c"  BitmapToQueue (bottom-up -> top-down) */

typedef struct gbbfs_step {
  int32_t kind;    /* GBBFS_STEP_*                                          */
  int32_t level;   /* BFS depth the step discovers (0 for e/c)             */
  int64_t count;   /* td: vertices claimed; bu: awake count; e/c: frontier */
  int64_t edges;   /* td: edges examined; bu: in-neighbours scanned (instrumented) */
  int64_t unvisited; /* bu: unvisited vertices at step start (instrumented) */
  double seconds;  /* device time of the step (0 when not measured)        */
} gbbfs_step;

typedef struct gbbfs_stats {
  /* in */
  gbbfs_step* steps;   /* caller array for the trace, may be NULL            */
  int32_t max_steps;   /* its capacity                                        */
  int32_t instrument;  /* 1: count scanned edges and algorithmic bytes (slower) */
  int32_t stepped;     /* 1: host-stepped loop, CUDA events around every step
                          kernel; 0: the whole search as one CUDA graph (step
                          times then come from device timer stamps)         */
  /* out */
  int32_t num_steps;   /* records the search produced (may exceed max_steps) */
  int32_t levels;      /* number of BFS levels discovered                   */
  double device_ms;    /* device time of the whole search, init included     */
  double init_seconds; /* device time of InitParent + frontier set-up ("i") */
  int64_t reached;     /* vertices with a parent (source included)          */
  int64_t alg_bytes;   /* algorithmic bytes of the search (instrument only) */
} gbbfs_stats;

typedef struct gbbfs_graph gbbfs_graph;

/* Upload a CSR graph to HBM.  Replaces the Graph that
 * Builder::MakeGraph returns (src/builder.h:314-338): offsets int64[n+1]
 * (offsets[0] == 0, non-decreasing), neigh int32[m_dir] with
 * m_dir == offsets[n].  The graph must be symmetric (undirected CSR, in-
 * neighbours == out-neighbours, src/graph.h:280-290) as every synthetic graph
 * of the reference is.  The caller keeps the host arrays. */
int gbbfs_graph_create(const int64_t* offsets, const int32_t* neigh, int64_t n,
                       int64_t m_dir, gbbfs_graph** out);

/* Builder::MakeGraph's CSR construction on the GPU (gapbs-verify/builder.h:
 * 73-206: count degrees, prefix sum, scatter both directions, per-row sort,
 * de-duplicate, drop self-loops): el_pairs holds `edges` (u, v) int32 pairs in
 * host or device memory, num_nodes < 0 takes the largest id + 1.  The CSR is
 * built in HBM (a radix sort of the directed edges) and becomes the handle's
 * graph; it equals gbbfs_build_csr's byte for byte.  No host CSR is made. */
int gbbfs_graph_create_from_edges(const int32_t* el_pairs, int64_t edges, int64_t num_nodes,
                                  gbbfs_graph** out);

/* Copy a handle's CSR to host memory: offsets int64[n+1] and neighbours
 * int32[m_dir] (either may be NULL). */
int gbbfs_graph_csr(const gbbfs_graph* g, int64_t* offsets_out, int32_t* neigh_out);

/* Free the device copy (the graph's destructor, src/graph.h). */
int gbbfs_graph_destroy(gbbfs_graph* g);

/* n, m_dir and the bytes this handle holds on the device. */
int gbbfs_graph_info(const gbbfs_graph* g, int64_t* n, int64_t* m_dir,
                     int64_t* device_bytes);

/* One direction-optimizing BFS from `source`: the kernel functor
 * DOBFS(g, source, alpha, beta) (src/bfs.cc:142-188,
 * gapbs-verify/bfs.cc:122-173).  alpha/beta <= 0 select the reference
 * defaults 15 and 18.  parent_out (host, n entries, may be NULL) receives the
 * BFS tree in the reference's output encoding: parent[source] == source,
 * -1 for unreached vertices (src/bfs.cc:224-228).  depth_out (host, may be
 * NULL) receives the BFS depth, -1 when unreached.  st (may be NULL) receives
 * the step trace and timings. */
int gbbfs_bfs(gbbfs_graph* g, int32_t source, int alpha, int beta,
              int32_t* parent_out, int32_t* depth_out, gbbfs_stats* st);

/* The benchmark's trial loop over sources (src/benchmark.h:126-131, one
 * DOBFS per trial) as one call: searches from sources[0..k) run back to
 * back, and search i's parent array goes to parent_out[i] (host, n entries;
 * pinned memory makes the copy asynchronous).  The searches alternate
 * between two parent arrays in HBM, and each is copied out on a second
 * stream while the next search runs.  Pointers may repeat: copies land in
 * source order, so the last one wins.  st may be NULL or hold k entries.
 * Allocates those two parent arrays on first use. */
int gbbfs_bfs_many(gbbfs_graph* g, const int32_t* sources, int64_t k, int alpha, int beta,
                   int32_t* const* parent_out, gbbfs_stats* st);

/* The same search with its results left in HBM (no device->host copy); read
 * them with gbbfs_results.  want_depth != 0 also maintains the depth array. */
int gbbfs_bfs_device(gbbfs_graph* g, int32_t source, int alpha, int beta,
                     int want_depth, gbbfs_stats* st);

/* The same search for callers that cannot allocate device memory when they
 * need it: plugins inside a framework whose own allocator owns the device
 * (memory taken behind its back is memory it cannot account for), and loops
 * that cannot afford the synchronisation cudaMalloc / cudaFree may cause.  No
 * counterpart in the reference.  Everything is caller-owned device memory:
 * d_offsets int64[n+1], d_neigh int32[m_dir] (symmetric CSR), d_parent_out
 * int32[n] (same encoding as gbbfs_bfs), d_depth_out int32[n] or NULL; stream
 * is a cudaStream_t (NULL = the default stream) and the call returns when the
 * results are in place.  Intermediates live in one fixed device array that
 * is part of the library (about 8.2 MB, held on every GPU that loads the
 * library until exit), so graphs are limited to n <= 262144 vertices
 * (GBBFS_ERR_ARG beyond).  Nothing is allocated, by this call or the
 * library.  The first call on a device looks up that array's address (and
 * the kernels' launch grids) once.  All calls share the array: calls that
 * overlap on the GPU race and must be serialised by the caller.  The search
 * is stepped from the host, with a stream synchronisation after every step,
 * so the stream must not be one that is being captured into a CUDA graph
 * (GBBFS_ERR_STATE, the stream untouched). */
int gbbfs_bfs_noalloc(const int64_t* d_offsets, const int32_t* d_neigh, int64_t n,
                      int64_t m_dir, int32_t source, int alpha, int beta,
                      int32_t* d_parent_out, int32_t* d_depth_out, void* stream);

/* Copy the results of the last search to the host (either may be NULL). */
int gbbfs_results(gbbfs_graph* g, int32_t* parent_out, int32_t* depth_out);

/* Device pointers of the last search's results (valid until the next call
 * on the handle).  *depth is NULL if the search did not keep depths. */
int gbbfs_result_device_ptrs(gbbfs_graph* g, const int32_t** parent,
                             const int32_t** depth);

/* BC's BFS phase from `source` (src/bc.cc:55-102; gapbs-verify/bc.cc:51-92):
 * a level-synchronous BFS over every edge of each level.  Host outputs, each
 * may be NULL:
 *   path_counts uint64[n]  shortest paths from the source (the reference's
 *                          unsigned long long adds, so modulo 2^64); 0 when
 *                          unreached
 *   depth       int32[n]   -1 when unreached
 *   succ        uint32[(m_dir+31)/32]  bit e%32 of word e/32 set when the
 *                          directed edge at CSR position e leads one level
 *                          down (the successor bitmap)
 *   order       int32[n]   the reached vertices level by level (the order
 *                          inside a level is not specified)
 *   level_start int64[n+1] level d is order[level_start[d] .. level_start[d+1])
 * *levels (may be NULL) receives the number of levels, the source's being 0. */
int gbbfs_bc_bfs(gbbfs_graph* g, int32_t source, uint64_t* path_counts, int32_t* depth,
                 uint32_t* succ, int32_t* order, int64_t* level_start, int32_t* levels);

/* Approximate betweenness centrality, Brandes' algorithm over k sources
 * (src/bc.cc:106-171): for each source the BFS phase above, then the
 * dependencies from the deepest level up (delta[u] = sum over successor
 * edges of path_counts[u] / path_counts[v] * (1 + delta[v])) added to the
 * scores.  scores_out (host, n floats) receives the scores divided by their
 * maximum, as the reference returns them.  Float sums run in another order
 * than the reference's, so scores agree to the tolerance its verifier uses
 * (1e-6 on the normalized scores), not bit for bit. */
int gbbfs_bc(gbbfs_graph* g, const int32_t* sources, int64_t k, float* scores_out);

/* ---- Batched multi-source BFS (no reference counterpart) ----
 * Many sources of one graph at once, 32, 64, 128 or 256 per batch as a bitmask per
 * vertex, in one persistent kernel per batch captured in a CUDA graph.  Its
 * results are defined by the single-source search above: depth[s][v] equals
 * the depth gbbfs_bfs (and the reference's DOBFS, src/bfs.cc:142-188) gives v
 * from sources[s]. */
typedef struct gbbfs_ms_config {
  int32_t lanes;  /* sources per batch: 32, 64, 128 or 256               */
  int32_t batch;  /* neighbours one thread reads per bottom-up round: 4, 8, 16 */
  int32_t alpha;  /* a level runs top-down while its frontier's summed degree
                     is <= m_dir / alpha, bottom-up above                 */
} gbbfs_ms_config;

typedef struct gbbfs_ms_stats {
  double device_ms;  /* device time of all batches                       */
  int32_t batches;
  int32_t levels;    /* deepest level of any batch                       */
  int32_t lanes, batch, alpha;  /* configuration used                     */
  int32_t td_levels, bu_levels; /* levels run top-down / bottom-up (all batches) */
  int32_t pad;
  double td_ms, bu_ms;          /* device time spent in them            */
  /* share of warp time per kernel phase: top-down expansion, bottom-up
   * small-vertex stream, bottom-up per-vertex scans, depth writes and
   * queueing, hub chunks, frontier clear, frontier install, grid barriers */
  double phase_share[8];
  /* per level l (1..31), summed over batches: device time, frontier
   * vertices, their summed degree, and how many batches ran it bottom-up */
  double level_ms[32];
  double level_frontier[32];
  double level_edges[32];
  int32_t level_bu[32];
} gbbfs_ms_stats;

/* BFS depths from k sources.  depth_out (host) receives k rows of n entries,
 * row s for sources[s]: depth_bytes == 1 gives uint8 with 255 = unreached
 * (GBBFS_ERR_ARG if a depth exceeds 254), depth_bytes == 4 gives int32 with
 * -1 = unreached.  Batches run back to back; the copy of one batch overlaps
 * the next batch's search (pinned depth_out makes the copy asynchronous).
 * More sources than one batch holds are batched in gbbfs_msbfs_order's
 * order; rows still land at their sources' positions. */
int gbbfs_msbfs(gbbfs_graph* g, const int32_t* sources, int64_t k, int depth_bytes,
                void* depth_out, gbbfs_ms_stats* st);

/* One batch (k <= lanes) with the depths left in HBM; *depth_dev points at
 * its k x n rows (valid until the next batched call on the handle). */
int gbbfs_msbfs_device(gbbfs_graph* g, const int32_t* sources, int64_t k, int depth_bytes,
                       const void** depth_dev, gbbfs_ms_stats* st);

/* The order to batch sources[0..k) in: order_out[j] (k entries) is the index
 * of the j-th source to run.  A batch costs about as many full bottom-up
 * levels as its slowest source needs, so sources that reach the bulk of the
 * graph at the same level are put together: sorted (stably) by BFS depth
 * from the highest-degree vertex (lowest id among ties), then by the sum of
 * the source's neighbours' degrees, highest first, in quarter-octave steps
 * (over the first 256 neighbours, scaled, for larger degrees).  The first call on a handle runs
 * that one search (replacing the handle's last single-source result) and
 * keeps two bytes per vertex on the host. */
int gbbfs_msbfs_order(gbbfs_graph* g, const int32_t* sources, int64_t k, int32_t* order_out);

/* HBM (bytes) the batched search state of a graph with n vertices and m_dir
 * directed edges takes: the figure the query server admits graphs against. */
int64_t gbbfs_msbfs_state_bytes(int64_t n, int64_t m_dir, int depth_bytes);

/* Choose or read the batched configuration. */
int gbbfs_msbfs_set_config(gbbfs_graph* g, const gbbfs_ms_config* cfg);
int gbbfs_msbfs_get_config(const gbbfs_graph* g, gbbfs_ms_config* cfg);

/* Autotuner: time every configuration of the built-in grid (lanes x batch x
 * alpha) on the given sample sources (up to 512 of them, in whole batches
 * of each width), keep the fastest per query on the handle and return it in
 * *best. */
int gbbfs_msbfs_autotune(gbbfs_graph* g, const int32_t* sample, int64_t k, int depth_bytes,
                         gbbfs_ms_config* best);

/* ---- Query server (no reference counterpart) ----
 * (graph, source) queries answered as they arrive.  A host thread batches
 * the pending queries of each resident graph into the lanes of the
 * multi-source search: whenever one of a graph's two batch buffers is free,
 * up to max_batch queued queries of that graph launch together, so queries
 * that arrive while a batch runs join the next one, and batches of different
 * graphs overlap on the device.  Per-graph search state is admitted against
 * free HBM (and the optional budget); an idle graph's state is released when
 * another graph needs the room.  Results carry timestamps for latency and a
 * digest of the depth row; the row itself is copied out when the query gives
 * a host buffer.  The server drives the graph handles it is given until it
 * is closed: do not call other functions on them meanwhile. */
typedef struct gbbfs_server gbbfs_server;

typedef struct gbbfs_server_config {
  int32_t mode;              /* 0: batched multi-source; 1: one plain search per query */
  int32_t max_batch;         /* queries per batch, <= lanes (default 256)        */
  int64_t hbm_budget_bytes;  /* cap on per-graph search state, 0 = none          */
  int64_t hbm_reserve_bytes; /* free HBM to leave untouched                      */
  int32_t order;             /* 0: when more queries of a graph wait than a batch
                                holds, batch those with close batching keys
                                (gbbfs_msbfs_order) around the oldest; 1: strict
                                arrival order                                   */
  int32_t batches_only;      /* mode 0: 0 lets a launch of k queries run as k
                                plain searches when the graph's measured costs
                                say they take less than one batch; 1: always a
                                batch                                           */
  int32_t grid_policy;       /* mode 0: 0 every batch spans the whole GPU (the
                                graphs' batches take turns); 1 the SMs are split
                                among the admitted graphs (16 kept for the small
                                kernels around batches, at least 8 per graph,
                                the rest by the square root of each graph's
                                measured batch cost), so the batches of
                                different graphs run side by side          */
  int32_t max_inflight;      /* batches of one graph on the GPU at once: 1 or 2
                                (0 = 1)                                       */
  int32_t priorities;        /* 0: all graph streams equal; 1: CUDA stream
                                priorities by measured batch cost, the cheapest
                                graph first (under load the costliest graphs
                                can starve: measured, not the default)       */
} gbbfs_server_config;

typedef struct gbbfs_result {
  uint64_t ticket;
  int32_t graph_id;
  int32_t source;
  int32_t status;      /* GBBFS_OK or the error that ended the query             */
  int32_t batch_size;  /* queries in the batch that answered it                  */
  double submit_s, start_s, done_s;  /* server clock (gbbfs_server_clock)       */
  /* digest of the uint8 depth row d (255 = unreached):
   * sum over v of (d[v] + 1) * ((v + 1) * 0x9E3779B97F4A7C15), mod 2^64 */
  uint64_t checksum;
  int64_t reached;     /* vertices with a depth                                  */
  int32_t max_depth;
  int32_t plain;       /* 1 if a plain single-source search answered it          */
  /* device clock (%globaltimer, ns) at the start and end of the batch search
   * kernel that answered it; 0 for a plain search */
  uint64_t device_begin_ns, device_end_ns;
} gbbfs_result;

int gbbfs_server_open(const gbbfs_server_config* cfg, gbbfs_server** out);
int gbbfs_server_add_graph(gbbfs_server* s, gbbfs_graph* g, int32_t* graph_id);
/* depth_out: host buffer of n bytes for the uint8 depth row, or NULL. */
int gbbfs_server_submit(gbbfs_server* s, int32_t graph_id, int32_t source, uint8_t* depth_out,
                        uint64_t* ticket);
/* count queries at once (a burst a front end received together): they are
 * queued under one lock, so the batcher sees all of them before it fills
 * lanes.  depth_out may be NULL, or hold count entries (each NULL or n
 * bytes).  tickets (may be NULL) receives count tickets, in order. */
int gbbfs_server_submit_many(gbbfs_server* s, int64_t count, const int32_t* graph_ids,
                             const int32_t* sources, uint8_t* const* depth_out,
                             uint64_t* tickets);
/* Up to max finished results; waits up to wait_us for the first one. */
int gbbfs_server_poll(gbbfs_server* s, gbbfs_result* out, int32_t max, int32_t* count,
                      int32_t wait_us);
/* Wait until every submitted query has a result (GBBFS_ERR_TIMEOUT otherwise). */
int gbbfs_server_drain(gbbfs_server* s, int32_t timeout_ms);
/* Seconds since the server was opened (the clock of the result timestamps). */
double gbbfs_server_clock(const gbbfs_server* s);
int gbbfs_server_close(gbbfs_server* s);

/* Human-readable name of a status code. */
const char* gbbfs_strerror(int status);

/* Detail of the last failure on the calling thread ("" if none). */
const char* gbbfs_last_error(void);

/* ---- Host side of the path (C++ inside the library, no GPU needed) ---- */

/* Build the symmetrized synthetic graph the reference builds for -g/-u
 * <scale> -k <degree>: Generator::GenerateEL (gapbs-verify/generator.h:54-130,
 * src/generator.h:66-167) then Builder::MakeGraphFromEL + SquishGraph
 * (gapbs-verify/builder.h:191-252).  Bit-identical to the reference on the
 * same libstdc++.  *offsets_out / *neigh_out are allocated with malloc; free
 * them with gbbfs_free_host. */
int gbbfs_generate(int scale, int degree, int uniform, int64_t** offsets_out,
                   int32_t** neigh_out, int64_t* n_out, int64_t* m_dir_out);

void gbbfs_free_host(void* p);

/* The two halves of gbbfs_generate.  gbbfs_generate_edges returns the raw
 * edge list (2 int32 per edge: u, v) of Generator::GenerateEL; gbbfs_build_csr
 * turns any edge list into the symmetrized, squished CSR of
 * Builder::MakeGraphFromEL + SquishGraph.  num_nodes < 0 means "largest id +
 * 1" (gapbs-verify/builder.h:213-214). */
int gbbfs_generate_edges(int scale, int degree, int uniform, int32_t** el_out,
                         int64_t* edges_out);
int gbbfs_build_csr(int32_t* el_pairs, int64_t edges, int64_t num_nodes,
                    int64_t** offsets_out, int32_t** neigh_out, int64_t* n_out,
                    int64_t* m_dir_out);

/* Read a graph file the way Builder::MakeGraph does for -f
 * (src/reader.h:57-257, :291-345): ".sg" serialized graphs (undirected only),
 * ".el" / ".wel" edge lists ("u v [w]" per line, weights ignored) and DIMACS
 * ".gr" ("a u v w" lines, 1-based ids), METIS ".graph" files (one line of
 * 1-based neighbours per vertex, gapbs-verify/reader.h:88-140; undirected by
 * the format) and Matrix Market ".mtx" coordinate files (src/reader.h:186-256;
 * 1-based, values ignored).  Edge lists must be symmetrized (symmetrize != 0,
 * the -s flag) unless the file says it is symmetric: this engine runs on
 * undirected CSR only.  Weighted serialized graphs (".wsg") are refused with
 * GBBFS_ERR_ARG, as the reference's BFS refuses them (its Reader checks that
 * a serialized file's weightedness matches the graph type,
 * gapbs-verify/reader.h:254-267). */
int gbbfs_read_graph(const char* path, int symmetrize, int64_t** offsets_out,
                     int32_t** neigh_out, int64_t* n_out, int64_t* m_dir_out);

/* Write an undirected CSR as a ".sg" serialized graph (src/writer.h:39-69):
 * bool directed, int64 num_edges_directed, int64 num_nodes, int64
 * offsets[n+1], int32 neigh[m]. */
int gbbfs_write_sg(const char* path, const int64_t* offsets, const int32_t* neigh,
                   int64_t n, int64_t m_dir);

/* SourcePicker::PickNext repeated `count` times (src/benchmark.h:49-88,
 * gapbs-verify/benchmark.h:46-68): mt19937(27491095), uniform over [0, n-1],
 * skipping out-degree-0 vertices; given != -1 (the -r flag) repeats it. */
int gbbfs_pick_sources(const int64_t* offsets, int64_t n, int64_t given,
                       int count, int32_t* out);

/* Append one trial to a bfs_output.txt-format file: n lines, one decimal
 * parent per line, -1 for every parent < 0 (BFSVerifier writer,
 * src/bfs.cc:213-235). */
int gbbfs_append_bfs_output(const char* path, const int32_t* parent, int64_t n);

#ifdef __cplusplus
}
#endif

#endif /* GBBFS_H_ */
