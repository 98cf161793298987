/*
 * gtc.h -- C ABI of libgtc, a GB300 (sm_103a) implementation of
 * graph-tool-rs's centrality power iteration.
 *
 * The entry points replace, one for one, the Rust functions of the reference
 * project's gt-algo crate (paths below are inside that project):
 *
 *   gtc_pagerank     pagerank / pagerank_with    crates/gt-algo/src/centrality.rs:234-248, 261-384
 *   gtc_eigenvector  eigenvector                 crates/gt-algo/src/centrality.rs:405-497
 *
 * and, around that path:
 *
 *   gtc_betweenness      betweenness                crates/gt-algo/src/centrality.rs:633-689
 *   gtc_weighted_degree  weighted_out/in_degree     crates/gt-algo/src/degree.rs:122-160
 *   gtc_gt_*             gt_io::gt::read            crates/gt-io/src/gt.rs:555-820
 *   gtc_ppr_batch, gtc_graph_batch_*, gtc_pagerank_batch, gtc_pagerank_adjoint,
 *   gtc_pagerank_noalloc (no counterparts: batched, many-graph, gradient and
 *   allocation-free forms of pagerank)
 *
 * and the graph they run over is the reference's adjacency storage,
 * crates/gt-core/src/adj/list.rs:67-79 (AdjList) with its per-vertex blocks
 * crates/gt-core/src/adj/block.rs:54-57: a handle built by replaying
 * AdjList::add_edge (list.rs:258-280) over an edge list reproduces every
 * block's out-half and in-half order exactly, so the pull visits in-edges in
 * the order the reference's `in_edges` yields them (crates/gt-core/src/graph.rs:228-237,
 * crates/gt-core/src/adj/list.rs:156-161).
 *
 * Conventions
 *   - Every function returns a gtc_status; on failure gtc_last_error() holds
 *     a message for the calling thread.  Nothing aborts the process.  Error
 *     classes follow the reference's Python boundary
 *     (crates/gt-py/src/module.rs:78-114): GTC_ERR_ARG -> ValueError,
 *     GTC_ERR_INDEX -> IndexError, the rest -> RuntimeError/MemoryError.
 *   - Vertex and edge indices are uint32 (the reference's Raw = u32,
 *     crates/gt-core/src/ids.rs:25-32).
 *   - "Host" pointers are ordinary CPU memory; they may be pageable or
 *     pinned.  Calls are synchronous with respect to host buffers.
 *   - A handle is not thread-safe; use one handle per thread or lock.
 *   - A handle keeps what its graph alone determines, built by the first
 *     call that needs it: the FP32 sweep schedules of the plain and reversed
 *     views, their unweighted degrees, sink flags and FP32 inverse degrees
 *     (13 bytes per vertex and view), and, for the last weight map an FP32
 *     call used (same address, type and contents), that map's FP32 layouts
 *     and weighted degrees.  A filtered view builds its own per call.
 *   - No entry point falls back to the CPU: without a usable CUDA device
 *     they return GTC_ERR_NO_DEVICE.
 */
#ifndef GTC_H
#define GTC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum gtc_status {
    GTC_OK = 0,
    GTC_ERR_ARG = 1,       /* invalid argument (ValueError)                       */
    GTC_ERR_OOM = 2,       /* device or host allocation failed (MemoryError)      */
    GTC_ERR_CUDA = 3,      /* a CUDA call failed (RuntimeError)                   */
    GTC_ERR_TIMEOUT = 4,   /* a bounded device-side wait gave up (RuntimeError)   */
    GTC_ERR_INDEX = 5,     /* an index outside its bound (IndexError)             */
    GTC_ERR_NO_DEVICE = 6  /* no CUDA device is usable (RuntimeError)             */
} gtc_status;

/* Arithmetic of a solve.
 *   GTC_PREC_F32        FP32 vectors and edge weights, compensated FP32 row
 *                       sums, FP64 dangling mass, L1 delta and
 *                       normalisation (the fast path).
 *   GTC_PREC_F64_EXACT  FP64 throughout with the reference's evaluation and
 *                       fold order (per-edge divide, Plan-chunk folds): the
 *                       result and the sweep count are bit-identical to the
 *                       reference's for the same Plan. */
typedef enum gtc_precision { GTC_PREC_F32 = 0, GTC_PREC_F64_EXACT = 1 } gtc_precision;

typedef struct gtc_graph gtc_graph;

/* PowerIteration, crates/gt-algo/src/centrality.rs:79-99.
 *   plan_len    must equal the vertex bound (else GTC_ERR_ARG with the
 *               reference's panic message "sweep: the plan must cover the
 *               output exactly", centrality.rs:145-149)
 *   plan_chunks Plan::chunks() of the caller's Plan (plan.rs:55-61); it fixes
 *               the FP64 fold order of GTC_PREC_F64_EXACT.  0 means
 *               Plan::new(plan_len, 4096). */
typedef struct gtc_power_iteration {
    double epsilon;       /* L1 change below which the sweeps stop          */
    uint64_t max_iter;    /* hard cap on sweeps; 0 = no cap                 */
    uint64_t plan_len;
    uint64_t plan_chunks;
} gtc_power_iteration;

/* The directed view a solve runs on (dispatch_bidi,
 * crates/gt-py/src/dispatch.rs:315-339): the graph, its reversal (Rev,
 * crates/gt-core/src/view/reversed.rs:109-138), and either of them filtered
 * by two host uint8 masks (Filtered with MaskFilter,
 * crates/gt-core/src/view/filtered.rs:299-319): non-zero keeps.  An incident
 * edge survives iff its edge and its other endpoint survive.  A NULL view
 * pointer is the unfiltered graph. */
typedef struct gtc_view {
    int32_t reversed;
    int32_t reserved;
    const uint8_t* vmask;  /* NULL or length == vertex bound */
    uint64_t vmask_len;
    const uint8_t* emask;  /* NULL or length == edge bound   */
    uint64_t emask_len;
} gtc_view;

/* Sweep kernels of the GTC_PREC_F32 PageRank and eigenvector solves.  Every
 * kernel computes the same values (the per-row sums and the reductions do
 * not depend on the schedule), so a choice changes speed only.  AUTO times
 * the candidates on the first solve of a (graph view, mode, weighting) and
 * caches the fastest on the handle. */
typedef enum gtc_schedule {
    GTC_SCHED_AUTO = 0,
    GTC_SCHED_L1 = 1,      /* in-degree tiers, every gather through L1/L2        */
    GTC_SCHED_HOT32K = 2,  /* in-degree tiers, the 32,768 most gathered entries
                              of the gathered vector in shared memory            */
    GTC_SCHED_HOT24K = 3,  /* ... 24,576 entries                                 */
    GTC_SCHED_HOT16K = 4,  /* ... 16,384 entries                                 */
    GTC_SCHED_HOT8K = 5    /* ... 8,192 entries                                  */
} gtc_schedule;

/* Gather kernels of the batched personalised PageRank (gtc_ppr_batch). */
typedef enum gtc_ppr_gather {
    GTC_PPR_BULK = 0,  /* rows of the iterate staged by cp.async.bulk (default) */
    GTC_PPR_REGS = 1   /* rows gathered into registers                         */
} gtc_ppr_gather;

/* Per-call options.  A NULL pointer means all defaults. */
typedef struct gtc_options {
    int32_t precision;   /* gtc_precision, default GTC_PREC_F32                */
    int32_t schedule;    /* gtc_schedule, default GTC_SCHED_AUTO               */
    void* stream;        /* cudaStream_t to run on; NULL = the handle's        */
    int32_t timing;      /* non-zero: time every sweep kernel (sweep_ms)       */
    int32_t ppr_gather;  /* gtc_ppr_gather, default GTC_PPR_BULK               */
} gtc_options;

/* What a solve reports back. */
typedef struct gtc_result {
    uint64_t iterations;   /* sweeps performed (the reference's return)    */
    double last_delta;     /* L1 change of the last sweep                   */
    double eigenvalue;     /* eigenvector only: the last norm (0 if none)   */
    double device_ms;      /* device time from the first to the last sweep  */
    uint64_t launches;     /* kernels launched by this call                 */
    double sweep_ms;       /* with opt->timing: summed sweep-kernel time    */
    uint64_t sweep_launches; /* sweep kernels launched (the timed ones)     */
} gtc_result;

/* A vector in device memory (device variants of the entry points). */
typedef enum gtc_dtype { GTC_F64 = 0, GTC_F32 = 1 } gtc_dtype;
typedef struct gtc_dvec {
    void* ptr;        /* device pointer (NULL: absent)                   */
    uint64_t len;     /* elements                                        */
    int32_t dtype;    /* gtc_dtype                                       */
    int32_t reserved;
} gtc_dvec;

/* ---- library ---------------------------------------------------------- */

const char* gtc_version(void);
/* Message of the last failure on the calling thread ("" if none). */
const char* gtc_last_error(void);

/* ---- graphs ----------------------------------------------------------- */

/* Build a graph of n vertices by replaying AdjList::add_edge(src[k], tgt[k])
 * for k = 0..m-1 (crates/gt-core/src/adj/list.rs:258-280): edge k gets
 * EdgeId k (alloc.rs:58-71, no removals), every out-half keeps insertion
 * order and every in-half the push-swap rotation order of
 * crates/gt-core/src/adj/block.rs:171-209.  Host arrays.  Replaces building
 * an AdjList with AdjList::with_vertices + add_edge (or ParBuilder,
 * crates/gt-core/src/adj/builder.rs:143-197, whose merge is the same call
 * sequence). */
int gtc_graph_create(uint64_t n, uint64_t m, const uint32_t* src, const uint32_t* tgt,
                     gtc_graph** out);

/* As gtc_graph_create, with src/tgt in device memory of the current device;
 * `stream` (a cudaStream_t, may be NULL) orders the reads. */
int gtc_graph_create_device(uint64_t n, uint64_t m, const uint32_t* d_src,
                            const uint32_t* d_tgt, void* stream, gtc_graph** out);

/* Build a graph from the reference's adjacency blocks as they are stored,
 * whatever history made them (add_edge, remove_edge with its swap-remove,
 * crates/gt-core/src/adj/block.rs:241-291, edge ids reused from the LIFO free
 * list, crates/gt-core/src/adj/alloc.rs:58-90): the drop-in for a caller
 * holding an AdjList (crates/gt-core/src/adj/list.rs:26-40).  Vertex v's
 * Block (block.rs:54-57) is entries[block_off[v] .. block_off[v+1]), its
 * out-half the first out_len[v] of them and its in-half the rest; an entry
 * is the 8-byte AdjEntry {other, idx} (crates/gt-core/src/adj/entry.rs:39-48)
 * as two uint32, so a concatenation of every Block::all() can be passed as
 * is.  edge_bound is AdjList::edge_bound (list.rs:130); ids below it that no
 * entry uses are removed edges, and weight maps stay indexed by EdgeId up to
 * it.  Every live edge must appear once in its source's out-half and once in
 * its target's in-half (else GTC_ERR_ARG; an index out of range is
 * GTC_ERR_INDEX).  The pull visits every in-half in the given order, so the
 * FP64-exact solves are bit-identical to the reference's on this graph.
 * Host arrays. */
int gtc_graph_create_blocks(uint64_t n, uint64_t edge_bound, const uint64_t* block_off,
                            const uint32_t* out_len, const uint32_t* entries, gtc_graph** out);

int gtc_graph_destroy(gtc_graph* g);

/* Vertex bound, edge bound (AdjList::vertex_bound / edge_bound,
 * crates/gt-core/src/graph.rs:63-67) and live edge count (below the edge
 * bound when ids have holes, gtc_graph_create_blocks). */
int gtc_graph_info(const gtc_graph* g, uint64_t* n, uint64_t* edge_bound, uint64_t* num_edges);

/* Copy the blocks back to host memory: for every vertex its out-half
 * (other, idx) entries (Block::out, block.rs:99-102) and its in-half
 * (Block::inc, block.rs:108-111), in storage order, with n+1 offsets each.
 * Any pointer may be NULL to skip that array. */
int gtc_graph_export(const gtc_graph* g, uint64_t* out_off, uint32_t* out_other,
                     uint32_t* out_idx, uint64_t* in_off, uint32_t* in_other, uint32_t* in_idx);

/* Stream the handle's work is ordered on (a cudaStream_t; NULL restores the
 * handle's own stream). */
int gtc_graph_set_stream(gtc_graph* g, void* stream);

/* ---- the .gt file format -----------------------------------------------
 *
 * Replaces gt_io::gt::read (crates/gt-io/src/gt.rs:555-626, read_adjacency
 * :628-678, read_column :724-820) for graphs headed for the solvers.
 *
 * gtc_gt_open parses the framing of a .gt document held in host memory
 * (bytes[0 .. len), copied into the handle): header, one record per vertex,
 * property table.  Everything a field declares must lie inside the
 * document.  Errors (all GTC_ERR_ARG, the message names the byte offset
 * where one applies): a bad magic or a short head, a version other than 1,
 * truncation anywhere, a vertex or edge count beyond the index space, a
 * property domain above 2, a value-type index above 14, a name or a string
 * value that is not UTF-8.  Vertex indices inside the lists are checked by
 * gtc_gt_graph, on the device.
 *
 * Property kinds are the indices of ValueKind::ALL
 * (crates/gt-core/src/prop/value.rs:79-95): 0 bool, 1 int16, 2 int32,
 * 3 int64, 4 double, 5 long double, 6 string, 7-13 the vector kinds,
 * 14 python object.  Domains: 0 graph (1 value), 1 vertex (n), 2 edge (m);
 * an edge column's i-th value belongs to edge i (gt.rs:44-58). */
typedef struct gtc_gt_file gtc_gt_file;

int gtc_gt_open(const uint8_t* bytes, uint64_t len, gtc_gt_file** out);
int gtc_gt_close(gtc_gt_file* f);

/* Vertices, edges, the directed flag, the byte-order flag of the document,
 * and the number of properties. */
int gtc_gt_info(const gtc_gt_file* f, uint64_t* n, uint64_t* m, int32_t* directed,
                int32_t* big_endian, uint64_t* nprops);

/* The header comment (valid while the handle lives). */
int gtc_gt_comment(const gtc_gt_file* f, const char** text, uint64_t* len);

/* Property i: name (valid while the handle lives), domain, kind and number
 * of values. */
int gtc_gt_property(const gtc_gt_file* f, uint64_t i, const char** name, uint64_t* name_len,
                    int32_t* domain, int32_t* kind, uint64_t* count);

/* The values of a numeric scalar column (kinds 0-4) as doubles; out_len >=
 * the column's count.  Other kinds are GTC_ERR_ARG. */
int gtc_gt_property_f64(const gtc_gt_file* f, uint64_t i, double* out, uint64_t out_len);

/* The column's bytes exactly as stored (in the document's byte order). */
int gtc_gt_property_bytes(const gtc_gt_file* f, uint64_t i, const uint8_t** data, uint64_t* len);

/* The graph of the document: its lists are decoded on the device and
 * replayed as add_edge(v, u) for every vertex v in order and every entry u of
 * v's list in file order (gt.rs:648-674), so edge k is the document's k-th
 * list entry and every block matches the reference reader's.  An index not
 * below n is GTC_ERR_INDEX, naming the first such index in file order. */
int gtc_gt_graph(const gtc_gt_file* f, gtc_graph** out);

/* ---- centrality ------------------------------------------------------- */

/* PageRank: pagerank (pers == NULL) and pagerank_with (pers != NULL),
 * crates/gt-algo/src/centrality.rs:234-384.
 *
 *   weight     NULL = Unity (deg = out_degree); else f64 by EdgeId, length
 *              >= edge bound (DenseProp<f64, EdgeTag> after sized_for)
 *   pers       NULL = Constant(1/num_vertices of the view); else f64 by
 *              vertex index, length >= vertex bound.  Not normalised.
 *   damping    d in nv = (1-d)*pv + d*r
 *   rank       the caller's vertex map, length rank_len >= vertex bound: the
 *              initial iterate AND the output.  Slots [rank_had, n) are
 *              seeded with pers (seed_new_slots, centrality.rs:198-205), the
 *              slots below rank_had are a warm start (sized_for,
 *              crates/gt-core/src/prop/dense.rs:88-125).
 *   result     iterations = the reference's return value.
 * All arrays are host memory. */
int gtc_pagerank(gtc_graph* g, const gtc_view* view, const double* weight, uint64_t weight_len,
                 const double* pers, uint64_t pers_len, double damping,
                 const gtc_power_iteration* params, double* rank, uint64_t rank_len,
                 uint64_t rank_had, const gtc_options* opt, gtc_result* result);

/* Eigenvector centrality, crates/gt-algo/src/centrality.rs:405-497.
 * x is the initial iterate and the output (slots [x_had, n) seeded with
 * 1/num_vertices); result->eigenvalue is the last norm, 0 if no sweep ran.
 * All arrays are host memory. */
int gtc_eigenvector(gtc_graph* g, const gtc_view* view, const double* weight,
                    uint64_t weight_len, const gtc_power_iteration* params, double* x,
                    uint64_t x_len, uint64_t x_had, const gtc_options* opt, gtc_result* result);

/* weighted_out_degree (in_edges == 0) and weighted_in_degree (in_edges != 0),
 * crates/gt-algo/src/degree.rs:122-160, of every vertex of the view: the
 * FP64 sum of the weight map over the vertex's out-half (in-half) in storage
 * order, as a left fold from 0.0 (sum_weights, degree.rs:68-82), so the
 * result is bit-identical to the reference's; weight == NULL is Unity (the
 * degree).  The degree pass of pagerank (centrality.rs:281-297) is this fold
 * over the out-half.  deg: vertex bound entries, by vertex index; 0 for a
 * vertex outside the view.  Host arrays. */
int gtc_weighted_degree(gtc_graph* g, const gtc_view* view, int32_t in_edges, const double* weight,
                        uint64_t weight_len, double* deg, uint64_t deg_len, const gtc_options* opt);

/* Betweenness centrality (Brandes), crates/gt-algo/src/centrality.rs:633-689:
 * unweighted, every vertex of the view a source, unnormalised.  Both maps are
 * overwritten (init_centrality_map): vertex_bc by vertex index (vertex_len >=
 * vertex bound), edge_bc by EdgeId (edge_len >= edge bound); a vertex or edge
 * outside the view gets 0; either pointer may be NULL to skip that map.
 * undirected != 0 runs on the undirected view (Und,
 * crates/gt-core/src/view/undirected.rs:106-125: every incident edge is an
 * out-edge), whose maps are halved (centrality.rs:680-688).  FP64; path counts
 * are exact below 2^53; sums are associated differently from the reference's
 * (deterministic, within the reference tests' 1e-9 of it).
 * result->iterations = sources run.  Host arrays. */
int gtc_betweenness(gtc_graph* g, const gtc_view* view, int32_t undirected, double* vertex_bc,
                    uint64_t vertex_len, double* edge_bc, uint64_t edge_len,
                    const gtc_options* opt, gtc_result* result);

/* Device variants: the same solves with every vector in device memory of
 * the handle's device (e.g. torch tensors), FP32 or FP64.  NULL or ptr ==
 * NULL means absent (Unity weights / uniform pers).  rank / x must be
 * present.  Nothing is copied to or from the host. */
int gtc_pagerank_device(gtc_graph* g, const gtc_view* view, const gtc_dvec* weight,
                        const gtc_dvec* pers, double damping, const gtc_power_iteration* params,
                        gtc_dvec* rank, uint64_t rank_had, const gtc_options* opt,
                        gtc_result* result);

int gtc_eigenvector_device(gtc_graph* g, const gtc_view* view, const gtc_dvec* weight,
                           const gtc_power_iteration* params, gtc_dvec* x, uint64_t x_had,
                           const gtc_options* opt, gtc_result* result);

/* ---- batched personalised PageRank -------------------------------------
 *
 * B personalised PageRanks over one edge stream (an SpMM over B right-hand
 * sides; the reference calls pagerank_with, centrality.rs:261-384, once per
 * vector).  Vector b's personalisation is its seed set
 * seed_vertices[seed_off[b] .. seed_off[b+1]) with seed_values (NULL:
 * 1/|set| each); each column starts from its personalisation (a fresh map,
 * centrality.rs:198-205) and stops at the first sweep whose L1 change is
 * below params->epsilon (or at max_iter); iters[b] receives its sweep count.
 * ranks is [B][n] (row b = vector b, by vertex index).  1 <= B <= 512.
 * GTC_PREC_F32; plain or reversed views.  Host arrays except as named.
 * The handle keeps two iterate buffers of n x 32 ceil(B / 32) floats between
 * calls (released by gtc_graph_destroy); batched calls on one handle must
 * not overlap. */
int gtc_ppr_batch(gtc_graph* g, const gtc_view* view, const double* weight, uint64_t weight_len,
                  uint32_t B, const uint64_t* seed_off, const uint32_t* seed_vertices,
                  const double* seed_values, double damping, const gtc_power_iteration* params,
                  double* ranks, uint64_t* iters, const gtc_options* opt, gtc_result* result);

/* As gtc_ppr_batch with the weights and the [B][n] ranks in device memory
 * (the seed arrays and iters stay host arrays). */
int gtc_ppr_batch_device(gtc_graph* g, const gtc_view* view, const gtc_dvec* weight, uint32_t B,
                         const uint64_t* seed_off, const uint32_t* seed_vertices,
                         const double* seed_values, double damping,
                         const gtc_power_iteration* params, gtc_dvec* ranks, uint64_t* iters,
                         const gtc_options* opt, gtc_result* result);

/* ---- many graphs in one call --------------------------------------------
 *
 * G graphs packed as one block-diagonal graph (no counterpart in the
 * reference, which solves one graph per call): graph k has n_k = voff[k+1] -
 * voff[k] vertices and the edges eoff[k] .. eoff[k+1]-1 of src/tgt, whose
 * endpoints are LOCAL indices (0 .. n_k - 1), added in array order as
 * add_edge calls of that graph (crates/gt-core/src/adj/list.rs:299-321).
 * voff[0] = eoff[0] = 0; voff[G] and eoff[G] are the totals (voff[G] <=
 * 2^32 - 4096, eoff[G] <= 2^32 - 2).
 * Host arrays. */
typedef struct gtc_graph_batch gtc_graph_batch;

int gtc_graph_batch_create(uint64_t G, const uint64_t* voff, const uint64_t* eoff,
                           const uint32_t* src, const uint32_t* tgt, gtc_graph_batch** out);
int gtc_graph_batch_destroy(gtc_graph_batch* b);
int gtc_graph_batch_info(const gtc_graph_batch* b, uint64_t* graphs, uint64_t* vertices,
                         uint64_t* edges);

/* pagerank (centrality.rs:234-248) of every graph of the batch: uniform
 * personalisation 1/n_k, each graph with its own dangling mass, L1 change and
 * stop (the first sweep whose change is below epsilon, or max_iter; 0 =
 * uncapped).  weight: per edge of the packed edge list (NULL = Unity);
 * rank: per vertex of the packed vertex list (out, fresh start); iters[k]:
 * sweeps of graph k.  GTC_PREC_F32.  Persistent kernels solve all graphs,
 * largest first: a cluster of two CTAs per graph of up to 114,688 vertices
 * (its gathered vector in shared memory), one CTA per larger graph; the
 * launches of a solve are captured into a CUDA graph and replayed while the
 * arrays keep their addresses.  The device loop is bounded: max_iter 0 with
 * epsilon <= 0 is GTC_ERR_ARG; a graph whose L1 change is not finite stops
 * at once (GTC_ERR_ARG after the call); an uncapped graph still running
 * after 100,000 sweeps stops there (GTC_ERR_TIMEOUT).  In both error cases
 * rank and iters are still written.  Host arrays. */
int gtc_pagerank_batch(gtc_graph_batch* b, const double* weight, uint64_t weight_len,
                       double damping, double epsilon, uint64_t max_iter, double* rank,
                       uint64_t rank_len, uint64_t* iters, const gtc_options* opt,
                       gtc_result* result);

/* Test hook: the number of sweeps after which an uncapped batch solve
 * (max_iter 0) gives up with GTC_ERR_TIMEOUT (0 restores the default,
 * 100,000).  It lets a test reach the timeout path in a few sweeps.
 * Process-wide; not for use while batch solves run. */
int gtc_debug_set_batch_sweep_limit(uint64_t limit);

/* As gtc_pagerank_batch with weight and rank in device memory (FP32 or
 * FP64); iters stays a host array. */
int gtc_pagerank_batch_device(gtc_graph_batch* b, const gtc_dvec* weight, double damping,
                              double epsilon, uint64_t max_iter, gtc_dvec* rank, uint64_t* iters,
                              const gtc_options* opt, gtc_result* result);

/* ---- gradients ---------------------------------------------------------
 *
 * The adjoint of PageRank (no counterpart in the reference, which has no
 * differentiation): for a scalar L(pi) of the converged PageRank pi, with
 * grad_pi = dL/dpi, solve lambda = grad_pi + d (A^T lambda + s (p . lambda))
 * (A^T pulled over the out-halves, s the dangling vertices) until the L1 norm
 * of the fixed-point residual is below epsilon * |grad_pi|_1 (the iterate is
 * kept on the exact constraint p . lambda = (pi . grad_pi) / (1 - d), which
 * removes the slowest error mode), then
 *   grad_pers[v]   = lambda_v ((1-d) + d (s . pi))
 *   grad_weight[e] = d (pi_s / deg_s) (lambda_t - (A^T lambda)_s)   e: s -> t
 * (0 for edges out of a vertex of zero weighted degree).  Only the converged
 * pi is used (implicit-function theorem): no iterate history is kept.
 * weight / pers / damping are the forward solve's (NULL = Unity / uniform).
 * GTC_PREC_F32 only; plain or reversed views.  grad_weight (edge bound) and
 * grad_pers (vertex bound) may be NULL to skip them. */
int gtc_pagerank_adjoint(gtc_graph* g, const gtc_view* view, const double* weight,
                         uint64_t weight_len, const double* pers, uint64_t pers_len, double damping,
                         const gtc_power_iteration* params, const double* pi, const double* grad_pi,
                         double* grad_weight, double* grad_pers, const gtc_options* opt,
                         gtc_result* result);

/* As gtc_pagerank_adjoint with every vector in device memory (FP32 or FP64). */
int gtc_pagerank_adjoint_device(gtc_graph* g, const gtc_view* view, const gtc_dvec* weight,
                                const gtc_dvec* pers, double damping,
                                const gtc_power_iteration* params, const gtc_dvec* pi,
                                const gtc_dvec* grad_pi, gtc_dvec* grad_weight, gtc_dvec* grad_pers,
                                const gtc_options* opt, gtc_result* result);

/* ---- PageRank without any allocation ------------------------------------
 *
 * No counterpart in the reference: an addition for callers that cannot
 * allocate device memory when they run PageRank (a runtime that reserved all
 * GPU memory up front and forbids later allocations, or a code path where an
 * allocation would stall or fail).  It calls no cudaMalloc, cudaFree or any
 * other allocating routine: the caller passes the graph and the output, and
 * every intermediate vector lives in one static device array compiled into
 * the library (about 12.6 MB, held by every GPU that loads the library until
 * the process exits).
 *
 *   n             vertices, at most 1,048,576 (larger n is GTC_ERR_ARG)
 *   d_off, d_src  the pull adjacency in device memory: the in-edges of v are
 *                 d_src[d_off[v] .. d_off[v+1]) (sources < n), the order the
 *                 reference's in_edges yields (gtc_graph_export's in-halves)
 *   d_out_degree  out-degree of every vertex (device, n entries)
 *   d_rank        output, device, n floats: PageRank from the uniform start
 *                 (pagerank with a Unity weight, centrality.rs:234-248)
 *   stream        a cudaStream_t (NULL = the legacy default stream)
 *
 * FP32 vectors, compensated row sums, FP64 delta and dangling mass.  There
 * is one static array per GPU and every call on that GPU shares it; it keeps
 * the last call's contents (each call clears what must start at zero), and
 * calls that overlap on the GPU (two streams, two host threads) race on it.
 * max_iter = 0 with epsilon <= 0 would never stop and is GTC_ERR_ARG.
 * The first call on a device does a one-time set-up: it looks the array's
 * device address up (cudaGetSymbolAddress with that device current).  Make
 * that first call before any stream capture.  The call is blocking: after
 * every sweep it waits for the stream to read the L1 change on the host,
 * and it returns when the result is in d_rank. */
int gtc_pagerank_noalloc(uint64_t n, const uint32_t* d_off, const uint32_t* d_src,
                         const uint32_t* d_out_degree, double damping, double epsilon,
                         uint64_t max_iter, float* d_rank, uint64_t* iters_out, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* GTC_H */
