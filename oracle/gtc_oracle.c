/*
 * gtc_oracle.c -- CPU restatement of graph-tool-rs's centrality power
 * iteration, in plain C11 with IEEE-754 binary64 arithmetic.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity checker for the CUDA
 * library and the timed CPU baseline beside it; no product code path links,
 * loads or calls it.  It must be compiled with -ffp-contract=off (no fused
 * multiply-add) so that every product is rounded before it is summed, as the
 * reference's Rust code does.
 *
 * Parity is pinned by the known answers of the reference's own tests
 * (crates/gt-algo/tests/u16_centrality.rs and the push-swap layout test in
 * crates/gt-core/src/adj/block.rs:347-368); the reference itself (Rust) cannot
 * be compiled on this machine.
 *
 * What is restated, and from where (paths are inside the reference project):
 *   - per-vertex adjacency blocks: out-half [0,out_len), in-half [out_len,len)
 *       crates/gt-core/src/adj/block.rs:54-57, 108-111
 *   - Block::insert_out push-swap      crates/gt-core/src/adj/block.rs:171-197
 *   - Block::insert_in append          crates/gt-core/src/adj/block.rs:205-209
 *   - Block::remove_at swap-remove     crates/gt-core/src/adj/block.rs:241-291
 *   - AdjList::add_edge / splice_in    crates/gt-core/src/adj/list.rs:258-280, 471-500
 *   - AdjList::remove_edge/splice_out  crates/gt-core/src/adj/list.rs:287-295, 511-545
 *   - EdgeIds::alloc / release (LIFO)  crates/gt-core/src/adj/alloc.rs:58-90
 *   - Plan::new / Plan::range          crates/gt-core/src/par/plan.rs:55-101
 *   - det_reduce chunk-order fold      crates/gt-core/src/par/reduce.rs:40-55
 *   - sweep chunk-order fold           crates/gt-algo/src/centrality.rs:141-167
 *   - active_mask / grain_of / seeding crates/gt-algo/src/centrality.rs:176-205
 *   - pagerank / pagerank_with         crates/gt-algo/src/centrality.rs:234-384
 *   - eigenvector                      crates/gt-algo/src/centrality.rs:405-497
 *   - Rev view (in <-> out)            crates/gt-core/src/view/reversed.rs:109-138
 *   - Filtered view (masks)            crates/gt-core/src/view/filtered.rs:299-319
 *   - betweenness (Brandes)            crates/gt-algo/src/centrality.rs:499-689
 *   - Und view (out_edges = all_edges)  crates/gt-core/src/view/undirected.rs:106-125,
 *                                      crates/gt-core/src/adj/list.rs:170-175
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORA_OK 0
#define ORA_ERR_ARG (-1)
#define ORA_ERR_OOM (-2)

typedef struct {
    uint32_t other; /* the endpoint that is not the block's owner */
    uint32_t idx;   /* edge id */
} ora_entry;        /* AdjEntry, crates/gt-core/src/adj/entry.rs:39-48 */

typedef struct {
    ora_entry *e;
    uint64_t len, cap, out_len;
} ora_block;

typedef struct {
    uint32_t src, tgt;
    uint64_t out_pos, in_pos; /* block positions (whole-block indexing) */
    int live;
} ora_slot;

typedef struct {
    uint64_t n;
    ora_block *blocks;
    ora_slot *slots;
    uint64_t slots_cap;
    uint64_t next_id; /* edge index bound */
    uint32_t *free_ids;
    uint64_t n_free, free_cap;
    uint64_t live;
} ora_graph;

static const char *g_err = "";
const char *ora_last_error(void) { return g_err; }

/* ------------------------------------------------------------------------ */
/* adjacency storage                                                         */
/* ------------------------------------------------------------------------ */

ora_graph *ora_graph_new(uint64_t n) {
    ora_graph *g = (ora_graph *)calloc(1, sizeof(ora_graph));
    if (!g) return NULL;
    g->n = n;
    g->blocks = (ora_block *)calloc(n ? n : 1, sizeof(ora_block));
    if (!g->blocks) {
        free(g);
        return NULL;
    }
    return g;
}

void ora_graph_free(ora_graph *g) {
    if (!g) return;
    for (uint64_t v = 0; v < g->n; ++v) free(g->blocks[v].e);
    free(g->blocks);
    free(g->slots);
    free(g->free_ids);
    free(g);
}

uint64_t ora_num_vertices(const ora_graph *g) { return g->n; }
uint64_t ora_edge_bound(const ora_graph *g) { return g->next_id; }
uint64_t ora_num_edges(const ora_graph *g) { return g->live; }

static int block_push(ora_block *b, ora_entry x) {
    if (b->len == b->cap) {
        uint64_t nc = b->cap ? 2 * b->cap : 4;
        ora_entry *ne = (ora_entry *)realloc(b->e, nc * sizeof(ora_entry));
        if (!ne) return ORA_ERR_OOM;
        b->e = ne;
        b->cap = nc;
    }
    b->e[b->len++] = x;
    return ORA_OK;
}

/* A notification that entry `id` now sits at block position `to`. */
static void on_move(ora_graph *g, uint32_t id, int in_half, uint64_t to) {
    if (in_half)
        g->slots[id].in_pos = to;
    else
        g->slots[id].out_pos = to;
}

/* Block::insert_out, block.rs:171-197: when the in-half is non-empty, its
 * FIRST entry moves to the back and the new out-entry takes its slot. */
static int insert_out(ora_graph *g, ora_block *b, ora_entry x, uint64_t *pos) {
    uint64_t at = b->out_len;
    if (at < b->len) {
        ora_entry displaced = b->e[at];
        if (block_push(b, displaced)) return ORA_ERR_OOM;
        b->e[at] = x;
        on_move(g, displaced.idx, 1, b->len - 1);
    } else {
        if (block_push(b, x)) return ORA_ERR_OOM;
    }
    b->out_len = at + 1;
    *pos = at;
    return ORA_OK;
}

/* Block::insert_in, block.rs:205-209: plain append. */
static int insert_in(ora_block *b, ora_entry x, uint64_t *pos) {
    *pos = b->len;
    return block_push(b, x);
}

/* EdgeIds::alloc, alloc.rs:58-71: LIFO off the free list, else next++. */
static int64_t alloc_id(ora_graph *g) {
    uint32_t id;
    if (g->n_free) {
        id = g->free_ids[--g->n_free];
    } else {
        if (g->next_id >= 0xFFFFFFFEull) return ORA_ERR_ARG; /* MAX_INDEX, ids.rs:32 */
        if (g->next_id == g->slots_cap) {
            uint64_t nc = g->slots_cap ? 2 * g->slots_cap : 16;
            ora_slot *ns = (ora_slot *)realloc(g->slots, nc * sizeof(ora_slot));
            if (!ns) return ORA_ERR_OOM;
            g->slots = ns;
            g->slots_cap = nc;
        }
        id = (uint32_t)g->next_id++;
    }
    g->live++;
    return (int64_t)id;
}

/* AdjList::add_edge + splice_in, list.rs:258-280 and 471-500.  The out
 * splice (which can move an in-entry of the same block, including the loop's
 * own block for a self-loop) happens before the in splice. */
int64_t ora_add_edge(ora_graph *g, uint64_t s, uint64_t t) {
    if (s >= g->n || t >= g->n) {
        g_err = "add_edge: no such vertex";
        return ORA_ERR_ARG;
    }
    int64_t id = alloc_id(g);
    if (id < 0) {
        g_err = "add_edge: edge id space exhausted or out of memory";
        return id;
    }
    ora_slot *sl = &g->slots[id];
    sl->src = (uint32_t)s;
    sl->tgt = (uint32_t)t;
    sl->live = 1;
    uint64_t op, ip;
    ora_entry eo = {(uint32_t)t, (uint32_t)id};
    ora_entry ei = {(uint32_t)s, (uint32_t)id};
    if (insert_out(g, &g->blocks[s], eo, &op)) return ORA_ERR_OOM;
    if (insert_in(&g->blocks[t], ei, &ip)) return ORA_ERR_OOM;
    g->slots[id].out_pos = op;
    g->slots[id].in_pos = ip;
    return id;
}

/* Block::remove_at, block.rs:241-291. */
static void remove_at(ora_graph *g, ora_block *b, uint64_t i, int in_half) {
    uint64_t n = b->len, split = b->out_len;
    if (!in_half) {
        if (i != split - 1) {
            ora_entry back = b->e[split - 1];
            b->e[i] = back;
            on_move(g, back.idx, 0, i);
        }
        if (n > split) {
            ora_entry last = b->e[n - 1];
            b->e[split - 1] = last;
            on_move(g, last.idx, 1, split - 1);
        }
        b->len--;
        b->out_len--;
    } else {
        if (i != n - 1) {
            ora_entry last = b->e[n - 1];
            b->e[i] = last;
            on_move(g, last.idx, 1, i);
        }
        b->len--;
    }
}

/* AdjList::remove_edge + splice_out, list.rs:287-295 and 511-545: unlink the
 * out-entry first, re-locate the in-entry afterwards (the out splice can move
 * it), unlink it, and return the id to the LIFO free list (alloc.rs:81-90). */
int ora_remove_edge(ora_graph *g, uint64_t id) {
    if (id >= g->next_id || !g->slots[id].live) {
        g_err = "remove_edge: no such edge";
        return ORA_ERR_ARG;
    }
    ora_slot *sl = &g->slots[id];
    remove_at(g, &g->blocks[sl->src], sl->out_pos, 0);
    remove_at(g, &g->blocks[sl->tgt], sl->in_pos, 1);
    sl->live = 0;
    if (g->n_free == g->free_cap) {
        uint64_t nc = g->free_cap ? 2 * g->free_cap : 16;
        uint32_t *nf = (uint32_t *)realloc(g->free_ids, nc * sizeof(uint32_t));
        if (!nf) return ORA_ERR_OOM;
        g->free_ids = nf;
        g->free_cap = nc;
    }
    g->free_ids[g->n_free++] = (uint32_t)id;
    g->live--;
    return ORA_OK;
}

/* Bulk add_edge in list order: the edge list IS the add_edge call sequence. */
int ora_add_edges(ora_graph *g, uint64_t m, const uint32_t *src, const uint32_t *tgt) {
    for (uint64_t k = 0; k < m; ++k) {
        int64_t r = ora_add_edge(g, src[k], tgt[k]);
        if (r < 0) return (int)r;
    }
    return ORA_OK;
}

uint64_t ora_out_degree(const ora_graph *g, uint64_t v) { return g->blocks[v].out_len; }
uint64_t ora_in_degree(const ora_graph *g, uint64_t v) {
    return g->blocks[v].len - g->blocks[v].out_len;
}

/* Flatten the blocks: CSR = every out-half in storage order, CSC = every
 * in-half in storage order.  Offsets have n+1 entries. */
void ora_export(const ora_graph *g, uint64_t *out_off, uint32_t *out_other, uint32_t *out_idx,
                uint64_t *in_off, uint32_t *in_other, uint32_t *in_idx) {
    uint64_t po = 0, pi = 0;
    for (uint64_t v = 0; v < g->n; ++v) {
        const ora_block *b = &g->blocks[v];
        if (out_off) out_off[v] = po;
        if (in_off) in_off[v] = pi;
        for (uint64_t k = 0; k < b->len; ++k) {
            if (k < b->out_len) {
                if (out_other) out_other[po] = b->e[k].other;
                if (out_idx) out_idx[po] = b->e[k].idx;
                po++;
            } else {
                if (in_other) in_other[pi] = b->e[k].other;
                if (in_idx) in_idx[pi] = b->e[k].idx;
                pi++;
            }
        }
    }
    if (out_off) out_off[g->n] = po;
    if (in_off) in_off[g->n] = pi;
}

/* ------------------------------------------------------------------------ */
/* views                                                                     */
/* ------------------------------------------------------------------------ */

/* A directed view of the storage: the plain graph, its reversal (Rev swaps
 * the halves, reversed.rs:109-138), optionally filtered by two u8 masks
 * (an incident entry survives iff its edge and its other endpoint survive,
 * filtered.rs:299-319). */
typedef struct {
    const ora_graph *g;
    int reversed;
    const uint8_t *vmask; /* NULL keeps every vertex; else length n        */
    const uint8_t *emask; /* NULL keeps every edge;   else length edge_bound */
} ora_view;

static inline int keep_v(const ora_view *w, uint64_t v) { return !w->vmask || w->vmask[v]; }
static inline int keep_inc(const ora_view *w, ora_entry e) {
    return (!w->emask || w->emask[e.idx]) && keep_v(w, e.other);
}
/* The half a view calls in_edges (want_in=1) or out_edges (want_in=0). */
static inline void half(const ora_view *w, uint64_t v, int want_in, const ora_entry **b,
                        const ora_entry **e) {
    const ora_block *bl = &w->g->blocks[v];
    int in_half = w->reversed ? !want_in : want_in;
    if (in_half) {
        *b = bl->e + bl->out_len;
        *e = bl->e + bl->len;
    } else {
        *b = bl->e;
        *e = bl->e + bl->out_len;
    }
}

/* ------------------------------------------------------------------------ */
/* Plan, det_reduce, sweep                                                   */
/* ------------------------------------------------------------------------ */

typedef struct {
    uint64_t n, chunks;
} ora_plan;

/* Plan::new, plan.rs:55-61: chunks = max(ceil(n/grain), 1). */
static ora_plan plan_new(uint64_t n, uint64_t grain) {
    ora_plan p;
    p.n = n;
    p.chunks = grain ? (n + grain - 1) / grain : 1;
    if (p.chunks == 0) p.chunks = 1;
    return p;
}
/* Plan::range, plan.rs:88-101: the first n % chunks chunks carry one extra. */
static void plan_range(ora_plan p, uint64_t k, uint64_t *start, uint64_t *end) {
    uint64_t base = p.n / p.chunks, rem = p.n % p.chunks;
    *start = k * base + (k < rem ? k : rem);
    *end = *start + base + (k < rem ? 1 : 0);
}
/* grain_of, centrality.rs:186-188. */
static uint64_t grain_of(ora_plan p) {
    uint64_t g = (p.n + p.chunks - 1) / p.chunks;
    return g ? g : 1;
}

void ora_plan_range(uint64_t n, uint64_t chunks, uint64_t k, uint64_t *start, uint64_t *end) {
    ora_plan p = {n, chunks ? chunks : 1};
    plan_range(p, k, start, end);
}

/* Left fold from 0.0 in chunk order (reduce.rs:54, centrality.rs:166). */
static double fold(const double *partials, uint64_t k) {
    double acc = 0.0;
    for (uint64_t i = 0; i < k; ++i) acc = acc + partials[i];
    return acc;
}

/* ------------------------------------------------------------------------ */
/* PageRank                                                                  */
/* ------------------------------------------------------------------------ */

/*
 * pagerank_with, centrality.rs:261-384 (and pagerank, :234-248, when
 * pers == NULL: Constant(1/num_vertices) where num_vertices counts the view's
 * vertices, 0 for an empty view).
 *
 *   weight     NULL = Unity (deg = out_degree, w = 1.0); else f64 by edge id
 *   pers       NULL = uniform constant; else f64 by vertex index (len n)
 *   rank       caller's map, length >= n; it is the initial iterate and the
 *              output.  Slots [had, n) are seeded with pers (seed_new_slots).
 *   plan_len   must equal n ("sweep: the plan must cover the output exactly")
 *   plan_chunks chunk count of the caller's Plan (Plan::new(n, grain))
 *
 * Returns the number of sweeps, or a negative error.
 */
int64_t ora_pagerank(const ora_graph *g, int reversed, const uint8_t *vmask, const uint8_t *emask,
                     const double *weight, const double *pers, double damping, double epsilon,
                     uint64_t max_iter, uint64_t plan_len, uint64_t plan_chunks, double *rank,
                     uint64_t had, int nthreads) {
    ora_view W = {g, reversed, vmask, emask};
    const ora_view *w = &W;
    uint64_t len = g->n;
    if (plan_len != len) {
        g_err = "sweep: the plan must cover the output exactly";
        return ORA_ERR_ARG;
    }
    ora_plan plan = {plan_len, plan_chunks ? plan_chunks : 1};

    uint8_t *active = (uint8_t *)calloc(len ? len : 1, 1);
    double *deg = (double *)calloc(len ? len : 1, sizeof(double));
    uint32_t *sinks = (uint32_t *)malloc((len ? len : 1) * sizeof(uint32_t));
    double *scratch = (double *)calloc(len ? len : 1, sizeof(double));
    double *partials = (double *)malloc((plan.chunks + 1) * sizeof(double));
    uint64_t n_sinks = 0, nv_count = 0;
    if (!active || !deg || !sinks || !scratch || !partials) {
        free(active), free(deg), free(sinks), free(scratch), free(partials);
        g_err = "out of memory";
        return ORA_ERR_OOM;
    }
    /* active_mask, centrality.rs:176-182 */
    for (uint64_t v = 0; v < len; ++v)
        if (keep_v(w, v)) active[v] = 1, nv_count++;
    double uniform = nv_count == 0 ? 0.0 : 1.0 / (double)nv_count;

    /* degree pass, centrality.rs:281-297: Unity counts the view's out-edges,
     * a weight map left-folds them in out-half order; sinks in vertex order. */
    for (uint64_t v = 0; v < len; ++v) {
        if (!active[v]) continue;
        const ora_entry *b, *e;
        half(w, v, 0, &b, &e);
        double k;
        if (!weight) {
            uint64_t c = 0;
            for (const ora_entry *p = b; p < e; ++p) c += keep_inc(w, *p);
            k = (double)c;
        } else {
            double acc = 0.0;
            for (const ora_entry *p = b; p < e; ++p)
                if (keep_inc(w, *p)) acc += weight[p->idx];
            k = acc;
        }
        deg[v] = k;
        if (k == 0.0) sinks[n_sinks++] = (uint32_t)v;
    }

    /* sized_for + seed_new_slots, centrality.rs:299-303, 198-205 */
    for (uint64_t i = had; i < len; ++i) rank[i] = pers ? pers[i] : uniform;

    double *cur = rank, *next = scratch;
    ora_plan sink_plan = plan_new(n_sinks, grain_of(plan));
    double *sink_partials = (double *)malloc((sink_plan.chunks + 1) * sizeof(double));
    if (!sink_partials) {
        free(active), free(deg), free(sinks), free(scratch), free(partials);
        return ORA_ERR_OOM;
    }
    const double d = damping;
    double delta = epsilon + 1.0;
    uint64_t iter = 0;
    int nt = nthreads > 0 ? nthreads : 1;
    (void)nt;

    while (delta >= epsilon) {
        const double *prev = cur;
        /* p_sink via det_reduce, centrality.rs:323-335 */
#pragma omp parallel for schedule(dynamic, 1) num_threads(nt)
        for (int64_t k = 0; k < (int64_t)sink_plan.chunks; ++k) {
            uint64_t s0, s1;
            plan_range(sink_plan, (uint64_t)k, &s0, &s1);
            double acc = 0.0;
            for (uint64_t j = s0; j < s1; ++j) acc += prev[sinks[j]];
            sink_partials[k] = acc;
        }
        double p_sink = fold(sink_partials, sink_plan.chunks);

        /* the sweep, centrality.rs:340-369 */
#pragma omp parallel for schedule(dynamic, 1) num_threads(nt)
        for (int64_t k = 0; k < (int64_t)plan.chunks; ++k) {
            uint64_t r0, r1;
            plan_range(plan, (uint64_t)k, &r0, &r1);
            double local = 0.0;
            for (uint64_t i = r0; i < r1; ++i) {
                if (!active[i]) {
                    next[i] = prev[i];
                    continue;
                }
                double pv = pers ? pers[i] : uniform;
                double r = p_sink * pv;
                const ora_entry *b, *e;
                half(w, i, 1, &b, &e);
                for (const ora_entry *p = b; p < e; ++p) {
                    if (!keep_inc(w, *p)) continue;
                    uint32_t s = p->other;
                    double ds = deg[s];
                    if (ds != 0.0) {
                        double we = weight ? weight[p->idx] : 1.0;
                        r += (prev[s] * we) / ds;
                    }
                }
                double nv = (1.0 - d) * pv + d * r;
                local += fabs(nv - prev[i]);
                next[i] = nv;
            }
            partials[k] = local;
        }
        delta = fold(partials, plan.chunks);

        double *tmp = cur;
        cur = next;
        next = tmp;
        iter++;
        if (max_iter > 0 && iter == max_iter) break;
    }
    /* centrality.rs:378-383: after an odd number of swaps the latest iterate
     * is in the scratch buffer; copy it into the caller's map. */
    if (iter % 2 == 1) memcpy(next, cur, len * sizeof(double));

    free(active), free(deg), free(sinks), free(scratch), free(partials), free(sink_partials);
    return (int64_t)iter;
}

/* ------------------------------------------------------------------------ */
/* Eigenvector                                                               */
/* ------------------------------------------------------------------------ */

/*
 * eigenvector, centrality.rs:405-497.  Returns the sweep count (or a negative
 * error) and writes the eigenvalue estimate (the last norm) to *eig.
 */
int64_t ora_eigenvector(const ora_graph *g, int reversed, const uint8_t *vmask,
                        const uint8_t *emask, const double *weight, double epsilon,
                        uint64_t max_iter, uint64_t plan_len, uint64_t plan_chunks, double *x,
                        uint64_t had, int nthreads, double *eig) {
    ora_view W = {g, reversed, vmask, emask};
    const ora_view *w = &W;
    uint64_t len = g->n;
    if (plan_len != len) {
        g_err = "sweep: the plan must cover the output exactly";
        return ORA_ERR_ARG;
    }
    ora_plan plan = {plan_len, plan_chunks ? plan_chunks : 1};
    uint8_t *active = (uint8_t *)calloc(len ? len : 1, 1);
    double *scratch = (double *)calloc(len ? len : 1, sizeof(double));
    double *partials = (double *)malloc((plan.chunks + 1) * sizeof(double));
    if (!active || !scratch || !partials) {
        free(active), free(scratch), free(partials);
        return ORA_ERR_OOM;
    }
    uint64_t nv_count = 0;
    for (uint64_t v = 0; v < len; ++v)
        if (keep_v(w, v)) active[v] = 1, nv_count++;
    double uniform = nv_count == 0 ? 0.0 : 1.0 / (double)nv_count;
    for (uint64_t i = had; i < len; ++i) x[i] = uniform;

    double *cur = x, *next = scratch;
    double norm = 0.0, delta = epsilon + 1.0;
    uint64_t iter = 0;
    int nt = nthreads > 0 ? nthreads : 1;
    (void)nt;
    while (delta >= epsilon) {
        const double *prev = cur;
        /* centrality.rs:446-465: unnormalised iterate and its squared norm */
#pragma omp parallel for schedule(dynamic, 1) num_threads(nt)
        for (int64_t k = 0; k < (int64_t)plan.chunks; ++k) {
            uint64_t r0, r1;
            plan_range(plan, (uint64_t)k, &r0, &r1);
            double acc = 0.0;
            for (uint64_t i = r0; i < r1; ++i) {
                if (!active[i]) {
                    next[i] = prev[i];
                    continue;
                }
                double s = 0.0;
                const ora_entry *b, *e;
                half(w, i, 1, &b, &e);
                for (const ora_entry *p = b; p < e; ++p) {
                    if (!keep_inc(w, *p)) continue;
                    double we = weight ? weight[p->idx] : 1.0;
                    s += we * prev[p->other];
                }
                next[i] = s;
                acc += s * s;
            }
            partials[k] = acc;
        }
        double sq = fold(partials, plan.chunks);
        norm = sqrt(sq);
        /* defect-3 guard, centrality.rs:469-471 */
        double scale = norm == 0.0 ? 1.0 : norm;
        /* centrality.rs:472-484 */
#pragma omp parallel for schedule(dynamic, 1) num_threads(nt)
        for (int64_t k = 0; k < (int64_t)plan.chunks; ++k) {
            uint64_t r0, r1;
            plan_range(plan, (uint64_t)k, &r0, &r1);
            double acc = 0.0;
            for (uint64_t i = r0; i < r1; ++i) {
                if (!active[i]) continue;
                next[i] /= scale;
                acc += fabs(next[i] - prev[i]);
            }
            partials[k] = acc;
        }
        delta = fold(partials, plan.chunks);
        double *tmp = cur;
        cur = next;
        next = tmp;
        iter++;
        if (max_iter > 0 && iter == max_iter) break;
    }
    if (iter % 2 == 1) memcpy(next, cur, len * sizeof(double));
    *eig = norm;
    free(active), free(scratch), free(partials);
    return (int64_t)iter;
}

/* ------------------------------------------------------------------------ */
/* Betweenness (Brandes), centrality.rs:499-689                              */
/* ------------------------------------------------------------------------ */

/* The edges a source's BFS walks from u: out_edges of the directed view, or
 * the whole block (out-half then in-half) for the undirected view. */
static inline void bc_edges(const ora_view *w, int undirected, uint64_t u, const ora_entry **b,
                            const ora_entry **e) {
    if (undirected) {
        const ora_block *bl = &w->g->blocks[u];
        *b = bl->e;
        *e = bl->e + bl->len;
    } else {
        half(w, u, 0, b, e);
    }
}

typedef struct {
    uint64_t v;  /* predecessor */
    uint32_t e;  /* edge */
} bc_pred;

/* Brandes::run for one source (centrality.rs:544-610): BFS in dequeue order,
 * predecessors pushed in discovery order, then the dependency accumulation
 * over the dequeue order reversed. */
static void bc_run(const ora_view *w, int undirected, const uint64_t *verts, uint64_t nverts,
                   uint64_t s, int64_t *dist, double *sigma, double *dep, bc_pred **inc,
                   uint64_t *inc_len, uint64_t *inc_cap, uint64_t *order, double *vb,
                   double *eb) {
    for (uint64_t k = 0; k < nverts; ++k) {
        uint64_t i = verts[k];
        inc_len[i] = 0;
        sigma[i] = 0.0;
        dep[i] = 0.0;
        dist[i] = -1;
    }
    uint64_t head = 0, tail = 0;
    sigma[s] = 1.0;
    dist[s] = 0;
    order[tail++] = s;  /* the order array doubles as the FIFO queue */
    while (head < tail) {
        uint64_t u = order[head++];
        int64_t du = dist[u];
        double su = sigma[u];
        const ora_entry *b, *e;
        bc_edges(w, undirected, u, &b, &e);
        for (const ora_entry *x = b; x < e; ++x) {
            if (!keep_inc(w, *x)) continue;
            uint64_t t = x->other;
            if (t == u) continue; /* a self-loop never shortens a path */
            int tree = 0;
            if (dist[t] < 0) { /* tree_edge: first discovery */
                dist[t] = du + 1;
                sigma[t] = su;
                tree = 1;
            } else if (dist[t] == du + 1) { /* non_tree_edge on a shortest path */
                sigma[t] += su;
            } else {
                continue;
            }
            if (inc_len[t] == inc_cap[t]) {
                uint64_t nc = inc_cap[t] ? 2 * inc_cap[t] : 4;
                inc[t] = (bc_pred *)realloc(inc[t], nc * sizeof(bc_pred));
                inc_cap[t] = nc;
            }
            inc[t][inc_len[t]].v = u;
            inc[t][inc_len[t]].e = x->idx;
            inc_len[t]++;
            if (tree) order[tail++] = t;
        }
    }
    for (uint64_t k = tail; k-- > 0;) {
        uint64_t u = order[k];
        double su = sigma[u];
        for (uint64_t j = 0; j < inc_len[u]; ++j) {
            uint64_t v = inc[u][j].v;
            double factor = (sigma[v] / su) * (1.0 + dep[u]);
            dep[v] += factor;
            eb[inc[u][j].e] += factor;
        }
        if (u != s) vb[u] += dep[u];
    }
}

/* betweenness(g, vertex_bc, edge_bc), centrality.rs:633-689: every vertex of
 * the view is a source; sources are cut by Plan::new(|V|, ceil(|V|/16)) and
 * each chunk's partial maps are folded in chunk order; an undirected run is
 * halved.  vb has n entries, eb edge_bound entries; both are overwritten. */
int ora_betweenness(const ora_graph *g, int reversed, int undirected, const uint8_t *vmask,
                    const uint8_t *emask, double *vb, double *eb, int threads) {
    ora_view w = {g, reversed, vmask, emask};
    const uint64_t n = g->n, ne = g->next_id;
    uint64_t nverts = 0;
    uint64_t *verts = (uint64_t *)malloc((n ? n : 1) * sizeof(uint64_t));
    if (!verts) return ORA_ERR_OOM;
    for (uint64_t v = 0; v < n; ++v)
        if (keep_v(&w, v)) verts[nverts++] = v;
    /* Plan::new(|V|, max(ceil(|V| / BETWEENNESS_CHUNKS), 1)), centrality.rs:115, 654 */
    uint64_t grain = (nverts + 15) / 16;
    ora_plan plan = plan_new(nverts, grain ? grain : 1);
    double *pv = (double *)calloc(plan.chunks * (n ? n : 1), sizeof(double));
    double *pe = (double *)calloc(plan.chunks * (ne ? ne : 1), sizeof(double));
    if (!pv || !pe) {
        free(verts), free(pv), free(pe);
        return ORA_ERR_OOM;
    }
#ifdef _OPENMP
    if (threads < 1) threads = 1;
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads)
#endif
    for (int64_t k = 0; k < (int64_t)plan.chunks; ++k) {
        uint64_t lo, hi;
        plan_range(plan, (uint64_t)k, &lo, &hi);
        uint64_t nn = n ? n : 1;
        int64_t *dist = (int64_t *)malloc(nn * sizeof(int64_t));
        double *sigma = (double *)malloc(nn * sizeof(double));
        double *dep = (double *)malloc(nn * sizeof(double));
        bc_pred **inc = (bc_pred **)calloc(nn, sizeof(bc_pred *));
        uint64_t *inc_len = (uint64_t *)calloc(nn, sizeof(uint64_t));
        uint64_t *inc_cap = (uint64_t *)calloc(nn, sizeof(uint64_t));
        uint64_t *order = (uint64_t *)malloc(nn * sizeof(uint64_t));
        for (uint64_t q = lo; q < hi; ++q)
            bc_run(&w, undirected, verts, nverts, verts[q], dist, sigma, dep, inc, inc_len,
                   inc_cap, order, pv + (uint64_t)k * n, pe + (uint64_t)k * ne);
        for (uint64_t i = 0; i < nn; ++i) free(inc[i]);
        free(dist), free(sigma), free(dep), free(inc), free(inc_len), free(inc_cap), free(order);
    }
    (void)threads; /* used by the OpenMP pragma only */
    for (uint64_t i = 0; i < n; ++i) vb[i] = 0.0;
    for (uint64_t i = 0; i < ne; ++i) eb[i] = 0.0;
    for (uint64_t k = 0; k < plan.chunks; ++k) {
        for (uint64_t i = 0; i < n; ++i) vb[i] += pv[k * n + i];
        for (uint64_t i = 0; i < ne; ++i) eb[i] += pe[k * ne + i];
    }
    if (undirected) {
        for (uint64_t i = 0; i < n; ++i) vb[i] /= 2.0;
        for (uint64_t i = 0; i < ne; ++i) eb[i] /= 2.0;
    }
    free(verts), free(pv), free(pe);
    return ORA_OK;
}

/* Number of OpenMP threads the library was built to use (1 without OpenMP). */
int ora_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ------------------------------------------------------------------------ */
/* SplitMix64, the generator the reference's tests use for their fixtures    */
/* (crates/gt-algo/tests/u16_centrality.rs:59-72).                           */
/* ------------------------------------------------------------------------ */
uint64_t ora_splitmix64_next(uint64_t *state) {
    *state += 0x9e3779b97f4a7c15ull;
    uint64_t z = *state;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}
