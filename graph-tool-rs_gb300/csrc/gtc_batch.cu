// gtc_batch.cu -- PageRank of many graphs of uneven sizes in one launch.
//
// The graphs are packed as one block-diagonal graph (their disjoint union in
// input order: graph k owns vertices [voff[k], voff[k+1]) and edges
// [eoff[k], eoff[k+1])).  Each graph is pagerank
// (crates/gt-algo/src/centrality.rs:234-248) on that graph alone: uniform
// personalisation 1/n_k, its own dangling mass, its own L1 change and its
// own stop (the first sweep whose change is below epsilon).
//
// Layout (batch_layout, once per batch): inside each graph the vertices are
// relabelled -- rows of more than GB_SL_CAP in-edges (a few hubs) first,
// then the others by descending in-degree inside windows of GB_WIN
// consecutive labels, so neighbouring vertices stay neighbours.  The hubs
// keep their pull entries in CSR order and are summed by a whole warp; the
// other rows are cut into slices of 32 consecutive rows stored column-major
// (sliced ELL), so lane i of a warp sums row i of a slice and every load of
// the entry stream is one coalesced line.  Slices never cross graphs.
//
// One persistent kernel (k_pr_graphs) solves the graphs: a worker takes the
// next graph (largest first, through an atomic work counter per queue) and
// runs its whole power iteration -- sweeps separated by CTA or cluster
// barriers only, no grid-wide barrier -- before it takes another.  Its
// workers are clusters of two CTAs.  Graphs larger than 2 * GB_CL_CAP
// vertices come first, a CTA each, gathering x = rank / out-degree from
// global memory; then graphs of up to 2 * GB_CL_CAP vertices, a cluster each,
// with half of x in each CTA's shared memory; then graphs of up to GB_CL_CAP
// vertices, a CTA each, with x in its shared memory.  A graph's rows are
// assigned and its sums folded in a fixed order, so its result does not
// depend on which worker took it.  The solve's launches (weight gathers,
// degrees, the kernel) are captured once into a CUDA graph and replayed
// while the inputs keep their addresses.
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <vector>

#include <cooperative_groups.h>

#include "gtc_view.cuh"

namespace cg = cooperative_groups;

namespace gtc {
namespace {

constexpr int GB_NT = 1024;  // threads of every solving CTA
constexpr int GB_WARPS = GB_NT / 32;
constexpr int GB_U = 4;      // in-edges a thread gathers together (the next GB_U loaded ahead)

// How a graph's gathered vector x = rank / out-degree is held.
enum GbMode : int {
    GB_PAIR = 0,    // a cluster of two CTAs, half of x in each one's shared memory
    GB_SINGLE = 1,  // one CTA, all of x in its shared memory
    GB_GLOBAL = 2   // one CTA, x in global memory (graphs beyond 2 * GB_CL_CAP)
};

struct GbArgs {
    // order lists the n_pair graphs of the pair queue, then the n_single of
    // the single queue, then the n_global of the global queue
    uint32_t n_pair, n_single, n_global;
    uint32_t G_all;                      // graphs in the batch
    const uint32_t* __restrict__ order;
    const uint32_t* __restrict__ voff;   // G + 1
    const uint32_t* __restrict__ off;    // pull offsets (relabelled vertices)
    const uint32_t* __restrict__ glong;  // the layout (gtc_graph_batch)
    const uint32_t* __restrict__ gsl;
    const uint32_t* __restrict__ gebase;
    const uint32_t* __restrict__ sl_off;
    const uint32_t* __restrict__ eidx;   // layout entries: source vertex
    const float* __restrict__ w;         // weights in layout order, or null
    const uint32_t* __restrict__ vperm;  // relabelled vertex -> packed label
    const float* __restrict__ invdeg;
    const uint8_t* __restrict__ sink;
    float* r0;
    float* r1;
    float* y0;
    float* y1;
    float one_minus_d, d;
    double epsilon;
    uint64_t max_iter;
    uint64_t sweep_limit;  // an uncapped solve gives up after this many sweeps
    void* out;
    int out_dtype;
    uint64_t* iters;     // per graph, then a flag word (GB_NONFINITE | GB_SWEEP_CAP)
    unsigned* counter;   // one work counter per queue (reset by the host)
};

// A graph stops at the first sweep whose L1 change is below epsilon, or at
// max_iter.  The device loop is always bounded: a change that is not a
// finite number (non-finite weights) stops the graph at once, and an
// uncapped solve (max_iter 0) gives up after GB_UNCAPPED sweeps; both set a
// flag the host turns into an error.
constexpr uint64_t GB_UNCAPPED = 100000;
uint64_t g_sweep_limit = GB_UNCAPPED;  // lowered only by gtc_debug_set_batch_sweep_limit
constexpr uint64_t GB_NONFINITE = 1, GB_SWEEP_CAP = 2;

__device__ __forceinline__ bool sweep_done(const GbArgs& A, double delta, uint64_t it) {
    if (delta < A.epsilon) return true;
    if (A.max_iter > 0) return it == A.max_iter;
    if (!(delta < HUGE_VAL)) {
        if (threadIdx.x == 0) atomicOr((unsigned long long*)(A.iters + A.G_all), GB_NONFINITE);
        return true;
    }
    if (it == A.sweep_limit) {
        if (threadIdx.x == 0) atomicOr((unsigned long long*)(A.iters + A.G_all), GB_SWEEP_CAP);
        return true;
    }
    return false;
}

// Fixed-order CTA sum of a compensated (s, c) pair per thread, for two
// quantities; every thread gets the totals.
__device__ __forceinline__ double2 cta_sum2(Kahan a, Kahan b, double2* sm) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    warp_merge_kahan(a);
    warp_merge_kahan(b);
    if (lane == 0) sm[warp] = make_double2((double)a.s + (double)a.c, (double)b.s + (double)b.c);
    __syncthreads();
    if (threadIdx.x == 0) {
        double x = 0.0, y = 0.0;
        for (int w = 0; w < GB_WARPS; ++w) x += sm[w].x, y += sm[w].y;
        sm[GB_WARPS] = make_double2(x, y);
    }
    __syncthreads();
    const double2 t = sm[GB_WARPS];
    __syncthreads();  // sm is reused by the next call
    return t;
}

// x of source o: PAIR -- o is the graph-local label, below h in ylo (the
// first half's CTA), else in yhi; SINGLE -- local label into ylo; GLOBAL --
// the packed label into ylo (the whole vector).
template <int MODE>
__device__ __forceinline__ float gx(const float* ylo, const float* yhi, uint32_t o, uint32_t h) {
    const float* base = MODE == GB_PAIR && o >= h ? yhi - h : ylo;
    return base[o];
}

// The in-sum of lane i's row of a slice: entry j at base + 32*j (base =
// the slice's first entry + i), len entries; lmax (the slice's first and
// longest row) bounds the warp-uniform loop.  Steps of GB_U entries: a
// step's values are gathered while the next step's sources and weights
// load, and every value of a step is loaded before any is added; the adds
// run in entry order, compensated.  (Measured on the 4096-graph SBM batch:
// steps of 8 without the look-ahead 32.8 ms, of 4 with it 26.7 ms; 2, 3
// and 6 with it 27.4, 27.3 and 28.2 ms.)
template <bool W, int MODE>
__device__ __forceinline__ float slice_sum(const GbArgs& A, const float* ylo, const float* yhi,
                                           uint32_t vb, uint32_t h, uint32_t base, uint32_t len,
                                           uint32_t lmax) {
    Kahan acc;
    const uint32_t sub = MODE == GB_GLOBAL ? 0u : vb;
    uint32_t o[GB_U];
    float wv[GB_U];
#pragma unroll
    for (int j = 0; j < GB_U; ++j) {
        const bool in = (uint32_t)j < len;
        o[j] = in ? A.eidx[base + 32u * j] - sub : 0u;
        if (W) wv[j] = in ? A.w[base + 32u * j] : 0.f;
    }
    for (uint32_t j0 = 0; j0 < lmax; j0 += GB_U) {
        uint32_t on[GB_U];
        float wn[GB_U];
#pragma unroll
        for (int j = 0; j < GB_U; ++j) {
            const bool in = j0 + GB_U + j < len;
            const uint32_t q = base + 32u * (j0 + GB_U + j);
            on[j] = in ? A.eidx[q] - sub : 0u;
            if (W) wn[j] = in ? A.w[q] : 0.f;
        }
        float x[GB_U];
#pragma unroll
        for (int j = 0; j < GB_U; ++j) x[j] = j0 + j < len ? gx<MODE>(ylo, yhi, o[j], h) : 0.f;
#pragma unroll
        for (int j = 0; j < GB_U; ++j)
            if (j0 + j < len) acc.add(W ? __fmul_rn(x[j], wv[j]) : x[j]);
#pragma unroll
        for (int j = 0; j < GB_U; ++j) {
            o[j] = on[j];
            if (W) wv[j] = wn[j];
        }
    }
    return acc.value();
}

// The in-sum of a long row by the whole warp: lane i takes entries i,
// i + 32, ... (four in flight), compensated in blocks of KB_BLOCK, merged
// across the lanes in a fixed butterfly; every lane gets the sum.
template <bool W, int MODE>
__device__ __forceinline__ float long_sum(const GbArgs& A, const float* ylo, const float* yhi,
                                          uint32_t vb, uint32_t h, uint32_t base, uint32_t len) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t sub = MODE == GB_GLOBAL ? 0u : vb;
    KahanBlocked acc;
    uint32_t q = lane;
    for (; q + 96 < len; q += 128) {
        uint32_t o[4];
        float x[4], wv[4];
#pragma unroll
        for (int t = 0; t < 4; ++t) {
            o[t] = A.eidx[base + q + 32u * t] - sub;
            if (W) wv[t] = A.w[base + q + 32u * t];
        }
#pragma unroll
        for (int t = 0; t < 4; ++t) x[t] = gx<MODE>(ylo, yhi, o[t], h);
#pragma unroll
        for (int t = 0; t < 4; ++t) acc.add(W ? __fmul_rn(x[t], wv[t]) : x[t]);
    }
    for (; q < len; q += 32) {
        const float x = gx<MODE>(ylo, yhi, A.eidx[base + q] - sub, h);
        acc.add(W ? __fmul_rn(x, A.w[base + q]) : x);
    }
    Kahan t = acc.fold();
    warp_merge_kahan(t);
    return t.value();
}

// What lane i's row of a slice needs besides its entries.
struct SliceRow {
    uint32_t len, base;  // entries; the slice's first entry
    float rc, idg;
    uint8_t sk;
    bool in;             // the lane holds a row
};

__device__ __forceinline__ SliceRow slice_row(const GbArgs& A, const float* rc, uint32_t v,
                                              uint32_t ve, uint32_t s, bool any) {
    SliceRow r{0u, 0u, 0.f, 0.f, 0, false};
    if (any) {
        r.base = A.sl_off[s];
        r.in = v < ve;
        if (r.in) {
            r.len = A.off[v + 1] - A.off[v];
            r.rc = rc[v];
            r.idg = A.invdeg[v];
            r.sk = A.sink[v];
        }
    }
    return r;
}

// The whole power iteration of graph gk by this CTA (PAIR: with its peer).
// A sweep deals the graph's long rows (a warp each), then its slices (a
// warp each, a row per lane), round-robin to the warps (of both CTAs in
// PAIR).  x lives in shared memory: in PAIR, CTA r keeps the
// rows [vb + r*h, ...) with h = ceil(n_k / 2).  Each sweep writes the new x
// to global y1; after the barrier that ends the sweep's gathers every CTA
// copies its rows of it back into shared memory.  The sums over the graph
// are folded thread -> warp -> CTA (-> rank 0 + rank 1) in fixed order, so
// a pair's CTAs see the same totals and stop together.
template <bool W, int MODE>
__device__ __forceinline__ void solve_graph(const GbArgs& A, uint32_t gk, float* ys,
                                            const float* ypeer, unsigned r, double2* sm,
                                            double2* part, const double2* ppeer) {
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t vb = A.voff[gk], ve = A.voff[gk + 1];
    const uint32_t nk = ve - vb;
    const uint32_t h = MODE == GB_PAIR ? (nk + 1) >> 1 : nk;
    const uint32_t lo = MODE == GB_PAIR ? vb + r * h : vb;
    const uint32_t hi = MODE == GB_PAIR && r == 0 ? vb + h : ve;
    const float* ylo = MODE == GB_PAIR && r ? ypeer : ys;
    const float* yhi = MODE == GB_PAIR && r == 0 ? ypeer : ys;
    const uint32_t n_long = A.glong[gk], s0 = A.gsl[gk];
    const uint32_t n_sl = A.gsl[gk + 1] - s0;
    const uint32_t eb = A.gebase[gk], ob = A.off[vb];
    const uint32_t wfirst = (MODE == GB_PAIR ? r * GB_WARPS : 0u) + warp;
    const uint32_t wstep = (MODE == GB_PAIR ? 2u : 1u) * GB_WARPS;
    // slices [qlo, qhi) belong to this CTA: in PAIR the ones whose first row
    // is in its half
    const uint32_t q_split =
        MODE == GB_PAIR ? (h > n_long ? min(n_sl, (h - n_long + 31u) >> 5) : 0u) : n_sl;
    const uint32_t qlo = MODE == GB_PAIR && r ? q_split : 0u;
    const uint32_t qend = MODE == GB_PAIR && r == 0 ? q_split : n_sl;
    auto sum2 = [&](Kahan a, Kahan b) -> double2 {
        const double2 t = cta_sum2(a, b, sm);
        if (MODE != GB_PAIR) return t;
        if (threadIdx.x == 0) *part = t;
        cg::this_cluster().sync();
        const double2 o = *ppeer;
        return r == 0 ? make_double2(t.x + o.x, t.y + o.y) : make_double2(o.x + t.x, o.y + t.y);
    };
    const float u = nk ? (float)(1.0 / (double)nk) : 0.f;
    Kahan ks, kz;
    for (uint32_t v = lo + threadIdx.x; v < hi; v += GB_NT) {
        A.r0[v] = u;
        const float x = __fmul_rn(u, A.invdeg[v]);
        if (MODE == GB_GLOBAL)
            A.y0[v] = x;
        else
            ys[v - lo] = x;
        if (A.sink[v]) ks.add(u);
    }
    double psink = sum2(ks, kz).x;  // its barrier also publishes the start
    float *rc = A.r0, *rn = A.r1, *yc = A.y0, *yn = A.y1;
    uint64_t it = 0;
    for (;;) {
        const float ps = (float)psink;
        const float base_r = __fmul_rn(ps, u);
        const float teleport = __fmul_rn(A.one_minus_d, u);
        const float* gl = MODE == GB_GLOBAL ? yc : ylo;
        Kahan kd, kk;
        auto finish = [&](uint32_t v, float sr, float rcv, float idg, uint8_t sk) {
            const float nv = __fadd_rn(teleport, __fmul_rn(A.d, __fadd_rn(base_r, sr)));
            rn[v] = nv;
            yn[v] = __fmul_rn(nv, idg);
            kd.add(fabsf(__fsub_rn(nv, rcv)));
            if (sk) kk.add(nv);
        };
        // long rows: the whole warp, lane 0 finishes the row
        for (uint32_t k = wfirst; k < n_long; k += wstep) {
            const uint32_t v = vb + k;
            const uint32_t pb = A.off[v];
            const float sr = long_sum<W, MODE>(A, gl, yhi, vb, h, eb + (pb - ob), A.off[v + 1] - pb);
            if (lane == 0) finish(v, sr, rc[v], A.invdeg[v], A.sink[v]);
        }
        // slices, row vb + n_long + 32*q + lane (in PAIR each CTA takes the
        // slices that start in its half, whose rows' x it holds).  Round k
        // gives warp w the slice 32k + ((w + 7k) mod 32) of its range: the
        // slices of a window run from long to short, and the rotation spreads
        // the long ones over the warps.  What the next slice's rows need
        // besides their entries is loaded while this one's are summed.
        auto slice_of = [&](uint32_t k) { return qlo + 32u * k + ((warp + 7u * k) & 31u); };
        uint32_t q = slice_of(0);
        SliceRow cur = slice_row(A, rc, vb + n_long + 32u * q + lane, ve, s0 + q, q < qend);
        for (uint32_t k = 0; 32u * k < qend - qlo; ++k) {  // k and q are warp-uniform
            const uint32_t qn = slice_of(k + 1);
            const SliceRow nx = slice_row(A, rc, vb + n_long + 32u * qn + lane, ve, s0 + qn, qn < qend);
            if (q < qend) {
                const uint32_t lmax = __reduce_max_sync(0xffffffffu, cur.len);
                const float sr = slice_sum<W, MODE>(A, gl, yhi, vb, h, cur.base + lane, cur.len, lmax);
                if (cur.in) finish(vb + n_long + 32u * q + lane, sr, cur.rc, cur.idg, cur.sk);
            }
            q = qn;
            cur = nx;
        }
        const double2 t = sum2(kd, kk);  // every gather of this sweep is done
        ++it;
        float* tr = rc;
        rc = rn, rn = tr;
        if (MODE == GB_GLOBAL) {
            float* ty = yc;
            yc = yn, yn = ty;
        }
        psink = t.y;
        if (sweep_done(A, t.x, it)) break;
        if (MODE != GB_GLOBAL) {
            // x back into shared memory: asynchronous 4-byte copies, all of a
            // thread's in flight at once
            for (uint32_t v = lo + threadIdx.x; v < hi; v += GB_NT) {
                const uint32_t dst = (uint32_t)__cvta_generic_to_shared(ys + (v - lo));
                asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(dst), "l"(yn + v) : "memory");
            }
            asm volatile("cp.async.wait_all;" ::: "memory");
            if (MODE == GB_PAIR)
                cg::this_cluster().sync();
            else
                __syncthreads();
        }
    }
    for (uint32_t v = lo + threadIdx.x; v < hi; v += GB_NT) {
        const uint32_t o = A.vperm[v];
        if (A.out_dtype == GTC_F64)
            ((double*)A.out)[o] = (double)rc[v];
        else
            ((float*)A.out)[o] = rc[v];
    }
    if ((MODE != GB_PAIR || r == 0) && threadIdx.x == 0) A.iters[gk] = it;
}

// The global queue, the pair queue, then the single queue.  Each CTA
// first draws global graphs alone.  Then a cluster takes pair graphs (rank
// 0 draws from the counter and its peer reads the draw from rank 0's shared
// memory) until the queue is empty; the first draw waits for both CTAs, so a
// CTA whose peer still solves a global graph waits for it.  From then on
// each CTA draws single graphs alone, with no cluster barrier and no access
// to the peer's shared memory, so the CTAs of a cluster may finish at
// different times.
template <bool W>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(GB_NT, 1) k_pr_graphs(GbArgs A) {
    extern __shared__ float ys[];
    __shared__ double2 sm[GB_WARPS + 1];
    __shared__ double2 part;
    __shared__ uint32_t s_graph;
    cg::cluster_group cl = cg::this_cluster();
    const unsigned r = cl.block_rank();
    const float* ypeer = cl.map_shared_rank(ys, r ^ 1u);
    const double2* ppeer = cl.map_shared_rank(&part, r ^ 1u);
    const uint32_t* graph0 = cl.map_shared_rank(&s_graph, 0u);
    for (;;) {
        if (threadIdx.x == 0) s_graph = atomicAdd(A.counter + 2, 1u);
        __syncthreads();
        const uint32_t k = s_graph;
        __syncthreads();
        if (k >= A.n_global) break;
        solve_graph<W, GB_GLOBAL>(A, A.order[A.n_pair + A.n_single + k], nullptr, nullptr, 0, sm,
                                  nullptr, nullptr);
    }
    for (;;) {
        if (r == 0 && threadIdx.x == 0) s_graph = atomicAdd(A.counter, 1u);
        cl.sync();
        const uint32_t k = *graph0;
        cl.sync();
        if (k >= A.n_pair) break;
        solve_graph<W, GB_PAIR>(A, A.order[k], ys, ypeer, r, sm, &part, ppeer);
    }
    for (;;) {
        if (threadIdx.x == 0) s_graph = atomicAdd(A.counter + 1, 1u);
        __syncthreads();
        const uint32_t k = s_graph;
        __syncthreads();
        if (k >= A.n_single) return;
        solve_graph<W, GB_SINGLE>(A, A.order[A.n_pair + k], ys, nullptr, 0, sm, nullptr, nullptr);
    }
}

// ---- layout build -----------------------------------------------------------

__global__ void k_bl_indeg(uint32_t m, const uint32_t* __restrict__ tgt, uint32_t* __restrict__ indeg) {
    const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e < m) atomicAdd(indeg + tgt[e], 1u);
}

// the graph whose vertex (or slice) range [start[g], start[g+1]) holds i
__device__ __forceinline__ uint32_t owner_of(const uint32_t* __restrict__ start, uint32_t G, uint32_t i) {
    uint32_t lo = 0, hi = G;
    while (hi - lo > 1) {
        const uint32_t mid = lo + ((hi - lo) >> 1);
        if (start[mid] <= i)
            lo = mid;
        else
            hi = mid;
    }
    return lo;
}

// gid[v]; key[v] puts a graph's rows of more than GB_SL_CAP in-edges first
// (in label order), then its other rows window by window (GB_WIN labels
// each, so vertices that were near each other stay near), each window by
// descending in-degree
__global__ void k_bl_keys(uint32_t n, uint32_t G, const uint32_t* __restrict__ voff,
                          const uint32_t* __restrict__ indeg, uint32_t* __restrict__ gid,
                          uint32_t* __restrict__ key) {
    const size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n) return;
    const uint32_t g = owner_of(voff, G, (uint32_t)v);
    gid[v] = g;
    const uint32_t d = indeg[v];
    key[v] = d > GB_SL_CAP ? 0u : 1u + ((uint32_t)v - voff[g]) / GB_WIN * (GB_SL_CAP + 1) + (GB_SL_CAP - d);
}

__global__ void k_bl_gkey(uint32_t n, const uint32_t* __restrict__ ord, const uint32_t* __restrict__ gid,
                          uint32_t* __restrict__ key) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) key[i] = gid[ord[i]];
}

__global__ void k_bl_perm(uint32_t n, const uint32_t* __restrict__ ord1, const uint32_t* __restrict__ ord2,
                          uint32_t* __restrict__ vperm, uint32_t* __restrict__ iperm) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t old = ord1[ord2[i]];
    vperm[i] = old;
    iperm[old] = (uint32_t)i;
}

__global__ void k_bl_relabel(uint32_t m, const uint32_t* __restrict__ iperm, uint32_t* __restrict__ a,
                             uint32_t* __restrict__ b) {
    const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= m) return;
    a[e] = iperm[a[e]];
    b[e] = iperm[b[e]];
}

// per graph: its long rows (they come first), slices and long entries
__global__ void k_bl_graph_rows(uint32_t G, const uint32_t* __restrict__ voff,
                                const uint32_t* __restrict__ off, uint32_t* __restrict__ glong,
                                uint32_t* __restrict__ nsl, uint32_t* __restrict__ longe) {
    const size_t g = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= G) return;
    const uint32_t vb = voff[g], ve = voff[g + 1];
    uint32_t lo = vb, hi = ve;
    while (lo < hi) {
        const uint32_t mid = lo + ((hi - lo) >> 1);
        if (off[mid + 1] - off[mid] > GB_SL_CAP)
            lo = mid + 1;
        else
            hi = mid;
    }
    glong[g] = lo - vb;
    nsl[g] = (ve - lo + 31) >> 5;
    longe[g] = off[lo] - off[vb];
}

// per slice: its graph and its length (its first row's)
__global__ void k_bl_slices(uint32_t S, uint32_t G, const uint32_t* __restrict__ gsl,
                            const uint32_t* __restrict__ voff, const uint32_t* __restrict__ glong,
                            const uint32_t* __restrict__ off, uint32_t* __restrict__ sgraph,
                            uint32_t* __restrict__ slen) {
    const size_t s = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= S) return;
    const uint32_t g = owner_of(gsl, G, (uint32_t)s);
    const uint32_t row0 = voff[g] + glong[g] + 32u * ((uint32_t)s - gsl[g]);
    const uint32_t rend = min(row0 + 32u, voff[g + 1]);
    uint32_t len = 0;
    for (uint32_t r = row0; r < rend; ++r) len = max(len, off[r + 1] - off[r]);
    sgraph[s] = g;
    slen[s] = len;
}

__global__ void k_bl_fill_long(uint32_t n, const uint32_t* __restrict__ gid,
                               const uint32_t* __restrict__ voff, const uint32_t* __restrict__ glong,
                               const uint32_t* __restrict__ gebase, const uint32_t* __restrict__ off,
                               const uint32_t* __restrict__ other, const uint32_t* __restrict__ eid,
                               uint32_t* __restrict__ eidx, uint32_t* __restrict__ eeid) {
    const size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n) return;
    const uint32_t g = gid[v], vb = voff[g];
    if ((uint32_t)v - vb >= glong[g]) return;
    const uint32_t pb = off[v], pe = off[v + 1];
    const uint32_t base = gebase[g] + (pb - off[vb]);
    for (uint32_t p = pb; p < pe; ++p) {
        eidx[base + (p - pb)] = other[p];
        eeid[base + (p - pb)] = eid[p];
    }
}

__global__ void k_bl_fill_slices(uint32_t S, const uint32_t* __restrict__ sgraph,
                                 const uint32_t* __restrict__ slen,
                                 const uint32_t* __restrict__ gsl, const uint32_t* __restrict__ voff,
                                 const uint32_t* __restrict__ glong, const uint32_t* __restrict__ sl_off,
                                 const uint32_t* __restrict__ off, const uint32_t* __restrict__ other,
                                 const uint32_t* __restrict__ eid, uint32_t* __restrict__ eidx,
                                 uint32_t* __restrict__ eeid) {
    const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (size_t)S * 32) return;
    const uint32_t s = (uint32_t)(t >> 5), lane = (uint32_t)(t & 31);
    const uint32_t g = sgraph[s], vb = voff[g], ve = voff[g + 1];
    const uint32_t row0 = vb + glong[g] + 32u * (s - gsl[g]);
    const uint32_t row = row0 + lane;
    const uint32_t lmax = slen[s];
    const uint32_t len = row < ve ? off[row + 1] - off[row] : 0u;
    const uint32_t pb = row < ve ? off[row] : 0u;
    for (uint32_t j = 0; j < lmax; ++j) {
        const uint32_t q = sl_off[s] + 32u * j + lane;
        eidx[q] = j < len ? other[pb + j] : vb;  // pads: any vertex of the graph
        eeid[q] = j < len ? eid[pb + j] : 0xFFFFFFFFu;
    }
}

// out[p] = w[eid[p]]; an edge id of ~0 (layout padding) gives 0
__global__ void k_gb_gather(uint32_t m, const uint32_t* __restrict__ eid, const void* __restrict__ w,
                            int wdt, float* __restrict__ out) {
    const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= m) return;
    const uint32_t e = eid[p];
    out[p] = e != 0xFFFFFFFFu ? ld_f32(w, wdt, e) : 0.f;
}

// weighted out-degree (8 lanes per vertex, compensated, fixed merge order) or
// the plain out-degree; its FP32 inverse and the sink flags
__global__ void k_gb_degree(uint32_t n, const uint32_t* __restrict__ push_off,
                            const float* __restrict__ wout, float* __restrict__ invdeg,
                            uint8_t* __restrict__ sink) {
    const uint32_t sub = threadIdx.x & 7;
    const size_t v = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 3;
    const bool in = v < n;
    KahanBlocked kb;
    if (in && wout)
        for (uint32_t p = push_off[v] + sub, e = push_off[v + 1]; p < e; p += 8) kb.add(wout[p]);
    Kahan k = kb.fold();
    for (int o = 4; o > 0; o >>= 1) {
        const float os = __shfl_xor_sync(0xffffffffu, k.s, o, 8);
        const float oc = __shfl_xor_sync(0xffffffffu, k.c, o, 8);
        k.merge(os, oc);
    }
    if (in && sub == 0) {  // FP32 only: a few FP64 operations per vertex cost more than its loads
        const float dg = wout ? k.value() : (float)(push_off[v + 1] - push_off[v]);
        invdeg[v] = dg != 0.f ? __frcp_rn(dg) : 0.f;
        sink[v] = dg == 0.f ? 1 : 0;
    }
}

}  // namespace

void batch_init(gtc_graph_batch* b, cudaStream_t s) {
    gtc_graph* u = b->u;
    const uint32_t n = u->n, m = u->m;
    cudaStream_t h = u->home;
    b->invdeg.alloc(n, h);
    b->sink.alloc(n, h);
    b->r0.alloc(n, h);
    b->r1.alloc(n, h);
    b->y0.alloc(n, h);
    b->y1.alloc(n, h);
    b->wout.alloc(m, h);
    b->wlay.alloc(b->n_lay, h);
    b->iters.alloc((size_t)b->G + 1, h);
    b->counter.alloc(3, h);
    GTC_CUDA(cudaStreamSynchronize(h));
    (void)s;
}

void batch_layout(gtc_graph_batch* b, uint32_t* ds, uint32_t* dt, cudaStream_t s) {
    gtc_graph* u = b->u;
    const uint32_t n = u->n, m = u->m, G = b->G;
    const unsigned TB = 256;
    uint64_t L = 0;
    b->vperm.alloc(n, s);
    {
        // relabel every graph's vertices by descending in-degree: stable by
        // length, then stable by graph (vertices stay inside their graph)
        DevBuf<uint32_t> indeg(n, s), gid(n, s), key(n, s), skey(n, s), ord1(n, s), ord2(n, s);
        DevBuf<uint32_t> iperm(n, s);
        if (n) {
            GTC_CUDA(cudaMemsetAsync(indeg.get(), 0, (size_t)n * 4, s));
            if (m) k_bl_indeg<<<grid_for(m, TB, 1u << 30), TB, 0, s>>>(m, dt, indeg.get());
            k_bl_keys<<<grid_for(n, TB, 1u << 30), TB, 0, s>>>(n, G, b->voff.get(), indeg.get(),
                                                               gid.get(), key.get());
            GTC_LAUNCHED();
            uint32_t nmax = 0;
            for (uint32_t g = 0; g < G; ++g) nmax = std::max(nmax, b->hvoff[g + 1] - b->hvoff[g]);
            const uint32_t kbound = 2u + (nmax / GB_WIN) * (GB_SL_CAP + 1) + GB_SL_CAP;
            sort_positions_by_key(key.get(), n, kbound, skey.get(), ord1.get(), s, &L);
            k_bl_gkey<<<grid_for(n, TB, 1u << 30), TB, 0, s>>>(n, ord1.get(), gid.get(), key.get());
            GTC_LAUNCHED();
            sort_positions_by_key(key.get(), n, G, skey.get(), ord2.get(), s, &L);
            k_bl_perm<<<grid_for(n, TB, 1u << 30), TB, 0, s>>>(n, ord1.get(), ord2.get(),
                                                               b->vperm.get(), iperm.get());
            GTC_LAUNCHED();
            if (m) {
                k_bl_relabel<<<grid_for(m, TB, 1u << 30), TB, 0, s>>>(m, iperm.get(), ds, dt);
                GTC_LAUNCHED();
            }
        }
        build_halves(u, ds, dt, /*relabel=*/false);
        // the long rows, slices and long entries of every graph
        DevBuf<uint32_t> nsl(G, s), longe(G, s);
        b->glong.alloc(G, s);
        k_bl_graph_rows<<<grid_for(G, TB, 1u << 30), TB, 0, s>>>(G, b->voff.get(), u->in.off.get(),
                                                                b->glong.get(), nsl.get(),
                                                                longe.get());
        GTC_LAUNCHED();
        std::vector<uint32_t> hnsl(G), hlonge(G), hgsl((size_t)G + 1);
        GTC_CUDA(cudaMemcpyAsync(hnsl.data(), nsl.get(), (size_t)G * 4, cudaMemcpyDeviceToHost, s));
        GTC_CUDA(cudaMemcpyAsync(hlonge.data(), longe.get(), (size_t)G * 4, cudaMemcpyDeviceToHost, s));
        GTC_CUDA(cudaStreamSynchronize(s));
        uint64_t S = 0;
        for (uint32_t g = 0; g < G; ++g) hgsl[g] = (uint32_t)S, S += hnsl[g];
        GTC_REQUIRE(S < 0xFFFFFFFFull, GTC_ERR_ARG, "batch too large for the slice layout");
        hgsl[G] = (uint32_t)S;
        b->gsl.alloc((size_t)G + 1, s);
        GTC_CUDA(cudaMemcpyAsync(b->gsl.get(), hgsl.data(), ((size_t)G + 1) * 4, cudaMemcpyHostToDevice, s));
        DevBuf<uint32_t> sgraph(S, s), slen(S, s);
        std::vector<uint32_t> hslen(S);
        if (S) {
            k_bl_slices<<<grid_for(S, TB, 1u << 30), TB, 0, s>>>(
                (uint32_t)S, G, b->gsl.get(), b->voff.get(), b->glong.get(), u->in.off.get(),
                sgraph.get(), slen.get());
            GTC_LAUNCHED();
            GTC_CUDA(cudaMemcpyAsync(hslen.data(), slen.get(), S * 4, cudaMemcpyDeviceToHost, s));
            GTC_CUDA(cudaStreamSynchronize(s));
        }
        // entry offsets: per graph its long rows' entries, then its slices
        std::vector<uint32_t> hbase(G), hsoff(S);
        uint64_t pos = 0;
        for (uint32_t g = 0; g < G; ++g) {
            hbase[g] = (uint32_t)pos;
            pos += hlonge[g];
            for (uint32_t q = hgsl[g]; q < hgsl[g + 1]; ++q) hsoff[q] = (uint32_t)pos, pos += 32ull * hslen[q];
            GTC_REQUIRE(pos < 0xFFFFFFFFull, GTC_ERR_ARG, "batch too large for the slice layout");
        }
        b->n_lay = pos;
        b->gebase.alloc(G, s);
        b->sl_off.alloc(S, s);
        GTC_CUDA(cudaMemcpyAsync(b->gebase.get(), hbase.data(), (size_t)G * 4, cudaMemcpyHostToDevice, s));
        if (S) GTC_CUDA(cudaMemcpyAsync(b->sl_off.get(), hsoff.data(), S * 4, cudaMemcpyHostToDevice, s));
        b->eidx.alloc(pos, s);
        b->eeid.alloc(pos, s);
        if (n) {
            k_bl_fill_long<<<grid_for(n, TB, 1u << 30), TB, 0, s>>>(
                n, gid.get(), b->voff.get(), b->glong.get(), b->gebase.get(), u->in.off.get(),
                u->in.other.get(), u->in.eid.get(), b->eidx.get(), b->eeid.get());
            GTC_LAUNCHED();
        }
        if (S) {
            k_bl_fill_slices<<<grid_for(S * 32, TB, 1u << 30), TB, 0, s>>>(
                (uint32_t)S, sgraph.get(), slen.get(), b->gsl.get(), b->voff.get(), b->glong.get(),
                b->sl_off.get(), u->in.off.get(), u->in.other.get(), u->in.eid.get(), b->eidx.get(),
                b->eeid.get());
            GTC_LAUNCHED();
        }
        GTC_CUDA(cudaStreamSynchronize(s));  // the host vectors and temporaries die here
    }
    u->launches += L;
}

void pagerank_batch(gtc_graph_batch* b, const DVec& weight, double damping, double epsilon,
                    uint64_t max_iter, void* out, int out_dtype, uint64_t* iters, bool timing,
                    gtc_result* res, cudaStream_t s) {
    gtc_graph* u = b->u;
    const uint32_t n = u->n, m = u->m;
    if (!b->invdeg.get()) batch_init(b, s);
    const bool W = weight.present();
    // the launches of one solve, captured once per set of inputs and replayed
    const BatchKey key{W ? weight.p : nullptr, W ? weight.dtype : -1, out, out_dtype, damping,
                       epsilon, max_iter, g_sweep_limit};
    if (!b->exec || !(b->key == key)) {
        if (b->exec) {
            cudaGraphExecDestroy(b->exec);
            b->exec = nullptr;
        }
        int sms = 0, dev = 0;
        GTC_CUDA(cudaGetDevice(&dev));
        GTC_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        void (*kern)(GbArgs) = W ? k_pr_graphs<true> : k_pr_graphs<false>;
        const uint32_t n_graphs = b->n_pair + b->n_single + b->n_global;
        unsigned grid = 0;
        const size_t smem = (size_t)std::max<uint32_t>(b->smem_floats, 1u) * sizeof(float);
        if (n_graphs) {
            GTC_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            cudaLaunchConfig_t cfg{};
            cfg.gridDim = dim3(2 * (unsigned)sms);
            cfg.blockDim = dim3(GB_NT);
            cfg.dynamicSmemBytes = smem;
            int clusters = 0;
            GTC_CUDA(cudaOccupancyMaxActiveClusters(&clusters, kern, &cfg));
            // every cluster that can have work: a pair graph, or two graphs of
            // the other queues
            const uint32_t useful = b->n_pair + (b->n_single + b->n_global + 1) / 2;
            grid = 2u * (unsigned)std::max(1, std::min<int>(clusters, (int)useful));
        }
        cudaGraph_t graph = nullptr;
        GTC_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        const unsigned TB = 256;
        if (W && m) {
            k_gb_gather<<<grid_for(m, TB, 1u << 30), TB, 0, s>>>(m, u->out.eid.get(), weight.p,
                                                                 weight.dtype, b->wout.get());
            if (b->n_lay)
                k_gb_gather<<<grid_for(b->n_lay, TB, 1u << 30), TB, 0, s>>>(
                    (uint32_t)b->n_lay, b->eeid.get(), weight.p, weight.dtype, b->wlay.get());
        }
        if (n)
            k_gb_degree<<<grid_for((size_t)n * 8, TB, 1u << 30), TB, 0, s>>>(
                n, u->out.off.get(), W ? b->wout.get() : nullptr, b->invdeg.get(), b->sink.get());
        cudaMemsetAsync(b->counter.get(), 0, 3 * sizeof(unsigned), s);
        cudaMemsetAsync(b->iters.get() + b->G, 0, sizeof(uint64_t), s);
        GbArgs A{};
        A.n_pair = b->n_pair;
        A.n_single = b->n_single;
        A.n_global = b->n_global;
        A.G_all = b->G;
        A.order = b->order.get();
        A.voff = b->voff.get();
        A.off = u->in.off.get();
        A.glong = b->glong.get();
        A.gsl = b->gsl.get();
        A.gebase = b->gebase.get();
        A.sl_off = b->sl_off.get();
        A.eidx = b->eidx.get();
        A.w = W ? b->wlay.get() : nullptr;
        A.vperm = b->vperm.get();
        A.invdeg = b->invdeg.get();
        A.sink = b->sink.get();
        A.r0 = b->r0.get(), A.r1 = b->r1.get(), A.y0 = b->y0.get(), A.y1 = b->y1.get();
        A.one_minus_d = (float)(1.0 - damping);
        A.d = (float)damping;
        A.epsilon = epsilon;
        A.max_iter = max_iter;
        A.sweep_limit = g_sweep_limit;
        A.out = out;
        A.out_dtype = out_dtype;
        A.iters = b->iters.get();
        A.counter = b->counter.get();
        if (n_graphs) kern<<<grid, GB_NT, smem, s>>>(A);
        const cudaError_t ce = cudaStreamEndCapture(s, &graph);
        GTC_CUDA(ce);
        GTC_LAUNCHED();
        const cudaError_t ie = cudaGraphInstantiate(&b->exec, graph, 0);
        cudaGraphDestroy(graph);
        GTC_CUDA(ie);
        b->key = key;
        b->launches_per_solve =
            (W && m ? 1 : 0) + (W && b->n_lay ? 1 : 0) + (n ? 1 : 0) + (n_graphs ? 1 : 0);
    }
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (timing) {
        GTC_CUDA(cudaEventCreate(&e0));
        GTC_CUDA(cudaEventCreate(&e1));
        GTC_CUDA(cudaEventRecord(e0, s));
    }
    GTC_CUDA(cudaGraphLaunch(b->exec, s));
    if (timing) GTC_CUDA(cudaEventRecord(e1, s));
    std::vector<uint64_t> hit((size_t)b->G + 1);
    GTC_CUDA(cudaMemcpyAsync(hit.data(), b->iters.get(), hit.size() * 8, cudaMemcpyDeviceToHost, s));
    GTC_CUDA(cudaStreamSynchronize(s));
    const uint64_t flags = hit[b->G];
    float ms = 0.f;
    if (timing) {
        GTC_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
    }
    uint64_t mx = 0, total = 0;
    for (uint32_t k = 0; k < b->G; ++k) {
        if (iters) iters[k] = hit[k];
        mx = std::max(mx, hit[k]);
        total += hit[k];
    }
    res->iterations = mx;
    res->last_delta = 0.0;
    res->eigenvalue = 0.0;
    res->device_ms = ms;
    res->launches = b->launches_per_solve;
    res->sweep_ms = ms;
    res->sweep_launches = 1;
    u->launches += b->launches_per_solve;
    (void)total;
    GTC_REQUIRE(!(flags & GB_NONFINITE), GTC_ERR_ARG,
                "a graph's L1 change is not a finite number (non-finite weights?)");
    GTC_REQUIRE(!(flags & GB_SWEEP_CAP), GTC_ERR_TIMEOUT,
                "an uncapped solve (max_iter 0) did not converge within " +
                    std::to_string(g_sweep_limit) + " sweeps");
}

}  // namespace gtc

extern "C" int gtc_debug_set_batch_sweep_limit(uint64_t limit) {
    gtc::g_sweep_limit = limit ? limit : gtc::GB_UNCAPPED;
    return GTC_OK;
}
