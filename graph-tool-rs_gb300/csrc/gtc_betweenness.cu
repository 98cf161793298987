// gtc_betweenness.cu -- betweenness centrality (Brandes) on the GPU.
//
// Replaces gt_algo::centrality::betweenness (crates/gt-algo/src/centrality.rs
// :499-689 of graph-tool-rs): unweighted, every vertex of the view a source,
// unnormalised vertex and edge maps, halved on the undirected view.
//
// Parallel shape.  One CTA runs one source at a time, and a persistent grid
// of G CTAs (as many as are resident at once) deals the sources out (CTA c
// takes sources c, c + G, ...).  Per source, a level-synchronous BFS whose
// phases walk each vertex of a level with a pair of lanes (a vertex with more
// than 32 edges to walk is set aside and walked by a whole warp once the
// pairs are done: the walks are chains of dependent loads, so many short
// walks in flight keep the SM busy):
//   expand   over the frontier's out-edges; a vertex joins the next level by
//            an atomic claim of its distance
//   sigma    each new vertex pulls its path count from the in-edges whose
//            source lies one level up (each parallel edge is a distinct
//            shortest path, as in the reference's non_tree_edge)
//   back     levels deepest first: each vertex v sums sigma_v * c_t over its
//            out-edges into the next level, c_t = (1 + dep_t) / sigma_t
//            formed once per vertex when its dependency is final, adds each
//            term to its edge and the sum to v
// The order a level is discovered in does not enter any sum: every sum is a
// pull over one vertex's edges in storage order, lane-strided and merged by
// a fixed shuffle tree (over the pair, or over the warp for a vertex with
// more than 32 edges), so the result is deterministic.  It differs from the
// reference's by the association of FP64 sums (the reference accumulates in
// BFS dequeue order) and in the last bits of each term (the reference forms
// (sigma_v / sigma_t)(1 + dep_t) per edge: one divide per edge, where an
// FP64 divide is a dozen FP64 instructions on a GPU whose FP64 pipe is the
// back phase's bound), which is why parity is stated as a tolerance, as the
// reference's own tests state it against their independent Brandes
// (crates/gt-algo/tests/u16_centrality.rs:707-760).  Path counts are sums of
// integers, exact while they stay below 2^53.
//
// Each CTA keeps its own partial vertex and edge maps; they are folded in
// CTA order at the end (the reference folds per-chunk partials in chunk
// order, centrality.rs:669-679).  Scratch per CTA: distance, path count,
// factor c, the BFS order, the set-aside list and level offsets (40 bytes per
// vertex with the partial vertex map) plus 8 bytes per edge; G is cut to fit
// a memory budget.
#include <algorithm>
#include <vector>

#include "gtc_view.cuh"

namespace gtc {
namespace {

constexpr int BC_NT = 256;
constexpr int BC_WARPS = BC_NT / 32;
// A vertex of a level is walked by a group of BC_GL lanes; one with more
// than BC_HEAVY edges to walk is set aside and walked by a whole warp.
constexpr int BC_GL = 2;
constexpr int BC_GPW = 32 / BC_GL;             // groups per warp
constexpr uint32_t BC_HEAVY = 32;

struct BcArgs {
    uint32_t n, nsrc;
    const uint32_t* __restrict__ sources;  // null: every label 0 .. n-1
    const uint32_t* __restrict__ push_off;
    const uint32_t* __restrict__ push_other;
    const uint32_t* __restrict__ push_eid;
    const uint32_t* __restrict__ pull_off;
    const uint32_t* __restrict__ pull_other;
    const uint32_t* __restrict__ pull_eid;
    int undirected;
    // per CTA c: [c * n] slices (lvl: [c * (n + 2)], ebp: [c * m])
    int* dist;
    double* sigma;
    double* coef;  // (1 + dependency) / path count, once the dependency is final
    uint32_t* order;
    uint32_t* lvl;
    uint32_t* heavy;  // the vertices of the current phase set aside for whole warps
    double* vbp;
    double* ebp;
    uint64_t m;
};

// Calls f(other, eid) for every edge the BFS walks from u: the view's
// out-edges, and on the undirected view its in-edges too.  Lanes l, l + S,
// l + 2S, ... of the walkers.
template <class F>
__device__ __forceinline__ void walk_out(const BcArgs& A, uint32_t u, uint32_t l, uint32_t S,
                                         F&& f) {
    for (uint32_t p = A.push_off[u] + l, e = A.push_off[u + 1]; p < e; p += S)
        f(A.push_other[p], A.push_eid[p]);
    if (A.undirected)
        for (uint32_t p = A.pull_off[u] + l, e = A.pull_off[u + 1]; p < e; p += S)
            f(A.pull_other[p], A.pull_eid[p]);
}

// The edges into w: its in-edges, and on the undirected view its out-edges.
template <class F>
__device__ __forceinline__ void walk_in(const BcArgs& A, uint32_t w, uint32_t l, uint32_t S,
                                        F&& f) {
    for (uint32_t p = A.pull_off[w] + l, e = A.pull_off[w + 1]; p < e; p += S)
        f(A.pull_other[p]);
    if (A.undirected)
        for (uint32_t p = A.push_off[w] + l, e = A.push_off[w + 1]; p < e; p += S)
            f(A.push_other[p]);
}

__device__ __forceinline__ uint32_t out_walk_len(const BcArgs& A, uint32_t u) {
    uint32_t k = A.push_off[u + 1] - A.push_off[u];
    if (A.undirected) k += A.pull_off[u + 1] - A.pull_off[u];
    return k;
}

__device__ __forceinline__ uint32_t in_walk_len(const BcArgs& A, uint32_t w) {
    uint32_t k = A.pull_off[w + 1] - A.pull_off[w];
    if (A.undirected) k += A.push_off[w + 1] - A.push_off[w];
    return k;
}

// Sum over the BC_GL lanes of a group, by a fixed tree.
__device__ __forceinline__ double group_sum_f64(double v) {
#pragma unroll
    for (int o = BC_GL / 2; o > 0; o >>= 1) v = __dadd_rn(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

__device__ __forceinline__ double warp_sum_rn(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = __dadd_rn(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

__global__ void __launch_bounds__(BC_NT) k_bc(BcArgs A) {
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t grp = lane / BC_GL, gl = lane % BC_GL;
    const size_t c = blockIdx.x;
    int* dist = A.dist + c * A.n;
    double* sigma = A.sigma + c * A.n;
    double* coef = A.coef + c * A.n;
    uint32_t* order = A.order + c * A.n;
    uint32_t* lvl = A.lvl + c * ((size_t)A.n + 2);
    uint32_t* heavy = A.heavy + c * A.n;
    double* vbp = A.vbp + c * A.n;
    double* ebp = A.ebp + c * A.m;
    __shared__ uint32_t s_tail, s_heavy;

    // Runs one phase over order[lo .. hi): groups walk the light vertices,
    // then whole warps the heavy ones.  walk(u, l, S) returns the lane's
    // partial sum over u's edges; done(u, total) is called by one lane.
    auto phase = [&](uint32_t lo, uint32_t hi, bool in_dir, auto&& walk, auto&& done) {
        for (uint32_t base = lo + warp * BC_GPW; base < hi; base += BC_WARPS * BC_GPW) {
            const uint32_t i = base + grp;
            uint32_t u = 0;
            bool light = false;
            if (i < hi) {
                u = order[i];
                const uint32_t k = in_dir ? in_walk_len(A, u) : out_walk_len(A, u);
                light = k <= BC_HEAVY;
                if (!light && gl == 0) heavy[atomicAdd(&s_heavy, 1u)] = u;
            }
            double acc = light ? walk(u, gl, (uint32_t)BC_GL) : 0.0;
            acc = group_sum_f64(acc);
            if (light && gl == 0) done(u, acc);
        }
        __syncthreads();
        const uint32_t nh = s_heavy;
        __syncthreads();  // every thread has read the count: clear it for the next phase
        if (threadIdx.x == 0) s_heavy = 0;
        for (uint32_t j = warp; j < nh; j += BC_WARPS) {
            const uint32_t u = heavy[j];
            double acc = warp_sum_rn(walk(u, lane, 32u));
            if (lane == 0) done(u, acc);
        }
        __syncthreads();
    };

    if (threadIdx.x == 0) s_heavy = 0;
    for (uint32_t k = blockIdx.x; k < A.nsrc; k += gridDim.x) {
        const uint32_t s = A.sources ? A.sources[k] : k;
        if (threadIdx.x == 0) {
            order[0] = s;
            dist[s] = 0;
            sigma[s] = 1.0;
            lvl[0] = 0;
            lvl[1] = 1;
            s_tail = 1;
        }
        __syncthreads();
        uint32_t L = 0;  // the frontier is order[lvl[L] .. lvl[L + 1])
        for (;;) {
            const uint32_t lo = lvl[L], hi = lvl[L + 1];
            if (lo == hi) break;
            // expand: claim the unvisited targets for level L + 1
            phase(lo, hi, false,
                  [&](uint32_t u, uint32_t l, uint32_t S) {
                      walk_out(A, u, l, S, [&](uint32_t t, uint32_t) {
                          if (t == u) return;  // a self-loop never shortens a path
                          if (atomicCAS(dist + t, -1, (int)(L + 1)) == -1)
                              order[atomicAdd(&s_tail, 1u)] = t;
                      });
                      return 0.0;
                  },
                  [&](uint32_t, double) {});
            if (threadIdx.x == 0) lvl[L + 2] = s_tail;
            __syncthreads();
            // path counts of level L + 1, pulled from level L
            phase(hi, lvl[L + 2], true,
                  [&](uint32_t w, uint32_t l, uint32_t S) {
                      double acc = 0.0;
                      walk_in(A, w, l, S, [&](uint32_t x) {
                          if (dist[x] == (int)L) acc = __dadd_rn(acc, sigma[x]);
                      });
                      return acc;
                  },
                  [&](uint32_t w, double acc) { sigma[w] = acc; });
            ++L;
        }
        // L levels are non-empty (0 .. L-1); the deepest has no dependency
        for (uint32_t i = lvl[L - 1] + threadIdx.x; i < lvl[L]; i += BC_NT) {
            const uint32_t v = order[i];
            coef[v] = __ddiv_rn(1.0, sigma[v]);
        }
        __syncthreads();
        for (int lev = (int)L - 2; lev >= 0; --lev) {
            phase(lvl[lev], lvl[lev + 1], false,
                  [&](uint32_t v, uint32_t l, uint32_t S) {
                      const double sv = sigma[v];
                      double acc = 0.0;
                      walk_out(A, v, l, S, [&](uint32_t t, uint32_t e) {
                          if (t == v || dist[t] != lev + 1) return;
                          const double f = __dmul_rn(sv, coef[t]);
                          acc = __dadd_rn(acc, f);
                          ebp[e] = __dadd_rn(ebp[e], f);  // one term per edge and source
                      });
                      return acc;
                  },
                  [&](uint32_t v, double acc) {
                      coef[v] = __ddiv_rn(__dadd_rn(1.0, acc), sigma[v]);
                      if (v != s) vbp[v] = __dadd_rn(vbp[v], acc);
                  });
        }
        // clear what this source touched (coef is written before it is read)
        const uint32_t tot = lvl[L];
        for (uint32_t i = threadIdx.x; i < tot; i += BC_NT) {
            const uint32_t v = order[i];
            dist[v] = -1;
            sigma[v] = 0.0;
        }
        __syncthreads();
    }
}

// out[i] = (sum over CTAs in order of part[c][i]) * scale, vertex maps
// scattered back to the caller's labels (perm[internal] = original).
__global__ void k_bc_fold(uint64_t len, uint32_t G, const double* __restrict__ part,
                          double scale, const uint32_t* __restrict__ perm, double* __restrict__ out) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= len) return;
    double a = 0.0;
    for (uint32_t c = 0; c < G; ++c) a = __dadd_rn(a, part[(size_t)c * len + i]);
    a = __dmul_rn(a, scale);
    out[perm ? perm[i] : i] = a;
}

}  // namespace

void betweenness(gtc_graph* g, const gtc_view* vw, bool undirected, double* vb_host,
                 double* eb_host, gtc_result* res, cudaStream_t s) {
    uint64_t L = 0;
    View view;
    view.prepare(g, vw, s, &L);
    const uint32_t n = view.n;
    const uint64_t m = view.m_total;
    struct Events {
        cudaEvent_t a = nullptr, b = nullptr;
        ~Events() {
            if (a) cudaEventDestroy(a);
            if (b) cudaEventDestroy(b);
        }
    } ev;
    GTC_CUDA(cudaEventCreate(&ev.a));
    GTC_CUDA(cudaEventCreate(&ev.b));
    // the sources: every vertex of the view, in label order
    std::vector<uint32_t> src;
    DevBuf<uint32_t> d_src;
    uint32_t nsrc = n;
    if (view.active_or_null()) {
        std::vector<uint8_t> act(n);
        GTC_CUDA(cudaMemcpyAsync(act.data(), view.active_or_null(), n, cudaMemcpyDeviceToHost, s));
        GTC_CUDA(cudaStreamSynchronize(s));
        for (uint32_t v = 0; v < n; ++v)
            if (act[v]) src.push_back(v);
        nsrc = (uint32_t)src.size();
        d_src.alloc(src.size(), s);
        if (!src.empty())
            GTC_CUDA(cudaMemcpyAsync(d_src.get(), src.data(), src.size() * 4,
                                     cudaMemcpyHostToDevice, s));
    }
    // CTAs: as many as are resident at once (each runs its own sources), fewer
    // when the per-CTA scratch would pass a quarter of the free device memory
    const uint64_t per_cta = 40ull * n + 8 + 8ull * m;
    size_t free_b = 0, total_b = 0;
    GTC_CUDA(cudaMemGetInfo(&free_b, &total_b));
    const uint64_t budget = std::max<uint64_t>(free_b / 4, per_cta);
    int per_sm = 0;
    GTC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_bc, BC_NT, 0));
    uint64_t G = std::min<uint64_t>({(uint64_t)std::max(per_sm, 1) * sm_count(),
                                     std::max<uint32_t>(nsrc, 1u), budget / per_cta});
    G = std::max<uint64_t>(G, 1);
    DevBuf<int> dist(G * n, s);
    DevBuf<double> sigma(G * n, s), coef(G * n, s), vbp(G * n, s), ebp(G * m, s);
    DevBuf<uint32_t> order(G * n, s), heavy(G * n, s), lvl(G * ((uint64_t)n + 2), s);
    if (n) {
        GTC_CUDA(cudaMemsetAsync(dist.get(), 0xFF, G * n * sizeof(int), s));
        GTC_CUDA(cudaMemsetAsync(sigma.get(), 0, G * n * sizeof(double), s));
        GTC_CUDA(cudaMemsetAsync(vbp.get(), 0, G * n * sizeof(double), s));
    }
    if (m) GTC_CUDA(cudaMemsetAsync(ebp.get(), 0, G * m * sizeof(double), s));
    GTC_CUDA(cudaEventRecord(ev.a, s));
    if (n && nsrc) {
        BcArgs A;
        A.n = n;
        A.nsrc = nsrc;
        A.sources = src.empty() && !view.active_or_null() ? nullptr : d_src.get();
        A.push_off = view.push_off, A.push_other = view.push_other, A.push_eid = view.push_eid;
        A.pull_off = view.pull_off, A.pull_other = view.pull_other, A.pull_eid = view.pull_eid;
        A.undirected = undirected ? 1 : 0;
        A.dist = dist.get(), A.sigma = sigma.get(), A.coef = coef.get();
        A.order = order.get(), A.lvl = lvl.get(), A.heavy = heavy.get();
        A.vbp = vbp.get(), A.ebp = ebp.get();
        A.m = m;
        k_bc<<<(unsigned)G, BC_NT, 0, s>>>(A);
        GTC_LAUNCHED();
        L++;
    }
    const double scale = undirected ? 0.5 : 1.0;  // divide_centrality_by_two
    DevBuf<double> vout(n, s), eout(m, s);
    if (n) {
        k_bc_fold<<<grid_for(n, 256, 1u << 30), 256, 0, s>>>(n, (uint32_t)G, vbp.get(), scale,
                                                            g->perm.get(), vout.get());
        GTC_LAUNCHED();
        L++;
    }
    if (m) {
        k_bc_fold<<<grid_for(m, 256, 1u << 30), 256, 0, s>>>(m, (uint32_t)G, ebp.get(), scale,
                                                            nullptr, eout.get());
        GTC_LAUNCHED();
        L++;
    }
    GTC_CUDA(cudaEventRecord(ev.b, s));
    if (vb_host && n)
        GTC_CUDA(cudaMemcpyAsync(vb_host, vout.get(), (size_t)n * 8, cudaMemcpyDeviceToHost, s));
    if (eb_host && m)
        GTC_CUDA(cudaMemcpyAsync(eb_host, eout.get(), (size_t)m * 8, cudaMemcpyDeviceToHost, s));
    GTC_CUDA(cudaStreamSynchronize(s));
    if (res) {
        float ms = 0.f;
        GTC_CUDA(cudaEventElapsedTime(&ms, ev.a, ev.b));
        *res = gtc_result{};
        res->iterations = nsrc;  // sources run
        res->device_ms = ms;
        res->launches = L;
    }
}

}  // namespace gtc
