// gtc_centrality.cu -- PageRank and eigenvector centrality on one GB300.
//
// The sweeps of crates/gt-algo/src/centrality.rs, in two arithmetics:
//
// GTC_PREC_F32 (the fast path).  Vectors and edge weights in FP32, the row
// sum of a pull as a compensated (TwoSum-based) FP32 sum, the dangling mass
// and the L1 delta folded in FP64 across blocks.  PageRank pulls
// y[s] = rank[s] / deg[s] (written by the previous sweep's epilogue), so the
// edge loop is one index load, one gather and, when weighted, one weight
// load per in-edge.  The sweep is fused: pull + damping + delta + next
// sweep's dangling mass in one kernel, reduced deterministically (per-block
// partials, folded in block order by the last block to finish).
//
// GTC_PREC_F64_EXACT.  The reference's arithmetic step for step: per-edge
// `(prev[s] * w) / ds` (centrality.rs:361), `nv = (1-d)*pv + d*r` (:364), the
// delta folded sequentially inside each Plan chunk and the chunk partials
// left-folded from 0.0 (sweep, :141-167; det_reduce, reduce.rs:40-55).  IEEE
// round-to-nearest intrinsics keep the compiler from fusing a multiply into
// an add.  Results are bit-identical to the reference's for the same Plan.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <utility>
#include <vector>

#include "gtc_sweep.cuh"
#include "gtc_view.cuh"

namespace gtc {

constexpr int PR_NT = 256;

// --------------------------------------------------------------------------
// per-call preparation kernels
// --------------------------------------------------------------------------

// deg[v]: Unity -> the view's out-degree; weighted -> a left fold of the
// view's out-edge weights in storage order, FP64, as centrality.rs:281-297.
__global__ void k_degree(uint32_t n, const uint32_t* __restrict__ push_off,
                         const uint32_t* __restrict__ push_eid, const void* __restrict__ w,
                         int wdt, const uint8_t* __restrict__ active, double* __restrict__ deg,
                         uint8_t* __restrict__ sink) {
    size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n) return;
    const uint32_t b = push_off[v], e = push_off[v + 1];
    double k;
    if (!w) {
        k = (double)(e - b);
    } else {
        k = 0.0;
        for (uint32_t p = b; p < e; ++p) k = __dadd_rn(k, ld_any(w, wdt, push_eid[p]));
    }
    const bool act = !active || active[v];
    deg[v] = act ? k : 0.0;
    sink[v] = (act && k == 0.0) ? 1 : 0;
}

// Merge a compensated partial over the 8 lanes of a lane group (fixed order).
__device__ __forceinline__ void group8_merge_kahan(Kahan& k) {
#pragma unroll
    for (int o = 4; o > 0; o >>= 1) {
        const float os = __shfl_xor_sync(0xffffffffu, k.s, o, 8);
        const float oc = __shfl_xor_sync(0xffffffffu, k.c, o, 8);
        k.merge(os, oc);
    }
}

// The FP32 path's weighted out-degree from the weights gathered in out-half
// order (wout[p] = w[push_eid[p]]): 8 lanes per vertex (4 vertices per
// warp), compensated FP32 sums merged in a fixed shuffle order.  (The FP64
// path keeps the reference's sequential fold above.)  The forward solve and
// the adjoint both use it, so their degrees have the same bits.
__global__ void k_degree_f32(uint32_t n, const uint32_t* __restrict__ push_off,
                             const float* __restrict__ wout, const uint8_t* __restrict__ active,
                             double* __restrict__ deg, uint8_t* __restrict__ sink) {
    const uint32_t sub = threadIdx.x & 7;
    const size_t v = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 3;
    const bool in = v < n;  // whole groups leave together: the shuffles stay full-warp
    KahanBlocked kb;
    if (in) {
        const uint32_t b = push_off[v], e = push_off[v + 1];
        uint32_t p = b + sub;
        for (; p + 24 < e; p += 32) {  // four loads in flight
            const float x0 = wout[p], x1 = wout[p + 8], x2 = wout[p + 16], x3 = wout[p + 24];
            kb.add(x0), kb.add(x1), kb.add(x2), kb.add(x3);
        }
        for (; p < e; p += 8) kb.add(wout[p]);
    }
    Kahan k = kb.fold();
    group8_merge_kahan(k);
    if (in && sub == 0) {
        const double kd = (double)k.s + (double)k.c;
        const bool act = !active || active[v];
        deg[v] = act ? kd : 0.0;
        sink[v] = (act && kd == 0.0) ? 1 : 0;
    }
}

__global__ void k_invdeg_f32(uint32_t n, const double* __restrict__ deg,
                             float* __restrict__ invdeg) {
    size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v < n) invdeg[v] = deg[v] != 0.0 ? (float)(1.0 / deg[v]) : 0.f;
}

// Weights into pull order (the order the sweep streams them).
template <class T>
__global__ void k_gather_w(uint32_t m, const uint32_t* __restrict__ eid,
                           const void* __restrict__ w, int wdt, T* __restrict__ out) {
    size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= m) return;
    if (sizeof(T) == 4)
        out[p] = (T)ld_f32(w, wdt, eid[p]);
    else
        out[p] = (T)ld_any(w, wdt, eid[p]);
}

// Initial iterate (FP64, internal labels): slots below `had` come from the
// caller's map, the rest are seeded (seed_new_slots, centrality.rs:198-205).
// The caller's maps are by original index: internal slot i is vertex perm[i].
__global__ void k_seed(uint32_t n, const uint32_t* __restrict__ perm, uint64_t had,
                       const void* __restrict__ x, int xdt, const void* __restrict__ pers, int pdt,
                       double uniform, double* __restrict__ x64) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t v = perm[i];
    x64[i] = v < had ? ld_any(x, xdt, v) : (pers ? ld_any(pers, pdt, v) : uniform);
}

// k_seed's pick for internal slot i (vertex o = perm[i]), rounded to FP32.
__device__ __forceinline__ float seed_f32(uint32_t o, uint64_t had, const void* __restrict__ x,
                                          int xdt, const void* __restrict__ pers, int pdt,
                                          float uniform) {
    return o < had ? ld_f32(x, xdt, o) : (pers ? ld_f32(pers, pdt, o) : uniform);
}

// The initial iterate straight into FP32, for a loop that keeps no FP64 copy
// (perm null: no map is read, every slot is seeded uniform).
__global__ void k_seed_f32(uint32_t n, const uint32_t* __restrict__ perm, uint64_t had,
                           const void* __restrict__ x, int xdt, const void* __restrict__ pers,
                           int pdt, float uniform, float* __restrict__ y) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = perm ? seed_f32(perm[i], had, x, xdt, pers, pdt, uniform) : uniform;
}

// The label map k_seed_f32 and k_pr_seed read the caller's maps through: none
// when no map is read.
inline const uint32_t* seed_perm(const gtc_graph* g, const SolveIn& in) {
    return (in.had > 0 || in.pers.present()) ? g->perm.get() : nullptr;
}

// FP32 copy; with `perm` the source is in original labels.
__global__ void k_to_f32(uint32_t n, const void* __restrict__ x, int xdt,
                         const uint32_t* __restrict__ perm, float* __restrict__ y) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = ld_f32(x, xdt, perm ? perm[i] : i);
}

// Store an iterate into the caller's map, in the map's type.  Slots of
// vertices outside a filtered view keep their FP64 initial value exactly (the
// reference carries them through untouched, centrality.rs:345-351).
template <class T>
__global__ void k_store(uint32_t n, const uint32_t* __restrict__ iperm, const T* __restrict__ src,
                        const uint8_t* __restrict__ active, const double* __restrict__ x64,
                        void* __restrict__ x, int xdt) {
    size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n) return;
    const uint32_t i = iperm[v];
    const double val = (active && !active[i]) ? x64[i] : (double)src[i];
    if (xdt == GTC_F64)
        ((double*)x)[v] = val;
    else
        ((float*)x)[v] = (float)val;
}

// y = rank * invdeg, plus the dangling mass of rank (summed exactly).
__global__ void __launch_bounds__(PR_NT) k_pr_prime(uint32_t n, const float* __restrict__ r,
                                                   const float* __restrict__ invdeg,
                                                   const uint8_t* __restrict__ sink,
                                                   float* __restrict__ y, ExactFold f) {
    ExactPR none, sacc;
    for (size_t v = (size_t)blockIdx.x * PR_NT + threadIdx.x; v < n;
         v += (size_t)gridDim.x * PR_NT) {
        float x = r[v];
        y[v] = __fmul_rn(x, invdeg[v]);
        if (sink[v]) sacc.add(x);
    }
    block_fold_exact<PR_NT>(none, sacc, f);
}

// The FP32 PageRank loop's first iterate in one pass: r = the initial iterate
// rounded to FP32 (from x64 when given, else picked as k_seed picks it),
// y = r * invdeg, yz = 0 on the dangling rows (a sweep stores no y there),
// entry n of both gathered vectors 0 (the slices' padding gathers it), and
// the dangling mass of r summed exactly.  perm null: no map is read, every
// slot is seeded uniform.
__global__ void __launch_bounds__(PR_NT) k_pr_seed(
    uint32_t n, const double* __restrict__ x64, const uint32_t* __restrict__ perm, uint64_t had,
    const void* __restrict__ x, int xdt, const void* __restrict__ pers, int pdt, float uniform,
    const float* __restrict__ invdeg, const uint8_t* __restrict__ sink, float* __restrict__ r,
    float* __restrict__ y, float* __restrict__ yz, ExactFold f) {
    ExactPR none, sacc;
    if (blockIdx.x == 0 && threadIdx.x == 0) y[n] = 0.f, yz[n] = 0.f;
    for (size_t v = (size_t)blockIdx.x * PR_NT + threadIdx.x; v < n;
         v += (size_t)gridDim.x * PR_NT) {
        const float xv = x64    ? (float)x64[v]
                         : perm ? seed_f32(perm[v], had, x, xdt, pers, pdt, uniform)
                                : uniform;
        r[v] = xv;
        y[v] = __fmul_rn(xv, invdeg[v]);
        if (sink[v]) {
            yz[v] = 0.f;
            sacc.add(xv);
        }
    }
    block_fold_exact<PR_NT>(none, sacc, f);
}

// --------------------------------------------------------------------------
// FP64 exact kernels
// --------------------------------------------------------------------------

// Plan::range (plan.rs:88-101)
__device__ __forceinline__ void plan_range(uint64_t n, uint64_t chunks, uint64_t k, uint64_t& s,
                                           uint64_t& e) {
    uint64_t base = n / chunks, rem = n % chunks;
    s = k * base + (k < rem ? k : rem);
    e = s + base + (k < rem ? 1 : 0);
}

// Weighted views: one thread per row, the in-edge loop sequential in storage
// order; rows of more than F64_SHORT entries are summed by a warp
// (k_pr_f64_long, k_ev_f64_long), whose 32 lanes form 32 terms per divide
// or multiply instruction.  Unweighted views: a thread per row of any length
// (k_pr_f64_rows_q, k_ev_f64_rows_u), the terms needing no per-edge FP64 work.
constexpr uint32_t F64_SHORT = 32;

// FP64 on this GPU: an add has a latency of about 64 cycles, and a warp
// instruction costs the FP64 pipe the same whether one lane or 32 are active
// (about 80 cycles of a sub-partition's pipe).  So a sequential fold (the
// reference's left fold, which fixes the bits) is cheapest with one chain
// per lane -- a thread per row or per chunk -- and its latency is hidden by
// keeping the next terms' loads in flight while a block of terms is added.

// acc + term(b) + term(b + 1) + ... + term(e - 1), added left to right.
// idx(p) loads the index of entry p, val(j) the term of index j.  While a
// block of FU terms is added, the terms of the next FD blocks and the
// indices of the one after those are loading, so a long chain of adds waits
// on no load (FD blocks of adds take longer than a gather from DRAM).
constexpr int FU = 8;
template <int FD, class Idx, class Val>
__device__ __forceinline__ double fold_seq(double acc, uint64_t b, uint64_t e, Idx&& idx,
                                           Val&& val) {
    double t[FD + 1][FU];
    uint32_t sn[FU];
#pragma unroll
    for (int k = 0; k < FD; ++k)
#pragma unroll
        for (int j = 0; j < FU; ++j) {
            const uint64_t p = b + (uint64_t)k * FU + j;
            const uint32_t si = p < e ? idx(p) : 0u;
            t[k][j] = p < e ? val(si) : 0.0;
        }
#pragma unroll
    for (int j = 0; j < FU; ++j) {
        const uint64_t p = b + (uint64_t)FD * FU + j;
        sn[j] = p < e ? idx(p) : 0u;
    }
    for (uint64_t p = b; p < e; p += FU) {
#pragma unroll
        for (int j = 0; j < FU; ++j) t[FD][j] = p + FD * FU + j < e ? val(sn[j]) : 0.0;
#pragma unroll
        for (int j = 0; j < FU; ++j) {
            const uint64_t q = p + (FD + 1) * FU + j;
            sn[j] = q < e ? idx(q) : 0u;
        }
#pragma unroll
        for (int j = 0; j < FU; ++j)
            if (p + j < e) acc = __dadd_rn(acc, t[0][j]);
#pragma unroll
        for (int k = 0; k < FD; ++k)
#pragma unroll
            for (int j = 0; j < FU; ++j) t[k][j] = t[k + 1][j];
    }
    return acc;
}

// Unweighted views: the reference's term (prev[s] * 1.0) / ds is prev[s] / ds,
// one value per source, so it is formed once per sweep here instead of once
// per edge.  Every source an active row gathers has ds >= 1 (in the view it
// keeps at least its edge into that row), so the reference's ds != 0 test
// never skips a term of these rows.
__global__ void k_pr_f64_q(uint32_t n, const double* __restrict__ prev,
                           const double* __restrict__ deg, double* __restrict__ q) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) q[i] = deg[i] != 0.0 ? __ddiv_rn(prev[i], deg[i]) : 0.0;
}

// Unweighted rows, every length: a thread per row folds q over its in-edges
// in storage order (centrality.rs:355-365).
__global__ void __launch_bounds__(128) k_pr_f64_rows_q(
    uint32_t n, const uint32_t* __restrict__ off, const uint32_t* __restrict__ other,
    const double* __restrict__ q, const uint8_t* __restrict__ active,
    const double* __restrict__ pers, double uniform, double one_minus_d, double d,
    const double* __restrict__ psink_p, const double* __restrict__ prev,
    double* __restrict__ next, double* __restrict__ diff) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (active && !active[i]) {
        next[i] = prev[i];
        diff[i] = 0.0;
        return;
    }
    const double pv = pers ? pers[i] : uniform;
    double r = __dmul_rn(*psink_p, pv);
    // one block of lookahead: deeper ones cost the short rows occupancy (a
    // long row's chain is bound by the FP64 pipe, not by its loads)
    r = fold_seq<1>(r, off[i], off[i + 1], [&](uint64_t p) { return other[p]; },
                 [&](uint32_t src) { return q[src]; });
    const double nv = __dadd_rn(__dmul_rn(one_minus_d, pv), __dmul_rn(d, r));
    diff[i] = fabs(__dsub_rn(nv, prev[i]));
    next[i] = nv;
}

// acc + t(lane 0) + t(lane 1) + ... + t(lane 31), left to right, skipping the
// lanes whose bit of `valid` is clear: the sequential fold of 32 terms the
// lanes computed in parallel.  Every lane ends with the same acc.
__device__ __forceinline__ double fold_lanes_in_order(double acc, double t, unsigned valid) {
#pragma unroll
    for (int k = 0; k < 32; ++k) {
        const double tk = __shfl_sync(0xffffffffu, t, k);
        if ((valid >> k) & 1u) acc = __dadd_rn(acc, tk);
    }
    return acc;
}

__global__ void k_pr_f64_rows(uint32_t n, const uint32_t* __restrict__ off,
                              const uint32_t* __restrict__ other, const double* __restrict__ w,
                              const double* __restrict__ deg, const uint8_t* __restrict__ active,
                              const double* __restrict__ pers, double uniform, double one_minus_d,
                              double d, const double* __restrict__ psink_p,
                              const double* __restrict__ prev, double* __restrict__ next,
                              double* __restrict__ diff) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (off[i + 1] - off[i] > F64_SHORT) return;  // k_pr_f64_long's
    if (active && !active[i]) {
        next[i] = prev[i];
        diff[i] = 0.0;
        return;
    }
    const double p_sink = *psink_p;
    const double pv = pers ? pers[i] : uniform;
    double r = __dmul_rn(p_sink, pv);
    for (uint32_t p = off[i], e = off[i + 1]; p < e; ++p) {
        const uint32_t s = other[p];
        const double ds = deg[s];
        if (ds != 0.0) {
            const double we = w ? w[p] : 1.0;
            r = __dadd_rn(r, __ddiv_rn(__dmul_rn(prev[s], we), ds));
        }
    }
    const double nv = __dadd_rn(__dmul_rn(one_minus_d, pv), __dmul_rn(d, r));
    diff[i] = fabs(__dsub_rn(nv, prev[i]));
    next[i] = nv;
}

// The rows k_pr_f64_rows leaves (more than F64_SHORT entries): a warp per
// row.  Lanes gather and form 32 terms (prev[s] * w) / ds at a time; the
// terms are then added to r one after the other in entry order, as the
// reference's loop does, so r has the same bits.
__global__ void k_pr_f64_long(uint32_t n, const uint32_t* __restrict__ off,
                              const uint32_t* __restrict__ other, const double* __restrict__ w,
                              const double* __restrict__ deg, const uint8_t* __restrict__ active,
                              const double* __restrict__ pers, double uniform, double one_minus_d,
                              double d, const double* __restrict__ psink_p,
                              const double* __restrict__ prev, double* __restrict__ next,
                              double* __restrict__ diff) {
    const unsigned lane = threadIdx.x & 31;
    const size_t warps = ((size_t)gridDim.x * blockDim.x) >> 5;
    for (size_t i = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < n; i += warps) {
        const uint32_t b = off[i], e = off[i + 1];
        if (e - b <= F64_SHORT) continue;
        if (active && !active[i]) {
            if (lane == 0) next[i] = prev[i], diff[i] = 0.0;
            continue;
        }
        const double pv = pers ? pers[i] : uniform;
        double r = __dmul_rn(*psink_p, pv);
        // Lane l's entry of chunk k is b + 32k + l.  While chunk k is folded,
        // chunk k + 1's gathers and chunk k + 2's sources are loading; chunk
        // k + 1's terms are formed after the fold, once those have arrived.
        auto src_at = [&](uint32_t p) { return p < e ? other[p] : 0u; };
        auto term = [&](uint32_t p, double pr, double ds, bool& ok) {
            ok = p < e && ds != 0.0;
            return ok ? __ddiv_rn(__dmul_rn(pr, w ? w[p] : 1.0), ds) : 0.0;
        };
        bool ok;
        double t;
        {
            const uint32_t p = b + lane, s0 = src_at(p);
            t = term(p, p < e ? prev[s0] : 0.0, p < e ? deg[s0] : 0.0, ok);
        }
        uint32_t s1 = src_at(b + 32 + lane);
        for (uint32_t base = b; base < e; base += 32) {
            const uint32_t p1 = base + 32 + lane;
            const double pr1 = p1 < e ? prev[s1] : 0.0, ds1 = p1 < e ? deg[s1] : 0.0;
            const uint32_t s2 = src_at(base + 64 + lane);
            r = fold_lanes_in_order(r, t, __ballot_sync(0xffffffffu, ok));
            t = term(p1, pr1, ds1, ok);
            s1 = s2;
        }
        if (lane == 0) {
            const double nv = __dadd_rn(__dmul_rn(one_minus_d, pv), __dmul_rn(d, r));
            diff[i] = fabs(__dsub_rn(nv, prev[i]));
            next[i] = nv;
        }
    }
}

// Plan-chunk partials: a thread per chunk folds it sequentially from 0.0, in
// index order (values through `gather` when given).
__global__ void __launch_bounds__(32) k_chunk_sums(uint64_t n, uint64_t chunks,
                                                   const double* __restrict__ v,
                                                   const uint32_t* __restrict__ gather,
                                                   double* __restrict__ part) {
    const uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= chunks) return;
    uint64_t s, e;
    plan_range(n, chunks, k, s, e);
    part[k] = gather ? fold_seq<4>(0.0, s, e, [&](uint64_t i) { return gather[i]; },
                                   [&](uint32_t j) { return v[j]; })
                     : fold_seq<4>(0.0, s, e, [&](uint64_t i) { return (uint32_t)i; },
                                   [&](uint32_t j) { return v[j]; });
}

// Left fold of the chunk partials from 0.0 (one warp, adds in order).  mode 0: out = sum;
// mode 1: out = sum and out2 = the eigenvector scale (sqrt, 1 if zero).
__global__ void k_fold(uint64_t chunks, const double* __restrict__ part, double* out,
                       double* out2, int mode) {
    if (blockIdx.x != 0 || threadIdx.x >= 32) return;
    const unsigned lane = threadIdx.x;
    double acc = 0.0;
    for (uint64_t base = 0; base < chunks; base += 32) {
        const bool ok = base + lane < chunks;
        acc = fold_lanes_in_order(acc, ok ? part[base + lane] : 0.0, __ballot_sync(0xffffffffu, ok));
    }
    if (lane != 0) return;
    *out = acc;
    if (mode == 1) {
        double norm = __dsqrt_rn(acc);
        out[1] = norm;
        *out2 = norm == 0.0 ? 1.0 : norm;
    }
}

// The sinks in original vertex order (the reference's `sinks` list,
// centrality.rs:281-297), as internal labels for gathering.
__global__ void k_compact_sinks(uint32_t n, const uint32_t* __restrict__ flag,
                                const uint32_t* __restrict__ iperm,
                                const uint32_t* __restrict__ pos, uint32_t* __restrict__ list) {
    size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v < n && flag[v]) list[pos[v]] = iperm[v];
}

// flag[v] (original order) = sink[iperm[v]]
__global__ void k_sink_flags(uint32_t n, const uint32_t* __restrict__ iperm,
                             const uint8_t* __restrict__ sink, uint32_t* __restrict__ flag) {
    size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v < n) flag[v] = sink[iperm[v]];
}

// Eigenvector sweep 1 (centrality.rs:446-465): s = sum w*prev[other] in
// storage order, sq[i] = s*s.
__global__ void k_ev_f64_rows(uint32_t n, const uint32_t* __restrict__ off,
                              const uint32_t* __restrict__ other, const double* __restrict__ w,
                              const uint8_t* __restrict__ active, const double* __restrict__ prev,
                              double* __restrict__ next, double* __restrict__ sq) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (off[i + 1] - off[i] > F64_SHORT) return;  // k_ev_f64_long's
    if (active && !active[i]) {
        next[i] = prev[i];
        sq[i] = 0.0;
        return;
    }
    double s = 0.0;
    for (uint32_t p = off[i], e = off[i + 1]; p < e; ++p) {
        const double we = w ? w[p] : 1.0;
        s = __dadd_rn(s, __dmul_rn(we, prev[other[p]]));
    }
    next[i] = s;
    sq[i] = __dmul_rn(s, s);
}

// Unweighted rows, every length: a thread per row folds prev over its
// in-edges in storage order from 0.0 (the reference's 1.0 * prev[s] is
// prev[s]).
__global__ void __launch_bounds__(128) k_ev_f64_rows_u(uint32_t n, const uint32_t* __restrict__ off,
                                                       const uint32_t* __restrict__ other,
                                                       const uint8_t* __restrict__ active,
                                                       const double* __restrict__ prev,
                                                       double* __restrict__ next,
                                                       double* __restrict__ sq) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (active && !active[i]) {
        next[i] = prev[i];
        sq[i] = 0.0;
        return;
    }
    const double s = fold_seq<1>(0.0, off[i], off[i + 1], [&](uint64_t p) { return other[p]; },
                                 [&](uint32_t src) { return prev[src]; });
    next[i] = s;
    sq[i] = __dmul_rn(s, s);
}

// The rows k_ev_f64_rows leaves: a warp per row, terms w * prev[other]
// formed 32 at a time and added in entry order.
__global__ void k_ev_f64_long(uint32_t n, const uint32_t* __restrict__ off,
                              const uint32_t* __restrict__ other, const double* __restrict__ w,
                              const uint8_t* __restrict__ active, const double* __restrict__ prev,
                              double* __restrict__ next, double* __restrict__ sq) {
    const unsigned lane = threadIdx.x & 31;
    const size_t warps = ((size_t)gridDim.x * blockDim.x) >> 5;
    for (size_t i = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < n; i += warps) {
        const uint32_t b = off[i], e = off[i + 1];
        if (e - b <= F64_SHORT) continue;
        if (active && !active[i]) {
            if (lane == 0) next[i] = prev[i], sq[i] = 0.0;
            continue;
        }
        // chunk k + 1's gathers and chunk k + 2's sources load while chunk k
        // is folded (as in k_pr_f64_long)
        auto src_at = [&](uint32_t p) { return p < e ? other[p] : 0u; };
        auto term = [&](uint32_t p, double pr) {
            return p < e ? __dmul_rn(w ? w[p] : 1.0, pr) : 0.0;
        };
        double s = 0.0;
        double t;
        {
            const uint32_t p = b + lane, s0 = src_at(p);
            t = term(p, p < e ? prev[s0] : 0.0);
        }
        uint32_t s1 = src_at(b + 32 + lane);
        for (uint32_t base = b; base < e; base += 32) {
            const uint32_t p = base + lane, p1 = p + 32;
            const double pr1 = p1 < e ? prev[s1] : 0.0;
            const uint32_t s2 = src_at(base + 64 + lane);
            s = fold_lanes_in_order(s, t, __ballot_sync(0xffffffffu, p < e));
            t = term(p1, pr1);
            s1 = s2;
        }
        if (lane == 0) {
            next[i] = s;
            sq[i] = __dmul_rn(s, s);
        }
    }
}

// Eigenvector sweep 2 (centrality.rs:472-484): next /= scale, |next - prev|.
__global__ void k_ev_f64_norm(uint32_t n, const uint8_t* __restrict__ active,
                              const double* __restrict__ scale_p, const double* __restrict__ prev,
                              double* __restrict__ next, double* __restrict__ diff) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (active && !active[i]) {
        diff[i] = 0.0;
        return;
    }
    const double x = __ddiv_rn(next[i], *scale_p);
    next[i] = x;
    diff[i] = fabs(__dsub_rn(x, prev[i]));
}

// --------------------------------------------------------------------------
// FP32 eigenvector
// --------------------------------------------------------------------------

// next /= scale (scale from the FP64 norm, 1 if zero) and the L1 change,
// summed exactly.
// The FP64 reciprocal is applied as an unevaluated sum hi + lo of two floats,
// so the stored value is (nearly always) the correctly rounded s / norm: a
// last-bit change of the norm between sweeps does not move every entry by an
// ulp, which would put a floor of ~sqrt(n) * 2^-24 under the L1 change.
__global__ void __launch_bounds__(PR_NT) k_ev_f32_norm(uint32_t n,
                                                      const uint8_t* __restrict__ active,
                                                      const double* __restrict__ sqnorm,
                                                      const float* __restrict__ prev,
                                                      float* __restrict__ next, ExactFold f) {
    if (f.stop && *f.stop) return;  // the iteration has stopped (same for every CTA)
    const double norm = sqrt(*sqnorm);
    const double inv = 1.0 / (norm == 0.0 ? 1.0 : norm);
    const float ih = (float)inv;
    const float il = (float)(inv - (double)ih);
    ExactPR dacc, none;
    for (size_t v = (size_t)blockIdx.x * PR_NT + threadIdx.x; v < n;
         v += (size_t)gridDim.x * PR_NT) {
        if (active && !active[v]) continue;
        const float sv = next[v];
        const float x = __fmaf_rn(sv, ih, __fmul_rn(sv, il));
        next[v] = x;
        dacc.add(fabsf(__fsub_rn(x, prev[v])));
    }
    block_fold_exact<PR_NT>(dacc, none, f);
}

// --------------------------------------------------------------------------
// host drivers
// --------------------------------------------------------------------------

namespace {

struct Timer {
    cudaEvent_t a = nullptr, b = nullptr;
    cudaStream_t s;
    explicit Timer(cudaStream_t st) : s(st) {
        GTC_CUDA(cudaEventCreate(&a));
        GTC_CUDA(cudaEventCreate(&b));
    }
    ~Timer() {
        if (a) cudaEventDestroy(a);
        if (b) cudaEventDestroy(b);
    }
    void start() { GTC_CUDA(cudaEventRecord(a, s)); }
    void stop() { GTC_CUDA(cudaEventRecord(b, s)); }
    // after the stream has passed stop()
    double ms() {
        GTC_CUDA(cudaEventSynchronize(b));
        float t = 0.f;
        GTC_CUDA(cudaEventElapsedTime(&t, a, b));
        return t;
    }
};

// Reduction scratch of one exactly-folded launch (at most FOLD_MAX_CTAS CTAs).
struct FoldBufs {
    DevBuf<uint4> part;
    DevBuf<double> out;
    DevBuf<unsigned> ticket;
    FoldBufs(unsigned blocks, cudaStream_t s)
        : part(2 * (size_t)std::max(blocks, 1u), s), out(4, s), ticket(1, s) {
        GTC_REQUIRE(blocks <= FOLD_MAX_CTAS, GTC_ERR_ARG, "grid exceeds the fold capacity");
        GTC_CUDA(cudaMemsetAsync(ticket.get(), 0, sizeof(unsigned), s));
        GTC_CUDA(cudaMemsetAsync(out.get(), 0, 4 * sizeof(double), s));
    }
    ExactFold fold(double* oa, double* ob) { return ExactFold{part.get(), ticket.get(), oa, ob}; }
};

unsigned persistent_blocks(uint32_t rows) {
    // one row per warp, at most 8 resident blocks of 256 threads per SM
    unsigned want = (rows + (PR_NT / 32) - 1) / (PR_NT / 32);
    unsigned cap = std::min<unsigned>((unsigned)sm_count() * 8, FOLD_MAX_CTAS);
    return want < 1 ? 1 : (want > cap ? cap : want);
}

// Sweeps a host loop enqueues between two reads of the device-side stop
// flag: a sweep after the stop returns at once, so at most STOP_BATCH - 1
// launches are wasted, against one host round trip per sweep saved.
constexpr int STOP_BATCH = 8;

// Device-side state of a power iteration's stop (ExactFold::stop/iters).
struct StopState {
    DevBuf<unsigned long long> words;  // [0] stop flag, [1] sweeps done
    explicit StopState(cudaStream_t s) : words(2, s) {
        GTC_CUDA(cudaMemsetAsync(words.get(), 0, 2 * sizeof(unsigned long long), s));
    }
    unsigned* stop() { return reinterpret_cast<unsigned*>(words.get()); }
    unsigned long long* iters() { return words.get() + 1; }
    void arm(ExactFold& f, double eps, uint64_t max_iter) {
        f.stop = stop();
        f.iters = iters();
        f.eps = eps;
        f.max_iter = max_iter;
    }
    // (stop flag, sweeps done), after the stream has reached this point
    std::pair<bool, uint64_t> read(cudaStream_t s) {
        unsigned long long h[2] = {0, 0};
        GTC_CUDA(cudaMemcpyAsync(h, words.get(), sizeof(h), cudaMemcpyDeviceToHost, s));
        GTC_CUDA(cudaStreamSynchronize(s));
        return {(h[0] & 0xFFFFFFFFull) != 0, h[1]};
    }
};

// Per-launch CUDA events of the sweeps of a batched loop; only the sweeps
// that ran (the first `done`) are summed.
struct SweepEvents {
    std::vector<cudaEvent_t> ev;
    ~SweepEvents() {
        for (cudaEvent_t e : ev) cudaEventDestroy(e);
    }
    void record(cudaStream_t s) {
        cudaEvent_t e = nullptr;
        GTC_CUDA(cudaEventCreate(&e));
        ev.push_back(e);
        GTC_CUDA(cudaEventRecord(e, s));
    }
    // events come in (start, stop) pairs, one pair per launch
    double ms(uint64_t done) {
        double t = 0.0;
        for (uint64_t k = 0; k < done && 2 * k + 1 < ev.size(); ++k) {
            GTC_CUDA(cudaEventSynchronize(ev[2 * k + 1]));
            float x = 0.f;
            GTC_CUDA(cudaEventElapsedTime(&x, ev[2 * k], ev[2 * k + 1]));
            t += x;
        }
        return t;
    }
};

// The pull schedule of a view: cached on the graph for the plain and the
// reversed view, cut per call for a filtered one.
Units* pull_units(gtc_graph* g, const View& view, Units& local, cudaStream_t s) {
    if (!view.filtered) {
        Units& u = view.reversed ? g->units_out : g->units_in;
        if (!u.built) {
            GTC_CUDA(cudaStreamSynchronize(s));
            build_units(view.pull_off, view.pull_other, view.pull_eid, view.n, g->home, u);
        }
        return &u;
    }
    build_units(view.pull_off, view.pull_other, view.pull_eid, view.n, s, local);
    return &local;
}

// Entries staged in shared memory by the HOT variant: the whole vector when
// it fits, else the hottest prefix; a multiple of 4 (float4 staging).
inline uint32_t hot_entries(uint32_t n) {
    const uint32_t h = n < (uint32_t)SP_HOT ? n : (uint32_t)SP_HOT;
    return h & ~3u;
}

// The kernel variants the autotuner chooses between.  They compute
// bit-identical results (the same per-item order and fold); they differ in
// where the gathers of the hottest entries are served:
//   VAR_L1     256-thread CTAs, 6 per SM, every gather through L1/L2
//   VAR_HOT    one 1024-thread CTA per SM, the first 32,768 entries of the
//              gathered vector (labels follow out-degree, so the most
//              gathered ones) in its shared memory
//   VAR_HOT24  the same kernel with 24,576,
//   VAR_HOT16  16,384
//   VAR_HOT8   and 8,192 hot entries: less shared memory leaves more of the
//              SM's L1 to the gathers in flight, which can matter more than
//              the entries given up (it does on the R-MAT and Chung-Lu
//              graphs measured)
enum SweepVariant {
    VAR_L1 = 0, VAR_HOT = 1, VAR_HOT24 = 2, VAR_HOT16 = 3, VAR_HOT8 = 4, N_VARIANTS = 5
};

struct VariantShape {
    unsigned grid, threads;
    size_t smem;
};

template <int MODE, bool W, int NT, bool HOT>
VariantShape variant_shape(uint32_t n_units, uint32_t hot_n) {
    static int per_sm = 0, sms = 0;
    const int dyn_max = HOT ? SP_HOT * (int)sizeof(float) : 0;
    if (!per_sm) {
        int dev = 0;
        GTC_CUDA(cudaGetDevice(&dev));
        GTC_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        if (HOT)
            GTC_CUDA(cudaFuncSetAttribute(k_sweep<MODE, W, NT, HOT>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, dyn_max));
        GTC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_sweep<MODE, W, NT, HOT>,
                                                               NT, dyn_max));
        if (per_sm < 1) per_sm = 1;
    }
    const unsigned cap = std::min<unsigned>((unsigned)(per_sm * sms), FOLD_MAX_CTAS);
    const unsigned want = (n_units + NT / 32 - 1) / (NT / 32);
    VariantShape v;
    v.grid = want < 1 ? 1u : (want < cap ? want : cap);
    v.threads = NT;
    v.smem = HOT ? (size_t)hot_n * sizeof(float) : 0;
    return v;
}

inline uint32_t variant_hot_cap(int var) {
    return var == VAR_HOT ? (uint32_t)SP_HOT
         : var == VAR_HOT24 ? 24576u
         : var == VAR_HOT16 ? 16384u
         : 8192u;
}

template <int MODE, bool W>
void launch_variant(int var, const SweepArgs& A, cudaStream_t s) {
    if (var == VAR_L1) {
        VariantShape v = variant_shape<MODE, W, 256, false>(A.n_units, A.hot_n);
        k_sweep<MODE, W, 256, false><<<v.grid, v.threads, v.smem, s>>>(A);
    } else {
        SweepArgs B = A;
        const uint32_t cap = variant_hot_cap(var);
        B.hot_n = (A.hot_n < cap ? A.hot_n : cap) & ~3u;
        VariantShape v = variant_shape<MODE, W, 1024, true>(B.n_units, B.hot_n);
        k_sweep<MODE, W, 1024, true><<<v.grid, v.threads, v.smem, s>>>(B);
    }
    GTC_LAUNCHED();
}

template <int MODE>
void launch_sweep(int var, const SweepArgs& A, bool weighted, cudaStream_t s) {
    if (weighted)
        launch_variant<MODE, true>(var, A, s);
    else
        launch_variant<MODE, false>(var, A, s);
}

// The autotuner: the first sweep of a (graph half, mode, weighting) runs every
// variant once on the real inputs (a sweep only reads prev and writes next,
// so the trial is harmless), keeps the fastest and caches the choice on the
// graph.  The variants compute bit-identical results (same per-item order and
// fold), so the choice changes speed only.
template <int MODE>
int tuned_variant(Units& u, const SweepArgs& A, bool weighted, int schedule, cudaStream_t s,
                  uint64_t* L) {
    switch (schedule) {  // a pinned kernel (gtc_schedule)
        case GTC_SCHED_L1: return VAR_L1;
        case GTC_SCHED_HOT32K: return VAR_HOT;
        case GTC_SCHED_HOT24K: return VAR_HOT24;
        case GTC_SCHED_HOT16K: return VAR_HOT16;
        case GTC_SCHED_HOT8K: return VAR_HOT8;
        default: break;
    }
    int& v = u.variant[MODE][weighted ? 1 : 0];
    if (v >= 0) return v;
    Timer trial(s);
    float best = 0.f;
    int best_v = VAR_L1;
    for (int rep = 0; rep < 2; ++rep) {  // the first round warms caches up
        for (int c = 0; c < N_VARIANTS; ++c) {
            trial.start();
            launch_sweep<MODE>(c, A, weighted, s);
            trial.stop();
            const float ms = (float)trial.ms();
            *L += 1;
            if (rep == 1 && (c == 0 || ms < best)) best = ms, best_v = c;
        }
    }
    v = best_v;
    return v;
}

void set_schedule(SweepArgs& A, const Units& u, const View& view) {
    A.units = u.units.get();
    A.longs = u.longs.get();
    A.med = u.med.get();
    A.slice_rows = u.slice_rows.get();
    A.slice_off = u.slice_off.get();
    A.sidx = u.sidx.get();
    A.partial = u.partial.get();
    A.counter = u.counter.get();
    A.n_units = u.n_units;
    A.n_long = u.n_long;
    A.off = view.pull_off;
    A.other = view.pull_other;
    A.hot_n = hot_entries(view.n);
}

// Weights of the sliced entries (0 for padding), per call.
__global__ void k_gather_sw(uint32_t q, const uint32_t* __restrict__ seid, const void* __restrict__ w,
                            int wdt, float* __restrict__ out) {
    size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p < q) {
        const uint32_t e = seid[p];
        out[p] = e != 0xFFFFFFFFu ? ld_f32(w, wdt, e) : 0.f;
    }
}

DevBuf<float> sliced_weights(const Units& u, const SolveIn& in, cudaStream_t s, uint64_t* L) {
    DevBuf<float> sw;
    if (in.weight.present() && u.n_sliced) {
        sw.alloc(u.n_sliced, s);
        k_gather_sw<<<grid_for(u.n_sliced, 256, 1u << 30), 256, 0, s>>>(
            u.n_sliced, u.seid.get(), in.weight.p, in.weight.dtype, sw.get());
        GTC_LAUNCHED();
        (*L)++;
    }
    return sw;
}

// A 64-bit hash of a weight map's bits: the sum over entries of a mixed
// (bits, index) word (the SplitMix64 finaliser), so any change of any entry
// changes it with overwhelming probability, and the sum does not depend on
// the grid.
__global__ void k_weight_hash(uint64_t m, const void* __restrict__ w, int wdt,
                              unsigned long long* __restrict__ out) {
    unsigned long long h = 0;
    unsigned bad = 0;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const unsigned long long bits = wdt == GTC_F64 ? ((const unsigned long long*)w)[i]
                                                       : ((const uint32_t*)w)[i];
        // a non-finite weight: all exponent bits set
        bad |= wdt == GTC_F64 ? ((bits >> 52) & 0x7FFull) == 0x7FFull
                              : ((bits >> 23) & 0xFFull) == 0xFFull;
        unsigned long long z = bits + (i + 1) * 0x9E3779B97F4A7C15ull;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        h += z ^ (z >> 31);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) h += __shfl_xor_sync(0xffffffffu, h, o);
    bad = __any_sync(0xffffffffu, bad);
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(out, h);
        if (bad) atomicOr(out + 1, 1ull);
    }
}

}  // namespace

// One read of a weight map by EdgeId (m entries): its 64-bit content hash,
// and a refusal (GTC_ERR_ARG) if it holds a NaN or an infinity.
unsigned long long scan_weights(const DVec& w, uint64_t m, cudaStream_t s, uint64_t* L) {
    DevBuf<unsigned long long> dh(2, s);
    GTC_CUDA(cudaMemsetAsync(dh.get(), 0, 2 * sizeof(unsigned long long), s));
    if (m) {
        k_weight_hash<<<(unsigned)sm_count() * 8, 256, 0, s>>>(m, w.p, w.dtype, dh.get());
        GTC_LAUNCHED();
        (*L)++;
    }
    unsigned long long h[2] = {0, 0};
    GTC_CUDA(cudaMemcpyAsync(h, dh.get(), sizeof(h), cudaMemcpyDeviceToHost, s));
    GTC_CUDA(cudaStreamSynchronize(s));
    GTC_REQUIRE(h[1] == 0, GTC_ERR_ARG, "weight map holds a non-finite value (NaN or infinity)");
    return h[0];
}

namespace {

// The handle's weight layouts for weight map w (FP32 path, unfiltered
// views): the cache is kept when w is the map it was built from (same
// address, dtype and content hash), cleared otherwise.
WeightCache& weight_cache(gtc_graph* g, const DVec& w, unsigned long long h) {
    WeightCache& c = g->wcache;
    if (!(c.valid && c.ptr == w.p && c.dtype == w.dtype && c.hash == h)) {
        GTC_CUDA(cudaStreamSynchronize(g->home));  // buffers of the old map are free to go
        c.reset();
        c.ptr = w.p, c.dtype = w.dtype, c.hash = h, c.valid = true;
    }
    return c;
}

// FP32 weights in the storage order of the in-halves (h = 0) or the
// out-halves (h = 1).
const float* cached_half_weights(gtc_graph* g, WeightCache& c, int h, cudaStream_t s,
                                 uint64_t* L) {
    const uint32_t m = g->m_live;
    if (!c.half[h].get()) {
        c.half[h].alloc(m, g->home);
        GTC_CUDA(cudaStreamSynchronize(s));
        if (m) {
            const Halves& hv = h ? g->out : g->in;
            k_gather_w<float><<<grid_for(m, 256, 1u << 30), 256, 0, g->home>>>(
                m, hv.eid.get(), c.ptr, c.dtype, c.half[h].get());
            GTC_LAUNCHED();
            (*L)++;
        }
        GTC_CUDA(cudaStreamSynchronize(g->home));
    }
    return c.half[h].get();
}

// Weighted degree (FP32 compensated sums, FP64 result) over the out-halves
// (h = 1, the plain view's push half) or the in-halves (h = 0).
void cached_degrees(gtc_graph* g, WeightCache& c, int h, cudaStream_t s, uint64_t* L,
                    const double** deg, const uint8_t** sink) {
    const uint32_t n = g->n;
    if (!c.deg[h].get()) {
        const float* wh = cached_half_weights(g, c, h, s, L);
        c.deg[h].alloc(n, g->home);
        c.sink[h].alloc(n, g->home);
        if (n) {
            k_degree_f32<<<grid_for((size_t)n * 8, 256, 1u << 30), 256, 0, g->home>>>(
                n, (h ? g->out : g->in).off.get(), wh, nullptr, c.deg[h].get(), c.sink[h].get());
            GTC_LAUNCHED();
            (*L)++;
        }
        GTC_CUDA(cudaStreamSynchronize(g->home));
    }
    *deg = c.deg[h].get();
    *sink = c.sink[h].get();
}

// The sliced entries' weights of a cached pull schedule (k = 0: units_in,
// k = 1: units_out).
const float* cached_sliced_weights(gtc_graph* g, WeightCache& c, int k, const Units& u,
                                   cudaStream_t s, uint64_t* L) {
    if (!u.n_sliced) return nullptr;
    if (!c.sliced[k].get()) {
        c.sliced[k].alloc(u.n_sliced, g->home);
        GTC_CUDA(cudaStreamSynchronize(s));
        k_gather_sw<<<grid_for(u.n_sliced, 256, 1u << 30), 256, 0, g->home>>>(
            u.n_sliced, u.seid.get(), c.ptr, c.dtype, c.sliced[k].get());
        GTC_LAUNCHED();
        (*L)++;
        GTC_CUDA(cudaStreamSynchronize(g->home));
    }
    return c.sliced[k].get();
}

// Out-degrees of the unweighted, unfiltered view over the in-halves (h = 0,
// the reversed view) or the out-halves (h = 1, the plain view), kept on the
// handle.
void cached_plain_degrees(gtc_graph* g, int h, uint64_t* L, const double** deg,
                          const uint8_t** sink) {
    const uint32_t n = g->n;
    DegCache& c = g->dcache;
    if (!c.deg[h].get()) {
        c.deg[h].alloc(n, g->home);
        c.sink[h].alloc(n, g->home);
        const Halves& hv = h ? g->out : g->in;
        if (n) {
            k_degree<<<grid_for(n, 256, 1u << 30), 256, 0, g->home>>>(
                n, hv.off.get(), hv.eid.get(), nullptr, GTC_F64, nullptr, c.deg[h].get(),
                c.sink[h].get());
            GTC_LAUNCHED();
            (*L)++;
        }
        GTC_CUDA(cudaStreamSynchronize(g->home));
    }
    *deg = c.deg[h].get();
    *sink = c.sink[h].get();
}

// Everything a sweep loop needs that does not change between sweeps.
struct Prep {
    View view;
    double uniform = 0.0;
    DevBuf<double> deg;
    DevBuf<uint8_t> sink;
    DevBuf<float> invdeg;
    const double* degp = nullptr;   // deg, or the handle's cached degrees
    const uint8_t* sinkp = nullptr;
    DevBuf<float>* inv_cache = nullptr;  // the handle's FP32 inverse of cached degrees
    WeightCache* wc = nullptr;      // the handle's weight layouts (FP32, unfiltered, weighted)
    DevBuf<double> x64;  // initial iterate, FP64 (left empty when the caller seeds FP32)
};

// The FP32 inverse degrees of the view: kept on the handle beside cached
// degrees, else computed for this call.
const float* invdeg_f32(gtc_graph* g, Prep& P, cudaStream_t s, uint64_t* L) {
    const uint32_t n = P.view.n;
    DevBuf<float>& b = P.inv_cache ? *P.inv_cache : P.invdeg;
    if (!b.get()) {
        // cached degrees were written on the home stream, which is idle
        cudaStream_t st = P.inv_cache ? g->home : s;
        b.alloc(n, st);
        if (n) {
            k_invdeg_f32<<<grid_for(n, 256, 1u << 30), 256, 0, st>>>(n, P.degp, b.get());
            GTC_LAUNCHED();
            (*L)++;
        }
        if (P.inv_cache) GTC_CUDA(cudaStreamSynchronize(g->home));
    }
    return b.get();
}

// seed_x64 false: the caller seeds its FP32 iterate itself (k_pr_seed or
// k_seed_f32) and P.x64 stays empty; only an unfiltered view may skip it,
// since k_store reads x64 for the vertices a filter leaves out.
void prepare(gtc_graph* g, const gtc_view* vw, const SolveIn& in, bool need_deg, Prep& P,
             cudaStream_t s, uint64_t* L, bool seed_x64 = true) {
    const unsigned TB = 256;
    P.view.prepare(g, vw, s, L);
    const uint32_t n = P.view.n;
    P.uniform = P.view.n_active == 0 ? 0.0 : 1.0 / (double)P.view.n_active;
    if (in.weight.present()) {
        const unsigned long long h = scan_weights(in.weight, g->m, s, L);
        if (in.precision == GTC_PREC_F32 && !P.view.filtered) P.wc = &weight_cache(g, in.weight, h);
    }
    const int hd = P.view.reversed ? 0 : 1;  // the halves the view pushes over
    if (need_deg && P.wc) {
        cached_degrees(g, *P.wc, hd, s, L, &P.degp, &P.sinkp);
        P.inv_cache = &P.wc->invdeg[hd];
    } else if (need_deg && !in.weight.present() && !P.view.filtered) {
        cached_plain_degrees(g, hd, L, &P.degp, &P.sinkp);
        P.inv_cache = &g->dcache.invdeg[hd];
    } else if (need_deg) {
        P.deg.alloc(n, s);
        P.sink.alloc(n, s);
        P.degp = P.deg.get();
        P.sinkp = P.sink.get();
        if (n && in.weight.present() && in.precision == GTC_PREC_F32) {
            const uint32_t mp = P.view.m_pull;  // the push half holds as many entries
            DevBuf<float> wout(mp, s);
            if (mp)
                k_gather_w<float><<<grid_for(mp, TB, 1u << 30), TB, 0, s>>>(
                    mp, P.view.push_eid, in.weight.p, in.weight.dtype, wout.get());
            k_degree_f32<<<grid_for((size_t)n * 8, TB, 1u << 30), TB, 0, s>>>(
                n, P.view.push_off, wout.get(), P.view.active_or_null(), P.deg.get(),
                P.sink.get());
            GTC_LAUNCHED();
            (*L) += 2;
        } else if (n) {
            k_degree<<<grid_for(n, TB, 1u << 30), TB, 0, s>>>(
                n, P.view.push_off, P.view.push_eid, in.weight.p, in.weight.dtype,
                P.view.active_or_null(), P.deg.get(), P.sink.get());
            GTC_LAUNCHED();
            (*L)++;
        }
    }
    if (!seed_x64 && !P.view.filtered) return;
    P.x64.alloc(n, s);
    if (n) {
        k_seed<<<grid_for(n, TB, 1u << 30), TB, 0, s>>>(n, g->perm.get(), in.had, in.x, in.x_dtype,
                                                        in.pers.p, in.pers.dtype, P.uniform,
                                                        P.x64.get());
        GTC_LAUNCHED();
        (*L)++;
    }
}

template <class T>
void store_result(gtc_graph* g, uint32_t n, const T* src, const Prep& P, const SolveIn& in,
                  cudaStream_t s, uint64_t* L) {
    if (!n) return;
    k_store<T><<<grid_for(n, 256, 1u << 30), 256, 0, s>>>(n, g->iperm.get(), src,
                                                          P.view.active_or_null(), P.x64.get(),
                                                          in.x, in.x_dtype);
    GTC_LAUNCHED();
    (*L)++;
}

// The FP32 weights a sweep streams: the handle's cached layouts for an
// unfiltered view, else gathered for this call into `own`.
struct SweepWeights {
    DevBuf<float> own_pull, own_sliced;
    const float* pull = nullptr;
    const float* sliced = nullptr;
};

template <class T>
DevBuf<T> pull_weights(const Prep& P, const SolveIn& in, cudaStream_t s, uint64_t* L) {
    DevBuf<T> w;
    const uint32_t mp = P.view.m_pull;
    if (in.weight.present() && mp) {
        w.alloc(mp, s);
        k_gather_w<T><<<grid_for(mp, 256, 1u << 30), 256, 0, s>>>(mp, P.view.pull_eid, in.weight.p,
                                                                 in.weight.dtype, w.get());
        GTC_LAUNCHED();
        (*L)++;
    }
    return w;
}

void sweep_weights(gtc_graph* g, const Prep& P, const SolveIn& in, const Units& U, bool rev,
                   cudaStream_t s, uint64_t* L, SweepWeights& out) {
    if (P.wc) {
        out.pull = cached_half_weights(g, *P.wc, rev ? 1 : 0, s, L);
        out.sliced = cached_sliced_weights(g, *P.wc, rev ? 1 : 0, U, s, L);
        return;
    }
    out.own_pull = pull_weights<float>(P, in, s, L);
    out.own_sliced = sliced_weights(U, in, s, L);
    out.pull = out.own_pull.get();
    out.sliced = out.own_sliced.get();
}

}  // namespace

void pagerank(gtc_graph* g, const gtc_view* vw, const SolveIn& in, gtc_result* res,
              cudaStream_t s) {
    uint64_t L = 0, SL = 0;
    const unsigned TB = 256;
    Prep P;
    prepare(g, vw, in, true, P, s, &L, in.precision == GTC_PREC_F64_EXACT);
    const View& view = P.view;
    const uint32_t n = view.n;
    const double d = in.damping;
    const uint8_t* act = view.active_or_null();
    const uint64_t max_iter = in.params.max_iter;
    const double eps = in.params.epsilon;
    uint64_t iter = 0;
    double delta = eps + 1.0, sweep_ms = 0.0;
    Timer total(s), sw(s);

    if (in.precision == GTC_PREC_F64_EXACT) {
        const uint64_t chunks = in.params.plan_chunks;
        // sinks in vertex order and their Plan (grain_of, centrality.rs:186-188, :311)
        DevBuf<uint32_t> flag32(n, s), pos((size_t)n + 1, s);
        if (n) {
            k_sink_flags<<<grid_for(n, TB, 1u << 30), TB, 0, s>>>(n, g->iperm.get(), P.sinkp,
                                                                  flag32.get());
            GTC_LAUNCHED();
            L++;
        }
        scan_exclusive_u32(flag32.get(), pos.get(), n, s, &L);
        uint32_t n_sinks = 0;
        GTC_CUDA(cudaMemcpyAsync(&n_sinks, pos.get() + n, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
        GTC_CUDA(cudaStreamSynchronize(s));
        DevBuf<uint32_t> sinks(n_sinks, s);
        if (n) {
            k_compact_sinks<<<grid_for(n, TB, 1u << 30), TB, 0, s>>>(n, flag32.get(), g->iperm.get(),
                                                                     pos.get(), sinks.get());
            GTC_LAUNCHED();
            L++;
        }
        const uint64_t grain = std::max<uint64_t>((n + chunks - 1) / chunks, 1);
        const uint64_t sink_chunks = std::max<uint64_t>((n_sinks + grain - 1) / grain, 1);
        DevBuf<double> wpull = pull_weights<double>(P, in, s, &L);
        DevBuf<double> scratch(n, s), diff(n, s), part(std::max(chunks, sink_chunks), s);
        DevBuf<double> q;  // unweighted: the per-source terms of a sweep
        if (!wpull.get()) q.alloc(n, s);
        DevBuf<double> scal(4, s);  // [p_sink, delta]
        const double* pers64 = nullptr;
        DevBuf<double> pbuf;
        if (in.pers.present()) {
            {  // pers by internal label
                pbuf.alloc(n, s);
                k_seed<<<grid_for(n, TB, 1u << 30), TB, 0, s>>>(n, g->perm.get(), n, in.pers.p,
                                                                in.pers.dtype, nullptr, 0, 0.0,
                                                                pbuf.get());
                GTC_LAUNCHED();
                L++;
                pers64 = pbuf.get();
            }
        }
        double* cur = P.x64.get();
        double* nxt = scratch.get();
        total.start();
        while (delta >= eps) {
            if (in.timing) sw.start();
            k_chunk_sums<<<grid_for(sink_chunks, 32, 1u << 30), 32, 0, s>>>(
                n_sinks, sink_chunks, cur, sinks.get(), part.get());
            k_fold<<<1, 32, 0, s>>>(sink_chunks, part.get(), scal.get(), nullptr, 0);
            if (n && !wpull.get()) {
                k_pr_f64_q<<<grid_for(n, 256, 1u << 30), 256, 0, s>>>(n, cur, P.degp, q.get());
                k_pr_f64_rows_q<<<grid_for(n, 128, 1u << 30), 128, 0, s>>>(
                    n, view.pull_off, view.pull_other, q.get(), act, pers64, P.uniform, 1.0 - d,
                    d, scal.get(), cur, nxt, diff.get());
            } else if (n) {
                k_pr_f64_rows<<<grid_for(n, 128, 1u << 30), 128, 0, s>>>(
                    n, view.pull_off, view.pull_other, wpull.get(), P.degp, act, pers64,
                    P.uniform, 1.0 - d, d, scal.get(), cur, nxt, diff.get());
                k_pr_f64_long<<<(unsigned)sm_count() * 8, 256, 0, s>>>(
                    n, view.pull_off, view.pull_other, wpull.get(), P.degp, act, pers64,
                    P.uniform, 1.0 - d, d, scal.get(), cur, nxt, diff.get());
            }
            // the delta is folded over the Plan in original vertex order
            k_chunk_sums<<<grid_for(chunks, 32, 1u << 30), 32, 0, s>>>(n, chunks, diff.get(),
                                                                         g->iperm.get(), part.get());
            k_fold<<<1, 32, 0, s>>>(chunks, part.get(), scal.get() + 1, nullptr, 0);
            GTC_LAUNCHED();
            if (in.timing) sw.stop();
            L += n ? 6 : 4;
            SL += n ? 6 : 4;
            GTC_CUDA(cudaMemcpyAsync(&delta, scal.get() + 1, sizeof(double), cudaMemcpyDeviceToHost, s));
            GTC_CUDA(cudaStreamSynchronize(s));
            if (in.timing) sweep_ms += sw.ms();
            std::swap(cur, nxt);
            iter++;
            if (max_iter > 0 && iter == max_iter) break;
        }
        total.stop();
        res->device_ms = total.ms();
        store_result<double>(g, n, cur, P, in, s, &L);
    } else {
        const float* invdeg = invdeg_f32(g, P, s, &L);
        DevBuf<float> pers32;
        if (in.pers.present() && n) {
            pers32.alloc(n, s);
            k_to_f32<<<grid_for(n, TB, 1u << 30), TB, 0, s>>>(n, in.pers.p, in.pers.dtype,
                                                              g->perm.get(), pers32.get());
            GTC_LAUNCHED();
            L++;
        }
        // the gathered vectors carry one more entry, kept 0: the slices'
        // padding gathers it (a sweep does not store y of a dangling row
        // either: k_pr_seed zeroes those in y1)
        DevBuf<float> r0(n, s), r1(n, s), y0((size_t)n + 1, s), y1((size_t)n + 1, s);
        const unsigned nb = persistent_blocks(n);
        FoldBufs fb(nb, s);
        double* dp = fb.out.get();  // [0] delta, [1] dangling mass of the current iterate
        k_pr_seed<<<nb, PR_NT, 0, s>>>(n, P.x64.get(), seed_perm(g, in), in.had, in.x,
                                      in.x_dtype, in.pers.p, in.pers.dtype, (float)P.uniform,
                                      invdeg, P.sinkp, r0.get(), y0.get(), y1.get(),
                                      fb.fold(dp + 2, dp + 1));
        GTC_LAUNCHED();
        L++;
        float *rc = r0.get(), *rn = r1.get(), *yc = y0.get(), *yn = y1.get();
        Units local;
        Units* U = pull_units(g, view, local, s);
        const bool W = in.weight.present();
        FoldBufs fs(1, s);
        double* dq = fs.out.get();
        // the dangling mass of the initial iterate seeds the first sweep
        GTC_CUDA(cudaMemcpyAsync(dq + 1, dp + 1, sizeof(double), cudaMemcpyDeviceToDevice, s));
        SweepArgs A{};
        set_schedule(A, *U, view);
        SweepWeights sw8;
        sweep_weights(g, P, in, *U, view.reversed, s, &L, sw8);
        A.sw = sw8.sliced;
        A.w = sw8.pull;
        A.active = act;
        A.invdeg = invdeg;
        A.sink = P.sinkp;
        A.pers = pers32.get();
        A.uniform = (float)P.uniform;
        A.one_minus_d = (float)(1.0 - d);
        A.d = (float)d;
        A.psink = dq + 1;
        A.fold = ExactFold{U->fold_part.get(), fs.ticket.get(), dq, dq + 1};
        A.x = yc, A.prev = rc, A.next = rn, A.ynext = yn;
        const int var = tuned_variant<MODE_PAGERANK>(*U, A, W, in.schedule, s, &L);
        // a tuning trial wrote the dangling mass of its output: restore it
        GTC_CUDA(cudaMemcpyAsync(dq + 1, dp + 1, sizeof(double), cudaMemcpyDeviceToDevice, s));
        // The loop of centrality.rs:318-376 with the stop decided on the
        // device: sweeps go out in batches and the host reads the stop flag
        // once a batch (a sweep after the stop returns at once).
        StopState st(s);
        st.arm(A.fold, eps, max_iter);
        A.stop = st.stop();
        SweepEvents evs;
        float* rb[2] = {rc, rn};
        float* ybuf[2] = {yc, yn};
        uint64_t launched = 0;
        total.start();
        for (bool stopped = false; !stopped;) {
            for (int k = 0; k < STOP_BATCH; ++k, ++launched) {
                const int c = (int)(launched & 1);
                A.x = ybuf[c], A.prev = rb[c], A.next = rb[c ^ 1], A.ynext = ybuf[c ^ 1];
                if (in.timing) evs.record(s);
                launch_sweep<MODE_PAGERANK>(var, A, W, s);
                if (in.timing) evs.record(s);
                L++;
                SL++;
            }
            const auto rs = st.read(s);
            stopped = rs.first;
            iter = rs.second;
        }
        total.stop();
        GTC_CUDA(cudaMemcpyAsync(&delta, dq, sizeof(double), cudaMemcpyDeviceToHost, s));
        res->device_ms = total.ms();
        if (in.timing) sweep_ms = evs.ms(iter);
        SL = iter;
        rc = rb[iter & 1];
        store_result<float>(g, n, rc, P, in, s, &L);
    }
    GTC_CUDA(cudaStreamSynchronize(s));
    res->iterations = iter;
    res->last_delta = iter ? delta : 0.0;
    res->eigenvalue = 0.0;
    res->launches = L;
    res->sweep_ms = sweep_ms;
    res->sweep_launches = SL;
    g->launches += L;
}

void eigenvector(gtc_graph* g, const gtc_view* vw, const SolveIn& in, gtc_result* res,
                 cudaStream_t s) {
    uint64_t L = 0, SL = 0;
    Prep P;
    prepare(g, vw, in, false, P, s, &L, in.precision == GTC_PREC_F64_EXACT);
    const View& view = P.view;
    const uint32_t n = view.n;
    const uint8_t* act = view.active_or_null();
    const uint64_t max_iter = in.params.max_iter;
    const double eps = in.params.epsilon;
    uint64_t iter = 0;
    double delta = eps + 1.0, norm = 0.0, sweep_ms = 0.0;
    Timer total(s), sw(s);
    if (in.precision == GTC_PREC_F64_EXACT) {
        const uint64_t chunks = in.params.plan_chunks;
        DevBuf<double> wpull = pull_weights<double>(P, in, s, &L);
        DevBuf<double> scratch(n, s), tmp(n, s), part(chunks, s), scal(4, s);
        double* cur = P.x64.get();
        double* nxt = scratch.get();
        total.start();
        while (delta >= eps) {
            if (in.timing) sw.start();
            if (n && !wpull.get()) {
                k_ev_f64_rows_u<<<grid_for(n, 128, 1u << 30), 128, 0, s>>>(
                    n, view.pull_off, view.pull_other, act, cur, nxt, tmp.get());
            } else if (n) {
                k_ev_f64_rows<<<grid_for(n, 128, 1u << 30), 128, 0, s>>>(
                    n, view.pull_off, view.pull_other, wpull.get(), act, cur, nxt, tmp.get());
                k_ev_f64_long<<<(unsigned)sm_count() * 8, 256, 0, s>>>(
                    n, view.pull_off, view.pull_other, wpull.get(), act, cur, nxt, tmp.get());
            }
            k_chunk_sums<<<grid_for(chunks, 32, 1u << 30), 32, 0, s>>>(n, chunks, tmp.get(),
                                                                         g->iperm.get(), part.get());
            // scal[0] = squared norm, scal[1] = norm, scal[2] = scale
            k_fold<<<1, 32, 0, s>>>(chunks, part.get(), scal.get(), scal.get() + 2, 1);
            if (n)
                k_ev_f64_norm<<<grid_for(n, 128, 1u << 30), 128, 0, s>>>(n, act, scal.get() + 2,
                                                                         cur, nxt, tmp.get());
            k_chunk_sums<<<grid_for(chunks, 32, 1u << 30), 32, 0, s>>>(n, chunks, tmp.get(),
                                                                         g->iperm.get(), part.get());
            k_fold<<<1, 32, 0, s>>>(chunks, part.get(), scal.get() + 3, nullptr, 0);
            GTC_LAUNCHED();
            if (in.timing) sw.stop();
            const uint64_t per_sweep = n ? (wpull.get() ? 7 : 6) : 4;
            L += per_sweep;
            SL += per_sweep;
            double hs[4];
            GTC_CUDA(cudaMemcpyAsync(hs, scal.get(), 4 * sizeof(double), cudaMemcpyDeviceToHost, s));
            GTC_CUDA(cudaStreamSynchronize(s));
            if (in.timing) sweep_ms += sw.ms();
            norm = hs[1];
            delta = hs[3];
            std::swap(cur, nxt);
            iter++;
            if (max_iter > 0 && iter == max_iter) break;
        }
        total.stop();
        res->device_ms = total.ms();
        store_result<double>(g, n, cur, P, in, s, &L);
    } else {
        DevBuf<float> x0((size_t)n + 1, s), x1((size_t)n + 1, s);  // x[n] == 0: slice padding
        GTC_CUDA(cudaMemsetAsync(x0.get() + n, 0, sizeof(float), s));
        GTC_CUDA(cudaMemsetAsync(x1.get() + n, 0, sizeof(float), s));
        if (n && P.x64.get()) {
            k_to_f32<<<grid_for(n, 256, 1u << 30), 256, 0, s>>>(n, P.x64.get(), GTC_F64, nullptr,
                                                                x0.get());
            GTC_LAUNCHED();
            L++;
        } else if (n) {
            k_seed_f32<<<grid_for(n, 256, 1u << 30), 256, 0, s>>>(
                n, seed_perm(g, in), in.had, in.x, in.x_dtype, in.pers.p, in.pers.dtype,
                (float)P.uniform, x0.get());
            GTC_LAUNCHED();
            L++;
        }
        Units local;
        Units* U = pull_units(g, view, local, s);
        const bool W = in.weight.present();
        const unsigned nb = persistent_blocks(n);
        FoldBufs f1(1, s), f2(nb, s);
        double* o1 = f1.out.get();
        double* o2 = f2.out.get();
        float *xc = x0.get(), *xn = x1.get();
        SweepArgs A{};
        set_schedule(A, *U, view);
        SweepWeights sw8;
        sweep_weights(g, P, in, *U, view.reversed, s, &L, sw8);
        A.sw = sw8.sliced;
        A.w = sw8.pull;
        A.active = act;
        A.fold = ExactFold{U->fold_part.get(), f1.ticket.get(), o1, o1 + 1};
        A.x = xc, A.prev = xc, A.next = xn;
        const int var = tuned_variant<MODE_EIGEN>(*U, A, W, in.schedule, s, &L);
        // the loop of centrality.rs:440-492, stopped on the device (as PageRank)
        StopState st(s);
        ExactFold fn = f2.fold(o2, o2 + 1);
        st.arm(fn, eps, max_iter);
        A.stop = st.stop();
        SweepEvents evs;
        float* xb[2] = {xc, xn};
        uint64_t launched = 0;
        total.start();
        for (bool stopped = false; !stopped;) {
            for (int k = 0; k < STOP_BATCH; ++k, ++launched) {
                const int c = (int)(launched & 1);
                A.x = xb[c], A.prev = xb[c], A.next = xb[c ^ 1];
                if (in.timing) evs.record(s);
                launch_sweep<MODE_EIGEN>(var, A, W, s);
                k_ev_f32_norm<<<nb, PR_NT, 0, s>>>(n, act, o1, xb[c], xb[c ^ 1], fn);
                GTC_LAUNCHED();
                if (in.timing) evs.record(s);
                L += 2;
            }
            const auto rs = st.read(s);
            stopped = rs.first;
            iter = rs.second;
        }
        total.stop();
        double sq = 0.0;
        GTC_CUDA(cudaMemcpyAsync(&sq, o1, sizeof(double), cudaMemcpyDeviceToHost, s));
        GTC_CUDA(cudaMemcpyAsync(&delta, o2, sizeof(double), cudaMemcpyDeviceToHost, s));
        GTC_CUDA(cudaStreamSynchronize(s));
        norm = iter ? std::sqrt(sq) : 0.0;
        res->device_ms = total.ms();
        if (in.timing) sweep_ms = evs.ms(iter);
        SL = 2 * iter;
        xc = xb[iter & 1];
        store_result<float>(g, n, xc, P, in, s, &L);
    }
    GTC_CUDA(cudaStreamSynchronize(s));
    res->iterations = iter;
    res->last_delta = iter ? delta : 0.0;
    res->eigenvalue = norm;
    res->launches = L;
    res->sweep_ms = sweep_ms;
    res->sweep_launches = SL;
    g->launches += L;
}

// --------------------------------------------------------------------------
// the PageRank adjoint
// --------------------------------------------------------------------------
//
// Forward fixed point pi = (1-d) p + d M pi, M = A + p s^T, A[t][s] =
// w_e/deg_s for deg_s != 0 (sinks s contribute through the dangling mass
// only).  For L(pi) with g = dL/dpi the adjoint lambda solves
//     lambda = T(lambda) = g + d M^T lambda = g + d (A^T lambda + s (p . lambda)),
// and (A^T lambda)_s = sum over s's out-edges of (w_e/deg_s) lambda_t, a pull
// over the out-halves.  By the implicit-function theorem only the converged
// pi is needed:
//     dL/dp_v = lambda_v ((1-d) + d (s . pi))
//     dL/dw_e = d (pi_s/deg_s) (lambda_t - (A^T lambda)_s)   (e: s->t, deg_s != 0)
// (the second term comes from deg_s depending on w_e).  Edges out of a vertex
// whose weighted degree is 0 get 0 (the map is not differentiable there).
//
// Deflation.  With sum(p) = 1, M^T 1 = 1: the all-ones direction is an
// eigenvector of d M^T with eigenvalue d, so plain iteration from g removes
// its error only by a factor d per sweep.  The fixed point obeys one exact
// linear constraint, from the forward system:
//     (1-d) p . lambda = ((I - d M) pi) . lambda = pi . ((I - d M^T) lambda) = pi . g,
// so every iterate is shifted along 1 to satisfy p . lambda = tau =
// (pi . g) / (1-d) before it is swept.  The shift is zero at the fixed point
// (which is unchanged) and the all-ones error component is re-set from the
// remaining error at every sweep instead of decaying by d.  The iteration
// stops when the L1 norm of the fixed-point residual T(lambda) - lambda of
// the shifted iterate falls below epsilon * |g|_1.

// (sum_v a_v x_v, sum_v b_v y_v) over n entries: a null a or b is the
// constant ua / ub, a null x or y is 1; `absy` sums |b_v y_v|.  Summed
// exactly into (out_a, out_b).
__global__ void __launch_bounds__(PR_NT) k_dot2(uint32_t n, const float* __restrict__ a, float ua,
                                               const float* __restrict__ x,
                                               const float* __restrict__ b, float ub,
                                               const float* __restrict__ y, bool absy, ExactFold f) {
    ExactPR ka, kb;
    for (size_t v = (size_t)blockIdx.x * PR_NT + threadIdx.x; v < n;
         v += (size_t)gridDim.x * PR_NT) {
        ka.add(__fmul_rn(a ? a[v] : ua, x ? x[v] : 1.f));
        const float t = __fmul_rn(b ? b[v] : ub, y ? y[v] : 1.f);
        kb.add(absy ? fabsf(t) : t);
    }
    block_fold_exact<PR_NT>(ka, kb, f);
}

// grad_p[v] = (lambda + alpha)[iperm v] * c (original labels)
__global__ void k_grad_pers(uint32_t n, const uint32_t* __restrict__ iperm,
                            const float* __restrict__ lam, float alpha,
                            const double* __restrict__ psink_pi, double one_minus_d, double d,
                            void* __restrict__ out, int dt) {
    size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n) return;
    const float c = (float)(one_minus_d + d * (*psink_pi));
    const float gv = __fmul_rn(__fadd_rn(lam[iperm[v]], alpha), c);
    if (dt == GTC_F64)
        ((double*)out)[v] = (double)gv;
    else
        ((float*)out)[v] = gv;
}

// rowid[p] = s for the entries p of row s (8 lanes per row).
__global__ void k_row_ids(uint32_t n, const uint32_t* __restrict__ off, uint32_t* __restrict__ rowid) {
    const uint32_t sub = threadIdx.x & 7;
    const size_t s = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 3;
    if (s >= n) return;
    for (uint32_t p = off[s] + sub, e = off[s + 1]; p < e; p += 8) rowid[p] = (uint32_t)s;
}

// grad_w over the out-half entries (a thread each, its row from rowid):
// d (pi_s / deg_s) (lambda_t - (A^T lambda)_s) with lambda = lam + alpha_K
// and A^T lambda = atl + alpha_{K-1} (the last sweep's): dalpha = the
// difference of the two shifts.
__global__ void k_grad_w(uint32_t m, const uint32_t* __restrict__ rowid,
                         const uint32_t* __restrict__ other, const uint32_t* __restrict__ eid,
                         const float* __restrict__ y, const float* __restrict__ lam,
                         const float* __restrict__ atl, const uint8_t* __restrict__ sink, float d,
                         float dalpha, void* __restrict__ out, int dt) {
    const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= m) return;
    const uint32_t s = rowid[p];
    const float gw = sink[s] ? 0.f
                             : __fmul_rn(__fmul_rn(d, y[s]),
                                         __fsub_rn(lam[other[p]], __fsub_rn(atl[s], dalpha)));
    const uint32_t e = eid[p];
    if (dt == GTC_F64)
        ((double*)out)[e] = (double)gw;
    else
        ((float*)out)[e] = gw;
}

void pagerank_adjoint(gtc_graph* g, const gtc_view* vw, const AdjointIn& in, gtc_result* res,
                      cudaStream_t s) {
    uint64_t L = 0, SL = 0;
    const unsigned TB = 256;
    GTC_REQUIRE(!vw || (!vw->vmask && !vw->emask), GTC_ERR_ARG,
                "the PageRank adjoint supports the graph and its reversal, not filtered views");
    // the forward view: degrees, sinks, pi
    SolveIn fin{};
    fin.weight = in.weight;
    fin.pers = in.pers;
    fin.x = const_cast<void*>(in.pi.p);
    fin.x_dtype = in.pi.dtype;
    fin.had = g->n;  // pi is the seed: x64 = pi (internal labels)
    fin.precision = GTC_PREC_F32;
    const bool W = in.weight.present();
    Prep P;
    // weighted: the degrees come from the out-half weights gathered below
    prepare(g, vw, fin, !W, P, s, &L);
    const uint32_t n = P.view.n;
    const double d = in.damping;
    // the adjoint pulls over the forward view's out-halves: the reversed view
    gtc_view rv{};
    rv.reversed = (vw && vw->reversed) ? 0 : 1;
    View av;
    av.prepare(g, &rv, s, &L);
    // the weights the adjoint streams and the forward's weighted degrees:
    // from the handle's cache (the forward solve normally built them)
    const int hav = av.reversed ? 1 : 0;  // the half the adjoint pulls over
    DevBuf<float> wpull_own;
    const float* wpull = nullptr;
    if (W && P.wc) {
        wpull = cached_half_weights(g, *P.wc, hav, s, &L);
        cached_degrees(g, *P.wc, hav, s, &L, &P.degp, &P.sinkp);
        P.inv_cache = &P.wc->invdeg[hav];
    } else if (W) {
        if (av.m_pull) {
            wpull_own.alloc(av.m_pull, s);
            k_gather_w<float><<<grid_for(av.m_pull, 256, 1u << 30), 256, 0, s>>>(
                av.m_pull, av.pull_eid, in.weight.p, in.weight.dtype, wpull_own.get());
            GTC_LAUNCHED();
            L++;
        }
        wpull = wpull_own.get();
        P.deg.alloc(n, s);
        P.sink.alloc(n, s);
        P.degp = P.deg.get();
        P.sinkp = P.sink.get();
        if (n) {
            k_degree_f32<<<grid_for((size_t)n * 8, TB, 1u << 30), TB, 0, s>>>(
                n, av.pull_off, wpull, nullptr, P.deg.get(), P.sink.get());
            GTC_LAUNCHED();
            L++;
        }
    }
    const float* invdeg = invdeg_f32(g, P, s, &L);
    DevBuf<float> pers32, g32(n, s), pi32(n, s), ypi((size_t)n + 1, s);
    if (n) {
        k_to_f32<<<grid_for(n, TB, 1u << 30), TB, 0, s>>>(n, P.x64.get(), GTC_F64, nullptr, pi32.get());
        k_to_f32<<<grid_for(n, TB, 1u << 30), TB, 0, s>>>(n, in.gpi.p, in.gpi.dtype, g->perm.get(),
                                                          g32.get());
        GTC_LAUNCHED();
        L += 2;
    }
    if (in.pers.present() && n) {
        pers32.alloc(n, s);
        k_to_f32<<<grid_for(n, TB, 1u << 30), TB, 0, s>>>(n, in.pers.p, in.pers.dtype, g->perm.get(),
                                                          pers32.get());
        GTC_LAUNCHED();
        L++;
    }
    const unsigned nb = persistent_blocks(n);
    FoldBufs fb(nb, s);
    double* dp = fb.out.get();  // [1] dangling mass of pi
    // y = pi / deg and the dangling mass of pi
    k_pr_prime<<<nb, PR_NT, 0, s>>>(n, pi32.get(), invdeg, P.sinkp, ypi.get(),
                                   fb.fold(dp + 2, dp + 1));
    GTC_LAUNCHED();
    L++;

    Units local;
    Units* U = pull_units(g, av, local, s);
    DevBuf<float> lam0((size_t)n + 1, s), lam1((size_t)n + 1, s), atl((size_t)n + 1, s);
    GTC_CUDA(cudaMemsetAsync(lam0.get() + n, 0, sizeof(float), s));
    GTC_CUDA(cudaMemsetAsync(lam1.get() + n, 0, sizeof(float), s));
    if (n) GTC_CUDA(cudaMemcpyAsync(lam0.get(), g32.get(), (size_t)n * 4, cudaMemcpyDeviceToDevice, s));
    // p . g, pi . g, sum(p), |g|_1
    FoldBufs fd(nb, s);
    const float uni = (float)P.uniform;
    k_dot2<<<nb, PR_NT, 0, s>>>(n, pers32.get(), uni, g32.get(), pi32.get(), 0.f, g32.get(), false,
                               fd.fold(fd.out.get(), fd.out.get() + 1));
    k_dot2<<<nb, PR_NT, 0, s>>>(n, pers32.get(), uni, nullptr, nullptr, 1.f, g32.get(), true,
                               fd.fold(fd.out.get() + 2, fd.out.get() + 3));
    GTC_LAUNCHED();
    L += 2;
    double h4[4] = {0, 0, 0, 0};
    GTC_CUDA(cudaMemcpyAsync(h4, fd.out.get(), sizeof(h4), cudaMemcpyDeviceToHost, s));
    GTC_CUDA(cudaStreamSynchronize(s));
    const double psum = h4[2], gnorm = h4[3];
    const bool deflate = psum > 0.0 && d < 1.0;
    double tau = deflate ? h4[1] / (1.0 - d) : h4[0];  // without deflation: p . lambda
    double alpha = deflate ? (tau - h4[0]) / psum : 0.0, alpha_prev = alpha;

    FoldBufs fs(1, s);
    double* dq = fs.out.get();  // [0] residual, [1] p . (next iterate before its shift)
    SweepArgs A{};
    set_schedule(A, *U, av);
    DevBuf<float> swt_own;
    const float* swt = nullptr;
    if (W && P.wc) {
        swt = cached_sliced_weights(g, *P.wc, hav, *U, s, &L);
    } else {
        swt_own = sliced_weights(*U, fin, s, &L);
        swt = swt_own.get();
    }
    A.sw = swt;
    A.w = wpull;
    A.invdeg = invdeg;
    A.sink = P.sinkp;
    A.pers = pers32.get();
    A.gvec = g32.get();
    A.uniform = uni;
    A.one_minus_d = (float)(1.0 - d);
    A.d = (float)d;
    A.psink = dq + 1;  // read but unused in this mode
    A.alpha = (float)alpha;
    A.tau = (float)tau;
    A.fold = ExactFold{U->fold_part.get(), fs.ticket.get(), dq, dq + 1};
    A.ynext = atl.get();
    float *lc = lam0.get(), *ln = lam1.get();
    A.x = lc, A.prev = lc, A.next = ln;
    const int var = tuned_variant<MODE_ADJOINT>(*U, A, W, GTC_SCHED_AUTO, s, &L);

    const uint64_t max_iter = in.params.max_iter;
    const double tol = in.params.epsilon * gnorm;
    uint64_t iter = 0;
    double delta = tol + 1.0, sweep_ms = 0.0;
    Timer total(s), sw(s);
    total.start();
    // g = 0 gives lambda = 0 (the start) and no sweep; a NaN stops at once
    while (gnorm > 0.0 && delta >= tol) {
        A.x = lc, A.prev = lc, A.next = ln;
        A.alpha = (float)alpha;
        A.tau = (float)tau;
        if (in.timing) sw.start();
        launch_sweep<MODE_ADJOINT>(var, A, W, s);
        if (in.timing) sw.stop();
        L++;
        SL++;
        double h2[2];
        GTC_CUDA(cudaMemcpyAsync(h2, dq, sizeof(h2), cudaMemcpyDeviceToHost, s));
        GTC_CUDA(cudaStreamSynchronize(s));
        if (in.timing) sweep_ms += sw.ms();
        delta = h2[0];
        alpha_prev = alpha;
        if (deflate)
            alpha = (tau - h2[1]) / psum;
        else
            tau = h2[1];
        std::swap(lc, ln);
        iter++;
        if (max_iter > 0 && iter == max_iter) break;
    }
    total.stop();
    res->device_ms = total.ms();
    // gradients, with lambda = lc + alpha
    if (in.grad_p && n) {
        k_grad_pers<<<grid_for(n, TB, 1u << 30), TB, 0, s>>>(n, g->iperm.get(), lc, (float)alpha,
                                                             dp + 1, 1.0 - d, d, in.grad_p,
                                                             in.grad_p_dtype);
        GTC_LAUNCHED();
        L++;
    }
    if (in.grad_w && av.m_pull) {
        DevBuf<uint32_t> rowid(av.m_pull, s);
        k_row_ids<<<grid_for((size_t)n * 8, TB, 1u << 30), TB, 0, s>>>(n, av.pull_off, rowid.get());
        k_grad_w<<<grid_for(av.m_pull, TB, 1u << 30), TB, 0, s>>>(
            av.m_pull, rowid.get(), av.pull_other, av.pull_eid, ypi.get(), lc, atl.get(),
            P.sinkp, (float)d, (float)(alpha - alpha_prev), in.grad_w, in.grad_w_dtype);
        GTC_LAUNCHED();
        L += 2;
    }
    GTC_CUDA(cudaStreamSynchronize(s));
    res->iterations = iter;
    res->last_delta = iter ? delta : 0.0;
    res->eigenvalue = 0.0;
    res->launches = L;
    res->sweep_ms = sweep_ms;
    res->sweep_launches = SL;
    g->launches += L;
}

// weighted_out_degree / weighted_in_degree (crates/gt-algo/src/degree.rs
// :122-160) of every vertex of a view: the FP64 left fold from 0.0 of the
// weights over the out-half (in-half) in storage order -- the reference's
// sum_weights (degree.rs:68-82) -- or the degree for a Unity map (weight
// NULL).  Vertices outside the view get 0.  Host arrays.
void weighted_degree(gtc_graph* g, const gtc_view* vw, const double* w_host, bool in_dir,
                     double* deg_host, cudaStream_t s) {
    uint64_t L = 0;
    View view;
    view.prepare(g, vw, s, &L);
    const uint32_t n = view.n;
    const uint64_t m = g->m;
    DevBuf<double> dw;
    if (w_host && m) {
        dw.alloc(m, s);
        GTC_CUDA(cudaMemcpyAsync(dw.get(), w_host, m * sizeof(double), cudaMemcpyHostToDevice, s));
    }
    if (n) {
        DevBuf<double> deg(n, s), out(n, s);
        DevBuf<uint8_t> sink(n, s);
        k_degree<<<grid_for(n, 256, 1u << 30), 256, 0, s>>>(
            n, in_dir ? view.pull_off : view.push_off, in_dir ? view.pull_eid : view.push_eid,
            w_host ? dw.get() : nullptr, GTC_F64, view.active_or_null(), deg.get(), sink.get());
        GTC_LAUNCHED();
        k_store<double><<<grid_for(n, 256, 1u << 30), 256, 0, s>>>(n, g->iperm.get(), deg.get(),
                                                                   nullptr, nullptr, out.get(),
                                                                   GTC_F64);
        GTC_LAUNCHED();
        L += 2;
        GTC_CUDA(cudaMemcpyAsync(deg_host, out.get(), (size_t)n * sizeof(double),
                                 cudaMemcpyDeviceToHost, s));
    }
    GTC_CUDA(cudaStreamSynchronize(s));
    g->launches += L;
}

}  // namespace gtc
