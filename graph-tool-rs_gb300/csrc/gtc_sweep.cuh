// gtc_sweep.cuh -- the pull sweep of PageRank and eigenvector centrality
// (FP32 fast path), scheduled by in-degree.
//
// The rows of a pull half are split by their number of entries into three
// tiers, laid out once per graph (build_units, gtc_sweep.cu):
//
//   sliced rows (<= SP_SLICE_MAX entries)  Inside windows of SP_WINDOW
//       consecutive rows, rows are ordered by entry count and cut into slices
//       of 32.  A slice is stored column-major (the sliced-ELL layout): entry
//       j of lane i's row sits at slice_base + 32*j + i, short rows padded
//       with an index that gathers 0.  One warp sums a slice, a row per lane:
//       every load of the index stream is one coalesced 128-byte line, no
//       lane idles (rows of a slice have nearly equal lengths), and no
//       shared memory or barrier is involved.
//   medium rows (<= SP_CAP entries)  one warp per row, lanes striding the
//       row's entries in the pull half, merged with TwoSum shuffles.
//   long rows  SP_CAP-entry chunks, one CTA each; the last CTA of a row
//       (atomic ticket) folds the chunk partials in chunk order.
//
// Every row sum is compensated (Kahan) in the row's storage order, and the
// per-row reduction terms (L1 change, dangling mass, squared norm) are
// summed exactly in 128-bit fixed point, so neither depends on the grid, on
// timing or on the kernel variant: the FP32 path is deterministic run to
// run and across variants.
#pragma once

#include "gtc_internal.cuh"

namespace gtc {

constexpr int SP_CAP = 2048;        // entries per long-row chunk; longest medium row
// Variant with a shared-memory copy of the hottest entries of the gathered
// vector: vertices are labelled by descending out-degree, so its first
// SP_HOT entries are the most gathered ones (the rest is read through
// L1/L2).  One 1024-thread CTA per SM holds them.
constexpr int SP_HOT = 32768;
constexpr int SP_BUCKET = 8;        // work items a warp takes together (one fold term)
constexpr int SP_SLICE_MAX = 128;   // longest row kept in a slice
constexpr int SP_WINDOW = 2048;     // rows sorted by length inside windows of this many
constexpr uint32_t NO_ROW = 0xFFFFFFFFu;

// Work items, one warp each (uint4.x = kind; .y/.z/.w as described).
constexpr uint32_t UNIT_LONG = 1;    // long row index y, chunk z
constexpr uint32_t UNIT_MEDIUM = 2;  // row y, its entries [z, w) of the pull half
constexpr uint32_t UNIT_SLICES = 3;  // slice y, first sliced entry z, w steps of 32

// Cut the rows of a pull half into the three tiers and the work list.
void build_units(const uint32_t* d_off, const uint32_t* d_other, const uint32_t* d_eid,
                 uint32_t n, cudaStream_t s, Units& u);

// PAGERANK: the pull sweep of pagerank_with.  EIGEN: the unnormalised sweep
// of eigenvector.  ADJOINT: one step of the adjoint fixed point
// lambda <- g + d (A^T lambda + s (p^T lambda)) of PageRank, pulled over the
// out-halves (A^T lambda at s is a sum over s's out-edges).
enum SweepMode { MODE_PAGERANK = 0, MODE_EIGEN = 1, MODE_ADJOINT = 2 };

struct SweepArgs {
    // schedule
    const uint4* __restrict__ units;
    const uint4* __restrict__ longs;
    const uint32_t* __restrict__ med;         // medium rows
    const uint32_t* __restrict__ slice_rows;  // 32 per slice (NO_ROW pads)
    const uint32_t* __restrict__ slice_off;   // first entry of each slice (n_slices + 1)
    const uint32_t* __restrict__ sidx;        // sliced entries: source vertex (n = padding)
    const float* __restrict__ sw;             // sliced entries: weight (null = Unity)
    float2* partial;
    unsigned* counter;
    uint32_t n_units, n_long;
    uint32_t hot_n;     // entries of x staged in shared memory (HOT variant)
    // pull half (medium and long rows)
    const uint32_t* __restrict__ off;
    const uint32_t* __restrict__ other;
    const float* __restrict__ w;   // pull-ordered weights or null
    const float* __restrict__ x;   // the gathered vector, n+1 entries, x[n] == 0
    // epilogue
    const uint8_t* __restrict__ active;
    const float* __restrict__ prev;
    float* __restrict__ next;
    float* __restrict__ ynext;          // PageRank only
    const float* __restrict__ invdeg;   // PageRank only
    const uint8_t* __restrict__ sink;   // PageRank only
    const float* __restrict__ pers;     // PageRank / adjoint (null = uniform)
    const float* __restrict__ gvec;     // adjoint: dL/dpi
    float uniform, one_minus_d, d;
    const double* psink;                // PageRank: dangling mass of prev
    float alpha, tau;                   // adjoint: shift of the iterate, p . (shifted iterate)
    // reduction: the rows' (a, b) terms, summed exactly
    ExactFold fold;
    const unsigned* stop;  // non-null and set: the iteration has stopped, return at once
};

// The exact format of a mode's reduction terms.
template <int MODE>
struct SweepAcc {
    using type = ExactPR;
};
template <>
struct SweepAcc<MODE_EIGEN> {
    using type = ExactEV;
};

// Classic Kahan accumulator for the inner loops (value = s - c), 4 flops a
// term; converted to a TwoSum pair (Kahan) to merge across lanes.
struct KahanLite {
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void add(float x) {
        const float y = __fsub_rn(x, c);
        const float t = __fadd_rn(s, y);
        c = __fsub_rn(__fsub_rn(t, s), y);
        s = t;
    }
    __device__ __forceinline__ float value() const { return __fsub_rn(s, c); }
    __device__ __forceinline__ Kahan full() const {
        Kahan k;
        k.s = s;
        k.c = -c;
        return k;
    }
};

// The per-row epilogue.  PageRank: (a, b) = (|nv - prev|, dangling mass of
// next).  Eigenvector: a = s^2 (the squared norm), next = s unnormalised.
// Streamed once per sweep: loaded and stored evict-first (.cs), so the
// gathered vector is what stays in L2.  The row's own operands are loaded
// by row_load as soon as the row is known -- before its gathers -- so their
// latency overlaps the gathers instead of following them.
struct RowIn {
    float prev = 0.f, invdeg = 0.f, pers = 0.f, g = 0.f;
    bool sink = false, active = true;
};

template <int MODE>
__device__ __forceinline__ RowIn row_load(const SweepArgs& A, uint32_t v) {
    RowIn r;
    if (A.active) r.active = A.active[v] != 0;
    if (MODE != MODE_EIGEN)
        r.prev = __ldcs(A.prev + v);
    else if (!r.active)  // eigenvector reads prev only to carry an inactive row
        r.prev = A.prev[v];
    if (MODE != MODE_EIGEN) {
        r.invdeg = __ldcs(A.invdeg + v);
        r.sink = __ldcs(A.sink + v) != 0;
        r.pers = A.pers ? __ldcs(A.pers + v) : A.uniform;
    }
    if (MODE == MODE_ADJOINT) r.g = __ldcs(A.gvec + v);
    return r;
}

template <int MODE>
__device__ __forceinline__ void row_finish(const SweepArgs& A, uint32_t v, const RowIn& in,
                                           float sum, float psink, float& ta, float& tb) {
    if (!in.active) {
        A.next[v] = in.prev;
        if (MODE == MODE_PAGERANK) A.ynext[v] = 0.f;
        ta = 0.f, tb = 0.f;
        return;
    }
    if (MODE == MODE_PAGERANK) {
        const float pv = in.pers;
        const float r = __fadd_rn(__fmul_rn(psink, pv), sum);
        const float nv = __fadd_rn(__fmul_rn(A.one_minus_d, pv), __fmul_rn(A.d, r));
        __stcs(A.next + v, nv);
        // y of a dangling row is 0 (invdeg 0) in both buffers already: not
        // storing it keeps those lines out of L2
        if (!in.sink) A.ynext[v] = __fmul_rn(nv, in.invdeg);
        ta = fabsf(__fsub_rn(nv, in.prev));
        tb = in.sink ? nv : 0.f;
    } else if (MODE == MODE_ADJOINT) {
        // The iterate is mu + alpha (a shift along the all-ones vector, which
        // the transposed map keeps: A^T 1 = 1 off the sinks).  sum = sum over
        // v's out-edges of w * mu[t], so (A^T (mu + alpha))_v = at + alpha off
        // the sinks, and a sink takes p . (mu + alpha) = tau.
        const float at = __fmul_rn(in.invdeg, sum);
        const float dn = __fadd_rn(at, in.sink ? A.tau : A.alpha);
        const float nv = __fadd_rn(in.g, __fmul_rn(A.d, dn));
        __stcs(A.next + v, nv);
        A.ynext[v] = at;  // kept for the weight gradient
        // the fixed-point residual of the shifted iterate
        ta = fabsf(__fsub_rn(__fsub_rn(nv, in.prev), A.alpha));
        tb = __fmul_rn(in.pers, nv);  // p . (next iterate, before its shift)
    } else {
        A.next[v] = sum;
        ta = __fmul_rn(sum, sum);
        tb = 0.f;
    }
}

template <int MODE>
__device__ __forceinline__ void sweep_row(const SweepArgs& A, uint32_t v, float sum, float psink,
                                          float& ta, float& tb) {
    row_finish<MODE>(A, v, row_load<MODE>(A, v), sum, psink, ta, tb);
}

template <bool HOT>
__device__ __forceinline__ float gather(const SweepArgs& A, const float* hot, uint32_t s) {
    return (HOT && s < A.hot_n) ? hot[s] : __ldg(A.x + s);
}

// NT threads per CTA; HOT: stage x[0 .. hot_n) in shared memory.
template <int MODE, bool WEIGHTED, int NT, bool HOT>
__global__ void __launch_bounds__(NT, HOT ? 1 : 6) k_sweep(SweepArgs A) {
    constexpr int SP_WARPS = NT / 32;
    constexpr bool ROUND8 = NT >= 1024;  // rounds of eight gathers a lane (see the slices)
    extern __shared__ float hot[];  // x[0 .. hot_n)
    using Acc = typename SweepAcc<MODE>::type;
    if (A.stop && *A.stop) return;  // the same for every CTA: before any barrier
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const float psink = MODE != MODE_EIGEN ? (float)*A.psink : 0.f;
    if (HOT) {
        const float4* src = reinterpret_cast<const float4*>(A.x);
        float4* dst = reinterpret_cast<float4*>(hot);
        const uint32_t n4 = A.hot_n / 4;  // hot_n is a multiple of 4
        for (uint32_t i = tid; i < n4; i += NT) dst[i] = __ldg(src + i);
        __syncthreads();
    }
    const bool H = HOT && A.hot_n != 0;

    const uint32_t gw = blockIdx.x * SP_WARPS + warp, nw = gridDim.x * SP_WARPS;
    // A warp takes buckets of up to SP_BUCKET items, bucket b being items
    // b, b + B, b + 2B, ... (B buckets): every bucket mixes heavy and light
    // items.  Every row's (a, b) terms are added exactly (Acc), so neither
    // the grid, the CTA size nor the assignment of items to warps changes a
    // single bit of the sums.
    Acc acc_a, acc_b;
    const uint32_t n_buckets = (A.n_units + SP_BUCKET - 1) / SP_BUCKET;
    for (uint32_t bk = gw; bk < n_buckets; bk += nw) {
    // the next item's descriptor is loaded while this item runs
    // (the work list and the slices' row lists are read once a sweep:
    // evict-first, like the index stream, so the gathered vector keeps L2)
    uint4 Unext = __ldcs(A.units + bk);
    for (uint32_t u = bk; u < A.n_units; u += n_buckets) {
        const uint4 U = Unext;
        if (u + n_buckets < A.n_units) Unext = __ldcs(A.units + u + n_buckets);
        if (U.x == UNIT_SLICES) {
            // {kind, slice, first entry, steps}: no table lookup before the
            // index stream starts
            const uint32_t k = U.y, b = U.z, len = U.w;
            const uint32_t row = __ldcs(A.slice_rows + 32 * k + lane);
            const uint32_t* ip = A.sidx + b + lane;
            const float* wp = WEIGHTED ? A.sw + b + lane : nullptr;
            KahanLite acc;
            uint32_t j = 0;
            // four entries a step; the next step's four indices are loaded
            // before this step's gathers, so an index load and a gather are
            // in flight together instead of one after the other
            auto step = [&](uint32_t s0, uint32_t s1, uint32_t s2, uint32_t s3) {
                float v0, v1, v2, v3;
                if (H) {
                    v0 = gather<HOT>(A, hot, s0), v1 = gather<HOT>(A, hot, s1);
                    v2 = gather<HOT>(A, hot, s2), v3 = gather<HOT>(A, hot, s3);
                } else {
                    v0 = __ldg(A.x + s0), v1 = __ldg(A.x + s1);
                    v2 = __ldg(A.x + s2), v3 = __ldg(A.x + s3);
                }
                if (WEIGHTED) {
                    v0 = __fmul_rn(v0, __ldcs(wp));
                    v1 = __fmul_rn(v1, __ldcs(wp + 32));
                    v2 = __fmul_rn(v2, __ldcs(wp + 64));
                    v3 = __fmul_rn(v3, __ldcs(wp + 96));
                    wp += 128;
                }
                acc.add(v0);
                acc.add(v1);
                acc.add(v2);
                acc.add(v3);
            };
            // rounds of eight entries (two steps), the next round's indices
            // loaded before this round's gathers; then at most one step of
            // four; then single entries.  Eight gathers in flight a lane
            // measured 1.3 % faster than four on RMAT-24 at the same 64
            // registers (fewer threads for more registers were slower); the
            // 256-thread kernel, at 40 registers, keeps rounds of four.
            RowIn rin;
            if (ROUND8 && len >= 8) {
                uint32_t sv[8];
#pragma unroll
                for (int k = 0; k < 8; ++k) sv[k] = __ldcs(ip + 32 * k);
                ip += 256;
                if (row != NO_ROW) rin = row_load<MODE>(A, row);
                for (; j + 16 <= len; j += 8) {
                    uint32_t nv[8];
#pragma unroll
                    for (int k = 0; k < 8; ++k) nv[k] = __ldcs(ip + 32 * k);
                    ip += 256;
                    step(sv[0], sv[1], sv[2], sv[3]);
                    step(sv[4], sv[5], sv[6], sv[7]);
#pragma unroll
                    for (int k = 0; k < 8; ++k) sv[k] = nv[k];
                }
                step(sv[0], sv[1], sv[2], sv[3]);
                step(sv[4], sv[5], sv[6], sv[7]);
                j += 8;
            } else if (row != NO_ROW) {
                rin = row_load<MODE>(A, row);
            }
            if (!ROUND8 && len >= 4) {
                uint32_t s0 = __ldcs(ip), s1 = __ldcs(ip + 32), s2 = __ldcs(ip + 64),
                         s3 = __ldcs(ip + 96);
                ip += 128;
                for (; j + 8 <= len; j += 4) {
                    const uint32_t n0 = __ldcs(ip), n1 = __ldcs(ip + 32), n2 = __ldcs(ip + 64),
                                   n3 = __ldcs(ip + 96);
                    ip += 128;
                    step(s0, s1, s2, s3);
                    s0 = n0, s1 = n1, s2 = n2, s3 = n3;
                }
                step(s0, s1, s2, s3);
                j += 4;
            } else if (j + 4 <= len) {
                const uint32_t s0 = __ldcs(ip), s1 = __ldcs(ip + 32), s2 = __ldcs(ip + 64),
                               s3 = __ldcs(ip + 96);
                ip += 128;
                step(s0, s1, s2, s3);
                j += 4;
            }
            for (; j < len; ++j) {
                float v = gather<HOT>(A, hot, __ldcs(ip));
                if (WEIGHTED) {
                    v = __fmul_rn(v, __ldcs(wp));
                    wp += 32;
                }
                acc.add(v);
                ip += 32;
            }
            if (row != NO_ROW) {
                float ta, tb;
                row_finish<MODE>(A, row, rin, acc.value(), psink, ta, tb);
                acc_a.add(ta);
                acc_b.add(tb);
            }
        } else {
            // a medium row, or one chunk of a long row: lanes stride entries
            uint32_t row, b, e;
            uint4 LR = make_uint4(0, 0, 0, 0);
            RowIn rin;
            if (U.x == UNIT_MEDIUM) {
                // {kind, row, first entry, end}
                row = U.y, b = U.z, e = U.w;
                rin = row_load<MODE>(A, row);
            } else {
                LR = A.longs[U.y];
                row = LR.x;
                b = __ldg(A.off + row) + U.z * SP_CAP;
                e = min(b + (uint32_t)SP_CAP, __ldg(A.off + row + 1));
            }
            KahanLite kl;
            uint32_t p = b + lane;
            // rounds of four entries a lane; the next round's indices are
            // loaded before this round's gathers (as in the slice loop)
            auto round = [&](uint32_t q, uint32_t s0, uint32_t s1, uint32_t s2, uint32_t s3) {
                float v0 = gather<HOT>(A, hot, s0), v1 = gather<HOT>(A, hot, s1);
                float v2 = gather<HOT>(A, hot, s2), v3 = gather<HOT>(A, hot, s3);
                if (WEIGHTED) {
                    v0 = __fmul_rn(v0, __ldcs(A.w + q));
                    v1 = __fmul_rn(v1, __ldcs(A.w + q + 32));
                    v2 = __fmul_rn(v2, __ldcs(A.w + q + 64));
                    v3 = __fmul_rn(v3, __ldcs(A.w + q + 96));
                }
                kl.add(v0);
                kl.add(v1);
                kl.add(v2);
                kl.add(v3);
            };
            // (the 1024-thread kernels: rounds of eight, as in the slices)
            if (ROUND8 && p + 224 < e) {
                uint32_t sv[8];
#pragma unroll
                for (int k = 0; k < 8; ++k) sv[k] = __ldcs(A.other + p + 32 * k);
                for (; p + 256 + 224 < e; p += 256) {
                    uint32_t nv[8];
#pragma unroll
                    for (int k = 0; k < 8; ++k) nv[k] = __ldcs(A.other + p + 256 + 32 * k);
                    round(p, sv[0], sv[1], sv[2], sv[3]);
                    round(p + 128, sv[4], sv[5], sv[6], sv[7]);
#pragma unroll
                    for (int k = 0; k < 8; ++k) sv[k] = nv[k];
                }
                round(p, sv[0], sv[1], sv[2], sv[3]);
                round(p + 128, sv[4], sv[5], sv[6], sv[7]);
                p += 256;
            }
            if (p + 96 < e) {
                uint32_t s0 = __ldcs(A.other + p), s1 = __ldcs(A.other + p + 32),
                         s2 = __ldcs(A.other + p + 64), s3 = __ldcs(A.other + p + 96);
                for (; p + 128 + 96 < e; p += 128) {
                    const uint32_t n0 = __ldcs(A.other + p + 128), n1 = __ldcs(A.other + p + 160),
                                   n2 = __ldcs(A.other + p + 192), n3 = __ldcs(A.other + p + 224);
                    round(p, s0, s1, s2, s3);
                    s0 = n0, s1 = n1, s2 = n2, s3 = n3;
                }
                round(p, s0, s1, s2, s3);
                p += 128;
            }
            for (; p < e; p += 32) {
                float v = gather<HOT>(A, hot, __ldcs(A.other + p));
                if (WEIGHTED) v = __fmul_rn(v, __ldcs(A.w + p));
                kl.add(v);
            }
            Kahan k = kl.full();
            warp_merge_kahan(k);
            if (U.x == UNIT_MEDIUM) {
                if (lane == 0) {
                    float ta, tb;
                    row_finish<MODE>(A, row, rin, k.value(), psink, ta, tb);
                    acc_a.add(ta);
                    acc_b.add(tb);
                }
            } else {
                // long row: the last warp to finish a chunk folds the chunks
                bool last = false;
                if (lane == 0) {
                    A.partial[LR.y + U.z] = make_float2(k.s, k.c);
                    __threadfence();
                    const unsigned done = atomicAdd(&A.counter[U.y], 1u);
                    last = (done == LR.z - 1);
                    if (last) {
                        __threadfence();
                        Kahan t;
                        for (uint32_t q = 0; q < LR.z; ++q) {
                            const float2 pq = __ldcg(&A.partial[LR.y + q]);
                            t.merge(pq.x, pq.y);
                        }
                        A.counter[U.y] = 0u;
                        float ta, tb;
                        sweep_row<MODE>(A, row, t.value(), psink, ta, tb);
                        acc_a.add(ta);
                        acc_b.add(tb);
                    }
                }
            }
        }
    }

    }

    // ---- the CTA's exact sums, added up by the last CTA ----
    __syncthreads();
    block_fold_exact<NT>(acc_a, acc_b, A.fold);
}

}  // namespace gtc
