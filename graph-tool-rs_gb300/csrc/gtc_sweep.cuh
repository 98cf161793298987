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
// Every row sum is compensated (Kahan).  A persistent grid walks the work
// list with a fixed stride, so a row's sum, and the per-CTA partials folded
// in CTA order at the end, do not depend on timing: the FP32 path is
// deterministic run to run.
#pragma once

#include "gtc_internal.cuh"

namespace gtc {

constexpr int SP_NT = 256;
constexpr int SP_WARPS = SP_NT / 32;
constexpr int SP_CAP = 2048;        // entries per long-row chunk; longest medium row
constexpr int SP_SLICE_MAX = 128;   // longest row kept in a slice
constexpr int SP_WINDOW = 2048;     // rows sorted by length inside windows of this many
constexpr uint32_t NO_ROW = 0xFFFFFFFFu;

// Work-unit kinds (uint4.x); .y/.z as described.
constexpr uint32_t UNIT_LONG = 1;    // long row index y, chunk z
constexpr uint32_t UNIT_MEDIUM = 2;  // medium rows med[y .. z), one per warp
constexpr uint32_t UNIT_SLICES = 3;  // slices [y, z), strided over the warps
constexpr uint32_t SLICES_PER_UNIT = 4 * SP_WARPS;

// Cut the rows of a pull half into the three tiers and the work list.
void build_units(const uint32_t* d_off, const uint32_t* d_other, const uint32_t* d_eid,
                 uint32_t n, cudaStream_t s, Units& u);

enum SweepMode { MODE_PAGERANK = 0, MODE_EIGEN = 1 };

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
    double2* long_out;
    uint32_t n_units, n_long;
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
    const float* __restrict__ pers;     // PageRank only (null = uniform)
    float uniform, one_minus_d, d;
    const double* psink;                // PageRank: dangling mass of prev
    // reduction: per-CTA partials, folded by the last CTA
    double* part_a;
    double* part_b;
    unsigned* ticket;
    double* out;  // [a, b]
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
// gathered vector is what stays in L2.
template <int MODE>
__device__ __forceinline__ void sweep_row(const SweepArgs& A, uint32_t v, float sum, float psink,
                                          float& ta, float& tb) {
    if (A.active && !A.active[v]) {
        A.next[v] = A.prev[v];
        if (MODE == MODE_PAGERANK) A.ynext[v] = 0.f;
        ta = 0.f, tb = 0.f;
        return;
    }
    if (MODE == MODE_PAGERANK) {
        const float pv = A.pers ? __ldcs(A.pers + v) : A.uniform;
        const float r = __fadd_rn(__fmul_rn(psink, pv), sum);
        const float nv = __fadd_rn(__fmul_rn(A.one_minus_d, pv), __fmul_rn(A.d, r));
        __stcs(A.next + v, nv);
        A.ynext[v] = __fmul_rn(nv, __ldcs(A.invdeg + v));
        ta = fabsf(__fsub_rn(nv, __ldcs(A.prev + v)));
        tb = __ldcs(A.sink + v) ? nv : 0.f;
    } else {
        A.next[v] = sum;
        ta = __fmul_rn(sum, sum);
        tb = 0.f;
    }
}

template <int MODE, bool WEIGHTED>
__global__ void __launch_bounds__(SP_NT, 6) k_sweep(SweepArgs A) {
    __shared__ float2 red[SP_WARPS];
    __shared__ double fa[SP_WARPS], fb[SP_WARPS];
    __shared__ bool flag;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const float psink = MODE == MODE_PAGERANK ? (float)*A.psink : 0.f;
    KahanLite acc_a, acc_b;

    for (uint32_t u = blockIdx.x; u < A.n_units; u += gridDim.x) {
        const uint4 U = A.units[u];
        if (U.x == UNIT_SLICES) {
            // this warp's slices: U.y + warp, + SP_WARPS, ...
            for (uint32_t k = U.y + warp; k < U.z; k += SP_WARPS) {
                const uint32_t b = __ldg(A.slice_off + k);
                const uint32_t len = (__ldg(A.slice_off + k + 1) - b) >> 5;
                const uint32_t row = __ldg(A.slice_rows + 32 * k + lane);
                const uint32_t* ip = A.sidx + b + lane;
                const float* wp = WEIGHTED ? A.sw + b + lane : nullptr;
                KahanLite acc;
                uint32_t j = 0;
                for (; j + 4 <= len; j += 4) {
                    const uint32_t s0 = __ldcs(ip), s1 = __ldcs(ip + 32), s2 = __ldcs(ip + 64),
                                   s3 = __ldcs(ip + 96);
                    float v0 = A.x[s0], v1 = A.x[s1], v2 = A.x[s2], v3 = A.x[s3];
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
                    ip += 128;
                }
                for (; j < len; ++j) {
                    float v = A.x[__ldcs(ip)];
                    if (WEIGHTED) {
                        v = __fmul_rn(v, __ldcs(wp));
                        wp += 32;
                    }
                    acc.add(v);
                    ip += 32;
                }
                if (row != NO_ROW) {
                    float ta, tb;
                    sweep_row<MODE>(A, row, acc.value(), psink, ta, tb);
                    acc_a.add(ta);
                    acc_b.add(tb);
                }
            }
        } else if (U.x == UNIT_MEDIUM) {
            const uint32_t q = U.y + warp;
            if (q < U.z) {
                const uint32_t row = __ldg(A.med + q);
                const uint32_t b = __ldg(A.off + row), e = __ldg(A.off + row + 1);
                KahanLite kl;
                uint32_t p = b + lane;
                for (; p + 96 < e; p += 128) {
                    const uint32_t s0 = __ldcs(A.other + p), s1 = __ldcs(A.other + p + 32),
                                   s2 = __ldcs(A.other + p + 64), s3 = __ldcs(A.other + p + 96);
                    float v0 = A.x[s0], v1 = A.x[s1], v2 = A.x[s2], v3 = A.x[s3];
                    if (WEIGHTED) {
                        v0 = __fmul_rn(v0, __ldcs(A.w + p));
                        v1 = __fmul_rn(v1, __ldcs(A.w + p + 32));
                        v2 = __fmul_rn(v2, __ldcs(A.w + p + 64));
                        v3 = __fmul_rn(v3, __ldcs(A.w + p + 96));
                    }
                    kl.add(v0);
                    kl.add(v1);
                    kl.add(v2);
                    kl.add(v3);
                }
                for (; p < e; p += 32) {
                    float v = A.x[__ldcs(A.other + p)];
                    if (WEIGHTED) v = __fmul_rn(v, __ldcs(A.w + p));
                    kl.add(v);
                }
                Kahan k = kl.full();
                warp_merge_kahan(k);
                if (lane == 0) {
                    float ta, tb;
                    sweep_row<MODE>(A, row, k.value(), psink, ta, tb);
                    acc_a.add(ta);
                    acc_b.add(tb);
                }
            }
        } else {  // UNIT_LONG
            const uint4 LR = A.longs[U.y];
            const uint32_t row = LR.x, c = U.z;
            const uint32_t b = __ldg(A.off + row) + c * SP_CAP;
            const uint32_t e = min(b + (uint32_t)SP_CAP, __ldg(A.off + row + 1));
            constexpr int IPT = SP_CAP / SP_NT;
            uint32_t idx[IPT];
            float wv[IPT];
#pragma unroll
            for (int k = 0; k < IPT; ++k) {
                const uint32_t p = b + tid + k * SP_NT;
                idx[k] = p < e ? __ldcs(A.other + p) : 0u;
                if (WEIGHTED) wv[k] = p < e ? __ldcs(A.w + p) : 0.f;
            }
            KahanLite kl;
#pragma unroll
            for (int k = 0; k < IPT; ++k) {
                const uint32_t p = b + tid + k * SP_NT;
                if (p < e) {
                    const float xv = A.x[idx[k]];
                    kl.add(WEIGHTED ? __fmul_rn(xv, wv[k]) : xv);
                }
            }
            Kahan k = kl.full();
            warp_merge_kahan(k);
            if (lane == 0) red[warp] = make_float2(k.s, k.c);
            __syncthreads();
            if (tid == 0) {
                Kahan t;
                for (int w = 0; w < SP_WARPS; ++w) t.merge(red[w].x, red[w].y);
                A.partial[LR.y + c] = make_float2(t.s, t.c);
                __threadfence();
                const unsigned done = atomicAdd(&A.counter[U.y], 1u);
                flag = (done == LR.z - 1);
            }
            __syncthreads();
            if (flag && tid == 0) {
                __threadfence();
                Kahan t;
                for (uint32_t q = 0; q < LR.z; ++q) {
                    const float2 pq = __ldcg(&A.partial[LR.y + q]);
                    t.merge(pq.x, pq.y);
                }
                A.counter[U.y] = 0u;
                float ta, tb;
                sweep_row<MODE>(A, row, t.value(), psink, ta, tb);
                // a long row's terms are folded by index, not by whichever
                // CTA happened to finish it, so the sums stay deterministic
                A.long_out[U.y] = make_double2((double)ta, (double)tb);
            }
            __syncthreads();
        }
    }

    // ---- deterministic fold: CTA partials, then long-row terms, in order ----
    double a = (double)acc_a.s - (double)acc_a.c;
    double b = (double)acc_b.s - (double)acc_b.c;
    a = warp_sum_f64(a);
    b = warp_sum_f64(b);
    if (lane == 0) fa[warp] = a, fb[warp] = b;
    __syncthreads();
    if (tid == 0) {
        double ta = 0.0, tb = 0.0;
        for (int w = 0; w < SP_WARPS; ++w) ta += fa[w], tb += fb[w];
        A.part_a[blockIdx.x] = ta;
        A.part_b[blockIdx.x] = tb;
        __threadfence();
        const unsigned t = atomicAdd(A.ticket, 1u);
        flag = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (flag && warp == 0) {
        __threadfence();
        double ta = 0.0, tb = 0.0;
        for (unsigned i = lane; i < gridDim.x; i += 32) {
            ta += __ldcg(A.part_a + i);
            tb += __ldcg(A.part_b + i);
        }
        for (unsigned i = lane; i < A.n_long; i += 32) {
            const double2 q = __ldcg(A.long_out + i);
            ta += q.x;
            tb += q.y;
        }
        ta = warp_sum_f64(ta);
        tb = warp_sum_f64(tb);
        if (lane == 0) {
            A.out[0] = ta;
            A.out[1] = tb;
            *A.ticket = 0u;
        }
    }
}

}  // namespace gtc
