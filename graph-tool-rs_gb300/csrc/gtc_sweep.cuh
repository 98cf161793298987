// gtc_sweep.cuh -- the pull sweep of PageRank and eigenvector centrality
// (FP32 fast path), scheduled by degree.
//
// The rows of the pull half are cut once per graph into work units
// (build_units, host side, one O(n) pass over the offsets):
//
//   short unit  a run of consecutive rows whose entries plus rows fit in
//               SP_CAP merge items.  A CTA streams the run's source indices
//               (coalesced), gathers y[src] (x w) into shared memory, then
//               sums each row there: rows of <= SP_WARP_ROW entries one
//               thread each, longer rows one warp each.
//   long chunk  SP_CAP entries of a row too long for a short unit.  A CTA
//               sums its chunk; the last CTA of the row (atomic ticket) folds
//               the chunk partials in chunk order and finishes the row.
//
// A persistent grid walks the units with a fixed stride, so every row is
// summed in a fixed order and the per-CTA partials are folded in CTA order:
// the FP32 path is deterministic run to run.
#pragma once

#include "gtc_internal.cuh"

namespace gtc {

constexpr int SP_NT = 256;
constexpr int SP_WARPS = SP_NT / 32;
constexpr int SP_CAP = 2048;       // merge items per short unit / entries per long chunk
constexpr int SP_WARP_ROW = 32;    // rows with more entries are summed by a warp

// Work-unit kinds (uint4.x); .y/.z as described.
constexpr uint32_t UNIT_SHORT = 0;  // rows [y, z)
constexpr uint32_t UNIT_LONG = 1;   // long row index y, chunk z

// Cut the rows of a pull half (offsets in device memory) into work units.
void build_units(const uint32_t* d_off, uint32_t n, cudaStream_t s, Units& u);

// --------------------------------------------------------------------------
// sweep arguments
// --------------------------------------------------------------------------

enum SweepMode { MODE_PAGERANK = 0, MODE_EIGEN = 1 };

struct SweepArgs {
    // schedule
    const uint4* __restrict__ units;
    const uint4* __restrict__ longs;
    float2* partial;
    unsigned* counter;
    double2* long_out;
    uint32_t n_units, n_long;
    // pull half
    const uint32_t* __restrict__ off;
    const uint32_t* __restrict__ other;
    const float* __restrict__ w;   // pull-ordered weights or null
    const float* __restrict__ x;   // the gathered vector (PageRank: y = rank/deg)
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

// The per-row epilogue.  PageRank: (a, b) = (|nv - prev|, dangling mass of
// next).  Eigenvector: a = s^2 (the squared norm), next = s unnormalised.
template <int MODE>
__device__ __forceinline__ void sweep_row(const SweepArgs& A, uint32_t v, float sum, float psink,
                                          float& ta, float& tb) {
    // Streamed once per sweep: loaded and stored evict-first (.cs), so the
    // gathered vector is what stays in L2.
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

// Classic Kahan accumulator for the inner loops (value = s - c); 4 flops per
// term.  Merged across lanes with TwoSum (Kahan::merge).
struct KahanLite {
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void add(float x) {
        const float y = __fsub_rn(x, c);
        const float t = __fadd_rn(s, y);
        c = __fsub_rn(__fsub_rn(t, s), y);
        s = t;
    }
    __device__ __forceinline__ Kahan full() const {
        Kahan k;
        k.s = s;
        k.c = -c;
        return k;
    }
};

constexpr int SP_IPT = SP_CAP / SP_NT;  // entries per thread in a unit / chunk

template <int MODE, bool WEIGHTED>
__global__ void __launch_bounds__(SP_NT, 5) k_sweep(SweepArgs A) {
    __shared__ float vals[SP_CAP];
    __shared__ uint32_t roff[SP_CAP + 1];
    __shared__ uint32_t wrows[SP_CAP];  // rows of this unit a warp sums
    __shared__ uint32_t n_wrows;
    __shared__ float2 red[SP_WARPS];
    __shared__ double fa[SP_WARPS], fb[SP_WARPS];
    __shared__ bool flag;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const float psink = MODE == MODE_PAGERANK ? (float)*A.psink : 0.f;
    KahanLite acc_a, acc_b;
    if (tid == 0) n_wrows = 0;

    for (uint32_t u = blockIdx.x; u < A.n_units; u += gridDim.x) {
        const uint4 U = A.units[u];
        if (U.x == UNIT_SHORT) {
            const uint32_t r0 = U.y, nr = U.z - U.y;
            const uint32_t z0 = __ldg(A.off + r0);
            const uint32_t nz = __ldg(A.off + U.z) - z0;
            // all index loads first, then all gathers: two round trips per unit
            uint32_t idx[SP_IPT];
            float wv[SP_IPT];
#pragma unroll
            for (int k = 0; k < SP_IPT; ++k) {
                const uint32_t i = tid + k * SP_NT;
                idx[k] = i < nz ? __ldcs(A.other + z0 + i) : 0u;
                if (WEIGHTED) wv[k] = i < nz ? __ldcs(A.w + z0 + i) : 0.f;
            }
            uint32_t ro[SP_IPT + 1];
#pragma unroll
            for (int k = 0; k <= SP_IPT; ++k) {
                const uint32_t i = tid + k * SP_NT;
                ro[k] = i <= nr ? __ldcs(A.off + r0 + i) : 0u;
            }
            float xv[SP_IPT];
#pragma unroll
            for (int k = 0; k < SP_IPT; ++k) {
                const uint32_t i = tid + k * SP_NT;
                xv[k] = i < nz ? A.x[idx[k]] : 0.f;
            }
#pragma unroll
            for (int k = 0; k <= SP_IPT; ++k) {
                const uint32_t i = tid + k * SP_NT;
                if (i <= nr) roff[i] = ro[k] - z0;
            }
#pragma unroll
            for (int k = 0; k < SP_IPT; ++k) {
                const uint32_t i = tid + k * SP_NT;
                if (i < nz) vals[i] = WEIGHTED ? __fmul_rn(xv[k], wv[k]) : xv[k];
            }
            __syncthreads();
            for (uint32_t r = tid; r < nr; r += SP_NT) {
                const uint32_t b = roff[r], e = roff[r + 1];
                if (e - b <= SP_WARP_ROW) {
                    KahanLite k;
                    for (uint32_t j = b; j < e; ++j) k.add(vals[j]);
                    float ta, tb;
                    sweep_row<MODE>(A, r0 + r, __fsub_rn(k.s, k.c), psink, ta, tb);
                    acc_a.add(ta);
                    acc_b.add(tb);
                } else {
                    wrows[atomicAdd(&n_wrows, 1u)] = r;
                }
            }
            __syncthreads();
            const uint32_t nw = n_wrows;
            for (uint32_t q = warp; q < nw; q += SP_WARPS) {
                const uint32_t r = wrows[q];
                const uint32_t b = roff[r], e = roff[r + 1];
                KahanLite kl;
                for (uint32_t j = b + lane; j < e; j += 32) kl.add(vals[j]);
                Kahan k = kl.full();
                warp_merge_kahan(k);
                if (lane == 0) {
                    float ta, tb;
                    sweep_row<MODE>(A, r0 + r, k.value(), psink, ta, tb);
                    acc_a.add(ta);
                    acc_b.add(tb);
                }
            }
            __syncthreads();
            if (tid == 0) n_wrows = 0;
        } else {
            const uint4 LR = A.longs[U.y];
            const uint32_t row = LR.x, c = U.z;
            const uint32_t b = __ldg(A.off + row) + c * SP_CAP;
            const uint32_t e = min(b + (uint32_t)SP_CAP, __ldg(A.off + row + 1));
            uint32_t idx[SP_IPT];
            float wv[SP_IPT];
#pragma unroll
            for (int k = 0; k < SP_IPT; ++k) {
                const uint32_t p = b + tid + k * SP_NT;
                idx[k] = p < e ? __ldcs(A.other + p) : 0u;
                if (WEIGHTED) wv[k] = p < e ? __ldcs(A.w + p) : 0.f;
            }
            KahanLite kl;
#pragma unroll
            for (int k = 0; k < SP_IPT; ++k) {
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
