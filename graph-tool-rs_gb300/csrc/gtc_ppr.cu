// gtc_ppr.cu -- many personalised PageRanks over one edge stream (an SpMM).
//
// B personalisation vectors (seed sets) are solved together: pagerank_with
// (crates/gt-algo/src/centrality.rs:261-384) for every column b, each from
// its own start (a fresh map is seeded with pers_b, centrality.rs:198-205),
// each stopping at the first sweep whose L1 change falls below epsilon
// (centrality.rs:372-381), its value the iterate of that sweep.
//
// Layout.  Z is [n x P] row-major with a pitch P fixed for the whole call
// (32 slots per line, lines for all B columns); a sweep uses the first S =
// 32 * C slots of each row (C = 1-4, 6, 8, 12 or 16 lines of 128 bytes), and
// a warp reads them with C / V coalesced vector loads of V floats per lane
// (Lanes<C>).  Z[v][j] holds rank_b[v] / deg_v of the column b in slot j
// for a vertex with out-edges, and rank_b[v] itself for a sink (a sink is
// never gathered).
//
// Rows without in-edges.  A vertex with no in-edge that is no column's seed
// has rank 0 in every column at every sweep ((1 - d) * 0 + d * (mass * 0 +
// an empty sum)), and so does its change; both iterate buffers start zeroed
// and the sweeps skip these rows (about half the vertices of an R-MAT
// graph).  The fixed pitch keeps a skipped row's slots at zero when the
// active columns are repacked.  Seeds without in-edges are finished by the
// sweep's second kernel with an empty sum.
//
// Active columns only.  Columns converge at very different sweeps (for an
// R-MAT graph and seed sets of 1-64 vertices the last column takes ~2.5x the
// mean).  A column that converged is written to the output right away and
// is no longer computed: the survivors keep their slots (a converged
// column's slot becomes a hole, written as 0) until they fit in fewer lines,
// then they are packed into the lowest slots, so a sweep reads and writes
// about ceil(active / 32) lines per row, not B / 32.  The sweep that drops a
// column still gathers it (its input layout is the previous sweep's output
// layout).
//
// Narrow rows.  With at most 16 columns left (8), the iterate is repacked
// into rows of 16 (8) floats, two (one) 32-byte sectors a row, and a group of
// 16 (8) lanes takes a work item, lane k summing column k (k_ppr_narrow):
// one sector request per gathered row instead of a 128-byte line, and two
// (four) rows per warp instruction.  When at most PPR_HANDOFF columns are
// left, each is finished by the single-vector solver (gtc_centrality.cu) from
// its current iterate.
//
// Schedule.  Rows with more than PPR_CHUNK in-edges are cut into chunks of
// PPR_CHUNK entries; the first kernel of a sweep runs every chunk (a warp
// each, partials to memory) and every other row (a warp each, heaviest
// first), the second merges each long row's chunk partials in chunk order and
// finishes it, the third sums the new iterate over the sink rows (the
// dangling mass of the next sweep) and the fourth folds the CTAs' partials.
// Assignments are fixed strides and every fold runs in a fixed order, so the
// results do not depend on timing.
//
// Latency.  A warp loads its next work item while it works on the current
// one, and a row's epilogue inputs (degree, seeds, previous values) are
// loaded before its gathers, so a row costs one index load plus its gather
// rounds on the critical path.
//
// Precision.  Row sums are FP32 with Kahan compensation.  The L1 change per
// column is one FP32 partial per slot and warp (a warp finishes about
// n / 2,400 rows of a sweep; the rounding errors of its partial are
// unbiased, so the total's relative error is about 1e-7 / sqrt(warps)),
// folded over warps and CTAs in FP64; shared memory goes to the gather rings
// instead (see pb_rows).  The dangling mass per column is summed with Kahan
// compensation per warp from the new iterate's sink rows and folded in FP64.
// In narrow rows both are compensated per lane.  The per-row work stays off
// the FP64 pipe (on this GPU a few FP64 operations per row cost more than the
// row's gathers): degrees and their inverses are precomputed in FP32.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "gtc_view.cuh"

namespace gtc {
namespace {

constexpr int PPR_NT = 256;
constexpr int PPR_WARPS = PPR_NT / 32;
constexpr uint32_t PPR_CHUNK = 1024;  // rows with more in-edges are cut into chunks
constexpr uint32_t PPR_MAXB = 512;    // largest batch (16 lines per row)
constexpr uint32_t PPR_NONE = 0xFFFFFFFFu;
// At most this many columns left: narrow rows (k_ppr_narrow).
constexpr uint32_t PPR_NARROW = 16;
// At most this many columns left: each is finished by the single-vector
// solver from its current iterate (a narrow sweep of 8 columns costs about
// as much as three single-vector sweeps).
constexpr uint32_t PPR_HANDOFF = 2;
// Narrow rows: items of at least this many entries take a whole warp.
constexpr uint32_t PPR_HEAVY = 64;

struct PprArgs {
    uint32_t n, s_in, s_out;             // slots used per row of zin and zout
    uint32_t pitch;                      // floats per row of zin and zout
    uint32_t in_place;                   // out_slot[j] is j or PPR_NONE for every j
    const uint4* __restrict__ items;     // chunks, then single rows
    uint32_t n_items, n_chunks;
    const uint4* __restrict__ longs;     // {row, first chunk, chunks, 0}
    uint32_t n_long;
    const uint32_t* __restrict__ eseeds; // seed rows without in-edges
    uint32_t n_eseeds;
    uint32_t n_heavy;                    // items of at least PPR_HEAVY entries (the first)
    const uint32_t* __restrict__ other;
    const float* __restrict__ w;         // pull-ordered weights or null
    const float* __restrict__ zin;       // [n][pitch], slots [0, s_in) used
    float* __restrict__ zout;            // [n][pitch], slots [0, s_out) written
    const float2* __restrict__ dinv;     // {FP32 out-degree, its inverse}; {-1, 0} for a sink
    const uint32_t* __restrict__ seed_off;  // per vertex: seeds [seed_off[v], seed_off[v+1])
    const uint2* __restrict__ seeds;        // {column, float bits of the value}
    const uint32_t* __restrict__ col_in;    // [s_in] column in each input slot (PPR_NONE: empty)
    const uint32_t* __restrict__ out_slot;  // [s_in] its output slot (PPR_NONE: not computed)
    const float* __restrict__ psink;        // [s_in] dangling mass of zin per input slot
    float one_minus_d, d;
    float2* cpart;     // [n_chunks][s_in] compensated chunk partials (s, -c)
    double* part;      // [CTAs of both kernels][2][s_in]
    uint32_t part_base;
    int* err;          // set when a bounded wait gave up
};

// Two FP32 lanes per instruction (add/sub/mul.rn.f32x2, sm_100 and later):
// each half is the IEEE round-to-nearest operation of its own operands, so a
// pair operation gives bit for bit the two scalar results, in half the
// instructions.  The per-slot sums below are issue-bound, so they use pairs.
__device__ __forceinline__ void f2_add(float& dx, float& dy, float ax, float ay, float bx,
                                       float by) {
    asm("{\n\t.reg .b64 a, b, d;\n\tmov.b64 a, {%2, %3};\n\tmov.b64 b, {%4, %5};\n\t"
        "add.rn.f32x2 d, a, b;\n\tmov.b64 {%0, %1}, d;\n\t}"
        : "=f"(dx), "=f"(dy)
        : "f"(ax), "f"(ay), "f"(bx), "f"(by));
}
__device__ __forceinline__ void f2_sub(float& dx, float& dy, float ax, float ay, float bx,
                                       float by) {
    asm("{\n\t.reg .b64 a, b, d;\n\tmov.b64 a, {%2, %3};\n\tmov.b64 b, {%4, %5};\n\t"
        "sub.rn.f32x2 d, a, b;\n\tmov.b64 {%0, %1}, d;\n\t}"
        : "=f"(dx), "=f"(dy)
        : "f"(ax), "f"(ay), "f"(bx), "f"(by));
}
__device__ __forceinline__ void f2_mul(float& dx, float& dy, float ax, float ay, float bx,
                                       float by) {
    asm("{\n\t.reg .b64 a, b, d;\n\tmov.b64 a, {%2, %3};\n\tmov.b64 b, {%4, %5};\n\t"
        "mul.rn.f32x2 d, a, b;\n\tmov.b64 {%0, %1}, d;\n\t}"
        : "=f"(dx), "=f"(dy)
        : "f"(ax), "f"(ay), "f"(bx), "f"(by));
}

// Classic Kahan accumulation of C slots (value s - c).
template <int C>
struct Acc {
    float s[C], c[C];
    __device__ __forceinline__ void zero() {
#pragma unroll
        for (int k = 0; k < C; ++k) s[k] = 0.f, c[k] = 0.f;
    }
    __device__ __forceinline__ void add(int k, float x) {
        const float y = __fsub_rn(x, c[k]);
        const float t = __fadd_rn(s[k], y);
        c[k] = __fsub_rn(__fsub_rn(t, s[k]), y);
        s[k] = t;
    }
    // slots k and k + 1 at once, the same operations as two add() calls
    __device__ __forceinline__ void add2(int k, float x0, float x1) {
        float y0, y1, t0, t1, u0, u1;
        f2_sub(y0, y1, x0, x1, c[k], c[k + 1]);
        f2_add(t0, t1, s[k], s[k + 1], y0, y1);
        f2_sub(u0, u1, t0, t1, s[k], s[k + 1]);
        f2_sub(c[k], c[k + 1], u0, u1, y0, y1);
        s[k] = t0, s[k + 1] = t1;
    }
    // every slot: pairs, and the last one alone when C is odd
    __device__ __forceinline__ void add_all(const float (&x)[C]) {
#pragma unroll
        for (int q = 0; q + 1 < C; q += 2) add2(q, x[q], x[q + 1]);
        if (C % 2) add(C - 1, x[C - 1]);
    }
};

// t[q] += x[q] (W: x[q] * w) for every slot, in pairs.
template <int C, bool W>
__device__ __forceinline__ void slots_accumulate(float (&t)[C], const float (&x)[C], float w) {
#pragma unroll
    for (int q = 0; q + 1 < C; q += 2) {
        float a = x[q], b = x[q + 1];
        if (W) f2_mul(a, b, a, b, w, w);
        f2_add(t[q], t[q + 1], t[q], t[q + 1], a, b);
    }
    if (C % 2) t[C - 1] = __fadd_rn(t[C - 1], W ? __fmul_rn(x[C - 1], w) : x[C - 1]);
}

// The slots of a lane.  A row of S = 32 * C slots is read by the warp as C
// / V vector loads of V floats per lane (V = 4 when C is a multiple of 4, 2
// when C is 2, else 1); the lane's q-th value is slot slot(lane, q).
template <int C>
struct Lanes {
    static constexpr int V = C % 4 == 0 ? 4 : (C % 2 == 0 ? 2 : 1);
    __device__ __forceinline__ static uint32_t slot(int lane, int q) {
        return 32 * V * (q / V) + V * lane + (q % V);
    }
    // the lane's C values of a row (global memory through the read-only
    // path, or shared memory)
    template <bool GLOBAL>
    __device__ __forceinline__ static void load(const float* row, int lane, float (&x)[C]) {
#pragma unroll
        for (int t = 0; t < C / V; ++t) {
            const float* p = row + 32 * V * t + V * lane;
            if (V == 4) {
                const float4 f = GLOBAL ? __ldg(reinterpret_cast<const float4*>(p))
                                        : *reinterpret_cast<const float4*>(p);
                x[4 * t] = f.x, x[4 * t + 1] = f.y, x[4 * t + 2] = f.z, x[4 * t + 3] = f.w;
            } else if (V == 2) {
                const float2 f = GLOBAL ? __ldg(reinterpret_cast<const float2*>(p))
                                        : *reinterpret_cast<const float2*>(p);
                x[2 * t] = f.x, x[2 * t + 1] = f.y;
            } else {
                x[t] = GLOBAL ? __ldg(p) : *p;
            }
        }
    }
};

// Sum of zin rows over the pull entries [pb, pe) for a lane's C slots: the
// warp loads 32 entries at a time and keeps U gathered rows in flight.  The
// U rows of a round are summed plainly and the round's sum is added with
// compensation (blocked Kahan summation).
template <int C, int U, bool W>
__device__ __forceinline__ void gather(const PprArgs& A, uint32_t pb, uint32_t pe, int lane,
                                       Acc<C>& acc) {
    for (uint32_t p0 = pb; p0 < pe; p0 += 32) {
        const uint32_t cnt = min(32u, pe - p0);
        uint32_t my = 0;
        float mw = 1.f;
        if ((uint32_t)lane < cnt) {
            my = __ldg(A.other + p0 + lane);
            if (W) mw = __ldg(A.w + p0 + lane);
        }
        for (uint32_t k = 0; k < cnt; k += U) {
            float v[U][C];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const uint32_t src = __shfl_sync(0xffffffffu, my, (k + u) & 31);
                if (k + u < cnt) Lanes<C>::template load<true>(A.zin + (size_t)src * A.pitch, lane, v[u]);
            }
            float t[C];
#pragma unroll
            for (int q = 0; q < C; ++q) t[q] = 0.f;
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const float ww = W ? __shfl_sync(0xffffffffu, mw, (k + u) & 31) : 1.f;
                if (k + u < cnt) {
#pragma unroll
                    for (int q = 0; q < C; ++q)
                        t[q] = __fadd_rn(t[q], W ? __fmul_rn(v[u][q], ww) : v[u][q]);
                }
            }
#pragma unroll
            for (int q = 0; q < C; ++q) acc.add(q, t[q]);
        }
    }
}

// What the epilogue of row v reads besides the row sums, loaded before the
// gathers so that its latency overlaps them.
template <int C>
struct RowIn {
    float2 dd;
    uint32_t sb, se;
    float z[C];  // zin[v] of the lane's slots
    __device__ __forceinline__ void load(const PprArgs& A, uint32_t v, int lane) {
        dd = A.dinv[v];
        sb = A.seed_off[v];
        se = A.seed_off[v + 1];
        Lanes<C>::template load<true>(A.zin + (size_t)v * A.pitch, lane, z);
    }
};

// Row v's new values for a lane's C input slots, stored to zout.  The L1
// change goes to the warp's accumulator in shared memory (the lane's q-th
// slot at 32 q + lane: conflict-free), one FP32 partial per slot and warp,
// folded over warps and CTAs in FP64; the dangling mass is summed from zout
// afterwards (k_ppr_sinks).  Nothing here runs on the FP64 pipe.
template <int C>
__device__ __forceinline__ void finish_row(const PprArgs& A, uint32_t v, const RowIn<C>& r,
                                           const float (&sum)[C], int lane, float* dz,
                                           uint32_t amask) {
    const bool snk = r.dd.x < 0.f;
    const bool seeded = r.se > r.sb;
    uint32_t osv[C];
    float outv[C];
#pragma unroll
    for (int q = 0; q < C; ++q) {
        const uint32_t j = Lanes<C>::slot(lane, q);
        outv[q] = 0.f;
        if (!((amask >> q) & 1u)) {
            osv[q] = PPR_NONE;
            continue;
        }
        // in place the output slot is the input slot
        osv[q] = A.in_place ? j : __ldg(A.out_slot + j);
        const float prev = snk ? r.z[q] : __fmul_rn(r.z[q], r.dd.x);
        float nv;
        if (!seeded) {
            // no seed in any column: pv = 0, where the general form below
            // gives x = 0 + sum = sum and nv = 0 + d x, bit for bit
            nv = __fmul_rn(A.d, sum[q]);
        } else {
            const uint32_t col = __ldg(A.col_in + j);
            float pv = 0.f;
            for (uint32_t t = r.sb; t < r.se; ++t) {
                const uint2 sd = A.seeds[t];
                if (sd.x == col) pv = __uint_as_float(sd.y);
            }
            const float x = __fadd_rn(__fmul_rn(__ldg(A.psink + j), pv), sum[q]);
            nv = __fadd_rn(__fmul_rn(A.one_minus_d, pv), __fmul_rn(A.d, x));
        }
        float* a = dz + 32 * q + lane;
        *a = __fadd_rn(*a, fabsf(__fsub_rn(nv, prev)));
        outv[q] = snk ? nv : __fmul_rn(nv, r.dd.y);
    }
    // In place (every sweep but those that repack the columns), each lane's
    // V values go to its own input slots with vector stores, coalesced over
    // the warp (a converged column's slot gets 0: no sweep reads it again);
    // otherwise one store per computed slot.
    float* zn = A.zout + (size_t)v * A.pitch;
    constexpr int V = Lanes<C>::V;
    if (A.in_place) {
#pragma unroll
        for (int t = 0; t < C / V; ++t) {
            float* p = zn + Lanes<C>::slot(lane, V * t);
            if (V == 4)
                *reinterpret_cast<float4*>(p) =
                    make_float4(outv[4 * t], outv[4 * t + 1], outv[4 * t + 2], outv[4 * t + 3]);
            else if (V == 2)
                *reinterpret_cast<float2*>(p) = make_float2(outv[2 * t], outv[2 * t + 1]);
            else
                *p = outv[t];
        }
    } else {
#pragma unroll
        for (int q = 0; q < C; ++q)
            if (osv[q] != PPR_NONE) zn[osv[q]] = outv[q];
    }
}

// Bit q: the lane's q-th input slot is computed this sweep (out_slot is not
// PPR_NONE), read once per kernel.
template <int C>
__device__ __forceinline__ uint32_t active_mask(const PprArgs& A, int lane) {
    uint32_t m = 0;
#pragma unroll
    for (int q = 0; q < C; ++q)
        if (__ldg(A.out_slot + Lanes<C>::slot(lane, q)) != PPR_NONE) m |= 1u << q;
    return m;
}

// Shared memory of the register-gather and long-row kernels: per warp [s_in]
// partial L1 changes.
inline size_t ppr_smem(uint32_t s_in) { return (size_t)PPR_WARPS * s_in * sizeof(float); }

// The warp's accumulator (zeroed).
__device__ __forceinline__ float* warp_dz(float* sm, uint32_t s_in, int warp, int lane) {
    float* dz = sm + (size_t)warp * s_in;
    for (uint32_t j = lane; j < s_in; j += 32) dz[j] = 0.f;
    __syncwarp();
    return dz;
}

// The CTA's per-slot L1 change (warps in order, FP64) into its partial record
// {change per input slot, dangling mass per output slot (none here)}.
template <int C>
__device__ __forceinline__ void cta_fold(const PprArgs& A, const float* dz_all, int warps,
                                         uint32_t warp_stride) {
    __syncthreads();
    double* dst = A.part + (size_t)(A.part_base + blockIdx.x) * 2 * A.s_in;
    for (uint32_t pos = threadIdx.x; pos < A.s_in; pos += blockDim.x) {
        double a = 0.0;
        for (int w = 0; w < warps; ++w) a += (double)dz_all[(size_t)w * warp_stride + pos];
        dst[Lanes<C>::slot(pos & 31, pos >> 5)] = a;
        dst[A.s_in + pos] = 0.0;
    }
}

// Sweep, part 1: every long-row chunk (partials to cpart) and every single
// row (finished here).  Warp gw takes items gw, gw + warps, ... and loads
// each next item while it works on the current one.
template <int C, int U, bool W>
__global__ void __launch_bounds__(PPR_NT) k_ppr_rows(PprArgs A) {
    extern __shared__ float ppr_sm[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    float* dz = warp_dz(ppr_sm, A.s_in, warp, lane);
    const uint32_t amask = active_mask<C>(A, lane);
    const uint32_t gw = blockIdx.x * PPR_WARPS + warp, nw = gridDim.x * PPR_WARPS;
    uint4 nxt = gw < A.n_items ? A.items[gw] : make_uint4(0u, 0u, 0u, 0u);
    for (uint32_t it = gw; it < A.n_items; it += nw) {
        const uint4 cur = nxt;
        if (it + nw < A.n_items) nxt = A.items[it + nw];
        Acc<C> acc;
        acc.zero();
        if (it < A.n_chunks) {
            gather<C, U, W>(A, cur.y, cur.z, lane, acc);
            float2* dst = A.cpart + (size_t)it * A.s_in;
#pragma unroll
            for (int q = 0; q < C; ++q)
                __stcg(dst + Lanes<C>::slot(lane, q), make_float2(acc.s[q], -acc.c[q]));
        } else {
            RowIn<C> r;
            r.load(A, cur.x, lane);
            gather<C, U, W>(A, cur.y, cur.z, lane, acc);
            float sum[C];
#pragma unroll
            for (int q = 0; q < C; ++q) sum[q] = __fsub_rn(acc.s[q], acc.c[q]);
            finish_row<C>(A, cur.x, r, sum, lane, dz, amask);
        }
    }
    cta_fold<C>(A, ppr_sm, PPR_WARPS, A.s_in);
}


// --------------------------------------------------------------------------
// Sweep, part 1, bulk-copy variant.  The gather of a row of zin (S floats,
// 128-byte aligned) is one cp.async.bulk into shared memory, completed on an
// mbarrier, so the rows in flight sit in shared memory instead of registers.
// Each warp streams its items as batches of up to BT rows through a
// two-batch ring: while batch k is summed, the copies of batch k+1 are in
// flight and the source indices of batch k+2 are being loaded.
// --------------------------------------------------------------------------

constexpr int PB_WARPS = 4;
constexpr int PB_NT = 32 * PB_WARPS;
constexpr long long PB_WAIT_CYCLES = 4000000000ll;  // ~2 s: a copy that never lands
constexpr uint32_t PB_BLOCK = 8;                    // rows per plain partial sum

// rows per batch: about 4 KB of rows, 2..32
// rows per batch: 6 KB of rows, 2..32.  The sweep is bound by the bytes of
// rows in flight: four CTAs of four warps fit an SM (registers), and with
// the per-warp accumulators at one float per slot each warp's ring holds
// two batches of 6 KB in the same 54 KB a CTA had for 4 KB batches.  Per
// 256-column sweep of an R-MAT-22 graph: 8.90 ms (4 KB), 8.21 (5 KB), 7.80
// (6 KB); eight warps with 8 KB batches were slower than sixteen with 4 KB.
constexpr int pb_rows(int C) { return 48 / C < 2 ? 2 : (48 / C > 32 ? 32 : 48 / C); }

template <int C>
struct PbLayout {
    static constexpr int S = 32 * C;
    static constexpr int BT = pb_rows(C);
    static constexpr int RING = 2 * BT * S * 4;               // bytes
    static constexpr int DZ = RING + 16;                      // after the two mbarriers
    static constexpr int WARP = (DZ + S * 4 + 127) / 128 * 128;  // per-warp bytes
    static constexpr int CTA = PB_WARPS * WARP;
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint32_t bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void mbar_expect(uint32_t bar, uint32_t bytes) {
    asm volatile(
        "{\n\t.reg .b64 st;\n\t"
        "mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(bar),
        "r"(bytes)
        : "memory");
}

// Bounded wait for the phase of the given parity; false if it gave up.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
    const long long t0 = clock64();
    for (;;) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(bar), "r"(parity)
            : "memory");
        if (done) return true;
        if (clock64() - t0 > PB_WAIT_CYCLES) return false;
    }
}

__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes,
                                         uint32_t bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
        "l"(src), "r"(bytes), "r"(bar)
        : "memory");
}

struct PbBatch {
    uint32_t it, v, p, cnt;
    bool first, last, valid;
};

template <int C, bool W>
__global__ void __launch_bounds__(PB_NT) k_ppr_bulk(PprArgs A) {
    using Lay = PbLayout<C>;
    constexpr int S = Lay::S, BT = Lay::BT;
    extern __shared__ __align__(128) unsigned char pb_sm[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned char* wsm = pb_sm + warp * Lay::WARP;
    float* ring = reinterpret_cast<float*>(wsm);
    const uint32_t bar0 = smem_u32(wsm + Lay::RING);
    float* dz = reinterpret_cast<float*>(wsm + Lay::DZ);
    for (int j = lane; j < S; j += 32) dz[j] = 0.f;
    const uint32_t amask = active_mask<C>(A, lane);
    if (lane == 0) {
        mbar_init(bar0);
        mbar_init(bar0 + 8);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncwarp();

    const uint32_t gw = blockIdx.x * PB_WARPS + warp, nw = gridDim.x * PB_WARPS;
    // the batch generator (warp-uniform state)
    uint32_t g_it = gw;
    uint4 g_rec = g_it < A.n_items ? A.items[g_it] : make_uint4(0u, 0u, 0u, 0u);
    uint4 g_nxt = g_it + nw < A.n_items ? A.items[g_it + nw] : make_uint4(0u, 0u, 0u, 0u);
    uint32_t g_p = g_rec.y;
    auto next_batch = [&]() {
        PbBatch b{};
        if (g_it >= A.n_items) return b;
        b.valid = true;
        b.it = g_it;
        b.v = g_rec.x;
        b.p = g_p;
        b.cnt = min((uint32_t)BT, g_rec.z - g_p);
        b.first = g_p == g_rec.y;
        b.last = g_p + b.cnt == g_rec.z;
        g_p += b.cnt;
        if (b.last) {
            g_it += nw;
            g_rec = g_nxt;
            g_p = g_rec.y;
            if (g_it + nw < A.n_items) g_nxt = A.items[g_it + nw];
        }
        return b;
    };

    PbBatch bA = next_batch(), bB{}, bC{};
    uint32_t iA = 0;
    float wA = 1.f;
    if (bA.valid && (uint32_t)lane < bA.cnt) {
        iA = __ldg(A.other + bA.p + lane);
        if (W) wA = __ldg(A.w + bA.p + lane);
    }
    float wB = 1.f, wC = 1.f;
    RowIn<C> rB, rC;
    uint32_t hB = 0, parity = 0;  // half of the batch being issued; phase bit per half
    Acc<C> acc;
    acc.zero();
    bool ok = true;
    for (;;) {
        // stage 2: the copies of batch A into half hB
        bB = bA;
        wB = wA;
        if (bB.valid && bB.cnt > 0) {
            const uint32_t bar = bar0 + 8 * hB;
            if (lane == 0) mbar_expect(bar, bB.cnt * (uint32_t)(S * 4));
            __syncwarp();
            if ((uint32_t)lane < bB.cnt)
                bulk_g2s(smem_u32(ring + (size_t)(hB * BT + lane) * S), A.zin + (size_t)iA * A.pitch,
                         S * 4, bar);
        }
        if (bB.valid && bB.first && bB.it >= A.n_chunks) rB.load(A, bB.v, lane);
        // stage 1: the source indices of the batch after it
        bA = next_batch();
        if (bA.valid && (uint32_t)lane < bA.cnt) {
            iA = __ldg(A.other + bA.p + lane);
            if (W) wA = __ldg(A.w + bA.p + lane);
        }
        // stage 3: sum batch C (half hB ^ 1)
        if (bC.valid) {
            const uint32_t h = hB ^ 1u;
            if (bC.cnt > 0) {
                if (!mbar_wait(bar0 + 8 * h, (parity >> h) & 1u)) {
                    ok = false;
                    break;
                }
                parity ^= 1u << h;
            }
            if (bC.first) acc.zero();
            const float* rb = ring + (size_t)h * BT * S;
            for (uint32_t i0 = 0; i0 < bC.cnt; i0 += PB_BLOCK) {
                // blocked Kahan: up to PB_BLOCK rows summed plainly, then added
                float t[C];
#pragma unroll
                for (int q = 0; q < C; ++q) t[q] = 0.f;
                const uint32_t i1 = min(bC.cnt, i0 + PB_BLOCK);
                for (uint32_t i = i0; i < i1; ++i) {
                    const float ww = W ? __shfl_sync(0xffffffffu, wC, i) : 1.f;
                    float x[C];
                    Lanes<C>::template load<false>(rb + (size_t)i * S, lane, x);
                    slots_accumulate<C, W>(t, x, ww);
                }
                acc.add_all(t);
            }
            if (bC.last) {
                if (bC.it < A.n_chunks) {
                    float2* dst = A.cpart + (size_t)bC.it * A.s_in;
#pragma unroll
                    for (int q = 0; q < C; ++q)
                        __stcg(dst + Lanes<C>::slot(lane, q), make_float2(acc.s[q], -acc.c[q]));
                } else {
                    float sum[C];
#pragma unroll
                    for (int q = 0; q < C; ++q) sum[q] = __fsub_rn(acc.s[q], acc.c[q]);
                    finish_row<C>(A, bC.v, rC, sum, lane, dz, amask);
                }
            }
            // the half is refilled by the async proxy next: order our reads first
            __syncwarp();
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        }
        // rotate
        if (!bB.valid) break;
        bC = bB;
        wC = wB;
        if (bB.first) rC = rB;
        hB ^= 1u;
    }
    if (!ok) {
        // Report, then give every copy still in flight a bounded chance to
        // land before the block exits (its shared memory may go to another
        // block next): the copies into the half whose wait gave up (batch C,
        // half hB ^ 1) and the ones just issued into half hB (batch B).  The
        // host reads the flag and fails the call (GTC_ERR_CUDA) instead of
        // using this sweep.
        if (lane == 0) atomicExch(A.err, 1);
        const uint32_t hf = hB ^ 1u;
        if (bC.valid && bC.cnt > 0) (void)mbar_wait(bar0 + 8 * hf, (parity >> hf) & 1u);
        if (bB.valid && bB.cnt > 0) (void)mbar_wait(bar0 + 8 * hB, (parity >> hB) & 1u);
    }
    cta_fold<C>(A, reinterpret_cast<const float*>(pb_sm + Lay::DZ), PB_WARPS, Lay::WARP / 4);
}

// Sweep, part 2: every long row, its chunks' partials merged in chunk order,
// then every seed row without in-edges.
template <int C>
__global__ void __launch_bounds__(PPR_NT) k_ppr_long(PprArgs A) {
    extern __shared__ float ppr_sm[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    float* dz = warp_dz(ppr_sm, A.s_in, warp, lane);
    const uint32_t amask = active_mask<C>(A, lane);
    const uint32_t gw = blockIdx.x * PPR_WARPS + warp, nw = gridDim.x * PPR_WARPS;
    for (uint32_t k = gw; k < A.n_long; k += nw) {
        const uint4 lr = A.longs[k];
        RowIn<C> r;
        r.load(A, lr.x, lane);
        Kahan t[C];
        for (uint32_t c = lr.y; c < lr.y + lr.z; ++c) {
            const float2* src = A.cpart + (size_t)c * A.s_in;
#pragma unroll
            for (int q = 0; q < C; ++q) {
                const float2 pq = __ldcg(src + Lanes<C>::slot(lane, q));
                t[q].merge(pq.x, pq.y);
            }
        }
        float sum[C];
#pragma unroll
        for (int q = 0; q < C; ++q) sum[q] = t[q].value();
        finish_row<C>(A, lr.x, r, sum, lane, dz, amask);
    }
    // seed rows without in-edges: an empty sum
    for (uint32_t k = gw; k < A.n_eseeds; k += nw) {
        const uint32_t v = A.eseeds[k];
        RowIn<C> r;
        r.load(A, v, lane);
        float sum[C];
#pragma unroll
        for (int q = 0; q < C; ++q) sum[q] = 0.f;
        finish_row<C>(A, v, r, sum, lane, dz, amask);
    }
    cta_fold<C>(A, ppr_sm, PPR_WARPS, A.s_in);
}

// ---------------------------------------------------------------------------
// Narrow rows: Z is [n][K] (K = 8 or 16), slot k of every row is column
// col_in[k] (PPR_NONE: no longer computed, stored as 0).  A group of K lanes
// takes work items gg, gg + groups, ...; lane k of the group sums slot k.

// What a row's update reads besides its sum, for lane k (loaded before the
// gathers).
struct NarrowIn {
    float2 dd;
    uint32_t sb, se;
    float z;
    __device__ __forceinline__ void load(const PprArgs& A, uint32_t v, uint32_t K, uint32_t k) {
        dd = A.dinv[v];
        sb = A.seed_off[v];
        se = A.seed_off[v + 1];
        z = A.zin[(size_t)v * K + k];
    }
};

// The sources (and weights) of the pull entries [p0, min(p0 + K, e)) that
// lane k of a group holds: entry p0 + k.
template <bool W>
struct NarrowIdx {
    uint32_t src = 0;
    float w = 1.f;
    __device__ __forceinline__ void load(const PprArgs& A, uint32_t p0, uint32_t e, uint32_t k) {
        if (p0 + k < e) {
            src = __ldg(A.other + p0 + k);
            if (W) w = __ldg(A.w + p0 + k);
        }
    }
};

// Compensated sum (Kahan, value s + c) of slot k of the zin rows over the
// blocks of K pull entries starting at p0, p0 + step, ... below e: lane k
// holds a block's K sources (the next block's are loaded before this one's
// gathers) and the group shares them by shuffles; a block's gathers are all
// in flight before they are added.
template <int K, bool W>
__device__ __forceinline__ Kahan narrow_sum(const PprArgs& A, uint32_t p0, uint32_t step,
                                           uint32_t e, uint32_t k, uint32_t gmask) {
    Kahan acc;
    NarrowIdx<W> ix;
    if (p0 < e) ix.load(A, p0, e, k);
    for (; p0 < e; p0 += step) {
        const uint32_t cnt = min((uint32_t)K, e - p0);
        NarrowIdx<W> nx;
        if (p0 + step < e) nx.load(A, p0 + step, e, k);
        float v[K];
#pragma unroll
        for (int u = 0; u < K; ++u) {
            const uint32_t src = __shfl_sync(gmask, ix.src, u, K);
            v[u] = (uint32_t)u < cnt ? __ldg(A.zin + (size_t)src * K + k) : 0.f;
        }
#pragma unroll
        for (int u = 0; u < K; ++u) {
            const float ww = W ? __shfl_sync(gmask, ix.w, u, K) : 1.f;
            if ((uint32_t)u < cnt) acc.add(W ? __fmul_rn(v[u], ww) : v[u]);
        }
        ix = nx;
    }
    return acc;
}

// Row v's new value in slot k (the same arithmetic as finish_row), its
// change and dangling mass into the lane's compensated partials.
template <int K>
__device__ __forceinline__ void narrow_finish(const PprArgs& A, uint32_t v, const NarrowIn& r,
                                              float sum, uint32_t k, uint32_t os, uint32_t col,
                                              float ps, Kahan& kd, Kahan& kk) {
    float* zn = A.zout + (size_t)v * K + k;
    if (os == PPR_NONE) {
        *zn = 0.f;
        return;
    }
    const bool snk = r.dd.x < 0.f;
    const float prev = snk ? r.z : __fmul_rn(r.z, r.dd.x);
    float nv;
    if (r.se == r.sb) {
        nv = __fmul_rn(A.d, sum);  // no seed: the general form with pv = 0, bit for bit
    } else {
        float pv = 0.f;
        for (uint32_t t = r.sb; t < r.se; ++t) {
            const uint2 sd = A.seeds[t];
            if (sd.x == col) pv = __uint_as_float(sd.y);
        }
        const float x = __fadd_rn(__fmul_rn(ps, pv), sum);
        nv = __fadd_rn(__fmul_rn(A.one_minus_d, pv), __fmul_rn(A.d, x));
    }
    kd.add(fabsf(__fsub_rn(nv, prev)));
    if (snk) kk.add(nv);
    *zn = snk ? nv : __fmul_rn(nv, r.dd.y);
}

// The CTA's per-slot change and dangling mass (lanes in thread order, FP64)
// into its partial record.
template <int K>
__device__ __forceinline__ void narrow_fold(const PprArgs& A, Kahan kd, Kahan kk, float4* red) {
    red[threadIdx.x] = make_float4(kd.s, kd.c, kk.s, kk.c);
    __syncthreads();
    double* dst = A.part + (size_t)(A.part_base + blockIdx.x) * 2 * K;
    if (threadIdx.x < K) {
        double a = 0.0, b = 0.0;
        for (uint32_t t = threadIdx.x; t < blockDim.x; t += K) {
            const float4 x = red[t];
            a += (double)x.x + (double)x.y;
            b += (double)x.z + (double)x.w;
        }
        dst[threadIdx.x] = a;
        dst[K + threadIdx.x] = b;
    }
}

// Narrow sweep, part 1: every long-row chunk (partials to cpart) and every
// single row.  The first n_heavy items (chunks and rows of at least
// PPR_HEAVY entries) take a warp each, its groups summing alternate blocks
// of K entries and merged in group order; the others take a group each.
template <int K, bool W>
__global__ void __launch_bounds__(PPR_NT) k_ppr_narrow(PprArgs A) {
    __shared__ float4 red[PPR_NT];
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t k = lane % K, gl = lane / K;
    const uint32_t gmask = K == 32 ? 0xffffffffu : ((1u << K) - 1u) << (gl * K);
    constexpr uint32_t GPW = 32 / K;
    const uint32_t gw = blockIdx.x * PPR_WARPS + warp, nw = gridDim.x * PPR_WARPS;
    const uint32_t os = A.out_slot[k], col = A.col_in[k];
    const float ps = A.psink[k];
    Kahan kd, kk;
    for (uint32_t it = gw; it < A.n_heavy; it += nw) {
        const uint4 cur = A.items[it];
        NarrowIn r{};
        if (it >= A.n_chunks) r.load(A, cur.x, K, k);
        Kahan acc = narrow_sum<K, W>(A, cur.y + gl * K, GPW * K, cur.z, k, gmask);
#pragma unroll
        for (uint32_t g2 = 1; g2 < GPW; ++g2) {
            const float os2 = __shfl_sync(0xffffffffu, acc.s, (int)(g2 * K + k));
            const float oc2 = __shfl_sync(0xffffffffu, acc.c, (int)(g2 * K + k));
            if (gl == 0) acc.merge(os2, oc2);
        }
        if (gl == 0) {
            if (it < A.n_chunks)
                A.cpart[(size_t)it * A.s_in + k] = make_float2(acc.s, acc.c);
            else
                narrow_finish<K>(A, cur.x, r, acc.value(), k, os, col, ps, kd, kk);
        }
    }
    const uint32_t gg = gw * GPW + gl, ng = nw * GPW;
    for (uint32_t it = A.n_heavy + gg; it < A.n_items; it += ng) {
        const uint4 cur = A.items[it];
        NarrowIn r;
        r.load(A, cur.x, K, k);
        const Kahan acc = narrow_sum<K, W>(A, cur.y, K, cur.z, k, gmask);
        narrow_finish<K>(A, cur.x, r, acc.value(), k, os, col, ps, kd, kk);
    }
    narrow_fold<K>(A, kd, kk, red);
}

// Narrow sweep, part 2: every long row (its chunks' partials merged in chunk
// order), then every seed row without in-edges.
template <int K>
__global__ void __launch_bounds__(PPR_NT) k_ppr_narrow_long(PprArgs A) {
    __shared__ float4 red[PPR_NT];
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t k = lane % K, gl = lane / K;
    constexpr uint32_t GPW = 32 / K;
    const uint32_t gg = (blockIdx.x * PPR_WARPS + warp) * GPW + gl;
    const uint32_t ng = gridDim.x * PPR_WARPS * GPW;
    const uint32_t os = A.out_slot[k], col = A.col_in[k];
    const float ps = A.psink[k];
    Kahan kd, kk;
    for (uint32_t i = gg; i < A.n_long; i += ng) {
        const uint4 lr = A.longs[i];
        NarrowIn r;
        r.load(A, lr.x, K, k);
        Kahan t;
        for (uint32_t c = lr.y; c < lr.y + lr.z; ++c) {
            const float2 pq = __ldcg(A.cpart + (size_t)c * A.s_in + k);
            t.merge(pq.x, pq.y);
        }
        narrow_finish<K>(A, lr.x, r, t.value(), k, os, col, ps, kd, kk);
    }
    for (uint32_t i = gg; i < A.n_eseeds; i += ng) {
        const uint32_t v = A.eseeds[i];
        NarrowIn r;
        r.load(A, v, K, k);
        narrow_finish<K>(A, v, r, 0.f, k, os, col, ps, kd, kk);
    }
    narrow_fold<K>(A, kd, kk, red);
}

// zdst[v][k] = zsrc[v][slot[k]] (0 where slot[k] is PPR_NONE): the running
// columns into narrow rows.
__global__ void k_ppr_narrow_pack(uint32_t n, uint32_t K, uint32_t src_pitch,
                                  const uint32_t* __restrict__ slot, const float* __restrict__ zsrc,
                                  float* __restrict__ zdst) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (size_t)n * K) return;
    const uint32_t v = (uint32_t)(i / K), k = (uint32_t)(i % K);
    const uint32_t j = slot[k];
    zdst[i] = j == PPR_NONE ? 0.f : zsrc[(size_t)v * src_pitch + j];
}

// Sweep, part 3: the dangling mass of each output slot, the sum of zout over
// the sink rows (zout of a sink holds its rank itself).  A sink without
// in-edges and without a seed was skipped by the sweep and its row is zero,
// so only sinks with an in-edge or a seed are read.  Warp gw takes the
// 32-vertex groups gw, gw + warps, ... in vertex order, with compensation;
// the CTA folds its warps in order (FP64) into the dangling-mass half of its
// partial record.  C is the output width.
template <int C>
__global__ void __launch_bounds__(PPR_NT) k_ppr_sinks(PprArgs A, const uint32_t* __restrict__ pull_off) {
    extern __shared__ float2 ps_sm[];
    constexpr uint32_t S = 32 * C;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t gw = blockIdx.x * PPR_WARPS + warp, nw = gridDim.x * PPR_WARPS;
    Kahan t[C];
    for (uint32_t g = gw; (size_t)g * 32 < A.n; g += nw) {
        const uint32_t v = g * 32 + lane;
        bool take = false;
        if (v < A.n)
            take = A.dinv[v].x < 0.f &&
                   (pull_off[v + 1] > pull_off[v] || A.seed_off[v + 1] > A.seed_off[v]);
        uint32_t bits = __ballot_sync(0xffffffffu, take);
        while (bits) {
            const uint32_t b = (uint32_t)__ffs(bits) - 1;
            bits &= bits - 1;
            float x[C];
            Lanes<C>::template load<true>(A.zout + (size_t)(g * 32 + b) * A.pitch, lane, x);
#pragma unroll
            for (int q = 0; q < C; ++q) t[q].add(x[q]);
        }
    }
    float2* mine = ps_sm + (size_t)warp * S;
#pragma unroll
    for (int q = 0; q < C; ++q) mine[Lanes<C>::slot(lane, q)] = make_float2(t[q].s, t[q].c);
    __syncthreads();
    double* dst = A.part + (size_t)(A.part_base + blockIdx.x) * 2 * A.s_in;
    for (uint32_t pos = threadIdx.x; pos < A.s_in; pos += PPR_NT) {
        double b = 0.0;
        if (pos < S)
            for (int w = 0; w < PPR_WARPS; ++w) {
                const float2 x = ps_sm[(size_t)w * S + pos];
                b += (double)x.x + (double)x.y;
            }
        dst[pos] = 0.0;
        dst[A.s_in + pos] = b;
    }
}

// Sweep, part 4: out[j] = sum over the CTA partials of the three kernels, in
// a fixed order (a thread per value).
__global__ void k_ppr_fold(uint32_t n_values, uint32_t n_parts, const double* __restrict__ part,
                           double* __restrict__ out) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n_values) return;
    double t8[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    uint32_t k = 0;
    for (; k + 8 <= n_parts; k += 8) {
#pragma unroll
        for (int i = 0; i < 8; ++i) t8[i] += part[(size_t)(k + i) * n_values + j];
    }
    for (; k < n_parts; ++k) t8[0] += part[(size_t)k * n_values + j];
    double t = 0.0;
#pragma unroll
    for (int i = 0; i < 8; ++i) t += t8[i];
    out[j] = t;
}

// The start: rank_b = pers_b, stored as Z (slot = column) over a zeroed Z;
// each (vertex, column) seed appears once.
__global__ void k_ppr_init(uint32_t ns, uint32_t S, const uint32_t* __restrict__ sv,
                           const uint2* __restrict__ sd, const float2* __restrict__ dinv,
                           float* __restrict__ z) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= ns) return;
    const uint32_t v = sv[k];
    const float pv = __uint_as_float(sd[k].y);
    const float2 dd = dinv[v];
    z[(size_t)v * S + sd[k].x] = dd.x < 0.f ? pv : __fmul_rn(pv, dd.y);
}

// {FP32 degree, its inverse} per vertex; {-1, 0} marks a sink.
__global__ void k_ppr_dinv(uint32_t n, const double* __restrict__ deg, float2* __restrict__ dinv) {
    const size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n) return;
    const double dg = deg[v];
    dinv[v] = dg == 0.0 ? make_float2(-1.f, 0.f) : make_float2((float)dg, (float)(1.0 / dg));
}

// seed_off[v] = first seed record of vertex v (records sorted by vertex).
__global__ void k_ppr_seed_off(uint32_t n, uint32_t ns, const uint32_t* __restrict__ sv,
                               uint32_t* __restrict__ seed_off) {
    const size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v > n) return;
    uint32_t lo = 0, hi = ns;
    while (lo < hi) {
        const uint32_t mid = lo + (hi - lo) / 2;
        if (sv[mid] < v)
            lo = mid + 1;
        else
            hi = mid;
    }
    seed_off[v] = lo;
}

// Internal label and degree of each seed vertex.
// Internal label, degree and number of pull entries (in-edges) of each seed
// vertex.
__global__ void k_ppr_seed_lookup(uint32_t ns, const uint32_t* __restrict__ orig,
                                  const uint32_t* __restrict__ iperm, const double* __restrict__ deg,
                                  const uint32_t* __restrict__ pull_off, uint32_t* __restrict__ iv,
                                  double* __restrict__ dv, uint32_t* __restrict__ din) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= ns) return;
    const uint32_t v = iperm[orig[k]];
    iv[k] = v;
    dv[k] = deg[v];
    din[k] = pull_off[v + 1] - pull_off[v];
}

// out[col][o] = rank of column col at original vertex o (internal label
// iperm[o]), for K (slot, column) pairs in slot order, transposed through
// shared memory: a warp reads the 32 pairs' slots of one row (consecutive
// slots share sectors) and writes 32 consecutive vertices of one column.
__global__ void k_ppr_store(uint32_t n, uint32_t S, uint32_t K, const uint2* __restrict__ pairs,
                            const uint32_t* __restrict__ iperm, const float2* __restrict__ dinv,
                            const float* __restrict__ z, void* __restrict__ out, int dt) {
    __shared__ float tile[32][33];
    const uint32_t o0 = blockIdx.x * 32, k0 = blockIdx.y * 32;
    const uint32_t tx = threadIdx.x, ty = threadIdx.y;  // 32 x 8
    for (uint32_t r = ty; r < 32; r += 8) {
        const uint32_t o = o0 + r, k = k0 + tx;
        float val = 0.f;
        if (o < n && k < K) {
            const uint32_t i = iperm[o];
            const float zz = z[(size_t)i * S + pairs[k].x];
            const float2 dd = dinv[i];
            val = dd.x < 0.f ? zz : __fmul_rn(zz, dd.x);
        }
        tile[r][tx] = val;
    }
    __syncthreads();
    for (uint32_t r = ty; r < 32; r += 8) {
        const uint32_t k = k0 + r, o = o0 + tx;
        if (k < K && o < n) {
            const size_t at = (size_t)pairs[k].y * n + o;
            if (dt == GTC_F64)
                ((double*)out)[at] = (double)tile[tx][r];
            else
                ((float*)out)[at] = tile[tx][r];
        }
    }
}

// pers[v] = value, for the seeds of one column in order (the last value
// given for a vertex wins)
__global__ void k_ppr_pers(uint32_t k, const uint32_t* __restrict__ verts,
                           const float* __restrict__ vals, float* __restrict__ pers) {
    if (blockIdx.x == 0 && threadIdx.x == 0)
        for (uint32_t i = 0; i < k; ++i) pers[verts[i]] = vals[i];
}

__global__ void k_degree_ppr(uint32_t n, const uint32_t* __restrict__ push_off,
                             const uint32_t* __restrict__ push_eid, const void* __restrict__ w,
                             int wdt, double* __restrict__ deg) {
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
    deg[v] = k;
}

__global__ void k_gather_w_ppr(uint32_t m, const uint32_t* __restrict__ eid,
                               const void* __restrict__ w, int wdt, float* __restrict__ out) {
    size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p < m) out[p] = (float)ld_any(w, wdt, eid[p]);
}

// schedule keys: 0 for a row cut into chunks, else PPR_CHUNK + 1 - in-degree
// (cnt[0]: rows cut into chunks, cnt[1]: rows without pull entries, cnt[2]:
// single rows of at least PPR_HEAVY entries)
__global__ void k_ppr_keys(uint32_t n, const uint32_t* __restrict__ off, uint32_t* __restrict__ key,
                           unsigned* __restrict__ cnt) {
    const size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n) return;
    const uint32_t dg = off[v + 1] - off[v];
    key[v] = dg > PPR_CHUNK ? 0u : PPR_CHUNK + 1 - dg;
    if (dg > PPR_CHUNK) atomicAdd(cnt, 1u);
    if (dg == 0) atomicAdd(cnt + 1, 1u);
    if (dg >= PPR_HEAVY && dg <= PPR_CHUNK) atomicAdd(cnt + 2, 1u);
}

__global__ void k_ppr_row_items(uint32_t k, const uint32_t* __restrict__ pos,
                                const uint32_t* __restrict__ off, uint32_t flag,
                                uint4* __restrict__ rec) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= k) return;
    const uint32_t v = pos[i];
    rec[i] = make_uint4(v, off[v], off[v + 1], flag);
}

// The schedule of one unfiltered view, built on the graph's home stream and
// kept with the graph.
void build_ppr_schedule(gtc_graph* g, const View& view, cudaStream_t s, PprSched& S) {
    const uint32_t n = view.n;
    cudaStream_t h = g->home;
    GTC_CUDA(cudaStreamSynchronize(s));
    uint64_t L = 0;
    DevBuf<uint32_t> key(n, h), skey(n, h), pos(n, h);
    DevBuf<unsigned> cnt(3, h);
    GTC_CUDA(cudaMemsetAsync(cnt.get(), 0, 3 * sizeof(unsigned), h));
    if (n) {
        k_ppr_keys<<<grid_for(n, 256, 1u << 30), 256, 0, h>>>(n, view.pull_off, key.get(), cnt.get());
        GTC_LAUNCHED();
        L++;
        sort_positions_by_key(key.get(), n, PPR_CHUNK + 2, skey.get(), pos.get(), h, &L);
    }
    unsigned cnts[3] = {0, 0, 0};
    GTC_CUDA(cudaMemcpyAsync(cnts, cnt.get(), 3 * sizeof(unsigned), cudaMemcpyDeviceToHost, h));
    GTC_CUDA(cudaStreamSynchronize(h));
    const unsigned n_long = cnts[0];
    std::vector<uint4> lrec(n_long);
    if (n_long) {
        DevBuf<uint4> drec(n_long, h);
        k_ppr_row_items<<<grid_for(n_long, 256, 1u << 30), 256, 0, h>>>(
            n_long, pos.get(), view.pull_off, 0u, drec.get());
        GTC_LAUNCHED();
        L++;
        GTC_CUDA(cudaMemcpyAsync(lrec.data(), drec.get(), n_long * sizeof(uint4),
                                 cudaMemcpyDeviceToHost, h));
        GTC_CUDA(cudaStreamSynchronize(h));
    }
    std::vector<uint4> chunks, longs(n_long);
    for (uint32_t j = 0; j < n_long; ++j) {
        const uint4 r = lrec[j];
        const uint32_t first = (uint32_t)chunks.size();
        for (uint32_t b = r.y; b < r.z; b += PPR_CHUNK)
            chunks.push_back(make_uint4(r.x, b, std::min(r.z, b + PPR_CHUNK), j));
        longs[j] = make_uint4(r.x, first, (uint32_t)chunks.size() - first, 0u);
    }
    const uint32_t n_single = n - n_long;
    S.n_long = n_long;
    S.n_chunks = (uint32_t)chunks.size();
    S.n_items = S.n_chunks + n_single;
    S.n_empty = cnts[1];  // the last single rows (the highest key)
    S.n_heavy = S.n_chunks + cnts[2];  // chunks, then the single rows of the lowest keys
    S.items.alloc(S.n_items, h);
    S.longs.alloc(S.n_long, h);
    if (S.n_chunks)
        GTC_CUDA(cudaMemcpyAsync(S.items.get(), chunks.data(), chunks.size() * sizeof(uint4),
                                 cudaMemcpyHostToDevice, h));
    if (n_single) {
        k_ppr_row_items<<<grid_for(n_single, 256, 1u << 30), 256, 0, h>>>(
            n_single, pos.get() + n_long, view.pull_off, PPR_NONE, S.items.get() + S.n_chunks);
        GTC_LAUNCHED();
        L++;
    }
    if (S.n_long)
        GTC_CUDA(cudaMemcpyAsync(S.longs.get(), longs.data(), longs.size() * sizeof(uint4),
                                 cudaMemcpyHostToDevice, h));
    GTC_CUDA(cudaStreamSynchronize(h));
    S.built = true;
    g->launches += L;
}

inline uint32_t host_float_bits(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return u;
}

struct PprTimer {
    cudaEvent_t a = nullptr, b = nullptr;
    cudaStream_t s;
    explicit PprTimer(cudaStream_t st) : s(st) {
        GTC_CUDA(cudaEventCreate(&a));
        GTC_CUDA(cudaEventCreate(&b));
    }
    ~PprTimer() {
        if (a) cudaEventDestroy(a);
        if (b) cudaEventDestroy(b);
    }
    void start() { GTC_CUDA(cudaEventRecord(a, s)); }
    void stop() { GTC_CUDA(cudaEventRecord(b, s)); }
    double ms() {
        GTC_CUDA(cudaEventSynchronize(b));
        float t = 0.f;
        GTC_CUDA(cudaEventElapsedTime(&t, a, b));
        return t;
    }
};

// gathered rows in flight per warp: about 32 loads per lane
constexpr int ppr_unroll(int C) { return C <= 1 ? 16 : C <= 4 ? 8 : C <= 8 ? 4 : 2; }

// The two gather variants of part 1: loads into registers, or bulk copies
// into shared memory.
enum PprVariant { PPR_REGS = 0, PPR_BULK = 1 };

struct PprLaunch {
    unsigned grid1, threads1;
    size_t smem1;
};

// Part 1's launch shape: as many CTAs as fit on every SM at once.
template <int C>
PprLaunch ppr_shape(int variant, bool weighted) {
    int per_sm = 0, sms = 0, dev = 0;
    GTC_CUDA(cudaGetDevice(&dev));
    GTC_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const size_t smem_long = ppr_smem(32 * C);
    GTC_CUDA(cudaFuncSetAttribute(k_ppr_long<C>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)smem_long));
    PprLaunch L{};
    if (variant == PPR_BULK) {
        auto* f = weighted ? k_ppr_bulk<C, true> : k_ppr_bulk<C, false>;
        L.threads1 = PB_NT;
        L.smem1 = (size_t)PbLayout<C>::CTA;
        GTC_CUDA(cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L.smem1));
        GTC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, f, PB_NT, L.smem1));
    } else {
        auto* f = weighted ? k_ppr_rows<C, ppr_unroll(C), true> : k_ppr_rows<C, ppr_unroll(C), false>;
        L.threads1 = PPR_NT;
        L.smem1 = smem_long;
        GTC_CUDA(cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L.smem1));
        GTC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, f, PPR_NT, L.smem1));
    }
    L.grid1 = (unsigned)std::max(1, per_sm * sms);
    return L;
}

template <int C>
void launch_ppr(PprArgs A, int variant, const PprLaunch& L1, unsigned grid2, cudaStream_t s) {
    A.part_base = 0;
    if (variant == PPR_BULK) {
        if (A.w)
            k_ppr_bulk<C, true><<<L1.grid1, PB_NT, L1.smem1, s>>>(A);
        else
            k_ppr_bulk<C, false><<<L1.grid1, PB_NT, L1.smem1, s>>>(A);
    } else {
        if (A.w)
            k_ppr_rows<C, ppr_unroll(C), true><<<L1.grid1, PPR_NT, L1.smem1, s>>>(A);
        else
            k_ppr_rows<C, ppr_unroll(C), false><<<L1.grid1, PPR_NT, L1.smem1, s>>>(A);
    }
    GTC_LAUNCHED();
    A.part_base = L1.grid1;
    k_ppr_long<C><<<grid2, PPR_NT, ppr_smem(32 * C), s>>>(A);
    GTC_LAUNCHED();
}

template <int C>
void launch_sinks(PprArgs A, const uint32_t* pull_off, unsigned part_base, unsigned grid3,
                  cudaStream_t s) {
    A.part_base = part_base;
    k_ppr_sinks<C><<<grid3, PPR_NT, (size_t)PPR_WARPS * 32 * C * sizeof(float2), s>>>(A, pull_off);
    GTC_LAUNCHED();
}

void fold(const PprArgs& A, unsigned n_parts, double* out, cudaStream_t s) {
    const uint32_t nv = 2 * A.s_in;
    k_ppr_fold<<<(nv + 63) / 64, 64, 0, s>>>(nv, n_parts, A.part, out);
    GTC_LAUNCHED();
}

// line counts a sweep runs at: 1-4, 6, then multiples of 4 (vector loads)
#define GTC_PPR_C(X) X(1) X(2) X(3) X(4) X(6) X(8) X(12) X(16)

PprLaunch shape(uint32_t C, int variant, bool weighted) {
    switch (C) {
#define GTC_CASE(c) \
    case c: return ppr_shape<c>(variant, weighted);
        GTC_PPR_C(GTC_CASE)
#undef GTC_CASE
    }
    throw Error{GTC_ERR_CUDA, "batched personalised PageRank: bad slot count"};
}

void run_sweep(uint32_t C, const PprArgs& A, int variant, const PprLaunch& L1, unsigned grid2,
               cudaStream_t s) {
    switch (C) {
#define GTC_CASE(c) \
    case c: launch_ppr<c>(A, variant, L1, grid2, s); return;
        GTC_PPR_C(GTC_CASE)
#undef GTC_CASE
    }
    throw Error{GTC_ERR_CUDA, "batched personalised PageRank: bad slot count"};
}

void run_sinks(uint32_t c_out, const PprArgs& A, const uint32_t* pull_off, unsigned part_base,
               unsigned grid3, cudaStream_t s) {
    switch (c_out) {
#define GTC_CASE(c) \
    case c: launch_sinks<c>(A, pull_off, part_base, grid3, s); return;
        GTC_PPR_C(GTC_CASE)
#undef GTC_CASE
    }
    throw Error{GTC_ERR_CUDA, "batched personalised PageRank: bad slot count"};
}

template <int K>
void launch_narrow(PprArgs A, bool weighted, unsigned grid1, unsigned grid2, cudaStream_t s) {
    A.part_base = 0;
    if (weighted)
        k_ppr_narrow<K, true><<<grid1, PPR_NT, 0, s>>>(A);
    else
        k_ppr_narrow<K, false><<<grid1, PPR_NT, 0, s>>>(A);
    GTC_LAUNCHED();
    A.part_base = grid1;
    k_ppr_narrow_long<K><<<grid2, PPR_NT, 0, s>>>(A);
    GTC_LAUNCHED();
}

// CTAs of the narrow part 1: as many as fit on every SM at once.
unsigned narrow_grid(uint32_t K, bool weighted, int sms) {
    int per_sm = 0;
    if (K == 8)
        GTC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &per_sm, weighted ? k_ppr_narrow<8, true> : k_ppr_narrow<8, false>, PPR_NT, 0));
    else
        GTC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &per_sm, weighted ? k_ppr_narrow<16, true> : k_ppr_narrow<16, false>, PPR_NT, 0));
    return (unsigned)std::max(1, per_sm * sms);
}

// Lines per row for `active` columns: ceil(active / 32), rounded up to 6 or
// to a multiple of 4 above 4 lines (widths with vector loads).
inline uint32_t ppr_lines(uint32_t active) {
    const uint32_t c = (active + 31) / 32;
    return c <= 4 ? c : (c <= 6 ? 6 : (c + 3) / 4 * 4);
}

}  // namespace

void ppr_batch(gtc_graph* g, const gtc_view* vw, const PprIn& in, gtc_result* res,
               cudaStream_t s) {
    uint64_t L = 0, SL = 0, L_solver = 0;
    const unsigned TB = 256;
    GTC_REQUIRE(!vw || (!vw->vmask && !vw->emask), GTC_ERR_ARG,
                "batched personalised PageRank supports the graph and its reversal, not filtered "
                "views");
    GTC_REQUIRE(in.B >= 1 && in.B <= PPR_MAXB, GTC_ERR_ARG,
                "batched personalised PageRank takes 1 to 512 personalisation vectors");
    View view;
    view.prepare(g, vw, s, &L);
    const uint32_t n = view.n, B = in.B;
    const double d = in.damping;
    for (uint32_t b = 0; b < B; ++b)
        GTC_REQUIRE(in.seed_off[b + 1] >= in.seed_off[b], GTC_ERR_ARG,
                    "seed offsets must not decrease");
    const uint64_t ns_all = in.seed_off[B];
    GTC_REQUIRE(ns_all < (1ull << 31), GTC_ERR_ARG, "too many seeds");
    for (uint64_t k = 0; k < ns_all; ++k)
        GTC_REQUIRE(in.seed_vertices[k] < n, GTC_ERR_INDEX, "a seed vertex is outside the vertex bound");
    const uint32_t ns = (uint32_t)ns_all;

    if (in.weight.present()) (void)scan_weights(in.weight, g->m, s, &L);
    // degrees of the view and pull-ordered weights
    DevBuf<double> deg(n, s);
    if (n) {
        k_degree_ppr<<<grid_for(n, TB, 1u << 30), TB, 0, s>>>(n, view.push_off, view.push_eid,
                                                              in.weight.p, in.weight.dtype, deg.get());
        GTC_LAUNCHED();
        L++;
    }
    DevBuf<float> wpull;
    if (in.weight.present() && view.m_pull) {
        wpull.alloc(view.m_pull, s);
        k_gather_w_ppr<<<grid_for(view.m_pull, TB, 1u << 30), TB, 0, s>>>(
            view.m_pull, view.pull_eid, in.weight.p, in.weight.dtype, wpull.get());
        GTC_LAUNCHED();
        L++;
    }
    DevBuf<float2> dinv(n, s);
    if (n) {
        k_ppr_dinv<<<grid_for(n, TB, 1u << 30), TB, 0, s>>>(n, deg.get(), dinv.get());
        GTC_LAUNCHED();
        L++;
    }
    PprSched& S = g->ppr_sched[view.reversed ? 1 : 0];
    if (!S.built) build_ppr_schedule(g, view, s, S);

    // the seeds: internal labels, one record per (vertex, column) -- the
    // last value given for a pair wins -- sorted by vertex
    std::vector<uint32_t> iv(ns), inn(ns);
    std::vector<double> dv(ns);
    if (ns) {
        DevBuf<uint32_t> dorig(ns, s), div(ns, s), dinn(ns, s);
        DevBuf<double> ddv(ns, s);
        GTC_CUDA(cudaMemcpyAsync(dorig.get(), in.seed_vertices, (size_t)ns * 4, cudaMemcpyHostToDevice, s));
        k_ppr_seed_lookup<<<grid_for(ns, TB, 1u << 30), TB, 0, s>>>(
            ns, dorig.get(), g->iperm.get(), deg.get(), view.pull_off, div.get(), ddv.get(), dinn.get());
        GTC_LAUNCHED();
        L++;
        GTC_CUDA(cudaMemcpyAsync(iv.data(), div.get(), (size_t)ns * 4, cudaMemcpyDeviceToHost, s));
        GTC_CUDA(cudaMemcpyAsync(dv.data(), ddv.get(), (size_t)ns * 8, cudaMemcpyDeviceToHost, s));
        GTC_CUDA(cudaMemcpyAsync(inn.data(), dinn.get(), (size_t)ns * 4, cudaMemcpyDeviceToHost, s));
        GTC_CUDA(cudaStreamSynchronize(s));
    }
    // seed rows without in-edges (the sweeps' single rows skip every row
    // without in-edges), ascending
    std::vector<uint32_t> hes;
    for (uint32_t k = 0; k < ns; ++k)
        if (inn[k] == 0) hes.push_back(iv[k]);
    std::sort(hes.begin(), hes.end());
    hes.erase(std::unique(hes.begin(), hes.end()), hes.end());
    const uint32_t n_es = (uint32_t)hes.size();
    DevBuf<uint32_t> des(n_es ? n_es : 1, s);
    if (n_es)
        GTC_CUDA(cudaMemcpyAsync(des.get(), hes.data(), (size_t)n_es * 4, cudaMemcpyHostToDevice, s));
    struct Rec {
        uint32_t v, col;
        float val;
        double deg;
    };
    std::vector<Rec> recs;
    recs.reserve(ns);
    for (uint32_t b = 0; b < B; ++b) {
        const uint64_t sb = in.seed_off[b], se = in.seed_off[b + 1];
        for (uint64_t k = sb; k < se; ++k) {
            const double val = in.seed_values ? in.seed_values[k] : 1.0 / (double)(se - sb);
            recs.push_back({iv[k], b, (float)val, dv[k]});
        }
    }
    std::stable_sort(recs.begin(), recs.end(), [](const Rec& a, const Rec& b) {
        return a.v != b.v ? a.v < b.v : a.col < b.col;
    });
    std::vector<Rec> uniq;
    for (const Rec& r : recs) {
        if (!uniq.empty() && uniq.back().v == r.v && uniq.back().col == r.col)
            uniq.back() = r;
        else
            uniq.push_back(r);
    }
    const uint32_t nu = (uint32_t)uniq.size();
    std::vector<uint32_t> hsv(nu ? nu : 1);
    std::vector<uint2> hsd(nu ? nu : 1);
    std::vector<double> psink_col(B, 0.0);  // dangling mass of each column's iterate
    for (uint32_t k = 0; k < nu; ++k) {
        hsv[k] = uniq[k].v;
        hsd[k] = make_uint2(uniq[k].col, host_float_bits(uniq[k].val));
        if (uniq[k].deg == 0.0) psink_col[uniq[k].col] += (double)uniq[k].val;
    }
    DevBuf<uint32_t> dsv(hsv.size(), s), dso((size_t)n + 1, s);
    DevBuf<uint2> dsd(hsd.size(), s);
    GTC_CUDA(cudaMemcpyAsync(dsv.get(), hsv.data(), hsv.size() * 4, cudaMemcpyHostToDevice, s));
    GTC_CUDA(cudaMemcpyAsync(dsd.get(), hsd.data(), hsd.size() * sizeof(uint2), cudaMemcpyHostToDevice, s));
    k_ppr_seed_off<<<grid_for((size_t)n + 1, TB, 1u << 30), TB, 0, s>>>(n, nu, dsv.get(), dso.get());
    GTC_LAUNCHED();
    L++;

    // iterates: the first layout is slot = column; the row pitch stays P
    uint32_t C = ppr_lines(B);
    uint32_t s_in = 32 * C;
    const uint32_t P = s_in;
    const size_t zn = (size_t)n * P;
    // the two iterate buffers live on the handle: a later batch of the same
    // or a smaller width does not allocate them again
    if (g->ppr_z[0].n < zn || !g->ppr_z[0].get()) {
        GTC_CUDA(cudaStreamSynchronize(s));
        g->ppr_z[0].alloc(zn, g->home);
        g->ppr_z[1].alloc(zn, g->home);
        GTC_CUDA(cudaStreamSynchronize(g->home));
    }
    DevBuf<float>& z0 = g->ppr_z[0];
    DevBuf<float>& z1 = g->ppr_z[1];
    if (zn) {
        GTC_CUDA(cudaMemsetAsync(z0.get(), 0, zn * sizeof(float), s));
        GTC_CUDA(cudaMemsetAsync(z1.get(), 0, zn * sizeof(float), s));
    }
    if (nu && n) {
        k_ppr_init<<<grid_for(nu, TB, 1u << 30), TB, 0, s>>>(nu, s_in, dsv.get(), dsd.get(),
                                                             dinv.get(), z0.get());
        GTC_LAUNCHED();
        L++;
    }
    int sms = 0, dev = 0;
    GTC_CUDA(cudaGetDevice(&dev));
    GTC_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const unsigned grid1_max = (unsigned)sms * (2048 / 32);  // at most one CTA per warp slot
    const unsigned grid2 =
        std::max(1u, std::min((S.n_long + n_es + PPR_WARPS - 1) / PPR_WARPS, (unsigned)sms));
    DevBuf<float2> cpart((size_t)S.n_chunks * s_in, s);
    // the dangling-mass kernel: a warp per 32-vertex group, 2 CTAs per SM
    const unsigned grid3 =
        std::max(1u, std::min((unsigned)(((size_t)n + 32 * PPR_WARPS - 1) / (32 * PPR_WARPS)),
                              2u * (unsigned)sms));
    DevBuf<double> part((size_t)(grid1_max + grid2 + grid3) * 2 * s_in, s), out(2 * (size_t)s_in, s);
    DevBuf<uint32_t> dmap(2 * (size_t)s_in, s);  // col_in, then out_slot
    DevBuf<float> dps(s_in, s);
    DevBuf<uint2> dpairs(s_in, s);
    DevBuf<int> derr(1, s);
    GTC_CUDA(cudaMemsetAsync(derr.get(), 0, sizeof(int), s));
    const int variant = in.gather == GTC_PPR_REGS ? PPR_REGS : PPR_BULK;

    PprArgs A{};
    A.n = n;
    A.pitch = P;
    A.items = S.items.get(), A.n_items = S.n_items - S.n_empty, A.n_chunks = S.n_chunks;
    A.longs = S.longs.get(), A.n_long = S.n_long;
    A.eseeds = des.get(), A.n_eseeds = n_es;
    A.n_heavy = S.n_heavy;
    A.other = view.pull_other, A.w = wpull.get();
    A.dinv = dinv.get();
    A.seed_off = dso.get(), A.seeds = dsd.get();
    A.psink = dps.get();
    A.one_minus_d = (float)(1.0 - d), A.d = (float)d;
    A.cpart = cpart.get(), A.part = part.get(), A.err = derr.get();

    std::vector<uint32_t> col_in(s_in, PPR_NONE), out_slot, col_out, maps;
    for (uint32_t b = 0; b < B; ++b) col_in[b] = b;
    std::vector<uint8_t> done(B, 0);
    std::vector<double> hout;
    std::vector<float> hps;
    std::vector<uint2> store;
    std::fill(in.iters, in.iters + B, 0);
    uint32_t running = B;
    uint64_t sweeps = 0;
    double sweep_ms = 0.0;
    float *zc = z0.get(), *zx = z1.get();
    PprTimer total(s), tsw(s);
    total.start();
    uint32_t K = 0;  // narrow row width, 0 while the rows are lines
    uint32_t pitch = P;
    const bool W = A.w != nullptr;
    unsigned grid_n = 0;
    while (running > 0) {
        uint32_t running_slots = 0;
        for (uint32_t j = 0; j < s_in; ++j)
            if (col_in[j] != PPR_NONE && !done[col_in[j]]) ++running_slots;
        const uint32_t want = running_slots <= 8 ? 8u : running_slots <= PPR_NARROW ? 16u : 0u;
        if (want && want != K && n) {
            // the running columns, in slot order, into rows of `want` floats;
            // the other buffer's rows of that width start at zero (the rows
            // without in-edges are never written)
            std::vector<uint32_t> src_slot(want, PPR_NONE), ncol(want, PPR_NONE);
            for (uint32_t j = 0, k = 0; j < s_in; ++j) {
                const uint32_t c = col_in[j];
                if (c == PPR_NONE || done[c]) continue;
                src_slot[k] = j;
                ncol[k++] = c;
            }
            GTC_CUDA(cudaMemcpyAsync(dmap.get(), src_slot.data(), want * 4, cudaMemcpyHostToDevice, s));
            k_ppr_narrow_pack<<<grid_for((size_t)n * want, TB, 1u << 30), TB, 0, s>>>(
                n, want, pitch, dmap.get(), zc, zx);
            GTC_LAUNCHED();
            L++;
            GTC_CUDA(cudaMemsetAsync(zc, 0, (size_t)n * want * sizeof(float), s));
            std::swap(zc, zx);
            col_in = ncol;
            s_in = want;
            K = want;
            pitch = want;
            grid_n = std::min(grid1_max, narrow_grid(K, W, sms));
        }
        if (K) {
            // a narrow sweep: every running column keeps its slot
            out_slot.assign(K, PPR_NONE);
            hps.assign(K, 0.f);
            for (uint32_t k = 0; k < K; ++k) {
                const uint32_t c = col_in[k];
                if (c == PPR_NONE) continue;
                hps[k] = (float)psink_col[c];
                if (!done[c]) out_slot[k] = k;
            }
            maps.assign(col_in.begin(), col_in.end());
            maps.insert(maps.end(), out_slot.begin(), out_slot.end());
            GTC_CUDA(cudaMemcpyAsync(dmap.get(), maps.data(), maps.size() * 4, cudaMemcpyHostToDevice, s));
            GTC_CUDA(cudaMemcpyAsync(dps.get(), hps.data(), K * sizeof(float), cudaMemcpyHostToDevice, s));
            A.col_in = dmap.get(), A.out_slot = dmap.get() + K;
            A.s_in = A.s_out = K;
            A.pitch = K;
            A.in_place = 1u;
            A.zin = zc, A.zout = zx;
            if (in.timing) tsw.start();
            if (K == 8)
                launch_narrow<8>(A, W, grid_n, grid2, s);
            else
                launch_narrow<16>(A, W, grid_n, grid2, s);
            fold(A, grid_n + grid2, out.get(), s);
            if (in.timing) tsw.stop();
            L += 3;
            SL += 3;
            hout.resize(2 * (size_t)K);
            GTC_CUDA(cudaMemcpyAsync(hout.data(), out.get(), 2 * (size_t)K * sizeof(double),
                                     cudaMemcpyDeviceToHost, s));
            int herr = 0;
            GTC_CUDA(cudaMemcpyAsync(&herr, derr.get(), sizeof(int), cudaMemcpyDeviceToHost, s));
            GTC_CUDA(cudaStreamSynchronize(s));
            GTC_REQUIRE(herr == 0, GTC_ERR_CUDA,
                        "batched personalised PageRank: a gathered row did not arrive in time");
            if (in.timing) sweep_ms += tsw.ms();
            ++sweeps;
            store.clear();
            for (uint32_t k = 0; k < K; ++k) {
                const uint32_t c = col_in[k];
                if (c == PPR_NONE || out_slot[k] == PPR_NONE) continue;
                in.iters[c] = sweeps;
                psink_col[c] = hout[K + k];
                if (hout[k] < in.params.epsilon ||
                    (in.params.max_iter > 0 && sweeps == in.params.max_iter)) {
                    done[c] = 1;
                    --running;
                    store.push_back(make_uint2(k, c));
                }
            }
            if (!store.empty()) {
                const uint32_t nk = (uint32_t)store.size();
                GTC_CUDA(cudaMemcpyAsync(dpairs.get(), store.data(), nk * sizeof(uint2),
                                         cudaMemcpyHostToDevice, s));
                dim3 g2((n + 31) / 32, (nk + 31) / 32), blk(32, 8);
                k_ppr_store<<<g2, blk, 0, s>>>(n, K, nk, dpairs.get(), g->iperm.get(), dinv.get(),
                                              zx, in.out, in.out_dtype);
                GTC_LAUNCHED();
                L++;
            }
            std::swap(zc, zx);
            if (running > 0 && running <= PPR_HANDOFF) {
                // the last columns: their iterates to the output, then the
                // single-vector solver continues each from there (pagerank_with
                // from a warm start is the same iteration)
                const size_t esz = in.out_dtype == GTC_F64 ? 8 : 4;
                DevBuf<float> pers(n, s), dvals(64, s);
                DevBuf<uint32_t> dverts(64, s);
                for (uint32_t k = 0; k < K; ++k) {
                    const uint32_t c = col_in[k];
                    if (c == PPR_NONE || done[c]) continue;
                    const uint2 pair = make_uint2(k, c);
                    GTC_CUDA(cudaMemcpyAsync(dpairs.get(), &pair, sizeof(uint2), cudaMemcpyHostToDevice, s));
                    dim3 g2((n + 31) / 32, 1), blk(32, 8);
                    k_ppr_store<<<g2, blk, 0, s>>>(n, K, 1, dpairs.get(), g->iperm.get(), dinv.get(),
                                                  zc, in.out, in.out_dtype);
                    GTC_LAUNCHED();
                    const uint64_t sb = in.seed_off[c], se = in.seed_off[c + 1];
                    std::vector<uint32_t> hv;
                    std::vector<float> hval;
                    for (uint64_t t = sb; t < se; ++t) {
                        hv.push_back(in.seed_vertices[t]);
                        hval.push_back((float)(in.seed_values ? in.seed_values[t] : 1.0 / (double)(se - sb)));
                    }
                    if (hv.size() > dverts.n) dverts.alloc(hv.size(), s), dvals.alloc(hv.size(), s);
                    GTC_CUDA(cudaMemsetAsync(pers.get(), 0, (size_t)n * sizeof(float), s));
                    if (!hv.empty()) {
                        GTC_CUDA(cudaMemcpyAsync(dverts.get(), hv.data(), hv.size() * 4, cudaMemcpyHostToDevice, s));
                        GTC_CUDA(cudaMemcpyAsync(dvals.get(), hval.data(), hval.size() * 4, cudaMemcpyHostToDevice, s));
                        k_ppr_pers<<<1, 32, 0, s>>>((uint32_t)hv.size(), dverts.get(), dvals.get(), pers.get());
                        GTC_LAUNCHED();
                    }
                    L += 2;
                    SolveIn si{};
                    si.weight = in.weight;
                    si.pers.p = pers.get(), si.pers.len = n, si.pers.dtype = GTC_F32;
                    si.damping = in.damping;
                    si.params = in.params;
                    si.params.max_iter = in.params.max_iter > 0 ? in.params.max_iter - sweeps : 0;
                    si.x = static_cast<char*>(in.out) + (size_t)c * n * esz;
                    si.x_dtype = in.out_dtype;
                    si.had = n;
                    si.precision = GTC_PREC_F32;
                    gtc_result r{};
                    pagerank(g, vw, si, &r, s);
                    in.iters[c] = sweeps + r.iterations;
                    L_solver += r.launches;  // already counted on the handle by the solver
                    SL += r.sweep_launches;
                    done[c] = 1;
                }
                running = 0;
            }
            continue;
        }
        // the output layout: the columns still running keep their slots while
        // they need as many lines as now (a converged column leaves a hole),
        // and are packed into the lowest slots when they need fewer
        uint32_t active = 0;
        for (uint32_t j = 0; j < s_in; ++j)
            if (col_in[j] != PPR_NONE && !done[col_in[j]]) ++active;
        const uint32_t c_out = ppr_lines(active);
        const uint32_t s_out = 32 * c_out;
        const bool in_place = c_out == C;
        out_slot.assign(s_in, PPR_NONE);
        col_out.assign(s_out, PPR_NONE);
        for (uint32_t j = 0, k = 0; j < s_in; ++j) {
            const uint32_t c = col_in[j];
            if (c == PPR_NONE || done[c]) continue;
            out_slot[j] = in_place ? j : k++;
            col_out[out_slot[j]] = c;
        }
        A.in_place = in_place ? 1u : 0u;
        hps.assign(s_in, 0.f);
        for (uint32_t j = 0; j < s_in; ++j)
            if (col_in[j] != PPR_NONE) hps[j] = (float)psink_col[col_in[j]];
        maps.assign(col_in.begin(), col_in.end());
        maps.insert(maps.end(), out_slot.begin(), out_slot.end());
        GTC_CUDA(cudaMemcpyAsync(dmap.get(), maps.data(), maps.size() * 4, cudaMemcpyHostToDevice, s));
        GTC_CUDA(cudaMemcpyAsync(dps.get(), hps.data(), s_in * sizeof(float), cudaMemcpyHostToDevice, s));
        A.col_in = dmap.get(), A.out_slot = dmap.get() + s_in;
        A.s_in = s_in, A.s_out = s_out;
        A.pitch = P;
        A.zin = zc, A.zout = zx;
        PprLaunch L1 = shape(C, variant, A.w != nullptr);
        L1.grid1 = std::min(grid1_max, L1.grid1);
        if (in.timing) tsw.start();
        run_sweep(C, A, variant, L1, grid2, s);
        run_sinks(c_out, A, view.pull_off, L1.grid1 + grid2, grid3, s);
        fold(A, L1.grid1 + grid2 + grid3, out.get(), s);
        if (in.timing) tsw.stop();
        L += 4;
        SL += 4;
        hout.resize(2 * (size_t)s_in);
        GTC_CUDA(cudaMemcpyAsync(hout.data(), out.get(), 2 * (size_t)s_in * sizeof(double),
                                 cudaMemcpyDeviceToHost, s));
        int herr = 0;
        GTC_CUDA(cudaMemcpyAsync(&herr, derr.get(), sizeof(int), cudaMemcpyDeviceToHost, s));
        GTC_CUDA(cudaStreamSynchronize(s));
        GTC_REQUIRE(herr == 0, GTC_ERR_CUDA,
                    "batched personalised PageRank: a gathered row did not arrive in time");
        if (in.timing) sweep_ms += tsw.ms();
        ++sweeps;
        store.clear();
        for (uint32_t j = 0; j < s_in; ++j) {
            const uint32_t c = col_in[j];
            if (c == PPR_NONE || out_slot[j] == PPR_NONE) continue;
            in.iters[c] = sweeps;
            psink_col[c] = hout[s_in + out_slot[j]];  // the mass is per output slot
            if (hout[j] < in.params.epsilon ||
                (in.params.max_iter > 0 && sweeps == in.params.max_iter)) {
                done[c] = 1;
                --running;
                store.push_back(make_uint2(out_slot[j], c));
            }
        }
        // converged columns go to the output now, from this sweep's iterate
        // (a copy from pageable memory returns once the source is staged)
        if (!store.empty() && n) {
            const uint32_t nk = (uint32_t)store.size();
            GTC_CUDA(cudaMemcpyAsync(dpairs.get(), store.data(), nk * sizeof(uint2),
                                     cudaMemcpyHostToDevice, s));
            dim3 g2((n + 31) / 32, (nk + 31) / 32), blk(32, 8);
            k_ppr_store<<<g2, blk, 0, s>>>(n, P, nk, dpairs.get(), g->iperm.get(), dinv.get(), zx,
                                          in.out, in.out_dtype);
            GTC_LAUNCHED();
            L++;
        }
        col_in = col_out;
        s_in = s_out;
        C = c_out;
        std::swap(zc, zx);
    }
    total.stop();
    res->device_ms = total.ms();
    GTC_CUDA(cudaStreamSynchronize(s));
    res->iterations = B ? *std::max_element(in.iters, in.iters + B) : 0;
    res->last_delta = 0.0;
    res->eigenvalue = 0.0;
    res->launches = L + L_solver;
    res->sweep_ms = sweep_ms;
    res->sweep_launches = SL;
    g->launches += L;
}

}  // namespace gtc
