// gtc_ppr.cu -- many personalised PageRanks over one edge stream (an SpMM).
//
// B personalisation vectors (seed sets) are solved together: pagerank_with
// (crates/gt-algo/src/centrality.rs:261-384) for every column b, each from
// its own start (a fresh map is seeded with pers_b, centrality.rs:198-205),
// each stopping at the first sweep whose L1 change falls below epsilon.
//
// Layout.  Z is [n x Bp] row-major (Bp = B rounded up to 128 columns): one
// vertex's Bp values are contiguous, so the pull of an in-edge s -> v reads
// Z[s][*] as whole 1 KB lines (B = 256) -- the gather of the single solve,
// amortised over all columns.  Z[v][b] holds rank_b[v] / deg_v for a vertex
// with out-edges and rank_b[v] itself for a sink (a sink is never gathered),
// so one pair of ping-pong arrays carries both what is gathered and what the
// L1 change is measured against.
//
// Schedule.  One warp per row (a lane owns Bp/32 consecutive columns, read
// as float4), heaviest rows first; rows with more than PPR_LONG in-edges take
// a whole CTA whose warps' compensated partials merge in warp order.  The
// per-column FP64 change and dangling mass are folded per CTA and then, by
// the last CTA, over CTAs in a fixed order: deterministic.  A column that
// converged is frozen (carried unchanged) for the remaining sweeps.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "gtc_view.cuh"

namespace gtc {
namespace {

constexpr int PPR_NT = 256;
constexpr int PPR_WARPS = PPR_NT / 32;
constexpr uint32_t PPR_LONG = 4096;   // rows with more in-edges take a whole CTA
constexpr uint32_t PPR_MAXB = 512;    // largest batch

struct PprArgs {
    uint32_t n, Bp;
    const uint32_t* __restrict__ rows;   // warp rows, heaviest first
    uint32_t n_rows;
    const uint32_t* __restrict__ longs;  // CTA rows
    uint32_t n_long;
    const uint32_t* __restrict__ off;
    const uint32_t* __restrict__ other;
    const float* __restrict__ w;         // pull-ordered weights or null
    const float* __restrict__ zprev;     // [n][Bp]
    float* __restrict__ znext;
    const double* __restrict__ deg;
    const uint8_t* __restrict__ sink;
    const uint32_t* __restrict__ seed_off;  // per vertex: seeds [seed_off[v], seed_off[v+1])
    const uint2* __restrict__ seeds;        // {column, float bits of the value}
    const uint8_t* __restrict__ frozen;     // per column
    const double* __restrict__ psink;       // per column: dangling mass of prev
    float one_minus_d, d;
    double* part;      // per CTA: 2*Bp doubles (delta[b], dangling mass[b])
    unsigned* ticket;
    double* out;       // 2*Bp: delta[b], then dangling mass of next [b]
};

__device__ __forceinline__ float ldf(const float4& v, int k) {
    return k == 0 ? v.x : (k == 1 ? v.y : (k == 2 ? v.z : v.w));
}

// Compensated accumulation of C columns (classic Kahan, value s - c).
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
    // a lane's C consecutive values of gathered row `src`
    __device__ __forceinline__ void add_row(const float* __restrict__ z, uint32_t Bp, uint32_t src,
                                            uint32_t c0, float w, bool weighted) {
        const float4* r = reinterpret_cast<const float4*>(z + (size_t)src * Bp + c0);
#pragma unroll
        for (int q = 0; q < C / 4; ++q) {
            const float4 a = __ldg(r + q);
#pragma unroll
            for (int k = 0; k < 4; ++k) add(4 * q + k, weighted ? __fmul_rn(ldf(a, k), w) : ldf(a, k));
        }
    }
};

// Epilogue of row v for a lane's C columns (c0 = first column).
template <int C>
__device__ __forceinline__ void ppr_row(const PprArgs& A, uint32_t v, const float* sum,
                                        uint32_t c0, float* dacc, float* sacc, const float* ps,
                                        uint32_t frozen_bits) {
    const double dg = A.deg[v];
    const bool snk = A.sink[v];
    const float fdeg = (float)dg;
    const float inv = dg != 0.0 ? (float)(1.0 / dg) : 0.f;
    const uint32_t sb = A.seed_off[v], se = A.seed_off[v + 1];
    const float* zp = A.zprev + (size_t)v * A.Bp + c0;
    float* zn = A.znext + (size_t)v * A.Bp + c0;
#pragma unroll
    for (int q = 0; q < C / 4; ++q) {
        const float4 z4 = *reinterpret_cast<const float4*>(zp + 4 * q);
        float o[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int c = 4 * q + k;
            const float z = ldf(z4, k);
            const float prev = snk ? z : __fmul_rn(z, fdeg);
            float pv = 0.f;
            for (uint32_t t = sb; t < se; ++t) {
                const uint2 sd = A.seeds[t];
                if (sd.x == c0 + c) pv = __uint_as_float(sd.y);
            }
            float nv;
            if ((frozen_bits >> c) & 1u) {
                nv = prev;
            } else {
                const float r = __fadd_rn(__fmul_rn(ps[c], pv), sum[c]);
                nv = __fadd_rn(__fmul_rn(A.one_minus_d, pv), __fmul_rn(A.d, r));
                dacc[c] = __fadd_rn(dacc[c], fabsf(__fsub_rn(nv, prev)));
            }
            if (snk) sacc[c] = __fadd_rn(sacc[c], nv);
            o[k] = snk ? nv : __fmul_rn(nv, inv);
        }
        *reinterpret_cast<float4*>(zn + 4 * q) = make_float4(o[0], o[1], o[2], o[3]);
    }
}

// One sweep over all B columns.  Phase 1: each long row by one CTA (warp w
// sums in-edges w, w+8, ... in order; the warps' partials merge in warp
// order).  Phase 2: a warp per remaining row, heaviest first.  Every
// assignment is a fixed stride, so the sums do not depend on timing.
template <int C>
__global__ void __launch_bounds__(PPR_NT) k_ppr_sweep(PprArgs A) {
    extern __shared__ float2 lpart[];  // [PPR_WARPS][Bp] for phase 1
    __shared__ double red[PPR_WARPS][128];
    __shared__ bool last;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t c0 = lane * C;
    const bool W = A.w != nullptr;
    float ps[C], dacc[C], sacc[C];
    uint32_t frozen_bits = 0;
#pragma unroll
    for (int c = 0; c < C; ++c) {
        ps[c] = (float)A.psink[c0 + c];
        dacc[c] = 0.f, sacc[c] = 0.f;
        if (A.frozen[c0 + c]) frozen_bits |= 1u << c;
    }
    Acc<C> acc;
    // ---- phase 1: long rows, a CTA each ----
    for (uint32_t k = blockIdx.x; k < A.n_long; k += gridDim.x) {
        const uint32_t v = A.longs[k];
        const uint32_t b = A.off[v], e = A.off[v + 1];
        acc.zero();
        for (uint32_t p = b + warp; p < e; p += PPR_WARPS)
            acc.add_row(A.zprev, A.Bp, __ldg(A.other + p), c0, W ? __ldg(A.w + p) : 1.f, W);
#pragma unroll
        for (int c = 0; c < C; ++c) lpart[warp * A.Bp + c0 + c] = make_float2(acc.s[c], -acc.c[c]);
        __syncthreads();
        if (warp == 0) {
            float sum[C];
#pragma unroll
            for (int c = 0; c < C; ++c) {
                Kahan t;
                for (int wv = 0; wv < PPR_WARPS; ++wv) {
                    const float2 q = lpart[wv * A.Bp + c0 + c];
                    t.merge(q.x, q.y);
                }
                sum[c] = t.value();
            }
            ppr_row<C>(A, v, sum, c0, dacc, sacc, ps, frozen_bits);
        }
        __syncthreads();
    }
    // ---- phase 2: a warp per row ----
    const uint32_t gw = blockIdx.x * PPR_WARPS + warp, nw = gridDim.x * PPR_WARPS;
    for (uint32_t it = gw; it < A.n_rows; it += nw) {
        const uint32_t v = A.rows[it];
        const uint32_t b = A.off[v], e = A.off[v + 1];
        acc.zero();
        uint32_t p = b;
        for (; p + 2 <= e; p += 2) {  // two gathered rows in flight
            const uint32_t s0 = __ldg(A.other + p), s1 = __ldg(A.other + p + 1);
            const float w0 = W ? __ldg(A.w + p) : 1.f, w1 = W ? __ldg(A.w + p + 1) : 1.f;
            acc.add_row(A.zprev, A.Bp, s0, c0, w0, W);
            acc.add_row(A.zprev, A.Bp, s1, c0, w1, W);
        }
        if (p < e) acc.add_row(A.zprev, A.Bp, __ldg(A.other + p), c0, W ? __ldg(A.w + p) : 1.f, W);
        float sum[C];
#pragma unroll
        for (int c = 0; c < C; ++c) sum[c] = __fsub_rn(acc.s[c], acc.c[c]);
        ppr_row<C>(A, v, sum, c0, dacc, sacc, ps, frozen_bits);
    }
    // ---- per-column fold: warps -> CTA partial, CTAs -> last CTA (fixed order) ----
    const uint32_t Bp = A.Bp;
    for (uint32_t base = 0; base < Bp; base += 64) {
#pragma unroll
        for (int c = 0; c < C; ++c) {
            const uint32_t bc = c0 + c;
            if (bc >= base && bc < base + 64) {
                red[warp][bc - base] = (double)dacc[c];
                red[warp][64 + bc - base] = (double)sacc[c];
            }
        }
        __syncthreads();
        if (tid < 128) {
            double t = 0.0;
            for (int wv = 0; wv < PPR_WARPS; ++wv) t += red[wv][tid];
            const uint32_t bc = base + (tid & 63);
            A.part[(size_t)blockIdx.x * 2 * Bp + (tid < 64 ? bc : Bp + bc)] = t;
        }
        __syncthreads();
    }
    if (tid == 0) {
        __threadfence();
        last = atomicAdd(A.ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (last) {
        __threadfence();
        for (uint32_t bc = tid; bc < 2 * Bp; bc += PPR_NT) {
            double t8[8] = {0, 0, 0, 0, 0, 0, 0, 0};
            unsigned k = 0;
            for (; k + 8 <= gridDim.x; k += 8) {
#pragma unroll
                for (int j = 0; j < 8; ++j) t8[j] += __ldcg(A.part + (size_t)(k + j) * 2 * Bp + bc);
            }
            for (; k < gridDim.x; ++k) t8[0] += __ldcg(A.part + (size_t)k * 2 * Bp + bc);
            double t = 0.0;
#pragma unroll
            for (int j = 0; j < 8; ++j) t += t8[j];
            A.out[bc] = t;
        }
        if (tid == 0) *A.ticket = 0u;
    }
}

// Initial iterate: rank_b = pers_b (a fresh map), stored as Z; and the
// per-column dangling mass of it (host-side sum over the seeds, as seeds
// are few).
__global__ void k_ppr_init(uint32_t n, uint32_t Bp, const double* __restrict__ deg,
                           const uint32_t* __restrict__ seed_off, const uint2* __restrict__ seeds,
                           float* __restrict__ z) {
    const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (size_t)n * Bp) return;
    const uint32_t v = (uint32_t)(t / Bp), b = (uint32_t)(t % Bp);
    float pv = 0.f;
    for (uint32_t k = seed_off[v]; k < seed_off[v + 1]; ++k)
        if (seeds[k].x == b) pv = __uint_as_float(seeds[k].y);
    const double dg = deg[v];
    z[t] = dg != 0.0 ? __fmul_rn(pv, (float)(1.0 / dg)) : pv;
}

// out[b][v] = rank_b of original vertex v (transpose through shared memory)
__global__ void k_ppr_store(uint32_t n, uint32_t B, uint32_t Bp, const uint32_t* __restrict__ perm,
                            const double* __restrict__ deg, const uint8_t* __restrict__ sink,
                            const float* __restrict__ z, void* __restrict__ out, int dt) {
    __shared__ float tile[32][33];
    const uint32_t i0 = blockIdx.x * 32, b0 = blockIdx.y * 32;
    const uint32_t tx = threadIdx.x, ty = threadIdx.y;  // 32 x 8
    for (uint32_t r = ty; r < 32; r += 8) {
        const uint32_t i = i0 + r, b = b0 + tx;
        float val = 0.f;
        if (i < n && b < Bp) {
            const float zz = z[(size_t)i * Bp + b];
            val = sink[i] ? zz : __fmul_rn(zz, (float)deg[i]);
        }
        tile[r][tx] = val;
    }
    __syncthreads();
    for (uint32_t r = ty; r < 32; r += 8) {
        const uint32_t b = b0 + r, i = i0 + tx;
        if (b < B && i < n) {
            const size_t o = (size_t)b * n + perm[i];
            if (dt == GTC_F64)
                ((double*)out)[o] = (double)tile[tx][r];
            else
                ((float*)out)[o] = tile[tx][r];
        }
    }
}

struct PprSchedule {
    DevBuf<uint32_t> rows, longs;
    uint32_t n_rows = 0, n_long = 0;
};

// Rows of the pull half: the longest go to CTAs, the rest to warps, heaviest
// first (a stable order, so the schedule is a function of the graph).
void build_ppr_schedule(const uint32_t* d_off, uint32_t n, cudaStream_t s, PprSchedule& S) {
    std::vector<uint32_t> off((size_t)n + 1);
    GTC_CUDA(cudaMemcpyAsync(off.data(), d_off, ((size_t)n + 1) * 4, cudaMemcpyDeviceToHost, s));
    GTC_CUDA(cudaStreamSynchronize(s));
    std::vector<uint32_t> rows, longs;
    rows.reserve(n);
    for (uint32_t v = 0; v < n; ++v) (off[v + 1] - off[v] > PPR_LONG ? longs : rows).push_back(v);
    std::stable_sort(rows.begin(), rows.end(), [&](uint32_t a, uint32_t b) {
        return off[a + 1] - off[a] > off[b + 1] - off[b];
    });
    std::stable_sort(longs.begin(), longs.end(), [&](uint32_t a, uint32_t b) {
        return off[a + 1] - off[a] > off[b + 1] - off[b];
    });
    S.n_rows = (uint32_t)rows.size();
    S.n_long = (uint32_t)longs.size();
    S.rows.alloc(rows.size(), s);
    S.longs.alloc(longs.size(), s);
    if (!rows.empty())
        GTC_CUDA(cudaMemcpyAsync(S.rows.get(), rows.data(), rows.size() * 4, cudaMemcpyHostToDevice, s));
    if (!longs.empty())
        GTC_CUDA(cudaMemcpyAsync(S.longs.get(), longs.data(), longs.size() * 4, cudaMemcpyHostToDevice, s));
    GTC_CUDA(cudaStreamSynchronize(s));
}

inline uint32_t host_float_bits(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return u;
}
inline float host_bits_float(uint32_t u) {
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}

struct Timer_ {
    cudaEvent_t a = nullptr, b = nullptr;
    cudaStream_t s;
    explicit Timer_(cudaStream_t st) : s(st) {
        GTC_CUDA(cudaEventCreate(&a));
        GTC_CUDA(cudaEventCreate(&b));
    }
    ~Timer_() {
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

template <int C>
void launch_ppr(const PprArgs& A, unsigned grid, cudaStream_t s) {
    const size_t dyn = (size_t)PPR_WARPS * A.Bp * sizeof(float2);
    k_ppr_sweep<C><<<grid, PPR_NT, dyn, s>>>(A);
    GTC_LAUNCHED();
}

template <int C>
unsigned ppr_grid(uint32_t Bp) {
    int per_sm = 0, sms = 0, dev = 0;
    const int dyn = PPR_WARPS * (int)Bp * (int)sizeof(float2);
    GTC_CUDA(cudaGetDevice(&dev));
    GTC_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    GTC_CUDA(cudaFuncSetAttribute(k_ppr_sweep<C>, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn));
    GTC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_ppr_sweep<C>, PPR_NT, dyn));
    return (unsigned)std::max(1, per_sm * sms);
}

__global__ void k_degree_ppr(uint32_t n, const uint32_t* __restrict__ push_off,
                             const uint32_t* __restrict__ push_eid, const void* __restrict__ w,
                             int wdt, double* __restrict__ deg, uint8_t* __restrict__ sink) {
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
    sink[v] = k == 0.0 ? 1 : 0;
}

__global__ void k_gather_w_ppr(uint32_t m, const uint32_t* __restrict__ eid,
                               const void* __restrict__ w, int wdt, float* __restrict__ out) {
    size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p < m) out[p] = (float)ld_any(w, wdt, eid[p]);
}

}  // namespace

void ppr_batch(gtc_graph* g, const gtc_view* vw, const PprIn& in, gtc_result* res,
               cudaStream_t s) {
    uint64_t L = 0, SL = 0;
    const unsigned TB = 256;
    GTC_REQUIRE(!vw || (!vw->vmask && !vw->emask), GTC_ERR_ARG,
                "batched personalised PageRank supports the graph and its reversal, not filtered "
                "views");
    GTC_REQUIRE(in.B >= 1 && in.B <= PPR_MAXB, GTC_ERR_ARG,
                "batched personalised PageRank takes 1 to 512 personalisation vectors");
    View view;
    view.prepare(g, vw, s, &L);
    const uint32_t n = view.n, B = in.B;
    const uint32_t Bp = (B + 127) / 128 * 128;  // 128, 256, 384 or 512 columns
    const double d = in.damping;
    // the seeds, by internal vertex label
    std::vector<uint32_t> perm(n);
    if (n) GTC_CUDA(cudaMemcpyAsync(perm.data(), g->perm.get(), (size_t)n * 4, cudaMemcpyDeviceToHost, s));
    GTC_CUDA(cudaStreamSynchronize(s));
    std::vector<uint32_t> iperm(n);
    for (uint32_t i = 0; i < n; ++i) iperm[perm[i]] = i;
    std::vector<uint32_t> cnt((size_t)n + 1, 0);
    const uint64_t ns = in.seed_off[B];
    for (uint64_t k = 0; k < ns; ++k) {
        GTC_REQUIRE(in.seed_vertices[k] < n, GTC_ERR_INDEX, "a seed vertex is outside the vertex bound");
        cnt[iperm[in.seed_vertices[k]] + 1]++;
    }
    for (uint32_t v = 0; v < n; ++v) cnt[v + 1] += cnt[v];
    std::vector<uint2> seeds(ns ? ns : 1);
    {
        std::vector<uint32_t> fill(cnt.begin(), cnt.end() - 1);
        for (uint32_t b = 0; b < B; ++b) {
            const uint64_t sb = in.seed_off[b], se = in.seed_off[b + 1];
            GTC_REQUIRE(se >= sb, GTC_ERR_ARG, "seed offsets must not decrease");
            for (uint64_t k = sb; k < se; ++k) {
                const double val = in.seed_values ? in.seed_values[k] : 1.0 / (double)(se - sb);
                const float fv = (float)val;
                seeds[fill[iperm[in.seed_vertices[k]]]++] = make_uint2(b, host_float_bits(fv));
            }
        }
    }
    DevBuf<uint32_t> dso((size_t)n + 1, s);
    DevBuf<uint2> dseeds(seeds.size(), s);
    GTC_CUDA(cudaMemcpyAsync(dso.get(), cnt.data(), ((size_t)n + 1) * 4, cudaMemcpyHostToDevice, s));
    GTC_CUDA(cudaMemcpyAsync(dseeds.get(), seeds.data(), seeds.size() * sizeof(uint2),
                             cudaMemcpyHostToDevice, s));
    // degrees and sinks of the view
    DevBuf<double> deg(n, s);
    DevBuf<uint8_t> sink(n, s);
    if (n) {
        k_degree_ppr<<<grid_for(n, TB, 1u << 30), TB, 0, s>>>(n, view.push_off, view.push_eid,
                                                              in.weight.p, in.weight.dtype,
                                                              deg.get(), sink.get());
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
    PprSchedule sched;
    PprSchedule* S = &sched;
    build_ppr_schedule(view.pull_off, n, s, sched);
    // iterates and per-column state
    const size_t zn = (size_t)n * Bp;
    DevBuf<float> z0(zn, s), z1(zn, s);
    DevBuf<unsigned> ticket(1, s);
    GTC_CUDA(cudaMemsetAsync(ticket.get(), 0, sizeof(unsigned), s));
    if (zn) {
        k_ppr_init<<<grid_for(zn, TB, 1u << 30), TB, 0, s>>>(n, Bp, deg.get(), dso.get(),
                                                             dseeds.get(), z0.get());
        GTC_LAUNCHED();
        L++;
    }
    // dangling mass of the start (the seeds on sinks), on the host
    std::vector<uint8_t> hsink(n);
    if (n) GTC_CUDA(cudaMemcpyAsync(hsink.data(), sink.get(), n, cudaMemcpyDeviceToHost, s));
    GTC_CUDA(cudaStreamSynchronize(s));
    std::vector<double> hps(Bp, 0.0);
    for (uint32_t v = 0; v < n; ++v)
        if (hsink[v])
            for (uint32_t k = cnt[v]; k < cnt[v + 1]; ++k)
                hps[seeds[k].x] += (double)host_bits_float(seeds[k].y);
    DevBuf<double> out(2 * (size_t)Bp, s), psink(Bp, s);
    GTC_CUDA(cudaMemcpyAsync(psink.get(), hps.data(), Bp * sizeof(double), cudaMemcpyHostToDevice, s));
    std::vector<uint8_t> frozen(Bp, 0);
    for (uint32_t b = B; b < Bp; ++b) frozen[b] = 1;  // padding columns never run
    DevBuf<uint8_t> dfrozen(Bp, s);
    const unsigned cap = Bp == 128 ? ppr_grid<4>(Bp) : Bp == 256 ? ppr_grid<8>(Bp)
                       : Bp == 384 ? ppr_grid<12>(Bp) : ppr_grid<16>(Bp);
    const unsigned grid = std::max(1u, std::min(cap, (S->n_rows + PPR_WARPS - 1) / PPR_WARPS +
                                                         S->n_long));
    DevBuf<double> part((size_t)grid * 2 * Bp, s);

    PprArgs A{};
    A.n = n, A.Bp = Bp;
    A.rows = S->rows.get(), A.n_rows = S->n_rows;
    A.longs = S->longs.get(), A.n_long = S->n_long;
    A.off = view.pull_off, A.other = view.pull_other, A.w = wpull.get();
    A.deg = deg.get(), A.sink = sink.get();
    A.seed_off = dso.get(), A.seeds = dseeds.get();
    A.frozen = dfrozen.get();
    A.psink = psink.get();
    A.one_minus_d = (float)(1.0 - d), A.d = (float)d;
    A.part = part.get(), A.ticket = ticket.get(), A.out = out.get();

    std::vector<double> hout(2 * (size_t)Bp);
    std::fill(in.iters, in.iters + B, 0);
    uint32_t running = B;
    uint64_t sweep = 0;
    float *zc = z0.get(), *zx = z1.get();
    Timer_ total(s);
    total.start();
    while (running > 0) {
        GTC_CUDA(cudaMemcpyAsync(dfrozen.get(), frozen.data(), Bp, cudaMemcpyHostToDevice, s));
        A.zprev = zc, A.znext = zx;
        if (Bp == 128)
            launch_ppr<4>(A, grid, s);
        else if (Bp == 256)
            launch_ppr<8>(A, grid, s);
        else if (Bp == 384)
            launch_ppr<12>(A, grid, s);
        else
            launch_ppr<16>(A, grid, s);
        L++;
        SL++;
        GTC_CUDA(cudaMemcpyAsync(hout.data(), out.get(), 2 * Bp * sizeof(double),
                                 cudaMemcpyDeviceToHost, s));
        GTC_CUDA(cudaStreamSynchronize(s));
        ++sweep;
        for (uint32_t b = 0; b < B; ++b) {
            if (frozen[b]) continue;
            in.iters[b] = sweep;
            if (hout[b] < in.params.epsilon ||
                (in.params.max_iter > 0 && sweep == in.params.max_iter)) {
                frozen[b] = 1;
                --running;
            }
        }
        // next sweep's dangling mass per column
        GTC_CUDA(cudaMemcpyAsync(psink.get(), out.get() + Bp, Bp * sizeof(double),
                                 cudaMemcpyDeviceToDevice, s));
        std::swap(zc, zx);
    }
    total.stop();
    res->device_ms = total.ms();
    if (n) {
        dim3 grid2((n + 31) / 32, (Bp + 31) / 32), blk(32, 8);
        k_ppr_store<<<grid2, blk, 0, s>>>(n, B, Bp, g->perm.get(), deg.get(), sink.get(), zc,
                                          in.out, in.out_dtype);
        GTC_LAUNCHED();
        L++;
    }
    GTC_CUDA(cudaStreamSynchronize(s));
    res->iterations = sweep;
    res->last_delta = 0.0;
    res->eigenvalue = 0.0;
    res->launches = L;
    res->sweep_ms = 0.0;
    res->sweep_launches = SL;
    g->launches += L;
}

}  // namespace gtc
