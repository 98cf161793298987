// gtc_internal.cuh -- shared internals of libgtc (CUDA, sm_103a).
//
// Everything here is private to the library: the public surface is the C ABI
// in include/gtc.h.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "gtc.h"

namespace gtc {

// --------------------------------------------------------------------------
// errors
// --------------------------------------------------------------------------

// Per-thread message of the last failing call (gtc_last_error()).
void set_error(const std::string& msg);

// Throws GTC_ERR_NO_DEVICE unless a CUDA device is usable (and makes its
// context current).
void require_device();

struct Error {
    int status;
    std::string msg;
};

#define GTC_CUDA(call)                                                              \
    do {                                                                            \
        cudaError_t e_ = (call);                                                    \
        if (e_ != cudaSuccess)                                                      \
            throw ::gtc::Error{GTC_ERR_CUDA, std::string(#call) + ": " +            \
                                                 cudaGetErrorString(e_)};           \
    } while (0)

#define GTC_REQUIRE(cond, status, msg)                                              \
    do {                                                                            \
        if (!(cond)) throw ::gtc::Error{(status), (msg)};                           \
    } while (0)

// Launch check: a launch error is reported, a pending asynchronous fault is
// left for the next synchronising call to report.
#define GTC_LAUNCHED() GTC_CUDA(cudaGetLastError())

// --------------------------------------------------------------------------
// device buffers
// --------------------------------------------------------------------------

// A stream-ordered device allocation released when the owner goes out of
// scope.  Graph-lifetime arrays and per-call scratch both use it.
template <class T>
struct DevBuf {
    T* p = nullptr;
    size_t n = 0;
    cudaStream_t s = nullptr;
    DevBuf() = default;
    DevBuf(size_t count, cudaStream_t stream) { alloc(count, stream); }
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    DevBuf(DevBuf&& o) noexcept : p(o.p), n(o.n), s(o.s) { o.p = nullptr, o.n = 0; }
    DevBuf& operator=(DevBuf&& o) noexcept {
        if (this != &o) {
            release();
            p = o.p, n = o.n, s = o.s;
            o.p = nullptr, o.n = 0;
        }
        return *this;
    }
    void alloc(size_t count, cudaStream_t stream) {
        release();
        s = stream;
        n = count;
        size_t bytes = (count ? count : 1) * sizeof(T);
        cudaError_t e = cudaMallocAsync((void**)&p, bytes, s);
        if (e != cudaSuccess) {
            p = nullptr;
            (void)cudaGetLastError();
            throw Error{e == cudaErrorMemoryAllocation ? GTC_ERR_OOM : GTC_ERR_CUDA,
                        std::string("device allocation of ") + std::to_string(bytes) +
                            " bytes failed: " + cudaGetErrorString(e)};
        }
    }
    void release() {
        if (p) cudaFreeAsync(p, s);
        p = nullptr;
        n = 0;
    }
    ~DevBuf() { release(); }
    T* get() const { return p; }
    size_t bytes() const { return n * sizeof(T); }
};

// --------------------------------------------------------------------------
// graph
// --------------------------------------------------------------------------

// One direction of the adjacency, flattened: the block halves of every vertex
// in storage order.  off has n+1 entries; other/eid have m.
struct Halves {
    DevBuf<uint32_t> off, other, eid;
};

// Pull schedule of one half (gtc_sweep.cuh): rows split into sliced rows,
// medium rows and long rows, and the work list over them.
struct Units {
    DevBuf<uint4> units;         // the work list
    DevBuf<uint4> longs;         // per long row: {row, first chunk slot, chunks, 0}
    DevBuf<float2> partial;      // per long chunk: compensated partial (s, c)
    DevBuf<unsigned> counter;    // per long row: chunks done (reset by the last)
    DevBuf<uint4> fold_part;     // per CTA of a sweep: its exact (a, b) partials
    DevBuf<uint32_t> med;        // medium rows
    DevBuf<uint32_t> slice_rows; // 32 rows per slice (NO_ROW pads)
    DevBuf<uint32_t> slice_off;  // first sliced entry of each slice, n_slices + 1
    DevBuf<uint32_t> sidx;       // sliced entries: source vertex (n pads)
    DevBuf<uint32_t> seid;       // sliced entries: edge id (0xFFFFFFFF pads)
    uint32_t n_units = 0, n_long = 0, n_chunks = 0, n_med = 0, n_slices = 0;
    uint32_t n_sliced = 0;       // sliced entries including padding
    int variant[3][2] = {{-1, -1}, {-1, -1}, {-1, -1}};  // tuned kernel variant [mode][weighted]
    bool built = false;
};

// FP32 edge weights laid out for the sweeps, kept on the handle between
// solves (gtc_centrality.cu): the caller's weight map by EdgeId is gathered
// into the storage order of the in-halves and the out-halves, into the
// sliced entries of each pull schedule, and summed into weighted degrees,
// once; later solves with the same map reuse them.  The key is the map's
// address, dtype and a 64-bit hash of its contents (one sequential read per
// solve), so a map changed in place is gathered again.
struct WeightCache {
    const void* ptr = nullptr;
    int dtype = -1;
    unsigned long long hash = 0;
    bool valid = false;
    DevBuf<float> half[2];      // [0] in-half order, [1] out-half order
    DevBuf<float> sliced[2];    // sliced entries of units_in [0] / units_out [1]
    DevBuf<double> deg[2];      // weighted degree over the in-halves [0] / out-halves [1]
    DevBuf<uint8_t> sink[2];    // zero weighted degree
    DevBuf<float> invdeg[2];    // FP32 inverse of deg (0 on the sinks)
    void reset() {
        for (int h = 0; h < 2; ++h) half[h].release(), sliced[h].release(), deg[h].release(),
                                    sink[h].release(), invdeg[h].release();
        valid = false;
    }
};

// Degrees of the unweighted, unfiltered views over the in-halves [0] (the
// reversed view's out-degree) and the out-halves [1] (the plain view's):
// they depend on the graph alone, so the handle keeps them.
struct DegCache {
    DevBuf<double> deg[2];      // out-degree of the view, FP64
    DevBuf<uint8_t> sink[2];    // out-degree 0
    DevBuf<float> invdeg[2];    // FP32 inverse of deg (0 on the sinks)
};

// Pull schedule of the batched personalised PageRank (gtc_ppr.cu): rows with
// more in-edges than one chunk are cut into chunks, the rest are rows of
// their own, heaviest first.
struct PprSched {
    // work items: the chunks {row, first entry, end entry, long row index},
    // then the single rows {row, first entry, end entry, 0xFFFFFFFF} by
    // descending in-degree (ties by index)
    DevBuf<uint4> items;
    DevBuf<uint4> longs;    // {row, first chunk, chunks, 0}
    uint32_t n_items = 0, n_chunks = 0, n_long = 0;
    uint32_t n_empty = 0;  // single rows without pull entries (the last items)
    uint32_t n_heavy = 0;  // chunks and single rows of at least 64 pull entries (the first items)
    bool built = false;
};

}  // namespace gtc

namespace gtc {
// What a captured batch solve depends on besides the graph (gtc_batch.cu).
struct BatchKey {
    const void* w = nullptr;
    int wdt = -1;
    void* out = nullptr;
    int odt = -1;
    double d = 0.0, eps = 0.0;
    uint64_t max_iter = 0;
    uint64_t sweep_limit = 0;
    bool operator==(const BatchKey& o) const {
        return w == o.w && wdt == o.wdt && out == o.out && odt == o.odt && d == o.d &&
               eps == o.eps && max_iter == o.max_iter && sweep_limit == o.sweep_limit;
    }
};
}  // namespace gtc

struct gtc_graph;

// Many graphs packed as one block-diagonal graph (gtc_batch.cu): graph k owns
// vertices [voff[k], voff[k+1]) of the union `u`, whose labels are kept.
namespace gtc {
// Most vertices whose gathered vector (4 bytes each) one CTA of the batch
// kernels holds in shared memory: a graph of up to GB_CL_CAP vertices is
// solved by one CTA, one of up to 2 * GB_CL_CAP by a cluster of two.
constexpr uint32_t GB_CL_CAP = 57344;
// Longest row kept in the batch's 32-row slices; longer rows are summed by a
// whole warp.
constexpr uint32_t GB_SL_CAP = 128;
// The batch's rows are ordered by in-degree only inside windows of this many
// consecutive labels of their graph, which keeps the input's locality.
constexpr uint32_t GB_WIN = 1024;
}  // namespace gtc

struct gtc_graph_batch {
    gtc_graph* u = nullptr;
    uint32_t G = 0;
    std::vector<uint32_t> hvoff, heoff;      // host copies, G + 1 each
    // order: the n_pair graphs of GB_CL_CAP + 1 .. 2 * GB_CL_CAP vertices,
    // the n_single of at most GB_CL_CAP, then the n_global larger ones; each
    // queue by descending edges + vertices
    gtc::DevBuf<uint32_t> voff, order;
    // Layout (batch_layout, gtc_batch.cu).  Inside each graph the vertices
    // are relabelled: rows of more than GB_SL_CAP in-edges first, the others
    // by descending in-degree inside windows of GB_WIN labels; vperm[new] =
    // packed label.  A graph's first glong[g] rows keep their pull entries
    // in CSR order from gebase[g]; the others form slices of 32 rows, gsl[g]
    // .. gsl[g+1]-1, each stored column-major from sl_off[s] (entry j of lane
    // i at sl_off[s] + 32*j + i; short lanes padded).
    gtc::DevBuf<uint32_t> vperm, glong, gsl, gebase, sl_off;
    gtc::DevBuf<uint32_t> eidx, eeid;         // layout entries: source, edge id (pads ~0u)
    gtc::DevBuf<float> wlay;                  // weights in layout order
    uint64_t n_lay = 0;
    uint32_t n_pair = 0, n_single = 0, n_global = 0;
    uint32_t smem_floats = 0;                // x entries a CTA of the first two queues holds
    gtc::DevBuf<float> invdeg, r0, r1, y0, y1, wout;
    gtc::DevBuf<uint8_t> sink;
    gtc::DevBuf<uint64_t> iters;
    gtc::DevBuf<unsigned> counter;
    gtc::DevBuf<double> wstage, rstage;      // host-API staging
    cudaGraphExec_t exec = nullptr;          // the captured solve
    gtc::BatchKey key{};
    uint64_t launches_per_solve = 0;
};

struct gtc_graph {
    gtc_graph() = default;
    gtc_graph(uint32_t n_, uint32_t m_) : n(n_), m(m_), m_live(m_) {}
    int device = 0;
    uint32_t n = 0;       // vertex bound
    uint32_t m = 0;       // edge bound: edge ids are below it (weight maps hold m entries)
    uint32_t m_live = 0;  // live edges: the entries of each half (m unless ids have holes)
    cudaStream_t home = nullptr;    // owned; graph-lifetime buffers live on it
    cudaStream_t stream = nullptr;  // where solves run (home, or the caller's)
    // Internally vertices are relabelled by descending out-degree (ties by
    // index), which packs the most-gathered entries of a pull together.
    // perm[new] = old, iperm[old] = new.  Both halves are stored in the new
    // labels; every entry keeps its position inside its block.
    gtc::DevBuf<uint32_t> perm, iperm;
    gtc::Halves out;  // CSR: out-halves (out_edges order)
    gtc::Halves in;   // CSC: in-halves (in_edges order, the pull order)
    gtc::Units units_in, units_out;  // pull schedules of the plain and reversed views
    gtc::WeightCache wcache;         // FP32 weight layouts of the last weight map used
    gtc::DegCache dcache;            // unweighted degrees of the plain and reversed views
    gtc::PprSched ppr_sched[2];      // batched schedules of the plain and reversed views
    gtc::DevBuf<float> ppr_z[2];     // batched iterates, kept between calls (grown on demand)
    uint64_t launches = 0;  // kernels this handle has launched (diagnostics)
};

namespace gtc {

// graph build (gtc_build.cu)
void build_halves(gtc_graph* g, const uint32_t* d_src, const uint32_t* d_tgt, bool relabel = true);
void build_schedule(gtc_graph* g, bool in_dir, uint32_t cap);
// A graph from the reference's blocks as stored (gtc_graph_create_blocks).
void build_from_blocks(gtc_graph* g, const uint64_t* block_off, const uint32_t* out_len,
                       const uint32_t* entries);
void relabel_graph(gtc_graph* g, const uint32_t* src_of, const uint32_t* tgt_of, bool relabel,
                   uint64_t* launches);

// A device vector of either float type.
struct DVec {
    const void* p = nullptr;
    uint64_t len = 0;
    int dtype = GTC_F64;
    bool present() const { return p != nullptr; }
};

// One read of a weight map by EdgeId: its content hash; GTC_ERR_ARG if it
// holds a non-finite value (gtc_centrality.cu).
unsigned long long scan_weights(const DVec& w, uint64_t m, cudaStream_t s, uint64_t* launches);


// One solve's inputs, after the C ABI checked them.  Every vector is in
// device memory.
struct SolveIn {
    DVec weight;                 // by EdgeId, or absent (Unity)
    DVec pers;                   // by vertex index, or absent (uniform)
    double damping = 0.85;
    gtc_power_iteration params;  // plan_chunks resolved (never 0)
    void* x = nullptr;           // initial iterate and output
    int x_dtype = GTC_F64;
    uint64_t had = 0;            // slots the caller's map already had
    int precision = GTC_PREC_F32;
    int schedule = GTC_SCHED_AUTO;  // gtc_schedule: the FP32 sweep kernel, or the autotuner
    bool timing = false;
};

__device__ __forceinline__ double ld_any(const void* p, int dtype, size_t i) {
    return dtype == GTC_F64 ? ((const double*)p)[i] : (double)((const float*)p)[i];
}

// The same as FP32: an FP32 input is read as is, so no conversion runs on
// the FP64 pipe (on this GPU a conversion per element costs more than the
// element's memory traffic).
__device__ __forceinline__ float ld_f32(const void* p, int dtype, size_t i) {
    return dtype == GTC_F64 ? (float)((const double*)p)[i] : ((const float*)p)[i];
}

// batches of graphs (gtc_batch.cu)
void batch_layout(gtc_graph_batch* b, uint32_t* d_src, uint32_t* d_tgt, cudaStream_t s);
void pagerank_batch(gtc_graph_batch* b, const DVec& weight, double damping, double epsilon,
                    uint64_t max_iter, void* out, int out_dtype, uint64_t* iters, bool timing,
                    gtc_result* res, cudaStream_t s);

// Inputs of the PageRank adjoint (device vectors, original labels).
struct AdjointIn {
    DVec weight, pers;           // as the forward solve
    double damping = 0.85;
    gtc_power_iteration params;  // epsilon / max_iter of the adjoint iteration
    DVec pi;                     // the converged forward result
    DVec gpi;                    // dL/dpi
    void* grad_w = nullptr;      // out: dL/dw by EdgeId (may be null)
    int grad_w_dtype = GTC_F64;
    void* grad_p = nullptr;      // out: dL/dpers by vertex (may be null)
    int grad_p_dtype = GTC_F64;
    bool timing = false;
};

// Inputs of a batch of personalised PageRanks (gtc_ppr.cu).
struct PprIn {
    DVec weight;                      // by EdgeId, device, or absent (Unity)
    uint32_t B = 0;                   // personalisation vectors
    const uint64_t* seed_off = nullptr;       // host, B + 1
    const uint32_t* seed_vertices = nullptr;  // host, original labels
    const double* seed_values = nullptr;      // host, or null: 1/|set|
    double damping = 0.85;
    gtc_power_iteration params;
    void* out = nullptr;              // device [B][n] ranks (original labels)
    int out_dtype = GTC_F64;
    uint64_t* iters = nullptr;        // host, B: sweeps of every column
    int gather = GTC_PPR_BULK;        // gtc_ppr_gather
    bool timing = false;
};
void ppr_batch(gtc_graph* g, const gtc_view* vw, const PprIn& in, gtc_result* res,
               cudaStream_t s);

// One read of a weight map by EdgeId: its content hash; GTC_ERR_ARG if it
// holds a non-finite value (gtc_centrality.cu).
unsigned long long scan_weights(const DVec& w, uint64_t m, cudaStream_t s, uint64_t* launches);

// solves (gtc_centrality.cu)
void pagerank_adjoint(gtc_graph* g, const gtc_view* vw, const AdjointIn& in, gtc_result* res,
                      cudaStream_t s);
// Weighted out- or in-degree of every vertex of a view (host arrays).
void weighted_degree(gtc_graph* g, const gtc_view* vw, const double* w_host, bool in_dir,
                     double* deg_host, cudaStream_t s);
// Brandes betweenness of a view (gtc_betweenness.cu); host output arrays
// (vertex bound / edge bound entries), either may be null.
void betweenness(gtc_graph* g, const gtc_view* vw, bool undirected, double* vb_host,
                 double* eb_host, gtc_result* res, cudaStream_t s);
void pagerank(gtc_graph* g, const gtc_view* vw, const SolveIn& in, gtc_result* res,
              cudaStream_t s);
void eigenvector(gtc_graph* g, const gtc_view* vw, const SolveIn& in, gtc_result* res,
                 cudaStream_t s);

// Stable sort of the positions 0..n-1 by keys[] (every key < key_bound):
// keys_out gets the sorted keys, vals_out the positions (gtc_build.cu).
void sort_positions_by_key(const uint32_t* keys, size_t n, uint32_t key_bound,
                           uint32_t* keys_out, uint32_t* vals_out, cudaStream_t s,
                           uint64_t* launches);

// scans (gtc_build.cu): exclusive scan of n u32 values into out[0..n],
// out[n] = total.  `out` may alias `in` only if the caller passes the same
// pointer for both.
void scan_exclusive_u32(const uint32_t* in, uint32_t* out, size_t n, cudaStream_t s,
                        uint64_t* launches);

// --------------------------------------------------------------------------
// device helpers
// --------------------------------------------------------------------------

// Knuth's TwoSum: s + e == a + b exactly (round-to-nearest).
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// Compensated (Kahan-Babuska / Neumaier) accumulator in f32.
struct Kahan {
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void add(float x) {
        float t, e;
        two_sum(s, x, t, e);
        s = t;
        c = __fadd_rn(c, e);
    }
    // merge another compensated partial
    __device__ __forceinline__ void merge(float os, float oc) {
        float t, e;
        two_sum(s, os, t, e);
        s = t;
        c = __fadd_rn(c, __fadd_rn(oc, e));
    }
    __device__ __forceinline__ float value() const { return __fadd_rn(s, c); }
};

// Compensated sum of a long run of terms.  One (s, c) pair over many terms
// of similar size collects a systematic rounding error in c, and c, itself
// summed plainly, then loses about (terms x ulp(c)): 114,687 equal terms of
// 4.7e-6 lose 4e-7 of their 0.54.  Merging the pair of every block of
// KB_BLOCK terms into an outer pair keeps c small.  Up to KB_BLOCK terms the
// result is the single pair's, bit for bit.
constexpr uint32_t KB_BLOCK = 256;

struct KahanBlocked {
    Kahan outer, inner;
    uint32_t k = 0;
    __device__ __forceinline__ void add(float x) {
        inner.add(x);
        if (++k == KB_BLOCK) {
            outer.merge(inner.s, inner.c);
            inner = Kahan();
            k = 0;
        }
    }
    __device__ __forceinline__ Kahan fold() const {
        Kahan r = outer;
        r.merge(inner.s, inner.c);
        return r;
    }
};

__device__ __forceinline__ void warp_merge_kahan(Kahan& k) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        float os = __shfl_xor_sync(0xffffffffu, k.s, o);
        float oc = __shfl_xor_sync(0xffffffffu, k.c, o);
        k.merge(os, oc);
    }
}

// Exact sum of FP32 terms in 128-bit fixed point: the value is X * 2^-FRAC
// with X a two's-complement integer in four 32-bit words (w0 lowest).  A
// term x is added as the integer m * 2^(e - 150 + FRAC) (m the 24-bit
// significand, e the biased exponent), which is exact for |x| >= 2^(23 -
// FRAC) and truncated toward zero below; |x| must stay below 2^(127 -
// FRAC).  Integer addition is associative, so a sum does not depend on
// the order of its terms or on how partial sums are grouped: every thread,
// warp and CTA schedule gives the same bits.  The words add with the
// carry chain of add.cc/addc (no FP64 pipe, which is slow on this GPU).
template <int FRAC>
struct Exact128 {
    uint32_t w0 = 0u, w1 = 0u, w2 = 0u, w3 = 0u;

    __device__ __forceinline__ void add_words(uint32_t t0, uint32_t t1, uint32_t t2, uint32_t t3) {
        asm("add.cc.u32 %0, %0, %4;\n\t"
            "addc.cc.u32 %1, %1, %5;\n\t"
            "addc.cc.u32 %2, %2, %6;\n\t"
            "addc.u32 %3, %3, %7;"
            : "+r"(w0), "+r"(w1), "+r"(w2), "+r"(w3)
            : "r"(t0), "r"(t1), "r"(t2), "r"(t3));
    }
    __device__ __forceinline__ void sub_words(uint32_t t0, uint32_t t1, uint32_t t2, uint32_t t3) {
        asm("sub.cc.u32 %0, %0, %4;\n\t"
            "subc.cc.u32 %1, %1, %5;\n\t"
            "subc.cc.u32 %2, %2, %6;\n\t"
            "subc.u32 %3, %3, %7;"
            : "+r"(w0), "+r"(w1), "+r"(w2), "+r"(w3)
            : "r"(t0), "r"(t1), "r"(t2), "r"(t3));
    }
    __device__ __forceinline__ void add(float x) {
        const uint32_t b = __float_as_uint(x);
        const uint32_t e = (b >> 23) & 0xFFu;
        const uint32_t m = (b & 0x7FFFFFu) | (e ? 0x800000u : 0u);
        // value = m * 2^(max(e,1) - 150); as an integer of the format, m << s
        const int s = (int)(e ? e : 1u) - 150 + FRAC;
        uint32_t t0 = 0u, t1 = 0u, t2 = 0u, t3 = 0u;
        if (s < 0) {
            t0 = s > -32 ? m >> (-s) : 0u;
        } else {
            const int wi = s >> 5, bi = s & 31;
            const uint32_t lo = m << bi, hi = bi ? m >> (32 - bi) : 0u;
            t0 = wi == 0 ? lo : 0u;
            t1 = wi == 1 ? lo : (wi == 0 ? hi : 0u);
            t2 = wi == 2 ? lo : (wi == 1 ? hi : 0u);
            t3 = wi == 3 ? lo : (wi == 2 ? hi : 0u);
        }
        if (b >> 31)
            sub_words(t0, t1, t2, t3);
        else
            add_words(t0, t1, t2, t3);
    }
    __device__ __forceinline__ void merge(const Exact128& o) { add_words(o.w0, o.w1, o.w2, o.w3); }
    // Sum over the warp (every lane gets it).
    __device__ __forceinline__ void warp_merge() {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            Exact128 p;
            p.w0 = __shfl_xor_sync(0xffffffffu, w0, o);
            p.w1 = __shfl_xor_sync(0xffffffffu, w1, o);
            p.w2 = __shfl_xor_sync(0xffffffffu, w2, o);
            p.w3 = __shfl_xor_sync(0xffffffffu, w3, o);
            merge(p);
        }
    }
    // The value, rounded to FP64 (a fixed function of the bits).
    __device__ double value() const {
        const bool neg = (w3 >> 31) != 0u;
        uint32_t a0 = w0, a1 = w1, a2 = w2, a3 = w3;
        if (neg) {  // magnitude of the two's complement
            a0 = ~a0, a1 = ~a1, a2 = ~a2, a3 = ~a3;
            uint64_t c = (uint64_t)a0 + 1u;
            a0 = (uint32_t)c;
            c = (uint64_t)a1 + (c >> 32);
            a1 = (uint32_t)c;
            c = (uint64_t)a2 + (c >> 32);
            a2 = (uint32_t)c;
            a3 = a3 + (uint32_t)(c >> 32);
        }
        const double hi = (double)(((uint64_t)a3 << 32) | a2);
        const double lo = (double)(((uint64_t)a1 << 32) | a0);
        const double v = (hi * 18446744073709551616.0 + lo) * ldexp(1.0, -FRAC);
        return neg ? -v : v;
    }
};

// Exact fixed-point formats of the sweeps' reductions: PageRank and adjoint
// terms (changes of ranks, dangling mass) are far below 2^31, resolved to
// 2^-96; eigenvector norms (squares of row sums, up to the square of the
// largest weighted in-degree) are resolved to 2^-64 below 2^63.
using ExactPR = Exact128<96>;
using ExactEV = Exact128<64>;

// Where a kernel's two exact sums go: one pair of partials per CTA, summed by
// the last CTA to finish into *out_a, *out_b (FP64).
struct ExactFold {
    uint4* part;       // 2 x gridDim.x
    unsigned* ticket;  // zero before the launch; the last CTA resets it
    double* out_a;
    double* out_b;
    // Optional device-side stop of a power iteration (out_a is the sweep's
    // L1 change): the last CTA counts the sweep in *iters and sets *stop once
    // the change is not >= eps (the reference's `while delta >= epsilon`) or
    // *iters reaches max_iter (0 = no cap).  Kernels of later sweeps read
    // *stop and return at once.
    unsigned* stop = nullptr;
    unsigned long long* iters = nullptr;
    double eps = 0.0;
    unsigned long long max_iter = 0;
};

// Capacity of the per-CTA partials of an ExactFold (every grid is capped to it).
constexpr unsigned FOLD_MAX_CTAS = 4096;

// CTA of NT threads, every thread passing its (a, b): the CTA's sums go to
// part[2 * blockIdx.x + {0, 1}], and the last CTA adds all of them.  The
// totals are exact, so they do not depend on the grid or on which thread
// summed which terms.
template <int NT, class E>
__device__ __forceinline__ void block_fold_exact(E a, E b, const ExactFold& f) {
    __shared__ uint4 fa[NT / 32], fb[NT / 32];
    __shared__ bool last;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    a.warp_merge();
    b.warp_merge();
    if (lane == 0) {
        fa[warp] = make_uint4(a.w0, a.w1, a.w2, a.w3);
        fb[warp] = make_uint4(b.w0, b.w1, b.w2, b.w3);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        E ta, tb;
        for (int w = 0; w < NT / 32; ++w) {
            ta.add_words(fa[w].x, fa[w].y, fa[w].z, fa[w].w);
            tb.add_words(fb[w].x, fb[w].y, fb[w].z, fb[w].w);
        }
        f.part[2 * blockIdx.x] = make_uint4(ta.w0, ta.w1, ta.w2, ta.w3);
        f.part[2 * blockIdx.x + 1] = make_uint4(tb.w0, tb.w1, tb.w2, tb.w3);
        __threadfence();
        last = atomicAdd(f.ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (last && warp == 0) {
        __threadfence();
        E ta, tb;
        for (unsigned i = lane; i < gridDim.x; i += 32) {
            const uint4 pa = __ldcg(f.part + 2 * i), pb = __ldcg(f.part + 2 * i + 1);
            ta.add_words(pa.x, pa.y, pa.z, pa.w);
            tb.add_words(pb.x, pb.y, pb.z, pb.w);
        }
        ta.warp_merge();
        tb.warp_merge();
        if (lane == 0) {
            const double a = ta.value();
            *f.out_a = a;
            *f.out_b = tb.value();
            *f.ticket = 0u;
            if (f.stop) {
                const unsigned long long it = *f.iters + 1;
                *f.iters = it;
                if (!(a >= f.eps) || (f.max_iter && it == f.max_iter)) *f.stop = 1u;
            }
        }
    }
}

__device__ __forceinline__ double warp_sum_f64(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Streaming multiprocessors of the current device (queried once per device);
// persistent grids are sized from it.
int sm_count();

inline unsigned grid_for(size_t work, unsigned per_block, unsigned cap = 1u << 20) {
    size_t b = (work + per_block - 1) / per_block;
    if (b < 1) b = 1;
    if (b > cap) b = cap;
    return (unsigned)b;
}

}  // namespace gtc
