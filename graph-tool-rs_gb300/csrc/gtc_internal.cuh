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
    DevBuf<double2> long_out;    // per long row: its epilogue's reduction terms
    DevBuf<double2> item_out;    // per work item: its rows' reduction terms
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
    bool operator==(const BatchKey& o) const {
        return w == o.w && wdt == o.wdt && out == o.out && odt == o.odt && d == o.d &&
               eps == o.eps && max_iter == o.max_iter;
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
    cudaStream_t side = nullptr;             // the global queue's stream while captured
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
    gtc_graph(uint32_t n_, uint32_t m_) : n(n_), m(m_) {}
    int device = 0;
    uint32_t n = 0;  // vertex bound
    uint32_t m = 0;  // edge bound == live edges (ids 0..m-1)
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
    gtc::PprSched ppr_sched[2];      // batched schedules of the plain and reversed views
    gtc::DevBuf<float> ppr_z[2];     // batched iterates, kept between calls (grown on demand)
    uint64_t launches = 0;  // kernels this handle has launched (diagnostics)
};

namespace gtc {

// graph build (gtc_build.cu)
void build_halves(gtc_graph* g, const uint32_t* d_src, const uint32_t* d_tgt, bool relabel = true);
void build_schedule(gtc_graph* g, bool in_dir, uint32_t cap);

// A device vector of either float type.
struct DVec {
    const void* p = nullptr;
    uint64_t len = 0;
    int dtype = GTC_F64;
    bool present() const { return p != nullptr; }
};

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
