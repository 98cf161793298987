// gtc_batch.cu -- PageRank of many graphs of uneven sizes in one launch.
//
// The graphs are packed as one block-diagonal graph (their disjoint union in
// input order: graph k owns vertices [voff[k], voff[k+1]) and edges
// [eoff[k], eoff[k+1])), built with the reference's block layout and its
// labels kept, so every graph's rows and in-edges are contiguous.  Each graph
// is pagerank (crates/gt-algo/src/centrality.rs:234-248) on that graph alone:
// uniform personalisation 1/n_k, its own dangling mass, its own L1 change
// and its own stop (the first sweep whose change is below epsilon).
//
// One persistent kernel solves them all: a CTA takes the next graph (largest
// first, through an atomic work counter) and runs its whole power iteration
// -- sweeps separated by __syncthreads only, no grid-wide barrier -- before
// it takes another.  A graph is solved by one CTA with a fixed row
// assignment and fixed-order folds, so its result does not depend on which
// CTA took it.  The solve's launches (degrees, weight gathers, the kernel)
// are captured once into a CUDA graph and replayed while the inputs keep
// their addresses.
#include <algorithm>
#include <cstring>
#include <vector>

#include "gtc_view.cuh"

namespace gtc {
namespace {

constexpr int GB_NT = 512;
constexpr int GB_WARPS = GB_NT / 32;

struct GbArgs {
    uint32_t G;
    const uint32_t* __restrict__ order;  // graphs, largest first
    const uint32_t* __restrict__ voff;   // G + 1
    const uint32_t* __restrict__ off;    // in-halves (pull)
    const uint32_t* __restrict__ other;
    const float* __restrict__ w;         // pull-ordered weights, or null
    const float* __restrict__ invdeg;
    const uint8_t* __restrict__ sink;
    float* r0;
    float* r1;
    float* y0;
    float* y1;
    float one_minus_d, d;
    double epsilon;
    uint64_t max_iter;
    void* out;
    int out_dtype;
    uint64_t* iters;     // per graph
    unsigned* counter;   // work counter (reset by the host)
};

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

template <bool W>
__global__ void __launch_bounds__(GB_NT) k_pr_graphs(GbArgs A) {
    __shared__ double2 sm[GB_WARPS + 1];
    __shared__ uint32_t s_graph;
    for (;;) {
        if (threadIdx.x == 0) s_graph = atomicAdd(A.counter, 1u);
        __syncthreads();
        const uint32_t k = s_graph;
        __syncthreads();
        if (k >= A.G) return;
        const uint32_t gk = A.order[k];
        const uint32_t vb = A.voff[gk], ve = A.voff[gk + 1];
        const uint32_t nk = ve - vb;
        const float u = nk ? (float)(1.0 / (double)nk) : 0.f;
        // the uniform start and its dangling mass
        Kahan ks, kz;
        for (uint32_t v = vb + threadIdx.x; v < ve; v += GB_NT) {
            A.r0[v] = u;
            A.y0[v] = __fmul_rn(u, A.invdeg[v]);
            if (A.sink[v]) ks.add(u);
        }
        double psink = cta_sum2(ks, kz, sm).x;
        float *rc = A.r0, *rn = A.r1, *yc = A.y0, *yn = A.y1;
        uint64_t it = 0;
        for (;;) {
            const float ps = (float)psink;
            Kahan kd, kk;
            for (uint32_t v = vb + threadIdx.x; v < ve; v += GB_NT) {
                Kahan acc;
                const uint32_t b = A.off[v], e = A.off[v + 1];
                for (uint32_t p = b; p < e; ++p) {
                    const float x = yc[A.other[p]];
                    acc.add(W ? __fmul_rn(x, A.w[p]) : x);
                }
                const float r = __fadd_rn(__fmul_rn(ps, u), acc.value());
                const float nv = __fadd_rn(__fmul_rn(A.one_minus_d, u), __fmul_rn(A.d, r));
                rn[v] = nv;
                yn[v] = __fmul_rn(nv, A.invdeg[v]);
                kd.add(fabsf(__fsub_rn(nv, rc[v])));
                if (A.sink[v]) kk.add(nv);
            }
            const double2 t = cta_sum2(kd, kk, sm);  // also orders this sweep's writes
            ++it;
            float* tr = rc;
            rc = rn, rn = tr;
            float* ty = yc;
            yc = yn, yn = ty;
            psink = t.y;
            if (t.x < A.epsilon || (A.max_iter > 0 && it == A.max_iter)) break;
        }
        for (uint32_t v = vb + threadIdx.x; v < ve; v += GB_NT) {
            if (A.out_dtype == GTC_F64)
                ((double*)A.out)[v] = (double)rc[v];
            else
                ((float*)A.out)[v] = rc[v];
        }
        if (threadIdx.x == 0) A.iters[gk] = it;
        __syncthreads();
    }
}

__global__ void k_gb_gather(uint32_t m, const uint32_t* __restrict__ eid, const void* __restrict__ w,
                            int wdt, float* __restrict__ out) {
    const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p < m) out[p] = ld_f32(w, wdt, eid[p]);
}

// weighted out-degree (8 lanes per vertex, compensated, fixed merge order) or
// the plain out-degree; its FP32 inverse and the sink flags
__global__ void k_gb_degree(uint32_t n, const uint32_t* __restrict__ push_off,
                            const float* __restrict__ wout, float* __restrict__ invdeg,
                            uint8_t* __restrict__ sink) {
    const uint32_t sub = threadIdx.x & 7;
    const size_t v = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 3;
    const bool in = v < n;
    Kahan k;
    if (in && wout)
        for (uint32_t p = push_off[v] + sub, e = push_off[v + 1]; p < e; p += 8) k.add(wout[p]);
    for (int o = 4; o > 0; o >>= 1) {
        const float os = __shfl_xor_sync(0xffffffffu, k.s, o, 8);
        const float oc = __shfl_xor_sync(0xffffffffu, k.c, o, 8);
        k.merge(os, oc);
    }
    if (in && sub == 0) {
        const double dg = wout ? (double)k.s + (double)k.c : (double)(push_off[v + 1] - push_off[v]);
        invdeg[v] = dg != 0.0 ? (float)(1.0 / dg) : 0.f;
        sink[v] = dg == 0.0 ? 1 : 0;
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
    b->wpull.alloc(m, h);
    b->iters.alloc(b->G, h);
    b->counter.alloc(1, h);
    GTC_CUDA(cudaStreamSynchronize(h));
    (void)s;
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
                       epsilon, max_iter};
    if (!b->exec || !(b->key == key)) {
        if (b->exec) {
            cudaGraphExecDestroy(b->exec);
            b->exec = nullptr;
        }
        int sms = 0, dev = 0, per_sm = 0;
        GTC_CUDA(cudaGetDevice(&dev));
        GTC_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        GTC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &per_sm, W ? k_pr_graphs<true> : k_pr_graphs<false>, GB_NT, 0));
        const unsigned grid =
            (unsigned)std::max(1, std::min<int>(sms * std::max(per_sm, 1), (int)b->G));
        cudaGraph_t graph = nullptr;
        GTC_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        const unsigned TB = 256;
        if (W && m) {
            k_gb_gather<<<grid_for(m, TB, 1u << 30), TB, 0, s>>>(m, u->out.eid.get(), weight.p,
                                                                 weight.dtype, b->wout.get());
            k_gb_gather<<<grid_for(m, TB, 1u << 30), TB, 0, s>>>(m, u->in.eid.get(), weight.p,
                                                                 weight.dtype, b->wpull.get());
        }
        if (n)
            k_gb_degree<<<grid_for((size_t)n * 8, TB, 1u << 30), TB, 0, s>>>(
                n, u->out.off.get(), W ? b->wout.get() : nullptr, b->invdeg.get(), b->sink.get());
        cudaMemsetAsync(b->counter.get(), 0, sizeof(unsigned), s);
        GbArgs A{};
        A.G = b->G;
        A.order = b->order.get();
        A.voff = b->voff.get();
        A.off = u->in.off.get();
        A.other = u->in.other.get();
        A.w = W ? b->wpull.get() : nullptr;
        A.invdeg = b->invdeg.get();
        A.sink = b->sink.get();
        A.r0 = b->r0.get(), A.r1 = b->r1.get(), A.y0 = b->y0.get(), A.y1 = b->y1.get();
        A.one_minus_d = (float)(1.0 - damping);
        A.d = (float)damping;
        A.epsilon = epsilon;
        A.max_iter = max_iter;
        A.out = out;
        A.out_dtype = out_dtype;
        A.iters = b->iters.get();
        A.counter = b->counter.get();
        if (W)
            k_pr_graphs<true><<<grid, GB_NT, 0, s>>>(A);
        else
            k_pr_graphs<false><<<grid, GB_NT, 0, s>>>(A);
        const cudaError_t ce = cudaStreamEndCapture(s, &graph);
        GTC_CUDA(ce);
        GTC_LAUNCHED();
        const cudaError_t ie = cudaGraphInstantiate(&b->exec, graph, 0);
        cudaGraphDestroy(graph);
        GTC_CUDA(ie);
        b->key = key;
        b->launches_per_solve = (W && m ? 2 : 0) + (n ? 1 : 0) + 1;
    }
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (timing) {
        GTC_CUDA(cudaEventCreate(&e0));
        GTC_CUDA(cudaEventCreate(&e1));
        GTC_CUDA(cudaEventRecord(e0, s));
    }
    GTC_CUDA(cudaGraphLaunch(b->exec, s));
    if (timing) GTC_CUDA(cudaEventRecord(e1, s));
    std::vector<uint64_t> hit(b->G);
    if (b->G)
        GTC_CUDA(cudaMemcpyAsync(hit.data(), b->iters.get(), (size_t)b->G * 8, cudaMemcpyDeviceToHost, s));
    GTC_CUDA(cudaStreamSynchronize(s));
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
}

}  // namespace gtc
