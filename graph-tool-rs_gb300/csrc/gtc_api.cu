// gtc_api.cu -- the C ABI (include/gtc.h): argument checks, error capture,
// handle lifetime.  Every entry point catches everything; nothing unwinds
// into the caller.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <algorithm>
#include <new>

#include "gtc_view.cuh"

namespace gtc {

static thread_local std::string t_err;

void set_error(const std::string& msg) { t_err = msg; }

void require_device() {
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) {
        (void)cudaGetLastError();
        throw Error{GTC_ERR_NO_DEVICE,
                    std::string("no usable CUDA device: ") +
                        (e != cudaSuccess ? cudaGetErrorString(e) : "device count is 0")};
    }
    e = cudaFree(nullptr);  // the device's context exists before any handle is made
    if (e != cudaSuccess)
        throw Error{GTC_ERR_CUDA, std::string("context creation failed: ") + cudaGetErrorString(e)};
    // Solves allocate their scratch from the device's default memory pool
    // (cudaMallocAsync) and free it when they return.  With the pool's
    // default release threshold (0) the freed memory goes back to the driver
    // at the next synchronisation and the next solve maps it again; keeping
    // it in this process's pool makes repeated solves reuse it.
    static bool pool_kept[64] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) == cudaSuccess && dev >= 0 && dev < 64 && !pool_kept[dev]) {
        cudaMemPool_t pool = nullptr;
        if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
            uint64_t keep = UINT64_MAX;
            if (cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep) == cudaSuccess)
                pool_kept[dev] = true;
        }
        (void)cudaGetLastError();
    }
}

int sm_count() {
    static int cached[64] = {};
    int dev = 0;
    GTC_CUDA(cudaGetDevice(&dev));
    if (dev >= 0 && dev < 64 && cached[dev]) return cached[dev];
    int sms = 0;
    GTC_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    if (sms < 1) sms = 1;
    if (dev >= 0 && dev < 64) cached[dev] = sms;
    return sms;
}

template <class F>
static int guarded(F&& f) {
    try {
        f();
        t_err.clear();
        return GTC_OK;
    } catch (const Error& e) {
        t_err = e.msg;
        return e.status;
    } catch (const std::bad_alloc&) {
        t_err = "host allocation failed";
        return GTC_ERR_OOM;
    } catch (...) {
        t_err = "unexpected internal error";
        return GTC_ERR_CUDA;
    }
}

static gtc_graph* new_graph(uint64_t n, uint64_t m) {
    GTC_REQUIRE(n <= 0xFFFFFFFEull, GTC_ERR_ARG,
                "vertex count exceeds the index space (MAX_INDEX = 2^32 - 2)");
    GTC_REQUIRE(m <= 0xFFFFFFFEull, GTC_ERR_ARG,
                "edge count exceeds the index space (MAX_INDEX = 2^32 - 2)");
    require_device();
    gtc_graph* g = new gtc_graph((uint32_t)n, (uint32_t)m);
    cudaError_t e = cudaGetDevice(&g->device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&g->home, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete g;
        throw Error{GTC_ERR_CUDA, std::string("stream creation failed: ") + cudaGetErrorString(e)};
    }
    g->stream = g->home;
    return g;
}

static void destroy_graph(gtc_graph* g) {
    if (!g) return;
    cudaStream_t home = g->home;
    if (g->stream != home) cudaStreamSynchronize(g->stream);
    delete g;  // graph buffers are freed on the home stream
    if (home) {
        cudaStreamSynchronize(home);
        cudaStreamDestroy(home);
    }
}

static void check_params(const gtc_graph* g, const gtc_power_iteration* p, gtc_power_iteration& out) {
    GTC_REQUIRE(p, GTC_ERR_ARG, "params is NULL");
    out = *p;
    GTC_REQUIRE(out.plan_len == g->n, GTC_ERR_ARG, "sweep: the plan must cover the output exactly");
    if (out.plan_chunks == 0) out.plan_chunks = out.plan_len ? (out.plan_len + 4095) / 4096 : 1;
    if (out.plan_chunks == 0) out.plan_chunks = 1;
    GTC_REQUIRE(out.plan_chunks <= (out.plan_len ? out.plan_len : 1), GTC_ERR_ARG,
                "plan has more chunks than items");
    GTC_REQUIRE(!std::isnan(out.epsilon), GTC_ERR_ARG, "epsilon is NaN");
    // The sweeps stop at the first L1 change below epsilon or at max_iter.
    // An L1 change is never negative, so without a cap epsilon <= 0 would
    // never stop (the reference's loop would spin forever); refused here.
    GTC_REQUIRE(out.max_iter != 0 || out.epsilon > 0.0, GTC_ERR_ARG,
                "max_iter = 0 (uncapped) with epsilon <= 0 would never stop");
}

}  // namespace gtc

using namespace gtc;

extern "C" {

const char* gtc_version(void) { return "gtc 0.1.0 (sm_103a)"; }

const char* gtc_last_error(void) { return t_err.c_str(); }

int gtc_graph_create_device(uint64_t n, uint64_t m, const uint32_t* d_src, const uint32_t* d_tgt,
                            void* stream, gtc_graph** out) {
    return guarded([&] {
        GTC_REQUIRE(out, GTC_ERR_ARG, "out is NULL");
        *out = nullptr;
        GTC_REQUIRE(m == 0 || (d_src && d_tgt), GTC_ERR_ARG, "src/tgt is NULL");
        gtc_graph* g = new_graph(n, m);
        try {
            cudaEvent_t ev = nullptr;
            if (stream) {  // the caller's writes of src/tgt happen-before the build
                GTC_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
                GTC_CUDA(cudaEventRecord(ev, (cudaStream_t)stream));
                GTC_CUDA(cudaStreamWaitEvent(g->home, ev, 0));
                cudaEventDestroy(ev);
            }
            build_halves(g, d_src, d_tgt);
        } catch (...) {
            destroy_graph(g);
            throw;
        }
        *out = g;
    });
}

int gtc_graph_create(uint64_t n, uint64_t m, const uint32_t* src, const uint32_t* tgt,
                     gtc_graph** out) {
    return guarded([&] {
        GTC_REQUIRE(out, GTC_ERR_ARG, "out is NULL");
        *out = nullptr;
        GTC_REQUIRE(m == 0 || (src && tgt), GTC_ERR_ARG, "src/tgt is NULL");
        gtc_graph* g = new_graph(n, m);
        try {
            DevBuf<uint32_t> ds(m, g->home), dt(m, g->home);
            if (m) {
                GTC_CUDA(cudaMemcpyAsync(ds.get(), src, m * sizeof(uint32_t), cudaMemcpyHostToDevice,
                                         g->home));
                GTC_CUDA(cudaMemcpyAsync(dt.get(), tgt, m * sizeof(uint32_t), cudaMemcpyHostToDevice,
                                         g->home));
            }
            build_halves(g, ds.get(), dt.get());
        } catch (...) {
            destroy_graph(g);
            throw;
        }
        *out = g;
    });
}

int gtc_graph_create_blocks(uint64_t n, uint64_t edge_bound, const uint64_t* block_off,
                            const uint32_t* out_len, const uint32_t* entries, gtc_graph** out) {
    return guarded([&] {
        GTC_REQUIRE(out, GTC_ERR_ARG, "out is NULL");
        *out = nullptr;
        gtc_graph* g = new_graph(n, edge_bound);
        try {
            build_from_blocks(g, block_off, out_len, entries);
        } catch (...) {
            destroy_graph(g);
            throw;
        }
        *out = g;
    });
}

int gtc_graph_destroy(gtc_graph* g) {
    return guarded([&] { destroy_graph(g); });
}

int gtc_graph_info(const gtc_graph* g, uint64_t* n, uint64_t* edge_bound, uint64_t* num_edges) {
    return guarded([&] {
        GTC_REQUIRE(g, GTC_ERR_ARG, "graph is NULL");
        if (n) *n = g->n;
        if (edge_bound) *edge_bound = g->m;
        if (num_edges) *num_edges = g->m_live;
    });
}

int gtc_graph_export(const gtc_graph* g, uint64_t* out_off, uint32_t* out_other, uint32_t* out_idx,
                     uint64_t* in_off, uint32_t* in_other, uint32_t* in_idx) {
    return guarded([&] {
        GTC_REQUIRE(g, GTC_ERR_ARG, "graph is NULL");
        cudaStream_t s = g->home;
        const size_t n = g->n, m = g->m_live;
        std::vector<uint32_t> perm(n), iperm(n), off(n + 1), other(m), eid(m);
        if (n) GTC_CUDA(cudaMemcpyAsync(perm.data(), g->perm.get(), n * 4, cudaMemcpyDeviceToHost, s));
        GTC_CUDA(cudaStreamSynchronize(s));
        for (size_t i = 0; i < n; ++i) iperm[perm[i]] = (uint32_t)i;
        // one half, back in original labels and original block order
        auto half = [&](const Halves& h, uint64_t* hoff, uint32_t* hother, uint32_t* hidx) {
            if (!hoff && !hother && !hidx) return;
            GTC_CUDA(cudaMemcpyAsync(off.data(), h.off.get(), (n + 1) * 4, cudaMemcpyDeviceToHost, s));
            if (m) {
                GTC_CUDA(cudaMemcpyAsync(other.data(), h.other.get(), m * 4, cudaMemcpyDeviceToHost, s));
                GTC_CUDA(cudaMemcpyAsync(eid.data(), h.eid.get(), m * 4, cudaMemcpyDeviceToHost, s));
            }
            GTC_CUDA(cudaStreamSynchronize(s));
            uint64_t pos = 0;
            for (size_t v = 0; v < n; ++v) {
                if (hoff) hoff[v] = pos;
                const uint32_t i = iperm[v];
                for (uint32_t p = off[i]; p < off[i + 1]; ++p, ++pos) {
                    if (hother) hother[pos] = perm[other[p]];
                    if (hidx) hidx[pos] = eid[p];
                }
            }
            if (hoff) hoff[n] = pos;
        };
        half(g->out, out_off, out_other, out_idx);
        half(g->in, in_off, in_other, in_idx);
    });
}

int gtc_graph_set_stream(gtc_graph* g, void* stream) {
    return guarded([&] {
        GTC_REQUIRE(g, GTC_ERR_ARG, "graph is NULL");
        GTC_CUDA(cudaStreamSynchronize(g->stream));
        GTC_CUDA(cudaStreamSynchronize(g->home));
        g->stream = stream ? (cudaStream_t)stream : g->home;
    });
}

static cudaStream_t stream_of(const gtc_graph* g, const gtc_options* opt) {
    return (opt && opt->stream) ? (cudaStream_t)opt->stream : g->stream;
}

static void common_opts(const gtc_options* opt, SolveIn& in) {
    in.precision = opt ? opt->precision : GTC_PREC_F32;
    in.schedule = opt ? opt->schedule : GTC_SCHED_AUTO;
    in.timing = opt && opt->timing;
    GTC_REQUIRE(in.precision == GTC_PREC_F32 || in.precision == GTC_PREC_F64_EXACT, GTC_ERR_ARG,
                "unknown precision");
    GTC_REQUIRE(in.schedule >= GTC_SCHED_AUTO && in.schedule <= GTC_SCHED_HOT8K, GTC_ERR_ARG,
                "unknown schedule");
}

static DVec dvec_in(const gtc_dvec* v, uint64_t need, const char* what) {
    DVec d;
    if (!v || !v->ptr) return d;
    GTC_REQUIRE(v->dtype == GTC_F64 || v->dtype == GTC_F32, GTC_ERR_ARG,
                std::string(what) + ": unknown dtype");
    GTC_REQUIRE(v->len >= need, GTC_ERR_ARG,
                std::string(what) + " map is shorter than its index bound");
    d.p = v->ptr;
    d.len = v->len;
    d.dtype = v->dtype;
    return d;
}

// Host arrays staged through device buffers around the device solve.
struct HostStage {
    DevBuf<double> w, p, x;
};

static void stage_host(gtc_graph* g, cudaStream_t s, const double* weight, const double* pers,
                       double* x, uint64_t had, SolveIn& in, HostStage& st) {
    const uint32_t n = g->n, m = g->m;
    if (weight) {
        st.w.alloc(m, s);
        if (m) GTC_CUDA(cudaMemcpyAsync(st.w.get(), weight, (size_t)m * 8, cudaMemcpyHostToDevice, s));
        in.weight = DVec{st.w.get(), m, GTC_F64};
    }
    if (pers) {
        st.p.alloc(n, s);
        if (n) GTC_CUDA(cudaMemcpyAsync(st.p.get(), pers, (size_t)n * 8, cudaMemcpyHostToDevice, s));
        in.pers = DVec{st.p.get(), n, GTC_F64};
    }
    st.x.alloc(n, s);
    uint64_t k = std::min<uint64_t>(had, n);
    if (k) GTC_CUDA(cudaMemcpyAsync(st.x.get(), x, (size_t)k * 8, cudaMemcpyHostToDevice, s));
    in.x = st.x.get();
    in.x_dtype = GTC_F64;
    in.had = had;
}

static void unstage_host(gtc_graph* g, cudaStream_t s, double* x, HostStage& st) {
    if (g->n)
        GTC_CUDA(cudaMemcpyAsync(x, st.x.get(), (size_t)g->n * 8, cudaMemcpyDeviceToHost, s));
    GTC_CUDA(cudaStreamSynchronize(s));
}

int gtc_pagerank(gtc_graph* g, const gtc_view* view, const double* weight, uint64_t weight_len,
                 const double* pers, uint64_t pers_len, double damping,
                 const gtc_power_iteration* params, double* rank, uint64_t rank_len,
                 uint64_t rank_had, const gtc_options* opt, gtc_result* result) {
    return guarded([&] {
        GTC_REQUIRE(g, GTC_ERR_ARG, "graph is NULL");
        SolveIn in{};
        check_params(g, params, in.params);
        GTC_REQUIRE(!weight || weight_len >= g->m, GTC_ERR_ARG,
                    "weight map is shorter than the edge bound");
        GTC_REQUIRE(!pers || pers_len >= g->n, GTC_ERR_ARG,
                    "personalisation map is shorter than the vertex bound");
        GTC_REQUIRE(rank || g->n == 0, GTC_ERR_ARG, "rank is NULL");
        GTC_REQUIRE(rank_len >= g->n, GTC_ERR_ARG, "rank map is shorter than the vertex bound");
        GTC_REQUIRE(!std::isnan(damping), GTC_ERR_ARG, "damping is NaN");
        common_opts(opt, in);
        in.damping = damping;
        cudaStream_t s = stream_of(g, opt);
        HostStage st;
        stage_host(g, s, weight, pers, rank, rank_had, in, st);
        gtc_result r{};
        gtc::pagerank(g, view, in, &r, s);
        unstage_host(g, s, rank, st);
        if (result) *result = r;
    });
}

int gtc_weighted_degree(gtc_graph* g, const gtc_view* view, int32_t in_edges, const double* weight,
                        uint64_t weight_len, double* deg, uint64_t deg_len, const gtc_options* opt) {
    return guarded([&] {
        GTC_REQUIRE(g, GTC_ERR_ARG, "graph is NULL");
        GTC_REQUIRE(!weight || weight_len >= g->m, GTC_ERR_ARG,
                    "weight map is shorter than the edge bound");
        GTC_REQUIRE(deg || g->n == 0, GTC_ERR_ARG, "deg is NULL");
        GTC_REQUIRE(deg_len >= g->n, GTC_ERR_ARG, "degree map is shorter than the vertex bound");
        gtc::weighted_degree(g, view, weight, in_edges != 0, deg, stream_of(g, opt));
    });
}

int gtc_betweenness(gtc_graph* g, const gtc_view* view, int32_t undirected, double* vertex_bc,
                    uint64_t vertex_len, double* edge_bc, uint64_t edge_len,
                    const gtc_options* opt, gtc_result* result) {
    return guarded([&] {
        GTC_REQUIRE(g, GTC_ERR_ARG, "graph is NULL");
        GTC_REQUIRE(!vertex_bc || vertex_len >= g->n, GTC_ERR_ARG,
                    "vertex map is shorter than the vertex bound");
        GTC_REQUIRE(!edge_bc || edge_len >= g->m, GTC_ERR_ARG,
                    "edge map is shorter than the edge bound");
        gtc_result r{};
        gtc::betweenness(g, view, undirected != 0, vertex_bc, edge_bc, &r, stream_of(g, opt));
        if (result) *result = r;
    });
}

int gtc_eigenvector(gtc_graph* g, const gtc_view* view, const double* weight, uint64_t weight_len,
                    const gtc_power_iteration* params, double* x, uint64_t x_len, uint64_t x_had,
                    const gtc_options* opt, gtc_result* result) {
    return guarded([&] {
        GTC_REQUIRE(g, GTC_ERR_ARG, "graph is NULL");
        SolveIn in{};
        check_params(g, params, in.params);
        GTC_REQUIRE(!weight || weight_len >= g->m, GTC_ERR_ARG,
                    "weight map is shorter than the edge bound");
        GTC_REQUIRE(x || g->n == 0, GTC_ERR_ARG, "x is NULL");
        GTC_REQUIRE(x_len >= g->n, GTC_ERR_ARG, "centrality map is shorter than the vertex bound");
        common_opts(opt, in);
        cudaStream_t s = stream_of(g, opt);
        HostStage st;
        stage_host(g, s, weight, nullptr, x, x_had, in, st);
        gtc_result r{};
        gtc::eigenvector(g, view, in, &r, s);
        unstage_host(g, s, x, st);
        if (result) *result = r;
    });
}

int gtc_pagerank_device(gtc_graph* g, const gtc_view* view, const gtc_dvec* weight,
                        const gtc_dvec* pers, double damping, const gtc_power_iteration* params,
                        gtc_dvec* rank, uint64_t rank_had, const gtc_options* opt,
                        gtc_result* result) {
    return guarded([&] {
        GTC_REQUIRE(g, GTC_ERR_ARG, "graph is NULL");
        SolveIn in{};
        check_params(g, params, in.params);
        in.weight = dvec_in(weight, g->m, "weight");
        in.pers = dvec_in(pers, g->n, "personalisation");
        GTC_REQUIRE(rank && (rank->ptr || g->n == 0), GTC_ERR_ARG, "rank is NULL");
        DVec x = dvec_in(rank, g->n, "rank");
        GTC_REQUIRE(!std::isnan(damping), GTC_ERR_ARG, "damping is NaN");
        common_opts(opt, in);
        in.damping = damping;
        in.x = rank->ptr;
        in.x_dtype = x.p ? x.dtype : GTC_F64;
        in.had = rank_had;
        gtc_result r{};
        gtc::pagerank(g, view, in, &r, stream_of(g, opt));
        if (result) *result = r;
    });
}

int gtc_eigenvector_device(gtc_graph* g, const gtc_view* view, const gtc_dvec* weight,
                           const gtc_power_iteration* params, gtc_dvec* x, uint64_t x_had,
                           const gtc_options* opt, gtc_result* result) {
    return guarded([&] {
        GTC_REQUIRE(g, GTC_ERR_ARG, "graph is NULL");
        SolveIn in{};
        check_params(g, params, in.params);
        in.weight = dvec_in(weight, g->m, "weight");
        GTC_REQUIRE(x && (x->ptr || g->n == 0), GTC_ERR_ARG, "x is NULL");
        DVec xv = dvec_in(x, g->n, "centrality");
        common_opts(opt, in);
        in.x = x->ptr;
        in.x_dtype = xv.p ? xv.dtype : GTC_F64;
        in.had = x_had;
        gtc_result r{};
        gtc::eigenvector(g, view, in, &r, stream_of(g, opt));
        if (result) *result = r;
    });
}

int gtc_pagerank_adjoint_device(gtc_graph* g, const gtc_view* view, const gtc_dvec* weight,
                                const gtc_dvec* pers, double damping,
                                const gtc_power_iteration* params, const gtc_dvec* pi,
                                const gtc_dvec* grad_pi, gtc_dvec* grad_weight, gtc_dvec* grad_pers,
                                const gtc_options* opt, gtc_result* result) {
    return guarded([&] {
        GTC_REQUIRE(g, GTC_ERR_ARG, "graph is NULL");
        AdjointIn in{};
        check_params(g, params, in.params);
        in.weight = dvec_in(weight, g->m, "weight");
        in.pers = dvec_in(pers, g->n, "personalisation");
        GTC_REQUIRE(pi && (pi->ptr || g->n == 0), GTC_ERR_ARG, "pi is NULL");
        GTC_REQUIRE(grad_pi && (grad_pi->ptr || g->n == 0), GTC_ERR_ARG, "grad_pi is NULL");
        in.pi = dvec_in(pi, g->n, "pi");
        in.gpi = dvec_in(grad_pi, g->n, "grad_pi");
        if (grad_weight && grad_weight->ptr) {
            GTC_REQUIRE(grad_weight->len >= g->m, GTC_ERR_ARG, "grad_weight is shorter than the edge bound");
            GTC_REQUIRE(grad_weight->dtype == GTC_F64 || grad_weight->dtype == GTC_F32, GTC_ERR_ARG,
                        "grad_weight: unknown dtype");
            in.grad_w = grad_weight->ptr;
            in.grad_w_dtype = grad_weight->dtype;
        }
        if (grad_pers && grad_pers->ptr) {
            GTC_REQUIRE(grad_pers->len >= g->n, GTC_ERR_ARG, "grad_pers is shorter than the vertex bound");
            GTC_REQUIRE(grad_pers->dtype == GTC_F64 || grad_pers->dtype == GTC_F32, GTC_ERR_ARG,
                        "grad_pers: unknown dtype");
            in.grad_p = grad_pers->ptr;
            in.grad_p_dtype = grad_pers->dtype;
        }
        GTC_REQUIRE(!std::isnan(damping), GTC_ERR_ARG, "damping is NaN");
        GTC_REQUIRE(!opt || opt->precision == GTC_PREC_F32, GTC_ERR_ARG,
                    "the PageRank adjoint runs in GTC_PREC_F32");
        in.damping = damping;
        in.timing = opt && opt->timing;
        gtc_result r{};
        gtc::pagerank_adjoint(g, view, in, &r, stream_of(g, opt));
        if (result) *result = r;
    });
}

int gtc_pagerank_adjoint(gtc_graph* g, const gtc_view* view, const double* weight,
                         uint64_t weight_len, const double* pers, uint64_t pers_len, double damping,
                         const gtc_power_iteration* params, const double* pi, const double* grad_pi,
                         double* grad_weight, double* grad_pers, const gtc_options* opt,
                         gtc_result* result) {
    return guarded([&] {
        GTC_REQUIRE(g, GTC_ERR_ARG, "graph is NULL");
        GTC_REQUIRE(!weight || weight_len >= g->m, GTC_ERR_ARG, "weight map is shorter than the edge bound");
        GTC_REQUIRE(!pers || pers_len >= g->n, GTC_ERR_ARG,
                    "personalisation map is shorter than the vertex bound");
        GTC_REQUIRE((pi && grad_pi) || g->n == 0, GTC_ERR_ARG, "pi / grad_pi is NULL");
        cudaStream_t s = stream_of(g, opt);
        const uint32_t n = g->n, m = g->m;
        DevBuf<double> dw, dp, dpi(n, s), dg(n, s), dgw, dgp;
        if (weight) {
            dw.alloc(m, s);
            if (m) GTC_CUDA(cudaMemcpyAsync(dw.get(), weight, (size_t)m * 8, cudaMemcpyHostToDevice, s));
        }
        if (pers) {
            dp.alloc(n, s);
            if (n) GTC_CUDA(cudaMemcpyAsync(dp.get(), pers, (size_t)n * 8, cudaMemcpyHostToDevice, s));
        }
        if (n) {
            GTC_CUDA(cudaMemcpyAsync(dpi.get(), pi, (size_t)n * 8, cudaMemcpyHostToDevice, s));
            GTC_CUDA(cudaMemcpyAsync(dg.get(), grad_pi, (size_t)n * 8, cudaMemcpyHostToDevice, s));
        }
        if (grad_weight) dgw.alloc(m, s);
        if (grad_pers) dgp.alloc(n, s);
        gtc_dvec vw{dw.get(), m, GTC_F64, 0}, vp{dp.get(), n, GTC_F64, 0};
        gtc_dvec vpi{dpi.get(), n, GTC_F64, 0}, vg{dg.get(), n, GTC_F64, 0};
        gtc_dvec vgw{dgw.get(), m, GTC_F64, 0}, vgp{dgp.get(), n, GTC_F64, 0};
        gtc_options o = opt ? *opt : gtc_options{};
        o.stream = (void*)s;
        const int st = gtc_pagerank_adjoint_device(g, view, weight ? &vw : nullptr,
                                                   pers ? &vp : nullptr, damping, params, &vpi, &vg,
                                                   grad_weight ? &vgw : nullptr,
                                                   grad_pers ? &vgp : nullptr, &o, result);
        if (st != GTC_OK) throw Error{st, gtc_last_error()};
        if (grad_weight && m)
            GTC_CUDA(cudaMemcpyAsync(grad_weight, dgw.get(), (size_t)m * 8, cudaMemcpyDeviceToHost, s));
        if (grad_pers && n)
            GTC_CUDA(cudaMemcpyAsync(grad_pers, dgp.get(), (size_t)n * 8, cudaMemcpyDeviceToHost, s));
        GTC_CUDA(cudaStreamSynchronize(s));
    });
}

int gtc_ppr_batch_device(gtc_graph* g, const gtc_view* view, const gtc_dvec* weight, uint32_t B,
                         const uint64_t* seed_off, const uint32_t* seed_vertices,
                         const double* seed_values, double damping,
                         const gtc_power_iteration* params, gtc_dvec* ranks, uint64_t* iters,
                         const gtc_options* opt, gtc_result* result) {
    return guarded([&] {
        GTC_REQUIRE(g, GTC_ERR_ARG, "graph is NULL");
        PprIn in{};
        check_params(g, params, in.params);
        in.weight = dvec_in(weight, g->m, "weight");
        GTC_REQUIRE(seed_off && (seed_off[B] == 0 || seed_vertices), GTC_ERR_ARG,
                    "seed_off / seed_vertices is NULL");
        GTC_REQUIRE(iters, GTC_ERR_ARG, "iters is NULL");
        GTC_REQUIRE(ranks && (ranks->ptr || g->n == 0), GTC_ERR_ARG, "ranks is NULL");
        GTC_REQUIRE(ranks->len >= (uint64_t)B * g->n, GTC_ERR_ARG, "ranks holds fewer than B x n entries");
        GTC_REQUIRE(ranks->dtype == GTC_F64 || ranks->dtype == GTC_F32, GTC_ERR_ARG, "ranks: unknown dtype");
        GTC_REQUIRE(!std::isnan(damping), GTC_ERR_ARG, "damping is NaN");
        GTC_REQUIRE(!opt || opt->precision == GTC_PREC_F32, GTC_ERR_ARG,
                    "batched personalised PageRank runs in GTC_PREC_F32");
        in.B = B;
        in.seed_off = seed_off;
        in.seed_vertices = seed_vertices;
        in.seed_values = seed_values;
        in.damping = damping;
        in.out = ranks->ptr;
        in.out_dtype = ranks->dtype;
        in.iters = iters;
        in.timing = opt && opt->timing;
        in.gather = opt ? opt->ppr_gather : GTC_PPR_BULK;
        GTC_REQUIRE(in.gather == GTC_PPR_BULK || in.gather == GTC_PPR_REGS, GTC_ERR_ARG,
                    "unknown ppr_gather");
        gtc_result r{};
        gtc::ppr_batch(g, view, in, &r, stream_of(g, opt));
        if (result) *result = r;
    });
}

int gtc_ppr_batch(gtc_graph* g, const gtc_view* view, const double* weight, uint64_t weight_len,
                  uint32_t B, const uint64_t* seed_off, const uint32_t* seed_vertices,
                  const double* seed_values, double damping, const gtc_power_iteration* params,
                  double* ranks, uint64_t* iters, const gtc_options* opt, gtc_result* result) {
    return guarded([&] {
        GTC_REQUIRE(g, GTC_ERR_ARG, "graph is NULL");
        GTC_REQUIRE(!weight || weight_len >= g->m, GTC_ERR_ARG, "weight map is shorter than the edge bound");
        GTC_REQUIRE(ranks || g->n == 0 || B == 0, GTC_ERR_ARG, "ranks is NULL");
        cudaStream_t s = stream_of(g, opt);
        const uint32_t n = g->n, m = g->m;
        DevBuf<double> dw, dr((size_t)B * n, s);
        if (weight) {
            dw.alloc(m, s);
            if (m) GTC_CUDA(cudaMemcpyAsync(dw.get(), weight, (size_t)m * 8, cudaMemcpyHostToDevice, s));
        }
        gtc_dvec vw{dw.get(), m, GTC_F64, 0}, vr{dr.get(), (uint64_t)B * n, GTC_F64, 0};
        gtc_options o = opt ? *opt : gtc_options{};
        o.stream = (void*)s;
        const int st = gtc_ppr_batch_device(g, view, weight ? &vw : nullptr, B, seed_off,
                                            seed_vertices, seed_values, damping, params, &vr, iters,
                                            &o, result);
        if (st != GTC_OK) throw Error{st, gtc_last_error()};
        if ((size_t)B * n)
            GTC_CUDA(cudaMemcpyAsync(ranks, dr.get(), (size_t)B * n * 8, cudaMemcpyDeviceToHost, s));
        GTC_CUDA(cudaStreamSynchronize(s));
    });
}


static void destroy_batch(gtc_graph_batch* b) {
    if (!b) return;
    if (b->exec) cudaGraphExecDestroy(b->exec);
    gtc_graph* u = b->u;
    b->u = nullptr;
    delete b;  // its buffers are freed on the union's home stream
    destroy_graph(u);
}

int gtc_graph_batch_create(uint64_t G, const uint64_t* voff, const uint64_t* eoff,
                           const uint32_t* src, const uint32_t* tgt, gtc_graph_batch** out) {
    return guarded([&] {
        GTC_REQUIRE(out, GTC_ERR_ARG, "out is NULL");
        *out = nullptr;
        GTC_REQUIRE(G >= 1 && G < (1ull << 31), GTC_ERR_ARG, "a batch holds 1 to 2^31 - 1 graphs");
        GTC_REQUIRE(voff && eoff, GTC_ERR_ARG, "voff/eoff is NULL");
        GTC_REQUIRE(voff[0] == 0 && eoff[0] == 0, GTC_ERR_ARG, "voff[0] and eoff[0] must be 0");
        for (uint64_t k = 0; k < G; ++k) {
            GTC_REQUIRE(voff[k + 1] >= voff[k] && eoff[k + 1] >= eoff[k], GTC_ERR_ARG,
                        "voff/eoff must not decrease");
        }
        const uint64_t n = voff[G], m = eoff[G];
        GTC_REQUIRE(n <= 0xFFFFF000ull && m <= 0xFFFFFFFEull, GTC_ERR_ARG,
                    "the packed batch exceeds the index space (n <= 2^32 - 4096, m <= 2^32 - 2)");
        GTC_REQUIRE(m == 0 || (src && tgt), GTC_ERR_ARG, "src/tgt is NULL");
        // endpoints to packed labels, checked against their own graph
        std::vector<uint32_t> gs(m), gt(m);
        for (uint64_t k = 0; k < G; ++k) {
            const uint64_t nk = voff[k + 1] - voff[k];
            for (uint64_t e = eoff[k]; e < eoff[k + 1]; ++e) {
                GTC_REQUIRE(src[e] < nk && tgt[e] < nk, GTC_ERR_ARG,
                            "add_edge: no such vertex (an endpoint is >= its graph's n)");
                gs[e] = (uint32_t)(src[e] + voff[k]);
                gt[e] = (uint32_t)(tgt[e] + voff[k]);
            }
        }
        gtc_graph_batch* b = new gtc_graph_batch();
        try {
            b->u = new_graph(n, m);
            b->G = (uint32_t)G;
            cudaStream_t h = b->u->home;
            b->hvoff.resize(G + 1);
            b->heoff.resize(G + 1);
            for (uint64_t k = 0; k <= G; ++k) b->hvoff[k] = (uint32_t)voff[k], b->heoff[k] = (uint32_t)eoff[k];
            b->voff.alloc(G + 1, h);
            GTC_CUDA(cudaMemcpyAsync(b->voff.get(), b->hvoff.data(), (G + 1) * 4, cudaMemcpyHostToDevice, h));
            {
                DevBuf<uint32_t> ds(m, h), dt(m, h);
                if (m) {
                    GTC_CUDA(cudaMemcpyAsync(ds.get(), gs.data(), m * 4, cudaMemcpyHostToDevice, h));
                    GTC_CUDA(cudaMemcpyAsync(dt.get(), gt.data(), m * 4, cudaMemcpyHostToDevice, h));
                }
                batch_layout(b, ds.get(), dt.get(), h);
            }
            std::vector<uint32_t> order(G);
            for (uint32_t k = 0; k < G; ++k) order[k] = k;
            std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t c) {
                return (eoff[a + 1] - eoff[a]) + (voff[a + 1] - voff[a]) >
                       (eoff[c + 1] - eoff[c]) + (voff[c + 1] - voff[c]);
            });
            // three queues, in this order: graphs for a cluster pair (up to
            // 2 * GB_CL_CAP vertices), for one CTA (up to GB_CL_CAP), and the
            // larger ones, gathered from global memory
            auto queue = [&](uint32_t k) {
                const uint64_t nk = voff[k + 1] - voff[k];
                return nk <= GB_CL_CAP ? 1 : (nk + 1) / 2 <= GB_CL_CAP ? 0 : 2;
            };
            std::stable_sort(order.begin(), order.end(),
                             [&](uint32_t a, uint32_t c) { return queue(a) < queue(c); });
            b->n_pair = b->n_single = b->n_global = 0;
            b->smem_floats = 0;
            for (uint32_t k : order) {
                const uint32_t nk = (uint32_t)(voff[k + 1] - voff[k]);
                switch (queue(k)) {
                    case 0: ++b->n_pair, b->smem_floats = std::max(b->smem_floats, (nk + 1) / 2); break;
                    case 1: ++b->n_single, b->smem_floats = std::max(b->smem_floats, nk); break;
                    default: ++b->n_global;
                }
            }
            b->order.alloc(G, h);
            GTC_CUDA(cudaMemcpyAsync(b->order.get(), order.data(), G * 4, cudaMemcpyHostToDevice, h));
            GTC_CUDA(cudaStreamSynchronize(h));
        } catch (...) {
            destroy_batch(b);
            throw;
        }
        *out = b;
    });
}

int gtc_graph_batch_destroy(gtc_graph_batch* b) {
    return guarded([&] { destroy_batch(b); });
}

int gtc_graph_batch_info(const gtc_graph_batch* b, uint64_t* graphs, uint64_t* vertices,
                         uint64_t* edges) {
    return guarded([&] {
        GTC_REQUIRE(b, GTC_ERR_ARG, "batch is NULL");
        if (graphs) *graphs = b->G;
        if (vertices) *vertices = b->u->n;
        if (edges) *edges = b->u->m;
    });
}

int gtc_pagerank_batch_device(gtc_graph_batch* b, const gtc_dvec* weight, double damping,
                              double epsilon, uint64_t max_iter, gtc_dvec* rank, uint64_t* iters,
                              const gtc_options* opt, gtc_result* result) {
    return guarded([&] {
        GTC_REQUIRE(b, GTC_ERR_ARG, "batch is NULL");
        GTC_REQUIRE(max_iter > 0 || epsilon > 0, GTC_ERR_ARG,
                    "epsilon must be positive when max_iter is 0 (the solve would never stop)");
        GTC_REQUIRE(!std::isnan(damping) && !std::isnan(epsilon), GTC_ERR_ARG,
                    "damping or epsilon is NaN");
        GTC_REQUIRE(!opt || opt->precision == GTC_PREC_F32, GTC_ERR_ARG,
                    "batched PageRank runs in GTC_PREC_F32");
        const DVec w = dvec_in(weight, b->u->m, "weight");
        GTC_REQUIRE(rank && (rank->ptr || b->u->n == 0), GTC_ERR_ARG, "rank is NULL");
        GTC_REQUIRE(rank->len >= b->u->n, GTC_ERR_ARG, "rank holds fewer entries than the batch's vertices");
        GTC_REQUIRE(rank->dtype == GTC_F64 || rank->dtype == GTC_F32, GTC_ERR_ARG, "rank: unknown dtype");
        gtc_result r{};
        gtc::pagerank_batch(b, w, damping, epsilon, max_iter, rank->ptr, rank->dtype, iters,
                            opt && opt->timing, &r, stream_of(b->u, opt));
        if (result) *result = r;
    });
}

int gtc_pagerank_batch(gtc_graph_batch* b, const double* weight, uint64_t weight_len,
                       double damping, double epsilon, uint64_t max_iter, double* rank,
                       uint64_t rank_len, uint64_t* iters, const gtc_options* opt,
                       gtc_result* result) {
    return guarded([&] {
        GTC_REQUIRE(b, GTC_ERR_ARG, "batch is NULL");
        const uint32_t n = b->u->n, m = b->u->m;
        GTC_REQUIRE(!weight || weight_len >= m, GTC_ERR_ARG, "weight map is shorter than the edge bound");
        GTC_REQUIRE(rank || n == 0, GTC_ERR_ARG, "rank is NULL");
        GTC_REQUIRE(rank_len >= n, GTC_ERR_ARG, "rank map is shorter than the vertex bound");
        cudaStream_t s = stream_of(b->u, opt);
        // staging buffers live with the batch, so the captured solve is replayed
        if (weight && b->wstage.n < m) b->wstage.alloc(m, b->u->home);
        if (b->rstage.n < n || !b->rstage.get()) b->rstage.alloc(n, b->u->home);
        GTC_CUDA(cudaStreamSynchronize(b->u->home));
        if (weight && m)
            GTC_CUDA(cudaMemcpyAsync(b->wstage.get(), weight, (size_t)m * 8, cudaMemcpyHostToDevice, s));
        gtc_dvec vw{weight ? b->wstage.get() : nullptr, m, GTC_F64, 0};
        gtc_dvec vr{b->rstage.get(), n, GTC_F64, 0};
        gtc_options o = opt ? *opt : gtc_options{};
        o.stream = (void*)s;
        const int st = gtc_pagerank_batch_device(b, weight ? &vw : nullptr, damping, epsilon,
                                                 max_iter, &vr, iters, &o, result);
        if (st != GTC_OK) throw Error{st, gtc_last_error()};
        if (n) GTC_CUDA(cudaMemcpyAsync(rank, b->rstage.get(), (size_t)n * 8, cudaMemcpyDeviceToHost, s));
        GTC_CUDA(cudaStreamSynchronize(s));
    });
}

}  // extern "C"
