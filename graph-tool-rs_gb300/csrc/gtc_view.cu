// gtc_view.cu -- per-call materialisation of the directed view a solve runs
// on: the plain graph, its reversal, and either filtered by vertex / edge
// masks.
//
//   Rev (crates/gt-core/src/view/reversed.rs:109-138): in_edges(v) is the
//   base graph's out_edges(v), out_degree(v) its in_degree(v).
//   Filtered (crates/gt-core/src/view/filtered.rs:299-319): an incident entry
//   survives iff keep_edge(idx) && keep_vertex(other); vertices() yields the
//   kept vertices and num_vertices() counts them.
//
// Without masks nothing is copied: the view points at the graph's halves.
// With masks the pull half and the push half are compacted (stable, so the
// storage order the reference iterates in is kept).
#include "gtc_view.cuh"

namespace gtc {

__global__ void k_keep_flags(uint32_t m, const uint32_t* __restrict__ other,
                             const uint32_t* __restrict__ eid, const uint8_t* __restrict__ vmask,
                             const uint8_t* __restrict__ emask, uint32_t* __restrict__ flag) {
    size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= m) return;
    bool keep = (!emask || emask[eid[p]]) && (!vmask || vmask[other[p]]);
    flag[p] = keep ? 1u : 0u;
}

__global__ void k_compact(uint32_t m, const uint32_t* __restrict__ flag,
                          const uint32_t* __restrict__ pos, const uint32_t* __restrict__ other,
                          const uint32_t* __restrict__ eid, uint32_t* __restrict__ fo,
                          uint32_t* __restrict__ fe) {
    size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= m || !flag[p]) return;
    uint32_t q = pos[p];
    fo[q] = other[p];
    fe[q] = eid[p];
}

__global__ void k_remap_off(uint32_t n, const uint32_t* __restrict__ off,
                            const uint32_t* __restrict__ pos, uint32_t* __restrict__ foff) {
    size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v <= n) foff[v] = pos[off[v]];
}

// act[new] = vmask[perm[new]] != 0 (the caller's mask is by original index)
__global__ void k_active(uint32_t n, const uint8_t* __restrict__ vmask,
                         const uint32_t* __restrict__ perm, uint8_t* __restrict__ act,
                         uint32_t* __restrict__ count) {
    size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    bool a = v < n && vmask[perm[v]] != 0;
    if (v < n) act[v] = a ? 1 : 0;
    unsigned b = __ballot_sync(0xffffffffu, a);
    if ((threadIdx.x & 31) == 0 && b) atomicAdd(count, (unsigned)__popc(b));
}

static void compact_half(uint32_t n, uint32_t m, const uint32_t* off, const uint32_t* other,
                         const uint32_t* eid, const uint8_t* vmask, const uint8_t* emask,
                         Halves& out, cudaStream_t s, uint64_t* L) {
    const unsigned TB = 256;
    DevBuf<uint32_t> flag(m, s), pos((size_t)m + 1, s);
    if (m) {
        k_keep_flags<<<grid_for(m, TB, 1u << 30), TB, 0, s>>>(m, other, eid, vmask, emask,
                                                            flag.get());
        GTC_LAUNCHED();
        *L += 1;
    }
    scan_exclusive_u32(flag.get(), pos.get(), m, s, L);
    uint32_t kept = 0;
    GTC_CUDA(cudaMemcpyAsync(&kept, pos.get() + m, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    GTC_CUDA(cudaStreamSynchronize(s));
    out.off.alloc((size_t)n + 1, s);
    out.other.alloc(kept, s);
    out.eid.alloc(kept, s);
    if (m) {
        k_compact<<<grid_for(m, TB, 1u << 30), TB, 0, s>>>(m, flag.get(), pos.get(), other, eid,
                                                         out.other.get(), out.eid.get());
        GTC_LAUNCHED();
        *L += 1;
    }
    k_remap_off<<<grid_for((size_t)n + 1, TB, 1u << 30), TB, 0, s>>>(n, off, pos.get(),
                                                                   out.off.get());
    GTC_LAUNCHED();
    *L += 1;
}

void View::prepare(gtc_graph* g, const gtc_view* v, cudaStream_t s, uint64_t* L) {
    n = g->n;
    m_total = g->m;
    reversed = v && v->reversed;
    const Halves& pull_src = reversed ? g->out : g->in;
    const Halves& push_src = reversed ? g->in : g->out;
    const uint8_t* hv = v ? v->vmask : nullptr;
    const uint8_t* he = v ? v->emask : nullptr;
    if (hv) GTC_REQUIRE(v->vmask_len == n, GTC_ERR_ARG, "vertex mask length != vertex bound");
    if (he) GTC_REQUIRE(v->emask_len == g->m, GTC_ERR_ARG, "edge mask length != edge bound");
    filtered = hv || he;
    n_active = n;
    if (!filtered) {
        pull_off = pull_src.off.get(), pull_other = pull_src.other.get(),
        pull_eid = pull_src.eid.get();
        push_off = push_src.off.get(), push_other = push_src.other.get(),
        push_eid = push_src.eid.get();
        m_pull = g->m_live;
        return;
    }
    DevBuf<uint8_t> dv, de;
    if (hv) {
        dv.alloc(n, s);
        GTC_CUDA(cudaMemcpyAsync(dv.get(), hv, n, cudaMemcpyHostToDevice, s));
        active.alloc(n, s);
        DevBuf<uint32_t> cnt(1, s);
        GTC_CUDA(cudaMemsetAsync(cnt.get(), 0, sizeof(uint32_t), s));
        if (n) {
            k_active<<<grid_for(n, 256, 1u << 30), 256, 0, s>>>(n, dv.get(), g->perm.get(),
                                                                active.get(), cnt.get());
            GTC_LAUNCHED();
            *L += 1;
        }
        GTC_CUDA(cudaMemcpyAsync(&n_active, cnt.get(), sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    }
    if (he) {
        de.alloc(g->m, s);
        GTC_CUDA(cudaMemcpyAsync(de.get(), he, g->m, cudaMemcpyHostToDevice, s));
    }
    const uint8_t* vnew = hv ? active.get() : nullptr;  // the mask in internal labels
    compact_half(n, g->m_live, pull_src.off.get(), pull_src.other.get(), pull_src.eid.get(), vnew,
                 de.get(), fpull, s, L);
    compact_half(n, g->m_live, push_src.off.get(), push_src.other.get(), push_src.eid.get(), vnew,
                 de.get(), fpush, s, L);
    GTC_CUDA(cudaStreamSynchronize(s));
    pull_off = fpull.off.get(), pull_other = fpull.other.get(), pull_eid = fpull.eid.get();
    push_off = fpush.off.get(), push_other = fpush.other.get(), push_eid = fpush.eid.get();
    m_pull = (uint32_t)fpull.other.n;
}

}  // namespace gtc
