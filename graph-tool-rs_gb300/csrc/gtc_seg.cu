// gtc_seg.cu -- the segmented pull sweep of the FP32 PageRank path.
//
// The plain pull sweep (gtc_sweep.cuh) gathers y[src] for every in-edge
// straight from L2: one random 32-byte sector per edge.  On R-MAT graphs the
// rate of such requests, not HBM bandwidth, bounds that sweep.  The
// segmented sweep makes every gather a shared-memory read and streams
// everything else:
//
//   sources are cut into segments of SEG_P = 32768 vertices (128 KB of y);
//   destinations into groups of SEG_G = 1024 vertices;
//   a pair is (segment s, destination v) with at least one edge s -> v, its
//   edges contiguous; pairs longer than SEG_LMAX edges are cut into sub-pairs.
//
// Phase 1 (k_seg_pairs): a CTA stages y of one segment in shared memory and
// its warps sum the pairs of that segment, 32 edges at a time with a
// segmented warp scan (a pair's edges may span chunks: the open sum is
// carried with compensation).  Edges are 16-bit local source indices with
// the pair-start flag in bit 15; one float per pair is written, in the
// order phase 2 reads them.
//
// Phase 2 (k_seg_rows): a warp owns a destination group: it streams the
// group's pair sums (segment by segment) into compensated accumulators in
// shared memory, then runs the PageRank epilogue for its 1024 vertices and
// the fixed-order fold of the L1 change and dangling mass.  Within a "run"
// (the pairs of one segment, up to the next sub-pair) all destinations
// differ, so a run's pairs are added by the lanes at once; runs are added
// in order, so every sum has a fixed order.
//
// Per sweep the traffic is 2 bytes per edge, 10 bytes per pair and the
// epilogue's vectors; the plan (built once per direction, kept with the
// graph) needs n < 2^29 and an unfiltered view.
#include <algorithm>
#include <vector>

#include "gtc_view.cuh"

namespace gtc {
namespace {

constexpr uint32_t SEG_P = 32768;    // sources per segment (15-bit local index)
constexpr uint32_t SEG_G = 1024;     // destinations per group (10-bit local index)
constexpr uint32_t SEG_LMAX = 256;   // edges per sub-pair at most
constexpr uint32_t SEG_UMAX = 4096;  // edges per phase-1 unit (a warp's work), about
constexpr uint32_t SEG_ITEM = 65536; // edges per phase-1 CTA item, about
constexpr int P1_WARPS = 16;
constexpr int P1_NT = 32 * P1_WARPS;
constexpr int P2_WARPS = 16;
constexpr int P2_NT = 32 * P2_WARPS;

// ---- build ------------------------------------------------------------------

__global__ void k_seg_rowid(uint32_t n, const uint32_t* __restrict__ off, uint32_t* __restrict__ rowid) {
    const uint32_t sub = threadIdx.x & 7;
    const size_t v = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 3;
    if (v >= n) return;
    for (uint32_t p = off[v] + sub, e = off[v + 1]; p < e; p += 8) rowid[p] = (uint32_t)v;
}

__global__ void k_seg_key(uint32_t m, uint32_t ngroups, const uint32_t* __restrict__ other,
                          const uint32_t* __restrict__ rowid, uint32_t* __restrict__ key) {
    const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < m) key[k] = (other[k] / SEG_P) * ngroups + rowid[k] / SEG_G;
}

// first-level pair starts: a new (segment, group) key or a new destination
__global__ void k_seg_h1(uint32_t m, const uint32_t* __restrict__ perm, const uint32_t* __restrict__ skey,
                         const uint32_t* __restrict__ rowid, uint32_t* __restrict__ dest,
                         uint32_t* __restrict__ h1) {
    const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= m) return;
    const uint32_t v = rowid[perm[e]];
    dest[e] = v;
    h1[e] = (e == 0 || skey[e] != skey[e - 1] || v != rowid[perm[e - 1]]) ? 1u : 0u;
}

__global__ void k_seg_mark_start(uint32_t m, const uint32_t* __restrict__ h, const uint32_t* __restrict__ idx,
                                 uint32_t* __restrict__ start) {
    const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e < m && h[e]) start[idx[e]] = (uint32_t)e;
}

// sub-pair starts: every SEG_LMAX edges of a pair; xs marks the extra ones
__global__ void k_seg_h2(uint32_t m, const uint32_t* __restrict__ h1, const uint32_t* __restrict__ id1x,
                         const uint32_t* __restrict__ start1, uint32_t* __restrict__ h2,
                         uint8_t* __restrict__ xs) {
    const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= m) return;
    const uint32_t pid = id1x[e] + h1[e] - 1;
    const uint32_t local = (uint32_t)e - start1[pid];
    h2[e] = local % SEG_LMAX == 0 ? 1u : 0u;
    xs[e] = (local != 0 && local % SEG_LMAX == 0) ? 1 : 0;
}

// per final pair: its key, destination and extra-sub-pair flag; counts per key
__global__ void k_seg_pairs_info(uint32_t np, const uint32_t* __restrict__ pstart,
                                 const uint32_t* __restrict__ skey, const uint32_t* __restrict__ dest,
                                 const uint8_t* __restrict__ xs, uint32_t* __restrict__ pkey,
                                 uint32_t* __restrict__ pv, uint8_t* __restrict__ pxs,
                                 uint32_t* __restrict__ cntk) {
    const size_t f = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= np) return;
    const uint32_t e = pstart[f];
    pkey[f] = skey[e];
    pv[f] = dest[e];
    pxs[f] = xs[e];
    atomicAdd(cntk + skey[e], 1u);  // integer counts: the order does not matter
}

__global__ void k_seg_edge_counts(uint32_t m, const uint32_t* __restrict__ skey, uint32_t* __restrict__ ecnt) {
    const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e < m) atomicAdd(ecnt + skey[e], 1u);
}

__global__ void k_seg_transpose(uint32_t nseg, uint32_t ngroups, const uint32_t* __restrict__ cntk,
                                uint32_t* __restrict__ tcnt) {
    const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= (size_t)nseg * ngroups) return;
    const uint32_t s = (uint32_t)(k / ngroups), g = (uint32_t)(k % ngroups);
    tcnt[(size_t)g * nseg + s] = cntk[k];
}

// phase-2 position of every pair, its destination word, and the unit flags
__global__ void k_seg_place(uint32_t np, uint32_t nseg, uint32_t ngroups,
                            const uint32_t* __restrict__ pkey, const uint32_t* __restrict__ pv,
                            const uint8_t* __restrict__ pxs, const uint32_t* __restrict__ pstart,
                            const uint32_t* __restrict__ base1, const uint32_t* __restrict__ base2,
                            const uint32_t* __restrict__ kes, uint16_t* __restrict__ pdest,
                            uint32_t* __restrict__ p2, uint32_t* __restrict__ uflag) {
    const size_t f = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= np) return;
    const uint32_t key = pkey[f], s = key / ngroups, g = key % ngroups;
    const uint32_t first = base1[key];
    const uint32_t pos = base2[(size_t)g * nseg + s] + ((uint32_t)f - first);
    const bool run_start = (uint32_t)f == first || pxs[f];
    pdest[pos] = (uint16_t)((pv[f] % SEG_G) | (run_start ? 0x8000u : 0u));
    p2[f] = pos;
    const uint32_t e = pstart[f], ke = kes[key];
    bool unit = (uint32_t)f == first;
    if (!unit) unit = (e - ke) / SEG_UMAX != (pstart[f - 1] - ke) / SEG_UMAX;
    uflag[f] = unit ? 1u : 0u;
}

__global__ void k_seg_edges(uint32_t m, const uint32_t* __restrict__ perm, const uint32_t* __restrict__ other,
                            const uint32_t* __restrict__ eid, const uint32_t* __restrict__ h2,
                            uint16_t* __restrict__ src16, uint32_t* __restrict__ seid) {
    const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= m) return;
    const uint32_t k = perm[e];
    src16[e] = (uint16_t)((other[k] % SEG_P) | (h2[e] ? 0x8000u : 0u));
    seid[e] = eid[k];
}

__global__ void k_seg_units(uint32_t np, const uint32_t* __restrict__ uflag,
                            const uint32_t* __restrict__ uidx, const uint32_t* __restrict__ pstart,
                            const uint32_t* __restrict__ p2, const uint32_t* __restrict__ pkey,
                            uint32_t ngroups, uint32_t* __restrict__ unit_e,
                            uint32_t* __restrict__ unit_o, uint32_t* __restrict__ unit_s) {
    const size_t f = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= np || !uflag[f]) return;
    const uint32_t u = uidx[f];
    unit_e[u] = pstart[f];
    unit_o[u] = p2[f];
    unit_s[u] = pkey[f] / ngroups;
}

// ---- the sweep -------------------------------------------------------------

__device__ __forceinline__ uint32_t lanemask_le() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_le;" : "=r"(m));
    return m;
}

// One unit: the pairs of edges [eb, ee) (eb starts a pair, ee ends one),
// their sums to partial[ob ...].
template <bool W>
__device__ __forceinline__ void seg_unit(const SegArgs& A, const float* ys, uint32_t eb,
                                         uint32_t ee, uint32_t ob, int lane) {
    uint32_t k_pair = 0;  // pairs started so far in this unit
    Kahan carry;          // the open pair's sum
    for (uint32_t c = eb; c < ee; c += 32) {
        const uint32_t e = c + lane;
        const bool valid = e < ee;
        const uint32_t h = valid ? (uint32_t)A.src16[e] : 0u;
        const bool head = valid && (h >> 15) != 0;
        float x = valid ? ys[h & 0x7FFFu] : 0.f;
        if (W && valid) x = __fmul_rn(x, A.ws[e]);
        const uint32_t hm = __ballot_sync(0xffffffffu, head);
        // inclusive scan of x, restarted at every pair start
        float v = x;
        bool f = head;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const float nv = __shfl_up_sync(0xffffffffu, v, o);
            const bool nf = __shfl_up_sync(0xffffffffu, f, o) != 0;
            if (lane >= o && !f) {
                v = __fadd_rn(v, nv);
                f = nf;
            }
        }
        const bool cont = (hm & lanemask_le()) == 0;  // my pair began before this chunk
        bool next_head;
        if (lane < 31)
            next_head = ((hm >> (lane + 1)) & 1u) || !(e + 1 < ee);
        else
            next_head = !(c + 32 < ee) || (A.src16[c + 32] >> 15) != 0;
        const bool end = valid && next_head;
        const uint32_t idx = k_pair + __popc(hm & lanemask_le()) - 1;
        if (end) {
            float tot = v;
            if (cont) {
                Kahan t = carry;
                t.add(v);
                tot = t.value();
            }
            A.partial[ob + idx] = tot;
        }
        // the pair still open after lane 31 carries on
        const float v31 = __shfl_sync(0xffffffffu, v, 31);
        const bool cont31 = __shfl_sync(0xffffffffu, cont, 31) != 0;
        const bool open31 = __shfl_sync(0xffffffffu, valid && !end, 31) != 0;
        if (open31) {
            if (cont31) {
                carry.add(v31);
            } else {
                carry = Kahan();
                carry.add(v31);
            }
        } else {
            carry = Kahan();
        }
        k_pair += __popc(hm);
    }
}

template <bool W>
__global__ void __launch_bounds__(P1_NT, 1) k_seg_pairs(SegArgs A) {
    extern __shared__ float seg_ys[];  // y of the item's segment
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (uint32_t it = blockIdx.x; it < A.nitems; it += gridDim.x) {
        const uint4 item = A.items[it];  // {segment, first unit, end unit, 0}
        __syncthreads();                 // the previous item's readers are done
        const uint32_t base = item.x * SEG_P;
        const uint32_t cnt = min(SEG_P, A.n - base);
        const float4* src4 = reinterpret_cast<const float4*>(A.y + base);
        float4* dst4 = reinterpret_cast<float4*>(seg_ys);
        for (uint32_t i = threadIdx.x; i < cnt / 4; i += P1_NT) dst4[i] = __ldcg(src4 + i);
        for (uint32_t i = (cnt / 4) * 4 + threadIdx.x; i < cnt; i += P1_NT) seg_ys[i] = A.y[base + i];
        __syncthreads();
        for (uint32_t u = item.y + warp; u < item.z; u += P1_WARPS)
            seg_unit<W>(A, seg_ys, A.unit_e[u], A.unit_e[u + 1], A.unit_o[u], lane);
    }
}

__global__ void __launch_bounds__(P2_NT, 1) k_seg_rows(SegArgs A) {
    extern __shared__ float2 seg_acc[];  // [P2_WARPS][SEG_G] compensated sums
    __shared__ double fa[P2_WARPS], fb[P2_WARPS];
    __shared__ bool last;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    float2* acc = seg_acc + warp * SEG_G;
    for (uint32_t d = lane; d < SEG_G; d += 32) acc[d] = make_float2(0.f, 0.f);
    __syncwarp();
    const uint32_t g = blockIdx.x * P2_WARPS + warp;
    const uint32_t lm = lanemask_le();
    Kahan ka, kb;
    if (g < A.ngroups) {
        const uint32_t pb = A.gpair[g], pe = A.gpair[g + 1];
        uint32_t p = pb + lane;
        uint32_t pd = p < pe ? (uint32_t)A.pdest[p] : 0u;
        float x = p < pe ? A.partial[p] : 0.f;
        for (uint32_t w0 = pb; w0 < pe; w0 += 32) {
            const bool valid = w0 + lane < pe;
            const uint32_t cpd = pd;
            const float cx = x;
            // the next window's loads are in flight while this one is added
            const uint32_t pn = w0 + 32 + lane;
            if (pn < pe) pd = A.pdest[pn], x = A.partial[pn];
            const uint32_t rs = __ballot_sync(0xffffffffu, valid && (cpd >> 15));
            const uint32_t my_run = __popc(rs & lm);
            const uint32_t nruns = __popc(rs);
            for (uint32_t r = 0; r <= nruns; ++r) {
                if (valid && my_run == r) {
                    float2 a = acc[cpd & (SEG_G - 1)];
                    float t, e;
                    two_sum(a.x, cx, t, e);
                    a.x = t;
                    a.y = __fadd_rn(a.y, e);
                    acc[cpd & (SEG_G - 1)] = a;
                }
                __syncwarp();
            }
        }
        // the PageRank epilogue of the group's vertices
        const float psink = (float)*A.psink;
        for (uint32_t d = lane; d < SEG_G; d += 32) {
            const uint32_t v = g * SEG_G + d;
            if (v >= A.n) break;
            const float2 a = acc[d];
            const float sum = __fadd_rn(a.x, a.y);
            const float pv = A.pers ? __ldcs(A.pers + v) : A.uniform;
            const float r = __fadd_rn(__fmul_rn(psink, pv), sum);
            const float nv = __fadd_rn(__fmul_rn(A.one_minus_d, pv), __fmul_rn(A.d, r));
            __stcs(A.next + v, nv);
            A.ynext[v] = __fmul_rn(nv, __ldcs(A.invdeg + v));
            ka.add(fabsf(__fsub_rn(nv, __ldcs(A.prev + v))));
            if (__ldcs(A.sink + v)) kb.add(nv);
        }
    }
    // fold: lanes (fixed shuffle order), warps, CTAs (fixed order, last CTA)
    warp_merge_kahan(ka);
    warp_merge_kahan(kb);
    if (lane == 0) {
        fa[warp] = (double)ka.s + (double)ka.c;
        fb[warp] = (double)kb.s + (double)kb.c;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double ta = 0.0, tb = 0.0;
        for (int w = 0; w < P2_WARPS; ++w) ta += fa[w], tb += fb[w];
        A.part[2 * blockIdx.x] = ta;
        A.part[2 * blockIdx.x + 1] = tb;
        __threadfence();
        last = atomicAdd(A.ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (last && warp == 0) {
        __threadfence();
        double ta = 0.0, tb = 0.0;
        for (uint32_t b = lane; b < gridDim.x; b += 32) {
            ta += __ldcg(A.part + 2 * b);
            tb += __ldcg(A.part + 2 * b + 1);
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

__global__ void k_seg_gather_w(uint32_t m, const uint32_t* __restrict__ seid, const void* __restrict__ w,
                               int wdt, float* __restrict__ ws) {
    const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e < m) ws[e] = ld_f32(w, wdt, seid[e]);
}

}  // namespace

bool seg_supported(const View& view) {
    return !view.filtered && view.n > 0 && view.m_pull > 0 && view.n < (1u << 29);
}

// Builds the plan of an unfiltered view on the graph's home stream.
void build_seg(gtc_graph* g, const View& view, cudaStream_t s, SegPlan& P) {
    GTC_CUDA(cudaStreamSynchronize(s));
    cudaStream_t h = g->home;
    uint64_t L = 0;
    const uint32_t n = view.n, m = view.m_pull;
    const unsigned TB = 256;
    const uint32_t nseg = (n + SEG_P - 1) / SEG_P, ngroups = (n + SEG_G - 1) / SEG_G;
    const uint32_t nkeys = nseg * ngroups;
    P.n = n, P.m = m, P.nseg = nseg, P.ngroups = ngroups;

    DevBuf<uint32_t> rowid(m, h), key(m, h), skey(m, h), perm(m, h);
    k_seg_rowid<<<grid_for((size_t)n * 8, TB, 1u << 30), TB, 0, h>>>(n, view.pull_off, rowid.get());
    k_seg_key<<<grid_for(m, TB, 1u << 30), TB, 0, h>>>(m, ngroups, view.pull_other, rowid.get(), key.get());
    GTC_LAUNCHED();
    sort_positions_by_key(key.get(), m, nkeys, skey.get(), perm.get(), h, &L);
    key.release();
    DevBuf<uint32_t> dest(m, h), h1(m, h), id1x((size_t)m + 1, h);
    k_seg_h1<<<grid_for(m, TB, 1u << 30), TB, 0, h>>>(m, perm.get(), skey.get(), rowid.get(), dest.get(),
                                                      h1.get());
    GTC_LAUNCHED();
    rowid.release();
    scan_exclusive_u32(h1.get(), id1x.get(), m, h, &L);
    uint32_t np1 = 0;
    GTC_CUDA(cudaMemcpyAsync(&np1, id1x.get() + m, 4, cudaMemcpyDeviceToHost, h));
    GTC_CUDA(cudaStreamSynchronize(h));
    DevBuf<uint32_t> start1(np1, h), h2(m, h), fpx((size_t)m + 1, h);
    DevBuf<uint8_t> xs(m, h);
    k_seg_mark_start<<<grid_for(m, TB, 1u << 30), TB, 0, h>>>(m, h1.get(), id1x.get(), start1.get());
    k_seg_h2<<<grid_for(m, TB, 1u << 30), TB, 0, h>>>(m, h1.get(), id1x.get(), start1.get(), h2.get(),
                                                      xs.get());
    GTC_LAUNCHED();
    h1.release(), id1x.release(), start1.release();
    scan_exclusive_u32(h2.get(), fpx.get(), m, h, &L);
    uint32_t np = 0;
    GTC_CUDA(cudaMemcpyAsync(&np, fpx.get() + m, 4, cudaMemcpyDeviceToHost, h));
    GTC_CUDA(cudaStreamSynchronize(h));
    P.npairs = np;
    DevBuf<uint32_t> pstart(np, h), pkey(np, h), pv(np, h), cntk((size_t)nkeys + 1, h),
        ecnt((size_t)nkeys + 1, h);
    DevBuf<uint8_t> pxs(np, h);
    GTC_CUDA(cudaMemsetAsync(cntk.get(), 0, ((size_t)nkeys + 1) * 4, h));
    GTC_CUDA(cudaMemsetAsync(ecnt.get(), 0, ((size_t)nkeys + 1) * 4, h));
    k_seg_mark_start<<<grid_for(m, TB, 1u << 30), TB, 0, h>>>(m, h2.get(), fpx.get(), pstart.get());
    k_seg_pairs_info<<<grid_for(np, TB, 1u << 30), TB, 0, h>>>(np, pstart.get(), skey.get(), dest.get(),
                                                               xs.get(), pkey.get(), pv.get(), pxs.get(),
                                                               cntk.get());
    k_seg_edge_counts<<<grid_for(m, TB, 1u << 30), TB, 0, h>>>(m, skey.get(), ecnt.get());
    GTC_LAUNCHED();
    dest.release(), xs.release(), fpx.release();
    // pair bases in key order (phase 1) and transposed (phase 2), edge bases
    DevBuf<uint32_t> base1((size_t)nkeys + 1, h), kes((size_t)nkeys + 1, h), tcnt(nkeys, h),
        base2((size_t)nkeys + 1, h);
    scan_exclusive_u32(cntk.get(), base1.get(), nkeys, h, &L);
    scan_exclusive_u32(ecnt.get(), kes.get(), nkeys, h, &L);
    k_seg_transpose<<<grid_for(nkeys, TB, 1u << 30), TB, 0, h>>>(nseg, ngroups, cntk.get(), tcnt.get());
    GTC_LAUNCHED();
    scan_exclusive_u32(tcnt.get(), base2.get(), nkeys, h, &L);
    cntk.release(), ecnt.release(), tcnt.release();
    P.pdest.alloc(np, h);
    DevBuf<uint32_t> p2(np, h), uflag(np, h), uidx((size_t)np + 1, h);
    k_seg_place<<<grid_for(np, TB, 1u << 30), TB, 0, h>>>(np, nseg, ngroups, pkey.get(), pv.get(), pxs.get(),
                                                          pstart.get(), base1.get(), base2.get(), kes.get(),
                                                          P.pdest.get(), p2.get(), uflag.get());
    GTC_LAUNCHED();
    // group starts in phase-2 order: base2 at (g, segment 0)
    std::vector<uint32_t> hb2((size_t)nkeys + 1);
    GTC_CUDA(cudaMemcpyAsync(hb2.data(), base2.get(), ((size_t)nkeys + 1) * 4, cudaMemcpyDeviceToHost, h));
    // edges
    P.src16.alloc(m, h);
    P.seid.alloc(m, h);
    k_seg_edges<<<grid_for(m, TB, 1u << 30), TB, 0, h>>>(m, perm.get(), view.pull_other, view.pull_eid,
                                                         h2.get(), P.src16.get(), P.seid.get());
    GTC_LAUNCHED();
    perm.release(), h2.release(), skey.release();
    // units
    scan_exclusive_u32(uflag.get(), uidx.get(), np, h, &L);
    uint32_t nu = 0;
    GTC_CUDA(cudaMemcpyAsync(&nu, uidx.get() + np, 4, cudaMemcpyDeviceToHost, h));
    GTC_CUDA(cudaStreamSynchronize(h));
    P.nunits = nu;
    P.unit_e.alloc((size_t)nu + 1, h);
    P.unit_o.alloc(nu, h);
    DevBuf<uint32_t> unit_s(nu, h);
    k_seg_units<<<grid_for(np, TB, 1u << 30), TB, 0, h>>>(np, uflag.get(), uidx.get(), pstart.get(), p2.get(),
                                                          pkey.get(), ngroups, P.unit_e.get(),
                                                          P.unit_o.get(), unit_s.get());
    GTC_LAUNCHED();
    GTC_CUDA(cudaMemcpyAsync(P.unit_e.get() + nu, &m, 4, cudaMemcpyHostToDevice, h));
    std::vector<uint32_t> hue((size_t)nu + 1), hus(nu);
    GTC_CUDA(cudaMemcpyAsync(hue.data(), P.unit_e.get(), (size_t)nu * 4, cudaMemcpyDeviceToHost, h));
    GTC_CUDA(cudaMemcpyAsync(hus.data(), unit_s.get(), (size_t)nu * 4, cudaMemcpyDeviceToHost, h));
    GTC_CUDA(cudaStreamSynchronize(h));
    hue[nu] = m;
    // group starts
    std::vector<uint32_t> gp((size_t)ngroups + 1);
    for (uint32_t gg = 0; gg < ngroups; ++gg) gp[gg] = hb2[(size_t)gg * nseg];
    gp[ngroups] = np;
    P.gpair.alloc((size_t)ngroups + 1, h);
    GTC_CUDA(cudaMemcpyAsync(P.gpair.get(), gp.data(), gp.size() * 4, cudaMemcpyHostToDevice, h));
    // phase-1 CTA items: consecutive units of one segment, about SEG_ITEM edges
    std::vector<uint4> items;
    for (uint32_t u = 0; u < nu;) {
        uint32_t v = u + 1;
        while (v < nu && hus[v] == hus[u] && hue[v + 1] - hue[u] <= SEG_ITEM) ++v;
        items.push_back(make_uint4(hus[u], u, v, 0u));
        u = v;
    }
    P.nitems = (uint32_t)items.size();
    P.items.alloc(items.size(), h);
    GTC_CUDA(cudaMemcpyAsync(P.items.get(), items.data(), items.size() * sizeof(uint4),
                             cudaMemcpyHostToDevice, h));
    P.partial.alloc(np, h);
    GTC_CUDA(cudaStreamSynchronize(h));
    P.built = true;
    g->launches += L + 14;
}

void seg_gather_weights(const SegPlan& P, const DVec& w, float* ws, cudaStream_t s) {
    k_seg_gather_w<<<grid_for(P.m, 256, 1u << 30), 256, 0, s>>>((uint32_t)P.m, P.seid.get(), w.p,
                                                                w.dtype, ws);
    GTC_LAUNCHED();
}

void seg_sweep(const SegPlan& P, SegArgs A, bool weighted, cudaStream_t s) {
    A.n = P.n, A.ngroups = P.ngroups, A.nitems = P.nitems;
    A.src16 = P.src16.get(), A.unit_e = P.unit_e.get(), A.unit_o = P.unit_o.get();
    A.items = P.items.get(), A.pdest = P.pdest.get(), A.gpair = P.gpair.get();
    A.partial = P.partial.get();
    int sms = 0, dev = 0;
    GTC_CUDA(cudaGetDevice(&dev));
    GTC_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const size_t sm1 = SEG_P * sizeof(float), sm2 = (size_t)P2_WARPS * SEG_G * sizeof(float2);
    GTC_CUDA(cudaFuncSetAttribute(weighted ? k_seg_pairs<true> : k_seg_pairs<false>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm1));
    GTC_CUDA(cudaFuncSetAttribute(k_seg_rows, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm2));
    const unsigned g1 = (unsigned)std::min<uint32_t>(P.nitems, (uint32_t)sms);
    if (weighted)
        k_seg_pairs<true><<<std::max(1u, g1), P1_NT, sm1, s>>>(A);
    else
        k_seg_pairs<false><<<std::max(1u, g1), P1_NT, sm1, s>>>(A);
    GTC_LAUNCHED();
    const unsigned g2 = (P.ngroups + P2_WARPS - 1) / P2_WARPS;
    k_seg_rows<<<g2, P2_NT, sm2, s>>>(A);
    GTC_LAUNCHED();
}

uint32_t seg_part_slots(const SegPlan& P) { return 2 * ((P.ngroups + P2_WARPS - 1) / P2_WARPS); }

}  // namespace gtc
