// gtc_build.cu -- the bit-exact CSR/CSC build.
//
// Input: an edge list (src[k], tgt[k]), k = 0..m-1, read as the call sequence
// AdjList::add_edge(src[k], tgt[k]) of the reference
// (crates/gt-core/src/adj/list.rs:258-280).  Output: every vertex block's
// out-half and in-half, flattened, in exactly the storage order the reference
// leaves them in:
//
//   * out-half: Block::insert_out appends at out_len (block.rs:171-197), so
//     an out-half is its edges in insertion (= EdgeId) order.  A stable sort
//     of the edge ids by source gives it.
//   * in-half: Block::insert_in appends (block.rs:205-209), but every later
//     insert_out on the same block moves the in-half's FIRST entry to its
//     back.  Seen per vertex, the in-half is a FIFO queue: an in-edge pushes,
//     an out-edge (once the queue is non-empty) pops the front and pushes it
//     again.  A stable sort by target gives the pushes in order; k_fix_place
//     below moves every entry to the position the rotations leave it at.
//
// All kernels are integer-only; the result is compared byte for byte with the
// CPU oracle's blocks.
#include <algorithm>

#include "gtc_internal.cuh"

namespace gtc {

// --------------------------------------------------------------------------
// exclusive scan (u32), reduce-then-scan over tiles of 2048
// --------------------------------------------------------------------------

constexpr int SCAN_NT = 256, SCAN_IPT = 8, SCAN_TILE = SCAN_NT * SCAN_IPT;

// Block-wide exclusive scan of one value per thread (blockDim == 256).
__device__ __forceinline__ uint32_t block_exscan_256(uint32_t v, uint32_t* total) {
    __shared__ uint32_t wt[SCAN_NT / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) wt[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t t = lane < SCAN_NT / 32 ? wt[lane] : 0u;
#pragma unroll
        for (int o = 1; o < SCAN_NT / 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        if (lane < SCAN_NT / 32) wt[lane] = t;
    }
    __syncthreads();
    uint32_t off = warp ? wt[warp - 1] : 0u;
    *total = wt[SCAN_NT / 32 - 1];
    __syncthreads();
    return off + x - v;
}

__global__ void __launch_bounds__(SCAN_NT) k_tile_reduce(const uint32_t* __restrict__ in, size_t n,
                                                        uint32_t* __restrict__ sums) {
    size_t base = (size_t)blockIdx.x * SCAN_TILE;
    uint32_t s = 0;
#pragma unroll
    for (int i = 0; i < SCAN_IPT; ++i) {
        size_t idx = base + (size_t)i * SCAN_NT + threadIdx.x;
        if (idx < n) s += in[idx];
    }
    uint32_t tot;
    (void)block_exscan_256(s, &tot);
    if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

// Scans one tile; block offsets come from `offs` (already exclusive-scanned).
// The block holding the last element also writes out[n] = grand total.  `in`
// may equal `out`: a block reads its whole tile before writing it.
__global__ void __launch_bounds__(SCAN_NT) k_tile_scan(const uint32_t* in, uint32_t* out, size_t n,
                                                      const uint32_t* __restrict__ offs) {
    __shared__ uint32_t sm[SCAN_TILE];
    size_t base = (size_t)blockIdx.x * SCAN_TILE;
#pragma unroll
    for (int i = 0; i < SCAN_IPT; ++i) {
        size_t idx = base + (size_t)i * SCAN_NT + threadIdx.x;
        sm[i * SCAN_NT + threadIdx.x] = idx < n ? in[idx] : 0u;
    }
    __syncthreads();
    uint32_t loc[SCAN_IPT], s = 0;
#pragma unroll
    for (int i = 0; i < SCAN_IPT; ++i) {
        loc[i] = sm[threadIdx.x * SCAN_IPT + i];
        s += loc[i];
    }
    uint32_t tot;
    uint32_t ex = block_exscan_256(s, &tot);
    uint32_t off = offs ? offs[blockIdx.x] : 0u;
    uint32_t run = off + ex;
#pragma unroll
    for (int i = 0; i < SCAN_IPT; ++i) {
        sm[threadIdx.x * SCAN_IPT + i] = run;
        run += loc[i];
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < SCAN_IPT; ++i) {
        size_t idx = base + (size_t)i * SCAN_NT + threadIdx.x;
        if (idx < n) out[idx] = sm[i * SCAN_NT + threadIdx.x];
    }
    if (threadIdx.x == 0 && base + SCAN_TILE >= n) out[n] = off + tot;
}

void scan_exclusive_u32(const uint32_t* in, uint32_t* out, size_t n, cudaStream_t s,
                        uint64_t* launches) {
    if (n == 0) {
        GTC_CUDA(cudaMemsetAsync(out, 0, sizeof(uint32_t), s));
        return;
    }
    size_t tiles = (n + SCAN_TILE - 1) / SCAN_TILE;
    if (tiles == 1) {
        k_tile_scan<<<1, SCAN_NT, 0, s>>>(in, out, n, nullptr);
        GTC_LAUNCHED();
        if (launches) *launches += 1;
        return;
    }
    DevBuf<uint32_t> sums(tiles + 1, s);
    k_tile_reduce<<<(unsigned)tiles, SCAN_NT, 0, s>>>(in, n, sums.get());
    GTC_LAUNCHED();
    scan_exclusive_u32(sums.get(), sums.get(), tiles, s, launches);
    k_tile_scan<<<(unsigned)tiles, SCAN_NT, 0, s>>>(in, out, n, sums.get());
    GTC_LAUNCHED();
    if (launches) *launches += 2;
}

// --------------------------------------------------------------------------
// stable LSD radix sort of (key, value) pairs, 8-bit digits
// --------------------------------------------------------------------------

constexpr int RS_NT = 256, RS_IPT = 8, RS_TILE = RS_NT * RS_IPT, RS_WARPS = RS_NT / 32;

__global__ void __launch_bounds__(RS_NT) k_radix_hist(const uint32_t* __restrict__ keys, size_t n,
                                                     int shift, uint32_t* __restrict__ counts,
                                                     uint32_t ntiles) {
    __shared__ uint32_t h[256];
    for (int i = threadIdx.x; i < 256; i += RS_NT) h[i] = 0;
    __syncthreads();
    size_t base = (size_t)blockIdx.x * RS_TILE;
#pragma unroll
    for (int i = 0; i < RS_IPT; ++i) {
        size_t idx = base + (size_t)i * RS_NT + threadIdx.x;
        if (idx < n) atomicAdd(&h[(keys[idx] >> shift) & 255u], 1u);
    }
    __syncthreads();
    for (int d = threadIdx.x; d < 256; d += RS_NT) counts[(size_t)d * ntiles + blockIdx.x] = h[d];
}

// Stable scatter of one tile.  Warp w owns the contiguous slice
// [w*32*IPT, (w+1)*32*IPT) of the tile and walks it in rounds of 32
// consecutive items, so (warp, round, lane) is index order; equal digits
// inside a round are ranked by lane with __match_any_sync.
__global__ void __launch_bounds__(RS_NT) k_radix_scatter(
    const uint32_t* __restrict__ kin, const uint32_t* __restrict__ vin, uint32_t* __restrict__ kout,
    uint32_t* __restrict__ vout, size_t n, int shift, const uint32_t* __restrict__ offs,
    uint32_t ntiles) {
    __shared__ uint32_t wh[RS_WARPS][256];
    __shared__ uint32_t tb[256];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int i = threadIdx.x; i < RS_WARPS * 256; i += RS_NT) (&wh[0][0])[i] = 0;
    for (int d = threadIdx.x; d < 256; d += RS_NT) tb[d] = offs[(size_t)d * ntiles + blockIdx.x];
    __syncthreads();

    const size_t base = (size_t)blockIdx.x * RS_TILE + (size_t)warp * 32 * RS_IPT;
    uint32_t key[RS_IPT], val[RS_IPT], rank[RS_IPT];
#pragma unroll
    for (int r = 0; r < RS_IPT; ++r) {
        size_t idx = base + (size_t)r * 32 + lane;
        bool valid = idx < n;
        key[r] = valid ? kin[idx] : 0u;
        val[r] = valid ? (vin ? vin[idx] : (uint32_t)idx) : 0u;
        rank[r] = 0;
        unsigned act = __ballot_sync(0xffffffffu, valid);
        if (valid) {
            uint32_t d = (key[r] >> shift) & 255u;
            unsigned peers = __match_any_sync(act, d);
            int leader = __ffs(peers) - 1;
            uint32_t before = __popc(peers & ((1u << lane) - 1u));
            uint32_t old = 0;
            if (lane == leader) {
                old = wh[warp][d];
                wh[warp][d] = old + __popc(peers);
            }
            old = __shfl_sync(peers, old, leader);
            rank[r] = old + before;
        }
        __syncwarp();
    }
    __syncthreads();
    // exclusive scan of each digit's count over the warps, in warp order
    for (int d = threadIdx.x; d < 256; d += RS_NT) {
        uint32_t run = 0;
#pragma unroll
        for (int w = 0; w < RS_WARPS; ++w) {
            uint32_t t = wh[w][d];
            wh[w][d] = run;
            run += t;
        }
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < RS_IPT; ++r) {
        size_t idx = base + (size_t)r * 32 + lane;
        if (idx < n) {
            uint32_t d = (key[r] >> shift) & 255u;
            uint32_t dst = tb[d] + wh[warp][d] + rank[r];
            kout[dst] = key[r];
            vout[dst] = val[r];
        }
    }
}

// Stable sort of the index sequence 0..n-1 by keys[] (all keys < key_bound).
// keys_out receives the sorted keys, vals_out the original positions.
void sort_positions_by_key(const uint32_t* keys, size_t n, uint32_t key_bound,
                                  uint32_t* keys_out, uint32_t* vals_out, cudaStream_t s,
                                  uint64_t* launches) {
    if (n == 0) return;
    int bits = key_bound <= 1 ? 0 : 32 - __builtin_clz(key_bound - 1);
    int passes = std::max(1, (bits + 7) / 8);
    size_t ntiles = (n + RS_TILE - 1) / RS_TILE;
    DevBuf<uint32_t> counts(256 * ntiles + 1, s);
    DevBuf<uint32_t> kt(n, s), vt(n, s);
    // the last pass must land in the output buffers
    uint32_t* kb[2] = {keys_out, kt.get()};
    uint32_t* vb[2] = {vals_out, vt.get()};
    int dst = (passes % 2 == 1) ? 0 : 1;
    const uint32_t* kcur = keys;
    const uint32_t* vcur = nullptr;  // identity on the first pass
    for (int p = 0; p < passes; ++p) {
        int shift = 8 * p;
        k_radix_hist<<<(unsigned)ntiles, RS_NT, 0, s>>>(kcur, n, shift, counts.get(),
                                                       (uint32_t)ntiles);
        GTC_LAUNCHED();
        scan_exclusive_u32(counts.get(), counts.get(), 256 * ntiles, s, launches);
        k_radix_scatter<<<(unsigned)ntiles, RS_NT, 0, s>>>(kcur, vcur, kb[dst], vb[dst], n, shift,
                                                          counts.get(), (uint32_t)ntiles);
        GTC_LAUNCHED();
        if (launches) *launches += 2;
        kcur = kb[dst];
        vcur = vb[dst];
        dst ^= 1;
    }
}

// --------------------------------------------------------------------------
// offsets, gathers, validation
// --------------------------------------------------------------------------

// off[v] = first position p with sorted[p] >= v, for v in 0..n (off[n] = m).
__global__ void k_offsets_from_sorted(const uint32_t* __restrict__ sorted, uint32_t m, uint32_t n,
                                      uint32_t* __restrict__ off) {
    size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v > n) return;
    uint32_t lo = 0, hi = m;
    while (lo < hi) {
        uint32_t mid = lo + (hi - lo) / 2;
        if (sorted[mid] < (uint32_t)v)
            lo = mid + 1;
        else
            hi = mid;
    }
    off[v] = lo;
}

__global__ void k_gather_u32(const uint32_t* __restrict__ idx, const uint32_t* __restrict__ table,
                             uint32_t* __restrict__ out, uint32_t m) {
    size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p < m) out[p] = table[idx[p]];
}

__global__ void k_validate(const uint32_t* __restrict__ src, const uint32_t* __restrict__ tgt,
                           uint32_t m, uint32_t n, unsigned* bad) {
    size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    bool b = p < m && (src[p] >= n || tgt[p] >= n);
    if (__any_sync(0xffffffffu, b) && (threadIdx.x & 31) == 0) atomicOr(bad, 1u);
}

// --------------------------------------------------------------------------
// the in-half rotation
// --------------------------------------------------------------------------
//
// Per vertex v: the in-edges a_0 < a_1 < ... < a_{k-1} (ids, insertion order)
// and the out-edges b_0 < b_1 < ... (ids).  An out-edge b happens before
// in-edge a iff b <= a (a self-loop's out splice precedes its in splice,
// list.rs:480-487).  cnt_j = #{b <= a_j}.
//
// Queue model: in-edge j pushes; an out-edge after the first in-edge pops the
// front and pushes it again.  Number the pushes 0,1,2,...; the rotations
// between in-edge t and in-edge t+1 ("stretch t", queue length t+1) have
// ordinals [S_t, S_{t+1}) with S_t = cnt_t - cnt_0 and S_k = R = outdeg - cnt_0
// (rotations before the first in-edge rotate an empty queue and do nothing).
// In-edge j is push j + S_j.  The element of push p is popped by rotation
// ordinal p (FIFO) if p < R, and re-pushed as push p + (t+1) where t is the
// stretch holding ordinal p.  Inside one stretch that repeats with a fixed
// step t+1, so it is jumped in O(1).  The final queue is pushes [R, R+k), so
// an entry's position is (its last push) - R.

__global__ void k_fix_count(uint32_t m, const uint32_t* __restrict__ rowkey,
                            const uint32_t* __restrict__ in_sorted,
                            const uint32_t* __restrict__ out_off,
                            const uint32_t* __restrict__ out_eid, uint32_t* __restrict__ cnt) {
    size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= m) return;
    uint32_t v = rowkey[p], a = in_sorted[p];
    uint32_t b0 = out_off[v], lo = b0, hi = out_off[v + 1];
    while (lo < hi) {  // upper bound of a among the out-edge ids of v
        uint32_t mid = lo + (hi - lo) / 2;
        if (out_eid[mid] <= a)
            lo = mid + 1;
        else
            hi = mid;
    }
    cnt[p] = lo - b0;
}

__global__ void k_fix_place(uint32_t m, const uint32_t* __restrict__ rowkey,
                            const uint32_t* __restrict__ in_sorted,
                            const uint32_t* __restrict__ in_off,
                            const uint32_t* __restrict__ out_off, const uint32_t* __restrict__ cnt,
                            uint32_t* __restrict__ in_eid, unsigned* __restrict__ bad) {
    size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= m) return;
    const uint32_t v = rowkey[p];
    const uint32_t base = in_off[v];
    const uint32_t k = in_off[v + 1] - base;
    const uint32_t j = (uint32_t)p - base;
    const uint32_t c0 = cnt[base];
    const uint64_t R = (uint64_t)(out_off[v + 1] - out_off[v]) - c0;
    uint64_t pp = (uint64_t)j + (cnt[p] - c0);
    uint32_t tlo = j;  // the stretch of push pp is never before j
    while (pp < R) {
        // t = largest index in [tlo, k) with cnt[base+t] - c0 <= pp
        uint32_t lo = tlo + 1, hi = k;
        while (lo < hi) {
            uint32_t mid = lo + (hi - lo) / 2;
            if ((uint64_t)(cnt[base + mid] - c0) <= pp)
                lo = mid + 1;
            else
                hi = mid;
        }
        uint32_t t = lo - 1;
        uint64_t s_next = (t + 1 < k) ? (uint64_t)(cnt[base + t + 1] - c0) : R;
        uint64_t L = (uint64_t)t + 1;
        uint64_t steps = (s_next - pp + L - 1) / L;
        pp += steps * L;
        tlo = t + 1 < k ? t + 1 : t;
    }
    // pp - R < k holds by construction; a violation is reported, not written
    if (pp - R < k)
        in_eid[base + (uint32_t)(pp - R)] = in_sorted[p];
    else
        atomicOr(bad, 2u);
}

// --------------------------------------------------------------------------
// relabelling by descending out-degree
// --------------------------------------------------------------------------

__global__ void k_degree_key(uint32_t n, const uint32_t* __restrict__ off, uint32_t* __restrict__ deg,
                             unsigned* __restrict__ maxdeg) {
    size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t d = v < n ? off[v + 1] - off[v] : 0u;
    if (v < n) deg[v] = d;
    // warp max, one atomic per warp
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) d = max(d, __shfl_xor_sync(0xffffffffu, d, o));
    if ((threadIdx.x & 31) == 0) atomicMax(maxdeg, d);
}

__global__ void k_desc_key(uint32_t n, const uint32_t* __restrict__ deg, uint32_t maxdeg,
                           uint32_t* __restrict__ key) {
    size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v < n) key[v] = maxdeg - deg[v];
}

__global__ void k_invert(uint32_t n, const uint32_t* __restrict__ perm, uint32_t* __restrict__ iperm) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) iperm[perm[i]] = (uint32_t)i;
}

__global__ void k_new_degrees(uint32_t n, const uint32_t* __restrict__ perm,
                              const uint32_t* __restrict__ off, uint32_t* __restrict__ deg) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) deg[i] = off[perm[i] + 1] - off[perm[i]];
}

// One warp per new row: copy the old block half in order, relabelling the
// other endpoint (looked up by edge id in the original edge list).
__global__ void k_permute_rows(uint32_t n, const uint32_t* __restrict__ perm,
                               const uint32_t* __restrict__ iperm,
                               const uint32_t* __restrict__ old_off,
                               const uint32_t* __restrict__ old_eid,
                               const uint32_t* __restrict__ endpoint,
                               const uint32_t* __restrict__ new_off, uint32_t* __restrict__ new_eid,
                               uint32_t* __restrict__ new_other) {
    const unsigned lane = threadIdx.x & 31;
    const size_t nw = ((size_t)gridDim.x * blockDim.x) >> 5;
    for (size_t i = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < n; i += nw) {
        const uint32_t v = perm[i];
        const uint32_t b = old_off[v], e = old_off[v + 1], nb = new_off[i];
        for (uint32_t p = b + lane; p < e; p += 32) {
            const uint32_t id = old_eid[p];
            new_eid[nb + (p - b)] = id;
            new_other[nb + (p - b)] = iperm[endpoint[id]];
        }
    }
}

static void relabel_half(uint32_t n, uint32_t m, const uint32_t* perm, const uint32_t* iperm,
                         const uint32_t* endpoint, Halves& h, cudaStream_t s, uint64_t* L) {
    const unsigned TB = 256;
    Halves nh;
    nh.off.alloc((size_t)n + 1, s);
    nh.eid.alloc(m, s);
    nh.other.alloc(m, s);
    DevBuf<uint32_t> deg(n, s);
    if (n) {
        k_new_degrees<<<grid_for(n, TB, 1u << 30), TB, 0, s>>>(n, perm, h.off.get(), deg.get());
        GTC_LAUNCHED();
        *L += 1;
    }
    scan_exclusive_u32(deg.get(), nh.off.get(), n, s, L);
    if (n && m) {
        k_permute_rows<<<sm_count() * 16, TB, 0, s>>>(n, perm, iperm, h.off.get(), h.eid.get(), endpoint,
                                               nh.off.get(), nh.eid.get(), nh.other.get());
        GTC_LAUNCHED();
        *L += 1;
    }
    h = std::move(nh);
}

__global__ void k_iota(uint32_t n, uint32_t* __restrict__ a, uint32_t* __restrict__ b) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] = b[i] = (uint32_t)i;
}

void build_halves(gtc_graph* g, const uint32_t* d_src, const uint32_t* d_tgt, bool relabel) {
    cudaStream_t s = g->home;
    const uint32_t n = g->n, m = g->m;
    const unsigned TB = 256;
    uint64_t L = 0;

    g->out.off.alloc((size_t)n + 1, s);
    g->in.off.alloc((size_t)n + 1, s);
    g->out.other.alloc(m, s);
    g->out.eid.alloc(m, s);
    g->in.other.alloc(m, s);
    g->in.eid.alloc(m, s);

    if (m > 0) {
        DevBuf<unsigned> bad(1, s);
        GTC_CUDA(cudaMemsetAsync(bad.get(), 0, sizeof(unsigned), s));
        k_validate<<<grid_for(m, TB, 1u << 30), TB, 0, s>>>(d_src, d_tgt, m, n, bad.get());
        GTC_LAUNCHED();
        unsigned hbad = 0;
        GTC_CUDA(cudaMemcpyAsync(&hbad, bad.get(), sizeof(unsigned), cudaMemcpyDeviceToHost, s));
        GTC_CUDA(cudaStreamSynchronize(s));
        L += 1;
        GTC_REQUIRE(!hbad, GTC_ERR_ARG, "add_edge: no such vertex (an endpoint is >= n)");
    }

    DevBuf<uint32_t> keys(m, s);
    if (m > 0) {
        // out-halves: stable by source, insertion order inside
        sort_positions_by_key(d_src, m, n, keys.get(), g->out.eid.get(), s, &L);
    }
    k_offsets_from_sorted<<<grid_for((size_t)n + 1, TB, 1u << 30), TB, 0, s>>>(keys.get(), m, n,
                                                                            g->out.off.get());
    GTC_LAUNCHED();
    L += 1;

    // in-halves: stable by target (push order), then the rotation
    DevBuf<uint32_t> in_sorted(m, s);
    if (m > 0) sort_positions_by_key(d_tgt, m, n, keys.get(), in_sorted.get(), s, &L);
    k_offsets_from_sorted<<<grid_for((size_t)n + 1, TB, 1u << 30), TB, 0, s>>>(keys.get(), m, n,
                                                                            g->in.off.get());
    GTC_LAUNCHED();
    L += 1;
    if (m > 0) {
        DevBuf<uint32_t> cnt(m, s);
        DevBuf<unsigned> bad(1, s);
        GTC_CUDA(cudaMemsetAsync(bad.get(), 0, sizeof(unsigned), s));
        unsigned gb = grid_for(m, TB, 1u << 30);
        k_fix_count<<<gb, TB, 0, s>>>(m, keys.get(), in_sorted.get(), g->out.off.get(),
                                      g->out.eid.get(), cnt.get());
        GTC_LAUNCHED();
        k_fix_place<<<gb, TB, 0, s>>>(m, keys.get(), in_sorted.get(), g->in.off.get(),
                                      g->out.off.get(), cnt.get(), g->in.eid.get(), bad.get());
        GTC_LAUNCHED();
        unsigned hbad = 0;
        GTC_CUDA(cudaMemcpyAsync(&hbad, bad.get(), sizeof(unsigned), cudaMemcpyDeviceToHost, s));
        GTC_CUDA(cudaStreamSynchronize(s));
        GTC_REQUIRE(!hbad, GTC_ERR_CUDA, "in-half placement left its segment (internal error)");
        L += 2;
    }

    relabel_graph(g, d_src, d_tgt, relabel, &L);
    GTC_CUDA(cudaStreamSynchronize(s));
    g->launches += L;
}

// The relabelling of a graph whose halves are built in original labels:
// vertices by descending out-degree (stable: ties keep index order), or
// kept as they are (a packed batch of graphs: each graph stays contiguous),
// and both halves rewritten in the new labels with every block's order
// kept.  src_of / tgt_of: the endpoints of every edge id (edge bound
// entries; ids without an edge are never read).
void relabel_graph(gtc_graph* g, const uint32_t* src_of, const uint32_t* tgt_of, bool relabel,
                   uint64_t* Lp) {
    cudaStream_t s = g->home;
    const uint32_t n = g->n, m = g->m_live;
    const unsigned TB = 256;
    uint64_t& L = *Lp;
    g->perm.alloc(n, s);
    g->iperm.alloc(n, s);
    if (n && !relabel) {
        k_iota<<<grid_for(n, TB, 1u << 30), TB, 0, s>>>(n, g->perm.get(), g->iperm.get());
        GTC_LAUNCHED();
        L += 1;
    } else if (n) {
        DevBuf<uint32_t> deg(n, s), key(n, s), skey(n, s);
        DevBuf<unsigned> mx(1, s);
        GTC_CUDA(cudaMemsetAsync(mx.get(), 0, sizeof(unsigned), s));
        k_degree_key<<<grid_for(n, TB, 1u << 30), TB, 0, s>>>(n, g->out.off.get(), deg.get(), mx.get());
        GTC_LAUNCHED();
        unsigned maxdeg = 0;
        GTC_CUDA(cudaMemcpyAsync(&maxdeg, mx.get(), sizeof(unsigned), cudaMemcpyDeviceToHost, s));
        GTC_CUDA(cudaStreamSynchronize(s));
        k_desc_key<<<grid_for(n, TB, 1u << 30), TB, 0, s>>>(n, deg.get(), maxdeg, key.get());
        GTC_LAUNCHED();
        sort_positions_by_key(key.get(), n, maxdeg + 1, skey.get(), g->perm.get(), s, &L);
        k_invert<<<grid_for(n, TB, 1u << 30), TB, 0, s>>>(n, g->perm.get(), g->iperm.get());
        GTC_LAUNCHED();
        L += 3;
    }
    relabel_half(n, m, g->perm.get(), g->iperm.get(), tgt_of, g->out, s, &L);
    relabel_half(n, m, g->perm.get(), g->iperm.get(), src_of, g->in, s, &L);
}

void build_from_blocks(gtc_graph* g, const uint64_t* block_off, const uint32_t* out_len,
                       const uint32_t* entries) {
    cudaStream_t s = g->home;
    const uint32_t n = g->n, eb = g->m;
    constexpr uint32_t NONE = 0xFFFFFFFFu;
    uint64_t L = 0;
    // ---- the blocks, split into their halves, checked on the host ----
    GTC_REQUIRE(n == 0 || (block_off && out_len), GTC_ERR_ARG, "block_off / out_len is NULL");
    GTC_REQUIRE(n == 0 || block_off[0] == 0, GTC_ERR_ARG, "block_off[0] must be 0");
    uint64_t mo = 0, mi = 0;
    for (uint32_t v = 0; v < n; ++v) {
        GTC_REQUIRE(block_off[v + 1] >= block_off[v], GTC_ERR_ARG, "block offsets must not decrease");
        const uint64_t len = block_off[v + 1] - block_off[v];
        GTC_REQUIRE(out_len[v] <= len, GTC_ERR_ARG, "a block's out_len exceeds its length");
        mo += out_len[v];
        mi += len - out_len[v];
    }
    GTC_REQUIRE(mo == mi, GTC_ERR_ARG,
                "the blocks hold a different number of out-entries and in-entries");
    GTC_REQUIRE(mo <= eb, GTC_ERR_ARG, "more live edges than the edge bound");
    GTC_REQUIRE(mo == 0 || entries, GTC_ERR_ARG, "entries is NULL");
    const uint32_t m = (uint32_t)mo;
    g->m_live = m;
    std::vector<uint32_t> src_of(eb, NONE), tgt_of(eb, NONE);
    std::vector<uint32_t> oo((size_t)n + 1), io((size_t)n + 1), oth(m), oid(m), ith(m), iid(m);
    uint64_t po = 0;
    for (uint32_t v = 0; v < n; ++v) {  // out-halves: (target, id) in storage order
        oo[v] = (uint32_t)po;
        for (uint64_t k = block_off[v], e = block_off[v] + out_len[v]; k < e; ++k, ++po) {
            const uint32_t t = entries[2 * k], id = entries[2 * k + 1];
            GTC_REQUIRE(t < n, GTC_ERR_INDEX, "a block entry names a vertex >= n");
            GTC_REQUIRE(id < eb, GTC_ERR_INDEX, "a block entry names an edge id >= edge_bound");
            GTC_REQUIRE(src_of[id] == NONE, GTC_ERR_ARG, "an edge id appears in two out-halves");
            src_of[id] = v;
            tgt_of[id] = t;
            oth[po] = t;
            oid[po] = id;
        }
    }
    oo[n] = (uint32_t)po;
    std::vector<uint8_t> seen(eb, 0);
    uint64_t pi = 0;
    for (uint32_t v = 0; v < n; ++v) {  // in-halves: (source, id) in storage order
        io[v] = (uint32_t)pi;
        for (uint64_t k = block_off[v] + out_len[v], e = block_off[v + 1]; k < e; ++k, ++pi) {
            const uint32_t src = entries[2 * k], id = entries[2 * k + 1];
            GTC_REQUIRE(src < n, GTC_ERR_INDEX, "a block entry names a vertex >= n");
            GTC_REQUIRE(id < eb, GTC_ERR_INDEX, "a block entry names an edge id >= edge_bound");
            GTC_REQUIRE(src_of[id] == src && tgt_of[id] == v && !seen[id], GTC_ERR_ARG,
                        "an in-entry does not match its edge's out-entry");
            seen[id] = 1;
            ith[pi] = src;
            iid[pi] = id;
        }
    }
    io[n] = (uint32_t)pi;
    // ---- to the device, then the relabelling every handle gets ----
    auto up = [&](DevBuf<uint32_t>& d, const std::vector<uint32_t>& h) {
        d.alloc(h.size(), s);
        if (!h.empty())
            GTC_CUDA(cudaMemcpyAsync(d.get(), h.data(), h.size() * 4, cudaMemcpyHostToDevice, s));
    };
    up(g->out.off, oo);
    up(g->out.other, oth);
    up(g->out.eid, oid);
    up(g->in.off, io);
    up(g->in.other, ith);
    up(g->in.eid, iid);
    DevBuf<uint32_t> dso, dto;
    up(dso, src_of);
    up(dto, tgt_of);
    relabel_graph(g, dso.get(), dto.get(), true, &L);
    GTC_CUDA(cudaStreamSynchronize(s));  // the host vectors die here
    g->launches += L;
}

}  // namespace gtc
