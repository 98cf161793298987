// gtc_sweep.cu -- building the in-degree tiers of a pull half (see
// gtc_sweep.cuh): sliced rows in the column-major sliced-ELL layout, medium
// rows, long rows in chunks, and the work list.
#include <vector>

#include "gtc_sweep.cuh"

namespace gtc {

namespace {

constexpr uint32_t KEY_STRIDE = SP_SLICE_MAX + 2;  // per window: lengths 0..MAX, then "not sliced"

__global__ void k_tier_keys(uint32_t n, const uint32_t* __restrict__ off, uint32_t* __restrict__ key,
                            uint32_t* __restrict__ is_med, uint32_t* __restrict__ is_long) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t d = off[i + 1] - off[i];
    const uint32_t win = (uint32_t)(i / SP_WINDOW);
    // longest first inside a window; rows that are not sliced sort last
    key[i] = win * KEY_STRIDE + (d <= (uint32_t)SP_SLICE_MAX ? (uint32_t)SP_SLICE_MAX - d
                                                              : (uint32_t)SP_SLICE_MAX + 1);
    is_med[i] = (d > (uint32_t)SP_SLICE_MAX && d <= (uint32_t)SP_CAP) ? 1u : 0u;
    is_long[i] = d > (uint32_t)SP_CAP ? 1u : 0u;
}

// flag[p] = order[p] is a sliced row
__global__ void k_sliced_flags(uint32_t n, const uint32_t* __restrict__ order,
                               const uint32_t* __restrict__ off, uint32_t* __restrict__ flag) {
    size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const uint32_t r = order[p];
    flag[p] = (off[r + 1] - off[r] <= (uint32_t)SP_SLICE_MAX) ? 1u : 0u;
}

// out[pos[p]] = (src ? src[p] : p) where flag[p]
__global__ void k_compact_u32(uint32_t n, const uint32_t* __restrict__ flag,
                              const uint32_t* __restrict__ pos, const uint32_t* __restrict__ src,
                              uint32_t* __restrict__ out) {
    size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p < n && flag[p]) out[pos[p]] = src ? src[p] : (uint32_t)p;
}

// slice_rows (padded with NO_ROW) and 32 x the longest row of each slice
__global__ void k_slice_rows(uint32_t ns, uint32_t n_slices, const uint32_t* __restrict__ srows,
                             const uint32_t* __restrict__ off, uint32_t* __restrict__ slice_rows,
                             uint32_t* __restrict__ len32) {
    const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t k = (uint32_t)(t >> 5), lane = threadIdx.x & 31;
    if (k >= n_slices) return;  // whole warps exit together
    const size_t q = (size_t)k * 32 + lane;
    const uint32_t r = q < ns ? srows[q] : NO_ROW;
    slice_rows[q] = r;
    uint32_t d = r != NO_ROW ? off[r + 1] - off[r] : 0u;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) d = max(d, __shfl_xor_sync(0xffffffffu, d, o));
    if (lane == 0) len32[k] = 32u * d;
}

// column-major fill of every slice, one warp per slice
__global__ void k_slice_fill(uint32_t n, uint32_t n_slices, const uint32_t* __restrict__ slice_rows,
                             const uint32_t* __restrict__ slice_off, const uint32_t* __restrict__ off,
                             const uint32_t* __restrict__ other, const uint32_t* __restrict__ eid,
                             uint32_t* __restrict__ sidx, uint32_t* __restrict__ seid) {
    const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t k = (uint32_t)(t >> 5), lane = threadIdx.x & 31;
    if (k >= n_slices) return;
    const uint32_t b = slice_off[k], len = (slice_off[k + 1] - b) >> 5;
    const uint32_t r = slice_rows[(size_t)k * 32 + lane];
    const uint32_t rb = r != NO_ROW ? off[r] : 0u;
    const uint32_t d = r != NO_ROW ? off[r + 1] - rb : 0u;
    for (uint32_t j = 0; j < len; ++j) {
        const size_t q = (size_t)b + 32u * j + lane;
        sidx[q] = j < d ? other[rb + j] : n;
        seid[q] = j < d ? eid[rb + j] : 0xFFFFFFFFu;
    }
}

// (off[r], off[r+1]) of each listed row
__global__ void k_row_bounds(uint32_t k, const uint32_t* __restrict__ rows,
                             const uint32_t* __restrict__ off, uint32_t* __restrict__ out) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < k) {
        out[2 * i] = off[rows[i]];
        out[2 * i + 1] = off[rows[i] + 1];
    }
}

uint32_t fetch_u32(const uint32_t* d, cudaStream_t s) {
    uint32_t h = 0;
    GTC_CUDA(cudaMemcpyAsync(&h, d, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    GTC_CUDA(cudaStreamSynchronize(s));
    return h;
}

}  // namespace

void build_units(const uint32_t* d_off, const uint32_t* d_other, const uint32_t* d_eid,
                 uint32_t n, cudaStream_t s, Units& u) {
    const unsigned TB = 256;
    uint64_t L = 0;
    DevBuf<uint32_t> key(n, s), is_med(n, s), is_long(n, s), order(n, s), skey(n, s);
    DevBuf<uint32_t> pos((size_t)n + 1, s), flag(n, s);
    const unsigned gn = grid_for(n, TB, 1u << 30);
    if (n) {
        k_tier_keys<<<gn, TB, 0, s>>>(n, d_off, key.get(), is_med.get(), is_long.get());
        GTC_LAUNCHED();
        const uint32_t windows = (n + SP_WINDOW - 1) / SP_WINDOW;
        const uint64_t kb = (uint64_t)windows * KEY_STRIDE;
        GTC_REQUIRE(kb < 0xFFFFFFFFull, GTC_ERR_ARG, "graph too large for the slice layout");
    }
    // ---- sliced rows: window-sorted, compacted, cut into slices of 32 ----
    uint32_t ns = 0;
    if (n) {
        // stable: rows of equal length keep label order
        const uint32_t windows = (n + SP_WINDOW - 1) / SP_WINDOW;
        sort_positions_by_key(key.get(), n, windows * KEY_STRIDE, skey.get(), order.get(), s, &L);
        k_sliced_flags<<<gn, TB, 0, s>>>(n, order.get(), d_off, flag.get());
        GTC_LAUNCHED();
        scan_exclusive_u32(flag.get(), pos.get(), n, s, &L);
        ns = fetch_u32(pos.get() + n, s);
    }
    DevBuf<uint32_t> srows(ns, s);
    if (ns) {
        k_compact_u32<<<gn, TB, 0, s>>>(n, flag.get(), pos.get(), order.get(), srows.get());
        GTC_LAUNCHED();
    }
    const uint32_t n_slices = (ns + 31) / 32;
    u.slice_rows.alloc((size_t)n_slices * 32, s);
    u.slice_off.alloc((size_t)n_slices + 1, s);
    if (n_slices) {
        DevBuf<uint32_t> len32(n_slices, s);
        const unsigned gs = grid_for((size_t)n_slices * 32, TB, 1u << 30);
        k_slice_rows<<<gs, TB, 0, s>>>(ns, n_slices, srows.get(), d_off, u.slice_rows.get(),
                                       len32.get());
        GTC_LAUNCHED();
        scan_exclusive_u32(len32.get(), u.slice_off.get(), n_slices, s, &L);
        u.n_sliced = fetch_u32(u.slice_off.get() + n_slices, s);
    } else {
        GTC_CUDA(cudaMemsetAsync(u.slice_off.get(), 0, sizeof(uint32_t), s));
        u.n_sliced = 0;
    }
    u.sidx.alloc(u.n_sliced, s);
    u.seid.alloc(u.n_sliced, s);
    if (n_slices) {
        k_slice_fill<<<grid_for((size_t)n_slices * 32, TB, 1u << 30), TB, 0, s>>>(
            n, n_slices, u.slice_rows.get(), u.slice_off.get(), d_off, d_other, d_eid,
            u.sidx.get(), u.seid.get());
        GTC_LAUNCHED();
    }
    u.n_slices = n_slices;

    // ---- medium rows, in label order, with their entry ranges ----
    scan_exclusive_u32(is_med.get(), pos.get(), n, s, &L);
    u.n_med = n ? fetch_u32(pos.get() + n, s) : 0;
    u.med.alloc(u.n_med, s);
    std::vector<uint32_t> mrows(u.n_med), moff(2 * (size_t)u.n_med);
    if (u.n_med) {
        k_compact_u32<<<gn, TB, 0, s>>>(n, is_med.get(), pos.get(), nullptr, u.med.get());
        GTC_LAUNCHED();
        DevBuf<uint32_t> dmo(2 * (size_t)u.n_med, s);
        k_row_bounds<<<grid_for(u.n_med, TB, 1u << 30), TB, 0, s>>>(u.n_med, u.med.get(), d_off,
                                                                     dmo.get());
        GTC_LAUNCHED();
        GTC_CUDA(cudaMemcpyAsync(mrows.data(), u.med.get(), (size_t)u.n_med * 4,
                                 cudaMemcpyDeviceToHost, s));
        GTC_CUDA(cudaMemcpyAsync(moff.data(), dmo.get(), (size_t)u.n_med * 8,
                                 cudaMemcpyDeviceToHost, s));
        GTC_CUDA(cudaStreamSynchronize(s));
    }
    // the slices' first entries, for their work items
    std::vector<uint32_t> soff((size_t)n_slices + 1, 0u);
    if (n_slices) {
        GTC_CUDA(cudaMemcpyAsync(soff.data(), u.slice_off.get(), ((size_t)n_slices + 1) * 4,
                                 cudaMemcpyDeviceToHost, s));
        GTC_CUDA(cudaStreamSynchronize(s));
    }

    // ---- long rows: chunk table on the host ----
    scan_exclusive_u32(is_long.get(), pos.get(), n, s, &L);
    const uint32_t nl = n ? fetch_u32(pos.get() + n, s) : 0;
    std::vector<uint32_t> lrows(nl), loff(2 * (size_t)nl);
    if (nl) {
        DevBuf<uint32_t> dl(nl, s);
        k_compact_u32<<<gn, TB, 0, s>>>(n, is_long.get(), pos.get(), nullptr, dl.get());
        GTC_LAUNCHED();
        DevBuf<uint32_t> dlo(2 * (size_t)nl, s);
        k_row_bounds<<<grid_for(nl, TB, 1u << 30), TB, 0, s>>>(nl, dl.get(), d_off, dlo.get());
        GTC_LAUNCHED();
        GTC_CUDA(cudaMemcpyAsync(lrows.data(), dl.get(), (size_t)nl * 4, cudaMemcpyDeviceToHost, s));
        GTC_CUDA(cudaMemcpyAsync(loff.data(), dlo.get(), (size_t)nl * 8, cudaMemcpyDeviceToHost, s));
        GTC_CUDA(cudaStreamSynchronize(s));
    }

    // ---- the work list (one warp per item): long chunks, then medium rows,
    // then slices, so the heaviest items are spread over the warps first ----
    std::vector<uint4> units, longs;
    uint32_t slot = 0;
    for (uint32_t k = 0; k < nl; ++k) {
        const uint32_t len = loff[2 * k + 1] - loff[2 * k];
        const uint32_t chunks = (uint32_t)(((uint64_t)len + SP_CAP - 1) / SP_CAP);
        longs.push_back(make_uint4(lrows[k], slot, chunks, 0));
        for (uint32_t c = 0; c < chunks; ++c) units.push_back(make_uint4(UNIT_LONG, k, c, 0));
        slot += chunks;
    }
    for (uint32_t q = 0; q < u.n_med; ++q)
        units.push_back(make_uint4(UNIT_MEDIUM, mrows[q], moff[2 * (size_t)q], moff[2 * (size_t)q + 1]));
    for (uint32_t k = 0; k < n_slices; ++k)
        units.push_back(make_uint4(UNIT_SLICES, k, soff[k], (soff[k + 1] - soff[k]) >> 5));

    u.n_units = (uint32_t)units.size();
    u.n_long = (uint32_t)longs.size();
    u.n_chunks = slot;
    u.units.alloc(units.size(), s);
    u.longs.alloc(longs.size(), s);
    u.partial.alloc(slot, s);
    u.counter.alloc(longs.size(), s);
    u.fold_part.alloc(2 * (size_t)FOLD_MAX_CTAS, s);
    if (!units.empty())
        GTC_CUDA(cudaMemcpyAsync(u.units.get(), units.data(), units.size() * sizeof(uint4),
                                 cudaMemcpyHostToDevice, s));
    if (!longs.empty())
        GTC_CUDA(cudaMemcpyAsync(u.longs.get(), longs.data(), longs.size() * sizeof(uint4),
                                 cudaMemcpyHostToDevice, s));
    GTC_CUDA(cudaMemsetAsync(u.counter.get(), 0, (longs.empty() ? 1 : longs.size()) * sizeof(unsigned), s));
    GTC_CUDA(cudaStreamSynchronize(s));  // the host vectors die here
    u.built = true;
}

}  // namespace gtc
