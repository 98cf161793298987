// gtc_sweep.cu -- host side of the degree-binned pull schedule.
#include <vector>

#include "gtc_sweep.cuh"

namespace gtc {

void build_units(const uint32_t* d_off, uint32_t n, cudaStream_t s, Units& u) {
    std::vector<uint32_t> off((size_t)n + 1);
    GTC_CUDA(cudaMemcpyAsync(off.data(), d_off, ((size_t)n + 1) * sizeof(uint32_t),
                             cudaMemcpyDeviceToHost, s));
    GTC_CUDA(cudaStreamSynchronize(s));
    std::vector<uint4> units, longs;
    units.reserve((size_t)(off[n] + n) / SP_CAP + 16);
    uint32_t slot = 0;
    uint32_t r = 0;
    while (r < n) {
        uint32_t len = off[r + 1] - off[r];
        if ((uint64_t)len + 1 > (uint64_t)SP_CAP) {  // a long row: CTA-sized chunks
            const uint32_t chunks = (uint32_t)(((uint64_t)len + SP_CAP - 1) / SP_CAP);
            const uint32_t k = (uint32_t)longs.size();
            longs.push_back(make_uint4(r, slot, chunks, 0));
            for (uint32_t c = 0; c < chunks; ++c) units.push_back(make_uint4(UNIT_LONG, k, c, 0));
            slot += chunks;
            ++r;
            continue;
        }
        const uint32_t start = r;
        uint32_t items = 0;
        while (r < n) {
            len = off[r + 1] - off[r];
            if ((uint64_t)len + 1 > (uint64_t)SP_CAP || items + len + 1 > (uint32_t)SP_CAP) break;
            items += len + 1;
            ++r;
        }
        units.push_back(make_uint4(UNIT_SHORT, start, r, 0));
    }
    u.n_units = (uint32_t)units.size();
    u.n_long = (uint32_t)longs.size();
    u.n_chunks = slot;
    u.units.alloc(units.size(), s);
    u.longs.alloc(longs.size(), s);
    u.partial.alloc(slot, s);
    u.counter.alloc(longs.size(), s);
    u.long_out.alloc(longs.size(), s);
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
