// gtc_view.cuh -- the directed view of one solve (see gtc_view.cu).
#pragma once

#include "gtc_internal.cuh"

namespace gtc {

struct View {
    uint32_t n = 0;         // vertex bound (index space of every vertex map)
    uint32_t m_total = 0;   // edge bound
    uint32_t m_pull = 0;    // entries in the pull half after filtering
    uint32_t n_active = 0;  // num_vertices() of the view
    bool reversed = false, filtered = false;
    // pull: in_edges(v) of the view, storage order.  push: out_edges(v).
    const uint32_t *pull_off = nullptr, *pull_other = nullptr, *pull_eid = nullptr;
    const uint32_t *push_off = nullptr, *push_other = nullptr, *push_eid = nullptr;
    DevBuf<uint8_t> active;  // empty when every vertex is kept
    Halves fpull, fpush;     // compacted halves of a filtered view

    void prepare(gtc_graph* g, const gtc_view* v, cudaStream_t s, uint64_t* launches);
    const uint8_t* active_or_null() const { return active.p; }
};

}  // namespace gtc
