// gtc_gt.cu -- the native binary .gt format, read straight into a GPU graph.
//
// Replaces gt_io::gt::read (crates/gt-io/src/gt.rs:555-626, read_adjacency
// :628-678, read_column :724-820 of graph-tool-rs) for the centrality path:
// a .gt document is parsed and its adjacency becomes a gtc_graph whose
// blocks are the ones the reference's reader builds, because the reader
// replays add_edge(v, u) for every vertex v in order and every entry u of
// v's list in file order (gt.rs:648-674), and gtc_graph_create_device
// replays the same call sequence.
//
// Work split.  The host walks the framing, which is sequential by nature:
// the magic, version and byte-order flag, the comment, one (count, list)
// record per vertex and the property table.  It records where every list
// starts and checks that every field lies inside the document.  The device
// decodes the lists -- m indices of 1, 2, 4 or 8 bytes in the file's byte
// order, a warp per vertex -- checks each against the vertex count and
// writes the (source, target) edge list that the graph build consumes.
//
// Layout of a document (gt.rs:1-22):
//   magic "⛾ gt" (6 bytes), version u8 (== 1), big_endian u8,
//   comment (u64 length + bytes), directed u8, N u64,
//   N x (u64 count + count indices of width w(N)),
//   nprops u64, nprops x (domain u8, name, value-type u8, values)
// with every multi-byte field after the flag in the order it declares.
#include <cstring>
#include <string>
#include <vector>

#include "gtc_internal.cuh"

namespace gtc {
namespace {

// The value universe, by the index a file stores (ValueKind::ALL,
// crates/gt-core/src/prop/value.rs:79-95).
enum GtKind : int32_t {
    K_BOOL = 0, K_I16, K_I32, K_I64, K_F64, K_LONG_DOUBLE, K_STR,
    K_VEC_BOOL, K_VEC_I16, K_VEC_I32, K_VEC_I64, K_VEC_F64, K_VEC_LONG_DOUBLE, K_VEC_STR,
    K_PYOBJECT, K_COUNT
};

// Width of a fixed-size element of a kind (0 for the length-prefixed ones).
int scalar_width(int32_t k) {
    switch (k) {
        case K_BOOL: case K_VEC_BOOL: return 1;
        case K_I16: case K_VEC_I16: return 2;
        case K_I32: case K_VEC_I32: return 4;
        case K_I64: case K_F64: case K_VEC_I64: case K_VEC_F64: return 8;
        case K_LONG_DOUBLE: case K_VEC_LONG_DOUBLE: return 16;
        default: return 0;
    }
}

// Index width of the adjacency lists: the narrowest of u8/u16/u32/u64 that
// holds N (vint_width, gt.rs:689-699).
int vint_width(uint64_t n) {
    if (n <= 0xFFull) return 1;
    if (n <= 0xFFFFull) return 2;
    if (n <= 0xFFFFFFFFull) return 4;
    return 8;
}

// Strict UTF-8 (no overlong forms, no surrogates, nothing above U+10FFFF),
// the check String::from_utf8 makes; returns the length of the valid prefix.
size_t utf8_valid_prefix(const uint8_t* p, size_t n) {
    size_t i = 0;
    while (i < n) {
        const uint8_t c = p[i];
        if (c < 0x80) { ++i; continue; }
        int len;
        uint32_t lo = 0x80, hi = 0xBF;  // bounds of the second byte
        if (c >= 0xC2 && c <= 0xDF) len = 2;
        else if (c == 0xE0) len = 3, lo = 0xA0;
        else if (c >= 0xE1 && c <= 0xEC) len = 3;
        else if (c == 0xED) len = 3, hi = 0x9F;
        else if (c >= 0xEE && c <= 0xEF) len = 3;
        else if (c == 0xF0) len = 4, lo = 0x90;
        else if (c >= 0xF1 && c <= 0xF3) len = 4;
        else if (c == 0xF4) len = 4, hi = 0x8F;
        else return i;
        if (i + (size_t)len > n) return i;
        if (p[i + 1] < lo || p[i + 1] > hi) return i;
        for (int k = 2; k < len; ++k)
            if (p[i + k] < 0x80 || p[i + k] > 0xBF) return i;
        i += (size_t)len;
    }
    return n;
}

std::string at_byte(uint64_t at, const std::string& msg) {
    return "at byte " + std::to_string(at) + ": " + msg;
}

// A bounds-checked cursor over the document; every read that would pass the
// end is the reference's "unexpected end of file" parse error.
struct Cursor {
    const uint8_t* p;
    uint64_t len, pos = 0;
    bool big = false;

    void need(uint64_t k) const {
        if (k > len - pos)
            throw Error{GTC_ERR_ARG, at_byte(pos, "unexpected end of file, wanted " +
                                                      std::to_string(k) + " more bytes")};
    }
    uint64_t uint(int width) {
        need((uint64_t)width);
        uint64_t v = 0;
        for (int k = 0; k < width; ++k) {
            const uint64_t b = p[pos + (uint64_t)(big ? k : width - 1 - k)];
            v = (v << 8) | b;
        }
        pos += (uint64_t)width;
        return v;
    }
    uint8_t u8() { return (uint8_t)uint(1); }
    uint64_t u64() { return uint(8); }
    // a length-prefixed byte run; returns its first byte's offset
    uint64_t bytes(uint64_t* n_out) {
        const uint64_t n = u64();
        const uint64_t at = pos;
        if (n > len - pos)
            throw Error{GTC_ERR_ARG, at_byte(at, "string declares " + std::to_string(n) +
                                                     " bytes, " + std::to_string(len - pos) +
                                                     " are present")};
        pos += n;
        *n_out = n;
        return at;
    }
    // a string field that must be UTF-8
    uint64_t text(uint64_t* n_out, const std::string& what, bool as_parse_error,
                  const std::string& prop_name) {
        const uint64_t at0 = pos;
        const uint64_t at = bytes(n_out);
        const size_t ok = utf8_valid_prefix(p + at, (size_t)*n_out);
        if (ok != *n_out) {
            if (as_parse_error)
                throw Error{GTC_ERR_ARG, at_byte(at0, what + " is not valid UTF-8 at offset " +
                                                          std::to_string(ok))};
            throw Error{GTC_ERR_ARG, "property '" + prop_name +
                                         "' declared as string holds bytes that are not UTF-8"};
        }
        return at;
    }
};

}  // namespace
}  // namespace gtc

// One parsed document.  The bytes are copied in; everything else is offsets
// into that copy.
struct gtc_gt_file {
    std::vector<uint8_t> data;
    bool big = false, directed = false;
    uint64_t comment_at = 0, comment_len = 0;
    uint64_t n = 0, m = 0;
    int width = 1;
    std::vector<uint64_t> list_at;  // per vertex: first byte of its index list
    std::vector<uint32_t> e_off;    // per vertex: its first edge (n + 1)
    uint64_t adj_begin = 0, adj_end = 0;
    struct Prop {
        std::string name;
        int32_t domain = 0, kind = 0;
        uint64_t count = 0, at = 0, len = 0;  // values and their byte range
    };
    std::vector<Prop> props;
    std::string comment;
};

namespace gtc {
namespace {

void parse(gtc_gt_file& f) {
    Cursor c{f.data.data(), (uint64_t)f.data.size()};
    // magic: a short or foreign head is "not a .gt file" (gt.rs:558-575)
    static const uint8_t MAGIC[6] = {0xE2, 0x9B, 0xBE, 0x20, 0x67, 0x74};
    const uint64_t got = c.len < 6 ? c.len : 6;
    if (got != 6 || std::memcmp(c.p, MAGIC, 6) != 0)
        throw Error{GTC_ERR_ARG, "bad magic: not a .gt document"};
    c.pos = 6;
    const uint8_t version = c.u8();
    if (version != 1)
        throw Error{GTC_ERR_ARG, "unsupported .gt version " + std::to_string(version)};
    c.big = c.u8() != 0;  // one byte: readable before the order it declares
    f.big = c.big;
    f.comment_at = c.text(&f.comment_len, "the header comment", true, "");
    f.comment.assign((const char*)c.p + f.comment_at, (size_t)f.comment_len);

    // adjacency (read_adjacency, gt.rs:628-678)
    f.directed = c.u8() != 0;
    f.n = c.u64();
    if (f.n > 0 && f.n - 1 > 0xFFFFFFFEull)
        throw Error{GTC_ERR_ARG, "the document's vertex count exceeds the index space"};
    // every vertex record holds at least its 8-byte count: a document too
    // short for N of them is truncated, and nothing is sized from N first
    if (f.n > (c.len - c.pos) / 8)
        throw Error{GTC_ERR_ARG, at_byte(c.pos, "unexpected end of file, " + std::to_string(f.n) +
                                                    " vertex records need at least " +
                                                    std::to_string(f.n) + " x 8 bytes")};
    f.width = vint_width(f.n);
    f.list_at.resize((size_t)f.n);
    f.e_off.resize((size_t)f.n + 1);
    f.adj_begin = c.pos;
    uint64_t m = 0;
    for (uint64_t v = 0; v < f.n; ++v) {
        const uint64_t k = c.u64();
        f.e_off[(size_t)v] = (uint32_t)m;
        f.list_at[(size_t)v] = c.pos;
        if (k > (c.len - c.pos) / (uint64_t)f.width)
            throw Error{GTC_ERR_ARG, at_byte(c.pos, "unexpected end of file, wanted " +
                                                        std::to_string(k) + " indices of " +
                                                        std::to_string(f.width) + " bytes")};
        c.pos += k * (uint64_t)f.width;
        m += k;
        if (m > 0xFFFFFFFEull)
            throw Error{GTC_ERR_ARG, "the document's edge count exceeds the index space"};
    }
    f.e_off[(size_t)f.n] = (uint32_t)m;
    f.m = m;
    f.adj_end = c.pos;

    // properties (gt.rs:581-618, read_column :724-820)
    const uint64_t nprops = c.u64();
    for (uint64_t i = 0; i < nprops; ++i) {
        gtc_gt_file::Prop P;
        const uint64_t at = c.pos;
        const uint8_t dom = c.u8();
        if (dom > 2)
            throw Error{GTC_ERR_ARG, at_byte(at, "invalid property domain " + std::to_string(dom))};
        P.domain = dom;
        uint64_t nl = 0;
        const uint64_t na = c.text(&nl, "a property name", true, "");
        P.name.assign((const char*)c.p + na, (size_t)nl);
        const uint8_t kind = c.u8();
        if (kind >= K_COUNT)
            throw Error{GTC_ERR_ARG, "unknown value type index " + std::to_string(kind)};
        P.kind = kind;
        P.count = dom == 0 ? 1 : (dom == 1 ? f.n : f.m);
        P.at = c.pos;
        const int w = scalar_width(kind);
        uint64_t tmp = 0;
        if (kind <= K_LONG_DOUBLE) {
            if (P.count > (c.len - c.pos) / (uint64_t)w)
                throw Error{GTC_ERR_ARG, at_byte(c.pos, "unexpected end of file, wanted " +
                                                            std::to_string(P.count) + " values")};
            c.pos += P.count * (uint64_t)w;
        } else if (kind == K_STR) {
            for (uint64_t j = 0; j < P.count; ++j) c.text(&tmp, "", false, P.name);
        } else if (kind == K_VEC_STR) {
            for (uint64_t j = 0; j < P.count; ++j) {
                const uint64_t k = c.u64();
                for (uint64_t q = 0; q < k; ++q) c.text(&tmp, "", false, P.name);
            }
        } else if (kind == K_PYOBJECT || kind == K_VEC_BOOL) {
            for (uint64_t j = 0; j < P.count; ++j) c.bytes(&tmp);
        } else {  // vectors of fixed-width elements
            for (uint64_t j = 0; j < P.count; ++j) {
                const uint64_t k = c.u64();
                // compared before multiplying: a declared count near 2^64
                // would wrap k * w around to a small length
                if (k > (c.len - c.pos) / (uint64_t)w)
                    throw Error{GTC_ERR_ARG, at_byte(c.pos, "unexpected end of file, a vector of " +
                                                                std::to_string(k) + " elements")};
                c.pos += k * (uint64_t)w;
            }
        }
        P.len = c.pos - P.at;
        f.props.push_back(std::move(P));
    }
}

// A warp per vertex: lanes stride the vertex's list, decode each index in
// the document's byte order, write the edge (v, u) at its edge id and record
// the first edge whose index is not below n.
__global__ void __launch_bounds__(256) k_gt_decode(uint64_t n, const uint8_t* __restrict__ adj,
                                                   const uint64_t* __restrict__ list_at,
                                                   const uint32_t* __restrict__ e_off, int width,
                                                   int big, uint32_t* __restrict__ src,
                                                   uint32_t* __restrict__ tgt,
                                                   unsigned* __restrict__ first_bad) {
    const int lane = threadIdx.x & 31;
    const uint64_t nw = (uint64_t)gridDim.x * (blockDim.x >> 5);
    for (uint64_t v = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; v < n; v += nw) {
        const uint32_t e0 = e_off[v], e1 = e_off[v + 1];
        const uint8_t* lp = adj + list_at[v];
        for (uint32_t e = e0 + (uint32_t)lane; e < e1; e += 32) {
            const uint8_t* q = lp + (uint64_t)(e - e0) * (uint64_t)width;
            uint64_t u = 0;
            for (int k = 0; k < width; ++k) u = (u << 8) | (uint64_t)q[big ? k : width - 1 - k];
            src[e] = (uint32_t)v;
            tgt[e] = (uint32_t)u;
            if (u >= n) atomicMin(first_bad, e);
        }
    }
}

}  // namespace
}  // namespace gtc

using namespace gtc;

template <class F>
static int gt_guarded(F&& f) {
    try {
        f();
        set_error("");
        return GTC_OK;
    } catch (const Error& e) {
        set_error(e.msg);
        return e.status;
    } catch (const std::bad_alloc&) {
        set_error("host allocation failed");
        return GTC_ERR_OOM;
    } catch (...) {
        set_error("unexpected internal error");
        return GTC_ERR_CUDA;
    }
}

extern "C" {

int gtc_gt_open(const uint8_t* bytes, uint64_t len, gtc_gt_file** out) {
    return gt_guarded([&] {
        GTC_REQUIRE(out, GTC_ERR_ARG, "out is NULL");
        *out = nullptr;
        GTC_REQUIRE(bytes || len == 0, GTC_ERR_ARG, "bytes is NULL");
        gtc_gt_file* f = new gtc_gt_file;
        try {
            f->data.assign(bytes, bytes + len);
            parse(*f);
        } catch (...) {
            delete f;
            throw;
        }
        *out = f;
    });
}

int gtc_gt_close(gtc_gt_file* f) {
    return gt_guarded([&] { delete f; });
}

int gtc_gt_info(const gtc_gt_file* f, uint64_t* n, uint64_t* m, int32_t* directed,
                int32_t* big_endian, uint64_t* nprops) {
    return gt_guarded([&] {
        GTC_REQUIRE(f, GTC_ERR_ARG, "file is NULL");
        if (n) *n = f->n;
        if (m) *m = f->m;
        if (directed) *directed = f->directed ? 1 : 0;
        if (big_endian) *big_endian = f->big ? 1 : 0;
        if (nprops) *nprops = f->props.size();
    });
}

int gtc_gt_comment(const gtc_gt_file* f, const char** text, uint64_t* len) {
    return gt_guarded([&] {
        GTC_REQUIRE(f && text && len, GTC_ERR_ARG, "NULL argument");
        *text = f->comment.c_str();
        *len = f->comment.size();
    });
}

int gtc_gt_property(const gtc_gt_file* f, uint64_t i, const char** name, uint64_t* name_len,
                    int32_t* domain, int32_t* kind, uint64_t* count) {
    return gt_guarded([&] {
        GTC_REQUIRE(f, GTC_ERR_ARG, "file is NULL");
        GTC_REQUIRE(i < f->props.size(), GTC_ERR_INDEX,
                    "property " + std::to_string(i) + " of " + std::to_string(f->props.size()));
        const auto& P = f->props[(size_t)i];
        if (name) *name = P.name.c_str();
        if (name_len) *name_len = P.name.size();
        if (domain) *domain = P.domain;
        if (kind) *kind = P.kind;
        if (count) *count = P.count;
    });
}

int gtc_gt_property_bytes(const gtc_gt_file* f, uint64_t i, const uint8_t** data, uint64_t* len) {
    return gt_guarded([&] {
        GTC_REQUIRE(f && data && len, GTC_ERR_ARG, "NULL argument");
        GTC_REQUIRE(i < f->props.size(), GTC_ERR_INDEX,
                    "property " + std::to_string(i) + " of " + std::to_string(f->props.size()));
        const auto& P = f->props[(size_t)i];
        *data = f->data.data() + P.at;
        *len = P.len;
    });
}

int gtc_gt_property_f64(const gtc_gt_file* f, uint64_t i, double* out, uint64_t out_len) {
    return gt_guarded([&] {
        GTC_REQUIRE(f, GTC_ERR_ARG, "file is NULL");
        GTC_REQUIRE(i < f->props.size(), GTC_ERR_INDEX,
                    "property " + std::to_string(i) + " of " + std::to_string(f->props.size()));
        const auto& P = f->props[(size_t)i];
        GTC_REQUIRE(P.kind <= K_F64, GTC_ERR_ARG,
                    "property '" + P.name + "' is not a numeric scalar column");
        GTC_REQUIRE(out || P.count == 0, GTC_ERR_ARG, "out is NULL");
        GTC_REQUIRE(out_len >= P.count, GTC_ERR_ARG,
                    "out holds " + std::to_string(out_len) + " values, the column has " +
                        std::to_string(P.count));
        Cursor c{f->data.data(), (uint64_t)f->data.size()};
        c.big = f->big;
        c.pos = P.at;
        for (uint64_t j = 0; j < P.count; ++j) {
            switch (P.kind) {
                case K_BOOL: out[j] = (double)c.u8(); break;
                case K_I16: out[j] = (double)(int16_t)(uint16_t)c.uint(2); break;
                case K_I32: out[j] = (double)(int32_t)(uint32_t)c.uint(4); break;
                case K_I64: out[j] = (double)(int64_t)c.uint(8); break;
                default: {
                    const uint64_t b = c.uint(8);
                    double d;
                    std::memcpy(&d, &b, 8);
                    out[j] = d;
                }
            }
        }
    });
}

int gtc_gt_graph(const gtc_gt_file* f, gtc_graph** out) {
    return gt_guarded([&] {
        GTC_REQUIRE(out, GTC_ERR_ARG, "out is NULL");
        *out = nullptr;
        GTC_REQUIRE(f, GTC_ERR_ARG, "file is NULL");
        require_device();
        cudaStream_t s = nullptr;
        GTC_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
        struct StreamGuard {
            cudaStream_t s;
            ~StreamGuard() {
                cudaStreamSynchronize(s);
                cudaStreamDestroy(s);
            }
        } guard{s};
        const uint64_t n = f->n, m = f->m;
        DevBuf<uint32_t> d_src(m, s), d_tgt(m, s);
        if (m) {
            // the adjacency section, the per-vertex list offsets (relative to
            // it) and the edge offsets go to the device once
            const uint64_t span = f->adj_end - f->adj_begin;
            DevBuf<uint8_t> d_adj(span, s);
            DevBuf<uint64_t> d_at(n, s);
            DevBuf<uint32_t> d_eoff(n + 1, s);
            DevBuf<unsigned> d_bad(1, s);
            std::vector<uint64_t> rel(f->list_at.size());
            for (size_t v = 0; v < rel.size(); ++v) rel[v] = f->list_at[v] - f->adj_begin;
            GTC_CUDA(cudaMemcpyAsync(d_adj.get(), f->data.data() + f->adj_begin, span,
                                     cudaMemcpyHostToDevice, s));
            GTC_CUDA(cudaMemcpyAsync(d_at.get(), rel.data(), n * sizeof(uint64_t),
                                     cudaMemcpyHostToDevice, s));
            GTC_CUDA(cudaMemcpyAsync(d_eoff.get(), f->e_off.data(), (n + 1) * sizeof(uint32_t),
                                     cudaMemcpyHostToDevice, s));
            GTC_CUDA(cudaMemsetAsync(d_bad.get(), 0xFF, sizeof(unsigned), s));
            const unsigned blocks = grid_for(n * 32, 256, (unsigned)sm_count() * 8);
            k_gt_decode<<<blocks, 256, 0, s>>>(n, d_adj.get(), d_at.get(), d_eoff.get(), f->width,
                                               f->big ? 1 : 0, d_src.get(), d_tgt.get(),
                                               d_bad.get());
            GTC_LAUNCHED();
            unsigned bad = 0;
            GTC_CUDA(cudaMemcpyAsync(&bad, d_bad.get(), sizeof(unsigned), cudaMemcpyDeviceToHost, s));
            GTC_CUDA(cudaStreamSynchronize(s));
            if (bad != 0xFFFFFFFFu) {
                // the first out-of-range index in file order, as the
                // reference's reader reports it (gt.rs:658-664)
                size_t lo = 0, hi = (size_t)n;  // the vertex whose list holds edge `bad`
                while (hi - lo > 1) {
                    const size_t mid = (lo + hi) / 2;
                    if (f->e_off[mid] <= bad) lo = mid; else hi = mid;
                }
                Cursor c{f->data.data(), (uint64_t)f->data.size()};
                c.big = f->big;
                c.pos = f->list_at[lo] + (uint64_t)(bad - f->e_off[lo]) * (uint64_t)f->width;
                const uint64_t u = c.uint(f->width);
                throw Error{GTC_ERR_INDEX, "vertex index " + std::to_string(u) +
                                               " is out of range (bound " + std::to_string(n) + ")"};
            }
        }
        gtc_graph* g = nullptr;
        const int st = gtc_graph_create_device(n, m, d_src.get(), d_tgt.get(), s, &g);
        if (st != GTC_OK) throw Error{st, gtc_last_error()};
        *out = g;
    });
}

}  // extern "C"
