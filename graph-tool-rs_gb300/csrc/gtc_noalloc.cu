// gtc_noalloc.cu -- PageRank that allocates no memory (gtc_pagerank_noalloc).
//
// Who needs it: callers that cannot allocate device memory at the time they
// run PageRank.  Examples are a host runtime that reserves all GPU memory up
// front and forbids later allocations, and a latency-critical path where no
// allocator call is allowed because it could stall or fail.  For them this
// entry point takes the graph (a CSC in device memory) and the output
// buffer, and keeps every intermediate vector in one file-scope device
// array compiled into the library.
//
// The array is NOALLOC_BYTES large and every GPU that loads the library
// holds it until the process exits.  All calls share it and it keeps the
// last call's contents, so each call clears what must start at zero.  Calls
// that overlap on the GPU (two streams, or two host threads) race on it.
//
// The sweep is the FP32 fast path's arithmetic (compensated row sums, FP64
// delta and dangling mass) with a simpler one-warp-per-row schedule.
#include <mutex>

#include "gtc_internal.cuh"

namespace gtc {
namespace {

constexpr uint32_t NA_MAX_N = 1u << 20;  // the vertex limit of the entry point
constexpr int NA_NT = 256;
// Fixed grid of the sweep (4 CTAs per SM of a 152-SM part); the grid sizes
// the per-CTA partials of the scratch array, and any size gives the same
// result up to the FP64 fold order of those partials.
constexpr int NA_BLOCKS = 608;

// Layout of the scratch array (offsets in bytes, each 256-aligned).
constexpr size_t NA_VEC = ((size_t)(NA_MAX_N + 1) * sizeof(float) + 255) & ~(size_t)255;
constexpr size_t NA_OFF_Y0 = 0;                    // y = rank / deg (+1 zero entry)
constexpr size_t NA_OFF_Y1 = NA_OFF_Y0 + NA_VEC;
constexpr size_t NA_OFF_R1 = NA_OFF_Y1 + NA_VEC;   // the other rank buffer
constexpr size_t NA_OFF_PART = NA_OFF_R1 + NA_VEC; // per-block partials (double2)
constexpr size_t NA_OFF_SCAL = NA_OFF_PART + ((NA_BLOCKS * sizeof(double2) + 255) & ~(size_t)255);
constexpr size_t NA_BYTES = NA_OFF_SCAL + 256;     // scalars: ticket, delta, psink

__device__ __align__(256) unsigned char g_noalloc_scratch[NA_BYTES];

// Device address of the array, per device.  In host code the array's name is
// only a host-side handle; cudaGetSymbolAddress gives the address a kernel
// may use.  Looked up once per device, with that device current.
unsigned char* g_scratch_addr[64] = {};
std::mutex g_scratch_mu;

unsigned char* scratch_for_current_device() {
    int dev = 0;
    GTC_CUDA(cudaGetDevice(&dev));
    GTC_REQUIRE(dev >= 0 && dev < 64, GTC_ERR_ARG, "device index out of range");
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        GTC_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        g_scratch_addr[dev] = static_cast<unsigned char*>(p);
    }
    return g_scratch_addr[dev];
}

struct NaArgs {
    uint32_t n;
    const uint32_t* __restrict__ off;
    const uint32_t* __restrict__ src;
    const uint32_t* __restrict__ deg;  // out-degree per vertex
    float uniform, one_minus_d, d;
    const float* __restrict__ prev;
    const float* __restrict__ yprev;
    float* __restrict__ next;
    float* __restrict__ ynext;
    double2* part;       // per-block (delta, dangling mass)
    unsigned* ticket;    // zero at the first sweep; the last block resets it
    double* out;         // [0] delta, [1] dangling mass of next
    const double* psink; // dangling mass of prev
};

__device__ __forceinline__ void na_fold(double a, double b, const NaArgs& A) {
    __shared__ double sa[NA_NT / 32], sb[NA_NT / 32];
    __shared__ bool last;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    a = warp_sum_f64(a);
    b = warp_sum_f64(b);
    if (lane == 0) sa[warp] = a, sb[warp] = b;
    __syncthreads();
    if (threadIdx.x == 0) {
        double ta = 0.0, tb = 0.0;
        for (int w = 0; w < NA_NT / 32; ++w) ta += sa[w], tb += sb[w];
        A.part[blockIdx.x] = make_double2(ta, tb);
        __threadfence();
        last = atomicAdd(A.ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (last && warp == 0) {
        __threadfence();
        double ta = 0.0, tb = 0.0;
        for (unsigned i = lane; i < gridDim.x; i += 32) {
            const double2 q = __ldcg(A.part + i);
            ta += q.x, tb += q.y;
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

// Uniform start: rank = 1/n, y = rank / deg, and its dangling mass.
__global__ void __launch_bounds__(NA_NT) k_na_prime(NaArgs A, float* rank) {
    Kahan s;
    for (uint32_t v = blockIdx.x * NA_NT + threadIdx.x; v < A.n; v += gridDim.x * NA_NT) {
        const uint32_t dv = A.deg[v];
        rank[v] = A.uniform;
        A.ynext[v] = dv ? __fdiv_rn(A.uniform, (float)dv) : 0.f;
        if (!dv) s.add(A.uniform);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) A.ynext[A.n] = 0.f;
    na_fold(0.0, (double)s.s + (double)s.c, A);
}

// One sweep: a warp per row, compensated sum of y over the row's sources.
__global__ void __launch_bounds__(NA_NT) k_na_sweep(NaArgs A) {
    const int lane = threadIdx.x & 31;
    const uint32_t gw = (blockIdx.x * NA_NT + threadIdx.x) >> 5, nw = (gridDim.x * NA_NT) >> 5;
    const float psink = (float)*A.psink;
    Kahan da, sa;
    for (uint32_t v = gw; v < A.n; v += nw) {
        KahanBlocked kb;
        for (uint32_t p = A.off[v] + lane, e = A.off[v + 1]; p < e; p += 32)
            kb.add(A.yprev[A.src[p]]);
        Kahan k = kb.fold();
        warp_merge_kahan(k);
        if (lane == 0) {
            const float r = __fadd_rn(__fmul_rn(psink, A.uniform), k.value());
            const float nv = __fadd_rn(__fmul_rn(A.one_minus_d, A.uniform), __fmul_rn(A.d, r));
            const uint32_t dv = A.deg[v];
            A.next[v] = nv;
            A.ynext[v] = dv ? __fdiv_rn(nv, (float)dv) : 0.f;
            da.add(fabsf(__fsub_rn(nv, A.prev[v])));
            if (!dv) sa.add(nv);
        }
    }
    na_fold((double)da.s + (double)da.c, (double)sa.s + (double)sa.c, A);
}

}  // namespace
}  // namespace gtc

using namespace gtc;

extern "C" int gtc_pagerank_noalloc(uint64_t n, const uint32_t* d_off, const uint32_t* d_src,
                                    const uint32_t* d_out_degree, double damping,
                                    double epsilon, uint64_t max_iter, float* d_rank,
                                    uint64_t* iters_out, void* stream) {
    try {
        GTC_REQUIRE(n <= NA_MAX_N, GTC_ERR_ARG,
                    "gtc_pagerank_noalloc: more vertices than its static scratch holds (limit "
                    "1048576)");
        GTC_REQUIRE(!(damping != damping) && !(epsilon != epsilon), GTC_ERR_ARG,
                    "gtc_pagerank_noalloc: damping or epsilon is NaN");
        GTC_REQUIRE(max_iter != 0 || epsilon > 0.0, GTC_ERR_ARG,
                    "gtc_pagerank_noalloc: max_iter = 0 (uncapped) with epsilon <= 0 would never "
                    "stop");
        GTC_REQUIRE(n == 0 || (d_off && d_src && d_out_degree && d_rank), GTC_ERR_ARG,
                    "gtc_pagerank_noalloc: a device array is NULL");
        cudaStream_t s = (cudaStream_t)stream;
        unsigned char* base = scratch_for_current_device();
        if (iters_out) *iters_out = 0;
        if (n == 0) {
            set_error("");
            return GTC_OK;
        }
        NaArgs A;
        A.n = (uint32_t)n;
        A.off = d_off;
        A.src = d_src;
        A.deg = d_out_degree;
        A.uniform = (float)(1.0 / (double)n);
        A.one_minus_d = (float)(1.0 - damping);
        A.d = (float)damping;
        A.part = reinterpret_cast<double2*>(base + NA_OFF_PART);
        A.ticket = reinterpret_cast<unsigned*>(base + NA_OFF_SCAL);
        double* scal = reinterpret_cast<double*>(base + NA_OFF_SCAL + 64);
        A.out = scal;         // [0] delta, [1] dangling mass
        A.psink = scal + 1;
        float* y[2] = {reinterpret_cast<float*>(base + NA_OFF_Y0),
                       reinterpret_cast<float*>(base + NA_OFF_Y1)};
        float* r[2] = {d_rank, reinterpret_cast<float*>(base + NA_OFF_R1)};
        // the ticket and the zero entries the sweeps read must start cleared
        GTC_CUDA(cudaMemsetAsync(base + NA_OFF_SCAL, 0, 256, s));
        GTC_CUDA(cudaMemsetAsync(y[1] + n, 0, sizeof(float), s));
        A.ynext = y[0];
        k_na_prime<<<NA_BLOCKS, NA_NT, 0, s>>>(A, r[0]);
        GTC_LAUNCHED();
        uint64_t it = 0;
        double delta = epsilon + 1.0;
        int c = 0;
        while (delta >= epsilon) {
            A.prev = r[c], A.yprev = y[c], A.next = r[c ^ 1], A.ynext = y[c ^ 1];
            k_na_sweep<<<NA_BLOCKS, NA_NT, 0, s>>>(A);
            GTC_LAUNCHED();
            GTC_CUDA(cudaMemcpyAsync(&delta, scal, sizeof(double), cudaMemcpyDeviceToHost, s));
            GTC_CUDA(cudaStreamSynchronize(s));
            c ^= 1;
            ++it;
            if (max_iter > 0 && it == max_iter) break;
        }
        // the latest iterate belongs in the caller's buffer
        if (c == 1)
            GTC_CUDA(cudaMemcpyAsync(d_rank, r[1], (size_t)n * sizeof(float),
                                     cudaMemcpyDeviceToDevice, s));
        GTC_CUDA(cudaStreamSynchronize(s));
        if (iters_out) *iters_out = it;
        set_error("");
        return GTC_OK;
    } catch (const Error& e) {
        set_error(e.msg);
        return e.status;
    } catch (...) {
        set_error("unexpected internal error");
        return GTC_ERR_CUDA;
    }
}
