// Particle reordering by cell for gather locality (a counting sort on Morton
// cell keys).  Particles are independent, so their slot order never changes
// a result; sorting only makes the 32 particles of a warp fall into a few
// neighbouring cells, so each corner gather touches a few cache lines
// instead of 32.  The slot -> particle map travels with the positions and is
// undone once at the end (jt_unpermute).
#include <stdint.h>

#include <mutex>

#include "jt_internal.h"
#include "jt_kernels.cuh"

namespace jt {

constexpr int kScanBlock = 1024;            // threads of the scan kernels
constexpr int kScanItems = 2 * kScanBlock;  // bins per scan block

__global__ void __launch_bounds__(kBlock) k_cell_keys(jt_sort_grid g, const float* __restrict__ pos, int n,
                                                      uint32_t* __restrict__ keys, uint32_t* __restrict__ hist) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int lim = (1 << g.bits) - 1;
    uint32_t c[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float f = floorf((pos[3 * (int64_t)i + a] - g.origin[a]) * g.inv_cell[a]);
        int ci = (f != f) ? 0 : (f < 0.0f ? 0 : (f > (float)lim ? lim : (int)f));
        c[a] = (uint32_t)ci;
    }
    const uint32_t key = g.order == JT_ORDER_LINEAR ? (((c[2] << g.bits) | c[1]) << g.bits) | c[0]
                                                    : morton3(c[0], c[1], c[2]);
    keys[i] = key;
    atomicAdd(hist + key, 1u);
}

// Exclusive scan, phase 1: each block scans kScanItems bins in shared memory
// (Hillis-Steele over the per-thread pair sums) and records its total.
__global__ void __launch_bounds__(kScanBlock) k_scan_blocks(uint32_t* __restrict__ data, int64_t n,
                                                            uint32_t* __restrict__ sums) {
    __shared__ uint32_t s[kScanBlock];
    const int64_t base = (int64_t)blockIdx.x * kScanItems;
    const int t = threadIdx.x;
    const int64_t i0 = base + 2 * t, i1 = i0 + 1;
    const uint32_t a = i0 < n ? data[i0] : 0u, b = i1 < n ? data[i1] : 0u;
    s[t] = a + b;
    __syncthreads();
    for (int off = 1; off < kScanBlock; off <<= 1) {
        const uint32_t v = t >= off ? s[t - off] : 0u;
        __syncthreads();
        s[t] += v;
        __syncthreads();
    }
    const uint32_t excl = s[t] - (a + b);
    if (i0 < n) data[i0] = excl;
    if (i1 < n) data[i1] = excl + a;
    if (t == kScanBlock - 1) sums[blockIdx.x] = s[t];
}

// Phase 2: add the scanned block totals (sums holds an exclusive scan).
__global__ void __launch_bounds__(kScanBlock) k_scan_add(uint32_t* __restrict__ data, int64_t n,
                                                         const uint32_t* __restrict__ sums) {
    const int64_t base = (int64_t)blockIdx.x * kScanItems;
    const uint32_t add = sums[blockIdx.x];
    for (int k = threadIdx.x; k < kScanItems; k += kScanBlock) {
        const int64_t i = base + k;
        if (i < n) data[i] += add;
    }
}

__global__ void __launch_bounds__(kBlock) k_scatter(int n, const uint32_t* __restrict__ keys,
                                                    uint32_t* __restrict__ cursor, const float* __restrict__ pos_in,
                                                    const float* __restrict__ comp_in, const int32_t* __restrict__ ids_in,
                                                    float* __restrict__ pos_out, float* __restrict__ comp_out,
                                                    int32_t* __restrict__ ids_out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t slot = atomicAdd(cursor + keys[i], 1u);
    if (slot >= (uint32_t)n) return;  // impossible for a consistent histogram; never write out of range
    const int64_t s3 = 3 * (int64_t)slot, i3 = 3 * (int64_t)i;
    pos_out[s3] = pos_in[i3];
    pos_out[s3 + 1] = pos_in[i3 + 1];
    pos_out[s3 + 2] = pos_in[i3 + 2];
    if (comp_in != nullptr) {
        comp_out[s3] = comp_in[i3];
        comp_out[s3 + 1] = comp_in[i3 + 1];
        comp_out[s3 + 2] = comp_in[i3 + 2];
    }
    ids_out[slot] = ids_in != nullptr ? ids_in[i] : i;
}

__global__ void __launch_bounds__(kBlock) k_unpermute(int n, const float* __restrict__ src,
                                                      const int32_t* __restrict__ ids, float* __restrict__ dst) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int32_t d = ids[i];
    if (d < 0 || d >= n) return;
    dst[3 * (int64_t)d] = src[3 * (int64_t)i];
    dst[3 * (int64_t)d + 1] = src[3 * (int64_t)i + 1];
    dst[3 * (int64_t)d + 2] = src[3 * (int64_t)i + 2];
}

static int64_t n_bins(int bits) { return (int64_t)1 << (3 * bits); }

static int64_t scan_blocks(int64_t n) { return (n + kScanItems - 1) / kScanItems; }

int64_t scan_capacity() { return (int64_t)kScanItems * kScanItems * kScanItems; }

int64_t scan_partials(int64_t n) { return scan_blocks(n); }

int64_t scan_partials2(int64_t n) {
    const int64_t nb = scan_blocks(n);
    return nb > kScanItems ? scan_blocks(nb) + 1 : 1;
}

// Block scans, then the scan of the block totals: one block when they fit
// one (n <= kScanItems^2), else the same two levels again on them (sums2
// holds their block totals and the last total).
int exclusive_scan_u32(uint32_t* data, int64_t n, uint32_t* sums, uint32_t* sums2, cudaStream_t st) {
    if (n <= 0) return JT_OK;
    if (n > scan_capacity()) return set_error(JT_ERR_UNSUPPORTED, "scan of %lld items exceeds %lld", (long long)n,
                                              (long long)scan_capacity());
    const int64_t nb = scan_blocks(n);
    k_scan_blocks<<<(unsigned)nb, kScanBlock, 0, st>>>(data, n, sums);
    if (nb <= kScanItems) {
        k_scan_blocks<<<1, kScanBlock, 0, st>>>(sums, nb, sums2);
    } else {
        const int64_t nb2 = scan_blocks(nb);
        k_scan_blocks<<<(unsigned)nb2, kScanBlock, 0, st>>>(sums, nb, sums2);
        k_scan_blocks<<<1, kScanBlock, 0, st>>>(sums2, nb2, sums2 + nb2);
        k_scan_add<<<(unsigned)nb2, kScanBlock, 0, st>>>(sums, nb, sums2);
    }
    k_scan_add<<<(unsigned)nb, kScanBlock, 0, st>>>(data, n, sums);
    return cuda_status(cudaGetLastError(), "scan launch");
}

// Workspace layout (bytes, 256-aligned pieces): hist/cursor [bins], keys [n],
// block sums [scan_blocks(bins)], block-sum sums [1 block].
size_t sort_workspace_bytes(int32_t n, int32_t bits) {
    auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
    const int64_t bins = n_bins(bits);
    return al(bins * 4) + al((size_t)n * 4) + al(scan_blocks(bins) * 4) + al(4 * kScanItems);
}

int cell_sort(const jt_sort_grid& g, int32_t n, const float* pos_in, const float* comp_in, const int32_t* ids_in,
              float* pos_out, float* comp_out, int32_t* ids_out, void* ws, cudaStream_t st) {
    auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
    const int64_t bins = n_bins(g.bits);
    const int64_t nb = scan_blocks(bins);
    char* w = static_cast<char*>(ws);
    uint32_t* hist = reinterpret_cast<uint32_t*>(w);
    uint32_t* keys = reinterpret_cast<uint32_t*>(w + al(bins * 4));
    uint32_t* sums = reinterpret_cast<uint32_t*>(w + al(bins * 4) + al((size_t)n * 4));
    uint32_t* sums2 = reinterpret_cast<uint32_t*>(w + al(bins * 4) + al((size_t)n * 4) + al(nb * 4));
    cudaError_t e = cudaMemsetAsync(hist, 0, bins * 4, st);
    if (e != cudaSuccess) return cuda_status(e, "cell sort memset");
    k_cell_keys<<<grid_blocks(n), kBlock, 0, st>>>(g, pos_in, n, keys, hist);
    k_scan_blocks<<<(unsigned)nb, kScanBlock, 0, st>>>(hist, bins, sums);
    k_scan_blocks<<<1, kScanBlock, 0, st>>>(sums, nb, sums2);  // nb <= kScanItems (checked by the caller)
    k_scan_add<<<(unsigned)nb, kScanBlock, 0, st>>>(hist, bins, sums);
    k_scatter<<<grid_blocks(n), kBlock, 0, st>>>(n, keys, hist, pos_in, comp_in, ids_in, pos_out, comp_out, ids_out);
    return cuda_status(cudaGetLastError(), "cell sort launch");
}

}  // namespace jt

using namespace jt;

extern "C" size_t jt_cell_sort_workspace_bytes(int32_t n, int32_t bits) {
    if (n < 0 || bits < 1 || bits > 7) return 0;
    return sort_workspace_bytes(n, bits);
}

extern "C" int jt_cell_sort(const jt_sort_grid* g, int32_t n, const float* pos_in, const float* comp_in,
                            const int32_t* ids_in, float* pos_out, float* comp_out, int32_t* ids_out, void* workspace,
                            size_t workspace_bytes, void* stream) {
    if (g == nullptr) return set_error(JT_ERR_INVALID, "sort grid is NULL");
    if (g->bits < 1 || g->bits > 7) return set_error(JT_ERR_INVALID, "bits must be 1..7 (got %d)", g->bits);
    if (n < 0) return set_error(JT_ERR_INVALID, "n must be >= 0");
    if (n == 0) return JT_OK;
    if (pos_in == nullptr || pos_out == nullptr || ids_out == nullptr || workspace == nullptr)
        return set_error(JT_ERR_INVALID, "pos_in, pos_out, ids_out and workspace are required");
    if ((comp_in == nullptr) != (comp_out == nullptr))
        return set_error(JT_ERR_INVALID, "comp_in and comp_out go together");
    if (pos_in == pos_out || ids_in == ids_out) return set_error(JT_ERR_INVALID, "cell sort cannot run in place");
    if (workspace_bytes < sort_workspace_bytes(n, g->bits))
        return set_error(JT_ERR_NOMEM, "workspace of %zu bytes < %zu needed", workspace_bytes,
                         sort_workspace_bytes(n, g->bits));
    return cell_sort(*g, n, pos_in, comp_in, ids_in, pos_out, comp_out, ids_out, workspace, (cudaStream_t)stream);
}

extern "C" int jt_cell_list(const jt_sort_grid* g, int32_t n, const float* pos_in, float* pos_out, int32_t* ids_out,
                            uint32_t* cell_end, void* workspace, size_t workspace_bytes, void* stream) {
    if (cell_end == nullptr) return set_error(JT_ERR_INVALID, "cell_end is required");
    if (g == nullptr || g->bits < 1 || g->bits > 7) return set_error(JT_ERR_INVALID, "bits must be 1..7");
    cudaStream_t st = (cudaStream_t)stream;
    const int64_t bins = n_bins(g->bits);
    if (n == 0) return cuda_status(cudaMemsetAsync(cell_end, 0, bins * 4, st), "cell list memset");
    const int rc = jt_cell_sort(g, n, pos_in, nullptr, nullptr, pos_out, nullptr, ids_out, workspace, workspace_bytes,
                                stream);
    if (rc != JT_OK) return rc;
    // after the scatter the histogram words hold each cell's end offset
    return cuda_status(cudaMemcpyAsync(cell_end, workspace, bins * 4, cudaMemcpyDeviceToDevice, st),
                       "cell list copy");
}

// ---------------------------------------------------------------------------
// Allocation-free cell sort.
//
// Some callers cannot allocate device memory at the moment they call this
// library: a host application that owns all device memory through its own
// pool and lends the library nothing but its particle buffers, or a
// time-critical loop in which a cudaMalloc or cudaFree (both may synchronise
// the whole device) is not allowed.  jt_cell_sort_noalloc serves them: its
// scratch is one fixed-size array in the library's own device memory, sized
// for JT_NOALLOC_SORT_MAX_PARTICLES particles at up to
// JT_NOALLOC_SORT_MAX_BITS bits per axis (about 9 MiB, held on every GPU that
// loads the library until the process exits).
namespace {

constexpr size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

constexpr size_t sort_bytes_c(int64_t n, int bits) {
    return align256((size_t)(((int64_t)1 << (3 * bits)) * 4)) + align256((size_t)n * 4) +
           align256((size_t)((((int64_t)1 << (3 * bits)) + jt::kScanItems - 1) / jt::kScanItems) * 4) +
           align256((size_t)4 * jt::kScanItems);
}

constexpr size_t kNoAllocBytes = sort_bytes_c(JT_NOALLOC_SORT_MAX_PARTICLES, JT_NOALLOC_SORT_MAX_BITS);

// The scratch itself.  In host code this name is only a stand-in for the
// device array; the kernels get the device address obtained below.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

constexpr int kMaxDevices = 64;
static void* g_noalloc_addr[kMaxDevices];
static unsigned long long g_noalloc_ctx[kMaxDevices];  // context id the address belongs to
static std::mutex g_noalloc_mu;

// The driver's context queries, fetched through the runtime (the library
// does not link the driver library itself).
typedef int (*CtxGetCurrentFn)(void**);
typedef int (*CtxGetIdFn)(void*, unsigned long long*);
static CtxGetCurrentFn g_ctx_current = nullptr;
static CtxGetIdFn g_ctx_id = nullptr;
static std::once_flag g_ctx_once;

// Process-unique id of the calling thread's current context, 0 when there is
// none yet or the driver does not answer.  A device reset destroys the
// context; the next one gets a new id, and the scratch's module a possibly
// different address.
unsigned long long current_ctx_id() {
    std::call_once(g_ctx_once, [] {
        cudaDriverEntryPointQueryResult q;
        void* f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            g_ctx_current = reinterpret_cast<CtxGetCurrentFn>(f);
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            g_ctx_id = reinterpret_cast<CtxGetIdFn>(f);
    });
    if (g_ctx_current == nullptr || g_ctx_id == nullptr) return 0;
    void* ctx = nullptr;
    if (g_ctx_current(&ctx) != 0 || ctx == nullptr) return 0;
    unsigned long long id = 0;
    return g_ctx_id(ctx, &id) == 0 ? id : 0;
}

// Device address of the scratch on the current device, looked up with that
// device current and cached per device together with the id of the context
// it was looked up in: a call in another context (after a device reset) looks
// it up again.  Without a context id (no context yet, or a driver without
// the query) the lookup runs on every call.
int noalloc_scratch(void** out) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return jt::cuda_status(e, "cudaGetDevice");
    if (dev < 0 || dev >= kMaxDevices) return jt::set_error(JT_ERR_UNSUPPORTED, "device ordinal %d >= %d", dev, kMaxDevices);
    unsigned long long ctx = current_ctx_id();
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (g_noalloc_addr[dev] == nullptr || ctx == 0 || g_noalloc_ctx[dev] != ctx) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);  // makes the device's context current if none was
        if (e != cudaSuccess) return jt::cuda_status(e, "cudaGetSymbolAddress of the no-alloc sort scratch");
        if (ctx == 0) ctx = current_ctx_id();
        g_noalloc_addr[dev] = p;
        g_noalloc_ctx[dev] = ctx;
    }
    *out = g_noalloc_addr[dev];
    return JT_OK;
}

}  // namespace

extern "C" int jt_cell_sort_noalloc(const jt_sort_grid* g, int32_t n, const float* pos_in, const float* comp_in,
                                    const int32_t* ids_in, float* pos_out, float* comp_out, int32_t* ids_out,
                                    void* stream) {
    if (g == nullptr) return set_error(JT_ERR_INVALID, "sort grid is NULL");
    if (g->bits < 1 || g->bits > JT_NOALLOC_SORT_MAX_BITS)
        return set_error(JT_ERR_INVALID, "no-alloc sort takes 1..%d bits per axis (got %d)", JT_NOALLOC_SORT_MAX_BITS,
                         g->bits);
    if (n < 0) return set_error(JT_ERR_INVALID, "n must be >= 0");
    if (n > JT_NOALLOC_SORT_MAX_PARTICLES)
        return set_error(JT_ERR_INVALID, "no-alloc sort holds at most %d particles (got %d); use jt_cell_sort with a "
                         "workspace", JT_NOALLOC_SORT_MAX_PARTICLES, n);
    if (n == 0) return JT_OK;
    if (pos_in == nullptr || pos_out == nullptr || ids_out == nullptr)
        return set_error(JT_ERR_INVALID, "pos_in, pos_out and ids_out are required");
    if ((comp_in == nullptr) != (comp_out == nullptr))
        return set_error(JT_ERR_INVALID, "comp_in and comp_out go together");
    if (pos_in == pos_out || ids_in == ids_out) return set_error(JT_ERR_INVALID, "cell sort cannot run in place");
    void* ws = nullptr;
    const int rc = noalloc_scratch(&ws);
    if (rc != JT_OK) return rc;
    // cell_sort clears the histogram it accumulates into; every other scratch
    // word is written before it is read
    return cell_sort(*g, n, pos_in, comp_in, ids_in, pos_out, comp_out, ids_out, ws, (cudaStream_t)stream);
}

extern "C" int jt_unpermute(int32_t n, const float* pos_sorted, const int32_t* ids, float* pos_out, void* stream) {
    if (n < 0) return set_error(JT_ERR_INVALID, "n must be >= 0");
    if (n == 0) return JT_OK;
    if (pos_sorted == nullptr || ids == nullptr || pos_out == nullptr || pos_sorted == pos_out)
        return set_error(JT_ERR_INVALID, "pos_sorted, ids and a distinct pos_out are required");
    k_unpermute<<<grid_blocks(n), kBlock, 0, (cudaStream_t)stream>>>(n, pos_sorted, ids, pos_out);
    return cuda_status(cudaGetLastError(), "unpermute launch");
}
