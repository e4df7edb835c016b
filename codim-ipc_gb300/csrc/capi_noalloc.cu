// cipc_ccd_pairs_noalloc (include/cipc.h): the device-memory CCD over pairs
// with its kernel counters taken from a scratch array compiled into the library.
// Nothing on this path allocates: no cudaMalloc / cudaMallocAsync / cudaFree,
// no allocating library call; the only CUDA calls are cudaGetDevice, the
// context-id lookup, cudaGetSymbolAddress (once per device context),
// cudaMemsetAsync, the kernel launch
// and, when counts are asked for, one device-to-host copy of 24 bytes.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/cipc.h"
#include "ccd_core.cuh"
#include "cipc_internal.h"
#include "cipc_util.h"

using namespace cipc;

namespace {

constexpr int kSlots = CIPC_NOALLOC_SLOTS;
constexpr int kSlotWords = CIPC_NOALLOC_SLOT_BYTES / sizeof(unsigned long long);
// k_accd uses [0] work counter, [1] overflow count, [2] invalid-pair count
constexpr int kCcdWords = 3;
static_assert(kCcdWords <= kSlotWords, "CCD counters must fit one scratch slot");
static_assert(CIPC_NOALLOC_SLOT_BYTES % 128 == 0, "slots are whole 128-byte lines (no sharing across streams)");

// 16 slots x 128 bytes = 2 KB per device; one copy per device context
static __device__ __align__(256) unsigned long long g_ccd_scratch[kSlots * kSlotWords];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
unsigned long long* g_addr[kMaxDevices] = {};
unsigned long long g_ctx[kMaxDevices] = {};  // id of the context the address belongs to

// The address of g_ccd_scratch belongs to the device's current context.  After a
// cudaDeviceReset (or any new primary context) the old address is unmapped, so
// the cache is keyed on the driver's unique context id (cuCtxGetId, looked up
// through the runtime so that the library keeps no link-time libcuda
// dependency); without that entry point the id stays 0 and the address is
// looked up once per device.
typedef int (*PfnCtxGetCurrent)(void**);
typedef int (*PfnCtxGetId)(void*, unsigned long long*);

unsigned long long current_context_id()
{
    static PfnCtxGetCurrent get_cur = nullptr;
    static PfnCtxGetId get_id = nullptr;
    static bool looked_up = false;
    if (!looked_up) {
        looked_up = true;
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_cur = reinterpret_cast<PfnCtxGetCurrent>(f);
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<PfnCtxGetId>(f);
    }
    if (!get_cur || !get_id) return 0;
    void* ctx = nullptr;
    unsigned long long id = 0;
    if (get_cur(&ctx) != 0 || !ctx || get_id(ctx, &id) != 0) return 0;
    return id;
}

int scratch_slot(int slot, unsigned long long** out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return set_cuda_error(e, "cipc_ccd_pairs_noalloc: cudaGetDevice");
    if (dev < 0 || dev >= kMaxDevices)
        return set_error(CIPC_ERR_INVALID_ARG, "cipc_ccd_pairs_noalloc: device %d beyond %d", dev, kMaxDevices);
    std::lock_guard<std::mutex> lk(g_mu);
    const unsigned long long ctx = current_context_id();
    if (!g_addr[dev] || g_ctx[dev] != ctx) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_ccd_scratch);
        if (e != cudaSuccess) return set_cuda_error(e, "cipc_ccd_pairs_noalloc: cudaGetSymbolAddress");
        g_addr[dev] = static_cast<unsigned long long*>(p);
        g_ctx[dev] = ctx;
    }
    *out = g_addr[dev] + (size_t)slot * kSlotWords;
    return CIPC_OK;
}

}  // namespace

extern "C" int cipc_ccd_pairs_noalloc(int64_t n, const uint8_t* type, const int32_t* idx, int64_t nv,
                                      const double* x, const double* dx, double eta, double thickness,
                                      double toc_in, int precision, int slot, double* toc_out, uint8_t* hit,
                                      int64_t* n_overflow, void* stream)
{
    if (n < 0 || nv < 0 || (n > 0 && (!type || !idx || !x || !dx || !toc_out || !hit)))
        return set_error(CIPC_ERR_INVALID_ARG, "cipc_ccd_pairs_noalloc: null buffer or negative size");
    if (precision != CIPC_PRECISION_FP64 && precision != CIPC_PRECISION_MIXED)
        return set_error(CIPC_ERR_INVALID_ARG, "cipc_ccd_pairs_noalloc: unknown precision");
    if (slot < 0 || slot >= kSlots)
        return set_error(CIPC_ERR_INVALID_ARG, "cipc_ccd_pairs_noalloc: slot %d outside [0, %d)", slot, kSlots);
    if (!(eta > 0 && eta < 1) || !(thickness >= 0) || !(toc_in > 0))
        return set_error(CIPC_ERR_INVALID_ARG,
                         "cipc_ccd_pairs_noalloc: need 0 < eta < 1, thickness >= 0, toc_in > 0");
    if (n_overflow) *n_overflow = 0;
    if (n == 0) return CIPC_OK;
    int rc = ensure_device();
    if (rc != CIPC_OK) return rc;
    unsigned long long* counters = nullptr;
    if ((rc = scratch_slot(slot, &counters))) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = cudaMemsetAsync(counters, 0, kCcdWords * sizeof(unsigned long long), s);
    if (e != cudaSuccess) return set_cuda_error(e, "cipc_ccd_pairs_noalloc: zeroing the slot");
    CcdArgs a;
    a.n = n;
    a.type = type;
    a.idx = reinterpret_cast<const int4*>(idx);
    a.x = x;
    a.dx = dx;
    a.eta = eta;
    a.th = thickness;
    a.toc_in = toc_in;
    a.max_iter = 1 << 20;
    a.nv = nv;
    a.toc_out = toc_out;
    a.hit = hit;
    a.iters = nullptr;
    a.counter = counters;
    const bool exact = precision == CIPC_PRECISION_FP64;
    const int bps = exact ? accd_exact_blocks_per_sm() : accd_mixed_blocks_per_sm();
    int grid = num_sms() * bps;
    const int64_t need = (n + 255) / 256;
    if (need < grid) grid = (int)need;
    e = exact ? launch_accd_exact(a, grid, s) : launch_accd_mixed(a, grid, s);
    if (e != cudaSuccess) return set_cuda_error(e, "cipc_ccd_pairs_noalloc: launch");
    if (!n_overflow) return CIPC_OK;
    unsigned long long cnt[kCcdWords] = {0, 0, 0};
    e = cudaMemcpyAsync(cnt, counters, sizeof(cnt), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return set_cuda_error(e, "cipc_ccd_pairs_noalloc: reading the counters");
    *n_overflow = (int64_t)cnt[1];
    if (cnt[2])
        return set_error(CIPC_ERR_INDEX_RANGE, "cipc_ccd_pairs_noalloc: %llu pairs with a bad type or vertex index",
                         cnt[2]);
    if (cnt[1])
        return set_error(CIPC_ERR_ITER_CAP, "cipc_ccd_pairs_noalloc: %llu pairs reached the iteration cap", cnt[1]);
    return CIPC_OK;
}
