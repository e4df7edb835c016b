// C-ABI entry points for the per-pair contact kernels (include/cipc.h).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>

#include "../../include/cipc.h"
#include "ccd_core.cuh"
#include "cipc_internal.h"
#include "cipc_util.h"

using namespace cipc;

namespace {

// host-mode staging: copies n*bytes from host to a new device buffer
template <typename T>
cudaError_t stage_in(T** dptr, const T* h, size_t count, cudaStream_t s)
{
    *dptr = nullptr;
    if (count == 0) return cudaSuccess;
    cudaError_t e = cudaMallocAsync((void**)dptr, count * sizeof(T), s);
    if (e != cudaSuccess) return e;
    if (h) return cudaMemcpyAsync(*dptr, h, count * sizeof(T), cudaMemcpyHostToDevice, s);
    return cudaSuccess;
}

// Host memory the current device can address directly (page-locked by
// cudaHostAlloc / cudaHostRegister, as torch's pin_memory does): returns its device
// address, or null for pageable memory.  The whole range must be one mapping.
const void* mapped_host(const void* p, size_t bytes)
{
    if (!p || bytes == 0) return nullptr;
    cudaPointerAttributes a0, a1;
    if (cudaPointerGetAttributes(&a0, p) != cudaSuccess || a0.type != cudaMemoryTypeHost || !a0.devicePointer) {
        cudaGetLastError();
        return nullptr;
    }
    const char* last = static_cast<const char*>(p) + bytes - 1;
    if (cudaPointerGetAttributes(&a1, last) != cudaSuccess || a1.type != cudaMemoryTypeHost || !a1.devicePointer ||
        static_cast<const char*>(a1.devicePointer) - static_cast<const char*>(a0.devicePointer) !=
            (ptrdiff_t)(bytes - 1)) {
        cudaGetLastError();
        return nullptr;
    }
    return a0.devicePointer;
}

}  // namespace

extern "C" int cipc_ccd_pairs(int64_t n, const uint8_t* type, const int32_t* idx, int64_t nv, const double* x,
                              const double* dx, double eta, double thickness, double toc_in, int precision,
                              int mem, double* toc_out, uint8_t* hit, int64_t* n_overflow, void* stream)
{
    if (n < 0 || nv < 0 || (n > 0 && (!type || !idx || !x || !dx || !toc_out || !hit)))
        return set_error(CIPC_ERR_INVALID_ARG, "cipc_ccd_pairs: null buffer or negative size");
    if (precision != CIPC_PRECISION_FP64 && precision != CIPC_PRECISION_MIXED)
        return set_error(CIPC_ERR_INVALID_ARG, "cipc_ccd_pairs: unknown precision");
    if (mem != CIPC_MEM_HOST && mem != CIPC_MEM_DEVICE)
        return set_error(CIPC_ERR_INVALID_ARG, "cipc_ccd_pairs: unknown memory kind");
    if (!(eta > 0 && eta < 1) || !(thickness >= 0) || !(toc_in > 0))
        return set_error(CIPC_ERR_INVALID_ARG, "cipc_ccd_pairs: need 0 < eta < 1, thickness >= 0, toc_in > 0");
    if (n_overflow) *n_overflow = 0;
    if (n == 0) return CIPC_OK;
    int rc = ensure_device();
    if (rc != CIPC_OK) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    const bool host = mem == CIPC_MEM_HOST;
    const bool exact = precision == CIPC_PRECISION_FP64;

    // Host buffers: the vertex arrays are copied first (any pair may use any
    // vertex); the pair records then arrive in chunks (2.5M pairs or more, at
    // most 64) on a copy stream while the kernel runs on the chunks already
    // there, and each chunk's results go back on a third stream as soon as its
    // kernel ends.  Device buffers, or one chunk: everything on the caller's stream.
    // Host buffers that are page-locked: the kernel reads the pairs and vertices
    // and writes the results in place, over the CPU-GPU link (NVLink-C2C on
    // Grace-Blackwell), with no staging copies; the call returns when they are
    // written.  Pageable host buffers take the staged path below.
    if (host) {
        const void *m_type = mapped_host(type, (size_t)n), *m_idx = mapped_host(idx, (size_t)n * 16),
                   *m_x = mapped_host(x, (size_t)nv * 24), *m_dx = mapped_host(dx, (size_t)nv * 24),
                   *m_toc = mapped_host(toc_out, (size_t)n * 8), *m_hit = mapped_host(hit, (size_t)n);
        if (m_type && m_idx && m_x && m_dx && m_toc && m_hit) {
            // one pass here: its FP64 work hides the link's read latency, while
            // the two-pass form's set-up pass would wait on the link with nothing
            // to overlap and its stepping pass would read the positions again
            unsigned long long* cnt_d = nullptr;
            unsigned long long cnt[3] = {0, 0, 0};
            cudaError_t e2 = cudaMallocAsync((void**)&cnt_d, sizeof(cnt), s);
            if (e2 == cudaSuccess) e2 = cudaMemsetAsync(cnt_d, 0, sizeof(cnt), s);
            if (e2 == cudaSuccess) {
                CcdArgs a;
                a.n = n;
                a.type = static_cast<const uint8_t*>(m_type);
                a.idx = static_cast<const int4*>(m_idx);
                a.x = static_cast<const double*>(m_x);
                a.dx = static_cast<const double*>(m_dx);
                a.eta = eta;
                a.th = thickness;
                a.toc_in = toc_in;
                a.max_iter = 1 << 20;
                a.nv = nv;
                a.toc_out = static_cast<double*>(const_cast<void*>(m_toc));
                a.hit = static_cast<uint8_t*>(const_cast<void*>(m_hit));
                a.iters = nullptr;
                a.counter = cnt_d;
                const int bps = exact ? accd_exact_blocks_per_sm() : accd_mixed_blocks_per_sm();
                int grid = num_sms() * bps;
                const int64_t need = (n + 255) / 256;
                if (need < grid) grid = (int)need;
                e2 = exact ? launch_accd_exact(a, grid, s) : launch_accd_mixed(a, grid, s);
            }
            if (e2 == cudaSuccess) e2 = cudaMemcpyAsync(cnt, cnt_d, sizeof(cnt), cudaMemcpyDeviceToHost, s);
            if (cnt_d) cudaFreeAsync(cnt_d, s);
            const cudaError_t e3 = cudaStreamSynchronize(s);
            if (e2 == cudaSuccess) e2 = e3;
            if (e2 != cudaSuccess) return set_cuda_error(e2, "cipc_ccd_pairs (page-locked host buffers)");
            if (n_overflow) *n_overflow = (int64_t)cnt[1];
            if (cnt[2])
                return set_error(CIPC_ERR_INDEX_RANGE, "cipc_ccd_pairs: %llu pairs with a bad type or vertex index",
                                 cnt[2]);
            if (cnt[1])
                return set_error(CIPC_ERR_ITER_CAP, "cipc_ccd_pairs: %llu pairs reached the iteration cap", cnt[1]);
            return CIPC_OK;
        }
    }

    const int64_t chunk = std::max<int64_t>(2500000, (n + 63) / 64);
    const int nchunk = host ? (int)((n + chunk - 1) / chunk) : 1;
    const bool pipelined = nchunk > 1;
    uint8_t *t_type = nullptr, *t_hit = nullptr;
    int32_t* t_idx = nullptr;
    double *t_x = nullptr, *t_dx = nullptr, *t_toc = nullptr;
    unsigned long long* counters = nullptr;
    AccdState* state = nullptr;  // FP64: per-pair set-up state of the two-pass kernels (one chunk's worth)
    cudaStream_t cin = nullptr, cout_ = nullptr;
    cudaEvent_t ev_verts = nullptr, ev_in[64], ev_out[64];
    int n_ev = 0;
    cudaError_t e = cudaSuccess;
#define CK(call)                    \
    do {                            \
        e = (call);                 \
        if (e != cudaSuccess) goto done; \
    } while (0)
    CK(cudaMallocAsync((void**)&counters, 3 * (size_t)nchunk * sizeof(unsigned long long), s));
    // one record per pair of the largest launch: a chunk when pipelined, else the whole list
    if (exact) CK(cudaMallocAsync((void**)&state, (size_t)(pipelined ? chunk : n) * sizeof(AccdState), s));
    CK(cudaMemsetAsync(counters, 0, 3 * (size_t)nchunk * sizeof(unsigned long long), s));
    if (host) {
        CK(stage_in(&t_x, x, (size_t)nv * 3, s));
        CK(stage_in(&t_dx, dx, (size_t)nv * 3, s));
        CK(stage_in(&t_type, (const uint8_t*)nullptr, (size_t)n, s));
        CK(stage_in(&t_idx, (const int32_t*)nullptr, (size_t)n * 4, s));
        CK(stage_in(&t_toc, (const double*)nullptr, (size_t)n, s));
        CK(stage_in(&t_hit, (const uint8_t*)nullptr, (size_t)n, s));
    }
    if (pipelined) {
        CK(cudaStreamCreateWithFlags(&cin, cudaStreamNonBlocking));
        CK(cudaStreamCreateWithFlags(&cout_, cudaStreamNonBlocking));
        CK(cudaEventCreateWithFlags(&ev_verts, cudaEventDisableTiming));
        CK(cudaEventRecord(ev_verts, s));  // allocations and vertex copies done
        CK(cudaStreamWaitEvent(cin, ev_verts, 0));
        for (int c = 0; c < nchunk; ++c) {
            ev_in[c] = ev_out[c] = nullptr;
            n_ev = c + 1;
            CK(cudaEventCreateWithFlags(&ev_in[c], cudaEventDisableTiming));
            CK(cudaEventCreateWithFlags(&ev_out[c], cudaEventDisableTiming));
        }
    }
    {
        const int bps = exact ? accd_exact_steps_blocks_per_sm() : accd_mixed_blocks_per_sm();
        for (int c = 0; c < nchunk; ++c) {
            const int64_t off = (int64_t)c * chunk, m = std::min<int64_t>(chunk, n - off);
            if (host) {
                cudaStream_t cs = pipelined ? cin : s;
                CK(cudaMemcpyAsync(t_type + off, type + off, (size_t)m, cudaMemcpyHostToDevice, cs));
                CK(cudaMemcpyAsync(t_idx + 4 * off, idx + 4 * off, (size_t)m * 4 * sizeof(int32_t),
                                   cudaMemcpyHostToDevice, cs));
                if (pipelined) {
                    CK(cudaEventRecord(ev_in[c], cin));
                    CK(cudaStreamWaitEvent(s, ev_in[c], 0));
                }
            }
            CcdArgs a;
            a.n = host ? m : n;
            a.type = host ? t_type + off : type;
            a.idx = reinterpret_cast<const int4*>(host ? t_idx + 4 * off : idx);
            a.x = host ? t_x : x;
            a.dx = host ? t_dx : dx;
            a.eta = eta;
            a.th = thickness;
            a.toc_in = toc_in;
            a.max_iter = 1 << 20;
            a.nv = nv;
            a.toc_out = host ? t_toc + off : toc_out;
            a.hit = host ? t_hit + off : hit;
            a.iters = nullptr;
            a.counter = counters + 3 * c;
            int grid = num_sms() * bps;
            const int64_t need = (a.n + 255) / 256;
            if (need < grid) grid = (int)need;
            CK(exact ? launch_accd_exact_split(a, state, grid, s) : launch_accd_mixed(a, grid, s));
            if (host) {
                cudaStream_t cs = pipelined ? cout_ : s;
                if (pipelined) {
                    CK(cudaEventRecord(ev_out[c], s));
                    CK(cudaStreamWaitEvent(cout_, ev_out[c], 0));
                }
                CK(cudaMemcpyAsync(toc_out + off, t_toc + off, (size_t)m * sizeof(double), cudaMemcpyDeviceToHost,
                                   cs));
                CK(cudaMemcpyAsync(hit + off, t_hit + off, (size_t)m, cudaMemcpyDeviceToHost, cs));
            }
        }
    }
    if (n_overflow || host) {
        unsigned long long cnt[3 * 64];
        CK(cudaMemcpyAsync(cnt, counters, 3 * (size_t)nchunk * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                           s));
        CK(cudaStreamSynchronize(s));
        if (cout_) CK(cudaStreamSynchronize(cout_));
        unsigned long long over = 0, bad = 0;
        for (int c = 0; c < nchunk; ++c) {
            over += cnt[3 * c + 1];
            bad += cnt[3 * c + 2];
        }
        if (n_overflow) *n_overflow = (int64_t)over;
        if (bad)
            rc = set_error(CIPC_ERR_INDEX_RANGE, "cipc_ccd_pairs: %llu pairs with a bad type or vertex index", bad);
        else if (over)
            rc = set_error(CIPC_ERR_ITER_CAP, "cipc_ccd_pairs: %llu pairs reached the iteration cap", over);
    }
done:
    if (cout_) cudaStreamSynchronize(cout_);  // result copies finished before their sources are freed
    if (cin) cudaStreamSynchronize(cin);
    if (counters) cudaFreeAsync(counters, s);
    if (state) cudaFreeAsync(state, s);
    if (t_type) cudaFreeAsync(t_type, s);
    if (t_idx) cudaFreeAsync(t_idx, s);
    if (t_x) cudaFreeAsync(t_x, s);
    if (t_dx) cudaFreeAsync(t_dx, s);
    if (t_toc) cudaFreeAsync(t_toc, s);
    if (t_hit) cudaFreeAsync(t_hit, s);
    if (host) cudaStreamSynchronize(s);
    for (int c = 0; c < n_ev; ++c) {
        if (ev_in[c]) cudaEventDestroy(ev_in[c]);
        if (ev_out[c]) cudaEventDestroy(ev_out[c]);
    }
    if (ev_verts) cudaEventDestroy(ev_verts);
    if (cin) cudaStreamDestroy(cin);
    if (cout_) cudaStreamDestroy(cout_);
    if (e != cudaSuccess) return set_cuda_error(e, "cipc_ccd_pairs");
    return rc;
#undef CK
}

extern "C" int cipc_barrier_pairs(int64_t n, const uint8_t* type, const int32_t* idx, int64_t nv, const double* x,
                                  const double* x_rest, double dhat2, double xi, double kappa, int project_pd,
                                  int precision, int mem, double* energy, double* grad, void* hess,
                                  int64_t* n_nonpositive, void* stream)
{
    if (n < 0 || nv < 0 || (n > 0 && (!type || !idx || !x || !x_rest || !energy || !grad || !hess)))
        return set_error(CIPC_ERR_INVALID_ARG, "cipc_barrier_pairs: null buffer or negative size");
    if (precision != CIPC_PRECISION_FP64 && precision != CIPC_PRECISION_MIXED)
        return set_error(CIPC_ERR_INVALID_ARG, "cipc_barrier_pairs: unknown precision");
    if (mem != CIPC_MEM_HOST && mem != CIPC_MEM_DEVICE)
        return set_error(CIPC_ERR_INVALID_ARG, "cipc_barrier_pairs: unknown memory kind");
    if (!(dhat2 > 0) || !(xi >= 0) || !(kappa > 0))
        return set_error(CIPC_ERR_INVALID_ARG, "cipc_barrier_pairs: need dhat2 > 0, xi >= 0, kappa > 0");
    if (n_nonpositive) *n_nonpositive = 0;
    if (n == 0) return CIPC_OK;
    int rc = ensure_device();
    if (rc != CIPC_OK) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    const size_t hbytes = (size_t)n * 78 * (precision == CIPC_PRECISION_FP64 ? sizeof(double) : sizeof(float));

    const uint8_t* d_type = type;
    const int32_t* d_idx = idx;
    const double *d_x = x, *d_xr = x_rest;
    double *d_E = energy, *d_g = grad;
    void* d_h = hess;
    uint8_t* t_type = nullptr;
    int32_t* t_idx = nullptr;
    double *t_x = nullptr, *t_xr = nullptr, *t_E = nullptr, *t_g = nullptr;
    char* t_h = nullptr;
    unsigned long long* counters = nullptr;
    cudaError_t e = cudaSuccess;
#define CK(call)                    \
    do {                            \
        e = (call);                 \
        if (e != cudaSuccess) goto done; \
    } while (0)
    if (mem == CIPC_MEM_HOST) {
        CK(stage_in(&t_type, type, (size_t)n, s));
        CK(stage_in(&t_idx, idx, (size_t)n * 4, s));
        CK(stage_in(&t_x, x, (size_t)nv * 3, s));
        CK(stage_in(&t_xr, x_rest, (size_t)nv * 3, s));
        CK(stage_in(&t_E, (const double*)nullptr, (size_t)n, s));
        CK(stage_in(&t_g, (const double*)nullptr, (size_t)n * 12, s));
        CK(stage_in(&t_h, (const char*)nullptr, hbytes, s));
        d_type = t_type;
        d_idx = t_idx;
        d_x = t_x;
        d_xr = t_xr;
        d_E = t_E;
        d_g = t_g;
        d_h = t_h;
    }
    CK(cudaMallocAsync((void**)&counters, 4 * sizeof(unsigned long long), s));
    CK(cudaMemsetAsync(counters, 0, 4 * sizeof(unsigned long long), s));
    {
        BarrierLaunch L;
        L.n = n;
        L.type = d_type;
        L.idx = d_idx;
        L.x = d_x;
        L.x_rest = d_xr;
        L.xi2 = xi * xi;
        L.shat = dhat2 + 2 * std::sqrt(dhat2) * xi;
        L.kappa = kappa;
        L.project = project_pd ? 1 : 0;
        L.fp64_hessian = precision == CIPC_PRECISION_FP64;
        L.nv = nv;
        L.E = d_E;
        L.grad = d_g;
        L.hess = d_h;
        L.bad = counters;
        CK(launch_barrier(L, s));
    }
    if (mem == CIPC_MEM_HOST) {
        CK(cudaMemcpyAsync(energy, d_E, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost, s));
        CK(cudaMemcpyAsync(grad, d_g, (size_t)n * 12 * sizeof(double), cudaMemcpyDeviceToHost, s));
        CK(cudaMemcpyAsync(hess, d_h, hbytes, cudaMemcpyDeviceToHost, s));
    }
    if (n_nonpositive || mem == CIPC_MEM_HOST) {
        unsigned long long cnt[2] = {0, 0};
        CK(cudaMemcpyAsync(cnt, counters, sizeof(cnt), cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        if (n_nonpositive) *n_nonpositive = (int64_t)cnt[0];
        if (cnt[1])
            rc = set_error(CIPC_ERR_INDEX_RANGE, "cipc_barrier_pairs: %llu pairs with a bad type or vertex index",
                           cnt[1]);
        else if (cnt[0])
            rc = set_error(CIPC_ERR_NONPOSITIVE_DISTANCE, "cipc_barrier_pairs: %llu pairs at or below the offset",
                           cnt[0]);
    }
done:
    if (counters) cudaFreeAsync(counters, s);
    if (t_type) cudaFreeAsync(t_type, s);
    if (t_idx) cudaFreeAsync(t_idx, s);
    if (t_x) cudaFreeAsync(t_x, s);
    if (t_xr) cudaFreeAsync(t_xr, s);
    if (t_E) cudaFreeAsync(t_E, s);
    if (t_g) cudaFreeAsync(t_g, s);
    if (t_h) cudaFreeAsync(t_h, s);
    if (mem == CIPC_MEM_HOST) cudaStreamSynchronize(s);
    if (e != cudaSuccess) return set_cuda_error(e, "cipc_barrier_pairs");
    return rc;
#undef CK
}

extern "C" int cipc_encode_reference_constraint(int type, const int32_t* idx4, int mollified, int multiplicity,
                                                int32_t* code4)
{
    if (!idx4 || !code4 || type < 0 || type > 3 || multiplicity < 1)
        return set_error(CIPC_ERR_INVALID_ARG, "cipc_encode_reference_constraint: bad argument");
    const int32_t a = idx4[0], b = idx4[1], c = idx4[2], d = idx4[3];
    switch (type) {
        case CIPC_PAIR_PT: code4[0] = -a - 1; code4[1] = b; code4[2] = c; code4[3] = d; break;
        case CIPC_PAIR_PE: code4[0] = -a - 1; code4[1] = b; code4[2] = c; code4[3] = -multiplicity; break;
        case CIPC_PAIR_PP: code4[0] = -a - 1; code4[1] = b; code4[2] = -1; code4[3] = -multiplicity; break;
        default:
            code4[0] = a;
            code4[1] = b;
            code4[2] = mollified ? -c - 1 : c;
            code4[3] = d;
    }
    return CIPC_OK;
}
