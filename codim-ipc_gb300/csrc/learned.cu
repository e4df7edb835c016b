// Learned block-Jacobi correction for the Newton-system PCG: features, FP32
// forward/backward/Adam training kernels, the BF16 tensor-core inference path,
// triple capture and the C ABI (include/cipc.h, cipc_precond_*).
//
// Parameter layout (floats): W0 (H x 10), b0 (H), then per layer l: A_l, B_l,
// C_l (H x H each, row-major: out x in), b_l (H), then Wo (6 x H), bo (6).
// Activations are vertex-major (nv x H).  Every per-vertex formula is the one in
// oracle/oracle_learned.cpp, which the tests compare against.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <random>
#include <vector>

#include "../../include/cipc.h"
#include "cipc_util.h"
#include "constraint_eval.cuh"
#include "learned.h"
#include "sim_kernels.h"

namespace cipc {

namespace {

inline int nb(long long n, int bs) { return n > 0 ? (int)((n + bs - 1) / bs) : 1; }

struct LpOff {
    int W0, b0, Wo, bo;
    int A[8], B[8], C[8], b[8];
};

LpOff offsets(int H, int L)
{
    LpOff o;
    int p = 0;
    o.W0 = p;
    p += H * kLpFeatures;
    o.b0 = p;
    p += H;
    for (int l = 0; l < L; ++l) {
        o.A[l] = p;
        p += H * H;
        o.B[l] = p;
        p += H * H;
        o.C[l] = p;
        p += H * H;
        o.b[l] = p;
        p += H;
    }
    o.Wo = p;
    p += kLpOut * H;
    o.bo = p;
    return o;
}

int num_params(int H, int L) { return H * kLpFeatures + H + L * (3 * H * H + H) + kLpOut * H + kLpOut; }

__device__ __forceinline__ void inv3d(const double* A, double* inv)
{
    const double c00 = A[4] * A[8] - A[5] * A[7], c01 = A[5] * A[6] - A[3] * A[8], c02 = A[3] * A[7] - A[4] * A[6];
    const double det = A[0] * c00 + A[1] * c01 + A[2] * c02;
    if (!(fabs(det) > 0)) {
        for (int k = 0; k < 9; ++k) inv[k] = (k % 4 == 0) ? 1.0 : 0.0;
        return;
    }
    const double id = 1.0 / det;
    inv[0] = c00 * id;
    inv[3] = c01 * id;
    inv[6] = c02 * id;
    inv[1] = (A[2] * A[7] - A[1] * A[8]) * id;
    inv[4] = (A[0] * A[8] - A[2] * A[6]) * id;
    inv[7] = (A[1] * A[6] - A[0] * A[7]) * id;
    inv[2] = (A[1] * A[5] - A[2] * A[4]) * id;
    inv[5] = (A[2] * A[3] - A[0] * A[5]) * id;
    inv[8] = (A[0] * A[4] - A[1] * A[3]) * id;
}

// block sum of two doubles into red[0..1] (atomics, one per block)
__device__ __forceinline__ void block_add2(double a, double b, double* red)
{
    __shared__ double sh[2][32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, o);
        b += __shfl_down_sync(0xffffffffu, b, o);
    }
    if (lane == 0) {
        sh[0][wid] = a;
        sh[1][wid] = b;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double s0 = 0, s1 = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
            s0 += sh[0][w];
            s1 += sh[1][w];
        }
        atomicAdd(red, s0);
        atomicAdd(red + 1, s1);
    }
}

// ---------------------------------------------------------------------------
// features
// ---------------------------------------------------------------------------
__global__ void k_lp_count(int ncon, const int* ckind, const int4* cverts, int* ncnt)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncon) return;
    const int n = con_nv(ckind[c]);
    const int4 v = cverts[c];
    const int id[4] = {v.x, v.y, v.z, v.w};
    for (int q = 0; q < n; ++q) atomicAdd(ncnt + id[q], 1);
}

template <typename VT, typename CT>
__device__ __forceinline__ void diag_block(const LpSys<VT, CT>& S, int i, double* D)
{
    const VT* B = S.val + 9 * (size_t)S.diag[i];
    for (int q = 0; q < 9; ++q) D[q] = (double)B[q] + (double)S.cdiag[9 * (size_t)i + q];
}

// E = D^-1, Dn = |D|_F; red[0..1] += (trace(D)/3, 1) over free vertices
template <typename VT, typename CT>
__global__ void k_lp_diag(LpSys<VT, CT> S, float* E, float* Dn, double* red)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double tr = 0, one = 0;
    if (i < S.nv) {
        double D[9], inv[9];
        diag_block(S, i, D);
        inv3d(D, inv);
        double f = 0;
        for (int q = 0; q < 9; ++q) {
            E[9 * (size_t)i + q] = (float)inv[q];
            f += D[q] * D[q];
        }
        Dn[i] = (float)sqrt(f);
        if (!S.proj[i]) {
            tr = (D[0] + D[4] + D[8]) / 3;
            one = 1;
        }
    }
    block_add2(tr, one, red);
}

// edge weights a (K x nv), their row sums s, and the 10 features per vertex
template <typename VT, typename CT>
__global__ void k_lp_feat(LpSys<VT, CT> S, const float* Dn, const int* ncnt, const double* red, float* X, float* a,
                          float* s)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= S.nv) return;
    const int nv = S.nv;
    const double dbar = red[1] > 0 ? red[0] / red[1] : 1.0;
    const double dni = Dn[i];
    double sum = 0;
    for (int k = 0; k < S.K; ++k) {
        const size_t e = (size_t)k * nv + i;
        const int j = S.col[e];
        const VT* B = S.val + 9 * e;
        double bn = 0;
        for (int q = 0; q < 9; ++q) bn += (double)B[q] * (double)B[q];
        bn = sqrt(bn);
        const double dnj = Dn[j];
        double w = 0;
        if (j != i && bn > 0 && dni > 0 && dnj > 0) w = bn / sqrt(dni * dnj);
        a[e] = (float)w;
        sum += w;
    }
    s[i] = (float)sum;
    double D[9];
    diag_block(S, i, D);
    float* x = X + (size_t)kLpFeatures * i;
    for (int q = 0; q < 3; ++q) x[q] = (float)log(fmax(D[4 * q], 1e-30) / dbar);
    const double d0 = sqrt(fmax(D[0], 1e-30)), d1 = sqrt(fmax(D[4], 1e-30)), d2 = sqrt(fmax(D[8], 1e-30));
    x[3] = (float)(D[1] / (d0 * d1));
    x[4] = (float)(D[2] / (d0 * d2));
    x[5] = (float)(D[5] / (d1 * d2));
    x[6] = (float)log(1e-6 + sum);
    double cf = 0;
    for (int q = 0; q < 9; ++q) cf += (double)S.cdiag[9 * (size_t)i + q] * (double)S.cdiag[9 * (size_t)i + q];
    x[7] = dni > 0 ? (float)(sqrt(cf) / dni) : 0.f;
    x[8] = S.proj[i] ? 1.f : 0.f;
    x[9] = (float)(fmin((double)ncnt[i], 8.0) / 8.0);
}


// P = Cm E Cm^T with Cm = [[e0,0,0],[l3,e1,0],[l4,l5,e2]], e_a = exp(0.5 clamp(o_a, -2, 2)),
// l_a = clamp(o_a, -1, 1): the correction can rescale a block by at most e^2 and
// shear it by a bounded amount, so no network output makes PCG arbitrarily worse
// than block Jacobi
constexpr float kLpDiagClamp = 2.f, kLpOffClamp = 1.f;
__device__ __forceinline__ void lp_block(const float* o, const float* E, float* P, float* Cout)
{
    float e[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) e[a] = expf(0.5f * fminf(kLpDiagClamp, fmaxf(-kLpDiagClamp, o[a])));
    const float l3 = fminf(kLpOffClamp, fmaxf(-kLpOffClamp, o[3]));
    const float l4 = fminf(kLpOffClamp, fmaxf(-kLpOffClamp, o[4]));
    const float l5 = fminf(kLpOffClamp, fmaxf(-kLpOffClamp, o[5]));
    const float C[9] = {e[0], 0.f, 0.f, l3, e[1], 0.f, l4, l5, e[2]};
    float CE[9];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int q = 0; q < 3; ++q) CE[3 * r + q] = C[3 * r] * E[q] + C[3 * r + 1] * E[3 + q] + C[3 * r + 2] * E[6 + q];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int q = 0; q < 3; ++q)
            P[3 * r + q] = CE[3 * r] * C[3 * q] + CE[3 * r + 1] * C[3 * q + 1] + CE[3 * r + 2] * C[3 * q + 2];
    if (Cout)
#pragma unroll
        for (int k = 0; k < 9; ++k) Cout[k] = C[k];
}

// ---------------------------------------------------------------------------
// forward (FP32)
// ---------------------------------------------------------------------------
// h0 = relu(W0 x + b0), u0 = the pre-activation
template <int H>
__global__ void k_lp_in(int nv, const float* X, const float* W0, const float* b0, float* u0, float* h0)
{
    extern __shared__ float sw[];
    for (int k = threadIdx.x; k < H * kLpFeatures + H; k += blockDim.x)
        sw[k] = k < H * kLpFeatures ? W0[k] : b0[k - H * kLpFeatures];
    __syncthreads();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    float x[kLpFeatures];
#pragma unroll
    for (int f = 0; f < kLpFeatures; ++f) x[f] = X[(size_t)kLpFeatures * i + f];
#pragma unroll 1
    for (int r = 0; r < H; ++r) {
        float t = sw[H * kLpFeatures + r];
#pragma unroll
        for (int f = 0; f < kLpFeatures; ++f) t += sw[r * kLpFeatures + f] * x[f];
        u0[(size_t)H * i + r] = t;
        h0[(size_t)H * i + r] = fmaxf(t, 0.f);
    }
}

// g_i = sum_k a_ki h_col / s_i, one thread per (vertex, channel)
__global__ void k_lp_gather(int nv, int K, int H, const int* col, const float* a, const float* s, const float* h,
                            float* g)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)nv * H) return;
    const int i = (int)(t / H), q = (int)(t - (long long)i * H);
    const float si = s[i];
    float acc = 0;
    if (si > 0)
        for (int k = 0; k < K; ++k) {
            const size_t e = (size_t)k * nv + i;
            const float w = a[e];
            if (w != 0.f) acc += (w / si) * h[(size_t)H * col[e] + q];
        }
    g[t] = acc;
}

// acc_v += mean over the constraint's vertices of h, one thread per (constraint, channel)
__global__ void k_lp_con_acc(int ncon, int H, const int* ckind, const int4* cverts, const float* h, float* acc)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)ncon * H) return;
    const int c = (int)(t / H), q = (int)(t - (long long)c * H);
    const int n = con_nv(ckind[c]);
    const int4 v = cverts[c];
    const int id[4] = {v.x, v.y, v.z, v.w};
    float m = 0;
    for (int k = 0; k < n; ++k) m += h[(size_t)H * id[k] + q];
    m /= (float)n;
    for (int k = 0; k < n; ++k) atomicAdd(acc + (size_t)H * id[k] + q, m);
}

// c = acc / max(1, n); u = A h + B g + C c + b; h_out = relu(u) + h_in
template <int H>
__global__ void k_lp_layer(int nv, const float* h, const float* g, const float* acc, const int* ncnt,
                           const float* W, float* c, float* u, float* hout)
{
    extern __shared__ float sw[];  // A, B, C (H x H each), b (H)
    for (int k = threadIdx.x; k < 3 * H * H + H; k += blockDim.x) sw[k] = W[k];
    __syncthreads();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    float hv[H], gv[H], cv[H];
    const float inv = 1.f / fmaxf(1.f, (float)ncnt[i]);
#pragma unroll
    for (int q = 0; q < H; ++q) {
        hv[q] = h[(size_t)H * i + q];
        gv[q] = g[(size_t)H * i + q];
        cv[q] = acc[(size_t)H * i + q] * inv;
        c[(size_t)H * i + q] = cv[q];
    }
    const float* A = sw;
    const float* B = sw + H * H;
    const float* C = sw + 2 * H * H;
    const float* b = sw + 3 * H * H;
#pragma unroll 1
    for (int r = 0; r < H; ++r) {
        float t = b[r];
#pragma unroll
        for (int q = 0; q < H; ++q) t += A[r * H + q] * hv[q] + B[r * H + q] * gv[q] + C[r * H + q] * cv[q];
        u[(size_t)H * i + r] = t;
        hout[(size_t)H * i + r] = fmaxf(t, 0.f) + h[(size_t)H * i + r];
    }
}

// o = Wo h + bo; Cm from o; P = Cm E Cm^T; z = P r (if r), pinv = P (if pinv)
template <int H, typename PT>
__global__ void k_lp_out(int nv, const float* h, const float* Wo, const float* bo, const float* E, const float* r,
                         float* o_out, float* z, PT* pinv)
{
    __shared__ float sw[kLpOut * H + kLpOut];
    for (int k = threadIdx.x; k < kLpOut * H + kLpOut; k += blockDim.x)
        sw[k] = k < kLpOut * H ? Wo[k] : bo[k - kLpOut * H];
    __syncthreads();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    float hv[H];
#pragma unroll
    for (int q = 0; q < H; ++q) hv[q] = h[(size_t)H * i + q];
    float o[kLpOut];
#pragma unroll
    for (int k = 0; k < kLpOut; ++k) {
        float t = sw[kLpOut * H + k];
#pragma unroll
        for (int q = 0; q < H; ++q) t += sw[k * H + q] * hv[q];
        o[k] = t;
        if (o_out) o_out[(size_t)kLpOut * i + k] = t;
    }
    float P[9];
    lp_block(o, E + 9 * (size_t)i, P, nullptr);
    if (pinv)
#pragma unroll
        for (int k = 0; k < 9; ++k) pinv[9 * (size_t)i + k] = (PT)P[k];
    if (z) {
        const float r0 = r[3 * i], r1 = r[3 * i + 1], r2 = r[3 * i + 2];
        z[3 * i] = P[0] * r0 + P[1] * r1 + P[2] * r2;
        z[3 * i + 1] = P[3] * r0 + P[4] * r1 + P[5] * r2;
        z[3 * i + 2] = P[6] * r0 + P[7] * r1 + P[8] * r2;
    }
}


// ---------------------------------------------------------------------------
// loss and backward (FP32, reductions in FP64)
// ---------------------------------------------------------------------------
// y = H x of a captured system: elastic ELL rows (plain stores, one thread per
// scalar row), then contact blocks and friction terms (atomics)
__global__ void k_lp_spmv_ell(int nv, int K, const int* col, const float* val, const float* x, float* y)
{
    const int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= 3 * nv) return;
    const int i = w / 3, r = w - 3 * i;
    float acc = 0;
    for (int k = 0; k < K; ++k) {
        const size_t e = (size_t)k * nv + i;
        const int j = col[e];
        const float* B = val + 9 * e + 3 * r;
        acc += B[0] * x[3 * j] + B[1] * x[3 * j + 1] + B[2] * x[3 * j + 2];
    }
    y[w] = acc;
}

__global__ void k_lp_spmv_con(int ncon, const int* ckind, const int4* cverts, const float* chess, const float* x,
                              float* y)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncon) return;
    const int n = con_nv(ckind[c]), m = 3 * n;
    const int4 v = cverts[c];
    const int id[4] = {v.x, v.y, v.z, v.w};
    float xs[12], ys[12];
    for (int k = 0; k < 12; ++k) {
        xs[k] = (k < m) ? x[3 * id[k / 3] + k % 3] : 0.f;
        ys[k] = 0.f;
    }
    size_t h = 0;
    for (int p = 0; p < m; ++p) {
        ys[p] += chess[h * ncon + c] * xs[p];
        ++h;
        for (int q = p + 1; q < m; ++q, ++h) {
            const float hv = chess[h * ncon + c];
            ys[p] += hv * xs[q];
            ys[q] += hv * xs[p];
        }
    }
    for (int k = 0; k < m; ++k)
        if (ys[k] != 0.f) atomicAdd(y + 3 * id[k / 3] + k % 3, ys[k]);
}

__global__ void k_lp_spmv_fric(int nfric, const int* fkind, const int4* fverts, const float* fw, const float* fT,
                               const float* fM, const uint8_t* proj, const float* x, float* y)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nfric || fkind[c] >= kc_EEM) return;
    const int n = con_nv(fkind[c]);
    const int4 v = fverts[c];
    const int id[4] = {v.x, v.y, v.z, v.w};
    float s0 = 0, s1 = 0, s2 = 0;
    for (int q = 0; q < n; ++q) {
        if (proj[id[q]]) continue;
        const float w = fw[4 * c + q];
        s0 += w * x[3 * id[q]];
        s1 += w * x[3 * id[q] + 1];
        s2 += w * x[3 * id[q] + 2];
    }
    const float* T = fT + 6 * (size_t)c;
    const float t0 = T[0] * s0 + T[1] * s1 + T[2] * s2, t1 = T[3] * s0 + T[4] * s1 + T[5] * s2;
    const float u0 = fM[3 * c] * t0 + fM[3 * c + 1] * t1, u1 = fM[3 * c + 1] * t0 + fM[3 * c + 2] * t1;
    const float o0 = T[0] * u0 + T[3] * u1, o1 = T[1] * u0 + T[4] * u1, o2 = T[2] * u0 + T[5] * u1;
    for (int q = 0; q < n; ++q) {
        if (proj[id[q]]) continue;
        const float w = fw[4 * c + q];
        atomicAdd(y + 3 * id[q], w * o0);
        atomicAdd(y + 3 * id[q] + 1, w * o1);
        atomicAdd(y + 3 * id[q] + 2, w * o2);
    }
}

// red[0..2] += (z.r, z.Hz, r.p)
__global__ void k_lp_dots(int n, const float* z, const float* r, const float* hz, const float* p, double* red)
{
    __shared__ double sh[3][32];
    double a = 0, b = 0, c = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        a += (double)z[i] * r[i];
        b += (double)z[i] * hz[i];
        c += (double)r[i] * p[i];
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, o);
        b += __shfl_down_sync(0xffffffffu, b, o);
        c += __shfl_down_sync(0xffffffffu, c, o);
    }
    if (lane == 0) {
        sh[0][wid] = a;
        sh[1][wid] = b;
        sh[2][wid] = c;
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        double t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += sh[threadIdx.x][w];
        atomicAdd(red + threadIdx.x, t);
    }
}

// dz = f (-r + t Hz); dP = dz r^T; dCm = (dP + dP^T) Cm E; dout = d/do of Cm's entries
__global__ void k_lp_out_bwd(int nv, const float* o, const float* E, const float* r, const float* hz, float f, float t,
                             float* dout)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    float dz[3], rr[3], oo[kLpOut];
    for (int q = 0; q < 3; ++q) {
        rr[q] = r[3 * i + q];
        dz[q] = f * (-rr[q] + t * hz[3 * i + q]);
    }
    for (int k = 0; k < kLpOut; ++k) oo[k] = o[(size_t)kLpOut * i + k];
    const float* Ei = E + 9 * (size_t)i;
    float P[9], C[9];
    lp_block(oo, Ei, P, C);
    float S[9], CE[9], dC[9];
    for (int x = 0; x < 3; ++x)
        for (int y = 0; y < 3; ++y) S[3 * x + y] = dz[x] * rr[y] + dz[y] * rr[x];
    for (int x = 0; x < 3; ++x)
        for (int y = 0; y < 3; ++y) CE[3 * x + y] = C[3 * x] * Ei[y] + C[3 * x + 1] * Ei[3 + y] + C[3 * x + 2] * Ei[6 + y];
    for (int x = 0; x < 3; ++x)
        for (int y = 0; y < 3; ++y) dC[3 * x + y] = S[3 * x] * CE[y] + S[3 * x + 1] * CE[3 + y] + S[3 * x + 2] * CE[6 + y];
    float* d = dout + (size_t)kLpOut * i;
    for (int q = 0; q < 3; ++q)
        d[q] = (oo[q] > -kLpDiagClamp && oo[q] < kLpDiagClamp) ? dC[4 * q] * 0.5f * C[4 * q] : 0.f;
    d[3] = fabsf(oo[3]) < kLpOffClamp ? dC[3] : 0.f;
    d[4] = fabsf(oo[4]) < kLpOffClamp ? dC[6] : 0.f;
    d[5] = fabsf(oo[5]) < kLpOffClamp ? dC[7] : 0.f;
}

// din_i (+)= W^T dout_i, W (Ho x Hi)
template <int Ho, int Hi>
__global__ void k_lp_dense_T(int nv, const float* W, const float* dout, float* din, int accumulate)
{
    __shared__ float sw[Ho * Hi];
    for (int k = threadIdx.x; k < Ho * Hi; k += blockDim.x) sw[k] = W[k];
    __syncthreads();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    float d[Ho];
#pragma unroll
    for (int r = 0; r < Ho; ++r) d[r] = dout[(size_t)Ho * i + r];
#pragma unroll 1
    for (int q = 0; q < Hi; ++q) {
        float t = accumulate ? din[(size_t)Hi * i + q] : 0.f;
#pragma unroll
        for (int r = 0; r < Ho; ++r) t += sw[r * Hi + q] * d[r];
        din[(size_t)Hi * i + q] = t;
    }
}

__global__ void k_lp_relu_bwd(long long n, const float* dh, const float* u, float* du)
{
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) du[k] = u[k] > 0.f ? dh[k] : 0.f;
}

// transpose of k_lp_gather: dprev_j += (a_ki / s_i) dg_i
__global__ void k_lp_gather_T(int nv, int K, int H, const int* col, const float* a, const float* s, const float* dg,
                              float* dprev)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)nv * H) return;
    const int i = (int)(t / H), q = (int)(t - (long long)i * H);
    const float si = s[i];
    if (!(si > 0)) return;
    const float d = dg[t];
    if (d == 0.f) return;
    for (int k = 0; k < K; ++k) {
        const size_t e = (size_t)k * nv + i;
        const float w = a[e];
        if (w != 0.f) atomicAdd(dprev + (size_t)H * col[e] + q, (w / si) * d);
    }
}

// transpose of the contact gather
__global__ void k_lp_con_T(int ncon, int H, const int* ckind, const int4* cverts, const int* ncnt, const float* dc,
                           float* dprev)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)ncon * H) return;
    const int c = (int)(t / H), q = (int)(t - (long long)c * H);
    const int n = con_nv(ckind[c]);
    const int4 v = cverts[c];
    const int id[4] = {v.x, v.y, v.z, v.w};
    float s = 0;
    for (int k = 0; k < n; ++k) s += dc[(size_t)H * id[k] + q] / fmaxf(1.f, (float)ncnt[id[k]]);
    s /= (float)n;
    for (int k = 0; k < n; ++k) atomicAdd(dprev + (size_t)H * id[k] + q, s);
}

// dW += sum_i du_i in_i^T, db += sum_i du_i: tiles of 64 vertices in shared memory
template <int Ho, int Hi>
__global__ void __launch_bounds__(256) k_lp_wgrad(int nv, const float* du, const float* in, float* dW, float* db)
{
    constexpr int TV = 64, NE = (Ho * Hi + 255) / 256;
    __shared__ float sd[TV][Ho], si[TV][Hi];
    float acc[NE];
#pragma unroll
    for (int k = 0; k < NE; ++k) acc[k] = 0;
    float bacc = 0;
    for (int v0 = blockIdx.x * TV; v0 < nv; v0 += gridDim.x * TV) {
        __syncthreads();
        for (int k = threadIdx.x; k < TV * Ho; k += blockDim.x) {
            const int v = v0 + k / Ho;
            sd[k / Ho][k % Ho] = v < nv ? du[(size_t)Ho * v + k % Ho] : 0.f;
        }
        for (int k = threadIdx.x; k < TV * Hi; k += blockDim.x) {
            const int v = v0 + k / Hi;
            si[k / Hi][k % Hi] = v < nv ? in[(size_t)Hi * v + k % Hi] : 0.f;
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < NE; ++k) {
            const int e = threadIdx.x + 256 * k;
            if (e < Ho * Hi) {
                const int r = e / Hi, q = e % Hi;
                float t = 0;
                for (int v = 0; v < TV; ++v) t += sd[v][r] * si[v][q];
                acc[k] += t;
            }
        }
        if (db && threadIdx.x < Ho)
            for (int v = 0; v < TV; ++v) bacc += sd[v][threadIdx.x];
    }
#pragma unroll
    for (int k = 0; k < NE; ++k) {
        const int e = threadIdx.x + 256 * k;
        if (e < Ho * Hi && acc[k] != 0.f) atomicAdd(dW + e, acc[k]);
    }
    if (db && threadIdx.x < Ho && bacc != 0.f) atomicAdd(db + threadIdx.x, bacc);
}

__global__ void k_lp_adam(int n, float* p, const float* g, float* m, float* v, float lr, float b1, float b2, float eps,
                          float c1, float c2)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const float gk = g[k];
    const float mk = b1 * m[k] + (1.f - b1) * gk;
    const float vk = b2 * v[k] + (1.f - b2) * gk * gk;
    m[k] = mk;
    v[k] = vk;
    p[k] -= lr * (mk * c1) / (sqrtf(vk * c2) + eps);
}


// ---------------------------------------------------------------------------
// inference: message-passing layers on the BF16 tensor cores (FP32 accumulate)
// ---------------------------------------------------------------------------
// Wcat_l (H x 3H, bf16, row-major) = [A_l | B_l | C_l] for every layer
__global__ void k_lp_wcat_bf16(int H, int L, const float* params, int off0, int stride, __nv_bfloat16* out)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= L * 3 * H * H) return;
    const int l = k / (3 * H * H), e = k - l * 3 * H * H;
    const int r = e / (3 * H), q = e - r * 3 * H;
    const int part = q / H, qq = q - part * H;
    out[k] = __float2bfloat16(params[off0 + l * stride + part * H * H + r * H + qq]);
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi)
{
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t*>(&v);
}

// One warp per 16 vertices: u = [h | g | c] Wcat^T + b with mma.m16n8k16 (bf16 in,
// f32 accumulate); h_out = relu(u) + h.  c = acc / max(1, #contacts).
template <int H>
__global__ void __launch_bounds__(128) k_lp_layer_bf16(int nv, const float* h, const float* g, const float* acc,
                                                       const int* ncnt, const __nv_bfloat16* Wcat, const float* bias,
                                                       float* hout)
{
    constexpr int K3 = 3 * H, KT = K3 / 16, NT = H / 8;
    __shared__ __align__(16) __nv_bfloat16 sw[H * K3];
    __shared__ float sb[H];
    for (int k = threadIdx.x; k < H * K3; k += blockDim.x) sw[k] = Wcat[k];
    for (int k = threadIdx.x; k < H; k += blockDim.x) sb[k] = bias[k];
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int gq = lane >> 2, tq = lane & 3;
    const int v0 = (blockIdx.x * (blockDim.x >> 5) + warp) * 16;
    if (v0 >= nv) return;
    const int ra = v0 + gq, rb = v0 + gq + 8;
    const float ia = ra < nv ? 1.f / fmaxf(1.f, (float)ncnt[ra]) : 0.f;
    const float ib = rb < nv ? 1.f / fmaxf(1.f, (float)ncnt[rb]) : 0.f;
    // input element (row, column q of [h | g | c])
    auto in = [&](int row, float inv, int q) -> float {
        if (row >= nv) return 0.f;
        if (q < H) return h[(size_t)H * row + q];
        if (q < 2 * H) return g[(size_t)H * row + q - H];
        return acc[(size_t)H * row + q - 2 * H] * inv;
    };
    float d[NT][4];
#pragma unroll
    for (int n = 0; n < NT; ++n) d[n][0] = d[n][1] = d[n][2] = d[n][3] = 0.f;
#pragma unroll
    for (int kt = 0; kt < KT; ++kt) {
        const int c0 = 16 * kt + 2 * tq, c1 = c0 + 8;
        const uint32_t a0 = pack_bf16(in(ra, ia, c0), in(ra, ia, c0 + 1));
        const uint32_t a1 = pack_bf16(in(rb, ib, c0), in(rb, ib, c0 + 1));
        const uint32_t a2 = pack_bf16(in(ra, ia, c1), in(ra, ia, c1 + 1));
        const uint32_t a3 = pack_bf16(in(rb, ib, c1), in(rb, ib, c1 + 1));
#pragma unroll
        for (int n = 0; n < NT; ++n) {
            const __nv_bfloat16* wr = sw + (size_t)(8 * n + gq) * K3;
            const uint32_t b0 = *reinterpret_cast<const uint32_t*>(wr + c0);
            const uint32_t b1 = *reinterpret_cast<const uint32_t*>(wr + c1);
            asm volatile(
                "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                "{%0,%1,%2,%3};\n"
                : "+f"(d[n][0]), "+f"(d[n][1]), "+f"(d[n][2]), "+f"(d[n][3])
                : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
        }
    }
#pragma unroll
    for (int n = 0; n < NT; ++n) {
        const int col = 8 * n + 2 * tq;
        if (ra < nv) {
            hout[(size_t)H * ra + col] = fmaxf(d[n][0] + sb[col], 0.f) + h[(size_t)H * ra + col];
            hout[(size_t)H * ra + col + 1] = fmaxf(d[n][1] + sb[col + 1], 0.f) + h[(size_t)H * ra + col + 1];
        }
        if (rb < nv) {
            hout[(size_t)H * rb + col] = fmaxf(d[n][2] + sb[col], 0.f) + h[(size_t)H * rb + col];
            hout[(size_t)H * rb + col + 1] = fmaxf(d[n][3] + sb[col + 1], 0.f) + h[(size_t)H * rb + col + 1];
        }
    }
}

// ---------------------------------------------------------------------------
// k-step preconditioned steepest descent loss (loss kind 2)
// ---------------------------------------------------------------------------
// y_i = P_i x_i (3x3 blocks)
__global__ void k_lp_pmul(int nv, const float* P, const float* x, float* y)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    const float* B = P + 9 * (size_t)i;
    const float x0 = x[3 * i], x1 = x[3 * i + 1], x2 = x[3 * i + 2];
    y[3 * i] = B[0] * x0 + B[1] * x1 + B[2] * x2;
    y[3 * i + 1] = B[3] * x0 + B[4] * x1 + B[5] * x2;
    y[3 * i + 2] = B[6] * x0 + B[7] * x1 + B[8] * x2;
}
// y += a x ; with y_acc_p: y += a P x (blocks)
__global__ void k_lp_axpy(int n, float a, const float* x, float* y)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) y[k] += a * x[k];
}
__global__ void k_lp_pmul_acc(int nv, const float* P, const float* x, float* y)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    const float* B = P + 9 * (size_t)i;
    const float x0 = x[3 * i], x1 = x[3 * i + 1], x2 = x[3 * i + 2];
    y[3 * i] += B[0] * x0 + B[1] * x1 + B[2] * x2;
    y[3 * i + 1] += B[3] * x0 + B[4] * x1 + B[5] * x2;
    y[3 * i + 2] += B[6] * x0 + B[7] * x1 + B[8] * x2;
}
// out = a x + b y
__global__ void k_lp_lin2(int n, float a, const float* x, float b, const float* y, float* out)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) out[k] = a * x[k] + b * y[k];
}
// red += x . y
__global__ void k_lp_dot(int n, const float* x, const float* y, double* red)
{
    __shared__ double sh[32];
    double a = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) a += (double)x[i] * y[i];
    for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = a;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += sh[w];
        atomicAdd(red, t);
    }
}
// G_i += zb_i r_i^T
__global__ void k_lp_outer_acc(int nv, const float* zb, const float* r, float* G)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) G[9 * (size_t)i + 3 * a + b] += zb[3 * i + a] * r[3 * i + b];
}
// dout from the adjoint G of the preconditioner blocks: dCm = (G + G^T) Cm E
__global__ void k_lp_out_bwd_G(int nv, const float* o, const float* E, const float* Gb, float scale, float* dout)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    float oo[kLpOut];
    for (int k = 0; k < kLpOut; ++k) oo[k] = o[(size_t)kLpOut * i + k];
    const float* Ei = E + 9 * (size_t)i;
    const float* G = Gb + 9 * (size_t)i;
    float P[9], C[9], S[9], CE[9], dC[9];
    lp_block(oo, Ei, P, C);
    for (int x = 0; x < 3; ++x)
        for (int y = 0; y < 3; ++y) S[3 * x + y] = scale * (G[3 * x + y] + G[3 * y + x]);
    for (int x = 0; x < 3; ++x)
        for (int y = 0; y < 3; ++y) CE[3 * x + y] = C[3 * x] * Ei[y] + C[3 * x + 1] * Ei[3 + y] + C[3 * x + 2] * Ei[6 + y];
    for (int x = 0; x < 3; ++x)
        for (int y = 0; y < 3; ++y) dC[3 * x + y] = S[3 * x] * CE[y] + S[3 * x + 1] * CE[3 + y] + S[3 * x + 2] * CE[6 + y];
    float* d = dout + (size_t)kLpOut * i;
    for (int q = 0; q < 3; ++q)
        d[q] = (oo[q] > -kLpDiagClamp && oo[q] < kLpDiagClamp) ? dC[4 * q] * 0.5f * C[4 * q] : 0.f;
    d[3] = fabsf(oo[3]) < kLpOffClamp ? dC[3] : 0.f;
    d[4] = fabsf(oo[4]) < kLpOffClamp ? dC[6] : 0.f;
    d[5] = fabsf(oo[5]) < kLpOffClamp ? dC[7] : 0.f;
}

template <typename T>
__global__ void k_lp_cvt(long long n, const T* a, float* b)
{
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) b[k] = (float)a[k];
}

// chess (stride cap) -> dst (stride ncon), converted to float
template <typename T>
__global__ void k_lp_repack(int ncon, size_t cap, const T* src, float* dst)
{
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= 78LL * ncon) return;
    const int h = (int)(k / ncon), c = (int)(k - (long long)h * ncon);
    dst[k] = (float)src[(size_t)h * cap + c];
}

}  // namespace

void LpTriple::release()
{
    col.release();
    diag.release();
    val.release();
    cdiag.release();
    proj.release();
    ckind.release();
    cverts.release();
    chess.release();
    fkind.release();
    fverts.release();
    fw.release();
    fT.release();
    fM.release();
    r.release();
    p.release();
}

LpModel::~LpModel()
{
    if (stream) cudaStreamSynchronize(stream);
    for (LpTriple* t : data) {
        t->release();
        delete t;
    }
    for (DBuf<float>* b : {&params, &grad, &adam_m, &adam_v, &X, &E, &Dn, &a, &s, &u0, &o, &z, &hz, &dz, &dout, &dh, &dh2,
                           &du, &dg, &dc, &acc, &h, &g, &c, &u, &Pm, &Gb, &psd})
        b->release();
    wbf16.release();
    ncnt.release();
    red.release();
    if (stream) cudaStreamDestroy(stream);
}

namespace {

int ensure_work(LpModel* m, int nv, int K, int ncon)
{
    if (nv <= m->cap_nv && K <= m->cap_k && ncon <= m->cap_con) return CIPC_OK;
    const int H = m->H, L = m->L;
    const size_t n = (size_t)std::max(nv, m->cap_nv);
    const size_t k = (size_t)std::max(K, m->cap_k);
    cudaError_t e = cudaSuccess;
    auto A = [&](DBuf<float>& b, size_t cnt) {
        if (e == cudaSuccess) e = b.alloc(cnt);
    };
    A(m->X, n * kLpFeatures);
    A(m->E, 9 * n);
    A(m->Dn, n);
    A(m->a, k * n);
    A(m->s, n);
    A(m->u0, n * H);
    A(m->o, n * kLpOut);
    A(m->z, 3 * n);
    A(m->hz, 3 * n);
    A(m->dout, n * kLpOut);
    A(m->dh, n * H);
    A(m->dh2, n * H);
    A(m->du, n * H);
    A(m->dg, n * H);
    A(m->dc, n * H);
    A(m->acc, n * H);
    A(m->h, (size_t)(L + 1) * n * H);
    A(m->g, (size_t)L * n * H);
    A(m->c, (size_t)L * n * H);
    A(m->u, (size_t)L * n * H);
    A(m->Pm, 9 * n);
    A(m->Gb, 9 * n);
    A(m->psd, (size_t)(3 * kLpPsdSteps + 6) * 3 * n);
    if (e == cudaSuccess) e = m->ncnt.alloc(n);
    if (e == cudaSuccess && m->red.n < 8) e = m->red.alloc(8);
    if (e != cudaSuccess) return set_error(CIPC_ERR_CUDA, "learned preconditioner work buffers");
    m->cap_nv = (int)n;
    m->cap_k = (int)k;
    m->cap_con = std::max(ncon, m->cap_con);
    return CIPC_OK;
}

template <typename VT, typename CT>
void features(LpModel* m, const LpSys<VT, CT>& S, cudaStream_t st)
{
    cudaMemsetAsync(m->ncnt.p, 0, sizeof(int) * S.nv, st);
    cudaMemsetAsync(m->red.p, 0, 2 * sizeof(double), st);
    if (S.ncon > 0) k_lp_count<<<nb(S.ncon, 256), 256, 0, st>>>(S.ncon, S.ckind, S.cverts, m->ncnt.p);
    k_lp_diag<VT, CT><<<nb(S.nv, 256), 256, 0, st>>>(S, m->E.p, m->Dn.p, m->red.p);
    k_lp_feat<VT, CT><<<nb(S.nv, 256), 256, 0, st>>>(S, m->Dn.p, m->ncnt.p, m->red.p, m->X.p, m->a.p, m->s.p);
}

// FP32 forward; z = P r when r is given, pinv = P when pinv is given
template <int H, typename PT>
void forward(LpModel* m, int nv, int K, const int* col, int ncon, const int* ckind, const int4* cverts, const float* r,
             PT* pinv, cudaStream_t st)
{
    const LpOff of = offsets(H, m->L);
    const float* P = m->params.p;
    const size_t nh = (size_t)nv * H;
    k_lp_in<H><<<nb(nv, 128), 128, (H * kLpFeatures + H) * sizeof(float), st>>>(nv, m->X.p, P + of.W0, P + of.b0,
                                                                                m->u0.p, m->h.p);
    for (int l = 0; l < m->L; ++l) {
        const float* hl = m->h.p + (size_t)l * nh;
        float* gl = m->g.p + (size_t)l * nh;
        k_lp_gather<<<nb((long long)nh, 256), 256, 0, st>>>(nv, K, H, col, m->a.p, m->s.p, hl, gl);
        cudaMemsetAsync(m->acc.p, 0, sizeof(float) * nh, st);
        if (ncon > 0) k_lp_con_acc<<<nb((long long)ncon * H, 256), 256, 0, st>>>(ncon, H, ckind, cverts, hl, m->acc.p);
        k_lp_layer<H><<<nb(nv, 128), 128, (3 * H * H + H) * sizeof(float), st>>>(
            nv, hl, gl, m->acc.p, m->ncnt.p, P + of.A[l], m->c.p + (size_t)l * nh, m->u.p + (size_t)l * nh,
            m->h.p + (size_t)(l + 1) * nh);
    }
    k_lp_out<H, PT><<<nb(nv, 128), 128, 0, st>>>(nv, m->h.p + (size_t)m->L * nh, P + of.Wo, P + of.bo, m->E.p, r,
                                                 m->o.p, r ? m->z.p : nullptr, pinv);
}

// inference forward with the message-passing layers on the BF16 tensor cores
template <int H, typename PT>
int forward_bf16(LpModel* m, int nv, int K, const int* col, int ncon, const int* ckind, const int4* cverts, PT* pinv,
                 cudaStream_t st)
{
    const LpOff of = offsets(H, m->L);
    const float* P = m->params.p;
    const size_t nh = (size_t)nv * H;
    if (!m->wbf16_valid) {
        const int n = m->L * 3 * H * H;
        const int stride = m->L > 1 ? of.A[1] - of.A[0] : 3 * H * H + H;
        k_lp_wcat_bf16<<<nb(n, 256), 256, 0, st>>>(H, m->L, P, of.A[0], stride,
                                                    reinterpret_cast<__nv_bfloat16*>(m->wbf16.p));
        m->wbf16_valid = true;
    }
    k_lp_in<H><<<nb(nv, 128), 128, (H * kLpFeatures + H) * sizeof(float), st>>>(nv, m->X.p, P + of.W0, P + of.b0,
                                                                                m->u0.p, m->h.p);
    for (int l = 0; l < m->L; ++l) {
        const float* hl = m->h.p + (size_t)l * nh;
        float* gl = m->g.p + (size_t)l * nh;
        k_lp_gather<<<nb((long long)nh, 256), 256, 0, st>>>(nv, K, H, col, m->a.p, m->s.p, hl, gl);
        cudaMemsetAsync(m->acc.p, 0, sizeof(float) * nh, st);
        if (ncon > 0) k_lp_con_acc<<<nb((long long)ncon * H, 256), 256, 0, st>>>(ncon, H, ckind, cverts, hl, m->acc.p);
        k_lp_layer_bf16<H><<<nb(nv, 64), 128, 0, st>>>(
            nv, hl, gl, m->acc.p, m->ncnt.p, reinterpret_cast<const __nv_bfloat16*>(m->wbf16.p) + (size_t)l * 3 * H * H,
            P + of.b[l], m->h.p + (size_t)(l + 1) * nh);
    }
    k_lp_out<H, PT><<<nb(nv, 128), 128, 0, st>>>(nv, m->h.p + (size_t)m->L * nh, P + of.Wo, P + of.bo, m->E.p,
                                                 nullptr, m->o.p, nullptr, pinv);
    return CIPC_OK;
}

// network backward from dout (d loss / d o, nv x 6): parameter gradients into m->grad
template <int H>
void net_backward(LpModel* m, LpTriple* T, cudaStream_t st)
{
    const int nv = T->nv, K = T->K, L = m->L;
    const LpOff of = offsets(H, L);
    float* G = m->grad.p;
    const float* P = m->params.p;
    const size_t nh = (size_t)nv * H;
    const int wg = std::min(nb(nv, 64), 2 * num_sms());
    k_lp_wgrad<kLpOut, H><<<wg, 256, 0, st>>>(nv, m->dout.p, m->h.p + (size_t)L * nh, G + of.Wo, G + of.bo);
    k_lp_dense_T<kLpOut, H><<<nb(nv, 128), 128, 0, st>>>(nv, P + of.Wo, m->dout.p, m->dh.p, 0);
    for (int l = L - 1; l >= 0; --l) {
        const float* hl = m->h.p + (size_t)l * nh;
        k_lp_relu_bwd<<<nb((long long)nh, 256), 256, 0, st>>>((long long)nh, m->dh.p, m->u.p + (size_t)l * nh, m->du.p);
        k_lp_wgrad<H, H><<<wg, 256, 0, st>>>(nv, m->du.p, hl, G + of.A[l], G + of.b[l]);
        k_lp_wgrad<H, H><<<wg, 256, 0, st>>>(nv, m->du.p, m->g.p + (size_t)l * nh, G + of.B[l], nullptr);
        k_lp_wgrad<H, H><<<wg, 256, 0, st>>>(nv, m->du.p, m->c.p + (size_t)l * nh, G + of.C[l], nullptr);
        cudaMemcpyAsync(m->dh2.p, m->dh.p, sizeof(float) * nh, cudaMemcpyDeviceToDevice, st);
        k_lp_dense_T<H, H><<<nb(nv, 128), 128, 0, st>>>(nv, P + of.A[l], m->du.p, m->dh2.p, 1);
        k_lp_dense_T<H, H><<<nb(nv, 128), 128, 0, st>>>(nv, P + of.B[l], m->du.p, m->dg.p, 0);
        k_lp_dense_T<H, H><<<nb(nv, 128), 128, 0, st>>>(nv, P + of.C[l], m->du.p, m->dc.p, 0);
        k_lp_gather_T<<<nb((long long)nh, 256), 256, 0, st>>>(nv, K, H, T->col.p, m->a.p, m->s.p, m->dg.p, m->dh2.p);
        if (T->ncon > 0)
            k_lp_con_T<<<nb((long long)T->ncon * H, 256), 256, 0, st>>>(T->ncon, H, T->ckind.p, T->cverts.p, m->ncnt.p,
                                                                        m->dc.p, m->dh2.p);
        std::swap(m->dh.p, m->dh2.p);
    }
    k_lp_relu_bwd<<<nb((long long)nh, 256), 256, 0, st>>>((long long)nh, m->dh.p, m->u0.p, m->du.p);
    k_lp_wgrad<H, kLpFeatures><<<wg, 256, 0, st>>>(nv, m->du.p, m->X.p, G + of.W0, G + of.b0);
}

// Loss kind 2: relative H-norm error after kLpPsdSteps steps of preconditioned
// steepest descent from x = 0 on H x = r (x_k = sum alpha_j z_j, z_j = P r_j,
// alpha_j = (z_j.r_j)/(z_j.H z_j), r_{j+1} = r_j - alpha_j H z_j), and its
// gradient by reverse accumulation through the steps.  Unlike the one-step
// losses it depends on the whole spectrum of P H, as PCG's convergence does.
template <int H>
int loss_grad_psd(LpModel* m, LpTriple* T, float grad_scale, double* loss)
{
    cudaStream_t st = m->stream;
    int rc = ensure_work(m, T->nv, T->K, T->ncon);
    if (rc) return rc;
    const int nv = T->nv, K = T->K, n3 = 3 * nv, ks = kLpPsdSteps;
    LpSys<float, float> S{nv, K, T->col.p, T->diag.p, T->val.p, T->cdiag.p, T->proj.p, T->ncon, T->ckind.p, T->cverts.p};
    features(m, S, st);
    forward<H, float>(m, nv, K, T->col.p, T->ncon, T->ckind.p, T->cverts.p, nullptr, m->Pm.p, st);
    const size_t vb = 3 * (size_t)m->cap_nv;
    float* R = m->psd.p;
    float* Z = R + (ks + 1) * vb;
    float* Wv = Z + ks * vb;
    float* xb = Wv + ks * vb;
    float* rb = xb + vb;
    float* zb = rb + vb;
    float* wb = zb + vb;
    float* tmp = wb + vb;
    auto Rj = [&](int j) { return R + j * vb; };
    auto Zj = [&](int j) { return Z + j * vb; };
    auto Wj = [&](int j) { return Wv + j * vb; };
    auto spmv = [&](const float* x, float* y) {
        k_lp_spmv_ell<<<nb(n3, 256), 256, 0, st>>>(nv, K, T->col.p, T->val.p, x, y);
        if (T->ncon > 0)
            k_lp_spmv_con<<<nb(T->ncon, 128), 128, 0, st>>>(T->ncon, T->ckind.p, T->cverts.p, T->chess.p, x, y);
        if (T->nfric > 0)
            k_lp_spmv_fric<<<nb(T->nfric, 128), 128, 0, st>>>(T->nfric, T->fkind.p, T->fverts.p, T->fw.p, T->fT.p,
                                                             T->fM.p, T->proj.p, x, y);
    };
    cudaError_t e = cudaSuccess;
    auto dot = [&](const float* x, const float* y) -> double {
        double h = 0;
        cudaMemsetAsync(m->red.p + 5, 0, sizeof(double), st);
        k_lp_dot<<<std::min(nb(n3, 256), 512), 256, 0, st>>>(n3, x, y, m->red.p + 5);
        cudaMemcpyAsync(&h, m->red.p + 5, sizeof(double), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        return h;
    };
    const int t1 = nb(n3, 256), tv = nb(nv, 128);
    cudaMemcpyAsync(Rj(0), T->r.p, sizeof(float) * n3, cudaMemcpyDeviceToDevice, st);
    const double c = dot(T->r.p, T->p.p);
    double a[kLpPsdSteps], b[kLpPsdSteps], al[kLpPsdSteps];
    int kk = 0;
    for (int j = 0; j < ks; ++j) {
        k_lp_pmul<<<tv, 128, 0, st>>>(nv, m->Pm.p, Rj(j), Zj(j));
        spmv(Zj(j), Wj(j));
        a[j] = dot(Zj(j), Rj(j));
        b[j] = dot(Zj(j), Wj(j));
        if (!(b[j] > 0) || !(a[j] == a[j])) break;
        al[j] = a[j] / b[j];
        k_lp_lin2<<<t1, 256, 0, st>>>(n3, 1.f, Rj(j), (float)-al[j], Wj(j), Rj(j + 1));
        kk = j + 1;
    }
    if (e != cudaSuccess) return set_cuda_error(e, "learned preconditioner loss");
    if (!(c > 0) || kk == 0) {
        *loss = 0;
        return CIPC_OK;
    }
    // x = sum alpha_j z_j ; H x = r_0 - r_k ; |p - x|_H^2 = c - 2 x.r_0 + x.Hx
    cudaMemsetAsync(tmp, 0, sizeof(float) * n3, st);
    for (int j = 0; j < kk; ++j) k_lp_axpy<<<t1, 256, 0, st>>>(n3, (float)al[j], Zj(j), tmp);
    const double xr = dot(tmp, Rj(0));
    const double xHx = xr - dot(tmp, Rj(kk));
    if (e != cudaSuccess) return set_cuda_error(e, "learned preconditioner loss");
    *loss = (c - 2 * xr + xHx) / c;
    if (grad_scale == 0.f) return CIPC_OK;
    // reverse accumulation; xb = d loss / d x = -(2/c) r_k
    k_lp_lin2<<<t1, 256, 0, st>>>(n3, (float)(-2.0 / c), Rj(kk), 0.f, Rj(kk), xb);
    cudaMemsetAsync(rb, 0, sizeof(float) * n3, st);
    cudaMemsetAsync(m->Gb.p, 0, sizeof(float) * 9 * nv, st);
    for (int j = kk - 1; j >= 0; --j) {
        const double ab = -dot(rb, Wj(j)) + dot(xb, Zj(j));
        const double abar = ab / b[j], bbar = -ab * a[j] / (b[j] * b[j]);
        k_lp_lin2<<<t1, 256, 0, st>>>(n3, (float)al[j], xb, (float)abar, Rj(j), zb);
        k_lp_axpy<<<t1, 256, 0, st>>>(n3, (float)bbar, Wj(j), zb);
        k_lp_lin2<<<t1, 256, 0, st>>>(n3, (float)-al[j], rb, (float)bbar, Zj(j), wb);
        k_lp_axpy<<<t1, 256, 0, st>>>(n3, (float)abar, Zj(j), rb);
        spmv(wb, tmp);
        k_lp_axpy<<<t1, 256, 0, st>>>(n3, 1.f, tmp, zb);
        k_lp_outer_acc<<<tv, 128, 0, st>>>(nv, zb, Rj(j), m->Gb.p);
        k_lp_pmul_acc<<<tv, 128, 0, st>>>(nv, m->Pm.p, zb, rb);
    }
    if (e != cudaSuccess) return set_cuda_error(e, "learned preconditioner gradient");
    k_lp_out_bwd_G<<<tv, 128, 0, st>>>(nv, m->o.p, m->E.p, m->Gb.p, grad_scale, m->dout.p);
    net_backward<H>(m, T, st);
    return CIPC_OK;
}

// loss of triple T (and, if grad_scale != 0, its gradient times grad_scale added to m->grad)
template <int H>
int loss_grad(LpModel* m, LpTriple* T, float grad_scale, double* loss)
{
    cudaStream_t st = m->stream;
    int rc = ensure_work(m, T->nv, T->K, T->ncon);
    if (rc) return rc;
    const int nv = T->nv, K = T->K;
    LpSys<float, float> S{nv, K, T->col.p, T->diag.p, T->val.p, T->cdiag.p, T->proj.p, T->ncon, T->ckind.p, T->cverts.p};
    features(m, S, st);
    forward<H, float>(m, nv, K, T->col.p, T->ncon, T->ckind.p, T->cverts.p, T->r.p, (float*)nullptr, st);
    k_lp_spmv_ell<<<nb(3 * nv, 256), 256, 0, st>>>(nv, K, T->col.p, T->val.p, m->z.p, m->hz.p);
    if (T->ncon > 0)
        k_lp_spmv_con<<<nb(T->ncon, 128), 128, 0, st>>>(T->ncon, T->ckind.p, T->cverts.p, T->chess.p, m->z.p, m->hz.p);
    if (T->nfric > 0)
        k_lp_spmv_fric<<<nb(T->nfric, 128), 128, 0, st>>>(T->nfric, T->fkind.p, T->fverts.p, T->fw.p, T->fT.p, T->fM.p,
                                                         T->proj.p, m->z.p, m->hz.p);
    cudaMemsetAsync(m->red.p + 2, 0, 3 * sizeof(double), st);
    k_lp_dots<<<std::min(nb(3 * nv, 256), 1024), 256, 0, st>>>(3 * nv, m->z.p, T->r.p, m->hz.p, T->p.p, m->red.p + 2);
    double d[3];
    cudaMemcpyAsync(d, m->red.p + 2, sizeof(d), cudaMemcpyDeviceToHost, st);
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return set_cuda_error(e, "learned preconditioner loss");
    const double a = d[0], b = d[1], c = d[2];
    if (!(b > 0) || !(c > 0)) {
        *loss = 0;
        return CIPC_OK;
    }
    const bool unit = m->loss_kind == 1;
    *loss = unit ? (b - 2 * a + c) / c : 1 - a * a / (b * c);
    if (grad_scale == 0.f) return CIPC_OK;
    const double f = unit ? 2 / c : 2 * a / (b * c), t = unit ? 1.0 : a / b;
    k_lp_out_bwd<<<nb(nv, 128), 128, 0, st>>>(nv, m->o.p, m->E.p, T->r.p, m->hz.p, (float)f * grad_scale, (float)t,
                                              m->dout.p);
    net_backward<H>(m, T, st);
    return CIPC_OK;
}

int loss_grad_any(LpModel* m, LpTriple* T, float grad_scale, double* loss)
{
    if (m->loss_kind == 2)
        return m->H == 32 ? loss_grad_psd<32>(m, T, grad_scale, loss) : loss_grad_psd<16>(m, T, grad_scale, loss);
    if (m->H == 32) return loss_grad<32>(m, T, grad_scale, loss);
    return loss_grad<16>(m, T, grad_scale, loss);
}


template <typename T>
cudaError_t copy_cvt(DBuf<float>& dst, const T* src, size_t n, cudaStream_t st)
{
    cudaError_t e = dst.alloc(std::max<size_t>(n, 1));
    if (e == cudaSuccess && n) k_lp_cvt<T><<<nb((long long)n, 256), 256, 0, st>>>((long long)n, src, dst.p);
    return e;
}

template <typename T>
cudaError_t copy_raw(DBuf<T>& dst, const T* src, size_t n, cudaStream_t st)
{
    cudaError_t e = dst.alloc(std::max<size_t>(n, 1));
    if (e == cudaSuccess && n) e = cudaMemcpyAsync(dst.p, src, n * sizeof(T), cudaMemcpyDeviceToDevice, st);
    return e;
}

}  // namespace

int lp_create(int hidden, int layers, uint64_t seed, LpModel** out)
{
    if (hidden != 16 && hidden != 32) return set_error(CIPC_ERR_INVALID_ARG, "learned preconditioner: hidden must be 16 or 32");
    if (layers < 1 || layers > 8) return set_error(CIPC_ERR_INVALID_ARG, "learned preconditioner: layers must be 1..8");
    int rc = ensure_device();
    if (rc) return rc;
    LpModel* m = new LpModel();
    m->H = hidden;
    m->L = layers;
    m->seed = seed;
    m->nparams = num_params(hidden, layers);
    const int n = m->nparams;
    cudaError_t e = cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking);
    for (DBuf<float>* b : {&m->params, &m->grad, &m->adam_m, &m->adam_v})
        if (e == cudaSuccess) e = b->alloc(n);
    if (e == cudaSuccess) e = m->wbf16.alloc(n);
    // seeded initialisation: Gaussian weights scaled by 1/sqrt(fan-in) (0.5 of that
    // inside the residual layers), zero biases, zero output layer (= block Jacobi)
    std::vector<float> p(n, 0.f);
    std::mt19937_64 rng(seed);
    std::normal_distribution<float> nd(0.f, 1.f);
    const LpOff of = offsets(hidden, layers);
    for (int k = 0; k < hidden * kLpFeatures; ++k) p[of.W0 + k] = nd(rng) / std::sqrt((float)kLpFeatures);
    for (int l = 0; l < layers; ++l)
        for (int k = 0; k < hidden * hidden; ++k) {
            p[of.A[l] + k] = 0.5f * nd(rng) / std::sqrt((float)hidden);
            p[of.B[l] + k] = 0.5f * nd(rng) / std::sqrt((float)hidden);
            p[of.C[l] + k] = 0.5f * nd(rng) / std::sqrt((float)hidden);
        }
    if (e == cudaSuccess) e = cudaMemcpy(m->params.p, p.data(), sizeof(float) * n, cudaMemcpyHostToDevice);
    for (DBuf<float>* b : {&m->grad, &m->adam_m, &m->adam_v})
        if (e == cudaSuccess) e = cudaMemset(b->p, 0, sizeof(float) * n);
    if (e != cudaSuccess) {
        delete m;
        return set_cuda_error(e, "learned preconditioner creation");
    }
    *out = m;
    return CIPC_OK;
}

int lp_precond(Sim* s, LpModel* m)
{
    cudaStream_t st = s->stream;
    const int ncon = s->prm.withCollision ? s->ncon : 0;
    int rc = ensure_work(m, s->nv, s->ell_k, ncon);
    if (rc) return rc;
    const bool f32 = s->prm.precision == 1;
    if (f32) {
        LpSys<float, double> S{s->nv, s->ell_k, s->col.p, s->diag.p, (const float*)s->hval.p, s->pdiag.p, s->proj.p,
                               ncon, s->ckind.p, s->cverts.p};
        features(m, S, st);
    } else {
        LpSys<double, double> S{s->nv, s->ell_k, s->col.p, s->diag.p, (const double*)s->hval.p, s->pdiag.p, s->proj.p,
                                ncon, s->ckind.p, s->cverts.p};
        features(m, S, st);
    }
    const int nv = s->nv, K = s->ell_k;
    if (m->H == 32) {
        if (f32) forward_bf16<32, float>(m, nv, K, s->col.p, ncon, s->ckind.p, s->cverts.p, (float*)s->pinv.p, st);
        else forward_bf16<32, double>(m, nv, K, s->col.p, ncon, s->ckind.p, s->cverts.p, (double*)s->pinv.p, st);
    } else {
        if (f32) forward_bf16<16, float>(m, nv, K, s->col.p, ncon, s->ckind.p, s->cverts.p, (float*)s->pinv.p, st);
        else forward_bf16<16, double>(m, nv, K, s->col.p, ncon, s->ckind.p, s->cverts.p, (double*)s->pinv.p, st);
    }
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? CIPC_OK : set_cuda_error(e, "learned preconditioner");
}

int lp_capture(Sim* s, LpModel* m, const double* rhs, const double* sol)
{
    if ((int)m->data.size() >= m->capture_max) return CIPC_OK;
    cudaStream_t st = s->stream;
    LpTriple* T = new LpTriple();
    const int nv = s->nv, K = s->ell_k;
    const int ncon = s->prm.withCollision ? s->ncon : 0;
    const int nfric = (s->prm.withCollision && s->prm.mu > 0) ? s->nfric : 0;
    T->nv = nv;
    T->K = K;
    T->ncon = ncon;
    T->nfric = nfric;
    const bool f32 = s->prm.precision == 1;
    const size_t nb_ = (size_t)K * nv;
    cudaError_t e = copy_raw(T->col, s->col.p, nb_, st);
    if (e == cudaSuccess) e = copy_raw(T->diag, s->diag.p, (size_t)nv, st);
    if (e == cudaSuccess)
        e = f32 ? copy_cvt(T->val, (const float*)s->hval.p, 9 * nb_, st) : copy_cvt(T->val, (const double*)s->hval.p, 9 * nb_, st);
    if (e == cudaSuccess) e = copy_cvt(T->cdiag, s->pdiag.p, 9 * (size_t)nv, st);
    if (e == cudaSuccess) e = copy_raw(T->proj, s->proj.p, (size_t)nv, st);
    if (e == cudaSuccess) e = copy_raw(T->ckind, s->ckind.p, (size_t)ncon, st);
    if (e == cudaSuccess) e = copy_raw(T->cverts, s->cverts.p, (size_t)ncon, st);
    if (e == cudaSuccess) e = T->chess.alloc(std::max<size_t>(78 * (size_t)ncon, 1));
    if (e == cudaSuccess && ncon) {
        if (f32) k_lp_repack<float><<<nb(78LL * ncon, 256), 256, 0, st>>>(ncon, (size_t)s->cap_con, (const float*)s->chess.p, T->chess.p);
        else k_lp_repack<double><<<nb(78LL * ncon, 256), 256, 0, st>>>(ncon, (size_t)s->cap_con, (const double*)s->chess.p, T->chess.p);
    }
    if (e == cudaSuccess) e = copy_raw(T->fkind, s->fkind.p, (size_t)nfric, st);
    if (e == cudaSuccess) e = copy_raw(T->fverts, s->fverts.p, (size_t)nfric, st);
    if (e == cudaSuccess) e = copy_cvt(T->fw, s->fw.p, 4 * (size_t)nfric, st);
    if (e == cudaSuccess) e = copy_cvt(T->fT, s->fT.p, 6 * (size_t)nfric, st);
    if (e == cudaSuccess) e = copy_cvt(T->fM, (const double*)s->fhess.p, 3 * (size_t)nfric, st);
    if (e == cudaSuccess) e = copy_cvt(T->r, rhs, 3 * (size_t)nv, st);
    if (e == cudaSuccess) e = copy_cvt(T->p, sol, 3 * (size_t)nv, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        T->release();
        delete T;
        return set_cuda_error(e, "capturing a Newton system");
    }
    m->data.push_back(T);
    return CIPC_OK;
}

int lp_train(LpModel* m, int epochs, int batch, double lr, uint64_t seed, double* before, double* after)
{
    const int nt = (int)m->data.size();
    if (nt == 0) return set_error(CIPC_ERR_INVALID_ARG, "learned preconditioner: no captured systems to train on");
    if (epochs < 0 || batch < 1 || !(lr > 0)) return set_error(CIPC_ERR_INVALID_ARG, "learned preconditioner: bad training arguments");
    auto mean_loss = [&](double* out) {
        double sum = 0;
        for (LpTriple* T : m->data) {
            double l = 0;
            int rc = loss_grad_any(m, T, 0.f, &l);
            if (rc) return rc;
            sum += l;
        }
        *out = sum / nt;
        return (int)CIPC_OK;
    };
    int rc;
    if (before && (rc = mean_loss(before))) return rc;
    std::vector<int> order(nt);
    std::iota(order.begin(), order.end(), 0);
    std::mt19937_64 rng(seed);
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    for (int ep = 0; ep < epochs; ++ep) {
        std::shuffle(order.begin(), order.end(), rng);
        for (int b0 = 0; b0 < nt; b0 += batch) {
            const int bn = std::min(batch, nt - b0);
            cudaMemsetAsync(m->grad.p, 0, sizeof(float) * m->nparams, m->stream);
            for (int k = 0; k < bn; ++k) {
                double l = 0;
                if ((rc = loss_grad_any(m, m->data[order[b0 + k]], 1.f / bn, &l))) return rc;
            }
            ++m->adam_t;
            const float c1 = 1.f / (1.f - std::pow(b1, (float)m->adam_t)), c2 = 1.f / (1.f - std::pow(b2, (float)m->adam_t));
            k_lp_adam<<<nb(m->nparams, 256), 256, 0, m->stream>>>(m->nparams, m->params.p, m->grad.p, m->adam_m.p,
                                                                  m->adam_v.p, (float)lr, b1, b2, eps, c1, c2);
        }
    }
    m->wbf16_valid = false;
    if (after && (rc = mean_loss(after))) return rc;
    cudaError_t e = cudaStreamSynchronize(m->stream);
    return e == cudaSuccess ? CIPC_OK : set_cuda_error(e, "learned preconditioner training");
}

}  // namespace cipc

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
using namespace cipc;

struct cipc_precond {
    LpModel* m;
};

namespace cipc {
LpModel* lp_model(::cipc_precond* p) { return p ? p->m : nullptr; }
}  // namespace cipc

static int check_pc(const cipc_precond* p)
{
    return (p && p->m) ? CIPC_OK : set_error(CIPC_ERR_INVALID_ARG, "null preconditioner handle");
}

extern "C" int cipc_precond_create(int hidden, int layers, uint64_t seed, cipc_precond** out)
{
    if (!out) return set_error(CIPC_ERR_INVALID_ARG, "cipc_precond_create: null output");
    LpModel* m = nullptr;
    int rc = lp_create(hidden, layers, seed, &m);
    if (rc) return rc;
    *out = new cipc_precond{m};
    return CIPC_OK;
}

extern "C" int cipc_precond_destroy(cipc_precond* p)
{
    if (!p) return CIPC_OK;
    delete p->m;
    delete p;
    return CIPC_OK;
}

extern "C" int cipc_precond_num_params(const cipc_precond* p) { return check_pc(p) ? -1 : p->m->nparams; }

extern "C" int cipc_precond_get_params(const cipc_precond* p, float* out)
{
    if (int rc = check_pc(p)) return rc;
    if (!out) return set_error(CIPC_ERR_INVALID_ARG, "cipc_precond_get_params: null buffer");
    cudaError_t e = cudaMemcpy(out, p->m->params.p, sizeof(float) * p->m->nparams, cudaMemcpyDeviceToHost);
    return e == cudaSuccess ? CIPC_OK : set_cuda_error(e, "cipc_precond_get_params");
}

extern "C" int cipc_precond_set_params(cipc_precond* p, const float* in)
{
    if (int rc = check_pc(p)) return rc;
    if (!in) return set_error(CIPC_ERR_INVALID_ARG, "cipc_precond_set_params: null buffer");
    cudaError_t e = cudaMemcpy(p->m->params.p, in, sizeof(float) * p->m->nparams, cudaMemcpyHostToDevice);
    p->m->wbf16_valid = false;
    return e == cudaSuccess ? CIPC_OK : set_cuda_error(e, "cipc_precond_set_params");
}

extern "C" int cipc_precond_set_loss(cipc_precond* p, int kind)
{
    if (int rc = check_pc(p)) return rc;
    if (kind < 0 || kind > 2) return set_error(CIPC_ERR_INVALID_ARG, "cipc_precond_set_loss: kind must be 0, 1 or 2");
    p->m->loss_kind = kind;
    return CIPC_OK;
}

extern "C" int cipc_precond_num_systems(const cipc_precond* p) { return check_pc(p) ? -1 : (int)p->m->data.size(); }

extern "C" int cipc_precond_clear_systems(cipc_precond* p)
{
    if (int rc = check_pc(p)) return rc;
    for (LpTriple* t : p->m->data) {
        t->release();
        delete t;
    }
    p->m->data.clear();
    return CIPC_OK;
}

extern "C" int cipc_precond_train(cipc_precond* p, int epochs, int batch, double lr, uint64_t seed,
                                  double* loss_before, double* loss_after)
{
    if (int rc = check_pc(p)) return rc;
    return lp_train(p->m, epochs, batch, lr, seed, loss_before, loss_after);
}

extern "C" int cipc_precond_loss_grad(cipc_precond* p, int system, double* loss, float* grad)
{
    if (int rc = check_pc(p)) return rc;
    LpModel* m = p->m;
    if (system < 0 || system >= (int)m->data.size() || !loss)
        return set_error(CIPC_ERR_INVALID_ARG, "cipc_precond_loss_grad: bad system index or null output");
    cudaMemsetAsync(m->grad.p, 0, sizeof(float) * m->nparams, m->stream);
    int rc = loss_grad_any(m, m->data[system], grad ? 1.f : 0.f, loss);
    if (rc) return rc;
    if (grad) {
        cudaError_t e = cudaMemcpyAsync(grad, m->grad.p, sizeof(float) * m->nparams, cudaMemcpyDeviceToHost, m->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
        if (e != cudaSuccess) return set_cuda_error(e, "cipc_precond_loss_grad");
    }
    return CIPC_OK;
}

extern "C" int cipc_precond_infer(cipc_precond* p, int system, int bf16, float* out6, float* blocks9)
{
    if (int rc = check_pc(p)) return rc;
    LpModel* m = p->m;
    if (system < 0 || system >= (int)m->data.size())
        return set_error(CIPC_ERR_INVALID_ARG, "cipc_precond_infer: bad system index");
    LpTriple* T = m->data[system];
    int rc = ensure_work(m, T->nv, T->K, T->ncon);
    if (rc) return rc;
    cudaStream_t st = m->stream;
    LpSys<float, float> S{T->nv, T->K, T->col.p, T->diag.p, T->val.p, T->cdiag.p, T->proj.p, T->ncon, T->ckind.p,
                          T->cverts.p};
    features(m, S, st);
    const int nv = T->nv, K = T->K;
    if (bf16) {
        if (m->H == 32) forward_bf16<32, float>(m, nv, K, T->col.p, T->ncon, T->ckind.p, T->cverts.p, m->Pm.p, st);
        else forward_bf16<16, float>(m, nv, K, T->col.p, T->ncon, T->ckind.p, T->cverts.p, m->Pm.p, st);
    } else {
        if (m->H == 32) forward<32, float>(m, nv, K, T->col.p, T->ncon, T->ckind.p, T->cverts.p, nullptr, m->Pm.p, st);
        else forward<16, float>(m, nv, K, T->col.p, T->ncon, T->ckind.p, T->cverts.p, nullptr, m->Pm.p, st);
    }
    cudaError_t e = cudaSuccess;
    if (out6) e = cudaMemcpyAsync(out6, m->o.p, sizeof(float) * kLpOut * nv, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && blocks9) e = cudaMemcpyAsync(blocks9, m->Pm.p, sizeof(float) * 9 * nv, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    return e == cudaSuccess ? CIPC_OK : set_cuda_error(e, "cipc_precond_infer");
}

extern "C" int cipc_precond_system_sizes(const cipc_precond* p, int system, int32_t* sizes4)
{
    if (int rc = check_pc(p)) return rc;
    if (system < 0 || system >= (int)p->m->data.size() || !sizes4)
        return set_error(CIPC_ERR_INVALID_ARG, "cipc_precond_system_sizes: bad system index or null output");
    const LpTriple* T = p->m->data[system];
    sizes4[0] = T->nv;
    sizes4[1] = T->K;
    sizes4[2] = T->ncon;
    sizes4[3] = T->nfric;
    return CIPC_OK;
}

extern "C" int cipc_precond_system_export(const cipc_precond* p, int system, int32_t* col, float* val, float* cdiag,
                                          uint8_t* proj, int32_t* ckind, int32_t* cverts, float* chess, float* rhs,
                                          float* sol)
{
    if (int rc = check_pc(p)) return rc;
    if (system < 0 || system >= (int)p->m->data.size())
        return set_error(CIPC_ERR_INVALID_ARG, "cipc_precond_system_export: bad system index");
    const LpTriple* T = p->m->data[system];
    const size_t nbk = (size_t)T->K * T->nv, nc = (size_t)T->ncon;
    cudaError_t e = cudaSuccess;
    auto get = [&](void* dst, const void* src, size_t bytes) {
        if (e == cudaSuccess && dst && bytes) e = cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToHost);
    };
    get(col, T->col.p, sizeof(int) * nbk);
    get(val, T->val.p, sizeof(float) * 9 * nbk);
    get(cdiag, T->cdiag.p, sizeof(float) * 9 * T->nv);
    get(proj, T->proj.p, T->nv);
    get(ckind, T->ckind.p, sizeof(int) * nc);
    get(cverts, T->cverts.p, sizeof(int4) * nc);
    get(rhs, T->r.p, sizeof(float) * 3 * T->nv);
    get(sol, T->p.p, sizeof(float) * 3 * T->nv);
    if (e == cudaSuccess && chess && nc) {
        // stored entry-major (h * ncon + c); exported constraint-major (78 c + h)
        std::vector<float> tmp(78 * nc);
        get(tmp.data(), T->chess.p, sizeof(float) * tmp.size());
        for (size_t c = 0; c < nc; ++c)
            for (int h = 0; h < 78; ++h) chess[78 * c + h] = tmp[(size_t)h * nc + c];
    }
    return e == cudaSuccess ? CIPC_OK : set_cuda_error(e, "cipc_precond_system_export");
}
