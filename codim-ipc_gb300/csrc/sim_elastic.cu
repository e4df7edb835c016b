// Elastic and inertia terms of the incremental potential (INC_POTENTIAL.h:15-395):
// membrane and hinge bending per element, 1/2 (x - xtilde)^T M (x - xtilde), and
// the Dirichlet projection of the Hessian (CSR_MATRIX.h:130-141).
//
// Energies: FP64, one partial per block written to a reduction buffer and summed
// in a fixed order (deterministic).  Gradients: FP64 atomics into g.  Hessians:
// each element's PSD-projected blocks are added (atomically, in HT = float or
// double) into the block-sparse matrix at slots precomputed from the mesh;
// blocks that touch a Dirichlet vertex are skipped and Dirichlet diagonal blocks
// are set to the identity.
#include <cuda_runtime.h>

#include <vector>

#include "../../include/cipc.h"
#include "cipc_util.h"
#include "elements.cuh"
#include "rod.cuh"
#include "strain_limit.cuh"
#include "tet_nh.cuh"
#include "sim.h"
#include "sim_kernels.h"

namespace cipc {

__device__ __forceinline__ double block_sum(double v, double* sh)
{
    const int t = threadIdx.x;
    sh[t] = v;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (t < s) sh[t] += sh[t + s];
        __syncthreads();
    }
    const double r = sh[0];
    __syncthreads();
    return r;
}

__global__ void k_xtilde(int nv, const double* x, const double* v, const double* b, const double* m, double h,
                         double* xt)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    const double mi = m[i];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const double a = mi > 0 ? b[3 * i + d] / mi : 0.0;
        xt[3 * i + d] = x[3 * i + d] + h * v[3 * i + d] + h * h * a;
    }
}

// inertia energy partials, gradient m (x - xt) (g is overwritten: first term)
__global__ void __launch_bounds__(256) k_inertia(int nv, const double* x, const double* xt, const double* m, double* g,
                                                  double* red)
{
    __shared__ double sh[256];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double e = 0;
    if (i < nv) {
        const double mi = m[i];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const double dd = x[3 * i + d] - xt[3 * i + d];
            e += mi * dd * dd;
            if (g) g[3 * i + d] = mi * dd;
        }
    }
    const double s = block_sum(0.5 * e, sh);
    if (red && threadIdx.x == 0) red[blockIdx.x] = s;
}

template <typename HT>
__device__ __forceinline__ void scatter_blocks(HT* hval, const int* slots, const uint8_t* dbc, const int* vid, int nvb,
                                               const HT* H, int m)
{
    for (int a = 0; a < nvb; ++a) {
        if (dbc[vid[a]]) continue;
        for (int b = 0; b < nvb; ++b) {
            if (dbc[vid[b]]) continue;
            HT* dst = hval + 9 * (size_t)slots[nvb * a + b];
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int j = 0; j < 3; ++j) atomicAdd(dst + 3 * i + j, H[(3 * a + i) * m + 3 * b + j]);
        }
    }
}

template <typename HT>
__global__ void __launch_bounds__(128) k_membrane(ElasticArgs a, HT* hval)
{
    __shared__ double sh[128];
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    double e = 0;
    if (t < a.nt && !a.skip_membrane) {
        const int vid[3] = {a.tri[3 * t], a.tri[3 * t + 1], a.tri[3 * t + 2]};
        if (!(a.dbc[vid[0]] && a.dbc[vid[1]] && a.dbc[vid[2]])) {
            const d3 x[3] = {ld(a.x, vid[0]), ld(a.x, vid[1]), ld(a.x, vid[2])};
            MembraneOut o;
            double S[3], c;
            const double k = a.h * a.h * a.vol[t];
            membrane_eg(x, a.P + 3 * t, k, a.lam, a.mu, a.nh_model, o, S, c);
            e = o.E;
            if (a.g)
                for (int v = 0; v < 3; ++v)
#pragma unroll
                    for (int d = 0; d < 3; ++d) atomicAdd(a.g + 3 * vid[v] + d, o.g[3 * v + d]);
            if (hval) {
                HT H[9][9];
                membrane_hess<HT>(x, a.P + 3 * t, k, a.lam, a.mu, a.nh_model, S, c, H);
                project_translation_free<HT, 3>(H);
                scatter_blocks<HT>(hval, a.tri_slot + 9 * t, a.proj, vid, 3, &H[0][0], 9);
            }
        }
    }
    const double s = block_sum(e, sh);
    if (a.red && threadIdx.x == 0) a.red[blockIdx.x] = s;
}

template <typename HT>
__global__ void __launch_bounds__(128) k_bending(ElasticArgs a, HT* hval)
{
    __shared__ double sh[128];
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    double e = 0;
    if (t < a.nh && a.kbend != 0) {
        const int vid[4] = {a.hinge[4 * t], a.hinge[4 * t + 1], a.hinge[4 * t + 2], a.hinge[4 * t + 3]};
        if (!(a.dbc[vid[0]] && a.dbc[vid[1]] && a.dbc[vid[2]] && a.dbc[vid[3]])) {
            const d3 x[4] = {ld(a.x, vid[0]), ld(a.x, vid[1]), ld(a.x, vid[2]), ld(a.x, vid[3])};
            const double thetabar = a.hinfo[3 * t], c = a.h * a.h * a.kbend * a.hinfo[3 * t + 1] / a.hinfo[3 * t + 2];
            const double th = dihedral_angle(x);
            const double dth = th - thetabar;
            e = c * dth * dth;
            if (a.g || hval) {  // (line-search energy passes need neither)
                double gt[12];
                dihedral_grad(x, gt);
                if (a.g)
                    for (int v = 0; v < 4; ++v)
#pragma unroll
                        for (int d = 0; d < 3; ++d) atomicAdd(a.g + 3 * vid[v] + d, 2 * c * dth * gt[3 * v + d]);
                if (hval) {
                    // Hessian of theta in HT (FP32 in mixed precision) from FP64 edge
                    // vectors, formed in place in H
                    HT H[12][12];
                    const d3 ev[5] = {x[2] - x[1], x[0] - x[1], x[3] - x[1], x[0] - x[2], x[3] - x[2]};
                    HT E[5][3];
#pragma unroll
                    for (int k = 0; k < 5; ++k) {
                        E[k][0] = (HT)ev[k].x;
                        E[k][1] = (HT)ev[k].y;
                        E[k][2] = (HT)ev[k].z;
                    }
                    dihedral_hess_t<HT>(E, H);
                    const HT c2 = (HT)(2 * c), fd = (HT)dth;
                    HT gf[12];
#pragma unroll
                    for (int i = 0; i < 12; ++i) gf[i] = (HT)gt[i];
#pragma unroll
                    for (int i = 0; i < 12; ++i)
#pragma unroll
                        for (int j = 0; j < 12; ++j) H[i][j] = c2 * (gf[i] * gf[j] + fd * H[i][j]);
                    project_translation_free<HT, 4>(H);
                    scatter_blocks<HT>(hval, a.hinge_slot + 16 * t, a.proj, vid, 4, &H[0][0], 12);
                }
            }
        }
    }
    const double s = block_sum(e, sh);
    if (a.red && threadIdx.x == 0) a.red[blockIdx.x] = s;
}

// rod stretching (ROD_STRETCHING.h:9-107): K = h^2 pi t^2 / 4 E, E = K L / 2 (l/L - 1)^2
template <typename HT>
__global__ void __launch_bounds__(128) k_rod_spring(ElasticArgs a, HT* hval)
{
    __shared__ double sh[128];
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    double e = 0;
    if (t < a.nrs) {
        const int vid[2] = {a.rseg[2 * t], a.rseg[2 * t + 1]};
        if (!(a.dbc[vid[0]] && a.dbc[vid[1]])) {
            const d3 x0 = ld(a.x, vid[0]), x1 = ld(a.x, vid[1]);
            const double* ri = a.rinfo + 3 * t;
            const double K = a.h * a.h * M_PI * ri[2] * ri[2] / 4 * ri[0];
            double g[6];
            e = rod_spring_eg(x0, x1, ri[1], K, a.g ? g : nullptr);
            if (a.g)
                for (int v = 0; v < 2; ++v)
#pragma unroll
                    for (int d = 0; d < 3; ++d) atomicAdd(a.g + 3 * vid[v] + d, g[3 * v + d]);
            if (hval) {
                HT H[6][6];
                rod_spring_hess<HT>(x0, x1, ri[1], K, H);
                scatter_blocks<HT>(hval, a.rseg_slot + 4 * t, a.proj, vid, 2, &H[0][0], 6);
            }
        }
    }
    const double s = block_sum(e, sh);
    if (a.red && threadIdx.x == 0) a.red[blockIdx.x] = s;
}

// rod bending (ROD_BENDING.h:9-120): Kb = h^2 E bendMult t^4 pi / 64, E = Kb |kb|^2 / lsum
template <typename HT>
__global__ void __launch_bounds__(128) k_rod_bend(ElasticArgs a, HT* hval)
{
    __shared__ double sh[128];
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    double e = 0;
    if (t < a.nrh) {
        const int vid[3] = {a.rhinge[3 * t], a.rhinge[3 * t + 1], a.rhinge[3 * t + 2]};
        if (!(a.dbc[vid[0]] && a.dbc[vid[1]] && a.dbc[vid[2]])) {
            const d3 x0 = ld(a.x, vid[0]), x1 = ld(a.x, vid[1]), x2 = ld(a.x, vid[2]);
            const double* ri = a.rhinfo + 3 * t;
            const double t2 = ri[2] * ri[2];
            const double Kb = a.h * a.h * ri[0] * t2 * t2 * M_PI / 64;
            double g[9];
            e = rod_bend_eg(x0, x1, x2, ri[1], Kb, a.g ? g : nullptr);
            if (a.g)
                for (int v = 0; v < 3; ++v)
#pragma unroll
                    for (int d = 0; d < 3; ++d) atomicAdd(a.g + 3 * vid[v] + d, g[3 * v + d]);
            if (hval) {
                HT H[9][9];
                rod_bend_hess<HT>(x0, x1, x2, ri[1], Kb, H);
                scatter_blocks<HT>(hval, a.rhinge_slot + 9 * t, a.proj, vid, 3, &H[0][0], 9);
            }
        }
    }
    const double s = block_sum(e, sh);
    if (a.red && threadIdx.x == 0) a.red[blockIdx.x] = s;
}

// isotropic strain limiting (INEXT.h:120-466): barrier on the singular values of
// each triangle's deformation; an infeasible triangle sets *a.flag
template <typename HT>
__global__ void __launch_bounds__(128) k_strain_limit(ElasticArgs a, HT* hval)
{
    __shared__ double sh[128];
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    double e = 0;
    if (t < a.nt) {
        const int vid[3] = {a.tri[3 * t], a.tri[3 * t + 1], a.tri[3 * t + 2]};
        if (!(a.dbc[vid[0]] && a.dbc[vid[1]] && a.dbc[vid[2]])) {
            const d3 x[3] = {ld(a.x, vid[0]), ld(a.x, vid[1]), ld(a.x, vid[2])};
            const double kh = a.h * a.h * a.vol[t];
            double g[9];
            if (!sl_eg(x, a.P + 3 * t, a.sl, kh, e, a.g ? g : nullptr) && a.flag) *a.flag = 1.0;
            if (a.g)
                for (int v = 0; v < 3; ++v)
#pragma unroll
                    for (int d = 0; d < 3; ++d)
                        if (g[3 * v + d] != 0) atomicAdd(a.g + 3 * vid[v] + d, g[3 * v + d]);
            if (hval) {
                HT H[9][9];
                if (sl_hess<HT>(x, a.P + 3 * t, a.sl, kh, true, H))
                    scatter_blocks<HT>(hval, a.tri_slot + 9 * t, a.proj, vid, 3, &H[0][0], 9);
            }
        }
    }
    const double s = block_sum(e, sh);
    if (a.red && threadIdx.x == 0) a.red[blockIdx.x] = s;
}

// volumetric Neo-Hookean tetrahedra (INC_POTENTIAL.h:97-109, 228-229, 354-364);
// an inverted tetrahedron (J <= 0) sets *a.flag
template <typename HT>
__global__ void __launch_bounds__(128) k_tet_nh(ElasticArgs a, HT* hval)
{
    __shared__ double sh[128];
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    double e = 0;
    if (t < a.ntet) {
        const int vid[4] = {a.tet[4 * t], a.tet[4 * t + 1], a.tet[4 * t + 2], a.tet[4 * t + 3]};
        if (!(a.dbc[vid[0]] && a.dbc[vid[1]] && a.dbc[vid[2]] && a.dbc[vid[3]])) {
            const d3 x[4] = {ld(a.x, vid[0]), ld(a.x, vid[1]), ld(a.x, vid[2]), ld(a.x, vid[3])};
            const double w = a.h * a.h * a.tvol[t];
            double g[12];
            const bool ok = tet_nh_eg(x, a.tDinv + 9 * t, w, a.tlam, a.tmu, e, a.g ? g : nullptr);
            if (!ok && a.flag) *a.flag = 1.0;
            if (a.g && ok)
                for (int v = 0; v < 4; ++v)
#pragma unroll
                    for (int d = 0; d < 3; ++d) atomicAdd(a.g + 3 * vid[v] + d, g[3 * v + d]);
            if (hval && ok) {
                HT H[12][12];
                tet_nh_hess<HT>(x, a.tDinv + 9 * t, w, a.tlam, a.tmu, true, H);
                scatter_blocks<HT>(hval, a.tet_slot + 16 * t, a.proj, vid, 4, &H[0][0], 12);
            }
        }
    }
    const double s = block_sum(e, sh);
    if (a.red && threadIdx.x == 0) a.red[blockIdx.x] = s;
}

// kappa_s update test (IMPLICIT_EULER.h:606-628): a triangle whose largest
// stretch was within thr of the limit s0 after the previous Newton iteration and
// still is sets *flag; prev[] takes the current stretches (1 for triangles with
// all vertices Dirichlet, as in Compute_Inextensibility)
__global__ void k_strain_update(int nt, const int* tri, const uint8_t* dbc, const double* x, const double* P,
                                double s0, double thr, int have_prev, double* prev, unsigned long long* flag)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nt) return;
    const int v0 = tri[3 * t], v1 = tri[3 * t + 1], v2 = tri[3 * t + 2];
    double st = 1;
    if (!(dbc[v0] && dbc[v1] && dbc[v2])) {
        const d3 xs[3] = {ld(x, v0), ld(x, v1), ld(x, v2)};
        st = sl_max_strain(xs, P + 3 * t);
    }
    if (have_prev && s0 - prev[t] < thr && s0 - st < thr) *flag = 1ull;
    prev[t] = st;
}

// mass (+ Dirichlet penalty k m on penalized vertices) on free diagonal blocks,
// identity on projected diagonal blocks
template <typename HT>
__global__ void k_mass_diag(int nv, const double* m, const uint8_t* proj, const uint8_t* dbc, double stiff,
                            const int* diag, HT* hval)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    HT* d = hval + 9 * (size_t)diag[i];
    const HT v = proj[i] ? HT(1) : (HT)(m[i] * (dbc[i] ? 1.0 + stiff : 1.0));
    d[0] += v;
    d[4] += v;
    d[8] += v;
}

__global__ void k_zero_dbc(int nv, const uint8_t* proj, double* g)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nv && proj[i]) g[3 * i] = g[3 * i + 1] = g[3 * i + 2] = 0;
}

// Dirichlet penalty 1/2 k m |x - target|^2 (Shell/DIRICHLET.h:26-94)
__global__ void __launch_bounds__(256) k_dbc_penalty(int nd, const int* idx, const double* tgt, const double* m,
                                                      const double* x, double stiff, double* g, double* red)
{
    __shared__ double sh[256];
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    double e = 0;
    if (k < nd) {
        const int v = idx[k];
        double p = 0;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const double dd = tgt[3 * k + d] - x[3 * v + d];
            p += dd * dd;
            if (g) g[3 * v + d] += stiff * m[v] * (-dd);
        }
        e = p * m[v];
    }
    const double s = block_sum(e, sh);
    if (red && threadIdx.x == 0) red[blockIdx.x] = 0.5 * stiff * s;
}

__global__ void __launch_bounds__(256) k_dbc_dist2(int nd, const int* idx, const double* tgt, const double* x,
                                                    double* red)
{
    __shared__ double sh[256];
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    double p = 0;
    if (k < nd) {
        const int v = idx[k];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const double dd = tgt[3 * k + d] - x[3 * v + d];
            p += dd * dd;
        }
    }
    const double s = block_sum(p, sh);
    if (threadIdx.x == 0) red[blockIdx.x] = s;
}

// sum of n partials in a fixed order (single block)
__global__ void k_sum(const double* red, int n, double* out)
{
    __shared__ double sh[1024];
    double s = 0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) s += red[i];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = sh[0];
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
static inline int nblk(int n, int bs) { return n > 0 ? (n + bs - 1) / bs : 1; }

void launch_xtilde(Sim* s)
{
    k_xtilde<<<nblk(s->nv, 256), 256, 0, s->stream>>>(s->nv, s->x.p, s->v.p, s->b.p, s->mass.p, s->prm.h, s->xt.p);
}

ElasticArgs elastic_args(Sim* s, const double* x, double* g)
{
    ElasticArgs a;
    a.nt = s->nt;
    a.nh = s->nh;
    a.tri = s->tri.p;
    a.hinge = s->hinge.p;
    a.P = s->P.p;
    a.vol = s->vol.p;
    a.hinfo = s->hinfo.p;
    a.tri_slot = s->tri_slot.p;
    a.hinge_slot = s->hinge_slot.p;
    a.dbc = s->dbc.p;
    a.proj = s->proj.p;
    a.x = x;
    a.g = g;
    a.h = s->prm.h;
    a.lam = s->lam;
    a.mu = s->mu;
    a.kbend = s->kbend;
    a.nh_model = s->nh_model;
    a.red = nullptr;
    a.nrs = s->nrs;
    a.nrh = s->nrh;
    a.rseg = s->rseg.p;
    a.rhinge = s->rhinge.p;
    a.rseg_slot = s->rseg_slot.p;
    a.rhinge_slot = s->rhinge_slot.p;
    a.rinfo = s->rinfo.p;
    a.rhinfo = s->rhinfo.p;
    a.sl = s->sl;
    a.flag = nullptr;
    a.ntet = s->ntet;
    a.tet = s->tet.p;
    a.tet_slot = s->tet_slot.p;
    a.tDinv = s->tDinv.p;
    a.tvol = s->tvol.p;
    a.tlam = s->tlam;
    a.tmu = s->tmu;
    a.skip_membrane = 0;
    if (s->elastic_off) {
        a.skip_membrane = 1;
        a.nh = 0;
        a.nrs = 0;
        a.nrh = 0;
        a.ntet = 0;
    }
    return a;
}

// Energy partial layout: [inertia | membrane | bending | rod stretching | rod
// bending | strain limiting (when on) | tetrahedra]; returns the partial count.
// flag (device double, may be null) is set to 1 by a strain-infeasible triangle
// or an inverted tetrahedron.
int elastic_energy_partials(Sim* s, const double* x, double* red, double* flag)
{
    const int b0 = nblk(s->nv, 256), b1 = nblk(s->nt, 128), b2 = nblk(s->nh, 128);
    const int b3 = nblk(s->nrs, 128), b4 = nblk(s->nrh, 128);
    k_inertia<<<b0, 256, 0, s->stream>>>(s->nv, x, s->xt.p, s->mass.p, nullptr, red);
    ElasticArgs a = elastic_args(s, x, nullptr);
    a.red = red + b0;
    k_membrane<double><<<b1, 128, 0, s->stream>>>(a, nullptr);
    a.red = red + b0 + b1;
    k_bending<double><<<b2, 128, 0, s->stream>>>(a, nullptr);
    a.red = red + b0 + b1 + b2;
    k_rod_spring<double><<<b3, 128, 0, s->stream>>>(a, nullptr);
    a.red = red + b0 + b1 + b2 + b3;
    k_rod_bend<double><<<b4, 128, 0, s->stream>>>(a, nullptr);
    int n = b0 + b1 + b2 + b3 + b4;
    a.flag = flag;
    if (s->sl.k0 > 0) {
        a.red = red + n;
        k_strain_limit<double><<<b1, 128, 0, s->stream>>>(a, nullptr);
        n += b1;
    }
    if (s->ntet > 0) {
        a.red = red + n;
        k_tet_nh<double><<<nblk(s->ntet, 128), 128, 0, s->stream>>>(a, nullptr);
        n += nblk(s->ntet, 128);
    }
    return n;
}

int elastic_feasible(Sim* s, const double* x, bool* ok)
{
    *ok = true;
    if (!(s->sl.k0 > 0) && s->ntet == 0) return CIPC_OK;
    double* flag = s->red.p + s->red.n - 1;
    cudaMemsetAsync(flag, 0, sizeof(double), s->stream);
    ElasticArgs a = elastic_args(s, x, nullptr);
    a.flag = flag;
    if (s->sl.k0 > 0) k_strain_limit<double><<<nblk(s->nt, 128), 128, 0, s->stream>>>(a, nullptr);
    if (s->ntet > 0) k_tet_nh<double><<<nblk(s->ntet, 128), 128, 0, s->stream>>>(a, nullptr);
    double h = 0;
    cudaMemcpyAsync(&h, flag, sizeof(double), cudaMemcpyDeviceToHost, s->stream);
    cudaError_t e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) return set_cuda_error(e, "elastic feasibility");
    *ok = h == 0;
    return CIPC_OK;
}

int strain_kappa_update(Sim* s, const double* x, bool* raise)
{
    *raise = false;
    if (!(s->sl.k0 > 0) || s->nt == 0) return CIPC_OK;
    if (s->sl_prev.n < (size_t)s->nt && s->sl_prev.alloc(s->nt) != cudaSuccess)
        return set_error(CIPC_ERR_CUDA, "strain buffer");
    unsigned long long* flag = s->cnt.p + 40;
    cudaMemsetAsync(flag, 0, sizeof(unsigned long long), s->stream);
    k_strain_update<<<nblk(s->nt, 256), 256, 0, s->stream>>>(s->nt, s->tri.p, s->dbc.p, x, s->P.p, s->sl.s0,
                                                             1.0e-4 * (s->sl.s0 - s->sl.sh0), s->sl_have_prev ? 1 : 0,
                                                             s->sl_prev.p, flag);
    unsigned long long h = 0;
    cudaMemcpyAsync(&h, flag, sizeof(h), cudaMemcpyDeviceToHost, s->stream);
    cudaError_t e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) return set_cuda_error(e, "strain update");
    s->sl_have_prev = true;
    *raise = h != 0;
    return CIPC_OK;
}

void elastic_grad_hess(Sim* s, const double* x, double* g, bool want_hess)
{
    k_inertia<<<nblk(s->nv, 256), 256, 0, s->stream>>>(s->nv, x, s->xt.p, s->mass.p, g, nullptr);
    ElasticArgs a = elastic_args(s, x, g);
    const bool f32 = s->prm.precision == 1;
    if (want_hess) cudaMemsetAsync(s->hval.p, 0, 9 * (size_t)s->nnzb * (f32 ? 4 : 8), s->stream);
    if (f32) {
        float* hv = want_hess ? (float*)s->hval.p : nullptr;
        k_membrane<float><<<nblk(s->nt, 128), 128, 0, s->stream>>>(a, hv);
        k_bending<float><<<nblk(s->nh, 128), 128, 0, s->stream>>>(a, hv);
        if (s->nrs) k_rod_spring<float><<<nblk(s->nrs, 128), 128, 0, s->stream>>>(a, hv);
        if (s->nrh) k_rod_bend<float><<<nblk(s->nrh, 128), 128, 0, s->stream>>>(a, hv);
        if (s->sl.k0 > 0) k_strain_limit<float><<<nblk(s->nt, 128), 128, 0, s->stream>>>(a, hv);
        if (s->ntet > 0) k_tet_nh<float><<<nblk(s->ntet, 128), 128, 0, s->stream>>>(a, hv);
        if (want_hess)
            k_mass_diag<float><<<nblk(s->nv, 256), 256, 0, s->stream>>>(s->nv, s->mass.p, s->proj.p, s->dbc.p,
                                                                      s->dbc_stiff, s->diag.p, hv);
    } else {
        double* hv = want_hess ? (double*)s->hval.p : nullptr;
        k_membrane<double><<<nblk(s->nt, 128), 128, 0, s->stream>>>(a, hv);
        k_bending<double><<<nblk(s->nh, 128), 128, 0, s->stream>>>(a, hv);
        if (s->nrs) k_rod_spring<double><<<nblk(s->nrs, 128), 128, 0, s->stream>>>(a, hv);
        if (s->nrh) k_rod_bend<double><<<nblk(s->nrh, 128), 128, 0, s->stream>>>(a, hv);
        if (s->sl.k0 > 0) k_strain_limit<double><<<nblk(s->nt, 128), 128, 0, s->stream>>>(a, hv);
        if (s->ntet > 0) k_tet_nh<double><<<nblk(s->ntet, 128), 128, 0, s->stream>>>(a, hv);
        if (want_hess)
            k_mass_diag<double><<<nblk(s->nv, 256), 256, 0, s->stream>>>(s->nv, s->mass.p, s->proj.p, s->dbc.p,
                                                                       s->dbc_stiff, s->diag.p, hv);
    }
}

void zero_dbc(Sim* s, double* g) { k_zero_dbc<<<nblk(s->nv, 256), 256, 0, s->stream>>>(s->nv, s->proj.p, g); }

int dbc_penalty_partials(Sim* s, const double* x, double* red, double* g)
{
    const int nd = (int)s->dbc_idx_h.size();
    if (nd == 0 || s->dbc_stiff == 0) return 0;
    k_dbc_penalty<<<nblk(nd, 256), 256, 0, s->stream>>>(nd, s->dbc_idx.p, s->dbc_tgt.p, s->mass.p, x, s->dbc_stiff,
                                                        g, red);
    return red ? nblk(nd, 256) : 0;
}

double dbc_dist2(Sim* s, const double* x)
{
    const int nd = (int)s->dbc_idx_h.size();
    if (nd == 0) return 0;
    const int nb = nblk(nd, 256);
    k_dbc_dist2<<<nb, 256, 0, s->stream>>>(nd, s->dbc_idx.p, s->dbc_tgt.p, x, s->red.p);
    std::vector<double> h(nb);
    cudaMemcpyAsync(h.data(), s->red.p, sizeof(double) * nb, cudaMemcpyDeviceToHost, s->stream);
    cudaStreamSynchronize(s->stream);
    double t = 0;
    for (double v : h) t += v;
    return t;
}

void sum_partials(Sim* s, const double* red, int n, double* out)
{
    k_sum<<<1, 1024, 0, s->stream>>>(red, n, out);
}

}  // namespace cipc
