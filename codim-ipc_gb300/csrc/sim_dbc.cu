// Dirichlet motion on the device and the OBJ frame writer.
//
// Init_Dirichlet (Library/FEM/BOUNDARY_CONDITION.h:16-104): the vertices of an
// index range whose positions lie in a box given relative to the range's bounding
// box become Dirichlet vertices, their current positions the targets, and the
// group gets a motion (velocity v, rotation about rotCenter / rotAxis at angVelDeg
// degrees per second).  Step_Dirichlet (:106-157) advances every target by the
// rotation of angle angVelDeg * pi / 180 * h about the axis through rotCenter
// (the axis-angle matrix c I + (1 - c) a a^T + s [a]x, a as given), then by v h.
// Here the targets stay resident and one kernel advances them, so a driver that
// only moves its boundary this way sends nothing to the device between steps.
//
// Write_TriMesh_Obj (Library/Utils/MESHIO.h:182-213): "v %le %le %le" per vertex,
// "f i j k" (1-based) per triangle.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <vector>

#include "../../include/cipc.h"
#include "cipc_util.h"
#include "sim.h"
#include "sim_handle.h"

namespace cipc {

__global__ void k_step_dirichlet(int ngroups, const DbcMotion* g, double h, double* tgt)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    int k = 0;
    while (k < ngroups && !(i >= g[k].begin && i < g[k].end)) ++k;
    if (k == ngroups) return;
    const DbcMotion m = g[k];
    double* t = tgt + 3 * (size_t)i;
    if (m.ang_deg != 0) {
        const double th = m.ang_deg / 180 * M_PI * h;
        const double c = cos(th), s = sin(th), c1 = 1 - c;
        const double ax = m.axis[0], ay = m.axis[1], az = m.axis[2];
        const double R[3][3] = {{c + c1 * ax * ax, c1 * ax * ay - s * az, c1 * ax * az + s * ay},
                                {c1 * ay * ax + s * az, c + c1 * ay * ay, c1 * ay * az - s * ax},
                                {c1 * az * ax - s * ay, c1 * az * ay + s * ax, c + c1 * az * az}};
        const double x[3] = {t[0] - m.center[0], t[1] - m.center[1], t[2] - m.center[2]};
        for (int r = 0; r < 3; ++r) t[r] = R[r][0] * x[0] + R[r][1] * x[1] + R[r][2] * x[2] + m.center[r];
    }
    for (int r = 0; r < 3; ++r) t[r] += m.v[r] * h;
}

}  // namespace cipc

using namespace cipc;

extern "C" int cipc_sim_init_dirichlet(cipc_sim* h, const double* rel_min, const double* rel_max, const double* v,
                                       const double* rot_center, const double* rot_axis, double ang_vel_deg,
                                       int v_begin, int v_end, int* added)
{
    if (int rc = check_sim(h)) return rc;
    Sim* s = h->s;
    if (!rel_min || !rel_max || !v || !rot_center || !rot_axis)
        return set_error(CIPC_ERR_INVALID_ARG, "cipc_sim_init_dirichlet: null argument");
    v_begin = std::max(0, v_begin);
    if (v_end < 0 || v_end > s->nv) v_end = s->nv;
    if (v_begin >= v_end) return set_error(CIPC_ERR_INVALID_ARG, "cipc_sim_init_dirichlet: empty vertex range");
    const int n_old = (int)s->dbc_idx_h.size();
    std::vector<double> x(3 * (size_t)s->nv), tg(3 * (size_t)n_old);
    cudaError_t e = cudaMemcpyAsync(x.data(), s->x.p, sizeof(double) * x.size(), cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess && n_old)
        e = cudaMemcpyAsync(tg.data(), s->dbc_tgt.p, sizeof(double) * tg.size(), cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) return set_cuda_error(e, "cipc_sim_init_dirichlet");
    double bmin[3], bmax[3];
    for (int d = 0; d < 3; ++d) bmin[d] = bmax[d] = x[3 * (size_t)v_begin + d];
    for (int i = v_begin; i < v_end; ++i)
        for (int d = 0; d < 3; ++d) {
            bmin[d] = std::min(bmin[d], x[3 * (size_t)i + d]);
            bmax[d] = std::max(bmax[d], x[3 * (size_t)i + d]);
        }
    double lo[3], hi[3];
    for (int d = 0; d < 3; ++d) {
        lo[d] = rel_min[d] * (bmax[d] - bmin[d]) + bmin[d];
        hi[d] = rel_max[d] * (bmax[d] - bmin[d]) + bmin[d];
    }
    std::vector<int> idx = s->dbc_idx_h;
    for (int i = v_begin; i < v_end; ++i) {
        const double* p = &x[3 * (size_t)i];
        if (p[0] >= lo[0] && p[0] <= hi[0] && p[1] >= lo[1] && p[1] <= hi[1] && p[2] >= lo[2] && p[2] <= hi[2]) {
            idx.push_back(i);
            tg.insert(tg.end(), p, p + 3);
        }
    }
    const int n = (int)idx.size();
    if (added) *added = n - n_old;
    DbcMotion m;
    m.begin = n_old;
    m.end = n;
    for (int d = 0; d < 3; ++d) {
        m.v[d] = v[d];
        m.center[d] = rot_center[d];
        m.axis[d] = rot_axis[d];
    }
    m.ang_deg = ang_vel_deg;
    std::vector<DbcMotion> motion = s->dbc_motion;
    motion.push_back(m);
    // the list is replaced as a whole (cipc_sim_set_dbc clears the motions), then
    // the motions are put back
    int rc = cipc_sim_set_dbc(h, n, idx.data(), tg.data());
    if (rc) return rc;
    s->dbc_motion = motion;
    if (s->dbc_motion_d.alloc(s->dbc_motion.size()) != cudaSuccess) return set_error(CIPC_ERR_CUDA, "motion buffer");
    e = cudaMemcpyAsync(s->dbc_motion_d.p, s->dbc_motion.data(), sizeof(DbcMotion) * s->dbc_motion.size(),
                        cudaMemcpyHostToDevice, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    return e == cudaSuccess ? CIPC_OK : set_cuda_error(e, "cipc_sim_init_dirichlet");
}

extern "C" int cipc_sim_step_dirichlet(cipc_sim* h, double dt)
{
    if (int rc = check_sim(h)) return rc;
    Sim* s = h->s;
    const int n = (int)s->dbc_idx_h.size();
    if (s->dbc_motion.empty() || n == 0) return CIPC_OK;
    k_step_dirichlet<<<(n + 255) / 256, 256, 0, s->stream>>>((int)s->dbc_motion.size(), s->dbc_motion_d.p, dt,
                                                             s->dbc_tgt.p);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? CIPC_OK : set_cuda_error(e, "cipc_sim_step_dirichlet");
}

extern "C" int cipc_sim_get_dbc(cipc_sim* h, int cap, int* idx, double* targets, int* count)
{
    if (int rc = check_sim(h)) return rc;
    Sim* s = h->s;
    const int n = (int)s->dbc_idx_h.size();
    if (count) *count = n;
    const int m = std::min(std::max(cap, 0), n);
    if (idx && m) std::copy(s->dbc_idx_h.begin(), s->dbc_idx_h.begin() + m, idx);
    if (targets && m) {
        cudaError_t e = cudaMemcpyAsync(targets, s->dbc_tgt.p, sizeof(double) * 3 * m, cudaMemcpyDeviceToHost,
                                        s->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
        if (e != cudaSuccess) return set_cuda_error(e, "cipc_sim_get_dbc");
    }
    return CIPC_OK;
}

extern "C" int cipc_sim_write_obj(cipc_sim* h, const char* path)
{
    if (int rc = check_sim(h)) return rc;
    Sim* s = h->s;
    if (!path) return set_error(CIPC_ERR_INVALID_ARG, "cipc_sim_write_obj: null path");
    std::vector<double> x(3 * (size_t)s->nv);
    std::vector<int> tri(3 * (size_t)s->nt);
    cudaError_t e = cudaMemcpyAsync(x.data(), s->x.p, sizeof(double) * x.size(), cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess && s->nt)
        e = cudaMemcpyAsync(tri.data(), s->tri.p, sizeof(int) * tri.size(), cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) return set_cuda_error(e, "cipc_sim_write_obj");
    FILE* f = std::fopen(path, "w");
    if (!f) return set_error(CIPC_ERR_INVALID_ARG, "cipc_sim_write_obj: cannot create %s", path);
    for (int i = 0; i < s->nv; ++i) std::fprintf(f, "v %le %le %le\n", x[3 * i], x[3 * i + 1], x[3 * i + 2]);
    for (int t = 0; t < s->nt; ++t) std::fprintf(f, "f %d %d %d\n", tri[3 * t] + 1, tri[3 * t + 1] + 1, tri[3 * t + 2] + 1);
    const bool ok = std::fclose(f) == 0;
    return ok ? CIPC_OK : set_error(CIPC_ERR_INVALID_ARG, "cipc_sim_write_obj: write to %s failed", path);
}
