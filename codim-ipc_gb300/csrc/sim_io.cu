// Run logs, checkpoints and frame restarts of a simulation (include/cipc.h).
//
// The reference writes residual.txt / counter.txt / Hessian_info.txt into the
// driver's output folder during Advance_One_Step_IE_Hinge
// (Library/FEM/Shell/IMPLICIT_EULER.h:531-534, 647-670, 868-875); here the same
// lines are appended when an output folder is set.  It restarts a run from an OBJ
// frame plus a finite-difference velocity from the frame before
// (Python/Drivers/FEMDiscreteShellBase.py:244-253, MeshIO.Read_TriMesh_Obj and
// Load_Velocity, Library/Utils/MESHIO.h:967-984); cipc_sim_load_obj_frames does
// that, and cipc_sim_save_state / cipc_sim_load_state keep a run's exact state
// (positions and velocities bit for bit, the barrier stiffness kappa and its
// maximum, which the reference keeps only in memory, IMPLICIT_EULER.h:578-580,
// and the strain-limit stiffness), so that a restored run continues exactly.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/cipc.h"
#include "cipc_util.h"
#include "sim.h"
#include "sim_handle.h"

using namespace cipc;

namespace {

constexpr char kMagic[8] = {'C', 'I', 'P', 'C', 'S', 'T', 'A', '1'};

struct StateHeader {
    char magic[8];
    int64_t nv;
    double kappa, kappa_max;
    double sl_k0, sl_k1;
    int64_t step_count;
};

// vertex lines "v x y z" of an OBJ file, in order
int read_obj_vertices(const char* path, std::vector<double>& out)
{
    FILE* f = std::fopen(path, "r");
    if (!f) return set_error(CIPC_ERR_INVALID_ARG, "cannot open %s", path);
    char line[512];
    out.clear();
    while (std::fgets(line, sizeof(line), f)) {
        if (line[0] == 'v' && (line[1] == ' ' || line[1] == '\t')) {
            double a, b, c;
            if (std::sscanf(line + 2, "%lf %lf %lf", &a, &b, &c) != 3) {
                std::fclose(f);
                return set_error(CIPC_ERR_INVALID_ARG, "%s: malformed vertex line", path);
            }
            out.push_back(a);
            out.push_back(b);
            out.push_back(c);
        }
    }
    std::fclose(f);
    return CIPC_OK;
}

}  // namespace

extern "C" int cipc_sim_set_output(cipc_sim* h, const char* folder)
{
    if (int rc = check_sim(h)) return rc;
    h->s->out_dir = folder ? std::string(folder) : std::string();
    return CIPC_OK;
}

extern "C" int cipc_sim_save_state(cipc_sim* h, const char* path)
{
    if (int rc = check_sim(h)) return rc;
    if (!path) return set_error(CIPC_ERR_INVALID_ARG, "cipc_sim_save_state: null path");
    Sim* s = h->s;
    const size_t n3 = 3 * (size_t)s->nv;
    std::vector<double> buf(2 * n3);
    cudaError_t e = cudaMemcpyAsync(buf.data(), s->x.p, sizeof(double) * n3, cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(buf.data() + n3, s->v.p, sizeof(double) * n3, cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) return set_cuda_error(e, "cipc_sim_save_state");
    StateHeader hd;
    std::memcpy(hd.magic, kMagic, 8);
    hd.nv = s->nv;
    hd.kappa = s->kappa;
    hd.kappa_max = s->kappa_max;
    hd.sl_k0 = s->sl.k0;
    hd.sl_k1 = s->sl.k1;
    hd.step_count = s->step_count;
    FILE* f = std::fopen(path, "wb");
    if (!f) return set_error(CIPC_ERR_INVALID_ARG, "cipc_sim_save_state: cannot create %s", path);
    bool ok = std::fwrite(&hd, sizeof(hd), 1, f) == 1 && std::fwrite(buf.data(), sizeof(double), buf.size(), f) == buf.size();
    ok = (std::fclose(f) == 0) && ok;
    return ok ? CIPC_OK : set_error(CIPC_ERR_INVALID_ARG, "cipc_sim_save_state: write to %s failed", path);
}

extern "C" int cipc_sim_load_state(cipc_sim* h, const char* path)
{
    if (int rc = check_sim(h)) return rc;
    if (!path) return set_error(CIPC_ERR_INVALID_ARG, "cipc_sim_load_state: null path");
    Sim* s = h->s;
    FILE* f = std::fopen(path, "rb");
    if (!f) return set_error(CIPC_ERR_INVALID_ARG, "cipc_sim_load_state: cannot open %s", path);
    StateHeader hd;
    if (std::fread(&hd, sizeof(hd), 1, f) != 1 || std::memcmp(hd.magic, kMagic, 8) != 0) {
        std::fclose(f);
        return set_error(CIPC_ERR_INVALID_ARG, "cipc_sim_load_state: %s is not a simulation state", path);
    }
    if (hd.nv != s->nv) {
        std::fclose(f);
        return set_error(CIPC_ERR_INVALID_ARG, "cipc_sim_load_state: %s holds %lld vertices, the simulation %d", path,
                         (long long)hd.nv, s->nv);
    }
    const size_t n3 = 3 * (size_t)s->nv;
    std::vector<double> buf(2 * n3);
    const bool ok = std::fread(buf.data(), sizeof(double), buf.size(), f) == buf.size();
    std::fclose(f);
    if (!ok) return set_error(CIPC_ERR_INVALID_ARG, "cipc_sim_load_state: %s is truncated", path);
    cudaError_t e = cudaMemcpyAsync(s->x.p, buf.data(), sizeof(double) * n3, cudaMemcpyHostToDevice, s->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(s->v.p, buf.data() + n3, sizeof(double) * n3, cudaMemcpyHostToDevice, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) return set_cuda_error(e, "cipc_sim_load_state");
    s->kappa = hd.kappa;
    s->kappa_max = hd.kappa_max;
    s->sl.k0 = hd.sl_k0;
    s->sl.k1 = hd.sl_k1;
    s->step_count = (int)hd.step_count;
    return CIPC_OK;
}

extern "C" int cipc_sim_load_obj_frames(cipc_sim* h, const char* obj_prev, const char* obj_last, double dt)
{
    if (int rc = check_sim(h)) return rc;
    if (!obj_last || (obj_prev && !(dt > 0)))
        return set_error(CIPC_ERR_INVALID_ARG, "cipc_sim_load_obj_frames: need the last frame and dt > 0");
    Sim* s = h->s;
    std::vector<double> x1, x0;
    int rc = read_obj_vertices(obj_last, x1);
    if (rc) return rc;
    if ((int64_t)x1.size() != 3 * (int64_t)s->nv)
        return set_error(CIPC_ERR_INVALID_ARG, "cipc_sim_load_obj_frames: %s has %zu vertices, the simulation %d",
                         obj_last, x1.size() / 3, s->nv);
    std::vector<double> v(x1.size(), 0.0);
    if (obj_prev) {
        if ((rc = read_obj_vertices(obj_prev, x0))) return rc;
        if (x0.size() != x1.size())
            return set_error(CIPC_ERR_INVALID_ARG, "cipc_sim_load_obj_frames: node count does not match");
        for (size_t k = 0; k < v.size(); ++k) v[k] = (x1[k] - x0[k]) / dt;
    }
    cudaError_t e = cudaMemcpyAsync(s->x.p, x1.data(), sizeof(double) * x1.size(), cudaMemcpyHostToDevice, s->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(s->v.p, v.data(), sizeof(double) * v.size(), cudaMemcpyHostToDevice, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    return e == cudaSuccess ? CIPC_OK : set_cuda_error(e, "cipc_sim_load_obj_frames");
}
