"""Contact-kernel microbenchmark: ACCD time of impact over 10M seeded contact pairs.

Workload (one "step"): one additive-CCD pass over 10,000,000 candidate pairs
(40% point-triangle, 40% edge-edge, 10% point-edge, 10% point-point), vertices
uniform in the unit cube, separations log-uniform in [1e-6, 1e-2], Gaussian
displacements with sigma = 0.5 x separation, eta = 0.1, offset xi = 1e-7,
step fraction 1.  Inputs are ~2 GB, larger than L2, so no flush is needed
between steps.  The headline `value` runs the mixed-precision kernel on
device-resident inputs; `e2e` runs the same pass through the C ABI with pinned
host buffers (copies in the timed region).  The FP64 kernel and the barrier
(energy/gradient/PSD Hessian) pass are reported under "variants".

Also reported (single GPU): "timestep", ms/timestep of the 200x200 cloth on the
rotating sphere for plain FP64 block-Jacobi PCG, FP32 Hessians with FP64
refinement, the learned block-Jacobi correction, and each with inexact-Newton
forcing; "scenes", absolute steps/s of the cloth-on-cube (with the CPU oracle
on the same steps), mixed codimensional (rods + particles + cloth) and stacked
shell scenes.

  python bench.py [--gpus N --steps K --warmup W] [--impl ours|reference]

Multi-GPU: each rank runs its own replica with its own seed (weak scaling, no
collective on the data path); the timing is the max over ranks.
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "codim-ipc_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "CCD Mpairs/s"
ETA, XI, TOC_IN = 0.1, 1e-7, 1.0
DHAT2, KAPPA = 1e-4, 1.0


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Clocks:
    """Samples SM clocks and throttle reasons with nvidia-smi while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


def _peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def _traffic(name, pairs=None):
    """DRAM bytes per launch from a committed ncu summary (profiles/<name>.txt):
    its `dram_bytes_per_launch:` line, or its `dram_bytes_per_pair:` line times
    `pairs` (a capture of a smaller case scaled to the launch); else None."""
    p = os.path.join(ROOT, "profiles", name + ".txt")
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.startswith("dram_bytes_per_launch:"):
            return float(line.split(":")[1])
        if line.startswith("dram_bytes_per_pair:") and pairs:
            return round(float(line.split(":")[1]) * pairs)
    return None


def _pair_sample(w, m):
    """m pairs evenly strided over the pair list (type and index arrays), so that
    a sample keeps the workload's mix of pair types."""
    n = w["type"].shape[0]
    sel = np.linspace(0, n - 1, m).astype(np.int64) if m < n else np.arange(n)
    return np.ascontiguousarray(w["type"][sel]), np.ascontiguousarray(w["idx"][sel])


def run_reference(args):
    """CPU arm: the CPU restatement of the reference's ACCD, all host threads."""
    ws, rank, _ = _dist()
    if rank != 0:
        return
    import workloads
    from oracle import oracle_ffi as orc
    w = workloads.contact_pairs(args.pairs, seed=0)
    n = w["type"].shape[0]
    cores = orc.num_threads()
    # each step is a bounded sample of the workload — m pairs evenly strided over
    # the list, so the PT/EE/PE/PP mix is kept — sized from the warm-up rate so
    # that the timed steps take about two minutes in all
    m0 = min(n, 100000)
    t0m, i0m = _pair_sample(w, m0)
    t0 = time.perf_counter()
    for _ in range(max(1, args.warmup)):
        orc.ccd_pairs(t0m, i0m, w["x"], w["dx"], ETA, XI, TOC_IN)
    rate = m0 * max(1, args.warmup) / (time.perf_counter() - t0)
    m = int(min(n, max(m0, rate * 120.0 / max(1, args.steps))))
    tm, im = _pair_sample(w, m)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        orc.ccd_pairs(tm, im, w["x"], w["dx"], ETA, XI, TOC_IN)
    dt = time.perf_counter() - t0
    v = m * args.steps / dt / 1e6
    line = {
        "impl": "reference", "metric": METRIC, "value": round(v, 3), "unit": "Mpairs/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(dt / args.steps * 1e3, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "ACCD time of impact, %d seeded contact pairs (PT/EE/PE/PP 40/40/10/10)" % n,
                   "pairs": n, "eta": ETA, "xi": XI},
        "cpu_baseline": {"value": round(v, 3), "unit": "Mpairs/s", "cores": cores, "kind": "port",
                         "sample": "%d of the %d pairs (evenly strided) per step" % (m, n)},
        "e2e": {"value": round(v, 3), "unit": "Mpairs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference (Eigen/CHOLMOD/Kokkos C++) cannot be built on this image; its ACCD is timed "
                "through the CPU restatement in oracle/ (OpenMP, FP64)",
    }
    print(json.dumps(line))


def max_over_ranks(value, device):
    """The largest of one float over all ranks (the whole job's time is the
    slowest replica's)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([value], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_mpairs(total_s, pairs_per_rank, steps, ws):
    """Mpairs/s of the whole job: every rank's pairs over the slowest rank's time."""
    return pairs_per_rank * ws * steps / total_s / 1e6


def mixed_vs_fp64(toc_a, hit_a, toc_b, hit_b, a_is_mixed):
    """Differences of the mixed-precision ACCD from the bit-exact FP64 one on the
    same pairs, by direction: an unsafe miss is a pair the mixed kernel lets move
    the whole step while FP64 finds an impact; a late time is a shared hit whose
    mixed time exceeds the FP64 time (both are unsafe for a step-size search)."""
    if not a_is_mixed:
        toc_a, hit_a, toc_b, hit_b = toc_b, hit_b, toc_a, hit_a
    m_hit, f_hit = hit_a == 1, hit_b == 1
    both = m_hit & f_hit
    rel = np.abs(toc_a[both] - toc_b[both]) / toc_b[both] if both.any() else np.zeros(1)
    n = float(hit_a.shape[0])
    return {"hit_mismatch_frac": float((m_hit != f_hit).mean()),
            "unsafe_miss": int((~m_hit & f_hit).sum()), "spurious_hit": int((m_hit & ~f_hit).sum()),
            "late_toc": int((toc_a[both] > toc_b[both]).sum()), "early_toc": int((toc_a[both] < toc_b[both]).sum()),
            "toc_bit_equal_frac": float(np.mean(toc_a.view(np.uint64) == toc_b.view(np.uint64))),
            "toc_rel_err_p999": float(np.quantile(rel, 0.999)), "toc_rel_err_max": float(rel.max()),
            "hit_frac": float(f_hit.mean()), "pairs": int(n),
            "note": "mixed = float-float ACCD (CIPC_PRECISION_MIXED), not bit-exact and not guaranteed conservative; "
                    "the timed value is the FP64 kernel"}


def _time_calls(fn, steps, stream):
    import torch
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    start = torch.cuda.Event(enable_timing=True)
    stop = torch.cuda.Event(enable_timing=True)
    start.record(stream)
    for e0, e1 in evs:
        e0.record(stream)
        fn()
        e1.record(stream)
    stop.record(stream)
    torch.cuda.synchronize()
    per = [e0.elapsed_time(e1) for e0, e1 in evs]
    return start.elapsed_time(stop), per


def timestep_variants(args):
    """ms/timestep of the cloth-on-rotating-sphere scene (200x200 cloth, 2 m, sphere
    r 0.5 m at 2 rad/s, mu 0.4, xi 0.5 mm, dhat 1 mm, dt 0.02, Newton tol 1e-3):
    plain FP64 block-Jacobi PCG vs FP32 Hessians + FP64 refinement, with block
    Jacobi and with the learned correction trained on systems the plain mixed
    solver captured while draping.  Every variant starts from the same draped
    state and advances ts_steps steps."""
    import cipc_ffi as F
    import workloads

    X, T, dbc, c = workloads.cloth_on_sphere(n=args.ts_n)
    dt, omega = 0.02, 2.0

    def target(k):
        return workloads.rotate_y(X[dbc], c, omega * dt * (k + 1))

    def make(prec, pre, forcing=0):
        s = F.Sim(X, T, 200.0, 1e5, 0.3, 1e-3)
        _, dhat2 = s.init_oipc(1e-3)
        prm = F.make_params(dt, dhat2, 5e-4, mu=0.4, epsv2=1e-6, fric_iters=1, newton_tol=1e-3, precision=prec,
                            pcg_tol=1e-4, preconditioner=pre, forcing=forcing)
        return s, prm

    ok = (F.CIPC_ERR_NOT_CONVERGED,)
    s, prm = make(F.MIXED, 0)
    pc = F.Precond(hidden=16, layers=2, seed=0)
    cap_from = max(0, args.ts_warm - 6)
    for k in range(args.ts_warm):
        if k == cap_from:
            F.sim_capture_systems(s, pc, 512)
        s.set_dbc(dbc, target(k))
        s.step(prm, allow=ok)
    F.sim_capture_systems(s, None, 0)
    x0, v0 = s.state()
    k0 = s.kappa()
    s.close()
    t0 = time.perf_counter()
    loss_before, loss_after = pc.train(epochs=args.ts_epochs, batch=8, lr=1e-3, seed=0)
    train_s = time.perf_counter() - t0
    out = {"workload": "cloth on rotating sphere, %dx%d cloth (%d vertices incl. sphere), %d steps from step %d"
                       % (args.ts_n, args.ts_n, X.shape[0], args.ts_steps, args.ts_warm),
           "unit": "ms/timestep", "newton_tol": 1e-3, "pcg_tol": 1e-4,
           "learned": {"systems": pc.num_systems(), "epochs": args.ts_epochs, "train_s": round(train_s, 2),
                       "loss_before": round(loss_before, 4), "loss_after": round(loss_after, 4)}}
    variants = (("fp64_block_jacobi", F.FP64, 0, 0), ("mixed_block_jacobi", F.MIXED, 0, 0),
                ("mixed_learned", F.MIXED, 1, 0), ("fp64_block_jacobi_inexact", F.FP64, 0, 1),
                ("mixed_block_jacobi_inexact", F.MIXED, 0, 1))
    for name, prec, pre, forcing in variants:
        sv, pv = make(prec, pre, forcing)
        if pre:
            F.sim_set_precond(sv, pc)
        sv.set_state(x0, v0)
        sv.set_kappa(k0[0], k0[1])
        rows = []
        for k in range(args.ts_warm, args.ts_warm + args.ts_steps):
            sv.set_dbc(dbc, target(k))
            st = sv.step(pv, allow=ok)
            rows.append(st.as_dict())
        sv.close()
        out[name] = {"ms_per_step": round(float(np.mean([r["ms"] for r in rows])), 2),
                     "newton_per_step": round(float(np.mean([r["newton_iters"] for r in rows])), 2),
                     "pcg_per_step": round(float(np.mean([r["pcg_iters"] for r in rows])), 1),
                     "fallbacks": int(sum(r["precond_fallbacks"] for r in rows)),
                     "min_dist2_min": float(min(r["min_dist2"] for r in rows)),
                     "intersection_free": bool(all(r["min_dist2"] > 0 or r["n_constraints"] == 0 for r in rows)),
                     "status": sorted(set(int(r["status"]) for r in rows))}
    out["speedup_mixed_learned_vs_fp64"] = round(out["fp64_block_jacobi"]["ms_per_step"]
                                                 / out["mixed_learned"]["ms_per_step"], 3)
    out["speedup_mixed_vs_fp64"] = round(out["fp64_block_jacobi"]["ms_per_step"]
                                         / out["mixed_block_jacobi"]["ms_per_step"], 3)
    out["speedup_mixed_inexact_vs_fp64"] = round(out["fp64_block_jacobi"]["ms_per_step"]
                                                 / out["mixed_block_jacobi_inexact"]["ms_per_step"], 3)
    out["note"] = ("*_inexact: Eisenstat-Walker forcing term for the Newton systems (cipc_step_params.forcing = 1); "
                   "the Newton tolerance is the same for every variant; the forcing term is not combined with the "
                   "learned correction")
    pc.close()
    return out


def _scene_stats(rows):
    ms = [r["ms"] for r in rows]
    con = [r for r in rows if r["n_constraints"] > 0]
    return {"steps": len(rows), "ms_per_step": round(float(np.mean(ms)), 2),
            "steps_per_s": round(1000.0 / float(np.mean(ms)), 3),
            "newton_per_step": round(float(np.mean([r["newton_iters"] for r in rows])), 2),
            "pcg_per_step": round(float(np.mean([r["pcg_iters"] for r in rows])), 1),
            "constraints_max": int(max(r["n_constraints"] for r in rows)),
            "min_dist2_min": float(min(r["min_dist2"] for r in con)) if con else None,
            "intersection_free": bool(all(r["min_dist2"] > 0 for r in con)),
            "status": sorted(set(int(r["status"]) for r in rows))}


def scene_runs(args):
    """Absolute steps/s of the other named scenes, each from its initial state:
    the 40x40 cloth falling on a fixed 0.3 m cube (StVK, 50 steps, dt 0.04, Newton
    tol 1e-2; FP64 and mixed, and the CPU oracle on its first steps), the mixed
    codimensional scene (1000 rods x 100 segments, 20000 particles, 120x120 cloth
    pinned at its corners; dt 0.01, mu 0.2) and the 8-layer stacked shells
    (8 x 180x180 cloths between a fixed and a descending plate at 0.05 m/s;
    dt 0.01, mu 0.3, xi = dhat = 0.5 mm)."""
    import cipc_ffi as F
    import workloads

    ok = (F.CIPC_ERR_NOT_CONVERGED,)

    def run(sim, prm, dbc, tgt, steps):
        rows = []
        for k in range(steps):
            sim.set_dbc(dbc, tgt(k))
            rows.append(sim.step(prm, allow=ok).as_dict())
        return rows

    out = {"precond": "block Jacobi", "pcg_tol": 1e-4}
    # cloth on cube
    X, T, dbc = workloads.cloth_on_box(n=40)
    c1 = {"workload": "40x40 cloth (1 m, StVK E 1e5, t 1 mm) falling 0.1 m onto a fixed 0.3 m cube, dt 0.04, "
                      "xi = dhat = 1 mm, Newton tol 1e-2, %d vertices incl. the cube" % X.shape[0]}
    for name, prec in (("fp64", F.FP64), ("mixed", F.MIXED)):
        s = F.Sim(X, T, 200.0, 1e5, 0.3, 1e-3, nh=False)
        _, dhat2 = s.init_oipc(1e-3)
        prm = F.make_params(0.04, dhat2, 1e-3, newton_tol=1e-2, precision=prec, pcg_tol=1e-4)
        rows = run(s, prm, dbc, lambda k: X[dbc], args.c1_steps)
        s.close()
        c1[name] = _scene_stats(rows)
        c1[name]["first_%d_ms_per_step" % args.c1_cpu_steps] = round(
            float(np.mean([r["ms"] for r in rows[:args.c1_cpu_steps]])), 2)
    if not args.no_cpu_baseline and args.c1_cpu_steps > 0:
        from oracle import oracle_ffi as orc
        sh = orc.Shell(X, T, 200.0, 1e5, 0.3, 1e-3, nh=False)
        k2, dhat2 = sh.init_oipc(1e-3)
        x, v = X.copy(), np.zeros_like(X)
        t0 = time.perf_counter()
        newton = []
        for _ in range(args.c1_cpu_steps):
            rc, st = sh.step(x, v, k2, dbc, X[dbc], 0.04, dhat2, 1e-3, tol=1e-2)
            newton.append(st["newton_iters"])
        cpu_ms = (time.perf_counter() - t0) * 1e3 / args.c1_cpu_steps
        c1["cpu_oracle"] = {"kind": "port", "cores": orc.num_threads(), "ms_per_step": round(cpu_ms, 1),
                            "newton_per_step": round(float(np.mean(newton)), 2),
                            "sample": "first %d steps, direct (skyline LDL^T) Newton solves" % args.c1_cpu_steps}
        c1["speedup_mixed_vs_cpu_oracle"] = round(cpu_ms / c1["mixed"]["first_%d_ms_per_step" % args.c1_cpu_steps], 1)
    out["cloth_on_cube_40"] = c1
    # mixed codimensional scene
    X, T, S, P, corners = workloads.rods_particles_on_cloth_full()
    codim = dict(segments=S, rod_E=1e7, rod_rho=1000.0, rod_thickness=1e-3, particles=P, particle_rho=1000.0,
                 particle_thickness=4e-3)
    s = F.Sim(X, T, 200.0, 1e5, 0.3, 1e-3, codim=codim)
    _, dhat2 = s.init_oipc(1e-3)
    prm = F.make_params(0.01, dhat2, 1e-3, mu=0.2, epsv2=1e-6, fric_iters=1, newton_tol=1e-2, precision=F.MIXED,
                        pcg_tol=1e-4)
    rows = run(s, prm, corners, lambda k: X[corners], args.sc_steps)
    s.close()
    out["rods_particles_on_cloth"] = dict(
        workload="1000 rods x 100 segments (0.5 m, E 1e7, 5 layers of 200 with seeded directions), 20000 particles "
                 "(4 mm), 120x120 cloth pinned at its corners; %d vertices; dt 0.01, xi = dhat = 1 mm, mu 0.2; "
                 "first %d steps, mixed precision" % (X.shape[0], args.sc_steps), **_scene_stats(rows))
    # stacked shells
    X, T, dbc, top = workloads.stacked_shells()
    s = F.Sim(X, T, 200.0, 1e5, 0.3, 1e-3)
    _, dhat2 = s.init_oipc(5e-4)
    prm = F.make_params(0.01, dhat2, 5e-4, mu=0.3, epsv2=1e-6, fric_iters=1, newton_tol=1e-2, precision=F.MIXED,
                        pcg_tol=1e-4)
    istop = np.isin(dbc, top)

    def plate(k):
        Y = X[dbc].copy()
        Y[istop, 1] -= 0.05 * 0.01 * (k + 1)
        return Y

    rows = run(s, prm, dbc, plate, args.sc_steps)
    s.close()
    out["stacked_shells_8x180"] = dict(
        workload="8 layers of 180x180 cloth (1 m, 5 mm apart, 1 mm seeded in-plane jitter) between a fixed plate and "
                 "a plate descending at 0.05 m/s; %d vertices; dt 0.01, xi = dhat = 0.5 mm, mu 0.3; first %d steps, "
                 "mixed precision" % (X.shape[0], args.sc_steps), **_scene_stats(rows))
    return out


def trace_scene(args):
    """Steps the cloth-on-rotating-sphere scene (args.trace_scene x args.trace_scene
    cloth) for args.trace_steps steps and prints each step's statistics (no JSON
    line): the workload of the committed time-step profiles."""
    import cipc_ffi as F
    import workloads

    X, T, dbc, c = workloads.cloth_on_sphere(n=args.trace_scene)
    prec = F.MIXED if args.trace_precision == "mixed" else F.FP64
    s = F.Sim(X, T, 200.0, 1e5, 0.3, 1e-3)
    _, dhat2 = s.init_oipc(1e-3)
    prm = F.make_params(0.02, dhat2, 5e-4, mu=0.4, epsv2=1e-6, fric_iters=1, newton_tol=1e-3, precision=prec,
                        pcg_tol=1e-4)
    for k in range(args.trace_steps):
        s.set_dbc(dbc, workloads.rotate_y(X[dbc], c, 2.0 * 0.02 * (k + 1)))
        st = s.step(prm, allow=(F.CIPC_ERR_NOT_CONVERGED,))
        print("step", k, st.as_dict(), flush=True)
    s.close()


def run_ours(args):
    import torch
    import torch.distributed as dist

    import cipc_ffi as F
    import workloads

    ws, rank, local = _dist()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if ws > 1:
        dist.init_process_group("nccl", device_id=dev)
    w = workloads.contact_pairs(args.pairs, seed=rank)
    n = w["type"].shape[0]
    d = {k: torch.from_numpy(np.ascontiguousarray(w[k])).to(dev) for k in ("type", "idx", "x", "dx")}
    toc = torch.empty(n, dtype=torch.float64, device=dev)
    hit = torch.empty(n, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream()
    prec = F.MIXED if args.precision == "mixed" else F.FP64

    def step(p=prec):
        F.ccd_pairs_async(d["type"], d["idx"], d["x"], d["dx"], toc, hit, ETA, XI, TOC_IN, p, stream)

    for _ in range(max(3, args.warmup)):
        step()
    st, ov = F.ccd_pairs(d["type"], d["idx"], d["x"], d["dx"], toc, hit, ETA, XI, TOC_IN, prec, F.MEM_DEVICE, stream)
    assert ov == 0, "iteration-cap overflow in warm-up"
    torch.cuda.synchronize()
    if ws > 1:
        dist.barrier()
    clocks = Clocks(local)
    clocks.start()
    total_ms, per = _time_calls(step, args.steps, stream)
    clk = clocks.stop()
    if ws > 1:
        dist.barrier()
        total_ms = max_over_ranks(total_ms, dev)
    ms = total_ms / args.steps
    value = whole_job_mpairs(total_ms / 1e3, n, args.steps, ws)

    # FP64 variant (same inputs) and barrier passes
    variants = {}
    step()
    torch.cuda.synchronize()
    toc_a, hit_a = toc.cpu().numpy(), hit.cpu().numpy()
    other = F.FP64 if prec == F.MIXED else F.MIXED
    _, per_o = _time_calls(lambda: step(other), 3, stream)
    variants["ccd_%s_mpairs_s" % ("fp64" if other == F.FP64 else "mixed")] = round(n / (np.mean(per_o) / 1e3) / 1e6, 2)
    toc_b, hit_b = toc.cpu().numpy(), hit.cpu().numpy()
    variants["ccd_mixed_vs_fp64"] = mixed_vs_fp64(toc_a, hit_a, toc_b, hit_b, prec == F.MIXED)
    nb = min(n, args.barrier_pairs)
    E = torch.empty(nb, dtype=torch.float64, device=dev)
    G = torch.empty((nb, 12), dtype=torch.float64, device=dev)
    outs = {}
    for bp, htype in ((F.MIXED, torch.float32), (F.FP64, torch.float64)):
        H = torch.empty((nb, 78), dtype=htype, device=dev)
        fn = lambda: F.barrier_pairs_async(d["type"][:nb], d["idx"][:nb], d["x"], d["x"], E, G, H, DHAT2, XI, KAPPA,
                                           True, bp, stream)
        fn()
        _, per_b = _time_calls(fn, 2, stream)
        key = "barrier_psd_%s_mpairs_s" % ("mixed" if bp == F.MIXED else "fp64")
        variants[key] = round(nb / (np.mean(per_b) / 1e3) / 1e6, 3)
        outs[bp] = (E.cpu().numpy(), G.cpu().numpy(), H.double().cpu().numpy())
        del H
    (Em, Gm, Hm), (Ed, Gd, Hd) = outs[F.MIXED], outs[F.FP64]
    hs = np.maximum(np.abs(Hd).max(1), 1e-300)
    gs = np.maximum(np.abs(Gd).max(1), 1e-300)
    variants["barrier_mixed_vs_fp64"] = {
        "energy_rel_err_max": float((np.abs(Em - Ed) / np.maximum(np.abs(Ed), 1e-300)).max()),
        "grad_rel_err_max": float((np.abs(Gm - Gd).max(1) / gs).max()),
        "hess_rel_err_p999": float(np.quantile(np.abs(Hm - Hd).max(1) / hs, 0.999)),
        "hess_rel_err_max": float((np.abs(Hm - Hd).max(1) / hs).max()),
        "note": "errors per pair relative to the pair's largest FP64 entry"}

    # end to end through the C ABI with pinned host buffers
    ph = {k: torch.from_numpy(np.ascontiguousarray(w[k])).pin_memory().numpy() for k in ("type", "idx", "x", "dx")}
    toc_h = torch.empty(n, dtype=torch.float64).pin_memory().numpy()
    hit_h = torch.empty(n, dtype=torch.uint8).pin_memory().numpy()
    F.ccd_pairs(ph["type"], ph["idx"], ph["x"], ph["dx"], toc_h, hit_h, ETA, XI, TOC_IN, prec, F.MEM_HOST, stream)
    e2e_steps = max(1, min(args.steps, 3))
    if ws > 1:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        F.ccd_pairs(ph["type"], ph["idx"], ph["x"], ph["dx"], toc_h, hit_h, ETA, XI, TOC_IN, prec, F.MEM_HOST, stream)
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    if ws > 1:
        e2e_s = max_over_ranks(e2e_s, dev)
    h2d = sum(ph[k].nbytes for k in ph)
    d2h = toc_h.nbytes + hit_h.nbytes + 24

    # roofline of the dominant kernel (k_accd): algorithmic bytes / launch duration
    ccd_bytes, _ = workloads.pair_bytes(w["type"])
    launch_s = float(np.mean(per)) / 1e3
    peak, peak_kind = _peaks()
    achieved = ccd_bytes / launch_s / 1e9
    traffic = _traffic("accd_mixed_10M_pairs") if prec == F.MIXED else _traffic("accd_fp64_2M_pairs", n)

    line = None
    if rank == 0:
        cpu = None
        if ws == 1 and not args.no_cpu_baseline:
            from oracle import oracle_ffi as orc
            m = min(n, 4_000_000)
            tm, im = _pair_sample(w, m)
            t0 = time.perf_counter()
            reps = 0
            while True:
                orc.ccd_pairs(tm, im, w["x"], w["dx"], ETA, XI, TOC_IN)
                reps += 1
                if time.perf_counter() - t0 > 8.0 or reps >= 10:
                    break
            cdt = time.perf_counter() - t0
            cpu = {"value": round(m * reps / cdt / 1e6, 3), "unit": "Mpairs/s", "cores": orc.num_threads(),
                   "kind": "port", "sample": "%d x %d pairs of the same workload (evenly strided)" % (reps, m)}
        line = {
            "metric": METRIC, "value": round(value, 2), "unit": "Mpairs/s", "n_gpus": ws, "steps": args.steps,
            "warmup": max(3, args.warmup), "ms_per_step": round(ms, 4), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+float-float" if prec == F.MIXED else "f64", "data": "synthetic",
            "config": {"workload": "ACCD time of impact, %d seeded contact pairs per GPU (PT/EE/PE/PP 40/40/10/10)"
                                   % n, "pairs_per_gpu": n, "precision": args.precision, "eta": ETA, "xi": XI,
                       "l2": "inputs (%.2f GB) larger than L2; no flush" % (ccd_bytes / 1e9)},
            "e2e": {"value": round(whole_job_mpairs(e2e_s, n, 1, ws), 2), "unit": "Mpairs/s",
                    "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
            "gpu_launches": args.steps,
            "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                         "frac": round(achieved / peak, 4), "traffic": traffic,
                         "kernel": ("k_accd_mixed" if prec == F.MIXED else
                                    "k_accd_setup + k_accd_steps (one two-pass launch pair, timed together)"),
                         "peak_source": peak_kind,
                         "fp64_pipe_busy": None if prec == F.MIXED else 0.866,
                         "note": ("ACCD is instruction-issue bound (FP32 and integer pipes: float-float "
                                  "distances, ~3.4 distance evaluations per pair), not HBM bound; bytes are the "
                                  "algorithmic minimum, read once" if prec == F.MIXED else
                                  "ACCD in FP64 is bound by the FP64 pipe (2 lanes per SM per clock on this part; "
                                  "86.6% busy in the stepping pass, profiles/accd_fp64_2M_pairs.txt), not by "
                                  "HBM; achieved counts the algorithmic bytes, read once; traffic also counts the "
                                  "128-byte per-pair state the set-up pass writes and the stepping pass reads")},
            "clocks": clk,
            "variants": variants,
            "cpu_baseline": cpu,
        }
        if ws == 1 and not args.no_timestep:
            line["timestep"] = timestep_variants(args)
        if ws == 1 and not args.no_scenes:
            line["scenes"] = scene_runs(args)
        print(json.dumps(line))
    if ws > 1:
        dist.barrier()
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--pairs", type=int, default=10_000_000)
    ap.add_argument("--barrier-pairs", type=int, default=2_000_000)
    ap.add_argument("--precision", default="fp64", choices=["mixed", "fp64"],
                    help="kernel timed as the headline (fp64: bit-exact with the CPU restatement)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-timestep", action="store_true", help="skip the cloth-on-sphere ms/timestep variants")
    ap.add_argument("--ts-n", type=int, default=200, help="cloth resolution of the time-step variants")
    ap.add_argument("--ts-warm", type=int, default=10, help="draping steps before the measured steps")
    ap.add_argument("--ts-steps", type=int, default=6, help="measured steps per variant")
    ap.add_argument("--ts-epochs", type=int, default=20, help="training epochs of the learned correction")
    ap.add_argument("--no-scenes", action="store_true", help="skip the cube / codimensional / stacked-shell scenes")
    ap.add_argument("--trace-scene", type=int, default=0,
                    help="only step the cloth-on-sphere scene at this resolution (profiling workload)")
    ap.add_argument("--trace-steps", type=int, default=12)
    ap.add_argument("--trace-precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--c1-steps", type=int, default=50, help="steps of the cloth-on-cube scene")
    ap.add_argument("--c1-cpu-steps", type=int, default=8, help="cloth-on-cube steps run by the CPU oracle")
    ap.add_argument("--sc-steps", type=int, default=6, help="steps of the codimensional and stacked scenes")
    args = ap.parse_args()
    if args.trace_scene > 0:
        trace_scene(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
