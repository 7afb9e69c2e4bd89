"""Benchmark of the GB300 Rosenbrock transport step.

Workload (default): the 512x512x128 cut-cell configuration on which the
FP32-refined vs FP64 comparison is stated -- Gaussian hill h=1 km, half-width
5 km, Gaussian-correlated roughness (sigma 50 m, 2 km), dx=dy=200 m,
dz 50->400 m, snapping + small-cell merge, N=0.01 1/s, u=10 m/s, moist, one
tracer; 10 cell components (Rho, six LR momentum components, Rho*theta,
Rho*qv, Rho*tracer); RosRK3 (3 stages), dt = 2 s, BiCGStab tolerance 1e-10,
6-sweep Gauss-Seidel preconditioner on the FP64 path.  --nx 256 --ny 256 gives
the 256x256x128 plain-FP64 configuration.  Seeded synthetic fields stand in
for the reference's (unpublished) decks.

One step = one Ros3MetC call: per stage ExchangeCell, (stage 1) the 7-diagonal
Jacobian, the flux RHS of all components, the stage combinations and a full
BiCGStab solve, then the state update.  The metric is Mcell-steps/s (interior
cells x steps / s).

Arms:
  (default)          ours: FP64 drop-in path (value), plus the FP32-refined path
                     (autotuned), the adjoint cost (128x128x64 hill, 40 steps),
                     the 48-domain batched ensemble, the pressure projection
                     (ProjectVelFace) of a closed block on the bench grid and
                     the Rosenbrock step of the dynamical core (prognostic
                     momentum, pressure gradient, buoyancy, projection) on
                     the same closed block
  --impl reference   the reference's CPU path (the oracle restatement of the
                     Fortran; the Fortran itself has no compiler here), one
                     process per host core on independent blocks.
"""
from __future__ import annotations

import argparse
import json
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "Mcell-steps/s"
# DRAM bytes of one PSolve per padded cell, measured with ncu on the 256x256x64
# workload (profiles/traffic_psolve_256x256x64.md), 10 components: the FP64
# Gauss-Seidel call and the refined mode's FP32 x-line call (without the
# once-per-matrix factors); scaled to a launch of the bench grid by padded cells
TRAFFIC_PSOLVE_FP64_PER_PCELL = 11553.6e6 / 4393224
TRAFFIC_PSOLVE_XLINE_PER_PCELL = (1622.97e6 - 55.0e6) / 4393224
BYTES_PER_CELL_FLUX = lambda ncomp: 64 + 16 * ncomp  # noqa: E731  algorithmic bytes per interior cell


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--nx", type=int, default=512)
    p.add_argument("--ny", type=int, default=512)
    p.add_argument("--nz", type=int, default=128)
    p.add_argument("--dt", type=float, default=2.0)
    p.add_argument("--tol", type=float, default=1e-10)
    p.add_argument("--no-refined", action="store_true")
    p.add_argument("--no-adjoint", action="store_true")
    p.add_argument("--no-batch", action="store_true")
    p.add_argument("--no-projection", action="store_true")
    p.add_argument("--no-dyn", action="store_true", help="skip the dynamical-core step")
    p.add_argument("--no-diffusion", action="store_true", help="skip the diffusion cost")
    p.add_argument("--no-restart", action="store_true", help="skip the restart-file throughput")
    p.add_argument("--restart-only", action="store_true", help="only the restart section; prints its JSON object")
    p.add_argument("--diffusion-only", action="store_true",
                   help="only the diffusion section (profiling); prints its JSON object")
    p.add_argument("--dyn-only", action="store_true",
                   help="only the dynamical-core section (profiling); prints its JSON object")
    p.add_argument("--probe", choices=["psolve", "inner_psolve"],
                   help="profiling: build the workload, compute its stage matrix, run exactly one PSolve "
                        "(FP64 Gauss-Seidel) or one FP32 inner PSolve (x-line) and exit")
    p.add_argument("--projection-only", action="store_true",
                   help="only the projection section (profiling); prints its JSON object")
    p.add_argument("--batch-members", type=int, default=48)
    p.add_argument("--batch-steps", type=int, default=20)
    p.add_argument("--batch-threads", type=int, default=0, help="host threads driving the members (0: one each)")
    p.add_argument("--adj-grid", default="128,128,64", help="nx,ny,nz of the adjoint-cost workload")
    p.add_argument("--adj-steps", type=int, default=40)
    p.add_argument("--adj-ckpt", type=int, default=8)
    p.add_argument("--precision", default="both", choices=["both", "fp64", "fp32_refined"],
                   help="which variants to run (profiling runs take one)")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--cpu-sample", type=int, default=48, help="edge of the oracle's CPU sample window")
    p.add_argument("--no-autotune", action="store_true", help="keep --inner/--inner-gs-iter instead of autotuning")
    p.add_argument("--inner", default="gauss_seidel", choices=["gauss_seidel", "line", "xline", "yline"],
                   help="preconditioner of the FP32 inner solver of the refined path")
    p.add_argument("--inner-gs-iter", type=int, default=1,
                   help="IterG of the refined path's FP32 inner Gauss-Seidel (the FP64 path keeps 5)")
    return p.parse_args()


def workload(nx, ny, nz, seed=2):
    from asam_gb300 import geometry as G

    return G.hill_case(nx, ny, nz, seed=seed)


def workload_config(a):
    return {"workload": f"cut-cell Gaussian hill {a.nx}x{a.ny}x{a.nz}, 10 components, RosRK3 dt={a.dt}s, "
                        f"BiCGStab tol {a.tol:g}, 6-sweep GS preconditioner",
            "nx": a.nx, "ny": a.ny, "nz": a.nz, "ncomp": 10, "method": "RosRK3", "dt": a.dt,
            "bicgstab_tol": a.tol,
            "l2": f"inputs larger than L2 (state {10 * 8 * (a.nx + 2) * (a.ny + 2) * (a.nz + 2) / 1e9:.2f} GB, "
                  f"matrix {8 * 8 * (a.nx + 2) * (a.ny + 2) * (a.nz + 2) / 1e9:.2f} GB)",
            "parallelism": "replicas" if a.gpus > 1 else "single GPU"}


# ---------------------------------------------------------------------------
# CPU baseline (oracle restatement of the reference Fortran), one block per process
# ---------------------------------------------------------------------------
def _cpu_worker(args):
    edge, nz, dt, tol, steps, seed = args
    import oracle
    from asam_gb300 import METHODS

    geo, vel, st = workload(edge, edge, nz, seed=seed)
    o = oracle.Oracle(geo)
    c = st.c.copy()
    t0 = time.perf_counter()
    for _ in range(steps):
        o.ros_step(c, vel, dt, method=METHODS["RosRK3"], tol=tol)
    return time.perf_counter() - t0, edge * edge * nz * steps


def cpu_baseline(edge, nz, dt, tol, steps, procs):
    ctx = mp.get_context("spawn")
    jobs = [(edge, nz, dt, tol, steps, 2 + i) for i in range(procs)]
    t0 = time.perf_counter()
    if procs == 1:
        res = [_cpu_worker(jobs[0])]
    else:
        with ctx.Pool(procs) as pool:
            res = pool.map(_cpu_worker, jobs)
    wall = time.perf_counter() - t0
    cells = sum(r[1] for r in res)
    slowest = max(r[0] for r in res)
    return cells / slowest / 1e6, wall


def cpu_model():
    try:
        for line in Path("/proc/cpuinfo").read_text().splitlines():
            if line.lower().startswith(("model name", "cpu part")):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return "unknown"


# ---------------------------------------------------------------------------
# clocks sampled during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.proc = None
        self.tmp = None

    def __enter__(self):
        self.tmp = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.tmp,
                                         stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.tmp.flush()
        rows = [r.split(",") for r in Path(self.tmp.name).read_text().strip().splitlines() if r.strip()]
        os.unlink(self.tmp.name)
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                smax = float(r[2])
                for n, v in zip(names, r[5:9]):
                    if v.strip().lower() == "active":
                        reasons.add(n)
            except (ValueError, IndexError):
                continue
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------
def run_reference(a, rank):
    """--impl reference: the reference's CPU path (oracle port) on all host cores."""
    if rank != 0:
        return
    procs = os.cpu_count() or 1
    edge = max(8, a.cpu_sample // 2)
    value, wall = cpu_baseline(edge, a.nz, a.dt, a.tol, a.steps, procs)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": a.gpus,
            "steps": a.steps, "warmup": a.warmup, "ms_per_step": None, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded generators)",
            "config": workload_config(a),
            "cpu_baseline": {"value": value, "unit": METRIC, "cores": procs, "kind": "port",
                             "sample": f"{procs} independent {edge}x{edge}x{a.nz} blocks of the same generator, "
                                       f"{a.steps} steps each (MPI-over-blocks model), oracle restatement of the "
                                       f"Fortran, {cpu_model()}"},
            "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def adjoint_cost(a, lib, torch, stream):
    """Cost of the checkpointed gradient against the forward run it differentiates.

    Workload: cut-cell Gaussian hill h=800 m, half-width 4 km on the adjoint grid
    (default 128x128x64), Rho, Rho*theta and a passive tracer, RosRK3 dt=2 s,
    adj_steps steps, checkpoints every adj_ckpt steps, J = sum over a 16x16x8 box
    of (tracer mixing ratio)^2 V at the final time; everything device-resident.
    """
    import ctypes as C

    import numpy as np

    import asam_gb300
    from asam_gb300 import _lib
    from asam_gb300 import geometry as G

    nx, ny, nz = (int(v) for v in a.adj_grid.split(","))
    geo, vel, st = G.hill_case(nx, ny, nz, seed=5, height=800.0, halfwidth=4000.0, moist=False, momentum=False,
                               tracer=True)
    ncomp = st.c.shape[0]
    comp = ncomp - 1
    tol = a.tol
    blk = asam_gb300.TransportBlock(geo, ncomp, method="RosRK3", bicgstab_tol=tol, bicgstab_maxiter=200)
    blk.set_velocity(*vel)
    blk.set_stream(stream.cuda_stream)
    c0 = torch.from_numpy(st.c.reshape(-1).copy()).cuda()
    cur = c0.clone()
    npad = geo.grid.npad
    grad = torch.empty(npad, dtype=torch.float64, device="cuda")
    lam = torch.zeros(npad, dtype=torch.float64, device="cuda")
    lam_out = torch.empty_like(lam)
    i0 = max(1, int(0.3 * nx) + 1)
    j0 = max(1, ny // 2 - 7)
    k0 = max(1, nz // 8)
    box = (C.c_int * 6)(i0, min(nx, i0 + 15), j0, min(ny, j0 + 15), k0, min(nz, k0 + 7))
    lamv = lam.view(nz + 2, ny + 2, nx + 2)
    lamv[k0:k0 + 8, j0:j0 + 16, i0:i0 + 16] = 1.0
    p = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731

    def fwd():
        iters = (C.c_int * 4)()
        resid = (C.c_double * 4)()
        _lib.check(lib.asam_ros_step(blk.h, p(cur), a.dt, iters, resid), "asam_ros_step", allow=(0, 1, 2))

    J = C.c_double()

    def gradient(nsteps):
        _lib.check(lib.asam_tracer_gradient(blk.h, p(c0), comp, nsteps, a.dt, a.adj_ckpt, box, tol, C.byref(J),
                                            p(grad)), "asam_tracer_gradient", allow=(0, 1))

    def adj_step():
        _lib.check(lib.asam_ros_step_adj(blk.h, p(c0), comp, p(lam), p(lam_out), a.dt, tol), "asam_ros_step_adj",
                   allow=(0, 1))

    uf, vf, wf = (np.ascontiguousarray(v, dtype=np.float64) for v in vel)
    gr = torch.empty(npad, dtype=torch.float64, device="cuda")
    gu = torch.empty(uf.size, dtype=torch.float64, device="cuda")
    gv = torch.empty(vf.size, dtype=torch.float64, device="cuda")
    gw = torch.empty(wf.size, dtype=torch.float64, device="cuda")

    def wind_gradient(nsteps):
        _lib.check(lib.asam_tracer_wind_gradient(blk.h, p(c0), comp, nsteps, a.dt, a.adj_ckpt, box, tol, C.byref(J),
                                                 p(grad), p(gr), p(gu), p(gv), p(gw)), "asam_tracer_wind_gradient",
                   allow=(0, 1))

    fwd()
    cur.copy_(c0)
    ms_fwd = time_region(torch, stream, fwd, a.adj_steps)
    gradient(a.adj_ckpt)
    ms_grad = time_region(torch, stream, lambda: gradient(a.adj_steps), 1)
    wind_gradient(a.adj_ckpt)
    ms_wgrad = time_region(torch, stream, lambda: wind_gradient(a.adj_steps), 1)
    cur.copy_(c0)
    ms_fwd1 = time_region(torch, stream, fwd, 3) / 3
    adj_step()
    ms_adj1 = time_region(torch, stream, adj_step, 3) / 3
    blk.close()
    return {"workload": f"cut-cell Gaussian hill h=800 m, half-width 4 km, {nx}x{ny}x{nz}, {ncomp} components "
                        f"(Rho, Rho*theta, Rho*tracer), RosRK3 dt={a.dt}s, {a.adj_steps} steps, checkpoint every "
                        f"{a.adj_ckpt}, J over a 16x16x8 box, BiCGStab tol {tol:g}",
            "forward_ms": ms_fwd, "gradient_ms": ms_grad, "gradient_over_forward": ms_grad / ms_fwd,
            "tracer_and_wind_gradient_ms": ms_wgrad, "tracer_and_wind_gradient_over_forward": ms_wgrad / ms_fwd,
            "forward_step_ms": ms_fwd1, "adjoint_step_ms": ms_adj1,
            "adjoint_step_over_forward_step": ms_adj1 / ms_fwd1,
            "note": "adjoint step = asam_ros_step_adj: the step's forward recomputation with stage states plus its "
                    "transpose; gradient = forward sweep with checkpoints + per step one recomputation, the stage "
                    "matrix rebuild and the adjoint step (tracer only, density and wind fixed); tracer-and-wind "
                    "gradient = the coupled density-tracer adjoint with the face mass fluxes as parameters (one "
                    "recomputation per step, the increments of Rho and the tracer stored per segment)",
            "J": J.value}


PROJ_BETA0 = 0.435866521508459  # beta0 of RosRK3 (the projection's beta0*dtP)


def vcycle_bytes(n1, n2, n3, R, gi2=1, gi3=1):
    """Algorithmic bytes of one multigrid V-cycle (Solve_3D, zebra order) on the
    (z,x,y) = (n1,n2,n3) hierarchy with R levels, counted from its schedule:
    per line-solve element 96 B (rhs b, the two neighbour-line x, the two x
    couplings, the z sub-diagonal, the pivot and its reciprocal, x written;
    the back substitution reads x and w and writes x), per plane right-hand
    side element 48 B, per residual element 64 B (plane) / 88 B (3D), per
    restriction fine element 8 B and coarse element 16 B, per prolongation fine
    element 16 B and coarse element 8 B, plus the two layout passes (16 B per
    cell each) of the call."""
    cd = lambda n, L: (n + (1 << L) - 1) >> L  # noqa: E731

    def mg2d(dims):
        t = 0
        nq = len(dims)
        for q, (c1, c2) in enumerate(dims):
            n = c1 * c2
            t += (2 * (q * gi2 + 1) * 2 * n * 96) if c2 > 1 else 2 * n * 96
            if q + 1 < nq:
                nc = dims[q + 1][0] * dims[q + 1][1]
                t += n * 64 + n * 8 + nc * 16 + n * 16 + nc * 8
        return t

    total = 2 * 16 * n1 * n2 * n3
    for L in range(R):
        m1, m2, m3 = cd(n1, L), cd(n2, L), cd(n3, L)
        dims = [(cd(n1, L2), cd(n2, L2)) for L2 in range(L, R)]
        plane = m1 * m2 * 48 + mg2d(dims)
        gi = L * gi3 + 1
        total += (2 * gi * 2 * m3 * plane) if m3 > 1 else 2 * plane
        if L + 1 < R:
            n = m1 * m2 * m3
            nc = cd(n1, L + 1) * cd(n2, L + 1) * cd(n3, L + 1)
            total += n * 88 + n * 8 + nc * 16 + n * 16 + nc * 8
    return total


def projection_bench(a, torch, stream, hbm_peak):
    """Pressure projection (ProjectVelFace: Rhs, FGMRES(10) on MatVec1 with the
    multigrid-preconditioned PSolve1, UpdateVelocity) of a closed-box cut-cell
    hill on the bench grid (h=600 m, half-width 800 m plus roughness, dx=dy=200 m,
    dz 50->400 m, RefLevel 4), seeded sound weights and face-velocity
    increments, dtP = dt, beta0 of RosRK3; device-resident fields.  The CPU
    baseline is the oracle (reference lexicographic smoother) on a 64x64x32
    block of the same generator, single-threaded."""
    import ctypes as C

    import numpy as np

    import asam_gb300
    import oracle
    from asam_gb300 import geometry as G

    nx, ny, nz = a.nx, a.ny, a.nz
    ncell = nx * ny * nz
    cpu_base = None
    if not a.no_cpu_baseline:
        cpu_base = _projection_cpu_baseline(a)

    geo = G.closed_hill_case(nx, ny, nz, seed=9)
    W, dx, dy, dz, (u, v, w) = G.projection_inputs(geo, seed=21)
    blk = asam_gb300.TransportBlock(geo, 3, rho_pos=0)
    blk.set_stream(stream.cuda_stream)
    blk.proj_setup(dx, dy, dz)
    blk.proj_weights(*W)
    lib = blk.lib
    P = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
    assemble_ms = time_region(torch, stream, lambda: blk.JacAccGrav(PROJ_BETA0, a.dt), 2) / 2
    du0, dv0, dw0 = (torch.from_numpy(q).cuda() for q in (u, v, w))
    du, dv, dw = du0.clone(), dv0.clone(), dw0.clone()
    incr = torch.zeros((3,) + geo.grid.pshape, dtype=torch.float64, device="cuda")
    steps, res = C.c_int(), C.c_double()

    def project():
        du.copy_(du0)
        dv.copy_(dv0)
        dw.copy_(dw0)
        rc = lib.asam_project_vel_face(blk.h, P(du), P(dv), P(dw), P(incr), None, 1, 0, None, 0, None,
                                       C.byref(steps), C.byref(res))
        if rc not in (0, 1):
            raise RuntimeError(f"asam_project_vel_face: {rc}")

    for _ in range(2):
        project()
    n_rep = 3
    l0 = lib.asam_launch_count()
    v0 = lib.asam_proj_vcycles(blk.h)
    proj_ms = time_region(torch, stream, project, n_rep) / n_rep
    launches = (lib.asam_launch_count() - l0) // n_rep
    vcyc = (lib.asam_proj_vcycles(blk.h) - v0) // n_rep
    bb = torch.randn(nz, ny, nx, dtype=torch.float64, device="cuda")
    xx = torch.zeros_like(bb)
    vc_ms = time_region(torch, stream, lambda: lib.asam_lapl_vcycle(blk.h, P(bb), P(xx)), 3) / 3
    yy = torch.zeros_like(bb)
    lib.asam_lapl_matvec(blk.h, P(xx), P(yy))
    red = float(torch.linalg.norm(bb - yy) / torch.linalg.norm(bb))
    vb = vcycle_bytes(nz, nx, ny, 4)
    gbs = vb / (vc_ms * 1e-3) / 1e9
    steps64, res64 = steps.value, res.value
    # the same with the FP32 copy of the multigrid preconditioning FGMRES
    blk.proj_set_precision("fp32")
    for _ in range(2):
        project()
    proj32_ms = time_region(torch, stream, project, n_rep) / n_rep
    steps32, res32 = steps.value, res.value
    vc32_ms = time_region(torch, stream, lambda: lib.asam_lapl_vcycle(blk.h, P(bb), P(xx)), 3) / 3
    gbs32 = vb / 2 / (vc32_ms * 1e-3) / 1e9
    blk.close()
    return {
        "workload": f"closed-box cut-cell hill {nx}x{ny}x{nz} (h=600 m, half-width 800 m, roughness 50 m / 600 m, "
                    f"dx=dy=200 m, dz 50->400 m), RefLevel 4, FGMRES(10) QMRTol 1e-6, dtP={a.dt} s, "
                    "seeded sound weights and velocity increments",
        "metric": "Mcell-projections/s", "value": ncell / (proj_ms * 1e-3) / 1e6, "ms_per_projection": proj_ms,
        "fgmres_steps": steps64, "fgmres_rel_residual": res64, "vcycles_per_projection": vcyc,
        "assemble_ms": assemble_ms, "vcycle_ms": vc_ms, "vcycle_residual_reduction": red,
        "gpu_launches_per_projection": launches,
        "roofline": {"kernel": "one V-cycle (k_plane_half zebra plane/line relaxations + 3D residual, restriction, "
                               "prolongation)", "bound": "hbm", "achieved": gbs, "peak": hbm_peak, "unit": "GB/s",
                     "frac": gbs / hbm_peak, "algorithmic_bytes_per_call": vb, "traffic": None,
                     "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)"},
        "fp32_multigrid": {"ms_per_projection": proj32_ms, "value": ncell / (proj32_ms * 1e-3) / 1e6,
                           "speedup_vs_fp64_multigrid": proj_ms / proj32_ms, "fgmres_steps": steps32,
                           "fgmres_rel_residual": res32, "vcycle_ms": vc32_ms,
                           "roofline": {"bound": "hbm", "achieved": gbs32, "peak": hbm_peak, "unit": "GB/s",
                                        "frac": gbs32 / hbm_peak, "algorithmic_bytes_per_call": vb // 2,
                                        "traffic": None}},
        "cpu_baseline": cpu_base,
    }


def _projection_cpu_baseline(a):
    """The oracle (reference lexicographic smoother) projecting a 64x64x32
    closed block of the same generator on one host core."""
    import numpy as np

    import oracle
    from asam_gb300 import geometry as G

    cgeo = G.closed_hill_case(64, 64, 32, seed=9)
    cW, cdx, cdy, cdz, (cu, cv, cw) = G.projection_inputs(cgeo, seed=21)
    t0 = time.perf_counter()
    op = oracle.OracleProj(cgeo, cdx, cdy, cdz, cW, zebra=0)
    op.lapl_compute(PROJ_BETA0, a.dt)
    b = op.rhs(cu, cv, cw)
    x = np.zeros_like(b)
    csteps, _, _ = op.fgmres(x, b)
    op.update(x, cu.copy(), cv.copy(), cw.copy())
    cpu_s = time.perf_counter() - t0
    op.close()

    return {"value": 64 * 64 * 32 / cpu_s / 1e6, "unit": "Mcell-projections/s", "cores": 1, "kind": "port",
            "sample": f"64x64x32 block of the same generator, oracle restatement with the reference's "
                      f"lexicographic smoother, {csteps} FGMRES steps ({cpu_s:.1f} s)"}


def _dyn_kinds(ncomp, mom):
    """Closed box with free-slip walls: the momentum component normal to a wall
    is ZeroValue there, everything else ZeroGrad."""
    k = [[1] * 6 for _ in range(ncomp)]
    for q, p in enumerate(mom):
        for sd in range(6):
            k[p][sd] = 2 if q // 2 == sd // 2 else 1
    return k


def dyn_bench(a, torch, stream):
    """Rosenbrock step of the dynamical core (asam_ros_step_dyn: per stage the
    face->cell velocities, thermodynamics, FcnMet with pressure gradient and
    buoyancy, the transport BiCGStab, cell->face, ProjectVelFace; the
    Jacobian and the Laplacian hierarchy at the first stage) on a closed-box
    cut-cell hill of the bench grid with a warm bubble, moisture and a tracer;
    device-resident state.  Run with the FP64 transport solve and with the
    FP32-refined one (x-line inner preconditioner); the two end states are
    compared.  The CPU baseline is the oracle on a 64x64x32 block of the same
    generator, single-threaded."""
    import ctypes as C

    import numpy as np

    import asam_gb300
    import oracle
    from asam_gb300 import geometry as G

    nx, ny, nz = a.nx, a.ny, a.nz
    geo, vel, st, pos, (dx, dy, dz), bc = G.dyn_case(nx, ny, nz, seed=11, moist=True, tracer=True)
    nc = st.c.shape[0]

    def run(prec):
        kw = {"inner_precond": "xline"} if prec == "fp32_refined" else {}
        blk = asam_gb300.TransportBlock(geo, nc, rho_pos=0, method="RosRK3", bicgstab_tol=a.tol, precision=prec, **kw)
        blk.set_stream(stream.cuda_stream)
        blk.set_velocity(*vel)
        blk.proj_setup(dx, dy, dz)
        blk.dyn_setup(pos["th"], pos["mom"], rv_pos=pos["qv"], bound_cells=bc, scalars=[pos["qv"], pos["tracer"]])
        lib = blk.lib
        c = torch.from_numpy(st.c).cuda()
        it = (C.c_int * 4)()
        rs = (C.c_double * 4)()
        ps = (C.c_int * 4)()
        pr = (C.c_double * 4)()

        def step():
            rc = lib.asam_ros_step_dyn(blk.h, C.c_void_p(c.data_ptr()), a.dt, it, rs, ps, pr)
            if rc not in (0, 1, 2):
                raise RuntimeError(f"asam_ros_step_dyn: {rc}")

        step()  # warm-up
        n_rep = 2
        l0 = lib.asam_launch_count()
        ms = time_region(torch, stream, step, n_rep) / n_rep
        launches = (lib.asam_launch_count() - l0) // n_rep
        blk.close()
        return ms, launches, c, list(it[:3]), list(ps[:3]), list(pr[:3])

    ms, launches, c, its, pss, prs = run("fp64")
    ms_r, _, c_r, its_r, _, _ = run("fp32_refined")
    err = float(max(((c_r[q] - c[q]).abs().max() / c[q].abs().max().clamp_min(1e-300)).item() for q in range(nc)))
    vol = torch.from_numpy(geo.volc).cuda()
    mass = float((c[0] * vol)[1:-1, 1:-1, 1:-1].sum())
    mass0 = float(np.sum((st.c[0] * geo.volc)[1:-1, 1:-1, 1:-1]))
    cpu = None
    if not a.no_cpu_baseline:
        cgeo, cvel, cst, cpos, (cdx, cdy, cdz), cbc = G.dyn_case(64, 64, 32, seed=11, moist=True, tracer=True)
        o = oracle.Oracle(cgeo, bc=_dyn_kinds(cst.c.shape[0], cpos["mom"]))
        op = oracle.OracleProj(cgeo, cdx, cdy, cdz, G.projection_inputs(cgeo)[0], zebra=0)
        cc = cst.c.copy()
        cu = [q.copy() for q in cvel]
        t0 = time.perf_counter()
        o.ros_step_dyn(op, cc, cu, a.dt, rho_pos=0, th_pos=cpos["th"], pos=cpos["mom"], dx=cdx, dy=cdy, dz=cdz,
                       rv_pos=cpos["qv"], bound=cbc, scalars=[cpos["qv"], cpos["tracer"]], bicg_tol=a.tol)
        cpu_s = time.perf_counter() - t0
        op.close()
        cpu = {"value": 64 * 64 * 32 / cpu_s / 1e6, "unit": "Mcell-steps/s", "cores": 1, "kind": "port",
               "sample": f"one step of a 64x64x32 block of the same generator, oracle restatement with the "
                         f"reference's lexicographic smoother ({cpu_s:.2f} s)"}
    return {
        "workload": f"dynamical core, closed-box cut-cell hill {nx}x{ny}x{nz} (h=600 m, half-width 800 m, "
                    f"roughness, dx=dy=200 m, dz 50->400 m), N=0.01 1/s, 2 K warm bubble, moisture and a tracer "
                    f"({nc} components), {len(bc)} boundary cells, free-slip walls, RosRK3 dt={a.dt} s, "
                    f"BiCGStab tol {a.tol}, FGMRES(10) QMRTol 1e-6",
        "metric": "Mcell-steps/s", "value": nx * ny * nz / (ms * 1e-3) / 1e6, "ms_per_step": ms,
        "bicgstab_iterations": its, "fgmres_steps": pss, "fgmres_rel_residual": prs,
        "gpu_launches_per_step": launches, "mass_rel_change": (mass - mass0) / mass0,
        "fp32_refined": {"value": nx * ny * nz / (ms_r * 1e-3) / 1e6, "ms_per_step": ms_r,
                         "speedup_vs_fp64": ms / ms_r, "bicgstab_iterations": its_r,
                         "max_rel_err_vs_fp64_after_3_steps": err},
        "cpu_baseline": cpu,
    }


def diffusion_bench(a, torch, stream):
    """Cost of the diffusion terms on the bench workload (faces of zero-volume
    cells closed, seeded density-weighted diffusivities 50 / 5 m^2/s decaying
    with height): the flux right-hand side with and without diffusion, and the
    FP64 Rosenbrock step with diffusion and its Jacobian."""
    import copy
    import ctypes as C

    import asam_gb300
    from asam_gb300 import geometry as G

    geo, vel, st = workload(a.nx, a.ny, a.nz)
    geo = G.close_dead_faces(copy.deepcopy(geo))
    dh, dv = G.diffusion_coefficients(geo, st.c[0], seed=5)
    blk = asam_gb300.TransportBlock(geo, st.c.shape[0], method="RosRK3", bicgstab_tol=a.tol)
    blk.set_stream(stream.cuda_stream)
    blk.set_velocity(*vel)
    lib = blk.lib
    c = torch.from_numpy(st.c).cuda()
    f = torch.empty_like(c)
    P = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
    fcn = lambda: lib.asam_fcn(blk.h, P(c), P(f))  # noqa: E731
    fcn()
    ms_plain = time_region(torch, stream, fcn, 3) / 3
    blk.set_diffusion(dh, dv)
    fcn()
    ms_diff = time_region(torch, stream, fcn, 3) / 3
    it = (C.c_int * 4)()
    rs = (C.c_double * 4)()

    def step():
        rc = lib.asam_ros_step(blk.h, P(c), a.dt, it, rs)
        if rc not in (0, 1, 2):
            raise RuntimeError(f"asam_ros_step: {rc}")

    step()
    ms_step = time_region(torch, stream, step, 2) / 2
    blk.close()
    return {"workload": f"bench grid {a.nx}x{a.ny}x{a.nz}, zero-volume cells' faces closed, DiffKoeff 50/5 m^2/s x Rho "
                        "decaying with height, +-20 % seeded", "flux_rhs_ms": ms_diff, "flux_rhs_ms_without": ms_plain,
            "flux_rhs_diffusion_overhead": ms_diff / ms_plain - 1.0, "ms_per_step": ms_step,
            "value": a.nx * a.ny * a.nz / (ms_step * 1e-3) / 1e6, "metric": METRIC,
            "krylov_iterations": list(it[:3])}


def restart_bench(a, torch):
    """Restart file of the bench state (WriteRestart / ReadRestart): the
    device-resident components and face velocities streamed to a file and
    back through the pinned staging buffers.  Wall-clock timed: the write
    ends when the file is closed (page cache, no fsync, like the reference's
    CLOSE); the read follows it."""
    import numpy as np

    from asam_gb300 import restart as R

    geo, vel, st = workload(a.nx, a.ny, a.nz)
    g = geo.grid
    c = torch.from_numpy(st.c).cuda().reshape(st.c.shape[0], -1)
    veld = [torch.from_numpy(np.ascontiguousarray(v).ravel()).cuda() for v in vel]
    blk = R.block(g.nx, g.ny, g.nz, c, *veld)
    c2 = torch.empty_like(c)
    vel2 = [torch.empty_like(v) for v in veld]
    blk2 = R.block(g.nx, g.ny, g.nz, c2, *vel2)
    nbytes = (c.numel() + sum(v.numel() for v in veld)) * 8
    d = tempfile.mkdtemp(prefix="asam_restart_")
    path = os.path.join(d, "Hill.0")
    try:
        tw, tr = [], []
        for _ in range(2):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            R.write_restart(path, [blk], 100.0, 1, 0.0)
            tw.append(time.perf_counter() - t0)
            t0 = time.perf_counter()
            R.read_restart(path, [blk2])
            tr.append(time.perf_counter() - t0)
        ok = bool(torch.equal(c2, c) and all(torch.equal(x, y) for x, y in zip(vel2, veld)))
        fsize = os.path.getsize(path)
    finally:
        if os.path.exists(path):
            os.remove(path)
        os.rmdir(d)
    return {"workload": f"bench state {g.nx}x{g.ny}x{g.nz}, {st.c.shape[0]} components + face velocities, "
                        "device-resident, one file", "bytes": nbytes, "file_bytes": fsize,
            "write_s": min(tw), "read_s": min(tr), "write_gbs": nbytes / min(tw) / 1e9,
            "read_gbs": nbytes / min(tr) / 1e9, "roundtrip_bitwise": ok}


def batch_members(n, seed=4):
    """Ensemble of independent cut-cell domains: sizes between 64x64x48 and
    192x160x96, Gaussian hill 0-1.5 km high with half-width 2-8 km, u 5-15 m/s,
    N 0.008-0.012 1/s, all drawn from the seed."""
    import numpy as np

    from asam_gb300 import geometry as G

    rng = np.random.default_rng(seed)
    out = []
    for m in range(n):
        nx, ny, nz = int(rng.integers(64, 193)), int(rng.integers(64, 161)), int(rng.integers(48, 97))
        height, halfwidth = float(rng.uniform(0.0, 1500.0)), float(rng.uniform(2000.0, 8000.0))
        u0, nbv = float(rng.uniform(5.0, 15.0)), float(rng.uniform(0.008, 0.012))
        out.append(G.hill_case(nx, ny, nz, seed=seed * 1000 + m, height=height, halfwidth=halfwidth, u0=u0, n_bv=nbv))
    return out


def batch_bench(a, torch, members):
    """Batched ensemble: all members advanced batch_steps RosRK3 steps (dt=2 s)
    in one asam_batch_ros_step call, device-resident states; FP64 and refined."""
    import asam_gb300

    cells = sum(g.grid.nx * g.grid.ny * g.grid.nz for g, _, _ in members)
    res = {"workload": f"{len(members)} independent cut-cell domains (64x64x48 to 192x160x96, hill 0-1.5 km, "
                       f"half-width 2-8 km, u 5-15 m/s, N 0.008-0.012), {cells / 1e6:.1f} M cells in total, "
                       f"{members[0][2].c.shape[0]} components, RosRK3 dt=2 s, {a.batch_steps} steps, "
                       f"BiCGStab tol {a.tol:g}", "cells": cells, "steps": a.batch_steps}
    for prec in ("fp64", "fp32_refined"):
        blocks, dev = [], []
        t_tune, choices = 0.0, {}
        for geo, vel, st in members:
            b = asam_gb300.TransportBlock(geo, st.c.shape[0], method="RosRK3", bicgstab_tol=a.tol,
                                          bicgstab_maxiter=30, precision=prec, inner_gs_iter=a.inner_gs_iter)
            b.set_velocity(*vel)
            if not a.no_autotune:  # each member picks its own solver settings
                t0 = time.perf_counter()
                ch = b.autotune(st.c, 2.0)
                t_tune += time.perf_counter() - t0
                key = (f"{ch['inner_precond']}/iterg{ch['inner_gs_iter']}/{ch['gs_schedule']}/g{ch['gs_group']}"
                       if prec == "fp32_refined" else "fp64") + ("/graphs" if ch["graphs"] else "")
                choices[key] = choices.get(key, 0) + 1
            blocks.append(b)
            dev.append(torch.from_numpy(st.c.reshape(-1).copy()).cuda())
        torch.cuda.synchronize()
        ptrs = [t.data_ptr() for t in dev]
        with asam_gb300.Batch(blocks, nthreads=a.batch_threads) as batch:
            batch.ros_step(ptrs, 2.0, nsteps=1)  # warm-up
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            its, status = batch.ros_step(ptrs, 2.0, nsteps=a.batch_steps)
            torch.cuda.synchronize()
            wall = time.perf_counter() - t0
        for b in blocks:
            b.close()
        del dev
        torch.cuda.empty_cache()
        res[prec] = {"value": cells * a.batch_steps / wall / 1e6, "unit": METRIC, "seconds": wall,
                     "members_not_ok": int((status != 0).sum())}
        if choices:
            res[prec]["autotuned"] = {"settings": choices, "tuning_seconds": t_tune}
    res["speedup_refined_vs_fp64"] = res["fp32_refined"]["value"] / res["fp64"]["value"]
    return res


# ---------------------------------------------------------------------------
# replicas (N > 1): one independent block per rank, no data-path collective;
# the timed region's maximum over ranks and the whole-job aggregate
# ---------------------------------------------------------------------------
def reduce_max(dist, x, device):
    """Maximum of x over the ranks (x itself without a process group)."""
    if dist is None:
        return x
    import torch

    t = torch.tensor([float(x)], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_rate(world, units_per_rank, steps, ms_max):
    """Whole-job rate in M units per second: every rank processed units_per_rank
    per step, the job took the slowest rank's time."""
    return world * units_per_rank * steps / (ms_max * 1e-3) / 1e6


def time_region(torch, stream, fn, n):
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    s.record(stream)
    for _ in range(n):
        fn()
    e.record(stream)
    torch.cuda.synchronize()
    return s.elapsed_time(e)


def main():
    a = parse()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if a.impl == "reference":
        run_reference(a, rank)
        return

    if a.projection_only:
        import torch

        import __graft_entry__

        __graft_entry__.build()
        stream = torch.cuda.Stream()
        torch.cuda.set_stream(stream)
        pk0 = ROOT / "MEASURED_PEAKS.json"
        hp = json.loads(pk0.read_text()).get("hbm_gbs", 6800.0) if pk0.exists() else 6800.0
        print(json.dumps(projection_bench(a, torch, stream, hp)), flush=True)
        return
    if a.probe:
        import ctypes as C

        import torch

        import __graft_entry__
        import asam_gb300

        __graft_entry__.build()
        geo, vel, st = workload(a.nx, a.ny, a.nz)
        refined = a.probe == "inner_psolve"
        blk = asam_gb300.TransportBlock(geo, st.c.shape[0], method="RosRK3", bicgstab_tol=a.tol,
                                        precision="fp32_refined" if refined else "fp64",
                                        inner_precond="xline" if refined else "gauss_seidel")
        blk.set_velocity(*vel)
        c = torch.from_numpy(st.c).cuda()
        out = torch.empty_like(c)
        P = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
        blk.lib.asam_jac(blk.h, P(c), a.dt)
        fn = blk.lib.asam_inner_psolve if refined else blk.lib.asam_psolve
        torch.cuda.synchronize()
        n0 = blk.lib.asam_launch_count()
        rc = fn(blk.h, P(c), P(out))
        torch.cuda.synchronize()
        print(json.dumps({"probe": a.probe, "rc": rc, "launches": blk.lib.asam_launch_count() - n0,
                          "npad": (a.nx + 2) * (a.ny + 2) * (a.nz + 2), "ncomp": st.c.shape[0]}), flush=True)
        blk.close()
        return
    if a.restart_only:
        import torch

        import __graft_entry__

        __graft_entry__.build()
        print(json.dumps(restart_bench(a, torch)), flush=True)
        return
    if a.diffusion_only:
        import torch

        import __graft_entry__

        __graft_entry__.build()
        stream = torch.cuda.Stream()
        torch.cuda.set_stream(stream)
        print(json.dumps(diffusion_bench(a, torch, stream)), flush=True)
        return
    if a.dyn_only:
        import torch

        import __graft_entry__

        __graft_entry__.build()
        stream = torch.cuda.Stream()
        torch.cuda.set_stream(stream)
        print(json.dumps(dyn_bench(a, torch, stream)), flush=True)
        return
    # CPU baseline first (before any GPU call), rank 0, N=1 only
    cpu = None
    if rank == 0 and world == 1 and not a.no_cpu_baseline:
        edge = a.cpu_sample
        value, wall = cpu_baseline(edge, a.nz, a.dt, a.tol, 1, 1)
        cpu = {"value": value, "unit": METRIC, "cores": 1, "kind": "port",
               "sample": f"one {edge}x{edge}x{a.nz} window of the same generator, 1 step, single-threaded oracle "
                         f"restatement of the Fortran ({wall:.1f} s), {cpu_model()}"}

    import ctypes as C

    import numpy as np
    import torch

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")

    import __graft_entry__

    __graft_entry__.build()
    import asam_gb300
    from asam_gb300 import _lib

    lib = _lib.load()
    geo, vel, st = workload(a.nx, a.ny, a.nz)
    ncomp = st.c.shape[0]
    ncell = a.nx * a.ny * a.nz
    # one non-default stream for torch and the library alike (the library
    # captures its Krylov half-iterations as CUDA graphs on it)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)

    def barrier():
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()

    def max_over_ranks(x):
        return reduce_max(dist, x, "cuda")

    results = {}
    gpu_launches = {}
    precs = ["fp64"] + ([] if a.no_refined else ["fp32_refined"])
    if a.precision != "both":
        precs = [a.precision]
    for prec in precs:
        blk = asam_gb300.TransportBlock(geo, ncomp, method="RosRK3", bicgstab_tol=a.tol, bicgstab_maxiter=30,
                                        precision=prec, inner_precond=a.inner, inner_gs_iter=a.inner_gs_iter)
        blk.set_velocity(*vel)
        blk.set_stream(stream.cuda_stream)
        tuned = None
        if not a.no_autotune:
            t0 = time.perf_counter()
            tuned = blk.autotune(st.c, a.dt)
            tuned["tuning_seconds"] = time.perf_counter() - t0
        dptr = blk.state_device_ptr()
        host0 = torch.from_numpy(st.c.reshape(-1).copy())
        dstate = torch.empty(st.c.size, dtype=torch.float64, device="cuda")
        dstate.copy_(host0)
        ctypes_dptr = C.c_void_p(dstate.data_ptr())
        iters_all = []

        def step():
            iters = (C.c_int * 4)()
            resid = (C.c_double * 4)()
            rc = lib.asam_ros_step(blk.h, ctypes_dptr, a.dt, iters, resid)
            _lib.check(rc, "asam_ros_step", allow=(0, 1, 2))
            iters_all.append([iters[i] for i in range(blk.nstage)])

        for _ in range(a.warmup):
            step()
        barrier()
        iters_all.clear()
        n0 = lib.asam_launch_count()
        with ClockSampler(local) as clk:
            ms = time_region(torch, stream, step, a.steps)
        barrier()
        gpu_launches[prec] = lib.asam_launch_count() - n0
        ms = max_over_ranks(ms)
        final = dstate.cpu().numpy().copy()

        # end to end through the public API with pinned host buffers
        pinned = torch.empty(st.c.size, dtype=torch.float64).pin_memory()
        pinned.copy_(host0)
        hptr = C.c_void_p(pinned.data_ptr())

        def step_e2e():
            iters = (C.c_int * 4)()
            resid = (C.c_double * 4)()
            _lib.check(lib.asam_ros_step(blk.h, hptr, a.dt, iters, resid), "asam_ros_step", allow=(0, 1, 2))

        step_e2e()
        barrier()
        t0 = time.perf_counter()
        ms_e2e = time_region(torch, stream, step_e2e, a.steps)
        wall_e2e = (time.perf_counter() - t0) * 1e3
        ms_e2e = max_over_ranks(max(ms_e2e, wall_e2e))

        # dominant kernels, timed alone with CUDA events on the same stream
        f_out = torch.empty_like(dstate)
        kt = {}
        nrep = 5
        kt["flux_rhs_ms"] = time_region(torch, stream, lambda: _lib.check(
            lib.asam_fcn(blk.h, ctypes_dptr, C.c_void_p(f_out.data_ptr())), "asam_fcn"), nrep) / nrep
        kt["psolve_ms"] = time_region(torch, stream, lambda: _lib.check(
            lib.asam_psolve(blk.h, C.c_void_p(f_out.data_ptr()), ctypes_dptr), "asam_psolve"), nrep) / nrep
        dstate.copy_(torch.from_numpy(final.reshape(-1)))
        kt["matvec_ms"] = time_region(torch, stream, lambda: _lib.check(
            lib.asam_matvec(blk.h, ctypes_dptr, C.c_void_p(f_out.data_ptr())), "asam_matvec"), nrep) / nrep
        if prec == "fp32_refined":
            kt["inner_psolve_ms"] = time_region(torch, stream, lambda: _lib.check(
                lib.asam_inner_psolve(blk.h, ctypes_dptr, C.c_void_p(f_out.data_ptr())), "asam_inner_psolve"),
                nrep) / nrep
        results[prec] = {"ms": ms, "ms_e2e": ms_e2e, "final": final, "iters": iters_all, "clocks": clk.summary(),
                         "kernels": kt, "tuned": tuned}
        blk.close()
        del dstate, f_out, pinned
        torch.cuda.empty_cache()

    adj = None
    if not a.no_adjoint and world == 1:
        adj = adjoint_cost(a, lib, torch, stream)
    bat = None
    if not a.no_batch and world == 1:
        bat = batch_bench(a, torch, batch_members(a.batch_members))
    proj = None
    if not a.no_projection and world == 1:
        pk0 = ROOT / "MEASURED_PEAKS.json"
        hp = json.loads(pk0.read_text()).get("hbm_gbs", 6800.0) if pk0.exists() else 6800.0
        proj = projection_bench(a, torch, stream, hp)
    dyn = None
    if not a.no_dyn and world == 1:
        dyn = dyn_bench(a, torch, stream)
    diff = None
    if not a.no_diffusion and world == 1:
        diff = diffusion_bench(a, torch, stream)
    rst = None
    if not a.no_restart and world == 1:
        rst = restart_bench(a, torch)
    if "fp64" not in results:  # a profiling run of one variant: no comparison line
        rr = results[precs[0]]
        if rank == 0:
            print(json.dumps({"variant": precs[0], "ms_per_step": rr["ms"] / a.steps, "kernels_ms": rr["kernels"],
                              "krylov_iterations": rr["iters"], "gpu_launches": gpu_launches[precs[0]]}), flush=True)
        if dist is not None:
            dist.destroy_process_group()
        return
    gf = C.c_double()
    lib.asam_probe_fp64_fma(20000, C.byref(gf))
    peaks = {}
    pk = ROOT / "MEASURED_PEAKS.json"
    if pk.exists():
        peaks = json.loads(pk.read_text())
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    r64 = results["fp64"]
    ms_step = r64["ms"] / a.steps
    value = aggregate_rate(world, ncell, a.steps, r64["ms"])
    e2e = aggregate_rate(world, ncell, a.steps, r64["ms_e2e"])
    npad = (a.nx + 2) * (a.ny + 2) * (a.nz + 2)
    nsweep = 6
    # dominant kernel of the FP64 step: the Gauss-Seidel wavefront (one PSolve call =
    # nlev + 10 launches of k_gs_pipe); algorithmic bytes per padded cell and sweep:
    # the 8 matrix slots (64 B) + b, x_old and x_new of every component (24 B each)
    gs_bytes = npad * nsweep * (64 + 24 * ncomp)
    # FP64 instructions per cell, component and sweep: 6 products + 6 differences
    # (upper and lower part) + 3 for the corrected division
    gs_dp = npad * nsweep * ncomp * 15
    ps_s = r64["kernels"]["psolve_ms"] * 1e-3
    gs_gbs = gs_bytes / ps_s / 1e9
    fp64_peak_inst = gf.value / 2.0  # DFMA instructions per ns = GFLOP/s / 2
    flux_bytes = ncell * BYTES_PER_CELL_FLUX(ncomp)
    flux_gbs = flux_bytes / (r64["kernels"]["flux_rhs_ms"] * 1e-3) / 1e9
    nbytes_state = st.c.size * 8
    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded cut-cell generators)", "config": workload_config(a),
        "e2e": {"value": e2e, "unit": METRIC, "h2d_bytes_per_step": nbytes_state, "d2h_bytes_per_step": nbytes_state},
        "roofline": {"kernel": "k_gs_pipe (one PSolve: 1+IterG Gauss-Seidel sweeps)", "bound": "hbm",
                     "achieved": gs_gbs, "peak": hbm_peak, "unit": "GB/s", "frac": gs_gbs / hbm_peak,
                     "traffic": TRAFFIC_PSOLVE_FP64_PER_PCELL * npad if ncomp == 10 else None,
                     "traffic_source": "ncu dram__bytes_read.sum+dram__bytes_write.sum of one PSolve at 256x256x64, "
                                       "scaled by padded cells (profiles/traffic_psolve_256x256x64.md)",
                     "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)",
                     "algorithmic_bytes_per_call": gs_bytes,
                     "fp64_pipe": {"achieved_ginst_s": gs_dp / ps_s / 1e9, "peak_ginst_s": fp64_peak_inst,
                                   "frac": gs_dp / ps_s / 1e9 / fp64_peak_inst,
                                   "peak_source": "asam_probe_fp64_fma (measured live)"},
                     "note": "FP64 kernels on GB300 are bounded by the FP64 pipe (ridge 0.16 flop/B)"},
        "flux_roofline": {"achieved": flux_gbs, "unit": "GB/s", "frac": flux_gbs / hbm_peak,
                          "algorithmic_bytes_per_call": flux_bytes},
        "fp64_fma_peak_gflops_probe": gf.value,
        "kernels_ms": r64["kernels"],
        "krylov_iterations": r64["iters"],
        "solver_settings": r64["tuned"],
        "clocks": r64["clocks"],
        "gpu_launches": gpu_launches["fp64"],
    }
    if "fp32_refined" in results:
        rr = results["fp32_refined"]
        ref = r64["final"].reshape(st.c.shape)
        got = rr["final"].reshape(st.c.shape)
        errs = []
        for i in range(ncomp):
            den = max(float(np.abs(ref[i]).max()), 1e-300)
            d = np.abs(got[i] - ref[i])
            errs.append({"field": st.names[i], "max_rel": float(d.max() / den),
                         "rms_rel": float(np.sqrt(np.mean(d ** 2)) / den)})
        # dominant kernel of the refined step: the FP32 Gauss-Seidel wavefront; algorithmic
        # bytes per padded cell and sweep: the 8 matrix slots (32 B) + b, x_old, x_new of
        # every component (12 B each); the timed call adds two conversion passes
        # (FP64 in -> FP32 -> FP64 out: 20 B per value), counted too
        inner = (rr["tuned"] or {}).get("inner_precond", a.inner)
        if inner == "gauss_seidel":
            nsw32 = 1 + (rr["tuned"] or {}).get("inner_gs_iter", a.inner_gs_iter)
            gs32_bytes = npad * nsw32 * (32 + 12 * ncomp) + npad * ncomp * 2 * 12
            kname = (f"k_gs_persist<float> (one FP32 inner PSolve: {nsw32} sweeps, persistent tile schedule, "
                     "with its FP64<->FP32 conversions)")
        else:
            # line solve of one call: the per-matrix factors (sub-diagonal, 1/den, w: 12 B per cell), per
            # component b in, g out and back, x out (16 B), PSolve's copy of the input (8 B), and the two
            # conversion passes of the call (FP64 -> FP32 in, FP32 -> FP64 out: 12 B per value each)
            gs32_bytes = npad * (12 + ncomp * (16 + 8 + 24))
            kname = (f"{'k_xline_solve' if inner == 'xline' else 'k_line_psolve'}<float> (one FP32 inner PSolve: "
                     f"{inner} Thomas, with its copy and FP64<->FP32 conversions)")
        gs32_s = rr["kernels"]["inner_psolve_ms"] * 1e-3
        line["roofline_refined"] = {
            "kernel": kname, "bound": "hbm",
            "achieved": gs32_bytes / gs32_s / 1e9, "peak": hbm_peak, "unit": "GB/s",
            "frac": gs32_bytes / gs32_s / 1e9 / hbm_peak,
            "traffic": TRAFFIC_PSOLVE_XLINE_PER_PCELL * npad if (inner == "xline" and ncomp == 10) else None,
            "traffic_source": "ncu dram__bytes_read.sum+dram__bytes_write.sum of one x-line inner PSolve at "
                              "256x256x64, scaled by padded cells (profiles/traffic_psolve_256x256x64.md)",
            "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)", "algorithmic_bytes_per_call": gs32_bytes}
        line["fp32_refined"] = {"value": world * ncell * a.steps / (rr["ms"] * 1e-3) / 1e6,
                                "ms_per_step": rr["ms"] / a.steps,
                                "speedup_vs_fp64": r64["ms"] / rr["ms"],
                                "max_rel_err_vs_fp64": max(e["max_rel"] for e in errs), "fields": errs,
                                "inner_solver": rr["tuned"] or {"inner_precond": a.inner,
                                                                "inner_gs_iter": a.inner_gs_iter},
                                "krylov_iterations": rr["iters"], "kernels_ms": rr["kernels"],
                                "gpu_launches": gpu_launches["fp32_refined"],
                                "clocks": rr["clocks"]}
    if adj is not None:
        line["adjoint"] = adj
    if bat is not None:
        line["batch"] = bat
    if proj is not None:
        line["projection"] = proj
    if dyn is not None:
        line["dyn"] = dyn
    if diff is not None:
        line["diffusion"] = diff
    if rst is not None:
        line["restart"] = rst
    if cpu is not None:
        line["cpu_baseline"] = cpu
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
