"""Benchmark of the GB300 implicit Rosenbrock stage of ASAM.

Headline workload: one full Rosenbrock step of the dynamical core
(asam_ros_step_dyn) on the 512x512x128 cut-cell configuration of the mixed
precision comparison -- periodic in x and y, rigid bottom and lid, Gaussian
hill h=1 km, half-width 5 km, Gaussian-correlated roughness (sigma 50 m,
2 km), dx=dy=200 m, dz 50->400 m, snapping + small-cell merge (the faces of
zero-volume cells closed), N=0.01 1/s, u=10 m/s, moist, one tracer; 10 cell
components (Rho, six LR momentum components, Rho*theta, Rho*qv, Rho*tracer);
RosRK3 (3 stages), dt = 2 s, BiCGStab and FGMRES tolerances 1e-10 (the
Krylov tolerance of the configurations).  Seeded synthetic fields stand in
for the reference's (unpublished) decks.

One step = one Ros3MetC call with prognostic momentum: per stage
ExchangeCell, face->cell velocities, the wall rules, thermodynamics, (stage 1)
the 7-diagonal Jacobian and the pressure-Laplacian hierarchies, FcnMet with
pressure gradient and buoyancy, the stage combination, the transport
BiCGStab, cell->face velocities, ProjectVelFace (FGMRES(10) on the
PressureVelocity system with the boundary face unknowns of the periodic
sides, PSolve1 = multigrid PressurePre, SchurPreFull, PressurePre), the
face-velocity and state updates.  Metric: Mcell-steps/s (interior cells x
steps / s).

Arms:
  (default)          ours: the FP64 drop-in step (value, e2e), the
                     FP32-refined step with its per-field error against the
                     FP64 run, the transport-only step (prescribed winds) with
                     its roofline, the adjoint cost (128x128x64 hill, 40
                     steps), the 48-domain batched ensemble, the diffusion
                     cost and the restart-file throughput
  --impl reference   the reference's CPU path (the oracle restatement of the
                     Fortran; the Fortran itself has no compiler here), the
                     same step on bounded samples of the same generator, one
                     process per host core on independent blocks.
"""
from __future__ import annotations

import argparse
import copy
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
BYTES_PER_CELL_FLUX = lambda ncomp: 64 + 16 * ncomp  # noqa: E731  algorithmic bytes per interior cell


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--nx", type=int, default=512)
    p.add_argument("--ny", type=int, default=512)
    p.add_argument("--nz", type=int, default=128)
    p.add_argument("--dt", type=float, default=2.0)
    p.add_argument("--tol", type=float, default=1e-10, help="BiCGStab tolerance")
    p.add_argument("--proj-tol", type=float, default=1e-10, help="FGMRES tolerance of the projection")
    p.add_argument("--seed", type=int, default=3, help="seed of the headline workload's generator")
    p.add_argument("--no-refined", action="store_true")
    p.add_argument("--no-transport", action="store_true", help="skip the transport-only step")
    p.add_argument("--no-adjoint", action="store_true")
    p.add_argument("--no-batch", action="store_true")
    p.add_argument("--no-diffusion", action="store_true", help="skip the diffusion cost")
    p.add_argument("--no-restart", action="store_true", help="skip the restart-file throughput")
    p.add_argument("--restart-only", action="store_true", help="only the restart section; prints its JSON object")
    p.add_argument("--diffusion-only", action="store_true",
                   help="only the diffusion section; prints its JSON object")
    p.add_argument("--transport-only", action="store_true",
                   help="only the transport-only step (prescribed winds); prints its JSON object")
    p.add_argument("--probe", choices=["psolve", "inner_psolve", "vcycle", "vcycle_refined", "step", "step_refined",
                                       "fp64_chain"],
                   help="for profiling: one transport PSolve call on the transport workload (psolve, "
                        "inner_psolve); one FGMRES preconditioner call on the headline block (vcycle: the FP64 "
                        "V-cycle; vcycle_refined: the refined mode's FP32 periodic-Laplacian V-cycle); or "
                        "--warmup + --steps bare dynamical steps of the headline workload (step, step_refined); "
                        "cycles per dependent FP64 FMA against active lanes and warps on one SM (fp64_chain)")
    p.add_argument("--batch-members", type=int, default=48)
    p.add_argument("--batch-steps", type=int, default=20)
    p.add_argument("--batch-threads", type=int, default=0, help="host threads driving the members (0: one each)")
    p.add_argument("--adj-grid", default="128,128,64", help="nx,ny,nz of the adjoint-cost workload")
    p.add_argument("--adj-steps", type=int, default=40)
    p.add_argument("--adj-ckpt", type=int, default=8)
    p.add_argument("--gauss-iter2", type=int, default=1, help="GaussIter2 of the projection multigrid")
    p.add_argument("--gauss-iter3", type=int, default=1, help="GaussIter3 of the projection multigrid")
    p.add_argument("--accuracy", action="store_true",
                   help="only the accuracy study of the refined step (FP64 and refined at the configured and at a "
                        "tight tolerance); prints its JSON object")
    p.add_argument("--accuracy-steps", type=int, default=5)
    p.add_argument("--tight-tol", type=float, default=1e-13, help="Krylov tolerance of the tight runs")
    p.add_argument("--no-tight", action="store_true", help="accuracy study without the tight-tolerance runs")
    p.add_argument("--batch-only", action="store_true", help="only the ensemble section; prints its JSON object")
    p.add_argument("--no-column", action="store_true", help="skip the column-solve line")
    p.add_argument("--column-only", action="store_true", help="only the column-solve line; prints its JSON object")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--cpu-sample", type=int, default=32, help="edge of the oracle's CPU sample window")
    p.add_argument("--no-autotune", action="store_true", help="keep --inner/--inner-gs-iter instead of autotuning")
    p.add_argument("--inner", default="gauss_seidel", choices=["gauss_seidel", "line", "xline", "yline"],
                   help="inner preconditioner of the refined transport-only step")
    p.add_argument("--inner-gs-iter", type=int, default=1,
                   help="Gauss-Seidel sweeps after the first of the refined mode's inner preconditioner")
    return p.parse_args()


def workload(nx, ny, nz, seed=2):
    """Transport-only workload (prescribed steady winds): hill_case."""
    from asam_gb300 import geometry as G

    return G.hill_case(nx, ny, nz, seed=seed)


def dyn_workload(nx, ny, nz, seed=3):
    """Headline workload: the periodic cut-cell hill with prognostic momentum."""
    from asam_gb300 import geometry as G

    return G.hill_dyn_case(nx, ny, nz, seed=seed)


def dyn_config(a):
    npad = (a.nx + 2) * (a.ny + 2) * (a.nz + 2)
    return {"workload": f"full Rosenbrock step with prognostic momentum and pressure projection, cut-cell Gaussian "
                        f"hill {a.nx}x{a.ny}x{a.nz} periodic in x/y (h=1 km, half-width 5 km, roughness 50 m / "
                        f"2 km, dx=dy=200 m, dz 50->400 m), N=0.01 1/s, u=10 m/s, moist, tracer, 10 components, "
                        f"RosRK3 dt={a.dt}s, BiCGStab tol {a.tol:g} (6-sweep Gauss-Seidel), FGMRES(10) tol "
                        f"{a.proj_tol:g} (multigrid PSolve1 with the Schur step of the periodic sides)",
            "nx": a.nx, "ny": a.ny, "nz": a.nz, "ncomp": 10, "method": "RosRK3", "dt": a.dt,
            "bicgstab_tol": a.tol, "fgmres_tol": a.proj_tol, "seed": a.seed,
            "l2": f"inputs larger than L2 (state {10 * 8 * npad / 1e9:.2f} GB, transport matrix "
                  f"{8 * 8 * npad / 1e9:.2f} GB, Laplacian hierarchies ~{2 * 11 * 8 * 1.45 * npad / 1e9:.0f} GB)",
            "parallelism": "replicas" if a.gpus > 1 else "single GPU"}


def _dyn_kinds(ncomp, mom):
    """Free-slip walls: the momentum component normal to a wall is ZeroValue
    there, everything else ZeroGrad (periodic sides have no halo rule)."""
    k = [[1] * 6 for _ in range(ncomp)]
    for q, p in enumerate(mom):
        for sd in range(6):
            k[p][sd] = 2 if q // 2 == sd // 2 else 1
    return k


# ---------------------------------------------------------------------------
# CPU baseline (oracle restatement of the reference Fortran), one block per process
# ---------------------------------------------------------------------------
def _cpu_worker(args):
    """One block of the headline generator advanced `steps` full Rosenbrock
    steps by the oracle (reference lexicographic smoother)."""
    edge, nz, dt, tol, ptol, steps, seed = args
    import oracle
    from asam_gb300 import geometry as G

    geo, vel, st, pos, (dx, dy, dz), bc = dyn_workload(edge, edge, nz, seed=seed)
    o = oracle.Oracle(geo, bc=_dyn_kinds(st.c.shape[0], pos["mom"]))
    op = oracle.OracleProj(geo, dx, dy, dz, G.projection_inputs(geo)[0], zebra=0)
    c = st.c.copy()
    u = [q.copy() for q in vel]
    t0 = time.perf_counter()
    for _ in range(steps):
        o.ros_step_dyn(op, c, u, dt, rho_pos=0, th_pos=pos["th"], pos=pos["mom"], dx=dx, dy=dy, dz=dz,
                       rv_pos=pos["qv"], bound=bc, scalars=[pos["qv"], pos["tracer"]], bicg_tol=tol, proj_tol=ptol,
                       proj_maxiter=20)
    wall = time.perf_counter() - t0
    op.close()
    return wall, edge * edge * nz * steps


def cpu_baseline(edge, nz, dt, tol, ptol, steps, procs):
    ctx = mp.get_context("spawn")
    jobs = [(edge, nz, dt, tol, ptol, steps, 3 + i) for i in range(procs)]
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
    """--impl reference: the reference's CPU path (oracle port of the Fortran)
    on all host cores: one process per core, each advancing an independent
    block of the headline generator (the reference's MPI-over-blocks model)."""
    if rank != 0:
        return
    procs = os.cpu_count() or 1
    edge = max(8, a.cpu_sample)
    value, wall = cpu_baseline(edge, a.nz, a.dt, a.tol, a.proj_tol, a.steps, procs)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": a.gpus,
            "steps": a.steps, "warmup": a.warmup, "ms_per_step": None, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded generators)",
            "config": dyn_config(a),
            "cpu_baseline": {"value": value, "unit": METRIC, "cores": procs, "kind": "port",
                             "sample": f"{procs} independent {edge}x{edge}x{a.nz} blocks of the same generator, "
                                       f"{a.steps} full Rosenbrock steps each (MPI-over-blocks model), oracle "
                                       f"restatement of the Fortran with its lexicographic smoother, "
                                       f"{cpu_model()}, {wall:.0f} s"},
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


def column_bench(a, torch, stream, hbm_peak):
    """The batched vertical-column Thomas solve (Solve_1D) through the
    allocation-free entry: 32768 columns of 128 levels (4.19 M unknowns, the
    entry's maximum), device-resident, diagonally dominant seeded systems.
    Algorithmic bytes: d, u, l, b read and x written, 40 B per unknown (168 MB
    per call, above the L2 size)."""
    import ctypes as C

    from asam_gb300 import _lib

    lib = _lib.load()
    ncol, n1 = 32768, 128
    gen = torch.Generator(device="cpu").manual_seed(11)
    d = (3.0 + 0.5 * torch.rand(ncol * n1, generator=gen, dtype=torch.float64)).cuda()
    u = (2.0 * torch.rand(ncol * (n1 - 1), generator=gen, dtype=torch.float64) - 1.0).cuda()
    lo = (2.0 * torch.rand(ncol * (n1 - 1), generator=gen, dtype=torch.float64) - 1.0).cuda()
    b = torch.randn(ncol * n1, generator=gen, dtype=torch.float64).cuda()
    P = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
    sp = C.c_void_p(stream.cuda_stream)

    def solve():
        _lib.check(lib.asam_tri_solve_noalloc(ncol, n1, P(d), P(u), P(lo), P(b), sp), "asam_tri_solve_noalloc")

    for _ in range(3):
        solve()
    n = 20
    ms = time_region(torch, stream, solve, n) / n
    nbytes = 40 * ncol * n1
    gbs = nbytes / (ms * 1e-3) / 1e9
    return {"workload": f"{ncol} columns x {n1} levels, FP64, device-resident (asam_tri_solve_noalloc)",
            "ms_per_call": ms, "algorithmic_bytes_per_call": nbytes, "achieved_gbs": gbs,
            "hbm_frac": gbs / hbm_peak, "munknowns_per_s": ncol * n1 / (ms * 1e-3) / 1e6}


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
    in one asam_batch_ros_step call, device-resident states; FP64 and refined,
    each with host threads driving the members and as one graph launch of
    the whole run (`one_graph`)."""
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
        graph = None
        with asam_gb300.Batch(blocks, nthreads=a.batch_threads) as batch:
            batch.ros_step(ptrs, 2.0, nsteps=1)  # warm-up
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            its, status = batch.ros_step(ptrs, 2.0, nsteps=a.batch_steps)
            torch.cuda.synchronize()
            wall = time.perf_counter() - t0
            # the whole run of every member as one graph launch: recorded by a
            # first call of the same length, replayed by the timed one
            batch.set_graph(True)
            t0 = time.perf_counter()
            batch.ros_step(ptrs, 2.0, nsteps=a.batch_steps)
            torch.cuda.synchronize()
            t_rec = time.perf_counter() - t0
            t0 = time.perf_counter()
            _, gstatus = batch.ros_step(ptrs, 2.0, nsteps=a.batch_steps)
            torch.cuda.synchronize()
            gwall = time.perf_counter() - t0
            batch.set_graph(False)
            graph = {"value": cells * a.batch_steps / gwall / 1e6, "unit": METRIC, "seconds": gwall,
                     "launches_per_call": 1, "record_and_first_run_seconds": t_rec,
                     "members_not_ok": int((gstatus != 0).sum())}
        for b in blocks:
            b.close()
        del dev
        torch.cuda.empty_cache()
        res[prec] = {"value": cells * a.batch_steps / wall / 1e6, "unit": METRIC, "seconds": wall,
                     "members_not_ok": int((status != 0).sum())}
        if graph is not None:
            res[prec]["one_graph"] = graph
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


def dyn_measure(a, torch, stream, prec, work, lib_mod, e2e=True, kernels=True, clocks=True):
    """Warm-up and timed Rosenbrock steps of the dynamical core in one
    precision: device-resident state and face velocities (value), then the
    same call with the state and the face velocities in pinned host memory,
    copied in and out every step (e2e)."""
    import ctypes as C

    import numpy as np

    import asam_gb300

    _lib = lib_mod
    geo, vel, st, pos, (dx, dy, dz), bc = work
    nc = st.c.shape[0]
    kw = {"inner_precond": "xline"} if prec == "fp32_refined" else {}
    blk = asam_gb300.TransportBlock(geo, nc, rho_pos=0, method="RosRK3", bicgstab_tol=a.tol, bicgstab_maxiter=30,
                                    precision=prec, **kw)
    blk.set_stream(stream.cuda_stream)
    blk.set_velocity(*vel)
    blk.proj_setup(dx, dy, dz, tol=a.proj_tol, max_restart=20, gauss_iter2=a.gauss_iter2, gauss_iter3=a.gauss_iter3)
    blk.dyn_setup(pos["th"], pos["mom"], rv_pos=pos["qv"], bound_cells=bc, scalars=[pos["qv"], pos["tracer"]])
    lib = blk.lib
    c = torch.from_numpy(st.c.reshape(-1).copy()).cuda()
    P = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
    it, rs, ps, pr = (C.c_int * 4)(), (C.c_double * 4)(), (C.c_int * 4)(), (C.c_double * 4)()
    iters = []

    def step():
        _lib.check(lib.asam_ros_step_dyn(blk.h, P(c), a.dt, it, rs, ps, pr), "asam_ros_step_dyn", allow=(0, 1, 2))
        iters.append({"bicgstab": list(it[:3]), "fgmres": list(ps[:3])})

    for _ in range(a.warmup):
        step()
    iters.clear()
    torch.cuda.synchronize()
    l0, v0 = lib.asam_launch_count(), lib.asam_proj_vcycles(blk.h)
    if clocks:
        with ClockSampler(0) as clk:
            ms = time_region(torch, stream, step, a.steps)
        clk_sum = clk.summary()
    else:
        ms = time_region(torch, stream, step, a.steps)
        clk_sum = None
    launches = lib.asam_launch_count() - l0
    vcycles = (lib.asam_proj_vcycles(blk.h) - v0) / a.steps
    final = c.cpu().numpy().reshape(st.c.shape).copy()
    out = {"ms": ms, "final": final, "iters": iters[:], "launches": launches, "vcycles_per_step": vcycles,
           "clocks": clk_sum}
    if e2e:
        # the reference's caller owns the state and VelF: both cross the boundary every step
        hc = torch.from_numpy(final.reshape(-1).copy()).pin_memory()
        g = geo.grid
        hv = [torch.empty(n, dtype=torch.float64).pin_memory() for n in
              ((g.nx + 1) * g.ny * g.nz, g.nx * (g.ny + 1) * g.nz, g.nx * g.ny * (g.nz + 1))]
        blk_vel = [q.numpy() for q in hv]
        _lib.check(lib.asam_get_velocity(blk.h, *[P(q) for q in hv]), "asam_get_velocity")

        def step_e2e():
            _lib.check(lib.asam_set_velocity(blk.h, *[P(q) for q in hv]), "asam_set_velocity")
            _lib.check(lib.asam_ros_step_dyn(blk.h, P(hc), a.dt, it, rs, ps, pr), "asam_ros_step_dyn",
                       allow=(0, 1, 2))
            _lib.check(lib.asam_get_velocity(blk.h, *[P(q) for q in hv]), "asam_get_velocity")

        torch.cuda.synchronize()
        t0 = time.perf_counter()
        # at most two steps: the FP64 step takes seconds, and the host copies
        # add the same time to every step
        ne = min(a.steps, 2)
        ms_e2e = time_region(torch, stream, step_e2e, ne)
        ms_e2e = max(ms_e2e, (time.perf_counter() - t0) * 1e3)
        out["ms_e2e"] = ms_e2e
        out["e2e_steps"] = ne
        out["e2e_bytes"] = st.c.size * 8 + sum(q.numel() for q in hv) * 8
        del blk_vel
    if kernels:
        g = geo.grid
        kt = {}
        bb = torch.randn(g.nz, g.ny, g.nx, dtype=torch.float64, device="cuda")
        xx = torch.zeros_like(bb)
        kt["vcycle_ms"] = time_region(torch, stream, lambda: lib.asam_lapl_vcycle(blk.h, P(bb), P(xx)), 3) / 3
        # a refined context of a periodic block preconditions with the periodic
        # Laplacian and assembles no Dirichlet hierarchy
        if lib.asam_lapl_vcycle_dirichlet(blk.h, P(bb), P(xx)) == 0:
            kt["vcycle_dirichlet_ms"] = time_region(
                torch, stream, lambda: lib.asam_lapl_vcycle_dirichlet(blk.h, P(bb), P(xx)), 3) / 3
            pre_key = "psolve1_ms"
        else:
            pre_key = "periodic_laplacian_pre_ms"
        xv = torch.randn(g.nx * g.ny * g.nz + blk.proj_nface, dtype=torch.float64, device="cuda")
        yv = torch.zeros_like(xv)
        kt[pre_key] = time_region(torch, stream, lambda: lib.asam_proj_psolve1(blk.h, P(xv), P(yv)), 3) / 3
        kt["matvec1_ms"] = time_region(torch, stream, lambda: lib.asam_proj_matvec1(blk.h, P(xv), P(yv)), 3) / 3
        f = torch.empty_like(c)
        kt["flux_rhs_ms"] = time_region(torch, stream, lambda: lib.asam_fcn(blk.h, P(c), P(f)), 3) / 3
        out["kernels"] = kt
    blk.close()
    del c
    torch.cuda.empty_cache()
    return out


def probe_dyn(a, torch, stream):
    """Profiling probes on the headline workload.  vcycle: the projection of
    the headline block assembled once (seeded sound weights), then exactly one
    FP64 V-cycle on the Neumann hierarchy (asam_lapl_vcycle, the bench's
    roofline kernel); vcycle_refined: the refined context's FGMRES
    preconditioner once (one FP32 V-cycle on the periodic Laplacian and the
    face elimination around it).  The V-cycle kernels (k_plane_half,
    k_matvec3, k_restrict3, k_prolong3) run nowhere else in the process, so a
    capture filtered to them covers exactly one V-cycle.  step / step_refined:
    --warmup then --steps bare dynamical steps, CUDA-event timed."""
    import ctypes as C

    import asam_gb300
    from asam_gb300 import _lib
    from asam_gb300 import geometry as G

    refined = a.probe.endswith("_refined")
    prec = "fp32_refined" if refined else "fp64"
    if a.probe.startswith("step"):
        r = dyn_measure(a, torch, stream, prec, dyn_workload(a.nx, a.ny, a.nz, seed=a.seed), _lib, e2e=False,
                        kernels=False, clocks=False)
        return {"probe": a.probe, "nx": a.nx, "ny": a.ny, "nz": a.nz, "ms_per_step": r["ms"] / a.steps,
                "launches_per_step": r["launches"] / a.steps, "vcycles_per_step": r["vcycles_per_step"],
                "krylov_iterations": r["iters"]}
    geo = G.hill_dyn_case(a.nx, a.ny, a.nz, seed=a.seed)[0]
    W, dx, dy, dz, _ = G.projection_inputs(geo)
    blk = asam_gb300.TransportBlock(geo, 3, rho_pos=0, precision=prec)
    blk.set_stream(stream.cuda_stream)
    blk.proj_setup(dx, dy, dz, tol=a.proj_tol, max_restart=20)
    blk.proj_weights(*W)
    blk.JacAccGrav(0.435866521508459, a.dt)
    lib = blk.lib
    P = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
    g = geo.grid
    nc = g.nx * g.ny * g.nz
    xv = torch.randn(nc + blk.proj_nface, dtype=torch.float64, device="cuda")
    yv = torch.zeros_like(xv)
    torch.cuda.synchronize()
    n0, v0 = lib.asam_launch_count(), lib.asam_proj_vcycles(blk.h)
    if refined:
        ms = time_region(torch, stream, lambda: _lib.check(lib.asam_proj_psolve1(blk.h, P(xv), P(yv)),
                                                           "asam_proj_psolve1"), 1)
    else:
        ms = time_region(torch, stream, lambda: _lib.check(lib.asam_lapl_vcycle(blk.h, P(xv[:nc]), P(yv[:nc])),
                                                           "asam_lapl_vcycle"), 1)
    out = {"probe": a.probe, "nx": a.nx, "ny": a.ny, "nz": a.nz, "ms": ms,
           "launches": lib.asam_launch_count() - n0, "vcycles": lib.asam_proj_vcycles(blk.h) - v0,
           "vcycle_bytes": vcycle_bytes(a.nz, a.nx, a.ny, 4)}
    blk.close()
    return out


def field_errors(names, got, ref, mom=()):
    """Per-field max and RMS error relative to the field's largest magnitude;
    the momentum components (indices mom) also relative to the largest
    momentum component ("max_rel_vec": they are the components of one vector,
    and the cross-wind component of a flow along x is nearly zero)."""
    import numpy as np

    vscale = max((float(np.abs(ref[q]).max()) for q in mom), default=0.0)
    out = []
    for i, nm in enumerate(names):
        den = max(float(np.abs(ref[i]).max()), 1e-300)
        d = np.abs(got[i] - ref[i])
        e = {"field": nm, "max_rel": float(d.max() / den), "rms_rel": float(np.sqrt(np.mean(d ** 2)) / den)}
        e["max_rel_vec"] = float(d.max() / max(vscale, 1e-300)) if i in mom else e["max_rel"]
        out.append(e)
    return out


def accuracy_study(a, torch, stream, work, lib_mod):
    """The error of the FP32-refined dynamical step split into Krylov
    truncation and arithmetic: the plain FP64 step and the refined step at the
    configured tolerances, and both again at a tight tolerance, each run for
    the same number of steps from the same state.  Pairs: refined vs FP64 (as
    configured), each of them vs the tight FP64 run (how far each is from the
    converged solution), and tight refined vs tight FP64 (the arithmetic
    alone)."""
    names, mom = work[2].names, work[3]["mom"]
    runs = {}
    kinds = [("fp64", "fp64", False), ("refined", "fp32_refined", False)]
    if not a.no_tight:
        kinds += [("fp64_tight", "fp64", True), ("refined_tight", "fp32_refined", True)]
    for key, prec, tight in kinds:
        b = copy.copy(a)
        b.warmup, b.steps = 0, a.accuracy_steps
        if tight:
            b.tol = b.proj_tol = a.tight_tol
        r = dyn_measure(b, torch, stream, prec, work, lib_mod, e2e=False, kernels=False, clocks=False)
        runs[key] = {"final": r["final"], "ms_per_step": r["ms"] / b.steps, "krylov_iterations": r["iters"],
                     "vcycles_per_step": r["vcycles_per_step"], "bicgstab_tol": b.tol, "fgmres_tol": b.proj_tol}
    out = {"steps": a.accuracy_steps, "runs": {k: {q: v for q, v in r.items() if q != "final"}
                                               for k, r in runs.items()}, "pairs": {}}
    for got, ref in (("refined", "fp64"), ("fp64", "fp64_tight"), ("refined", "fp64_tight"),
                     ("refined_tight", "fp64_tight")):
        if got not in runs or ref not in runs:
            continue
        errs = field_errors(names, runs[got]["final"], runs[ref]["final"], mom)
        out["pairs"][f"{got}_vs_{ref}"] = {
            "max_rel": max(e["max_rel"] for e in errs), "max_rel_state": max(e["max_rel_vec"] for e in errs),
            "max_rms_rel": max(e["rms_rel"] for e in errs),
            "fields": [[e["field"], float(f"{e['max_rel']:.3g}"), float(f"{e['rms_rel']:.3g}"),
                        float(f"{e['max_rel_vec']:.3g}")] for e in errs]}
    return out


def transport_bench(a, torch, stream, hbm_peak, fp64_inst_peak):
    """The transport-only Rosenbrock step (prescribed steady winds, no
    projection) on the 512x512x128 hill of hill_case (seed 2): FP64 drop-in
    and autotuned FP32-refined, with the roofline of the dominant kernels."""
    import ctypes as C

    import numpy as np

    import asam_gb300
    from asam_gb300 import _lib

    lib = _lib.load()
    geo, vel, st = workload(a.nx, a.ny, a.nz)
    ncomp = st.c.shape[0]
    ncell = a.nx * a.ny * a.nz
    npad = (a.nx + 2) * (a.ny + 2) * (a.nz + 2)
    res = {}
    for prec in ("fp64", "fp32_refined"):
        blk = asam_gb300.TransportBlock(geo, ncomp, method="RosRK3", bicgstab_tol=a.tol, bicgstab_maxiter=30,
                                        precision=prec, inner_precond=a.inner, inner_gs_iter=a.inner_gs_iter)
        blk.set_velocity(*vel)
        blk.set_stream(stream.cuda_stream)
        tuned = None
        if not a.no_autotune:
            t0 = time.perf_counter()
            tuned = blk.autotune(st.c, a.dt)
            tuned["tuning_seconds"] = time.perf_counter() - t0
        dstate = torch.from_numpy(st.c.reshape(-1).copy()).cuda()
        dp = C.c_void_p(dstate.data_ptr())
        iters_all = []

        def step():
            iters = (C.c_int * 4)()
            resid = (C.c_double * 4)()
            _lib.check(lib.asam_ros_step(blk.h, dp, a.dt, iters, resid), "asam_ros_step", allow=(0, 1, 2))
            iters_all.append([iters[i] for i in range(blk.nstage)])

        for _ in range(a.warmup):
            step()
        iters_all.clear()
        ms = time_region(torch, stream, step, a.steps)
        final = dstate.cpu().numpy().copy()
        f_out = torch.empty_like(dstate)
        kt = {}
        nrep = 5
        kt["flux_rhs_ms"] = time_region(torch, stream, lambda: _lib.check(
            lib.asam_fcn(blk.h, dp, C.c_void_p(f_out.data_ptr())), "asam_fcn"), nrep) / nrep
        kt["psolve_ms"] = time_region(torch, stream, lambda: _lib.check(
            lib.asam_psolve(blk.h, C.c_void_p(f_out.data_ptr()), dp), "asam_psolve"), nrep) / nrep
        dstate.copy_(torch.from_numpy(final.reshape(-1)))
        kt["matvec_ms"] = time_region(torch, stream, lambda: _lib.check(
            lib.asam_matvec(blk.h, dp, C.c_void_p(f_out.data_ptr())), "asam_matvec"), nrep) / nrep
        if prec == "fp32_refined":
            kt["inner_psolve_ms"] = time_region(torch, stream, lambda: _lib.check(
                lib.asam_inner_psolve(blk.h, dp, C.c_void_p(f_out.data_ptr())), "asam_inner_psolve"),
                nrep) / nrep
        res[prec] = {"ms": ms, "final": final, "iters": iters_all, "kernels": kt, "tuned": tuned}
        blk.close()
        del dstate, f_out
        torch.cuda.empty_cache()
    r64, rr = res["fp64"], res["fp32_refined"]
    nsweep = 6
    # the Gauss-Seidel wavefront of one PSolve call: 8 matrix slots (64 B) and b,
    # x_old, x_new of every component (24 B each) per padded cell and sweep
    gs_bytes = npad * nsweep * (64 + 24 * ncomp)
    gs_dp = npad * nsweep * ncomp * 15  # FP64 instructions per cell, component and sweep
    ps_s = r64["kernels"]["psolve_ms"] * 1e-3
    flux_bytes = ncell * BYTES_PER_CELL_FLUX(ncomp)
    ref = r64["final"].reshape(st.c.shape)
    got = rr["final"].reshape(st.c.shape)
    inner = (rr["tuned"] or {}).get("inner_precond", a.inner)
    if inner == "gauss_seidel":
        nsw32 = 1 + (rr["tuned"] or {}).get("inner_gs_iter", a.inner_gs_iter)
        b32 = npad * nsw32 * (32 + 12 * ncomp) + npad * ncomp * 2 * 12
    else:
        b32 = npad * (12 + ncomp * (16 + 8 + 24))
    s32 = rr["kernels"]["inner_psolve_ms"] * 1e-3
    return {
        "workload": f"transport-only step (prescribed steady winds, no projection), cut-cell Gaussian hill "
                    f"{a.nx}x{a.ny}x{a.nz} periodic in x/y, {ncomp} components, RosRK3 dt={a.dt}s, BiCGStab tol "
                    f"{a.tol:g}",
        "value": ncell * a.steps / (r64["ms"] * 1e-3) / 1e6, "unit": METRIC, "ms_per_step": r64["ms"] / a.steps,
        "krylov_iterations": r64["iters"], "kernels_ms": r64["kernels"],
        "roofline": {"kernel": "k_gs_pipe_reg (one PSolve: 1+IterG Gauss-Seidel sweeps)", "bound": "hbm",
                     "achieved": gs_bytes / ps_s / 1e9, "peak": hbm_peak, "unit": "GB/s",
                     "frac": gs_bytes / ps_s / 1e9 / hbm_peak, "traffic": None,
                     "algorithmic_bytes_per_call": gs_bytes,
                     "fp64_pipe": {"achieved_ginst_s": gs_dp / ps_s / 1e9, "peak_ginst_s": fp64_inst_peak,
                                   "frac": gs_dp / ps_s / 1e9 / fp64_inst_peak}},
        "flux_roofline": {"achieved": flux_bytes / (r64["kernels"]["flux_rhs_ms"] * 1e-3) / 1e9, "unit": "GB/s",
                          "frac": flux_bytes / (r64["kernels"]["flux_rhs_ms"] * 1e-3) / 1e9 / hbm_peak,
                          "algorithmic_bytes_per_call": flux_bytes},
        "fp32_refined": {"value": ncell * a.steps / (rr["ms"] * 1e-3) / 1e6, "ms_per_step": rr["ms"] / a.steps,
                         "speedup_vs_fp64": r64["ms"] / rr["ms"],
                         "max_rel_err_vs_fp64": max(e["max_rel"] for e in field_errors(st.names, got, ref)),
                         "inner_solver": rr["tuned"] or {"inner_precond": a.inner, "inner_gs_iter": a.inner_gs_iter},
                         "krylov_iterations": rr["iters"], "kernels_ms": rr["kernels"],
                         "roofline": {"kernel": f"one FP32 inner PSolve ({inner})", "bound": "hbm",
                                      "achieved": b32 / s32 / 1e9, "peak": hbm_peak, "unit": "GB/s",
                                      "frac": b32 / s32 / 1e9 / hbm_peak, "algorithmic_bytes_per_call": b32}},
    }


def main():
    a = parse()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if a.impl == "reference":
        run_reference(a, rank)
        return

    def peaks():
        pk = ROOT / "MEASURED_PEAKS.json"
        return json.loads(pk.read_text()) if pk.exists() else {}

    if (a.restart_only or a.diffusion_only or a.transport_only or a.probe or a.accuracy or a.column_only
            or a.batch_only):
        import ctypes as C

        import torch

        import __graft_entry__

        __graft_entry__.build()
        stream = torch.cuda.Stream()
        torch.cuda.set_stream(stream)
        if a.restart_only:
            print(json.dumps(restart_bench(a, torch)), flush=True)
        elif a.batch_only:
            print(json.dumps(batch_bench(a, torch, batch_members(a.batch_members))), flush=True)
        elif a.column_only:
            print(json.dumps(column_bench(a, torch, stream, peaks().get("hbm_gbs", 6800.0))), flush=True)
        elif a.accuracy:
            from asam_gb300 import _lib

            out = accuracy_study(a, torch, stream, dyn_workload(a.nx, a.ny, a.nz, seed=a.seed), _lib)
            out["config"] = dyn_config(a)
            print(json.dumps(out), flush=True)
        elif a.diffusion_only:
            print(json.dumps(diffusion_bench(a, torch, stream)), flush=True)
        elif a.transport_only:
            from asam_gb300 import _lib

            gf = C.c_double()
            _lib.load().asam_probe_fp64_fma(20000, C.byref(gf))
            tb = transport_bench(a, torch, stream, peaks().get("hbm_gbs", 6800.0), gf.value / 2.0)
            print(json.dumps(tb), flush=True)
        elif a.probe == "fp64_chain":
            from asam_gb300 import _lib

            lib, out = _lib.load(), []
            for warps, lanes in ((1, 1), (1, 8), (1, 32), (4, 4), (4, 32), (8, 32), (16, 32), (32, 1), (32, 32)):
                cyc = C.c_double()
                _lib.check(lib.asam_probe_fp64_chain(warps, lanes, 20000, C.byref(cyc)), "asam_probe_fp64_chain")
                out.append({"warps": warps, "lanes": lanes, "cycles_per_dependent_fma": cyc.value})
            print(json.dumps({"probe": a.probe, "results": out}), flush=True)
        elif a.probe in ("vcycle", "vcycle_refined", "step", "step_refined"):
            print(json.dumps(probe_dyn(a, torch, stream)), flush=True)
        else:
            import asam_gb300

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

    # CPU baseline first (before any GPU call), rank 0, N=1 only
    cpu = None
    if rank == 0 and world == 1 and not a.no_cpu_baseline:
        edge = a.cpu_sample
        value, wall = cpu_baseline(edge, a.nz, a.dt, a.tol, a.proj_tol, 1, 1)
        cpu = {"value": value, "unit": METRIC, "cores": 1, "kind": "port",
               "sample": f"one {edge}x{edge}x{a.nz} block of the same generator, 1 full Rosenbrock step, "
                         f"single-threaded oracle restatement of the Fortran ({wall:.1f} s), {cpu_model()}"}

    import ctypes as C

    import torch

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")

    import __graft_entry__

    __graft_entry__.build()
    from asam_gb300 import _lib

    lib = _lib.load()
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    work = dyn_workload(a.nx, a.ny, a.nz, seed=a.seed)
    names = work[2].names
    ncell = a.nx * a.ny * a.nz

    def barrier():
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()

    barrier()
    r64 = dyn_measure(a, torch, stream, "fp64", work, _lib)
    barrier()
    ms = reduce_max(dist, r64["ms"], "cuda")
    ms_e2e = reduce_max(dist, r64["ms_e2e"], "cuda")
    rr = None
    if not a.no_refined:
        rr = dyn_measure(a, torch, stream, "fp32_refined", work, _lib, e2e=False)
    gf = C.c_double()
    lib.asam_probe_fp64_fma(20000, C.byref(gf))
    pk = peaks()
    hbm_peak = pk.get("hbm_gbs", 6800.0)
    tb = None
    if not a.no_transport and world == 1:
        tb = transport_bench(a, torch, stream, hbm_peak, gf.value / 2.0)
    adj = None
    if not a.no_adjoint and world == 1:
        adj = adjoint_cost(a, lib, torch, stream)
    bat = None
    if not a.no_batch and world == 1:
        bat = batch_bench(a, torch, batch_members(a.batch_members))
    diff = None
    if not a.no_diffusion and world == 1:
        diff = diffusion_bench(a, torch, stream)
    rst = None
    if not a.no_restart and world == 1:
        rst = restart_bench(a, torch)
    col = None
    if not a.no_column and world == 1:
        col = column_bench(a, torch, stream, hbm_peak)

    # the dominant kernel of the step: the multigrid V-cycle (k_plane_half zebra
    # plane/line relaxations with the 3D residual, restriction and prolongation),
    # about 90 % of the FP64 step; algorithmic bytes counted from its schedule
    vb = vcycle_bytes(a.nz, a.nx, a.ny, 4)
    # DRAM bytes of one such V-cycle at 512x512x128 from one ncu capture of
    # `python bench.py --probe vcycle` (dram__bytes_read.sum +
    # dram__bytes_write.sum over its 91 launches; one pass, so taken at full
    # size); ncu cannot run inside the timed program
    traffic = 101.389e9 if (a.nx, a.ny, a.nz, a.seed) == (512, 512, 128, 3) else None
    vc_s = r64["kernels"]["vcycle_ms"] * 1e-3
    vgbs = vb / vc_s / 1e9
    line = {
        "metric": METRIC, "value": aggregate_rate(world, ncell, a.steps, ms), "unit": METRIC, "n_gpus": world,
        "steps": a.steps, "warmup": a.warmup, "ms_per_step": ms / a.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded cut-cell generators)",
        "config": dyn_config(a),
        "e2e": {"value": aggregate_rate(world, ncell, r64["e2e_steps"], ms_e2e), "unit": METRIC,
                "h2d_bytes_per_step": r64["e2e_bytes"], "d2h_bytes_per_step": r64["e2e_bytes"],
                "steps": r64["e2e_steps"]},
        "roofline": {"kernel": "one multigrid V-cycle (Solve_3D: k_plane_half zebra plane/x-line/z-column "
                               "relaxations, 3D residual, restriction, prolongation) on the Neumann hierarchy",
                     "bound": "hbm", "achieved": vgbs, "peak": hbm_peak, "unit": "GB/s", "frac": vgbs / hbm_peak,
                     "traffic": traffic, "algorithmic_bytes_per_call": vb,
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum over the 91 launches of one "
                                       "V-cycle of this workload (bench.py --probe vcycle), one pass",
                     "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)",
                     "vcycles_per_step": r64["vcycles_per_step"],
                     "share_of_step": r64["vcycles_per_step"] * r64["kernels"]["vcycle_ms"] / (ms / a.steps),
                     "note": "FP64 V-cycle: bounded by the FP64 pipe (GB300 ridge ~0.16 flop/B) and the serial "
                             "column recurrences of the coarse plane levels, see fp64_fma_peak_gflops_probe"},
        "fp64_fma_peak_gflops_probe": gf.value,
        "kernels_ms": r64["kernels"],
        "clocks": r64["clocks"],
        "gpu_launches": r64["launches"],
    }
    if cpu is not None:
        line["cpu_baseline"] = cpu
    if tb is not None:
        line["transport"] = tb
    if bat is not None:
        line["batch"] = bat
    if diff is not None:
        line["diffusion"] = diff
    if rst is not None:
        line["restart"] = rst
    if col is not None:
        line["column_solve"] = col
    if adj is not None:
        line["adjoint_detail"] = adj
    # the short keys last: the tail of the line carries the headline comparisons
    if adj is not None:
        line["adjoint"] = {k: adj[k] for k in ("gradient_over_forward", "tracer_and_wind_gradient_over_forward",
                                               "adjoint_step_over_forward_step", "forward_step_ms",
                                               "adjoint_step_ms")}
    if rr is not None:
        errs = field_errors(names, rr["final"], r64["final"], work[3]["mom"])
        line["fp32_refined"] = {
            "value": aggregate_rate(world, ncell, a.steps, rr["ms"]), "ms_per_step": rr["ms"] / a.steps,
            "speedup_vs_fp64": r64["ms"] / rr["ms"], "kernels_ms": rr["kernels"],
            "vcycles_per_step": rr["vcycles_per_step"], "gpu_launches": rr["launches"], "clocks": rr["clocks"],
            "krylov_iterations": rr["iters"],
            "preconditioner": "FGMRES(10) preconditioned by one FP32 V-cycle on the periodic Laplacian (face "
                              "unknowns eliminated, one sweep per level); transport BiCGStab in FP32 with the "
                              "x-line preconditioner inside FP64 refinement",
            "max_rel_err_vs_fp64": max(e["max_rel"] for e in errs),
            "max_rel_err_vs_fp64_state": max(e["max_rel_vec"] for e in errs),
            "error_note": "both runs stop their Krylov solves at a relative residual of the configured tolerance; "
                          "the difference is the FP64 run's own truncation error, which bench.py --accuracy "
                          "separates from the arithmetic by a run of both at a tight tolerance",
            "after_steps": a.warmup + a.steps,
            "fields": [[e["field"], float(f"{e['max_rel']:.3g}"), float(f"{e['rms_rel']:.3g}")] for e in errs]}
    line["krylov_iterations"] = r64["iters"]
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
