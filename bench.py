"""Benchmark of the turbulentBL time step on GB300.

Headline: grid-point-steps per second (Mpt-steps/s) of the plain FP64 method
on the 512 x 128 x 128 seeded box (nx x ny_wall x nz_span; reference arrays
n3d = (512, 130, 128)), GMRES restart 40, tol 1e-10, P = 8 virtual slabs.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
  python bench.py --adjoint [--window 50] [--ckpt 10] [--fd-dirs 4]

One "step" is one full time step of the reference time loop (inflow,
convection, implicit diffusion, pressure-Poisson GMRES, projection, BCs,
statistics and the every-cum rescaling).  Fields are 68-400 MB each, far above
the 129 MB L2, so no cache flush is needed between steps.

Arms:
  ours       libtblgpu.so on cuda:LOCAL_RANK.  `value` is device-timed (CUDA
             events around K steps, inputs resident); `e2e` drives K further
             steps through the C ABI with pinned host buffers: each step uploads
             u, v, w, p, p' and downloads u, v, w, p.
  reference  the CPU restatement of the reference (oracle/, C++ FP64 with P
             virtual MPI ranks, OpenMP over all host cores) on the same
             workload; steps run from the seeded field until a time budget is
             used (at least one full step).  The reference Fortran/MPI program
             cannot be built on these machines (no Fortran compiler, no MPI).
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

from turbulentbl_gb300 import abi  # noqa: E402
from turbulentbl_gb300.synth import WORKLOADS, make_state  # noqa: E402

FALLBACK_HBM_GBS = 6800.0
FP64_PEAK_TFLOPS = 1.2  # measured FMA throughput on this machine's GB300 (FP64 is 1/64 of FP32)

GROUP_NAMES = ["conv_q", "gs_sweep", "gs_resid", "ssor_fwd_matvec", "ssor_bwd", "mgs", "small", "vec", "bc", "stats",
               "total"]


def peaks():
    p = os.path.join(HERE, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def traffic_table():
    """Per-launch DRAM traffic of the kernel groups from a committed ncu summary."""
    p = os.path.join(HERE, "profiles", "traffic.json")
    try:
        with open(p) as f:
            return json.load(f)
    except Exception:
        return {}


class ClockSampler:
    """nvidia-smi clock/throttle sampling while the timed region runs."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.idx), f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def max_over_ranks(x, world, device="cuda"):
    """The slowest rank's time (replicas: the job ends when the last replica does)."""
    if world <= 1:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(points_per_step, steps, world, elapsed_s):
    """Whole-job Mpt-steps/s: every replica advances its own box by `steps` steps."""
    return points_per_step * steps * world / elapsed_s / 1e6


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def run_cpu(wl, nproc, budget_s, max_steps, variant=0):
    """Time the oracle (all host threads) from the seeded field for up to max_steps steps
    or until budget_s seconds are used; at least one step."""
    from oracle.bind import OracleRunner
    mesh, rp, st = make_state(wl, nproc=nproc)
    if variant:
        rp.use_variant(variant)
    o = OracleRunner(mesh, rp)
    o.upload(st)
    times, counts = [], []
    t_all = time.perf_counter()
    while len(times) < max(1, max_steps):
        t0 = time.perf_counter()
        o.step(1, check=False)
        times.append(time.perf_counter() - t0)
        counts.append(o.last_counts())
        if time.perf_counter() - t_all > budget_s:
            break
    threads = os.cpu_count() or 1
    mean_t = float(np.sum(times)) / len(times)
    value = wl.points / mean_t / 1e6
    iters = [int(np.sum(c[4:])) for c in counts]
    return {
        "value": value, "unit": "Mpt-steps/s", "cores": threads, "kind": "port",
        "sample": (f"{len(times)} full time step(s) of {wl.name} from the seeded field "
                   f"(steps 1..{len(times)}), C++ FP64 restatement with P={nproc} virtual ranks, "
                   f"OpenMP {threads} threads; GMRES Arnoldi iterations per step {iters}, "
                   f"GS sweeps per step {[c[:3] for c in counts]}"),
        "s_per_step": mean_t,
    }


def run_gpu(wl, nproc, steps, warmup, world, rank, local, do_e2e, do_cpu, cpu_budget, do_accuracy=True, rb=0,
            variant=0, extra_flags=0):
    """rb: 0 reference ordering, 1 red-black diffusion sweeps, 2 red-black
    diffusion sweeps and SSOR preconditioner.  variant: the reference program
    the step follows (tbl_config.variant), with that program's cum and
    recycling start."""
    import torch
    torch.cuda.set_device(local)
    from turbulentbl_gb300.lib import TblGpu
    mesh, rp, st = make_state(wl, nproc=nproc)
    if variant:
        rp.use_variant(variant)
    if wl.precision == abi.TBL_PREC_MIXED or rb:
        rp.flags |= abi.TBL_FLAG_PPE_RESIDUAL  # the true ||L7 p' - Q8|| / ||Q8|| every step (one extra pass)
    if rb:
        rp.flags |= abi.TBL_FLAG_RB_ORDER
    if rb > 1:
        rp.flags |= abi.TBL_FLAG_RB_PRECOND
    rp.flags |= extra_flags
    if extra_flags:
        rp.flags |= abi.TBL_FLAG_PPE_RESIDUAL
    g = TblGpu(mesh, rp)
    g.upload(st)
    for _ in range(warmup):
        g.step(1, check=False)
    L = g.lib
    L.tbl_profile.argtypes = [abi.C.c_void_p, abi.C.c_int]
    L.tbl_profile_read.argtypes = [abi.C.c_void_p, abi.C.POINTER(abi.C.c_double), abi.C.POINTER(abi.C.c_double),
                                   abi.C.POINTER(abi.C.c_int64), abi.C.c_int]
    L.tbl_profile(g._h, 1)
    launches0 = g.launches()
    if world > 1:
        torch.distributed.barrier()
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.4)
    torch.cuda.synchronize()
    # device time: CUDA events recorded by the library on its own stream
    # around the K steps (tbl_profile group "total"); host time alongside
    e0 = time.perf_counter()
    st_all, recs = g.step(steps, check=False)
    torch.cuda.synchronize()
    e1 = time.perf_counter()
    ng = len(GROUP_NAMES)
    ms = (abi.C.c_double * ng)()
    by = (abi.C.c_double * ng)()
    nl = (abi.C.c_int64 * ng)()
    L.tbl_profile_read(g._h, ms, by, nl, ng)
    dev_elapsed = ms[ng - 1] * 1e-3
    elapsed = max_over_ranks(dev_elapsed, world)
    clk = clocks.stop()
    launches = g.launches() - launches0
    L.tbl_profile(g._h, 0)
    groups = {GROUP_NAMES[q]: {"ms": ms[q], "bytes": by[q], "launches": nl[q]} for q in range(ng - 1)}
    out = {"elapsed": elapsed, "host_elapsed": e1 - e0, "recs": recs, "status": st_all, "launches": launches,
           "clocks": clk, "groups": groups}
    if (wl.precision == abi.TBL_PREC_MIXED or rb or extra_flags) and do_accuracy:
        out["mixed_state"] = g.download(fields=("u", "v", "w", "p"))
        out["mixed_stats"] = g.download_stats()
        out["accuracy_steps"] = warmup + steps
    g.close()
    if do_e2e:
        # The same K steps through the C ABI as a host driver would run them:
        # a second handle brought to the timed region's starting state (same
        # upload, same warm-up steps), then every step uploads the state the
        # host holds (u, v, w, p and the GMRES warm start p'), steps, and
        # downloads the new state into the same pinned buffers.  The round
        # trip is exact, so these steps repeat the timed ones (same iteration
        # counts) with the host copies added.
        nx, ny, nz = mesh.nx, mesh.ny, mesh.nz
        n = nx * ny * nz
        g = TblGpu(mesh, rp)
        g.upload(st)
        for _ in range(warmup):
            g.step(1, check=False)
        fields = ("u", "v", "w", "p", "pcorr")
        host = {f: torch.empty(n, dtype=torch.float64, pin_memory=True).numpy() for f in fields}
        d = g.download(fields=fields)
        for f in host:
            host[f][:] = np.asarray(d[f], order="F").reshape(-1, order="F")
        L = g.lib
        L.tbl_upload_fields.argtypes = [abi.C.c_void_p] + [abi.C.POINTER(abi.C.c_double)] * 5
        S = abi.TblState()
        ptr = {f: host[f].ctypes.data_as(abi.C.POINTER(abi.C.c_double)) for f in host}
        for f in fields:
            setattr(S, f, ptr[f])
        arr = (abi.TblStepStats * 1)()
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        t0 = time.perf_counter()
        e2e_recs = []
        for _ in range(steps):
            L.tbl_upload_fields(g._h, ptr["u"], ptr["v"], ptr["w"], ptr["p"], ptr["pcorr"])
            L.tbl_step(g._h, 1, arr)
            e2e_recs.append(arr[0].as_dict())
            L.tbl_download_state(g._h, abi.C.byref(S))
        t1 = time.perf_counter()
        te = t1 - t0
        te = max_over_ranks(te, world)
        out["e2e"] = {"elapsed": te, "h2d": 5 * n * 8, "d2h": 5 * n * 8,
                      "iters": [r["gmres_iters"] for r in e2e_recs]}
        g.close()
    if "mixed_state" in out and rank == 0:
        out["accuracy"] = mixed_accuracy(wl, nproc, variant, out.pop("mixed_state"), out.pop("mixed_stats"),
                                         out["accuracy_steps"], out["recs"])
    if do_cpu and rank == 0:
        out["cpu"] = run_cpu(wl, nproc, cpu_budget, 1, variant)
    return out


def mixed_accuracy(wl, nproc, variant, dm, sm, nsteps, recs):
    """The state of a mixed-precision or red-black run after nsteps steps
    against the FP64 library in the reference ordering (which matches the FP64
    oracle to 1e-12) from the same seeded start:
    per-field relative L2, the mean streamwise-velocity profile U(y) and the
    running statistics, plus the worst true PPE residual of the timed steps."""
    from turbulentbl_gb300.lib import TblGpu
    mesh, rp, st = make_state(wl, nproc=nproc)
    if variant:
        rp.use_variant(variant)
    rp.precision = abi.TBL_PREC_FP64
    g = TblGpu(mesh, rp)
    g.upload(st)
    g.step(nsteps, check=False)
    d = g.download(fields=("u", "v", "w", "p"))
    s64 = g.download_stats()
    g.close()
    rel = {f: float(np.linalg.norm(dm[f] - d[f]) / np.linalg.norm(d[f])) for f in ("u", "v", "w", "p")}
    prof = lambda u: u[1:-1, 1:-1, :].mean(axis=(0, 1))  # mean over x and span at each wall distance
    p64, pm = prof(d["u"]), prof(dm["u"])
    us64, usm = s64["usum"][1:-1, 1:-1], sm["usum"][1:-1, 1:-1]
    # per statistic: the running span sums of the means and products, the
    # rescaling's thicknesses and Re_theta, wall shear and mass flux
    per_stat = {}
    for f in list(abi.STATS_FIELDS) + ["deltastar", "theta", "ht", "reth", "tauw_sum", "ubulk"]:
        a, b = np.asarray(sm[f]), np.asarray(s64[f])
        n = float(np.linalg.norm(b))
        per_stat[f] = float(np.linalg.norm(a - b) / n) if n > 0 else float(np.linalg.norm(a))
    per_stat["lamda03"] = abs(sm["lamda03"] - s64["lamda03"]) / max(abs(s64["lamda03"]), 1e-300)
    return {"steps_compared": nsteps, "rel_l2": rel,
            "mean_profile_max_rel": float(np.abs(pm - p64).max() / np.abs(p64).max()),
            "usum_max_rel": float(np.abs(usm - us64).max() / max(np.abs(us64).max(), 1e-300)),
            "statistics_rel_l2": per_stat,
            "ppe_rel_resid_max": max(r["ppe_rel_resid"] for r in recs)}


def run_adjoint(wl, nproc, window, ckpt, n_fd, local):
    """Adjoint of a window on the adjoint workload: cost of tbl_backward_window
    (recomputation from checkpoints + adjoint steps) against tbl_forward_window,
    and the gradient against central differences of the forward window."""
    import torch
    torch.cuda.set_device(local)
    from turbulentbl_gb300.lib import TblGpu
    mesh, rp, st = make_state(wl, nproc=nproc)
    # tight solves, so that central differences with a small step resolve the
    # directional derivative (a small step keeps Peclet-window crossings of
    # the perturbed runs rare: the map is only piecewise smooth)
    rp.errorstop = 1e-12
    rp.errtol = 1e-12
    rp.cum = 10 ** 6      # no rescaling inside the window
    g = TblGpu(mesh, rp)
    g.upload(st)
    rng = np.random.default_rng(wl.seed)
    c = rng.normal(0.0, 1e-3, (mesh.nx, mesh.ny - 2))
    g.set_wall_control(c)
    g.step(2)
    x0 = g.download()
    patch = (10.0, 14.0)

    def fwd(cc, mode=abi.TBL_BRANCH_FREE):
        g.upload(x0)
        g.set_wall_control(cc)
        J, recs = g.forward_window(window, patch[0], patch[1], ckpt, mode)
        return J, recs

    fwd(c)  # warm-up (allocates the tape)
    J, recs = fwd(c)  # timed forward window (reference behaviour)
    grad, _, ast = g.backward_window(1.0)
    # gradient checks: the base window records its branch decisions, the
    # perturbed windows replay them (the map the adjoint differentiates); the
    # free-branch differences of the gradient direction are reported beside
    fwd(c, abi.TBL_BRANCH_RECORD)
    g.backward_window(1.0)
    fd = []
    gn = float(np.linalg.norm(grad))
    for q in range(n_fd + 1):
        free = q == n_fd
        # direction 0 (and the free-branch one): the normalised gradient; then seeded random directions
        d = grad / gn * 1e-3 * np.sqrt(grad.size) if (q == 0 or free) else rng.normal(0.0, 1e-3, c.shape)
        eps = 1e-4 if free else 1e-2
        mode = abi.TBL_BRANCH_FREE if free else abi.TBL_BRANCH_REPLAY
        Jp, _ = fwd(c + eps * d, mode)
        Jm, _ = fwd(c - eps * d, mode)
        fdv = (Jp - Jm) / (2 * eps)
        adv = float((grad * d).sum())
        fd.append({"direction": ("gradient" if q == 0 or free else f"random {q}"),
                   "branches": "free" if free else "replayed", "eps": eps, "fd": fdv, "adjoint": adv,
                   "rel_err": abs(fdv - adv) / abs(adv),
                   "err_vs_norms": abs(fdv - adv) / (gn * float(np.linalg.norm(d)))})
    g.close()
    return {"objective": J, "forward_ms": ast["forward_ms"], "backward_ms": ast["backward_ms"],
            "ratio": ast["backward_ms"] / ast["forward_ms"], "adjoint_stats": ast, "fd": fd,
            "gmres_iters_forward": sum(r["gmres_iters"] for r in recs),
            "gs_sweeps_forward": sum(sum(r["gs_sweeps"]) for r in recs), "grad_norm": float(np.linalg.norm(grad))}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=8)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="box512_fp64", choices=sorted(WORKLOADS))
    ap.add_argument("--nproc", type=int, default=8, help="virtual MPI ranks (slabs)")
    ap.add_argument("--cpu-budget", type=float, default=30.0, help="seconds of CPU time for the CPU sample")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-accuracy", action="store_true", help="mixed workloads: skip the FP64 comparison run")
    ap.add_argument("--rb", action="store_true",
                    help="red-black diffusion sweeps (TBL_FLAG_RB_ORDER): not the reference's sweep order")
    ap.add_argument("--rb-precond", action="store_true",
                    help="with --rb, the SSOR preconditioner red-black ordered too (TBL_FLAG_RB_PRECOND)")
    ap.add_argument("--span-blocks", action="store_true",
                    help="block SSOR on 32-row span blocks (TBL_FLAG_SSOR_SPAN_BLOCKS): not the reference's preconditioner")
    ap.add_argument("--stream-blocks", action="store_true",
                    help="block SSOR on two streamwise blocks per line (TBL_FLAG_SSOR_STREAM_BLOCKS): not the "
                         "reference's preconditioner")
    ap.add_argument("--variant", type=int, default=0, choices=[0, 1, 2],
                    help="the reference program the step follows: 0 dnstbl2, 1 originalTBL, 2 dnssetbl")
    ap.add_argument("--adjoint", action="store_true",
                    help="time the discrete adjoint of a window on the 256x96x96 adjoint workload instead")
    ap.add_argument("--window", type=int, default=50)
    ap.add_argument("--ckpt", type=int, default=10)
    ap.add_argument("--fd-dirs", type=int, default=16)
    ap.add_argument("--no-mixed", action="store_true",
                    help="leave out the mixed-precision arm of the default line")
    ap.add_argument("--no-adjoint", action="store_true",
                    help="leave out the adjoint/forward cost block of the default line")
    args = ap.parse_args()
    world, rank, local = dist_setup()
    if args.adjoint:
        if rank != 0:
            return
        wl = WORKLOADS["box256_adjoint"]
        r = run_adjoint(wl, args.nproc, args.window, args.ckpt, args.fd_dirs, local)
        line = {"metric": "adjoint/forward cost", "value": r["ratio"], "unit": "x", "n_gpus": 1,
                "higher_is_better": False, "dtype": "f64", "data": "synthetic (seeded)",
                "config": {"workload": wl.name, "reference_n3d": list(wl.n3d), "window_steps": args.window,
                           "checkpoint_every": args.ckpt, "objective": "mean wall shear, x in [10, 14]",
                           "control": "wall-normal blowing, nx x (ny-2), N(0, 1e-3)", "gs_errorstop": 1e-12,
                           "gmres_tol": 1e-12, "virtual_ranks": args.nproc},
                "forward_ms": r["forward_ms"], "backward_ms": r["backward_ms"],
                "objective": r["objective"], "grad_norm": r["grad_norm"],
                "fd_check": r["fd"],
                "max_fd_rel_err_replayed_branches": max([x["rel_err"] for x in r["fd"] if x["branches"] == "replayed"]
                                                        or [0.0]),
                "adjoint_stats": r["adjoint_stats"], "gmres_iters_forward": r["gmres_iters_forward"],
                "gs_sweeps_forward": r["gs_sweeps_forward"]}
        print(json.dumps(line), flush=True)
        return
    wl = WORKLOADS[args.workload]
    dtype = "f64" if wl.precision == 0 else "f32+f64"
    config = {"workload": wl.name, "grid_nx_ny_nz": [wl.nx, wl.ny_wall, wl.nz_span],
              "reference_n3d": list(wl.n3d), "virtual_ranks": args.nproc, "gmres_restart": wl.kmax,
              "gmres_tol": wl.errtol, "re_theta": wl.re_theta, "cfl": wl.cfl, "seed": wl.seed,
              "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
              "l2": "inputs larger than L2 (fields 68 MB+, Krylov basis 2.8 GB)",
              "ordering": ("red-black Gauss-Seidel and SSOR (throughput mode, not the reference's sweep order)"
                           if args.rb and args.rb_precond else
                           "red-black Gauss-Seidel, reference block SSOR (throughput mode, not the reference's "
                           "sweep order)" if args.rb else
                           "reference (lexicographic block Gauss-Seidel / block SSOR)"),
              "program": ["dnstbl2", "originalTBL", "dnssetbl"][args.variant],
              "preconditioner": ("block SSOR on the slabs (reference)" if not (args.span_blocks or args.stream_blocks)
                                 else "block SSOR on slabs" + (" x 32-row span blocks" if args.span_blocks else "")
                                 + (" x 2 streamwise blocks" if args.stream_blocks else "")
                                 + " (throughput mode, not the reference's)")}
    metric = "Mpt-steps/s"
    if args.impl == "reference":
        if rank != 0:
            return
        cpu = run_cpu(wl, args.nproc, max(args.cpu_budget, 1.0) * max(args.steps, 1), args.steps, args.variant)
        line = {"metric": metric, "value": cpu["value"], "unit": "Mpt-steps/s", "n_gpus": world,
                "steps": args.steps, "warmup": 0, "ms_per_step": cpu["s_per_step"] * 1e3, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": dtype, "data": "synthetic (seeded)",
                "config": config, "impl": "reference",
                "cpu_baseline": {k: cpu[k] for k in ("value", "unit", "cores", "kind", "sample")},
                "e2e": {"value": cpu["value"], "unit": "Mpt-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return
    if world > 1:
        import torch
        torch.distributed.init_process_group("nccl", device_id=torch.device("cuda", local))
    r = run_gpu(wl, args.nproc, args.steps, max(args.warmup, 3), world, rank, local, not args.no_e2e,
                not args.no_cpu, args.cpu_budget, not args.no_accuracy,
                (2 if args.rb and args.rb_precond else 1 if args.rb else 0), args.variant,
                (abi.TBL_FLAG_SSOR_SPAN_BLOCKS if args.span_blocks else 0) |
                (abi.TBL_FLAG_SSOR_STREAM_BLOCKS if args.stream_blocks else 0))
    if rank != 0:
        return
    K = args.steps
    line = gpu_line(wl, r, K, world, args.warmup, config)
    line["metric"] = metric
    if "cpu" in r:
        c = r["cpu"]
        line["cpu_baseline"] = {k: c[k] for k in ("value", "unit", "cores", "kind", "sample")}
    # the rest of the headline metric: the mixed-precision step on the same
    # box against this FP64 step, and the adjoint/forward cost of a window
    if not args.no_mixed and wl.name == "box512_fp64" and world == 1:
        wm = WORKLOADS["box512_mixed"]
        rm = run_gpu(wm, args.nproc, K, max(args.warmup, 3), world, rank, local, False, False, 0.0, True)
        ml = gpu_line(wm, rm, K, world, args.warmup, dict(config, workload=wm.name))
        mixed = {k: ml[k] for k in ("value", "unit", "ms_per_step", "roofline", "step_hbm", "groups_ms_per_step",
                                    "gmres_iters_per_step", "gs_sweeps_per_step", "status", "gpu_launches", "clocks")}
        mixed["workload"] = wm.name
        mixed["vs_fp64"] = ml["value"] / line["value"]
        mixed["ppe_rel_resid_max"] = ml.get("ppe_rel_resid_max")
        mixed["accuracy_vs_fp64"] = ml.get("accuracy_vs_fp64")
        mixed["precision"] = ("FP32 fields, stencils and inner GMRES (restart 40, inner tol 1e-5) in FP64 "
                              "iterative refinement to 1e-10 and a true PPE residual <= 1e-8; FP64 Gram-Schmidt "
                              "sums, Hessenberg, Givens, recycling and statistics")
        line["mixed"] = mixed
    if not args.no_adjoint and wl.name == "box512_fp64" and world == 1:
        wa = WORKLOADS["box256_adjoint"]
        ra = run_adjoint(wa, args.nproc, args.window, args.ckpt, args.fd_dirs, local)
        rep = [x["rel_err"] for x in ra["fd"] if x["branches"] == "replayed"]
        line["adjoint"] = {
            "workload": wa.name, "reference_n3d": list(wa.n3d), "window_steps": args.window,
            "checkpoint_every": args.ckpt, "forward_ms": ra["forward_ms"], "backward_ms": ra["backward_ms"],
            "ratio": ra["ratio"], "fd_directions": len(rep), "max_fd_rel_err": max(rep or [0.0]),
            "fd_free_branches_rel_err": [x["rel_err"] for x in ra["fd"] if x["branches"] == "free"],
            "objective": "mean wall shear over x in [10, 14], window-averaged",
            "control": "wall-normal blowing on the nx x (ny-2) wall grid, N(0, 1e-3) from seed 3"}
    print(json.dumps(line), flush=True)


def gpu_line(wl, r, K, world, warmup, config):
    """The JSON line of one GPU arm: whole-job rate, the roofline of the
    kernel group with the largest share of the step, per-group times."""
    value = whole_job_rate(wl.points, K, world, r["elapsed"])
    hbm, hbm_kind = peaks()
    groups = r["groups"]
    top = max(groups, key=lambda k: groups[k]["ms"])
    tg = groups[top]
    nl = max(tg["launches"], 1)
    per_launch_ms = tg["ms"] / nl
    bytes_per_launch = tg["bytes"] / nl
    achieved = bytes_per_launch / (per_launch_ms * 1e-3) / 1e9 if tg["ms"] > 0 else 0.0
    tab = traffic_table()
    tt = tab.get(f"{wl.name}/{top}", tab.get(top))
    traffic = tt.get("bytes_per_launch") if isinstance(tt, dict) else tt
    roofline = {"bound": "hbm", "kernel": top, "achieved": achieved, "peak": hbm, "unit": "GB/s",
                "frac": achieved / hbm, "peak_kind": f"{hbm_kind} (MEASURED_PEAKS.json hbm_gbs)",
                "traffic": traffic,
                "traffic_note": (f"ncu dram bytes of one {tt['launch']} vs {tt['algorithmic_bytes_per_launch']:.0f} "
                                 f"algorithmic ({tt['source']})") if isinstance(tt, dict) else None,
                "share_of_step": tg["ms"] / (r["elapsed"] * 1e3),
                "launches": tg["launches"], "per_launch_ms": per_launch_ms,
                "algorithmic_bytes_per_launch": bytes_per_launch,
                "dram_gbs": (traffic / (per_launch_ms * 1e-3) / 1e9) if traffic and per_launch_ms > 0 else None,
                "dram_frac": (traffic / (per_launch_ms * 1e-3) / 1e9 / hbm) if traffic and per_launch_ms > 0 else None,
                "how": ("algorithmic bytes of the group's launches / their CUDA-event time (events bracket each "
                        "group of launches on the library's stream), per launch")}
    step_bytes = sum(v["bytes"] for v in groups.values())
    dtype = "f64" if wl.precision == 0 else "f32+f64"
    line = {"metric": "Mpt-steps/s", "value": value, "unit": "Mpt-steps/s", "n_gpus": world, "steps": K,
            "warmup": max(warmup, 3), "ms_per_step": r["elapsed"] * 1e3 / K, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": dtype, "data": "synthetic (seeded 1/7-law + curl noise)",
            "config": config, "roofline": roofline,
            "step_hbm": {"algorithmic_gb_per_step": step_bytes / K / 1e9,
                         "achieved_gbs": step_bytes / r["elapsed"] / 1e9, "frac": step_bytes / r["elapsed"] / 1e9 / hbm},
            "groups_ms_per_step": {k: v["ms"] / K for k, v in groups.items()},
            "gmres_iters_per_step": [x["gmres_iters"] for x in r["recs"]],
            "gs_sweeps_per_step": [x["gs_sweeps"] for x in r["recs"]],
            "status": abi.STATUS_NAMES.get(r["status"], r["status"]),
            "host_ms_per_step": r["host_elapsed"] * 1e3 / K,
            "gpu_launches": r["launches"], "clocks": r["clocks"]}
    if "e2e" in r:
        e = r["e2e"]
        line["e2e"] = {"value": whole_job_rate(wl.points, K, world, e["elapsed"]), "unit": "Mpt-steps/s",
                       "h2d_bytes_per_step": e["h2d"], "d2h_bytes_per_step": e["d2h"],
                       "gmres_iters_per_step": e["iters"]}
    if any(x.get("ppe_rel_resid", 0.0) > 0.0 for x in r["recs"]):
        line["ppe_rel_resid_max"] = max(x["ppe_rel_resid"] for x in r["recs"])
    if "accuracy" in r:
        line["accuracy_vs_fp64"] = r["accuracy"]
    return line
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
