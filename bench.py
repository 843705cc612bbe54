"""Benchmark: DOF-stage updates/s of the GB300 DGSEM operator + LSERK stepper.

Workload (default): compressible Navier-Stokes Taylor-Green vortex, N=7 Gauss-Lobatto nodes,
split-form flux differencing with the Pirozzoli two-point flux, Roe surface flux, BR1 lifting,
24^3 periodic hexahedra on [-pi,pi]^3 (7 077 888 DOF x 5 variables), Ma 0.1, Re 1600, Pr 0.72,
Carpenter RK4-5.  A step is one LSERK step (5 RHS stages) over the whole mesh; inputs are seeded
synthetic TGV states (no dataset exists for this path).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--precision fp64|mixed]

One JSON line on rank 0.  Multi-GPU runs are replicas (each rank steps its own mesh; no collective
on the data path): value = all ranks' DOF-stages / max-over-ranks time, scaling "weak".
"""
import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    # name: (N, elems per direction, split, riemann, parabolic, mu0, flops/DOF-stage, bytes/DOF-stage)
    "tgv_n7_24cube_split_pi_roe_br1": dict(N=7, ne=24, SplitDG="pi", Riemann="roe", parabolic=True, mu0=1 / 1600.0),
    "tgv_n7_16cube_split_pi_roe_br1": dict(N=7, ne=16, SplitDG="pi", Riemann="roe", parabolic=True, mu0=1 / 1600.0),
    "tgv_n7_64cube_split_pi_roe_br1": dict(N=7, ne=64, SplitDG="pi", Riemann="roe", parabolic=True, mu0=1 / 1600.0),
}
# Algorithmic work per DOF-stage for the N=7 split-form NS path (FMA = 2 flops), per kernel:
#   prolong: ConsToPrim 14 ; lift: 30n+75 + 270/n + 15 ; face: 1200/n ; volume: 135N + 115 + 30n + 60/n + 30
ALG_FLOPS_N7 = {"prolong": 14.0, "lift": 30 * 8 + 75 + 270 / 8 + 15, "face": 1200 / 8,
                "volume": 135 * 7 + 115 + 30 * 8 + 60 / 8 + 30}
ALG_BYTES_N7 = 510.0  # compulsory HBM bytes per DOF-stage of a fully fused implementation (FP64)
# DRAM traffic and executed FP64 instructions are not measurable inside this process; they come from
# ncu captures of the same kernels on the 16^3 case of this workload (2 097 152 DOF; traffic grows
# with the number of elements, so it is scaled per DOF), one kernel and one launch per capture:
#   ncu --metrics dram__bytes_read.sum,dram__bytes_write.sum,gpu__time_duration.sum --clock-control none
#       -k regex:<kernel> -s 3 -c 1 python bench.py [--precision mixed] --workload tgv_n7_16cube_split_pi_roe_br1
#       --steps 2 --warmup 1 --no-e2e --no-cpu-baseline --no-profile --no-extras
#   and for k_volume (FP64) the executed DFMA + DADD + DMUL thread-instructions
#   (sm__sass_thread_inst_executed_op_{dfma,dadd,dmul}_pred_on.sum).
CAPTURE = {"fp64": "ncu, one kernel and one launch per capture, tgv_n7_16cube, 2026-12-04 19:11 UTC, commit 05fa055",
           "mixed": "ncu, one kernel and one launch per capture, tgv_n7_16cube, 2026-12-04 20:25 UTC, commit c00486e"}
_DOF16 = 2097152
DRAM_BYTES_PER_DOF = {  # read + write per launch
    "fp64": {"prolong": (84145920 + 196942336) / _DOF16, "lift": (329342464 + 302912256) / _DOF16,
             "face": (289529856 + 24906496) / _DOF16, "volume": (671186432 + 143390720) / _DOF16},
    "mixed": {"prolong": (84130048 + 69619200) / _DOF16, "lift": (157313792 + 127674624) / _DOF16,
              "face": (144744960 + 9332992) / _DOF16, "volume": (427753216 + 123999744) / _DOF16},
}
KVOL_FP64_INSTR_PER_DOF = (642252800 + 248512512 + 195297280) / _DOF16
FP64_ISSUE_PER_CYCLE = 304  # sm__sass_thread_inst_executed_op_dfma_pred_on.sum.peak_sustained (152 SMs x 2)
TGV_R = 71.42857
CFL = 0.8  # CFLscale / DFLscale of the reference's TGV regression (regressioncheck/checks/tgv/split/parameter.ini)
DFL = 0.8


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed"])
    ap.add_argument("--workload", default="tgv_n7_24cube_split_pi_roe_br1", choices=sorted(WORKLOADS))
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-profile", action="store_true", help="skip the per-kernel event timing and peak kernels")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the mixed-precision comparisons and the adjoint measurement")
    ap.add_argument("--adjoint-fd", type=int, default=16,
                    help="central-difference check of the adjoint gradient along this many random directions")
    ap.add_argument("--no-scale64", action="store_true", help="skip the 64^3 scale case among the extras")
    ap.add_argument("--adjoint-steps", type=int, default=None,
                    help="steps of the adjoint window (default 200 for the N=5 case, 50 for --only scale64)")
    ap.add_argument("--curved-ne", type=int, default=32,
                    help="elements per direction of the curved-box case (32; smaller for profiling)")
    ap.add_argument("--only", default=None, choices=["adjoint", "mixed_tgv", "mixed_curved", "scale64", "vortex"],
                    help="run one of the extra measurements alone and print its JSON (profiling runs)")
    args = ap.parse_args()
    args.steps_given = any(a == "--steps" or a.startswith("--steps=") for a in sys.argv[1:])
    return args


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu, self.samples, self._stop = gpu, [], threading.Event()
        self._t = threading.Thread(target=self._run, daemon=True)

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                if out.returncode == 0 and out.stdout.strip():
                    self.samples.append([x.strip() for x in out.stdout.strip().split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        self._t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        sm = sorted(float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit())
        mx = max(float(s[2]) for s in self.samples if s[2].replace(".", "").isdigit()) if sm else None
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for s in self.samples for k in range(4) if len(s) > 5 + k and s[5 + k] == "Active"})
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": mx, "reasons": reasons,
                "samples": len(self.samples)}


def dist_init(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        backend = "nccl" if args.impl == "ours" else "gloo"
        dist.init_process_group(backend)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(world, x, device=None):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def reference_setup(workload):
    """The workload's oracle, mesh and initial state built without the product library (oracle/
    standalone.py: periodic box with the oracle's own metrics, numpy TGV state)."""
    from oracle.oracle import Oracle
    from oracle.standalone import PeriodicBox, config, tgv_state
    w = WORKLOADS[workload]
    cfg = config(w["N"], "gauss-lobatto", w["Riemann"], w["SplitDG"], parabolic=w["parabolic"], R=TGV_R, mu0=w["mu0"])
    box = PeriodicBox(w["N"], 2, w["ne"], (-math.pi,) * 3, (math.pi,) * 3)
    U0 = tgv_state(box.Elem_xGP, mach=0.1, R=TGV_R)
    return Oracle(cfg, box, geometry="mesh"), box, U0


def cpu_baseline(workload, threads=None, target_s=12.0, warmup=1):
    """The oracle (CPU restatement of the reference formulas, OpenMP) on a bounded sample of the
    workload itself: as many full LSERK steps of the whole mesh as fit in about target_s."""
    from oracle.oracle import set_threads
    w = WORKLOADS[workload]
    nthreads = set_threads(threads or os.cpu_count() or 1)
    o, box, U0 = reference_setup(workload)
    dt, _ = o.calc_timestep(U0, CFL, DFL)
    U, Ut = np.array(U0), np.zeros_like(U0)
    for _ in range(max(1, warmup)):
        t0 = time.perf_counter()
        o.lserk_steps_inplace(U, Ut, dt, 1)
        one = time.perf_counter() - t0
    steps = max(1, min(2000, int(target_s / max(one, 1e-3))))
    t0 = time.perf_counter()
    o.lserk_steps_inplace(U, Ut, dt, steps)
    el = time.perf_counter() - t0
    o.close()
    val = box.nDOF * 5 * steps / el
    return {"value": val, "unit": "DOF-stage/s", "cores": nthreads, "kind": "port",
            "sample": "%d LSERK steps (5 stages) of the whole %d^3-element N=%d mesh (%d DOF), %.1f s" % (
                steps, w["ne"], w["N"], box.nDOF, el),
            "pid_s": nthreads * el / (box.nDOF * 5 * steps)}


def run_reference(args, world, rank):
    """Reference arm: the CPU restatement of the reference's formulas (the reference itself is CUDA
    Fortran and has no CPU build; it cannot be compiled here), all host threads, on the workload
    itself: W untimed and K timed LSERK steps of the whole mesh.  Mesh, metrics and state come from
    the oracle and numpy (no part of the product library is loaded)."""
    if rank != 0:
        return
    from oracle.oracle import set_threads
    w = WORKLOADS[args.workload]
    nthreads = set_threads(os.cpu_count() or 1)
    o, box, U0 = reference_setup(args.workload)
    dt, _ = o.calc_timestep(U0, CFL, DFL)
    U, Ut = np.array(U0), np.zeros_like(U0)
    o.lserk_steps_inplace(U, Ut, dt, max(0, args.warmup))
    t0 = time.perf_counter()
    o.lserk_steps_inplace(U, Ut, dt, args.steps)
    el = time.perf_counter() - t0
    o.close()
    val = box.nDOF * 5 * args.steps / el
    res = {"value": val, "unit": "DOF-stage/s", "cores": nthreads, "kind": "port",
           "sample": "%d timed LSERK steps (after %d untimed) of the whole %d^3-element N=%d mesh (%d DOF), %.1f s"
                     % (args.steps, args.warmup, w["ne"], w["N"], box.nDOF, el),
           "pid_s": nthreads * el / (box.nDOF * 5 * args.steps)}
    line = {"metric": "DOF-stage updates/s", "value": val, "unit": "DOF-stage/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": el * 1e3 / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (TGV initial state, generated mesh)", "impl": "reference",
            "config": {"workload": args.workload, "N": w["N"], "elements_per_dir": w["ne"], "nDOF": box.nDOF,
                       "form": "split PI", "riemann": w["Riemann"], "lifting": "BR1", "precision": "fp64",
                       "dt": dt},
            "cpu_baseline": res,
            "e2e": {"value": val, "unit": "DOF-stage/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args, world, rank, local):
    import torch
    import galaexi_gb300 as gx
    from galaexi_gb300 import _native as nat
    import ctypes

    torch.cuda.set_device(local)
    w = WORKLOADS[args.workload]
    N, ne = w["N"], w["ne"]
    cfg = gx.config(N=N, NodeType="gauss-lobatto", Riemann=w["Riemann"], SplitDG=w["SplitDG"],
                    parabolic=w["parabolic"], mu0=w["mu0"], R=TGV_R, precision=args.precision)
    mesh = gx.Mesh(N, 2, ne, ne, ne, (-math.pi,) * 3, (math.pi,) * 3)
    U0 = gx.tgv_state(mesh, mach=0.1, R=TGV_R)
    op = gx.DG(cfg, mesh)
    stream = torch.cuda.current_stream()
    U = torch.from_numpy(U0).cuda()
    Ut_tmp = torch.zeros_like(U)
    dt, err = op.CalcTimeStep(U, CFL, DFL)
    assert err == 0
    nDOF = mesh.nDOF
    # ---- device-resident timing
    for _ in range(args.warmup):
        op.TimeStepByLSERKW2(0.0, dt, U, Ut_tmp)
    torch.cuda.synchronize()
    barrier(world)
    launches0 = op.kernel_launches
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(args.steps):
            op.TimeStepByLSERKW2(0.0, dt, U, Ut_tmp)
        e1.record(stream)
        torch.cuda.synchronize()
    barrier(world)
    ms = e0.elapsed_time(e1)
    launches = op.kernel_launches - launches0
    ms = max_over_ranks(world, ms, device="cuda")
    value = world * nDOF * 5 * args.steps / (ms * 1e-3)
    bad = op.check_state(U)
    # ---- end-to-end through the public API with host buffers
    e2e = None
    if not args.no_e2e:
        # every step: its input state host->device from pinned memory, one LSERK step, its result
        # device->host; two device buffers so that the copies of one step run on a copy stream
        # while the other buffer's step computes
        Uh = torch.from_numpy(U0).pin_memory()
        Uout = [torch.empty_like(Uh).pin_memory() for _ in range(2)]
        Ud = [torch.empty_like(U) for _ in range(2)]
        Ut2 = torch.zeros_like(U)
        copy = torch.cuda.Stream()
        for b in range(2):  # warm-up of both buffers
            Ud[b].copy_(Uh, non_blocking=True)
            op.TimeStepByLSERKW2(0.0, dt, Ud[b], Ut2)
            Uout[b].copy_(Ud[b], non_blocking=True)
        torch.cuda.synchronize()
        barrier(world)
        loaded = [torch.cuda.Event() for _ in range(2)]
        stepped = [torch.cuda.Event() for _ in range(2)]
        e0.record(stream)
        copy.wait_event(e0)
        with torch.cuda.stream(copy):
            for b in range(min(2, args.steps)):
                Ud[b].copy_(Uh, non_blocking=True)
                loaded[b].record(copy)
        for k in range(args.steps):
            b = k % 2
            stream.wait_event(loaded[b])
            op.TimeStepByLSERKW2(0.0, dt, Ud[b], Ut2, stream=stream)
            stepped[b].record(stream)
            copy.wait_event(stepped[b])
            with torch.cuda.stream(copy):
                Uout[b].copy_(Ud[b], non_blocking=True)
                if k + 2 < args.steps:
                    Ud[b].copy_(Uh, non_blocking=True)
                    loaded[b].record(copy)
        stream.wait_stream(copy)
        e1.record(stream)
        torch.cuda.synchronize()
        ms_e2e = max_over_ranks(world, e0.elapsed_time(e1), device="cuda")
        ok = all(torch.equal(Uout[b], Uout[(args.steps - 1) % 2]) for b in range(min(2, args.steps)))
        e2e = {"value": world * nDOF * 5 * args.steps / (ms_e2e * 1e-3), "unit": "DOF-stage/s",
               "h2d_bytes_per_step": Uh.numel() * 8, "d2h_bytes_per_step": Uh.numel() * 8,
               "copies_overlap_compute": True, "results_identical": bool(ok)}
    # ---- per-kernel timing (CUDA events on the launching stream) for the roofline
    roofline = None
    if not args.no_profile:
        roofline = profile_roofline(args, op, U, dt, stream, nDOF, sm_mhz=clk.summary().get("sm_mhz"))
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(args.workload)
    extras = {}
    if not args.no_extras and args.precision == "fp64":
        # the mixed form over the workload's 200 steps, with its own roofline
        extras["mixed_vs_fp64"] = mixed_vs_fp64_tgv(args.workload, 200, stream, roofline=not args.no_profile)
        extras["mixed_vs_fp64_curved_br2"] = mixed_vs_fp64_curved_br2(stream)
        # the Euler vortex case (N=3 Gauss, weak, LF, 8^3): 100 steps against the exact solution
        extras["vortex_c1"] = vortex_c1(stream)
        # the discrete adjoint of 200 steps on the N=5 16^3 TGV, checked along 16 seeded directions
        extras["adjoint"] = adjoint_tgv(stream, steps=args.adjoint_steps or 200, fd_dirs=args.adjoint_fd)
        if not args.no_scale64:
            # the 64^3 scale case: 100 steps per form, the adjoint of a 50-step window in <= 180 GB
            extras["scale64"] = scale_c5(stream)
    if rank == 0:
        line = {"metric": "DOF-stage updates/s", "value": value, "unit": "DOF-stage/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f64" if args.precision == "fp64" else "f32-bulk/f64-rk",
                "data": "synthetic (seeded TGV initial state, generated mesh)",
                "config": {"workload": args.workload, "N": N, "elements_per_dir": ne, "nDOF": nDOF,
                           "form": "split PI", "riemann": w["Riemann"], "lifting": "BR1", "precision": args.precision,
                           "dt": dt, "l2": "inputs larger than L2 (state 283 MB)", "parallelism": "replicas"},
                "e2e": e2e, "roofline": roofline, "cpu_baseline": cpu, "clocks": clk.summary(),
                "gpu_launches": launches, "bad_nodes_after": bad}
        line.update(extras)
        print(json.dumps(line), flush=True)


def timed(fn, stream):
    """Run fn() between CUDA events on the stream; returns (ms, result)."""
    import torch
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    r = fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1), r


# Compulsory HBM bytes per DOF-stage of the mixed form (FP32 bulk) for a fully fused implementation at
# N=7: U and Ut_tmp read and written in FP64 (160), FP32 volume metrics and sJ (40), FP32 face geometry
# (10 values x 3 faces per n^3 nodes: 120/n = 15), the 15 FP32 lifted gradients written and read (120)
ALG_BYTES_N7_MIXED = 160.0 + 40.0 + 120.0 / 8 + 120.0


def mixed_vs_fp64_tgv(workload, steps, stream, roofline=False):
    """Mixed form against the FP64 form on the TGV workload: same initial state, same dt, `steps`
    LSERK steps each; kinetic-energy, mass and L2 differences of the end states, DOF-stage/s ratio;
    with roofline=True the mixed stage's per-kernel times and its HBM / FP32 roofline."""
    import torch
    import galaexi_gb300 as gx
    w = WORKLOADS[workload]
    mesh = gx.Mesh(w["N"], 2, w["ne"], w["ne"], w["ne"], (-math.pi,) * 3, (math.pi,) * 3)
    U0 = torch.from_numpy(gx.tgv_state(mesh, mach=0.1, R=TGV_R)).cuda()
    out, ops = {}, {}
    for prec in ("fp64", "mixed"):
        cfg = gx.config(N=w["N"], NodeType="gauss-lobatto", Riemann=w["Riemann"], SplitDG=w["SplitDG"],
                        parabolic=w["parabolic"], mu0=w["mu0"], R=TGV_R, precision=prec)
        ops[prec] = gx.DG(cfg, mesh)
    dt, _ = ops["fp64"].CalcTimeStep(U0, CFL, DFL)
    for prec, op in ops.items():
        U, K = U0.clone(), torch.zeros_like(U0)
        op.TimeStepByLSERKW2(0.0, dt, U, K)  # warm-up step (also fixes the mixed form's pressure offset)
        U, K = U0.clone(), torch.zeros_like(U0)
        ms, _ = timed(lambda: op.TimeStepByLSERKW2(0.0, dt, U, K, nSteps=steps), stream)
        out[prec] = (ms, U, ops["fp64"].integrals(U))
    ke64, kem = out["fp64"][2][5], out["mixed"][2][5]
    res = {"workload": workload, "steps": steps, "dt": dt,
           "speedup": out["fp64"][0] / out["mixed"][0],
           "dof_stage_per_s_fp64": mesh.nDOF * 5 * steps / (out["fp64"][0] * 1e-3),
           "dof_stage_per_s_mixed": mesh.nDOF * 5 * steps / (out["mixed"][0] * 1e-3),
           "ke_rel_err": abs(kem - ke64) / abs(ke64),
           "l2_rel": float((out["mixed"][1] - out["fp64"][1]).norm() / out["fp64"][1].norm()),
           "mass_rel_diff": abs(out["mixed"][2][0] - out["fp64"][2][0]) / abs(out["fp64"][2][0]),
           "reference": "FP64 path of this library (equal to the oracle to <=1e-12 per evaluation and "
                        "<=1e-10 after 100 steps of this workload)"}
    if roofline:
        res["roofline"] = mixed_roofline(ops["mixed"], U0, dt, stream, mesh.nDOF)
    for op in ops.values():
        op.close()
    return res


def mixed_roofline(op, U0, dt, stream, nDOF):
    """Per-kernel CUDA-event times of one mixed-form stage (dg_profile_stage) and the stage's rooflines:
    HBM on the compulsory FP32-bulk bytes, FP32 on the algorithmic flops."""
    import ctypes
    import torch
    from galaexi_gb300 import _native as nat
    out = (ctypes.c_double * 5)()
    Up, Utp = U0.clone(), torch.zeros_like(U0)
    nat.check(nat.lib().dg_profile_stage(op._h, ctypes.c_void_p(Up.data_ptr()), ctypes.c_void_p(Utp.data_ptr()),
                                         dt, 20, out, ctypes.c_void_p(stream.cuda_stream)), "dg_profile_stage")
    kms = {"prolong": out[0], "lift": out[1], "face": out[2], "volume": out[3], "stage": out[4]}
    peak32 = ctypes.c_double()
    nat.check(nat.lib().dg_measure_fma_peak(1, ctypes.byref(peak32)), "fma peak fp32")
    hbm_peak = measured_peaks().get("hbm_gbs")
    stage_s = kms["stage"] * 1e-3
    gbs = ALG_BYTES_N7_MIXED * nDOF / stage_s * 1e-9
    tflops = sum(ALG_FLOPS_N7.values()) * nDOF / stage_s * 1e-12
    return {"bound": "hbm", "unit": "GB/s", "alg_bytes_per_dof_stage": ALG_BYTES_N7_MIXED, "achieved": gbs,
            "peak": hbm_peak, "frac": gbs / hbm_peak if hbm_peak else None,
            "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured copy bandwidth)",
            "traffic_per_dof_stage": sum(DRAM_BYTES_PER_DOF["mixed"].values()),
            "traffic_per_dof_by_kernel": DRAM_BYTES_PER_DOF["mixed"],
            "traffic_source": "dram__bytes_read+write per DOF of one launch of each kernel (%s)" % CAPTURE["mixed"],
            "fp32_achieved_tflops": tflops, "fp32_peak_tflops_measured": peak32.value * 1e-3,
            "fp32_frac": tflops / (peak32.value * 1e-3), "kernel_ms": kms}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except Exception:
        return {}


def mixed_vs_fp64_curved_br2(stream, steps=500, ne=32):
    """Mixed form against the FP64 form on the curved-box BR2 case: Navier-Stokes, N=5 Gauss nodes,
    weak form, HLLC, BR2 (etaBR2 = 2), 32^3 elements (ne^3) on [0,1]^3 with every node displaced by
    0.05 sin(2 pi x) sin(2 pi y) sin(2 pi z), uniform flow rho=1, v=(0.3,0.2,0.1), p=1/1.4 plus
    seeded Gaussian noise 1e-3 on each conserved variable, mu=1e-3; 500 steps."""
    import numpy as np
    import torch
    import galaexi_gb300 as gx
    N = 5
    mesh = gx.Mesh(N, 1, ne, ne, ne, (0.0,) * 3, (1.0,) * 3, deform=0.05)
    U = gx.fill_ini(mesh, 1, [1.0, 0.3, 0.2, 0.1, 1.0 / 1.4])
    rng = np.random.default_rng(20261203)
    U = U + 1e-3 * rng.standard_normal(U.size).reshape(U.shape)
    U0 = torch.from_numpy(U).cuda()
    ops = {}
    for prec in ("fp64", "mixed"):
        cfg = gx.config(N=N, NodeType="gauss", Riemann="hllc", parabolic=True, mu0=1e-3, Lifting="br2", etaBR2=2.0,
                        precision=prec)
        ops[prec] = gx.DG(cfg, mesh)
    # CFLscale 0.9; DFLscale 0.45: the BR2 penalty (etaBR2 = 2) raises the viscous spectral radius
    # above the BR1 value the DFL alpha tables are made for -- with DFLscale 0.6 the oracle itself
    # diverges on this case within 10 steps at matching viscous/convective ratio, 0.45 is stable
    dt, _ = ops["fp64"].CalcTimeStep(U0, 0.9, 0.45)
    I0 = ops["fp64"].integrals(U0)
    out = {}
    for prec, op in ops.items():
        Uw, K = U0.clone(), torch.zeros_like(U0)
        op.TimeStepByLSERKW2(0.0, dt, Uw, K)
        Ur, K = U0.clone(), torch.zeros_like(U0)
        ms, _ = timed(lambda: op.TimeStepByLSERKW2(0.0, dt, Ur, K, nSteps=steps), stream)
        out[prec] = (ms, Ur, ops["fp64"].integrals(Ur))
    res = {"workload": "curved_n5_gauss_%dcube_weak_hllc_br2" % ne, "steps": steps, "dt": dt, "cfl": 0.9, "dfl": 0.45,
           "speedup": out["fp64"][0] / out["mixed"][0],
           "dof_stage_per_s_fp64": mesh.nDOF * 5 * steps / (out["fp64"][0] * 1e-3),
           "dof_stage_per_s_mixed": mesh.nDOF * 5 * steps / (out["mixed"][0] * 1e-3),
           "l2_rel": float((out["mixed"][1] - out["fp64"][1]).norm() / out["fp64"][1].norm()),
           "mass_drift_fp64": (out["fp64"][2][0] - I0[0]) / I0[0],
           "mass_drift_mixed": (out["mixed"][2][0] - I0[0]) / I0[0],
           "energy_drift_fp64": (out["fp64"][2][4] - I0[4]) / I0[4],
           "energy_drift_mixed": (out["mixed"][2][4] - I0[4]) / I0[4],
           "ke_rel_err": abs(out["mixed"][2][5] - out["fp64"][2][5]) / abs(out["fp64"][2][5]),
           "reference": "FP64 path of this library (matches the oracle to <=1e-12 per evaluation)"}
    for op in ops.values():
        op.close()
    return res


def vortex_c1(stream, steps=100):
    """Euler, Gauss N=3, weak form, Lax-Friedrichs, 8^3 elements on [0,10]^3, Shu vortex (beta 5,
    half-width 1, advected with (1,1,0); exactfunc.f90:482-502), `steps` LSERK steps at CFL 0.9 from
    the exact state: DOF-stage/s and the relative L2 distance of the end state from the exact
    advected vortex (the discretisation error of 4 nodes per element and direction)."""
    import torch
    import galaexi_gb300 as gx
    from galaexi_gb300 import _native as nat
    m = gx.Mesh(3, 1, 8, 8, 8, (0.0,) * 3, (10.0,) * 3)
    prm = [1, 1, 1, 0, 1, 5, 5, 0, 0, 0, 1, 5, 1]  # RefState, IniCenter, IniAxis, beta, half-width
    U0 = gx.fill_ini(m, nat.DG_EXACTFUNC_SHU_VORTEX, prm)
    op = gx.DG(gx.config(N=3, NodeType="gauss", Riemann="lf"), m)
    U = torch.from_numpy(U0).cuda()
    dt, _ = op.CalcTimeStep(U, 0.9)
    W, K = U.clone(), torch.zeros_like(U)
    op.TimeStepByLSERKW2(0.0, dt, W, K)  # warm-up
    K.zero_()
    ms, _ = timed(lambda: op.TimeStepByLSERKW2(0.0, dt, U, K, nSteps=steps), stream)
    exact = torch.from_numpy(gx.fill_ini(m, nat.DG_EXACTFUNC_SHU_VORTEX, prm, t=steps * dt)).cuda()
    res = {"workload": "vortex_n3_gauss_8cube_weak_lf", "nDOF": m.nDOF, "steps": steps, "dt": dt,
           "dof_stage_per_s": m.nDOF * 5 * steps / (ms * 1e-3), "ms_per_step": ms / steps,
           "l2_rel_vs_exact": float((U - exact).norm() / exact.norm())}
    op.close()
    return res


def scale_c5(stream, steps=100, adj_steps=50, budget_gb=180):
    """The 64^3 scale case (134 M DOF, N=7 GL, split PI, Roe, BR1): FP64 and mixed for `steps` LSERK
    steps from the TGV state, then the adjoint of an `adj_steps` window (kinetic-energy objective)
    with checkpoints in at most `budget_gb` of device memory (less if the operator, ~61 GB at this
    size, and the adjoint's work states and scratch leave less free)."""
    import gc
    import torch
    import galaexi_gb300 as gx
    # the checkpoint budget below is what the device has free: release what earlier measurements left
    gc.collect()
    torch.cuda.empty_cache()
    w = WORKLOADS["tgv_n7_64cube_split_pi_roe_br1"]
    N, ne = w["N"], w["ne"]
    mesh = gx.Mesh(N, 2, ne, ne, ne, (-math.pi,) * 3, (math.pi,) * 3)
    U0 = torch.from_numpy(gx.tgv_state(mesh, mach=0.1, R=TGV_R)).cuda()
    res = {"workload": "tgv_n7_64cube_split_pi_roe_br1", "nDOF": mesh.nDOF, "steps": steps}
    ends = {}
    dt = None
    for prec in ("fp64", "mixed"):
        cfg = gx.config(N=N, NodeType="gauss-lobatto", Riemann=w["Riemann"], SplitDG=w["SplitDG"],
                        parabolic=True, mu0=w["mu0"], R=TGV_R, precision=prec)
        op = gx.DG(cfg, mesh)
        if dt is None:
            dt, _ = op.CalcTimeStep(U0, CFL, DFL)
        U, K = U0.clone(), torch.zeros_like(U0)
        op.TimeStepByLSERKW2(0.0, dt, U, K)
        U, K = U0.clone(), torch.zeros_like(U0)
        ms, _ = timed(lambda: op.TimeStepByLSERKW2(0.0, dt, U, K, nSteps=steps), stream)
        res["dof_stage_per_s_" + prec] = mesh.nDOF * 5 * steps / (ms * 1e-3)
        res["ms_per_step_" + prec] = ms / steps
        ends[prec] = (U, op.integrals(U) if prec == "fp64" else None)
        if prec == "mixed":
            I64 = ends["fp64"][1]
            Im = gx.DG(gx.config(N=N, NodeType="gauss-lobatto", Riemann=w["Riemann"], SplitDG=w["SplitDG"],
                                 parabolic=True, mu0=w["mu0"], R=TGV_R), mesh)
            Imix = Im.integrals(U)
            Im.close()
            res["mixed_ke_rel_err"] = abs(Imix[5] - I64[5]) / abs(I64[5])
            res["mixed_l2_rel"] = float((U - ends["fp64"][0]).norm() / ends["fp64"][0].norm())
        op.close()
        del K
    res["mixed_speedup"] = res["dof_stage_per_s_mixed"] / res["dof_stage_per_s_fp64"]
    del ends, U
    torch.cuda.empty_cache()
    cfg = gx.config(N=N, NodeType="gauss-lobatto", Riemann=w["Riemann"], SplitDG=w["SplitDG"], parabolic=True,
                    mu0=w["mu0"], R=TGV_R)
    op = gx.DG(cfg, mesh)

    def fwd():
        U, K = U0.clone(), torch.zeros_like(U0)
        op.TimeStepByLSERKW2(0.0, dt, U, K, nSteps=adj_steps)
        return U

    ms_f = timed(fwd, stream)[0]
    gc.collect()
    torch.cuda.empty_cache()
    # checkpoint budget: at most budget_gb (decimal GB), and what is left of the device after the
    # operator, the adjoint's work states and scratch, the gradient tensor and a 2 GiB margin; the
    # end state is written over U0
    free, total = torch.cuda.mem_get_info()
    state = U0.numel() * 8
    budget = int(min(budget_gb * 1e9, free - op.adjoint_scratch_bytes() - state - 2 * 2 ** 30))
    res["device_free_gb_before_adjoint"] = free / 1e9
    res["device_total_gb"] = total / 1e9
    Uf, plan = None, None
    t_rec, (Uf, plan) = timed(lambda: op.adjoint_forward(dt, adj_steps, U0, budget, out=U0), stream)
    J, G = op.kinetic_energy(Uf, grad=True)
    del Uf
    t_rev, mub = timed(lambda: op.adjoint_reverse(G), stream)
    res.update({"adjoint_steps": adj_steps, "adjoint_budget_gb": budget / 1e9, "adjoint_plan": plan,
                "state_gb": U0.numel() * 8 / 1e9, "forward_window_ms": ms_f, "adjoint_record_ms": t_rec,
                "adjoint_reverse_ms": t_rev, "adjoint_over_forward": (t_rec + t_rev) / ms_f, "J": J, "dJ_dmu": mub,
                "grad_norm": float(G.norm())})
    op.close()
    return res


def adjoint_tgv(stream, steps=200, fd_dirs=0):
    """Discrete adjoint on the N=5, 16^3 TGV (split PI, Roe, BR1, FP64): J = kinetic-energy integral
    after `steps` LSERK steps at fixed dt; gradient w.r.t. the initial state and mu.  Reports the
    adjoint (record + reverse) to forward wall-time ratio and, with fd_dirs > 0, central differences
    (eps = 1e-6) along seeded random unit directions (default_rng(4))."""
    import numpy as np
    import torch
    import galaexi_gb300 as gx
    N, ne, mu = 5, 16, 1 / 1600.0
    cfg = gx.config(N=N, NodeType="gauss-lobatto", Riemann="roe", SplitDG="pi", parabolic=True, mu0=mu, R=TGV_R)
    mesh = gx.Mesh(N, 2, ne, ne, ne, (-math.pi,) * 3, (math.pi,) * 3)
    U0 = torch.from_numpy(gx.tgv_state(mesh, mach=0.1, R=TGV_R)).cuda()
    op = gx.DG(cfg, mesh)
    dt, _ = op.CalcTimeStep(U0, CFL, DFL)
    budget = 180 << 30

    def fwd(o=op, U_init=U0):
        U, K = U_init.clone(), torch.zeros_like(U_init)
        o.TimeStepByLSERKW2(0.0, dt, U, K, nSteps=steps)
        return U

    fwd()
    op.adjoint_window(dt, 2, U0, budget)
    ms_f, Uf = timed(fwd, stream)
    ms_a, (J, G, dJdmu, _) = timed(lambda: op.adjoint_window(dt, steps, U0, budget), stream)
    plan = 1 if 5 * steps * U0.numel() * 8 <= budget else 2  # the window's checkpoint rule (plan 1: all stage inputs)
    res = {"workload": "tgv_n5_16cube_split_pi_roe_br1_adjoint", "steps": steps, "dt": dt, "nDOF": mesh.nDOF,
           "forward_ms": ms_f, "adjoint_ms": ms_a, "adjoint_over_forward": ms_a / ms_f,
           "checkpoint_plan": plan, "checkpoint_budget_gb": budget / 2 ** 30,
           "J": J, "dJ_dmu": dJdmu, "grad_norm": float(G.norm())}
    if fd_dirs > 0:
        rng = np.random.default_rng(4)
        dirs = []
        for _ in range(fd_dirs):
            v = torch.from_numpy(rng.standard_normal(tuple(U0.shape))).cuda()
            dirs.append(v / v.norm())
        # central differences at the specified eps = 1e-6 and at larger eps: along a unit direction of
        # the 4.4 M-dimensional state J changes by ~1e-4 eps, so at small eps the round-off of J (and of
        # the two trajectories) dominates the difference quotient; the sweep shows where round-off and
        # truncation balance
        for eps in (1e-6, 1e-5, 1e-4, 1e-3):
            errs = []
            for v in dirs:
                Jp = op.kinetic_energy(fwd(op, U0 + eps * v))
                Jm = op.kinetic_energy(fwd(op, U0 - eps * v))
                fd = (Jp - Jm) / (2 * eps)
                ad = float((G * v).sum())
                errs.append(abs(fd - ad) / abs(ad))
            res["fd_max_rel_err_eps%.0e" % eps] = max(errs)
            res["fd_median_rel_err_eps%.0e" % eps] = float(np.median(errs))
        res["fd_directions"] = fd_dirs
        # exact directional derivatives from the tangent-linear model (dual numbers through the same
        # 200 steps): <dJ/dU(t_end), Udot(t_end)> against <dJ/dU0, v>
        errs = []
        for v in dirs[:4]:
            U, Ud, K = U0.clone(), v.clone(), torch.zeros_like(U0)
            op.tlm_steps(dt, U, Ud, K, nSteps=steps)
            _, Gend = op.kinetic_energy(U, grad=True)
            tl = float((Gend * Ud).sum())
            ad = float((G * v).sum())
            errs.append(abs(tl - ad) / abs(ad))
        res["tlm_max_rel_err"] = max(errs)
        res["tlm_directions"] = min(4, fd_dirs)
        ops = {}
        eps = 1e-6
        for sgn in (1, -1):
            c2 = gx.config(N=N, NodeType="gauss-lobatto", Riemann="roe", SplitDG="pi", parabolic=True,
                           mu0=mu + sgn * eps, R=TGV_R)
            o2 = gx.DG(c2, mesh)
            ops[sgn] = o2.kinetic_energy(fwd(o2, U0))
            o2.close()
        fdm = (ops[1] - ops[-1]) / (2 * eps)
        res["fd_mu_rel_err"] = abs(fdm - dJdmu) / abs(dJdmu)
    op.close()
    return res


def profile_roofline(args, op, U, dt, stream, nDOF, sm_mhz=None):
    import ctypes
    import torch
    from galaexi_gb300 import _native as nat
    out = (ctypes.c_double * 5)()
    Up = U.clone()
    Utp = torch.zeros_like(U)
    nat.check(nat.lib().dg_profile_stage(op._h, ctypes.c_void_p(Up.data_ptr()), ctypes.c_void_p(Utp.data_ptr()),
                                         dt, 20, out, ctypes.c_void_p(stream.cuda_stream)), "dg_profile_stage")
    kms = {"prolong": out[0], "lift": out[1], "face": out[2], "volume": out[3], "stage": out[4]}
    peak64 = ctypes.c_double()
    peak32 = ctypes.c_double()
    nat.check(nat.lib().dg_measure_fma_peak(0, ctypes.byref(peak64)), "fma peak fp64")
    nat.check(nat.lib().dg_measure_fma_peak(1, ctypes.byref(peak32)), "fma peak fp32")
    peak = peak64.value if args.precision == "fp64" else peak32.value
    vol_flops = ALG_FLOPS_N7["volume"] * nDOF
    achieved = vol_flops / (kms["volume"] * 1e-3) * 1e-12
    mp = measured_peaks()
    hbm_peak = mp.get("hbm_gbs", 6800.0)
    stage_s = kms["stage"] * 1e-3
    alg_b = ALG_BYTES_N7 if args.precision == "fp64" else ALG_BYTES_N7_MIXED
    roofline = {
        "kernel": ("k_volume" if args.precision == "fp64" else "k_volume_lines") +
                  " (split-form volume + viscous volume + surface integral + Jacobian + RK stage)",
        "bound": "fp64" if args.precision == "fp64" else "fp32",
        "achieved": achieved, "peak": peak * 1e-3, "unit": "TFLOP/s", "frac": achieved / (peak * 1e-3),
        "peak_source": "FMA-chain microkernel measured in this run (no FP64/FP32 CUDA-core peak in MEASURED_PEAKS.json)",
        "alg_flops_per_dof": ALG_FLOPS_N7["volume"],
        "traffic": DRAM_BYTES_PER_DOF[args.precision]["volume"] * nDOF,
        "traffic_source": "dram__bytes_read+write per DOF of one launch, scaled by nDOF (%s)" % CAPTURE[args.precision],
        # executed FP64 instructions (captured per DOF) over the FP64 issue capacity at the SM clock
        # sampled during the timed region
        "exec_fp64_issue_frac": (KVOL_FP64_INSTR_PER_DOF * nDOF / (kms["volume"] * 1e-3))
                                / (FP64_ISSUE_PER_CYCLE * (sm_mhz or 2070.0) * 1e6) if args.precision == "fp64" else None,
        "kernel_ms": kms,
        "stage": {"alg_flops_per_dof_stage": sum(ALG_FLOPS_N7.values()),
                  "achieved_tflops": sum(ALG_FLOPS_N7.values()) * nDOF / stage_s * 1e-12,
                  "alg_bytes_per_dof_stage": alg_b,
                  "traffic_per_dof_stage": sum(DRAM_BYTES_PER_DOF[args.precision].values()),
                  "traffic_per_dof_by_kernel": DRAM_BYTES_PER_DOF[args.precision],
                  "hbm_gbs_alg": alg_b * nDOF / stage_s * 1e-9,
                  "hbm_peak_gbs": hbm_peak,
                  "hbm_peak_source": "MEASURED_PEAKS.json" if "hbm_gbs" in mp else "fallback 6.8 TB/s",
                  "hbm_frac_of_measured": alg_b * nDOF / stage_s * 1e-9 / hbm_peak},
        "fp64_peak_tflops_measured": peak64.value * 1e-3,
        "fp32_peak_tflops_measured": peak32.value * 1e-3,
    }
    return roofline


def main():
    args = parse()
    world, rank, local = dist_init(args)
    if args.only:
        import torch
        torch.cuda.set_device(local)
        stream = torch.cuda.current_stream()
        if args.only == "adjoint":
            res = adjoint_tgv(stream, steps=args.adjoint_steps or 200, fd_dirs=args.adjoint_fd)
        elif args.only == "scale64":
            # the 64^3 case: 100 LSERK steps per form and a 50-step adjoint window unless given
            res = scale_c5(stream, steps=args.steps if args.steps_given else 100, adj_steps=args.adjoint_steps or 50)
        elif args.only == "mixed_tgv":
            res = mixed_vs_fp64_tgv(args.workload, args.steps, stream)
        elif args.only == "vortex":
            res = vortex_c1(stream)
        else:
            res = mixed_vs_fp64_curved_br2(stream, steps=args.steps, ne=args.curved_ne)
        if rank == 0:
            print(json.dumps({"only": args.only, **res}), flush=True)
        return
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_ours(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
