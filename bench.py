"""EXC+VXC time per SCF iteration on one GB300 (replicas across GPUs).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                  [--config IDX] [--lwd Default|GB300-FP64|GB300-Mixed]

Default: workload 4 (256 waters, PBE, 15360 bf) on the tensor-core path
("GB300-Mixed"), with the plain FP64 device path run once beside it for the
speed-up and the |dEXC| / max|dVXC| check.  Workload 3 is the batched case
(64 clusters, every SCF iteration one CUDA-graph launch).

A step is one eval_exc_vxc(P) call of the workload: the device-resident plan
(tasks, SSF weights, maps) is built during the untimed warm-up; each timed
call copies P in, runs the whole XC pass and copies VXC out.
  value  -- device time of the XC pass with P already in HBM (CUDA events on
            the library's stream, from after the P copy to before the VXC copy)
  e2e    -- wall time of the public C-ABI call with pinned host P / VXC
            (host->device copy, XC pass, device->host copy, synchronize)
--impl reference times the CPU restatement of the reference host integrator
(oracle/, OpenMP, all host cores) on a bounded sample of the same tasks and
extrapolates to one full iteration by the sample's share of sum npts*nbe^2.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "EXC+VXC time/SCF iter on 1 GB300: mixed-prec batched vs FP64 GPU at |\u0394EXC|\u22641e-8 Eh"
WORKLOADS = {
    0: "1 water, SVWN5, MK 75x302 unpruned, 60 bf",
    1: "32 waters (10 A cube), PBE, MK 99x590 Treutler, 1920 bf, nocc 160",
    2: "96 waters (14 A cube), PBE, MK 75x302 Treutler, 5760 bf, nocc 480",
    3: "64 clusters of 1-40 waters, half SVWN5 / half PBE, MK 75x302 Treutler, batch 128-1024, "
       "one CUDA-graph launch per SCF iteration",
    4: "256 waters (20 A cube), PBE, MK 75x302 Treutler, tol 1e-12, 15360 bf, nocc 1280",
    5: "profiling case: 4 waters (6 A cube), PBE, MK 99x590 Treutler, 240 bf",
}


class ClockSampler:
    """nvidia-smi clock / throttle-reason samples while the timed region runs."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", str(self.device)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, ValueError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.t.join(timeout=5)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax),
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def init_dist(ws):
    if ws <= 1:
        return None
    import torch.distributed as dist
    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    dist.init_process_group("gloo")
    return dist


def reduce_max(dist, x):
    if dist is None:
        return x
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(dist):
    if dist is not None:
        dist.barrier()


# ---------------------------------------------------------------------- workload
def setup_workload(cfg_idx, lwd):
    import gauxc_gb300 as g
    from gauxc_gb300 import workloads as W
    cfg = W.config(cfg_idx)
    s = cfg["systems"][0]
    t0 = time.perf_counter()
    mol, basis, mg, lb = W.build_system(s)
    t_lb = time.perf_counter() - t0
    tasks0 = None
    t0 = time.perf_counter()
    mw = g.MolecularWeightsFactory(g.ExecutionSpace.Device).get_instance()
    mw.modify_weights(lb)
    t_w = time.perf_counter() - t0
    integ = g.XCIntegratorFactory(g.ExecutionSpace.Device, "Replicated", "Default", lwd,
                                  "Default").get_instance(g.functional_type(s["functional"]), lb)
    return dict(cfg=cfg, sys=s, mol=mol, basis=basis, lb=lb, integ=integ, t_lb=t_lb, t_w=t_w,
                tasks0=tasks0)


def pinned_like(P):
    """Host P / VXC buffers page-locked in place through the library (what an
    SCF code does with the buffers it passes every iteration)."""
    import gauxc_gb300 as g
    a = np.asfortranarray(P).copy(order="F")
    v = np.zeros_like(a, order="F")
    try:
        g.host_register(a)
        g.host_register(v)
        pinned = True
    except Exception:
        pinned = False
    return a, v, pinned, (a, v)


def eval_into(integ, P, V):
    import ctypes
    import gauxc_gb300 as g
    from gauxc_gb300._capi import GauXCStatus, check
    L = g.lib()
    st = GauXCStatus()
    exc = ctypes.c_double()
    n = P.shape[0]
    dp = ctypes.POINTER(ctypes.c_double)
    L.gauxc_integrator_eval_exc_vxc_rks(ctypes.byref(st), integ._h, n, n, P.ctypes.data_as(dp), n,
                                        ctypes.byref(exc), V.ctypes.data_as(dp), n)
    check(st, L)
    return exc.value


# ---------------------------------------------------------------------- CPU baseline
def cpu_sample(lb, target_frac):
    """Deterministic strided sample of the tasks (reference order: npts*nbe desc)."""
    infos = [lb.task_info(i) for i in range(lb.ntasks())]
    order = sorted(range(len(infos)), key=lambda i: -infos[i]["npts"] * infos[i]["nbe"])
    stride = max(1, int(round(1.0 / target_frac)))
    pick = order[::stride]
    cost = np.array([infos[i]["npts"] * infos[i]["nbe"] ** 2 for i in range(len(infos))], float)
    return pick, cost[pick].sum() / cost.sum()


def time_cpu(W, basis, lb, P, func, budget_s=15.0, nthreads=0):
    """Oracle on growing strided samples until one takes >= budget/4; extrapolate."""
    import oracle
    l, pure, nprim, alpha, coeff, origin, _ = basis.arrays()
    ob = oracle.Basis(l, pure, nprim, alpha, coeff, origin)
    frac = 1.0 / 512
    while True:
        pick, share = cpu_sample(lb, frac)
        tasks = [lb.task(i) for i in pick]
        ot = [(t["points"], t["weights"], t["shell_list"]) for t in tasks]
        t0 = time.perf_counter()
        oracle.eval_exc_vxc(ob, ot, P, func, nthreads=nthreads)
        dt = time.perf_counter() - t0
        if dt >= budget_s / 4 or frac >= 1.0:
            return dt / share, dt, len(pick), share
        frac = min(1.0, frac * max(2.0, min(8.0, (budget_s / 4) / max(dt, 1e-3))))


# ---------------------------------------------------------------------- batched
def run_batched(args, dist, rank, local, ncores):
    """The batched workload: every cluster's EXC+VXC in one graph launch."""
    import gauxc_gb300 as g
    from gauxc_gb300 import workloads as W
    g.set_device(local)
    cfg = W.config(args.config)
    t0 = time.perf_counter()
    systems = []
    for s in cfg["systems"]:
        mol, basis, mg, lb = W.build_system(s)
        systems.append((s, mol, basis, mg, lb))
    t_lb = time.perf_counter() - t0
    t0 = time.perf_counter()
    mw = g.MolecularWeightsFactory(g.ExecutionSpace.Device).get_instance()
    for s, mol, basis, mg, lb in systems:
        mw.modify_weights(lb)
    t_w = time.perf_counter() - t0

    def make(lwd):
        f = g.XCIntegratorFactory(g.ExecutionSpace.Device, "Replicated", "Default", lwd, "Default")
        return [f.get_instance(g.functional_type(s["functional"]), lb)
                for s, mol, basis, mg, lb in systems]

    mixed = args.lwd.lower() == "gb300-mixed"
    integs = make(args.lwd)
    for integ in integs:  # the members share the GPU: 3 GB of work space each
        integ.set_plan_params(scratch_gb=3.0)
    Ps = [np.asfortranarray(s["P"]) for s, *_ in systems]
    Vs = [np.zeros_like(P, order="F") for P in Ps]
    tune = None
    if mixed and not args.no_autotune:
        t0 = time.perf_counter()
        choice = {}
        for integ, P in zip(integs, Ps):
            ms, prm = integ.autotune(P)
            key = (prm["pb_max_pts"], prm["nu2_weight"])
            choice[key] = choice.get(key, 0) + 1
        tune = dict(seconds=time.perf_counter() - t0,
                    chosen={f"pts{k[0]}_w{int(k[1])}": v for k, v in sorted(choice.items())})
    batch = g.IntegratorBatch(integs)
    for _ in range(max(args.warmup, 2)):  # the first call captures the graph
        batch.eval_exc_vxc(Ps, Vs)
    sampler = ClockSampler(local)
    barrier(dist)
    sampler.start()
    comp, wall = [], []
    t_all0 = time.perf_counter()
    for _ in range(args.steps):
        t0 = time.perf_counter()
        exc = batch.eval_exc_vxc(Ps, Vs)
        wall.append(time.perf_counter() - t0)
        tm = batch.timings()
        comp.append(tm["compute_ms"] * 1e-3)
    t_all = time.perf_counter() - t_all0
    barrier(dist)
    clocks = sampler.stop()
    value = reduce_max(dist, float(np.mean(comp)))
    e2e = reduce_max(dist, float(np.mean(wall)))
    if rank != 0:
        return 0
    stats = [i.plan_stats() for i in integs]
    nbfs = [P.shape[0] for P in Ps]
    launches = int(batch.timings()["gpu_launches"])
    if mixed:
        peaks = {}
        pp = os.path.join(ROOT, "MEASURED_PEAKS.json")
        if os.path.exists(pp):
            peaks = json.load(open(pp))
        peak = peaks.get("bf16_tflops_sustained")
        src = "MEASURED_PEAKS.json bf16_tflops_sustained (of measured)"
        if peak is None:
            peak, src = 1700.0, "fallback sustained bf16 1.7 PFLOP/s (of fallback)"
        fl = sum(st["tensor_flops_x"] + st["tensor_flops_v"] for st in stats)
        achieved = fl / value / 1e12
        roofline = dict(bound="tensor", kernel="whole graph (all stages of all members)",
                        achieved=achieved, peak=peak, unit="TFLOP/s", frac=achieved / peak,
                        traffic=None, peak_source=src, algorithmic_flops_per_step=fl)
    else:
        fp64_peak = g.measure_fp64_peak()
        fl = sum(4.0 * st["sum_npts_nbe2"] for st in stats)
        achieved = fl / value / 1e12
        roofline = dict(bound="fp64", kernel="whole graph (all stages of all members)",
                        achieved=achieved, peak=fp64_peak, unit="TFLOP/s", frac=achieved / fp64_peak,
                        traffic=None, peak_source="FP64 FMA probe measured in this run",
                        algorithmic_flops_per_step=fl)
    fp64_check = None
    if mixed and not args.no_fp64_check:
        batch = integs = None  # release the mixed plans first
        i64 = make("GB300-FP64")
        V64 = [np.zeros_like(P, order="F") for P in Ps]
        b64 = g.IntegratorBatch(i64)
        for _ in range(3):
            e64 = b64.eval_exc_vxc(Ps, V64)
        t64 = b64.timings()["compute_ms"] * 1e-3
        fp64_check = dict(delta_exc=float(np.abs(exc - e64).max()),
                          max_delta_vxc=float(max(np.abs(a - b).max() for a, b in zip(Vs, V64))),
                          fp64_value=t64, speedup_vs_fp64=t64 / value,
                          gates=dict(delta_exc=1e-8, max_delta_vxc=1e-8))
    cpu = None
    if not args.no_cpu_baseline:
        # oracle on a sample of the largest member, scaled by sum npts*nbe^2
        k = int(np.argmax([st["sum_npts_nbe2"] for st in stats]))
        s, mol, basis, mg, lb = systems[k]
        est, dt, ntask, share = time_cpu(W, basis, lb, s["P"], s["functional"],
                                         budget_s=args.cpu_budget)
        tot = sum(st["sum_npts_nbe2"] for st in stats)
        scale = tot / stats[k]["sum_npts_nbe2"]
        cpu = dict(value=est * scale, unit="s", cores=ncores, kind="port",
                   sample=f"{ntask} tasks of the largest cluster ({share:.4f} of its sum "
                          f"npts*nbe^2, {dt:.1f} s), scaled to all {len(systems)} clusters by "
                          f"sum npts*nbe^2")
    line = dict(
        metric=METRIC, value=value, unit="s", n_gpus=args.gpus, steps=args.steps,
        warmup=args.warmup, ms_per_step=value * 1e3, higher_is_better=False, scaling="weak",
        vs_baseline=None,
        dtype="bf16 digits (6 x 7 bit FP64 emulation, FP64 accumulate)" if mixed else "f64",
        data="synthetic: seeded water clusters, even-tempered basis, P=CC^T (no dataset)",
        config=dict(workload=WORKLOADS[args.config], config_index=args.config, lwd=args.lwd,
                    members=len(systems), nbf_total=int(sum(nbfs)), nbf_max=int(max(nbfs)),
                    npts=int(sum(st["npts"] for st in stats)),
                    ntasks=int(sum(st["ntasks"] for st in stats)),
                    l2="inputs larger than L2 (sum of members' P and VXC)",
                    parallelism=f"replicas x{args.gpus}"),
        e2e=dict(value=e2e, unit="s", h2d_bytes_per_step=int(sum(n * n * 8 for n in nbfs)),
                 d2h_bytes_per_step=int(sum(n * n * 8 + 16 for n in nbfs)), pinned=True),
        roofline=roofline, cpu_baseline=cpu, gpu_launches=launches,
        graph_launches_per_step=1, clocks=clocks, fp64_check=fp64_check, autotune=tune,
        grid_points_bf_per_s=sum(st["sum_npts_nbe"] for st in stats) / value,
        exc_sum=float(np.sum(exc)),
        setup_s=dict(load_balancer=t_lb, ssf_weights=t_w), timed_wall_s=t_all)
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------- main
def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    # default: the headline workload (256 waters, PBE) on the tensor-core path,
    # with the FP64 device path timed beside it for the speed-up and the errors
    ap.add_argument("--config", type=int, default=4)
    ap.add_argument("--lwd", default="GB300-Mixed")
    ap.add_argument("--cpu-budget", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64-check", action="store_true",
                    help="mixed path: skip the FP64 device pass used for dEXC / dVXC")
    ap.add_argument("--no-autotune", action="store_true",
                    help="batched workload: keep the default plan parameters")
    args = ap.parse_args()
    ws, rank, local = dist_env()
    dist = init_dist(ws)
    if ws > 1:
        # cluster multicast of GEMM operands only in single-GPU runs
        os.environ.setdefault("GAUXC_GB300_CLUSTER_MULTICAST", "0")

    import gauxc_gb300 as g
    from gauxc_gb300 import workloads as W

    ncores = os.cpu_count() or 1
    if args.impl == "reference":
        if rank != 0:
            return 0
        systems = W.config(args.config)["systems"]
        scale = 1.0
        if len(systems) > 1:
            # batched workload: the largest cluster is timed, the others are
            # accounted for by sum npts*nbe^2 of their (host-built) task lists
            costs = []
            for sd in systems:
                lbx = W.build_system(sd, device=False)[3]
                costs.append(sum(lbx.task_info(i)["npts"] * lbx.task_info(i)["nbe"] ** 2
                                 for i in range(lbx.ntasks())))
            k = int(np.argmax(costs))
            scale = sum(costs) / costs[k]
            s = systems[k]
        else:
            s = systems[0]
        mol, basis, mg, lb = W.build_system(s, device=False)
        # the reference integrator needs weighted tasks: SSF by the CPU oracle,
        # for the points of the sampled tasks only
        lbw = _SampledWeightedTasks(lb, mol)
        times = []
        for it in range(args.warmup + args.steps):
            est, dt, ntask, share = time_cpu(W, basis, lbw, s["P"], s["functional"],
                                             budget_s=args.cpu_budget / 2)
            if it >= args.warmup:
                times.append(est * scale)
        v = float(np.mean(times))
        line = dict(metric=METRIC, value=v, unit="s", n_gpus=args.gpus, steps=args.steps,
                    warmup=args.warmup, ms_per_step=v * 1e3, higher_is_better=False,
                    scaling="weak", vs_baseline=None, dtype="f64",
                    data="synthetic: seeded water cluster, even-tempered basis, P=CC^T",
                    config=dict(workload=WORKLOADS.get(args.config, str(args.config)),
                                config_index=args.config),
                    impl="reference",
                    cpu_baseline=dict(value=v, unit="s", cores=ncores, kind="port",
                                      sample=f"{ntask} of {lb.ntasks()} tasks (strided over the "
                                             f"npts*nbe order), {share:.4f} of sum npts*nbe^2, "
                                             f"extrapolated"),
                    e2e=dict(value=v, unit="s", h2d_bytes_per_step=0, d2h_bytes_per_step=0))
        print(json.dumps(line), flush=True)
        return 0

    if args.config == 3:
        return run_batched(args, dist, rank, local, ncores)

    g.set_device(local)
    ctx = setup_workload(args.config, args.lwd)
    integ, s = ctx["integ"], ctx["sys"]
    P, V, pinned, _keep = pinned_like(s["P"])
    nbf = s["nbf"]
    stats = integ.plan_stats()

    for _ in range(args.warmup):
        eval_into(integ, P, V)
    fp64_peak = g.measure_fp64_peak()
    integ.set_profiling(True)

    sampler = ClockSampler(local)
    barrier(dist)
    sampler.start()
    comp, wall, launches = [], [], 0
    kt, brk = {}, {}
    t_all0 = time.perf_counter()
    for _ in range(args.steps):
        t0 = time.perf_counter()
        exc = eval_into(integ, P, V)
        wall.append(time.perf_counter() - t0)
        tm = integ.timings()
        comp.append(tm["compute_ms"] * 1e-3)
        for k in ("h2d_ms", "compute_ms", "d2h_ms", "wall_ms"):
            brk.setdefault(k, []).append(tm.get(k, 0.0))
        st = integ.plan_stats()
        launches += int(st["gpu_launches"])
        for k, v in integ.kernel_times().items():
            e = kt.setdefault(k, dict(ms=0.0, launches=0))
            e["ms"] += v["ms"]
            e["launches"] += v["launches"]
    t_all = time.perf_counter() - t_all0
    barrier(dist)
    clocks = sampler.stop()
    integ.set_profiling(False)

    value = reduce_max(dist, float(np.mean(comp)))
    e2e = reduce_max(dist, float(np.mean(wall)))
    if rank != 0:
        return 0

    # roofline of the dominant kernel class
    mixed = args.lwd.lower() == "gb300-mixed"
    gga = s["functional"] != "SVWN5"
    dom = "density" if kt["density"]["ms"] >= kt["vxc"]["ms"] else "vxc"
    dom_s = kt[dom]["ms"] * 1e-3
    f_x = 2.0 * stats["sum_npts_nbe2"] + 2.0 * stats["sum_npts_nbe"] * (4 if gga else 1)
    f_v = 2.0 * stats["sum_npts_nbe2"]
    f64_flops = (f_x if dom == "density" else f_v) * args.steps
    traffic = None
    tp = os.path.join(ROOT, "profiles", "roofline_traffic.json")
    if os.path.exists(tp):
        try:
            traffic = json.load(open(tp)).get(f"config{args.config}_{args.lwd}_{dom}")
        except (ValueError, OSError):
            traffic = None
    if mixed:
        peaks = {}
        pp = os.path.join(ROOT, "MEASURED_PEAKS.json")
        if os.path.exists(pp):
            peaks = json.load(open(pp))
        peak = peaks.get("bf16_tflops_sustained")
        src = "MEASURED_PEAKS.json bf16_tflops_sustained (of measured)"
        if peak is None:
            peak, src = 1700.0, "fallback sustained bf16 1.7 PFLOP/s (of fallback)"
        tflops = (stats["tensor_flops_x"] if dom == "density" else stats["tensor_flops_v"]) * args.steps
        achieved = tflops / dom_s / 1e12
        roofline = dict(bound="tensor", kernel=f"ozaki_kernel<{'X' if dom == 'density' else 'V'}>",
                        achieved=achieved, peak=peak, unit="TFLOP/s", frac=achieved / peak,
                        traffic=traffic, peak_source=src,
                        traffic_note=("DRAM read+write bytes per launch (ncu launch list, "
                                      "profiles/launches_mixed_256water.md)" if traffic else None),
                        launches_per_step=kt[dom]["launches"] / args.steps,
                        algorithmic_flops_per_step=tflops / args.steps,
                        fp64_equivalent_tflops=f64_flops / dom_s / 1e12)
    else:
        achieved = f64_flops / dom_s / 1e12
        roofline = dict(bound="fp64", kernel=dom, achieved=achieved, peak=fp64_peak,
                        unit="TFLOP/s", frac=achieved / fp64_peak, traffic=traffic,
                        peak_source="FP64 FMA probe measured in this run (no FP64 figure in the "
                                    "measured-peaks file)",
                        algorithmic_flops_per_step=f64_flops / args.steps)

    fp64_check = None
    if mixed and not args.no_fp64_check:
        i64 = g.XCIntegratorFactory(g.ExecutionSpace.Device, "Replicated", "Default", "GB300-FP64",
                                    "Default").get_instance(g.functional_type(s["functional"]),
                                                            ctx["lb"])
        V64 = np.zeros_like(V)
        e64 = eval_into(i64, P, V64)  # builds the FP64 plan
        e64 = eval_into(i64, P, V64)
        t64 = i64.timings()["compute_ms"] * 1e-3
        fp64_check = dict(exc_fp64=e64, delta_exc=abs(exc - e64),
                          max_delta_vxc=float(np.abs(V - V64).max()),
                          delta_nel=abs(integ.last_nel() - i64.last_nel()),
                          fp64_value=t64, speedup_vs_fp64=t64 / value,
                          gates=dict(delta_exc=1e-8, max_delta_vxc=1e-8))

    cpu = None
    if not args.no_cpu_baseline:
        est, dt, ntask, share = time_cpu(W, ctx["basis"], ctx["lb"], s["P"], s["functional"],
                                         budget_s=args.cpu_budget)
        cpu = dict(value=est, unit="s", cores=ncores, kind="port",
                   sample=f"{ntask} of {int(stats['ntasks'])} tasks (strided over the npts*nbe "
                          f"order) = {share:.4f} of sum npts*nbe^2, {dt:.1f} s, extrapolated")

    line = dict(
        metric=METRIC, value=value, unit="s", n_gpus=args.gpus, steps=args.steps,
        warmup=args.warmup, ms_per_step=value * 1e3, higher_is_better=False, scaling="weak",
        vs_baseline=None,
        dtype="bf16 digits (6 x 7 bit FP64 emulation, FP64 accumulate)" if mixed else "f64",
        data="synthetic: seeded water cluster, even-tempered basis, P=CC^T (no dataset)",
        config=dict(workload=WORKLOADS.get(args.config, str(args.config)), config_index=args.config,
                    lwd=args.lwd, nbf=nbf, ntasks=int(stats["ntasks"]), npts=int(stats["npts"]),
                    nbatches=int(stats["nbatches"]),
                    l2="inputs larger than L2 (scratch %.1f GB per batch)" % (stats["scratch_bytes"] / 1e9),
                    parallelism=f"replicas x{args.gpus}"),
        e2e=dict(value=e2e, unit="s", h2d_bytes_per_step=nbf * nbf * 8,
                 d2h_bytes_per_step=nbf * nbf * 8 + 16, pinned=pinned,
                 breakdown_ms={k: float(np.mean(v)) for k, v in brk.items()}),
        roofline=roofline, cpu_baseline=cpu, gpu_launches=launches, clocks=clocks,
        fp64_check=fp64_check,
        exc=exc, nel=integ.last_nel(),
        grid_points_bf_per_s=stats["sum_npts_nbe"] / value,
        kernels={k: dict(ms_per_step=v["ms"] / args.steps, launches_per_step=v["launches"] / args.steps)
                 for k, v in kt.items()},
        setup_s=dict(load_balancer=ctx["t_lb"], ssf_weights=ctx["t_w"]),
        timed_wall_s=t_all)
    if mixed:
        for k, key in (("density", "tensor_flops_x"), ("vxc", "tensor_flops_v")):
            if k in line["kernels"] and kt[k]["ms"] > 0:
                line["kernels"][k]["tensor_tflops"] = stats[key] * args.steps / (kt[k]["ms"] * 1e-3) / 1e12
    print(json.dumps(line), flush=True)
    return 0


class _SampledWeightedTasks:
    """Load-balancer view whose task() applies SSF weights (CPU oracle) on
    demand, so that only the tasks a CPU sample touches are weighted."""

    def __init__(self, lb, mol):
        self.lb, self.coords, self.cache = lb, mol.coords(), {}

    def ntasks(self):
        return self.lb.ntasks()

    def task_info(self, i):
        return self.lb.task_info(i)

    def task(self, i):
        if i not in self.cache:
            import oracle
            t = dict(self.lb.task(i))
            n = t["npts"]
            t["weights"] = oracle.ssf_weights(t["points"], np.full(n, t["iParent"], np.int32),
                                              np.full(n, t["dist_nearest"]), self.coords,
                                              t["weights"])
            self.cache[i] = t
        return self.cache[i]


class _WeightedTasks:
    """Load-balancer-like view of tasks with replaced weights (CPU reference arm)."""

    def __init__(self, tasks, weights):
        self.tasks = []
        o = 0
        for t in tasks:
            t = dict(t)
            t["weights"] = weights[o:o + t["npts"]]
            o += t["npts"]
            self.tasks.append(t)

    def ntasks(self):
        return len(self.tasks)

    def task_info(self, i):
        return self.tasks[i]

    def task(self, i):
        return self.tasks[i]


if __name__ == "__main__":
    sys.exit(main())
