"""EXC+VXC time per SCF iteration on one GB300.

  python bench.py [--steps K] [--warmup W] [--impl gb300|reference]
                  [--config IDX] [--lwd Default|GB300-FP64|GB300-Mixed]

Default: workload 4 (256 waters, PBE, 15360 bf) on the tensor-core path
("GB300-Mixed"), with the plain FP64 device path run once beside it for the
speed-up and the |dEXC| / max|dVXC| check, and workload 3 (64 clusters, every
SCF iteration one CUDA-graph launch) measured after it on the batched path
(`batched`; --no-batched skips it).  --config 3 makes the batched case the
headline.

The integrator runs on one GPU: with --gpus N > 1 (or WORLD_SIZE > 1) this
arm prints one "unavailable" line and exits 0.

A step is one eval_exc_vxc(P) call of the workload: the device-resident plan
(tasks, SSF weights, maps) is built during the untimed warm-up; each timed
call copies P in, runs the whole XC pass and copies VXC out.
  value  -- device time of the XC pass with P already in HBM (CUDA events on
            the library's stream, from after the P copy to before the VXC copy)
  e2e    -- wall time of the public C-ABI call with pinned host P / VXC
            (host->device copy, XC pass, device->host copy, synchronize)
--impl reference times the CPU restatement of the reference host integrator
(oracle/: per-task collocation, BLAS dgemm / dsyr2k contractions as in the
reference host driver, OpenMP over tasks on all host cores, tasks in the
reference's npts*nbe order) on a fixed strided sample of the same tasks (the
same sample as the cpu_baseline leg of the default arm), extrapolated to one
full iteration: the per-call fixed cost (VXC zeroing and symmetrization) once,
the rest by the sample's share of sum npts*nbe^2 (the contractions' work).
"""
import argparse
import json
import os
import platform
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "EXC+VXC time/SCF iter on 1 GB300: mixed-prec batched vs FP64 GPU at |ΔEXC|≤1e-8 Eh"
WORKLOADS = {
    0: "1 water, SVWN5, MK 75x302 unpruned, 60 bf",
    1: "32 waters (10 A cube), PBE, MK 99x590 Treutler, 1920 bf, nocc 160",
    2: "96 waters (14 A cube), PBE, MK 75x302 Treutler, 5760 bf, nocc 480",
    3: "64 clusters of 1-40 waters, half SVWN5 / half PBE, MK 75x302 Treutler, batch 128-1024, "
       "one CUDA-graph launch per SCF iteration",
    4: "256 waters (20 A cube), PBE, MK 75x302 Treutler, tol 1e-12, 15360 bf, nocc 1280",
    5: "profiling case: 4 waters (6 A cube), PBE, MK 99x590 Treutler, 240 bf",
}
# Slice-pair products per emulated FP64 product (6 digits, levels i + j <= 5).
SLICE_PAIRS = 21
KCLASSES = ["collocation", "density", "zmat", "vxc", "other", "phi_digits", "p_digits"]


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


def cpu_model():
    """CPU model name and core count of this host."""
    name = None
    try:
        out = subprocess.run(["lscpu"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL,
                             text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.lower().startswith("model name"):
                name = ln.split(":", 1)[1].strip()
                break
    except (OSError, subprocess.SubprocessError):
        pass
    if not name:
        try:
            for ln in open("/proc/cpuinfo"):
                if ln.lower().startswith(("model name", "cpu model")):
                    name = ln.split(":", 1)[1].strip()
                    break
        except OSError:
            pass
    return f"{name or platform.processor() or platform.machine()} ({platform.machine()})"


def peaks():
    pp = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(pp):
        try:
            return json.load(open(pp)), "MEASURED_PEAKS.json"
        except (ValueError, OSError):
            pass
    return {}, None


def tensor_peak():
    pk, src = peaks()
    if pk.get("bf16_tflops_sustained"):
        return float(pk["bf16_tflops_sustained"]), "bf16_tflops_sustained (of measured)"
    return 1700.0, "sustained bf16 1.7 PFLOP/s (of fallback)"


def traffic_ratios():
    """DRAM bytes per algorithmic byte of each kernel class, from the small-case
    ncu capture summarised in profiles/roofline_traffic.json."""
    tp = os.path.join(ROOT, "profiles", "roofline_traffic.json")
    try:
        d = json.load(open(tp))
    except (OSError, ValueError):
        return {}, None
    return d.get("dram_bytes_per_algorithmic_byte", {}), d.get("case")


# ---------------------------------------------------------------------- workload
def config_dict(idx, stats_list, nbfs):
    """Workload description shared by both arms (same keys and values)."""
    d = dict(workload=WORKLOADS.get(idx, str(idx)), config_index=idx,
             nbf=int(max(nbfs)) if len(nbfs) == 1 else int(sum(nbfs)),
             ntasks=int(sum(s["ntasks"] for s in stats_list)),
             npts=int(sum(s["npts"] for s in stats_list)),
             l2=l2_note(sum(n * n * 8 for n in nbfs)))
    if len(nbfs) > 1:
        d["members"] = len(nbfs)
    return d


def l2_note(pbytes):
    state = ("larger than the 129 MB L2, no flush needed" if 2 * pbytes > 129e6
             else "within L2 (small case)")
    return f"P and VXC {pbytes / 1e9:.2f} GB each per step, {state}"


def host_stats(lb):
    infos = [lb.task_info(i) for i in range(lb.ntasks())]
    return dict(ntasks=len(infos), npts=sum(i["npts"] for i in infos)), infos


def setup_workload(cfg_idx, lwd, atom_stride=1):
    import gauxc_gb300 as g
    from gauxc_gb300 import workloads as W
    cfg = W.config(cfg_idx)
    s = cfg["systems"][0]
    t0 = time.perf_counter()
    mol, basis, mg, lb = W.build_system(s)
    t_lb = time.perf_counter() - t0
    if atom_stride > 1:
        # the tasks of every atom_stride-th atom: the full system's per-atom
        # blocks and P gathers on a fraction of the points (profiling case)
        keep = [i for i in range(lb.ntasks()) if lb.task_info(i)["iParent"] % atom_stride == 0]
        lb = lb.subset(keep)
    t0 = time.perf_counter()
    mw = g.MolecularWeightsFactory(g.ExecutionSpace.Device).get_instance()
    mw.modify_weights(lb)
    t_w = time.perf_counter() - t0
    integ = g.XCIntegratorFactory(g.ExecutionSpace.Device, "Replicated", "Default", lwd,
                                  "Default").get_instance(g.functional_type(s["functional"]), lb)
    return dict(cfg=cfg, sys=s, mol=mol, basis=basis, lb=lb, integ=integ, t_lb=t_lb, t_w=t_w)


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
    return a, v, pinned


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
# sum npts*nbe^2 of the timed sample: about 7 s of oracle work on 16
# Neoverse-V2 cores; a workload holding less is timed in full
CPU_SAMPLE_WORK = 3.0e11


def cpu_sample(infos, work=CPU_SAMPLE_WORK):
    """Deterministic stratified sample of the tasks holding about `work` of
    sum npts*nbe^2: one task of every k in the reference's order (npts*nbe
    descending), listed in that order; all tasks when the workload holds
    less.  Returns (task indices, their share of sum npts*nbe^2, k)."""
    order = sorted(range(len(infos)), key=lambda i: (-infos[i]["npts"] * infos[i]["nbe"], i))
    cost = np.array([infos[i]["npts"] * infos[i]["nbe"] ** 2 for i in range(len(infos))], float)
    total = cost.sum()
    stride = 1 if work >= total else max(1, int(round(total / work)))
    # one task from each run of `stride` consecutive tasks, at a seeded offset:
    # a fixed offset would alias with the molecule's repeat (equal tasks of
    # equivalent atoms sit side by side), so that the sample revisits a few
    # atoms' P and VXC blocks, which the full pass never does
    off = np.random.default_rng(stride).integers(0, stride, -(-len(order) // stride))
    pick = [order[b * stride + o] for b, o in enumerate(off) if b * stride + o < len(order)]
    return pick, cost[pick].sum() / total, stride


class WeightedSample:
    """Tasks of a sample with SSF weights from the oracle (host algorithm),
    computed once for the sampled points only."""

    def __init__(self, lb, coords, pick):
        import oracle
        self.tasks = []
        for i in pick:
            t = lb.task(i)
            n = t["npts"]
            w = oracle.ssf_weights(t["points"], np.full(n, t["iParent"], np.int32),
                                   np.full(n, t["dist_nearest"]), coords, t["weights"])
            self.tasks.append((t["points"], w, t["shell_list"]))


def oracle_basis(basis):
    import oracle
    l, pure, nprim, alpha, coeff, origin, _ = basis.arrays()
    return oracle.Basis(l, pure, nprim, alpha, coeff, origin)


def cpu_leg(basis, lb, mol, P, func, work=CPU_SAMPLE_WORK, infos=None):
    """One oracle pass over a bounded sample of the workload, after a warm-up
    pass, extrapolated to the full task list.  The per-call cost that does
    not depend on the tasks (VXC zeroing and symmetrization over nbf^2,
    argument marshalling), timed as a call on no tasks, counts once; the
    rest scales by the sample's share of sum npts*nbe^2."""
    import oracle
    if infos is None:
        infos = [lb.task_info(i) for i in range(lb.ntasks())]
    ob = oracle_basis(basis)
    pick, share, stride = cpu_sample(infos, work)
    ws = WeightedSample(lb, mol.coords(), pick)
    fixed = []
    for _ in range(2):
        t0 = time.perf_counter()
        oracle.eval_exc_vxc(ob, [], P, func)
        fixed.append(time.perf_counter() - t0)
    leg = dict(ws=ws, ob=ob, pick=pick, share=float(share), stride=stride, fixed=min(fixed),
               ntasks=len(infos), blas=oracle.blas_active())
    oracle.eval_exc_vxc(ob, ws.tasks, P, func)
    t0 = time.perf_counter()
    oracle.eval_exc_vxc(ob, ws.tasks, P, func)
    leg["dt"] = time.perf_counter() - t0
    leg["est"] = extrapolate(leg, leg["dt"])
    return leg


def extrapolate(leg, dt):
    """Full-iteration estimate from one timed pass over the leg's sample."""
    return leg["fixed"] + max(dt - leg["fixed"], 0.0) / leg["share"]


def cpu_baseline_dict(leg, value, cores, sample, extrapolated):
    """The line's cpu_baseline object (plain JSON types)."""
    return dict(value=float(value), unit="s", cores=int(cores), kind="port", cpu=cpu_model(),
                blas=bool(leg["blas"]), sample=sample, extrapolated=bool(extrapolated))


def sample_note(leg, dt):
    if leg["share"] >= 1.0:
        return f"all {leg['ntasks']} tasks (npts*nbe order, as the reference runs them), {dt:.2f} s"
    return (f"{len(leg['pick'])} of {leg['ntasks']} tasks (one of every {leg['stride']} in the "
            f"reference's npts*nbe order, run in that order) = {leg['share']:.4f} of sum "
            f"npts*nbe^2, {dt:.2f} s per pass after a warm-up pass; the per-call fixed cost "
            f"{leg['fixed']:.2f} s (VXC zeroing and symmetrization) counted once, the rest "
            f"extrapolated by that share")


# ---------------------------------------------------------------------- reference arm
def run_reference(args, ncores):
    """The reference's host algorithm (oracle port, BLAS contractions) on the
    host cores, on a fixed strided sample of the workload's tasks."""
    import oracle
    from gauxc_gb300 import workloads as W
    cfg = W.config(args.config)
    systems = cfg["systems"]
    built = [(sd,) + tuple(W.build_system(sd, device=False)) for sd in systems]
    stats, nbfs, costs, all_infos = [], [], [], []
    for sd, mol, basis, mg, lb in built:
        st, infos = host_stats(lb)
        stats.append(st)
        nbfs.append(sd["nbf"])
        costs.append(sum(i["npts"] * i["nbe"] ** 2 for i in infos))
        all_infos.append(infos)
    # the largest system is timed; the others count by their share of
    # sum npts*nbe^2 (batched workload)
    k = int(np.argmax(costs))
    scale = sum(costs) / costs[k]
    sd, mol, basis, mg, lb = built[k]
    leg = cpu_leg(basis, lb, mol, sd["P"], sd["functional"], args.cpu_work, all_infos[k])
    times, dts = [], []
    for it in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        oracle.eval_exc_vxc(leg["ob"], leg["ws"].tasks, sd["P"], sd["functional"])
        dt = time.perf_counter() - t0
        if it >= args.warmup:
            dts.append(dt)
            times.append(extrapolate(leg, dt) * scale)
    v = float(np.mean(times))
    sample = (("largest member: " if len(built) > 1 else "") + sample_note(leg, float(np.mean(dts)))
              + (f", x{scale:.2f} for all members by sum npts*nbe^2" if len(built) > 1 else ""))
    line = dict(metric=METRIC, value=v, unit="s", n_gpus=args.gpus, steps=args.steps,
                warmup=args.warmup, ms_per_step=v * 1e3, higher_is_better=False,
                scaling="weak", vs_baseline=None, dtype="f64",
                data="synthetic: seeded water clusters, even-tempered basis, P=CC^T (no dataset)",
                config=config_dict(args.config, stats, nbfs), impl="reference",
                cpu_baseline=cpu_baseline_dict(leg, v, ncores, sample,
                                               leg["share"] < 1.0 or len(built) > 1),
                e2e=dict(value=v, unit="s", h2d_bytes_per_step=0, d2h_bytes_per_step=0))
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------- batched
def batched_side(steps=3):
    """The 64-cluster workload (workload 3) on the batched one-graph path,
    measured beside the headline: every member's whole call (P in, kernels,
    VXC and EXC out) in one CUDA-graph launch per SCF iteration."""
    import gauxc_gb300 as g
    from gauxc_gb300 import workloads as W
    cfg = W.config(3)
    t0 = time.perf_counter()
    mw = g.MolecularWeightsFactory(g.ExecutionSpace.Device).get_instance()
    f = g.XCIntegratorFactory(g.ExecutionSpace.Device, "Replicated", "Default", "GB300-Mixed",
                              "Default")
    integs, Ps = [], []
    for sd in cfg["systems"]:
        mol, basis, mg, lb = W.build_system(sd)
        mw.modify_weights(lb)
        integ = f.get_instance(g.functional_type(sd["functional"]), lb)
        integ.set_plan_params(scratch_gb=3.0)  # the members share the GPU
        integs.append(integ)
        Ps.append(np.asfortranarray(sd["P"]))
    Vs = [np.zeros_like(P, order="F") for P in Ps]
    batch = g.IntegratorBatch(integs)
    for _ in range(2):  # the first call captures the graph
        batch.eval_exc_vxc(Ps, Vs)
    t_setup = time.perf_counter() - t0
    comp, wall = [], []
    for _ in range(steps):
        t1 = time.perf_counter()
        batch.eval_exc_vxc(Ps, Vs)
        wall.append(time.perf_counter() - t1)
        comp.append(batch.timings()["compute_ms"] * 1e-3)
    tm = batch.timings()
    return dict(workload=WORKLOADS[3], members=len(integs), value=float(np.mean(comp)),
                unit="s", e2e=float(np.mean(wall)), steps=steps,
                graph_launches_per_step=int(tm.get("graph_launch", 1)),
                gpu_launches_per_step=int(tm.get("gpu_launches", 0)),
                setup_s=t_setup, plan="default (no autotune), 3 GB work space per member")


def run_batched(args, ncores):
    """The batched workload: every cluster's EXC+VXC in one graph launch."""
    import gauxc_gb300 as g
    from gauxc_gb300 import workloads as W
    g.set_device(0)
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
    sampler = ClockSampler(0)
    sampler.start()
    comp, wall = [], []
    t_all0 = time.perf_counter()
    for _ in range(args.steps):
        t0 = time.perf_counter()
        exc = batch.eval_exc_vxc(Ps, Vs)
        wall.append(time.perf_counter() - t0)
        comp.append(batch.timings()["compute_ms"] * 1e-3)
    t_all = time.perf_counter() - t_all0
    clocks = sampler.stop()
    value = float(np.mean(comp))
    e2e = float(np.mean(wall))
    stats = [i.plan_stats() for i in integs]
    nbfs = [P.shape[0] for P in Ps]
    launches = int(batch.timings()["gpu_launches"])
    s2 = sum(st["sum_npts_nbe2"] for st in stats)
    if mixed:
        peak, src = tensor_peak()
        alg = SLICE_PAIRS * 4.0 * s2
        issued = sum(st["tensor_flops_x"] + st["tensor_flops_v"] for st in stats)
        roofline = dict(bound="tensor", kernel="whole graph (all stages of all members)",
                        achieved=alg / value / 1e12, peak=peak, unit="TFLOP/s",
                        frac=alg / value / 1e12 / peak, traffic=None, peak_source=src,
                        algorithmic_flops_per_step=alg, issued_flops_per_step=issued,
                        issued_over_algorithmic=issued / alg)
    else:
        fp64_peak = g.measure_fp64_peak()
        fl = 4.0 * s2
        roofline = dict(bound="fp64", kernel="whole graph (all stages of all members)",
                        achieved=fl / value / 1e12, peak=fp64_peak, unit="TFLOP/s",
                        frac=fl / value / 1e12 / fp64_peak, traffic=None,
                        peak_source="FP64 FMA probe measured in this run",
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
        k = int(np.argmax([st["sum_npts_nbe2"] for st in stats]))
        s, mol, basis, mg, lb = systems[k]
        leg = cpu_leg(basis, lb, mol, s["P"], s["functional"], args.cpu_work)
        scale = s2 / stats[k]["sum_npts_nbe2"]
        cpu = cpu_baseline_dict(
            leg, leg["est"] * scale, os.cpu_count() or 1,
            "largest cluster: " + sample_note(leg, leg["dt"])
            + f", x{scale:.2f} for all {len(systems)} clusters by sum npts*nbe^2",
            leg["share"] < 1.0 or len(systems) > 1)
    line = dict(
        metric=METRIC, value=value, unit="s", n_gpus=1, steps=args.steps,
        warmup=args.warmup, ms_per_step=value * 1e3, higher_is_better=False, scaling="weak",
        vs_baseline=None,
        dtype="bf16 digits (6 x 7 bit FP64 emulation, FP64 accumulate)" if mixed else "f64",
        data="synthetic: seeded water clusters, even-tempered basis, P=CC^T (no dataset)",
        config=config_dict(args.config, stats, nbfs), path=dict(lwd=args.lwd, parallelism="1 GPU"),
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
    ap.add_argument("--cpu-work", type=float, default=CPU_SAMPLE_WORK,
                    help="CPU legs: sum npts*nbe^2 of the timed task sample")
    ap.add_argument("--scratch-gb", type=float, default=0.0,
                    help="cap of the plan's work space per pass (0 = from free memory)")
    ap.add_argument("--atom-stride", type=int, default=1,
                    help="profiling case: only the tasks of every k-th atom (default: all)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64-check", action="store_true",
                    help="mixed path: skip the FP64 device pass used for dEXC / dVXC")
    ap.add_argument("--no-autotune", action="store_true",
                    help="batched workload: keep the default plan parameters")
    ap.add_argument("--no-batched", action="store_true",
                    help="headline workload: skip the 64-cluster batched measurement beside it")
    args = ap.parse_args()
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    ncores = os.cpu_count() or 1

    if args.impl == "reference":
        # CPU only: under torchrun rank 0 alone runs it
        return run_reference(args, ncores) if rank == 0 else 0

    if ws > 1 or args.gpus > 1:
        if rank == 0:
            print(json.dumps(dict(metric=METRIC, impl="gb300", n_gpus=max(ws, args.gpus),
                                  unavailable="single-GPU path: the XC integrator runs on one "
                                              "GPU per process (replicas only, no multi-GPU "
                                              "mode)")), flush=True)
        return 0

    import gauxc_gb300 as g

    if args.config == 3:
        return run_batched(args, ncores)

    g.set_device(0)
    ctx = setup_workload(args.config, args.lwd, args.atom_stride)
    integ, s = ctx["integ"], ctx["sys"]
    if args.scratch_gb > 0:
        integ.set_plan_params(scratch_gb=args.scratch_gb)
    P, V, pinned = pinned_like(s["P"])
    nbf = s["nbf"]

    # the first call builds the device plan (point blocks, AO order, digit
    # work lists) and uploads it, then evaluates
    t0 = time.perf_counter()
    eval_into(integ, P, V)
    t_first = time.perf_counter() - t0
    plan_ms = {k: v for k, v in integ.timings().items() if k.startswith("plan")}
    for _ in range(args.warmup - 1):
        eval_into(integ, P, V)
    stats = integ.plan_stats()
    fp64_peak = g.measure_fp64_peak()
    integ.set_profiling(True)

    sampler = ClockSampler(0)
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
        launches += int(integ.plan_stats()["gpu_launches"])
        for k, v in integ.kernel_times().items():
            e = kt.setdefault(k, dict(ms=0.0, launches=0))
            e["ms"] += v["ms"]
            e["launches"] += v["launches"]
    t_all = time.perf_counter() - t_all0
    clocks = sampler.stop()
    integ.set_profiling(False)
    value = float(np.mean(comp))
    e2e = float(np.mean(wall))

    # ---- roofline of the dominant kernel class (algorithmic work)
    mixed = args.lwd.lower() == "gb300-mixed"
    gga = s["functional"] != "SVWN5"
    dom = "density" if kt["density"]["ms"] >= kt["vxc"]["ms"] else "vxc"
    dom_s = kt[dom]["ms"] * 1e-3 / args.steps
    n_launch = kt[dom]["launches"] / args.steps
    s2, s1 = stats["sum_npts_nbe2"], stats["sum_npts_nbe"]
    # FP64 work of the contraction: X = 2 phi P (2 npts nbe^2) or the
    # symmetric rank-2k phi^T Z + Z^T phi on the triangle (2 npts nbe^2)
    f64_alg = 2.0 * s2
    ratios, case = traffic_ratios()
    kb = stats["kernel_bytes"]
    traffic = None
    if mixed and ratios.get(dom):
        traffic = ratios[dom] * kb[dom] / max(n_launch, 1)
    if mixed:
        peak, src = tensor_peak()
        alg = SLICE_PAIRS * f64_alg
        issued = stats["tensor_flops_x"] if dom == "density" else stats["tensor_flops_v"]
        roofline = dict(
            bound="tensor", kernel=f"ozaki_kernel<{'X' if dom == 'density' else 'V'}>",
            achieved=alg / dom_s / 1e12, peak=peak, unit="TFLOP/s",
            frac=alg / dom_s / 1e12 / peak, traffic=traffic, peak_source=src,
            work=f"{SLICE_PAIRS} BF16 slice-pair products x 2 sum(npts nbe^2) FP64 flops per call "
                 "(task nbe, unpadded)",
            algorithmic_flops_per_step=alg, issued_flops_per_step=issued,
            issued_over_algorithmic=issued / alg, issued_frac=issued / dom_s / 1e12 / peak,
            launches_per_step=n_launch, fp64_equivalent_tflops=f64_alg / dom_s / 1e12,
            traffic_algorithmic=kb[dom] / max(n_launch, 1),
            traffic_source=(f"DRAM read+write bytes per algorithmic byte of this kernel from an "
                            f"ncu capture of {case}, times this launch's algorithmic bytes"
                            if traffic else None))
    else:
        roofline = dict(bound="fp64", kernel=dom, achieved=f64_alg / dom_s / 1e12,
                        peak=fp64_peak, unit="TFLOP/s", frac=f64_alg / dom_s / 1e12 / fp64_peak,
                        traffic=None, peak_source="FP64 FMA probe measured in this run (no FP64 "
                                                  "figure in the measured-peaks file)",
                        algorithmic_flops_per_step=f64_alg)

    kernels = {}
    for k, v in kt.items():
        ms = v["ms"] / args.steps
        e = dict(ms_per_step=ms, launches_per_step=v["launches"] / args.steps)
        if kb.get(k):
            e["algorithmic_bytes_per_step"] = kb[k]
            if ms > 0:
                e["algorithmic_gbs"] = kb[k] / (ms * 1e-3) / 1e9
            if mixed and ratios.get(k):
                e["dram_bytes_per_step_est"] = ratios[k] * kb[k]
        kernels[k] = e
    if mixed:
        for k, key in (("density", "tensor_flops_x"), ("vxc", "tensor_flops_v")):
            if k in kernels and kt[k]["ms"] > 0:
                t = kt[k]["ms"] * 1e-3 / args.steps
                kernels[k]["tensor_tflops_issued"] = stats[key] / t / 1e12
                kernels[k]["tensor_tflops_algorithmic"] = SLICE_PAIRS * f64_alg / t / 1e12

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
        i64 = None

    cpu = None
    if not args.no_cpu_baseline:
        leg = cpu_leg(ctx["basis"], ctx["lb"], ctx["mol"], s["P"], s["functional"],
                      args.cpu_work)
        cpu = cpu_baseline_dict(leg, leg["est"], ncores, sample_note(leg, leg["dt"]),
                                leg["share"] < 1.0)

    nel = integ.last_nel()
    batched = None
    if mixed and args.config == 4 and args.atom_stride == 1 and not args.no_batched:
        # the headline workload's integrator (about 100 GB of work space) is
        # released first: the 64 members take 3 GB each
        integ = None
        ctx["integ"] = None
        import gc
        gc.collect()
        batched = batched_side()

    line = dict(
        metric=METRIC, value=value, unit="s", n_gpus=1, steps=args.steps,
        warmup=args.warmup, ms_per_step=value * 1e3, higher_is_better=False, scaling="weak",
        vs_baseline=None,
        dtype="bf16 digits (6 x 7 bit FP64 emulation, FP64 accumulate)" if mixed else "f64",
        data="synthetic: seeded water cluster, even-tempered basis, P=CC^T (no dataset)",
        config=config_dict(args.config, [stats], [nbf]),
        path=dict(lwd=args.lwd, parallelism="1 GPU", nbatches=int(stats["nbatches"]),
                  scratch_gb=stats["scratch_bytes"] / 1e9, atom_stride=args.atom_stride),
        e2e=dict(value=e2e, unit="s", h2d_bytes_per_step=nbf * nbf * 8,
                 d2h_bytes_per_step=nbf * nbf * 8 + 16, pinned=pinned,
                 breakdown_ms={k: float(np.mean(v)) for k, v in brk.items()}),
        roofline=roofline, cpu_baseline=cpu, gpu_launches=launches, clocks=clocks,
        fp64_check=fp64_check, exc=exc, nel=nel, batched=batched,
        grid_points_bf_per_s=s1 / value, kernels=kernels,
        setup_s=dict(load_balancer=ctx["t_lb"], ssf_weights=ctx["t_w"],
                     plan_build_and_first_call=t_first, plan_ms=plan_ms),
        timed_wall_s=t_all)
    print(json.dumps(line), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
