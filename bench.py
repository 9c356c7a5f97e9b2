"""Benchmark of the FP64 DNC5 residual + JVP hot path on GB300.

Default workload (the largest residual + JVP configuration that fits one GPU):
64 independent laminar boundary layers of uneven size, nx ~ U{200..1200},
ny ~ U{80..300}, Mach ~ U(0.3, 0.8) (default_rng(4), 9.59M interior cells),
Blasius state plus seeded 1e-4 noise, one seeded Gaussian direction per grid.
One step = the residual and one Jacobian-vector product of every grid, run
as one CUDA graph of persistent launches over the tiles of all grids.  The
metric is Mcells/s = interior cells / s (one residual + one JVP per cell).

  value : kernels only, inputs resident in HBM, L2 flushed between steps
  e2e   : through the C ABI (bcg_batch_run_host) with pinned host arrays:
          state, direction and metrics uploaded and the residual and tangent
          interiors downloaded inside the timed region, every step

The 256x256 cylinder line (residual + 32 directions, VJP) rides along as the
key "cylinder_256" (or alone with --workload cylinder); the other workloads
(jacobian, impli, newton, warmstart) print their own lines.

python bench.py [--gpus N --steps K --warmup W] [--impl reference]
Under torchrun each rank runs its own copy of the batch (weak scaling); rank 0
prints one JSON line.  --impl reference times the reference path's CPU
restatement (the oracle port, OpenMP on all host cores) on the same grids,
states and directions.
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
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "FP64 residual+JVP Mcells/s"
UNIT = "Mcells/s"
IM, JM, NDIR, GROUP = 256, 256, 32, 4


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class LibOps:
    """Host pre-processing through the library's host entry points."""

    @staticmethod
    def computegeom(*a):
        from broadcast_gb300.srcfv import f_geom
        f_geom.computegeom_2d(*a)

    @staticmethod
    def initblfv(muinf, xc, yc, w, field, im, gh, jm):
        from broadcast_gb300 import f_init
        f_init.initblfv(muinf, xc, yc, w, field, im, gh, jm)

    @staticmethod
    def set_bndbl(w, field, wbd, im, jm, gh):
        from broadcast_gb300 import f_init
        f_init.set_bndbl_2d(w, field, wbd, im, jm, gh)


def cylinder_bcs(c, w, wd=None):
    """Cylinder boundary sequence of handleBC.applyBC (order Jhi, Jlo, Ilo, Ihi)."""
    from broadcast_gb300.srcfv import f_bnd, f_lin
    g, ph, it = c["grid"], c["phys"], c["interf"]
    im, jm, gh = g["im"], g["jm"], g["gh"]
    if wd is None:
        f_bnd.bc_no_reflexion_2d(w, c["wbd"], "Jhi", it["Jhi"], g["nx"], g["ny"], ph["gam"], gh, im, jm)
        f_bnd.bc_wall_viscous_adia_2d(w, "Jlo", ph["gam"], it["Jlo"], gh, im, jm)
    else:
        f_lin.bc_no_reflexion_2d_d(w, wd, c["wbd"], "Jhi", it["Jhi"], g["nx"], g["ny"], ph["gam"], gh, im, jm)
        f_lin.bc_wall_viscous_adia_2d_d(w, wd, "Jlo", ph["gam"], it["Jlo"], gh, im, jm)
    for _ in range(2):
        for a in ([w] if wd is None else [wd, w]):
            f_bnd.jn_match_2d(a, it["prr1"], gh, gh, gh, gh, im, jm, a, it["prd2"], gh, gh, gh, gh, im, jm, it["tr"])
            f_bnd.jn_match_2d(a, it["prr2"], gh, gh, gh, gh, im, jm, a, it["prd1"], gh, gh, gh, gh, im, jm, it["tr"])


def build_workload():
    from broadcast_gb300 import cases
    c = cases.cyl_case(IM, JM, ops=LibOps)
    cylinder_bcs(c, c["w"])
    rng = np.random.default_rng(2)
    wds = []
    gh = cases.GH
    for _ in range(NDIR):
        wd = np.zeros_like(c["w"], order="F")
        wd[gh:-gh, gh:-gh, :] = rng.standard_normal((IM, JM, 5))
        wtmp = c["w"].copy(order="F")
        cylinder_bcs(c, wtmp, wd)
        wds.append(wd)
    return c, wds


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            t0 = time.perf_counter()  # nvidia-smi takes a moment to print its first sample
            while not self.lines and time.perf_counter() - t0 < 3.0 and self.proc.poll() is None:
                time.sleep(0.01)
        except Exception:
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
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax = float(p[2])
            except ValueError:
                continue
            for n, v in zip(names, p[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons), "samples": len(sm)}


def algorithmic_bytes(im, jm, gh, ndir):
    """Compulsory HBM bytes of one residual + ndir-direction JVP evaluation:
    w and the ndir tangent states (5 per padded cell each), vol and volf (3 per
    padded cell), nx and ny (4 per padded node), residual and ndir tangent
    outputs (5 per interior cell each)."""
    np_ = (im + 2 * gh) * (jm + 2 * gh)
    nn = (im + 2 * gh + 1) * (jm + 2 * gh + 1)
    nc = im * jm
    return 8 * ((5 + 5 * ndir + 3) * np_ + 4 * nn + 5 * (1 + ndir) * nc)


def flop_counts(c):
    from oracle import oracle as O
    primal, tangent, _ = O.opcount(c["grid"], c["phys"], c["w"])
    return primal, tangent


def cpu_baseline(c, wds, seconds=12.0, threads=None):
    """The oracle (C++ restatement of the reference Fortran) with OpenMP on the
    host cores: residual + 1-direction JVP evaluations of the full grid,
    repeated for about `seconds`."""
    from oracle import oracle as O
    if threads:
        os.environ["OMP_NUM_THREADS"] = str(threads)
    O.lib(openmp=True)
    import ctypes
    lib = O.lib(openmp=True)
    g, ph = c["grid"], c["phys"]
    res = np.zeros_like(c["w"], order="F")
    out = np.zeros_like(c["w"], order="F")
    args = (O._p(g["nx"]), O._p(g["ny"]), O._p(g["vol"]), O._p(g["volf"]), g["gh"], *O._phys(ph), g["im"], g["jm"])
    n, t0 = 0, time.perf_counter()
    while True:
        wd = wds[n % len(wds)]
        lib.orc_flux_num_dnc5_2d_d(O._p(res), O._p(out), O._p(c["w"]), O._p(wd), 1, *args)
        n += 1
        el = time.perf_counter() - t0
        if el >= seconds and n >= 2:
            break
    cells = g["im"] * g["jm"] * n
    return {"value": cells / el / 1e6, "unit": UNIT, "cores": threads or os.cpu_count(), "kind": "port",
            "sample": "%d residual+JVP (1 direction) evaluations of the %dx%d cylinder grid, %.1f s" % (n, IM, JM, el)}


def run_reference(args):
    ws, rank, _ = _dist()
    if rank != 0:
        return 0
    from broadcast_gb300 import cases

    class OracleOps:
        from oracle import oracle as _O
        computegeom = staticmethod(_O.computegeom)
        initblfv = staticmethod(_O.initblfv)
        set_bndbl = staticmethod(_O.set_bndbl)

    from oracle import oracle as O
    c = cases.cyl_case(IM, JM, ops=OracleOps)
    g, ph, it = c["grid"], c["phys"], c["interf"]
    w = c["w"]
    O.bc_noref(w, c["wbd"], "Jhi", it["Jhi"], g["nx"], g["ny"], ph["gam"], 3, IM, JM)
    O.bc_wall(w, "Jlo", ph["gam"], it["Jlo"], 3, IM, JM)
    for _ in range(2):
        O.jn_match(w, it["prr1"], (3,) * 4, IM, JM, w, it["prd2"], (3,) * 4, IM, JM, it["tr"], 5)
        O.jn_match(w, it["prr2"], (3,) * 4, IM, JM, w, it["prd1"], (3,) * 4, IM, JM, it["tr"], 5)
    rng = np.random.default_rng(2)
    wds = []
    for _ in range(4):
        wd = np.zeros_like(c["w"], order="F")
        wd[3:-3, 3:-3, :] = rng.standard_normal((IM, JM, 5))
        wds.append(wd)
    lib = O.lib(openmp=True)
    res = np.zeros_like(c["w"], order="F")
    out = np.zeros_like(c["w"], order="F")
    a = (O._p(g["nx"]), O._p(g["ny"]), O._p(g["vol"]), O._p(g["volf"]), g["gh"], *O._phys(ph), g["im"], g["jm"])
    # one step = a bounded sample of the workload: 4 residual+JVP evaluations
    per_step = 4

    def step():
        for k in range(per_step):
            lib.orc_flux_num_dnc5_2d_d(O._p(res), O._p(out), O._p(c["w"]), O._p(wds[k]), 1, *a)

    for _ in range(args.warmup):
        step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    el = time.perf_counter() - t0
    v = IM * JM * per_step * args.steps / el / 1e6
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": el / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "cylinder O-mesh %dx%d, Mach 0.1, Re 47, residual + JVP per direction" % (IM, JM),
                       "directions_per_step": per_step},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
                             "sample": "%d residual+JVP (1 direction) evaluations per step of the %dx%d grid, "
                                       "OpenMP over j-rows" % (per_step, IM, JM)},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


# FP64 lane instructions (warp instructions of the FP64 pipe x 32) and DRAM
# bytes per cell and direction of the passes of the 256x256 cylinder line
# (residual + 32 directions in groups of 4), from one ncu capture of that
# command:
#   ncu --clock-control none -k regex:"k_(prim|qrows|vpts|faces|balance)" -c 10
#       --metrics sm__inst_executed_pipe_fp64.sum,dram__bytes_read.sum,dram__bytes_write.sum
#       python bench.py --workload cylinder --steps 1 --warmup 1 --cpu-seconds 1
# divided by cells x directions.
CYL_NCU = {"fp64_inst_per_cell_dir": 664.9, "dram_bytes_per_cell_dir": 1381.8,
           "source": "ncu sm__inst_executed_pipe_fp64.sum x 32 lanes and DRAM bytes of the five passes of one "
                     "launch half (16 directions), per cell and direction, cold caches"}


def cylinder_measure(args, dev, extras_only=False, ws=1, rank=0):
    """Residual + JVP for NDIR directions on the 256x256 cylinder: kernel time
    (CUDA events, L2 flushed between steps), e2e through
    bcg_flux_num_dnc5_2d_dn with pinned host arrays, and the VJP with one and
    with NDIR cotangents per call."""
    import torch
    from broadcast_gb300 import _lib
    from broadcast_gb300.operator import Dnc5Operator, to_device
    c, wds = build_workload()
    op = Dnc5Operator(c["grid"], c["phys"], device=dev)
    w_dev = to_device(c["w"], dev)
    wd_dev = torch.stack([to_device(x, dev) for x in wds])
    res = op.new_state()
    resd = op.new_state(NDIR)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)  # 256 MB > L2
    stream = torch.cuda.current_stream(dev)
    steps = args.steps if not extras_only else min(args.steps, 10)

    def step():
        # one call: each pass runs the 8 groups of 4 directions as two
        # launches of 4 groups (blockIdx.y = group) on two streams
        op.jvp(w_dev, wd_dev, res=res, resd=resd)

    for _ in range(max(args.warmup, 1)):
        step()
    torch.cuda.synchronize()
    sampler = ClockSampler(dev.index or 0)
    if rank == 0 and not extras_only:
        sampler.start()
    t0 = time.perf_counter()
    while time.perf_counter() - t0 < 0.3:
        step()
        torch.cuda.synchronize()
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    for s_ in range(steps):
        flush.add_(1.0)
        ev[s_][0].record(stream)
        step()
        ev[s_][1].record(stream)
    torch.cuda.synchronize()
    if ws > 1:
        dist.barrier()
    clocks = sampler.stop() if (rank == 0 and not extras_only) else None
    if clocks:
        clocks["window"] = "0.3 s of the same step untimed, then the timed region"
    tot_ms = sum(a.elapsed_time(b) for a, b in ev)
    if ws > 1:
        t = torch.tensor([tot_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        tot_ms = float(t.item())
    out = {"value": IM * JM * NDIR * ws * steps / (tot_ms / 1e3) / 1e6, "unit": UNIT, "ms_per_step": tot_ms / steps,
           "steps": steps, "clocks": clocks,
           "workload": "cylinder O-mesh %dx%d (r 0.5..50 D, stretch 1.05), Mach 0.1, Re 47; residual + JVP for %d "
                       "seeded Gaussian directions per step, L2 flushed between steps" % (IM, JM, NDIR)}
    if rank != 0:
        return out
    # VJP on the same grid, device arrays: one cotangent per call, then NDIR in one call
    rb = torch.zeros_like(res)
    rb[:, 3:-3, 3:-3] = 1.0
    wb = op.new_state()
    op.vjp(w_dev, rb, wb)
    torch.cuda.synchronize()
    a_ev, b_ev = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    nv = 8
    a_ev.record(stream)
    for _ in range(nv):
        op.vjp(w_dev, rb, wb)
    b_ev.record(stream)
    torch.cuda.synchronize()
    vms = a_ev.elapsed_time(b_ev) / nv
    rbs = torch.zeros((NDIR,) + tuple(res.shape), dtype=res.dtype, device=res.device)
    rbs[:, :, 3:-3, 3:-3] = 1.0
    wbs = op.vjp(w_dev, rbs)
    torch.cuda.synchronize()
    a_ev.record(stream)
    for _ in range(2):
        op.vjp(w_dev, rbs, wbs)
    b_ev.record(stream)
    torch.cuda.synchronize()
    bms = a_ev.elapsed_time(b_ev) / 2
    out["vjp"] = {"value": IM * JM / (vms / 1e3) / 1e6, "unit": UNIT, "ms_per_vjp": vms,
                  "note": "flux_num_dnc5_2d_b (residual VJP, one cotangent) per call, device arrays, not L2-flushed",
                  "batched": {"value": IM * JM * NDIR / (bms / 1e3) / 1e6, "unit": UNIT, "cotangents_per_call": NDIR,
                              "ms_per_call": bms,
                              "note": "bcg_flux_num_dnc5_2d_bn: %d cotangents per call, device arrays" % NDIR}}
    # end to end through the C ABI with pinned host buffers
    pin = lambda shape: torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy()
    w_h = pin(c["w"].size)
    w_h[:] = np.ravel(c["w"], order="F")
    wd_h = pin(c["w"].size * NDIR)
    for k in range(NDIR):
        wd_h[k * c["w"].size:(k + 1) * c["w"].size] = np.ravel(wds[k], order="F")
    g = c["grid"]
    geo = {k: pin(g[k].size) for k in ("nx", "ny", "vol", "volf")}
    for k in geo:
        geo[k][:] = np.ravel(g[k], order="F")
    res_h, resd_h = pin(c["w"].size), pin(c["w"].size * NDIR)
    ph = [float(c["phys"][k]) for k in Dnc5Operator.PHYS_KEYS]

    def e2e_step():
        _lib.call("bcg_flux_num_dnc5_2d_dn", res_h, resd_h, w_h, wd_h, NDIR, None, None, geo["nx"], geo["ny"],
                  None, None, geo["vol"], geo["volf"], 3, *ph, IM, JM)

    for _ in range(max(args.warmup, 1)):
        e2e_step()
    t0 = time.perf_counter()
    for _ in range(steps):
        e2e_step()
    el = time.perf_counter() - t0
    np_, nn = (IM + 6) * (JM + 6), (IM + 7) * (JM + 7)
    h2d = 8 * (5 * np_ * (1 + NDIR) + 4 * nn + 3 * np_)
    d2h = 8 * 5 * IM * JM * (1 + NDIR)
    out["e2e"] = {"value": IM * JM * NDIR * steps / el / 1e6, "unit": UNIT, "h2d_bytes_per_step": h2d,
                  "d2h_bytes_per_step": d2h, "ms_per_step": el / steps * 1e3}
    group_ms = tot_ms / steps / (NDIR // GROUP)
    nb = algorithmic_bytes(IM, JM, 3, GROUP)
    hbm_peak = _hbm_peak()
    roof = {"bound": "fp64", "unit": "G FP64 inst/s", "achieved": None, "frac": None, "traffic": None,
            "kernel": "fused residual+JVP pass (prim, qrows, vpts, faces, balance) per group of %d directions"
                      % GROUP,
            "hbm": {"achieved": nb / (group_ms / 1e3) / 1e9, "peak": hbm_peak, "unit": "GB/s",
                    "frac": nb / (group_ms / 1e3) / 1e9 / hbm_peak, "algorithmic_bytes_per_group": nb}}
    if CYL_NCU:
        props = torch.cuda.get_device_properties(dev)
        mhz = (clocks or {}).get("sm_mhz") or 2070.0
        peak = 2.0 * props.multi_processor_count * mhz * 1e6 / 1e9
        inst = CYL_NCU["fp64_inst_per_cell_dir"] * IM * JM * NDIR
        roof.update(peak=peak, achieved=inst / (tot_ms / steps / 1e3) / 1e9)
        roof["frac"] = roof["achieved"] / peak
        roof["traffic"] = CYL_NCU["dram_bytes_per_cell_dir"] * IM * JM * GROUP
        roof["ncu_source"] = CYL_NCU["source"]
    out["roofline"] = roof
    out["gpu_launches"] = 5 * 2 * steps  # prim, qrows, vpts, faces, balance; two stream halves
    return out


def run_cylinder(args):
    """--workload cylinder: the 256x256 cylinder residual + 32-direction JVP line."""
    import torch
    ws, rank, local = _dist()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", init_method="env://")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    m = cylinder_measure(args, dev, ws=ws, rank=rank)
    if rank == 0:
        c, wds = build_workload()
        cpu = cpu_baseline(c, wds[:4], seconds=args.cpu_seconds)
        line = {"workload": "cylinder", "metric": METRIC, "value": m["value"], "unit": UNIT, "n_gpus": ws,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": m["ms_per_step"],
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic",
                "config": {"workload": m["workload"], "cells": IM * JM, "directions_per_step": NDIR,
                           "directions_per_launch_group": GROUP, "parallelism": "replicas" if ws > 1 else "single"},
                "roofline": m["roofline"], "cpu_baseline": cpu, "e2e": m["e2e"], "vjp": m["vjp"],
                "gpu_launches": m["gpu_launches"], "clocks": m["clocks"]}
        print(json.dumps(line))
    if ws > 1:
        dist.barrier()
        dist.destroy_process_group()
    return 0


def bl_bcs(c, w):
    """Boundary-layer sequence of BROADCAST_npz.py:1018-1021 through the library."""
    from broadcast_gb300.srcfv import f_bnd
    g, ph, it = c["grid"], c["phys"], c["interf"]
    im, jm, gh = g["im"], g["jm"], g["gh"]
    f_bnd.bc_supandsubinlet_2d(w, "Ilo", it["Ilo"], c["field"], g["nx"], g["ny"], ph["gam"], im, jm)
    f_bnd.bc_no_reflexion_2d(w, c["wbd"], "Jhi", it["Jhi"], g["nx"], g["ny"], ph["gam"], gh, im, jm)
    f_bnd.bc_extrapolate_o2_2d(w, "Ihi", it["Ihi"], im, jm, gh)
    f_bnd.bc_wall_viscous_adia_2d(w, "Jlo", ph["gam"], it["Jlo"], gh, im, jm)


def run_jacobian_workload(args):
    """Batched colored Jacobian of the 1024 x 512 boundary layer (the
    reference's third configuration): all 245 seeds (J / vol), Dz and Dzz as
    CSR, then J(beta) = J - beta^2 Dzz + i beta Dz for 16 beta in [0, 2],
    device-resident; beside it the reference loop (BROADCAST_npz.py:1068-1137)
    through the oracle on a sample of seeds, scaled to 245."""
    import torch
    from broadcast_gb300 import _lib, cases
    from broadcast_gb300._f2py import interf4
    im, jm = args.im or 1024, args.jm or 512
    c = cases.bl_case(im, jm, seed=3, ops=LibOps)
    bl_bcs(c, c["w"])
    g, ph, it = c["grid"], c["phys"], c["interf"]
    gh = g["gh"]
    nrow = 5 * im * jm
    dev = torch.device("cuda", 0)
    _lib.call("bcg_set_stream", torch.cuda.current_stream(dev).cuda_stream)
    keys = ("cp", "cv", "prandtl", "gam", "rgaz", "cs", "muref", "tref", "s_suth")
    common = [interf4(it["Ilo"]), interf4(it["Jhi"]), interf4(it["Ihi"]), interf4(it["Jlo"]), c["field"],
              c["field"].shape[0], c["wbd"], c["wbd"].shape[0]]
    geo = [c["w"], g["nx"], g["ny"], g["vol"], g["volf"], gh]
    cap = nrow * 245
    outs = {}
    for name in ("J", "Dz", "Dzz"):
        outs[name] = (torch.empty(nrow + 1, dtype=torch.int32, device=dev),
                      torch.empty(cap, dtype=torch.int32, device=dev),
                      torch.empty(cap, dtype=torch.float64, device=dev),
                      np.zeros(1, np.int64))

    def assemble(name):
        ip, ix, dv, nnz = outs[name]
        if name == "J":
            _lib.call("bcg_jacobian_dnc5_bl_csr", *geo, *[float(ph[k]) for k in keys + ("k2", "k4")], im, jm,
                      *common, None, 2e-16, 1, ip, ix, dv, ix.numel(), nnz)
        else:
            _lib.call("bcg_jacobian_dz_bl_csr", *geo, *[float(ph[k]) for k in keys], im, jm, *common,
                      1 if name == "Dz" else 2, 2e-16, ip, ix, dv, ix.numel(), nnz)
        return int(nnz[0])

    def timed(fn, reps):
        fn()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(reps):
            r = fn()
        torch.cuda.synchronize()
        return (time.perf_counter() - t0) / reps, r

    t_j, nnz_j = timed(lambda: assemble("J"), args.steps)
    t_dz, nnz_dz = timed(lambda: assemble("Dz"), args.steps)
    t_dzz, nnz_dzz = timed(lambda: assemble("Dzz"), args.steps)
    betas = torch.linspace(0.0, 2.0, 16, dtype=torch.float64)
    nb = np.zeros(1, np.int64)
    J, Dz, Dzz = outs["J"], outs["Dz"], outs["Dzz"]
    bargs = (nrow, J[0], J[1], J[2], Dz[0], Dz[1], Dz[2], Dzz[0], Dzz[1], Dzz[2], 16, betas.numpy())
    bp = torch.empty(nrow + 1, dtype=torch.int32, device=dev)
    try:
        _lib.call("bcg_csr_spanwise_beta", *bargs, bp, bp, bp, 0, nb)  # capacity 0: returns the union size
    except _lib.BroadcastError:
        pass
    nnz_u = int(nb[0])
    bi = torch.empty(nnz_u, dtype=torch.int32, device=dev)
    bv = torch.empty(2 * 16 * nnz_u, dtype=torch.float64, device=dev)
    t_beta, _ = timed(lambda: _lib.call("bcg_csr_spanwise_beta", *bargs, bp, bi, bv, nnz_u, nb), args.steps)
    # the same four outputs from one pass over the seeds (bcg_jacobian_span_bl_csr)
    one = [(torch.empty(nrow + 1, dtype=torch.int32, device=dev), torch.empty(n + 0, dtype=torch.int32, device=dev),
            torch.empty(n + 0, dtype=torch.float64, device=dev)) for n in (nnz_j, nnz_dz, nnz_dzz)]
    tab = [np.array([o[k].data_ptr() for o in one], np.uint64) for k in range(3)]
    caps, nnz3 = np.array([nnz_j, nnz_dz, nnz_dzz], np.int64), np.zeros(3, np.int64)
    op_ = torch.empty(nrow + 1, dtype=torch.int32, device=dev)
    oi, ov = torch.empty_like(bi), torch.empty_like(bv)
    onb = np.zeros(1, np.int64)

    def one_pass():
        _lib.call("bcg_jacobian_span_bl_csr", *geo, *[float(ph[k]) for k in keys + ("k2", "k4")], im, jm, *common,
                  2e-16, 1, tab[0], tab[1], tab[2], caps, nnz3, 16, betas.numpy(), op_, oi, ov, nnz_u, onb)

    t_one, _ = timed(one_pass, args.steps)
    same = (list(nnz3) == [nnz_j, nnz_dz, nnz_dzz] and int(onb[0]) == nnz_u
            and all(torch.equal(a[2], b[2][:a[2].numel()]) for a, b in zip(one, (J, Dz, Dzz)))
            and torch.equal(ov, bv))
    # reference loop through the oracle (OpenMP), a sample of seeds
    from oracle import oracle as O
    lib = O.lib(openmp=True)
    nsample = 4
    w = c["w"]
    res, resd = np.zeros_like(w), np.zeros_like(w)
    nb_ = im * jm * 49 * 25
    jac, ia, ja = np.zeros(nb_), np.zeros(nb_, np.int32), np.zeros(nb_, np.int32)
    t0 = time.perf_counter()
    for s in range(nsample):
        m, l, k = s % 5, (s // 5) % 7, s // 35
        wd = O.testvector(m, l, k, gh, im, jm)
        wtmp = w.copy(order="F")
        O.bc_inlet(wtmp, "Ilo", it["Ilo"], c["field"], g["nx"], g["ny"], ph["gam"], im, jm, gh, wd=wd)
        O.bc_noref(wtmp, c["wbd"], "Jhi", it["Jhi"], g["nx"], g["ny"], ph["gam"], gh, im, jm, wd=wd)
        O.bc_extrap(wtmp, "Ihi", it["Ihi"], im, jm, gh, wd=wd)
        O.bc_wall(wtmp, "Jlo", ph["gam"], it["Jlo"], gh, im, jm, wd=wd)
        lib.orc_flux_num_dnc5_2d_d(O._p(res), O._p(resd), O._p(w), O._p(wd), 1, O._p(g["nx"]), O._p(g["ny"]),
                                   O._p(g["vol"]), O._p(g["volf"]), gh, *O._phys(ph), im, jm)
        O.computejacobian(O.JAC_PLAIN, jac, ia, ja, resd, m, l, k, gh, im, jm, None)
    t_cpu = (time.perf_counter() - t0) / nsample * 245
    line = {"workload": "jacobian", "metric": "batched Jacobian assembly, seed-cells/s", "unit": "Mcells/s",
            "value": 245 * im * jm / t_j / 1e6, "higher_is_better": True, "dtype": "f64", "data": "synthetic",
            "config": {"grid": "boundary layer %dx%d, Mach 0.5, Re_x0 1e5, stretch 1.03, seed 3" % (im, jm),
                       "seeds": 245, "betas": 16, "steps": args.steps},
            "seconds": {"jacobian_csr": t_j, "dz_csr": t_dz, "dzz_csr": t_dzz, "j_beta_16": t_beta,
                        "separate_total": t_j + t_dz + t_dzz + t_beta, "one_pass_all_four": t_one},
            "one_pass_bit_identical": bool(same),
            "nnz": {"J": nnz_j, "Dz": nnz_dz, "Dzz": nnz_dzz, "union": nnz_u},
            "cpu_baseline": {"seconds_245_seeds": t_cpu, "kind": "port", "cores": os.cpu_count(),
                             "sample": "%d seeds of the reference loop (testvector, linearised boundary chain, "
                                       "tangent residual, COO fill) through the oracle with OpenMP, scaled to 245"
                                       % nsample}}
    print(json.dumps(line))
    return 0


def _flux_scale(c):
    """Per-variable face-flux magnitude max(|f| + |g|) * max face length."""
    w, g, gam = c["w"], c["grid"], c["phys"]["gam"]
    ro = w[..., 0]
    u, v, ww = w[..., 1] / ro, w[..., 2] / ro, w[..., 3] / ro
    p = (gam - 1.0) * (w[..., 4] - 0.5 * ro * (u * u + v * v + ww * ww))
    f = np.stack([w[..., 1], w[..., 1] * u + p, w[..., 1] * v, w[..., 1] * ww, (w[..., 4] + p) * u], -1)
    h = np.stack([w[..., 2], w[..., 2] * u, w[..., 2] * v + p, w[..., 2] * ww, (w[..., 4] + p) * v], -1)
    return (np.abs(f) + np.abs(h)).reshape(-1, 5).max(0) * np.sqrt(g["nx"] ** 2 + g["ny"] ** 2).max()


# FP64 lane instructions (warp instructions issued to the FP64 pipe x 32: the
# DFMA, DADD and DMUL that make up 97 % of them and the compares and
# conversions) and DRAM bytes per interior cell of each pass of one uneven-batch evaluation (residual + one
# JVP direction, boundary-layer grids), from one ncu capture of the first 6
# grids of the uneven batch (1.34M cells):
#   ncu --clock-control none -k regex:k_batch -c 6 --metrics
#       sm__inst_executed_pipe_fp64.sum,
#       sm__sass_thread_inst_executed_ops_dadd_dmul_dfma_pred_on.sum,
#       sm__pipe_fp64_cycles_active.avg.pct_of_peak_sustained_active,
#       dram__bytes_read.sum,dram__bytes_write.sum,gpu__time_duration.sum
#       python bench.py --grids 6 --steps 1 --warmup 1 --no-extras --tile 128,128,3 --cpu-seconds 1
# divided by the capture's cells; the full batch's figures scale with its cells.
BATCH_NCU = {
    "fp64_inst_per_cell": {"prim": 135.9, "sensor": 175.9, "qrows": 93.3, "vpts": 48.5, "faces": 833.7,
                           "balance": 30.0},
    "dram_bytes_per_cell": {"prim": 351.3, "sensor": 161.2, "qrows": 338.9, "vpts": 231.9, "faces": 900.7,
                            "balance": 219.4},
    "source": "ncu sm__inst_executed_pipe_fp64.sum x 32 lanes and dram__bytes_read.sum + dram__bytes_write.sum "
              "per k_batch launch, first 6 grids (1,344,226 cells), cold caches; per cell, scaled to this run's "
              "cells; prim includes the rectilinear-grid scan (k_batch_rect) that runs with it",
}
BATCH_PASSES = ("prim", "sensor", "qrows", "vpts", "faces", "balance")


def batch_inputs(n, ops, bcs):
    """The uneven batch (nx ~ U{200..1200}, ny ~ U{80..300}, Mach ~ U(0.3, 0.8),
    default_rng(4)): the first n grids with their boundary fills and one
    seeded N(0, 1) direction each."""
    from broadcast_gb300 import cases
    cs, wds = [], []
    for _, c, wd in cases.uneven_bl_batch(n, ops=ops):
        bcs(c, c["w"])
        cs.append(c)
        wds.append(wd)
    return cs, wds


def oracle_bl_bcs(c, w):
    from oracle import oracle as O
    g, ph, it = c["grid"], c["phys"], c["interf"]
    im, jm, gh = g["im"], g["jm"], g["gh"]
    O.bc_inlet(w, "Ilo", it["Ilo"], c["field"], g["nx"], g["ny"], ph["gam"], im, jm, gh)
    O.bc_noref(w, c["wbd"], "Jhi", it["Jhi"], g["nx"], g["ny"], ph["gam"], gh, im, jm)
    O.bc_extrap(w, "Ihi", it["Ihi"], im, jm, gh)
    O.bc_wall(w, "Jlo", ph["gam"], it["Jlo"], gh, im, jm)


class OracleOps:
    @staticmethod
    def computegeom(*a):
        from oracle import oracle as O
        O.computegeom(*a)

    @staticmethod
    def initblfv(*a):
        from oracle import oracle as O
        O.initblfv(*a)

    @staticmethod
    def set_bndbl(*a):
        from oracle import oracle as O
        O.set_bndbl(*a)


def oracle_jvp_batch(cs, wds, outs=None):
    """Residual + JVP of every grid through the oracle with OpenMP on all host
    cores (orc_flux_num_dnc5_2d_d); returns [(res, resd)]."""
    from oracle import oracle as O
    lib = O.lib(openmp=True)
    out = []
    for k, (c, wd) in enumerate(zip(cs, wds)):
        g, ph = c["grid"], c["phys"]
        r, rd = outs[k] if outs else (np.zeros_like(c["w"], order="F"), np.zeros_like(c["w"], order="F"))
        lib.orc_flux_num_dnc5_2d_d(O._p(r), O._p(rd), O._p(c["w"]), O._p(wd), 1, O._p(g["nx"]), O._p(g["ny"]),
                                   O._p(g["vol"]), O._p(g["volf"]), g["gh"], *O._phys(ph), g["im"], g["jm"])
        out.append((r, rd))
    return out


def batch_config(n, cells):
    return {"workload": "uneven batch of %d laminar boundary layers (grids %s of nx U{200..1200} x ny U{80..300}, "
                        "Mach U(0.3, 0.8), default_rng(4); Blasius + 1e-4 noise), residual + one JVP direction "
                        "per grid" % (n, "1-%d" % n), "grids": n, "cells": cells,
            "unit_of_work": "one residual plus one JVP of one interior cell"}


def batch_cpu_baseline(cs, wds, seconds):
    """The oracle port on all host cores over the grids of the batch, repeated
    for about `seconds`."""
    outs = [(np.zeros_like(c["w"], order="F"), np.zeros_like(c["w"], order="F")) for c in cs]
    cells, n, t0 = 0, 0, time.perf_counter()
    while True:
        k = n % len(cs)
        oracle_jvp_batch([cs[k]], [wds[k]], [outs[k]])
        cells += cs[k]["grid"]["im"] * cs[k]["grid"]["jm"]
        n += 1
        el = time.perf_counter() - t0
        if el >= seconds and n >= 2:
            break
    return {"value": cells / el / 1e6, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
            "sample": "%d grid evaluations (residual + 1 JVP direction, %d cells) of the uneven batch in grid order, "
                      "%.1f s, OpenMP over j-rows" % (n, cells, el)}


def run_batch_reference(args):
    """Reference arm of the default line: the oracle port (C++ restatement of
    the reference Fortran, OpenMP on all host cores) on the same grids, inputs
    and directions; one step = every grid's residual + JVP."""
    ws, rank, _ = _dist()
    if rank != 0:
        return 0
    n = args.grids or 64
    cs, wds = batch_inputs(n, OracleOps, oracle_bl_bcs)
    cells = sum(c["grid"]["im"] * c["grid"]["jm"] for c in cs)
    outs = [(np.zeros_like(c["w"], order="F"), np.zeros_like(c["w"], order="F")) for c in cs]
    for _ in range(args.warmup):
        oracle_jvp_batch(cs, wds, outs)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        oracle_jvp_batch(cs, wds, outs)
    el = time.perf_counter() - t0
    v = cells * args.steps / el / 1e6
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": el / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": batch_config(n, cells), "same_config": True,
            "inputs_sha": inputs_digest(cs, wds),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
                             "sample": "every step: all %d grids (%d cells), residual + 1 JVP direction each, "
                                       "OpenMP over j-rows" % (n, cells)},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def inputs_digest(cs, wds):
    """Digest of what both arms build bit-identically (host pre-processing
    through the library and through the oracle agree bit for bit): the
    grids' metrics, the interior states and the directions.  The ghost cells
    are filled by each arm's own boundary-fill code (library kernels, oracle)
    and compared numerically (parity.ghost_fill_vs_oracle_max_rel)."""
    import hashlib
    h = hashlib.sha256()
    for c, wd in zip(cs, wds):
        for a in (c["grid"]["nx"], c["grid"]["ny"], c["grid"]["vol"], c["grid"]["volf"], H_int(c["w"]), wd):
            h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()[:16]


def ghost_fill_difference(cs):
    """Largest difference, relative to the state's magnitude per variable,
    between the ghost cells the library filled and the oracle's fills of the
    same interior states."""
    worst = 0.0
    for c in cs:
        w = c["w"].copy(order="F")
        oracle_bl_bcs(c, w)
        sc = np.abs(w).reshape(-1, 5).max(0)
        worst = max(worst, float((np.abs(w - c["w"]).reshape(-1, 5) / sc).max()))
    return worst


def run_batch(args):
    """Default line: the uneven batch of 64 boundary layers (residual + one JVP
    per grid) as one CUDA graph of persistent launches; value from CUDA events
    with the inputs resident in HBM, e2e through bcg_batch_run_host with pinned
    host arrays."""
    import torch
    ws, rank, local = _dist()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", init_method="env://")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    from broadcast_gb300.batch import GridBatch
    from broadcast_gb300.operator import to_device, to_host
    n = args.grids or 64
    cs, wds = batch_inputs(n, LibOps, bl_bcs)
    cells = sum(c["grid"]["im"] * c["grid"]["jm"] for c in cs)
    gb = GridBatch([c["grid"] for c in cs], [c["phys"] for c in cs], ndir=1, device=dev)
    gb.set_states([to_device(c["w"], dev) for c in cs], [to_device(wd, dev) for wd in wds])
    if args.tile:  # fixed tile shapes (faces threads, cell threads, face CTAs per SM), no autotuning
        gb.configure(*[int(x) for x in args.tile.split(",")])
        tune = {"config": list(gb.config)}
    else:
        tune = gb.autotune(repeats=3, use_cache=False)
    stream = torch.cuda.current_stream(dev)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)  # 256 MB > L2

    def step():
        gb.run(use_graph=True)

    for _ in range(max(args.warmup, 1)):
        step()
    torch.cuda.synchronize()
    sampler = ClockSampler(local)
    if rank == 0:
        sampler.start()
    t0 = time.perf_counter()
    while time.perf_counter() - t0 < 0.3:  # the clock samples see the GPU under this load
        step()
        torch.cuda.synchronize()
    if ws > 1:
        dist.barrier()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    for s in range(args.steps):
        flush.add_(1.0)
        ev[s][0].record(stream)
        step()
        ev[s][1].record(stream)
    torch.cuda.synchronize()
    if ws > 1:
        dist.barrier()
    clocks = sampler.stop() if rank == 0 else None
    if clocks:
        clocks["window"] = "0.3 s of the same step untimed, then the timed region"
    tot_ms = sum(a.elapsed_time(b) for a, b in ev)
    if ws > 1:
        t = torch.tensor([tot_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        tot_ms = float(t.item())
    value = cells * ws * args.steps / (tot_ms / 1e3) / 1e6
    line = None
    if rank == 0:
        # each pass alone (events around one launch, L2 flushed before each)
        pass_ms = []
        for k in range(len(BATCH_PASSES)):
            a_ev, b_ev = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            tk = 0.0
            for _ in range(3):
                for q in range(k):  # the earlier passes produce this pass's inputs
                    gb.run_pass(q)
                flush.add_(1.0)
                a_ev.record(stream)
                gb.run_pass(k)
                b_ev.record(stream)
                torch.cuda.synchronize()
                tk += a_ev.elapsed_time(b_ev)
            pass_ms.append(tk / 3)
        # end to end: pinned host arrays through bcg_batch_run_host
        pin = lambda a: _pinned_copy(torch, a)
        w_h, wd_h = [pin(c["w"]) for c in cs], [pin(wd) for wd in wds]
        geo_h = [{k: pin(c["grid"][k]) for k in ("nx", "ny", "vol", "volf")} for c in cs]
        res_h, resd_h = [pin(np.zeros_like(c["w"], order="F")) for c in cs], [pin(np.zeros_like(c["w"], order="F")) for c in cs]
        nchunk = args.chunks
        if args.tile:
            gb.configure_host(*[int(x) for x in args.tile.split(",")])
            host_tune = {"config": list(gb.host_config)}
        else:  # the chunks' own tile shapes, timed with their copies (untimed here)
            host_tune = gb.autotune_host(w_h, wd_h, res_h, resd_h, geo_h, nchunk=nchunk)
        for _ in range(max(args.warmup, 1)):
            gb.run_host(w_h, wd_h, res_h, resd_h, geo_h, nchunk=nchunk)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            gb.run_host(w_h, wd_h, res_h, resd_h, geo_h, nchunk=nchunk)
        el = time.perf_counter() - t0
        nps = [(c["grid"]["im"] + 6) * (c["grid"]["jm"] + 6) for c in cs]
        nns = [(c["grid"]["im"] + 7) * (c["grid"]["jm"] + 7) for c in cs]
        h2d = sum(8 * (13 * a + 4 * b) for a, b in zip(nps, nns))
        d2h = 8 * 10 * cells
        e2e = {"value": cells * args.steps / el / 1e6, "unit": UNIT, "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": d2h, "ms_per_step": el / args.steps * 1e3, "chunks": nchunk,
               "chunk_tile": {"faces": host_tune["config"][0], "cells": host_tune["config"][1],
                              "ctas_per_sm": host_tune["config"][2]},
               "call": "bcg_batch_run_host (GridBatch.run_host): state, direction and metrics of every grid "
                       "uploaded, residual and tangent interiors downloaded, every step"}
        # parity of this run's outputs (device run and host-array run) with the oracle
        ref = oracle_jvp_batch(cs, wds)
        err_res, err_tan, above, host_dev = 0.0, 0.0, 0, 0.0
        for g, c in enumerate(cs):
            r, rd = to_host(gb.res[g]), to_host(gb.resd[g])
            host_dev = max(host_dev, float(np.abs(H_int(res_h[g]) - H_int(r)).max()),
                           float(np.abs(H_int(resd_h[g]) - H_int(rd)).max()))
            rr, rrd = ref[g]
            sc = _flux_scale(c)
            scd = np.abs(H_int(rrd)).reshape(-1, 5).max(0)
            err_res = max(err_res, float((np.abs(H_int(r) - H_int(rr)).reshape(-1, 5).max(0) / sc).max()))
            et = (np.abs(H_int(rd) - H_int(rrd)) / scd).max(axis=2)
            err_tan = max(err_tan, float(et.max()))
            above += int((et > 1e-11).sum())
        cpu = batch_cpu_baseline(cs, wds, args.cpu_seconds)
        roof = batch_roofline([(c["grid"]["im"], c["grid"]["jm"]) for c in cs], tot_ms / args.steps, pass_ms, clocks)
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": tot_ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic",
            "config": dict(batch_config(n, cells), parallelism="replicas" if ws > 1 else "single", graph=True,
                           l2="flushed between steps (256 MB write); the batch's arrays (~%.1f GB) exceed L2 anyway"
                              % (cells * 8 * 23 / 1e9),
                           tile={"faces": tune["config"][0], "cells": tune["config"][1],
                                 "ctas_per_sm": tune["config"][2]}),
            "roofline": roof,
            "pass_ms": dict(zip(BATCH_PASSES, pass_ms)),
            "parity": {"residual_vs_oracle_max": err_res, "tangent_vs_oracle_max": err_tan,
                       "tangent_cells_above_1e-11": above, "host_run_vs_device_run_max_abs": host_dev,
                       "ghost_fill_vs_oracle_max_rel": ghost_fill_difference(cs),
                       "note": "residual relative to the face-flux magnitude, tangent to max|R'v| per variable"},
            "inputs_sha": inputs_digest(cs, wds),
            "cpu_baseline": cpu,
            "e2e": e2e,
            "gpu_launches": 7 * args.steps,  # per graph replay: the rectilinear scan and the six passes
            "clocks": clocks,
        }
    if not args.no_extras and rank == 0:
        del gb
        torch.cuda.empty_cache()
        line["cylinder_256"] = cylinder_measure(args, dev, extras_only=True)
    if rank == 0:
        print(json.dumps(line))
    if ws > 1:
        dist.barrier()
        dist.destroy_process_group()
    return 0


def H_int(a):
    return a[3:-3, 3:-3]


def _pinned_copy(torch, a):
    t = torch.empty(a.size, dtype=torch.float64, pin_memory=True).numpy()
    t[:] = np.ravel(a, order="F")
    return t.reshape(a.shape, order="F")


def batch_roofline(dims, step_ms, pass_ms, clocks):
    """FP64-bound roofline of the evaluation and of its dominant pass (faces):
    executed FP64 lane instructions (ncu counts per cell, scaled to the batch's
    cells) over the FP64 issue peak of 2 lane instructions per clock per SM at
    the clock sampled during the timed region; DRAM traffic likewise from ncu
    per cell; the HBM fraction of the algorithmic bytes beside it."""
    import torch
    props = torch.cuda.get_device_properties(torch.cuda.current_device())
    nsm = props.multi_processor_count
    mhz = (clocks or {}).get("sm_mhz") or 2070.0
    peak = 2.0 * nsm * mhz * 1e6 / 1e9  # G FP64 lane instructions / s
    hbm_peak = _hbm_peak()
    faces_ms = pass_ms[BATCH_PASSES.index("faces")]
    out = {"bound": "fp64", "unit": "G FP64 inst/s", "peak": peak,
           "peak_source": "2 FP64 lane instructions per clock per SM x %d SMs x %.0f MHz (median SM clock sampled "
                          "in the timed region); GB300's FP64 FMA rate measured with FMA chains matches it" % (nsm, mhz),
           "kernel": "k_batch<DK<1>, faces> (face fluxes of all grids, one persistent launch), %.1f%% of the sum of "
                     "the passes timed alone" % (100 * faces_ms / sum(pass_ms)),
           "achieved": None, "frac": None, "traffic": None}
    cells = sum(i * j for i, j in dims)
    nb = sum(algorithmic_bytes(i, j, 3, 1) for i, j in dims)
    out["hbm"] = {"achieved": nb / (step_ms / 1e3) / 1e9, "peak": hbm_peak, "unit": "GB/s",
                  "frac": nb / (step_ms / 1e3) / 1e9 / hbm_peak,
                  "algorithmic_bytes_per_step": nb, "peak_source": "MEASURED_PEAKS.json hbm_gbs"}
    if BATCH_NCU:
        inst = {k: v * cells for k, v in BATCH_NCU["fp64_inst_per_cell"].items()}
        dram = {k: v * cells for k, v in BATCH_NCU["dram_bytes_per_cell"].items()}
        out["achieved"] = inst["faces"] / (faces_ms / 1e3) / 1e9
        out["frac"] = out["achieved"] / peak
        out["traffic"] = dram["faces"]
        out["algorithmic_fp64_inst_per_launch"] = inst["faces"]
        tot = sum(inst.values())
        out["whole_step"] = {"achieved": tot / (step_ms / 1e3) / 1e9, "frac": tot / (step_ms / 1e3) / 1e9 / peak,
                             "fp64_inst_per_step": tot, "traffic_per_step": sum(dram.values())}
        out["ncu_source"] = BATCH_NCU["source"]
    return out


def run_impli_workload(args):
    """The matrix-free implicit phase of the 'impli' time marching
    (impli_matrix_free_2d, BROADCAST_npz.py:911-941): lmax = 10 symmetric
    Gauss-Seidel sweeps on the residual of the boundary layer 400x150 (the
    reference's first configuration), cfl 5, dtcoef 1.  The sweeps are a
    wavefront of im + jm - 1 dependent anti-diagonals each, so the bound is
    the latency of one diagonal step, reported beside the throughput."""
    import torch
    from broadcast_gb300 import _lib, cases
    from broadcast_gb300.operator import to_device
    from broadcast_gb300.srcfv import f_lhs, f_sch
    from oracle import oracle as O
    im, jm, lmax, cfl, dtcoef = args.im or 400, args.jm or 150, args.lmax, 5.0, 1.0
    c = cases.bl_case(im, jm, seed=0, ops=LibOps)
    bl_bcs(c, c["w"])
    g, ph = c["grid"], c["phys"]
    dev = torch.device("cuda", 0)
    _lib.call("bcg_set_stream", torch.cuda.current_stream(dev).cuda_stream)
    res = np.zeros_like(c["w"])
    f_sch.flux_num_dnc5_2d(res, c["w"], g["x0"], g["y0"], g["nx"], g["ny"], g["xc"], g["yc"], g["vol"], g["volf"],
                           g["gh"], ph["cp"], ph["cv"], ph["prandtl"], ph["gam"], ph["rgaz"], ph["cs"], ph["muref"],
                           ph["tref"], ph["cs"], ph["k2"], ph["k4"], im, jm)
    fdev = lambda a: to_device(a, dev).permute(*reversed(range(a.ndim)))
    arrs = [fdev(g["nx"]), fdev(g["ny"]), fdev(c["w"]), fdev(res), fdev(g["vol"]), fdev(g["volf"])]
    dwi = fdev(np.zeros_like(c["w"]))
    scal = (dtcoef, cfl, ph["gam"], ph["rgaz"], ph["prandtl"], lmax, g["gh"], ph["cv"], ph["cs"], ph["muref"],
            ph["tref"], ph["cs"])
    call = lambda out, a: f_lhs.impli_matrix_free_2d(out, *a, *scal)
    for _ in range(max(args.warmup, 3)):
        call(dwi, arrs)
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream(dev)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    for s in range(args.steps):
        flush.add_(1.0)
        ev[s][0].record(stream)
        call(dwi, arrs)
        ev[s][1].record(stream)
    torch.cuda.synchronize()
    ms = sum(a.elapsed_time(b) for a, b in ev) / args.steps
    from broadcast_gb300.operator import to_host
    out = to_host(dwi.permute(*reversed(range(3))))
    # end to end: host arrays (uploads of w, dw and the metrics, download of dwi)
    host_args = [g["nx"], g["ny"], c["w"], res, g["vol"], g["volf"]]
    dwi_h = np.zeros_like(c["w"])
    call(dwi_h, host_args)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        call(dwi_h, host_args)
    e2e_ms = (time.perf_counter() - t0) / args.steps * 1e3
    # the CPU reference: the oracle's sequential sweeps (the algorithm is a
    # Gauss-Seidel recurrence, one thread), and the parity of the GPU result
    t0 = time.perf_counter()
    nrep = 0
    while True:
        ref = O.impli_matrix_free(g, ph, c["w"], res, dtcoef, cfl, lmax)
        nrep += 1
        if time.perf_counter() - t0 >= min(args.cpu_seconds, 10.0) and nrep >= 2:
            break
    cpu_ms = (time.perf_counter() - t0) / nrep * 1e3
    err = float(np.abs(out - ref).max() / np.abs(ref).max())
    steps = lmax * (im + jm - 1)
    cells = im * jm
    nbytes = 8 * (2 * 5 * (im + 6) * (jm + 6) + 4 * (im + 7) * (jm + 7) + 3 * (im + 6) * (jm + 6) + 5 * (im + 6) * (jm + 6))
    line = {"workload": "impli", "metric": "impli_matrix_free_2d calls/s (lmax %d, BL %dx%d)" % (lmax, im, jm),
            "unit": "calls/s",
            "value": 1e3 / ms, "ms_per_step": ms, "higher_is_better": True, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "boundary layer %dx%d, residual as right-hand side, lmax %d, cfl %g, dtcoef %g"
                                   % (im, jm, lmax, cfl, dtcoef), "l2": "flushed between steps (256 MB write)"},
            "latency": {"dependent_diagonal_steps": steps, "us_per_step": ms * 1e3 / steps,
                        "note": "each sweep is im + jm - 1 dependent anti-diagonal steps; one cluster barrier "
                                "per step"},
            "roofline": {"bound": "hbm", "achieved": nbytes / (ms / 1e3) / 1e9, "peak": _hbm_peak(), "unit": "GB/s",
                         "frac": nbytes / (ms / 1e3) / 1e9 / _hbm_peak(), "traffic": None,
                         "note": "formal: latency-bound wavefront (see latency), not bandwidth-bound"},
            "e2e": {"value": 1e3 / e2e_ms, "unit": "calls/s", "h2d_bytes_per_step": int(nbytes - 8 * 5 * (im + 6) * (jm + 6)),
                    "d2h_bytes_per_step": int(8 * 5 * (im + 6) * (jm + 6)), "ms_per_step": e2e_ms},
            "cpu_baseline": {"value": 1e3 / cpu_ms, "unit": "calls/s", "cores": 1, "kind": "port",
                             "sample": "%d oracle calls (sequential sweeps, the reference's loop order), %.1f ms each"
                                       % (nrep, cpu_ms)},
            "parity": {"max_abs_err_rel_to_max": err, "tolerance": 1e-12, "cells": cells},
            "gpu_launches": 5 * args.steps}  # cells, faces, diag, sweeps, out
    print(json.dumps(line))
    return 0


def run_newton_workload(args):
    """The SER Newton driver (the 'fixed_point' mode, BROADCAST_npz.py:985-1196)
    on the boundary layer 400x150 (the reference's first configuration) with the
    card's cfl = 1e10: GPU boundary fills, residual and norms, relaxed Jacobian
    assembly of all 245 colour seeds, and the GPU band-LU solve, iterated until
    the largest L2 residual norm is below 1e-10 (absolute) or 1e-11 of the first
    iterate's (the relative norm the reference prints, BROADCAST_npz.py:885; on
    this grid the absolute norm stalls at its round-off floor, ~8e-10, since
    the coordinates are local Reynolds numbers up to 6e5), or 40 iterations."""
    import torch
    from broadcast_gb300 import cases
    from broadcast_gb300.newton import BLNewton, CylNewton
    cyl = args.case == "cyl"
    im, jm = args.im or (256 if cyl else 400), args.jm or (256 if cyl else 150)
    # GMRES with the FP32 band-LU preconditioner above 20,000 cells unless --solver band
    krylov = args.solver == "krylov" or (args.solver == "auto" and im * jm > 20000)
    if cyl:  # cylinder.py:841-1068 on the 256 x 256 O-mesh, Newton (cfl 1e10)
        c = cases.cyl_case(im, jm, ops=LibOps)
        nt = CylNewton(c, solver="krylov" if krylov else None)
    else:
        c = cases.bl_case(im, jm, seed=0, ops=LibOps)
        nt = BLNewton(c, solver="krylov") if krylov else BLNewton(c)
    w = c["w"].copy(order="F")
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    converged, norm0, bad = None, None, 0
    for it in range(1, 41):
        norm, dw = nt.step(w, first=(it == 1))
        nmax = float(np.max(norm))
        norm0 = nmax if norm0 is None else norm0
        bad = bad + 1 if not (np.all(np.isfinite(dw)) and np.isfinite(nmax)) else 0
        if bad >= 3:  # the step-back (cfl halving) does not recover: stop
            converged = "diverged (non-finite updates)"
            break
        if nmax <= 1e-10:
            converged = "absolute 1e-10"
            break
        if nmax <= 1e-11 * norm0:
            converged = "relative 1e-11"
            break
    total = time.perf_counter() - t0
    hist = nt.history
    mean = lambda k: float(np.mean([h[k] for h in hist]))
    what = "cylinder O-mesh" if args.case == "cyl" else "BL"
    line = {"workload": "newton",
            "metric": "SER Newton time to max L2 norm <= 1e-10, or 1e-11 relative (%s %dx%d, cfl 1e10)" % (what, im, jm),
            "unit": "s", "value": total, "higher_is_better": False, "dtype": "f64", "data": "synthetic",
            "iterations": len(hist), "converged": converged, "final_norm": float(np.max(hist[-1]["norm"])),
            "final_norm_relative": float(np.max(hist[-1]["norm"])) / norm0,
            "norms": [float(np.max(h["norm"])) for h in hist],
            "seconds_per_iteration": {"total": mean("seconds"), "fills_residual_norms": mean("seconds_residual"),
                                      "jacobian_245_seeds": mean("seconds_jacobian"),
                                      "linear_solve": mean("seconds_solve")},
            "linear_solver": ("FP64 band LU (cuSOLVER getrf panels, cuBLAS trsm/gemm)" if not krylov else
                              "FP64 GMRES, FP32 band LU preconditioner reused across iterations"),
            "krylov": getattr(nt.solver, "log", None),
            "jacobian_nnz": hist[-1]["nnz"],
            "config": {"workload": ("cylinder O-mesh %dx%d, uniform flow + U(-1e-3, 1e-3) noise (seed 1), Mach 0.1, "
                                    "Re 47, band LU in the folded azimuthal order" % (im, jm)) if args.case == "cyl" else
                                   ("boundary layer %dx%d, Blasius polynomial state + U(-1e-4, 1e-4) noise (seed 0), "
                                    "card cfl 1e10" % (im, jm))},
            "cpu_baseline": {"value": None, "unit": "s", "kind": "port", "cores": 1,
                             "sample": "none at this size: the host sparse LU in the image (SuperLU) did not finish "
                                       "one factorisation of this Jacobian in 1500 s; the reference's MUMPS is absent"}}
    print(json.dumps(line))
    return 0


def run_warmstart_workload(args):
    """Learned warm start of the cylinder base flow (Re in [40, 200], Mach in
    [0.05, 0.3]): base flows at --ntrain seeded (Re, Mach) points (seed 5) by
    continuation with the GPU Newton iteration, the conditioned MLP trained on
    them by the BF16 kernels, then every one of --nheld held-out points (seed
    6) solved to max L2 norm <= 1e-10 from the network's guess (plain start as
    fallback) and from the nearest training base flow (plain continuation);
    value = mean time from the learned guess, beside the plain mean."""
    import torch
    from broadcast_gb300 import warmstart as WS
    im, jm = args.im or 512, args.jm or 256
    ratio = WS.radial_ratio(jm)
    solver = None
    if args.solver == "krylov" or (args.solver == "auto" and im * jm > 20000):
        from broadcast_gb300.linsolve import KrylovSolver, folded_ring_order
        solver = KrylovSolver(perm=folded_ring_order(im, jm))
    logs = []
    log = lambda msg: (logs.append(msg), print(msg, file=sys.stderr, flush=True))
    train = WS.sample_parameters(args.ntrain, seed=5)
    held = WS.sample_parameters(args.nheld, seed=6)
    t0 = time.perf_counter()
    states, recs = WS.solve_baseflows(train, im, jm, ratio=ratio, log=log, solver=solver)
    t_data = time.perf_counter() - t0
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0 = time.perf_counter()
    ev0.record()
    model, fit_log = WS.train_on_baseflows(train, states, im, jm, ratio=ratio, steps=args.train_steps,
                                           batch=args.batch, log_every=max(1, args.train_steps // 10))
    ev1.record()
    torch.cuda.synchronize()
    t_fit = time.perf_counter() - t0
    fit_ms = ev0.elapsed_time(ev1)
    d = WS.DIMS
    flops_step = 3 * 2 * args.batch * sum(d[i] * d[i + 1] for i in range(4))  # forward, data and weight gradients
    # each arm with its own Krylov solver, both without a factor at the first held-out point, each
    # keeping its own from point to point (a shared one would hand one arm the factor the other
    # built at the same point)
    solver_learned = None
    n_gen = len(solver.log) if solver is not None else 0
    if solver is not None:
        solver.close()
        solver_learned = KrylovSolver(perm=folded_ring_order(im, jm))
    out = WS.compare_starts(model, train, states, held, im, jm, ratio=ratio, log=log, solver=solver,
                            solver_learned=solver_learned)
    conv = [r for r in out if r["plain"]["converged"] and r["learned"]["converged"]]
    mean = lambda arm, k: float(np.mean([r[arm][k] for r in conv])) if conv else None
    line = {"workload": "warmstart",
            "metric": "baseflow time to max L2 norm <= 1e-10 from the learned guess (cylinder O-mesh %dx%d, "
                      "mean over %d held-out (Re, Mach))" % (im, jm, len(held)),
            "unit": "s", "value": mean("learned", "seconds"), "higher_is_better": False, "dtype": "f64 solver, bf16/f32 network",
            "data": "synthetic (solver-generated base flows)",
            "plain_continuation": {"seconds": mean("plain", "seconds"), "iterations": mean("plain", "iterations"),
                                   "first_norm": mean("plain", "first_norm")},
            "learned": {"seconds": mean("learned", "seconds"), "iterations": mean("learned", "iterations"),
                        "first_norm": mean("learned", "first_norm"),
                        "guess_seconds": mean("learned", "guess_seconds"),
                        "fallbacks": int(sum(r["learned"]["fallback"] for r in out))},
            "speedup_vs_plain": (mean("plain", "seconds") / mean("learned", "seconds")) if conv else None,
            "converged_both": len(conv), "held_out": len(out),
            "training_set": {"points": len(train), "converged": int(sum(s is not None for s in states)),
                             "seconds": t_data,
                             "newton_iterations_mean": float(np.mean([r["iterations"] for r in recs if r]))},
            "network": {"train_seconds": t_fit, "train_steps": args.train_steps, "batch": args.batch,
                        "loss_first": fit_log[0][1], "loss_last": fit_log[-1][1],
                        "gemm_tflops_bf16": flops_step * args.train_steps / (fit_ms / 1e3) / 1e12,
                        "note": "whole training loop (features, 4 forward, 3 backward-data, 4 weight-gradient "
                                "GEMMs, column sums, Adam) per step; TFLOP/s counts the GEMM flops only"},
            "per_point": [{"re": r["re"], "mach": r["mach"],
                           "plain": {k: r["plain"][k] for k in ("iterations", "seconds", "first_norm")},
                           "learned": {k: r["learned"][k] for k in ("iterations", "seconds", "first_norm", "fallback")}}
                          for r in out],
            "config": {"workload": "cylinder O-mesh %dx%d (r 0.5..50 D, radial ratio %.4f), Re U(40, 200), Mach "
                                   "U(0.05, 0.3); %d training points (seed 5), %d held out (seed 6); Newton cfl 1e10, "
                                   "GPU Jacobian, %s; the first base flow by grid sequencing %s" % (
                                       im, jm, ratio, len(train), len(held),
                                       "FP64 GMRES with a reused FP32 band LU preconditioner" if solver is not None
                                       else "FP64 band LU", " -> ".join("%dx%d" % lv for lv in WS.sequence_levels(im, jm)))},
            "linear_solves": None if solver is None else {
                "count": len(solver.log), "factorisations": int(sum(k["refactored"] for k in solver.log)),
                "gmres_iterations_mean": float(np.mean([k["iterations"] for k in solver.log])),
                "seconds_factor_total": float(sum(k["seconds_factor"] for k in solver.log)),
                "seconds_gmres_total": float(sum(k["seconds_gmres"] for k in solver.log))},
            "cpu_baseline": {"value": None, "unit": "s", "kind": "port", "cores": 0,
                             "sample": "none: both arms run the same GPU Newton iteration and differ only in "
                                       "the initial state; the comparison is learned vs plain start"}}
    if solver is not None:
        def stats(entries):
            return {"count": len(entries), "factorisations": int(sum(k["refactored"] for k in entries)),
                    "gmres_iterations": int(sum(k["iterations"] for k in entries)),
                    "seconds_factor": float(sum(k["seconds_factor"] for k in entries)),
                    "seconds_gmres": float(sum(k["seconds_gmres"] for k in entries))}
        line["held_out_linear_solves"] = {
            "protocol": "each arm its own Krylov solver, both without a factor at the first held-out point, each "
                        "keeping its own FP32 factor from point to point",
            "plain": stats(solver.log[n_gen:]), "learned": stats(solver_learned.log)}
    print(json.dumps(line))
    return 0


def _hbm_peak():
    """Measured HBM copy bandwidth (GB/s) of this GPU pool, else the fallback figure."""
    try:
        return float(json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["hbm_gbs"])
    except (OSError, KeyError, ValueError):
        return 6800.0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-extras", action="store_true", help="default line without the cylinder extra key")
    ap.add_argument("--lmax", type=int, default=10, help="impli workload: Gauss-Seidel sweeps per call")
    ap.add_argument("--chunks", type=int, default=16,
                    help="batch workload: chunks of grids whose uploads, graph replays and downloads overlap in the "
                         "host-array (e2e) run, 1..16")
    ap.add_argument("--case", default="bl", choices=["bl", "cyl"], help="newton workload: boundary layer or cylinder")
    ap.add_argument("--solver", default="auto", choices=["auto", "band", "krylov"],
                    help="newton / warmstart workloads: FP64 band LU, or FP64 GMRES with an FP32 band LU "
                         "preconditioner (auto: band for the newton workload, krylov above 20000 cells for warmstart)")
    ap.add_argument("--ntrain", type=int, default=200, help="warmstart workload: training base flows")
    ap.add_argument("--nheld", type=int, default=20, help="warmstart workload: held-out (Re, Mach) points")
    ap.add_argument("--train-steps", type=int, default=3000, help="warmstart workload: Adam steps")
    ap.add_argument("--batch", type=int, default=16384, help="warmstart workload: samples per Adam step")
    ap.add_argument("--workload", default="batch",
                    choices=["batch", "cylinder", "jacobian", "impli", "newton", "warmstart"],
                    help="batch (default): residual + JVP of the 64 uneven boundary-layer grids in one graph; "
                         "cylinder: the 256x256 cylinder residual + 32-direction JVP line; jacobian: the batched "
                         "Jacobian / Dz / Dzz / J(beta) assembly of the 1024x512 boundary layer")
    ap.add_argument("--grids", type=int, default=0, help="batch workload: the first N grids of the 64")
    ap.add_argument("--tile", default="", help="batch workload: fixed tile shapes F,C,N instead of the autotuner")
    ap.add_argument("--im", type=int, default=0)
    ap.add_argument("--jm", type=int, default=0)
    args = ap.parse_args()
    if args.workload == "jacobian":
        return run_jacobian_workload(args)
    if args.workload == "impli":
        return run_impli_workload(args)
    if args.workload == "newton":
        return run_newton_workload(args)
    if args.workload == "warmstart":
        return run_warmstart_workload(args)
    if args.workload == "cylinder":
        return run_reference(args) if args.impl == "reference" else run_cylinder(args)
    return run_batch_reference(args) if args.impl == "reference" else run_batch(args)


if __name__ == "__main__":
    sys.exit(main())
