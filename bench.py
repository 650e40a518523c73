"""Benchmark of the forward + adjoint k-ratio solve on the 2D workload (60 solves per step).

Workload: 256 (lateral) x 128 (depth) grid over 2 x 1 um, P_11 (78 active moments), Fe/Cr/Ni with
a seeded smooth mass-fraction field, 20 beam positions x {10, 15, 20} keV, forward + adjoint for
each of the 60 beam/energy combinations.  Synthetic data (seeded); the step counts follow the
stability estimate of the march (200, 372 and 702 steps for the three energies).

One bench step = all 60 forward + adjoint solves.
  value          FP64 "plain" solves/s: one solve at a time through the device-pointer C ABI
                 (inputs resident in HBM), per-solve latencies from CUDA events
  fp32_batched   the same 60 solves in FP32 (FP64 accumulators), all in flight at once
  e2e            FP64 plain through the host-pointer C ABI (pinned host buffers, copies timed)
  roofline       the sub-step kernel (dominant kernel): algorithmic bytes per launch / launch time
  cpu_baseline   the CPU oracle on the host cores, bounded sample, extrapolated to solves/s

`--impl reference` times the CPU oracle (the restatement of the reference's Julia path; Julia is
not available) on all host cores with the same metric and prints its own line.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "forward+adjoint k-ratio solves/s (2D, 60 beam/energy combinations)"
WORKLOAD = "2D 256x128 P11 Fe/Cr/Ni, 20 positions x {10,15,20} keV, forward+adjoint"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--positions", type=int, default=20, help="beam positions per energy (20 = full workload)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-sample-steps", type=int, default=3)
    ap.add_argument("--profile", action="store_true",
                    help="run one 10 keV solve (FP64 twice, FP32 once) for a profiler, print nothing else")
    ap.add_argument("--profile-batch", action="store_true",
                    help="run one FP32 batch (16 positions at 10 keV, 6 GiB of tapes) twice for a profiler")
    ap.add_argument("--serve", action="store_true",
                    help="served stream: Poisson requests (1D/2D/3D mix) through pn_server; prints its own line")
    ap.add_argument("--serve-requests", type=int, default=48)
    ap.add_argument("--serve-rate", type=float, default=200.0)
    ap.add_argument("--serve-budget-gb", type=float, default=150.0)
    return ap.parse_args()


# ------------------------------------------------------------------------------------------------
def workload(positions):
    from pnepma_gb300 import workloads
    return workloads.config2(n_positions=positions)


def algorithmic_bytes_per_step(solve, elem):
    """Bytes one energy step moves in the sub-step kernels: s_u (4 M_even + 5 M_odd) +
    8 n_e (2 C_odd + C_even), M = interior values, C = interior cells of each parity."""
    g = solve.problem.gspec
    from pnepma_gb300.moments import class_sizes, parity
    nm = class_sizes(solve.problem.N)
    M = [0, 0]
    C = [0, 0]
    for c in g.active_classes():
        if nm[c] == 0:
            continue
        rx, ry, rz = g.interior_ranges(c)
        cells = len(rx) * len(ry) * len(rz)
        M[parity(c)] += cells * nm[c]
        C[parity(c)] += cells
    ne = len(solve.problem.elements)
    return elem * (4 * M[0] + 5 * M[1]) + 8 * ne * (2 * C[1] + C[0]), M[0] + M[1]


class Clocks:
    """nvidia-smi sampling of the SM clock and throttle reasons during the timed region."""

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                mx = float(r[2])
                for n, v in zip(names, r[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(n)
            except (ValueError, IndexError):
                pass
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# ------------------------------------------------------------------------------------------------
def cpu_sample(solves, threads, sample_steps):
    """Oracle time of `threads` solves truncated to `sample_steps` steps, run concurrently; returns
    (seconds per energy step per core, description)."""
    sys.path.insert(0, os.path.join(HERE, "oracle"))
    import oracle
    from pnepma_gb300.problem import ForwardPNProblem
    picks = [solves[(i * 7) % len(solves)] for i in range(threads)]
    descs, keeps, rhos, noas, acss, ibars = [], [], [], [], [], []
    for s in picks:
        p = s.problem
        q = ForwardPNProblem(p.N, p.gspec, p.elements, p.beam_energy, p.beam_position, p.beam_direction,
                             p.E_initial, p.E_initial - sample_steps * p.delta_e, sample_steps)
        d, k = q.descriptor(s.x_rays)
        rho, noa, acs = s.inputs()
        descs.append(d)
        keeps.append((k, q))
        rhos.append(rho)
        noas.append(noa)
        acss.append(acs)
        ibars.append(np.ones(len(s.x_rays)))
    t0 = time.perf_counter()
    oracle.solve_many(descs, rhos, noas, acss, ibars, threads)
    wall = time.perf_counter() - t0
    per_step_core = wall / sample_steps
    desc = (f"{threads} of the 60 solves truncated to {sample_steps} energy steps each, forward+adjoint, "
            f"one solve per host thread; scaled by the full step counts")
    return per_step_core, desc, wall


def cpu_solves_per_s(solves, per_step_core, threads):
    total_steps = sum(s.problem.N_steps for s in solves)
    return len(solves) / (per_step_core * total_steps / threads)


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    solves = workload(args.positions)
    threads = os.cpu_count() or 1
    vals = []
    for _ in range(args.warmup):
        cpu_sample(solves, threads, args.cpu_sample_steps)
    walls = []
    for _ in range(args.steps):
        per, desc, wall = cpu_sample(solves, threads, args.cpu_sample_steps)
        vals.append(cpu_solves_per_s(solves, per, threads))
        walls.append(wall)
    v = float(np.median(vals))
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "solves/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * len(solves) / v,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded)",
        "config": {"workload": WORKLOAD, "solves_per_step": len(solves),
                   "energy_steps": sorted(set(s.problem.N_steps for s in solves)),
                   "reference_runtime": "Julia unavailable on this box: CPU FP64 restatement of the reference march"},
        "cpu_baseline": {"value": v, "unit": "solves/s", "cores": threads, "kind": "port",
                         "sample": desc},
        "e2e": {"value": v, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------------------------------------
def run_ours(args):
    import torch
    from pnepma_gb300 import capi
    from pnepma_gb300.problem import PN_FP32, PN_FP64

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    dev = torch.device("cuda", local)

    solves = workload(args.positions)
    nsol = len(solves)
    rho, noa, acs = solves[0].inputs()          # one material: all solves share the input arrays
    nr = len(solves[0].x_rays)

    def dbuf(a):
        return torch.from_numpy(np.ascontiguousarray(a)).to(dev)

    d_rho, d_noa, d_acs = dbuf(rho), dbuf(noa), dbuf(acs)
    handles64, handles32, ibars = [], [], []
    for s in solves:
        s.problem.precision = PN_FP64
        d, k = s.problem.descriptor(s.x_rays)
        handles64.append(capi.Handle(d, k))
    sz = handles64[0].sizes
    outI = torch.zeros((nsol, nr), dtype=torch.float64, device=dev)
    outI32 = torch.zeros((nsol, nr), dtype=torch.float64, device=dev)
    d_ibar = torch.ones((nsol, nr), dtype=torch.float64, device=dev)
    rb = [torch.zeros(sz.n_rho, dtype=torch.float64, device=dev) for _ in range(2)]
    nb = [torch.zeros(sz.n_noa, dtype=torch.float64, device=dev) for _ in range(2)]
    ab = [torch.zeros(max(sz.n_acs, 1), dtype=torch.float64, device=dev) for _ in range(2)]
    stream = torch.cuda.Stream(device=dev)
    sp = stream.cuda_stream
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)   # 256 MiB > L2

    def solve64(i, slot=0):
        h = handles64[i]
        h.forward_device(d_rho.data_ptr(), d_noa.data_ptr(), d_acs.data_ptr(), outI[i].data_ptr(), sp)
        h.adjoint_device(d_ibar[i].data_ptr(), rb[slot].data_ptr(), nb[slot].data_ptr(), ab[slot].data_ptr(), sp)

    # cotangents: dk/dI of a squared k-ratio loss scale like 1/I; use 1/|I| from one forward
    with torch.cuda.stream(stream):
        for i in range(nsol):
            handles64[i].forward_device(d_rho.data_ptr(), d_noa.data_ptr(), d_acs.data_ptr(), outI[i].data_ptr(), sp)
    stream.synchronize()
    d_ibar.copy_(1.0 / outI.abs())

    # ---------------- FP64 plain: one solve at a time
    def plain_step(record):
        ev = []
        with torch.cuda.stream(stream):
            flush.fill_(1.0)
            start = torch.cuda.Event(enable_timing=True)
            start.record(stream)
            for i in range(nsol):
                solve64(i)
                if record:
                    e = torch.cuda.Event(enable_timing=True)
                    e.record(stream)
                    ev.append(e)
            end = torch.cuda.Event(enable_timing=True)
            end.record(stream)
        return start, ev, end

    for _ in range(args.warmup):
        plain_step(False)
    stream.synchronize()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    steps_ms, lat = [], []
    with Clocks(local) as clk:
        t_wall = time.perf_counter()
        recs = [plain_step(True) for _ in range(args.steps)]
        stream.synchronize()
        torch.cuda.synchronize()
        t_wall = time.perf_counter() - t_wall
    for start, ev, end in recs:
        steps_ms.append(start.elapsed_time(end))
        prev = start
        for e in ev:
            lat.append(prev.elapsed_time(e))
            prev = e
    step_ms = float(np.mean(steps_ms))
    if dist:
        t = torch.tensor([step_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        step_ms = float(t.item())
    value = world * nsol / (step_ms / 1e3)

    # ---------------- FP32 batched: all 60 solves in one batch (one launch per sub-step)
    descs32, keep32 = [], []
    for s in solves:
        s.problem.precision = PN_FP32
        d, k = s.problem.descriptor(s.x_rays)
        descs32.append(d)
        keep32.append(k)
        s.problem.precision = PN_FP64
    batch = capi.Batch(descs32, keep32)
    rb32 = [torch.zeros(sz.n_rho, dtype=torch.float64, device=dev) for _ in range(nsol)]
    nb32 = [torch.zeros(sz.n_noa, dtype=torch.float64, device=dev) for _ in range(nsol)]
    ab32 = [torch.zeros(max(sz.n_acs, 1), dtype=torch.float64, device=dev) for _ in range(nsol)]
    p_rho = [d_rho.data_ptr()] * nsol
    p_noa = [d_noa.data_ptr()] * nsol
    p_acs = [d_acs.data_ptr()] * nsol
    p_I32 = [outI32[i].data_ptr() for i in range(nsol)]
    p_ib = [d_ibar[i].data_ptr() for i in range(nsol)]
    p_rb = [t.data_ptr() for t in rb32]
    p_nb = [t.data_ptr() for t in nb32]
    p_ab = [t.data_ptr() for t in ab32]

    def batched_step():
        with torch.cuda.stream(stream):
            flush.fill_(1.0)
            start = torch.cuda.Event(enable_timing=True)
            mid = torch.cuda.Event(enable_timing=True)
            end = torch.cuda.Event(enable_timing=True)
            start.record(stream)
            batch.forward(p_rho, p_noa, p_acs, p_I32, sp)
            mid.record(stream)
            batch.adjoint(p_ib, p_rb, p_nb, p_ab, sp)
            end.record(stream)
        return start, mid, end

    for _ in range(args.warmup):
        batched_step()
    torch.cuda.synchronize()
    b_ms, b_fwd = [], []
    for _ in range(args.steps):
        start, mid, end = batched_step()
        torch.cuda.synchronize()
        b_ms.append(start.elapsed_time(end))
        b_fwd.append(start.elapsed_time(mid))
    b_step = float(np.mean(b_ms))
    fp32_value = world * nsol / (b_step / 1e3)
    bytes32_step, _m = algorithmic_bytes_per_step(solves[0], 4)
    fwd_bytes32 = bytes32_step * sum(s.problem.N_steps for s in solves)
    fp32_fwd_gbs = fwd_bytes32 / (float(np.mean(b_fwd)) / 1e3) / 1e9
    b_lat = b_ms   # every solve of the batch completes with the batch
    binfo = batch.info()

    # accuracy of the FP32 batch against the FP64 plain results (same inputs)
    I64 = outI.cpu().numpy()
    I32 = outI32.cpu().numpy()
    k_err = float(np.max(np.abs(I32 - I64) / np.abs(I64)))
    # gradient error on one solve of each energy
    g_err = 0.0
    for i in range(0, nsol, max(1, nsol // 3)):
        with torch.cuda.stream(stream):
            solve64(i)
        stream.synchronize()
        g64 = rb[0].cpu().numpy()
        g32 = rb32[i].cpu().numpy()
        g_err = max(g_err, float(np.max(np.abs(g32 - g64)) / np.max(np.abs(g64))))

    # ---------------- e2e through the host-pointer ABI with pinned buffers
    p_rho = torch.from_numpy(rho).pin_memory()
    p_noa = torch.from_numpy(noa).pin_memory()
    p_acs = torch.from_numpy(acs).pin_memory()
    p_I = torch.zeros(nr, dtype=torch.float64).pin_memory()
    p_ibar = d_ibar.cpu().pin_memory()
    p_rb = torch.zeros(sz.n_rho, dtype=torch.float64).pin_memory()
    p_nb = torch.zeros(sz.n_noa, dtype=torch.float64).pin_memory()
    p_ab = torch.zeros(max(sz.n_acs, 1), dtype=torch.float64).pin_memory()
    L = capi.lib()
    P = capi._ptr

    def e2e_step():
        for i in range(nsol):
            h = handles64[i]
            h._check(L.pn_forward(h._h, P(p_rho.data_ptr()), P(p_noa.data_ptr()), P(p_acs.data_ptr()),
                                  P(p_I.data_ptr())))
            h._check(L.pn_adjoint(h._h, P(p_ibar[i].data_ptr()), P(p_rb.data_ptr()), P(p_nb.data_ptr()),
                                  P(p_ab.data_ptr())))

    e2e_step()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e2e_step()
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    h2d = nsol * (rho.nbytes + noa.nbytes + acs.nbytes + 8 * nr)
    d2h = nsol * (8 * nr + 8 * (sz.n_rho + sz.n_noa + sz.n_acs))

    # ---------------- roofline of the sub-step kernel (timed via the forward graph)
    fwd_ms = []
    for i in (0, nsol // 2, nsol - 1):
        h = handles64[i]
        with torch.cuda.stream(stream):
            flush.fill_(1.0)
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            h.forward_device(d_rho.data_ptr(), d_noa.data_ptr(), d_acs.data_ptr(), outI[i].data_ptr(), sp)
            b.record(stream)
        stream.synchronize()
        fwd_ms.append((a.elapsed_time(b), solves[i].problem.N_steps))
    bytes_step, m_active = algorithmic_bytes_per_step(solves[0], 8)
    launches = sum(3 * n for _t, n in fwd_ms)
    t_launch = sum(t for t, _n in fwd_ms) / launches * 1e-3
    achieved = (bytes_step / 3) / t_launch / 1e9
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(HERE, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    peak = float(peaks.get("hbm_gbs", 6800.0))
    traffic = None
    try:
        prof = json.load(open(os.path.join(HERE, "profiles", "substep_fp64_traffic.json")))
        traffic = prof.get("dram_bytes_per_launch")
    except Exception:
        pass

    gpu_launches = args.steps * sum(h.info().forward_kernels + h.info().adjoint_kernels for h in handles64)
    mcu = sum(2 * s.problem.N_steps for s in solves) * m_active

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        per, desc, wall = cpu_sample(solves, threads, args.cpu_sample_steps)
        cpu = {"value": cpu_solves_per_s(solves, per, threads), "unit": "solves/s", "cores": threads,
               "kind": "port", "sample": desc}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
            "config": {"workload": WORKLOAD, "solves_per_step": nsol,
                       "energy_steps": sorted(set(s.problem.N_steps for s in solves)),
                       "configured_energy_steps": 200, "precision": "FP64 plain, one solve at a time",
                       "l2": "256 MiB buffer written before every timed step; each solve's tape exceeds L2",
                       "replicas": "each GPU runs its own 60 solves"},
            "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                           "mean": float(np.mean(lat))},
            "fp32_batched": {"value": fp32_value, "unit": "solves/s", "ms_per_step": b_step,
                             "speedup_vs_fp64_plain": fp32_value / value,
                             "latency_ms": {"p50": float(np.percentile(b_lat, 50)),
                                            "p99": float(np.percentile(b_lat, 99))},
                             "forward_ms": float(np.mean(b_fwd)),
                             "max_rel_err_intensity_vs_fp64": k_err, "max_rel_err_rho_bar_vs_fp64": g_err,
                             "checkpoint_stride": binfo.checkpoint_stride,
                             "forward_roofline": {"bound": "hbm", "achieved": fp32_fwd_gbs,
                                                  "peak": float(json.load(open(os.path.join(HERE, "MEASURED_PEAKS.json"))).get("hbm_gbs", 6800.0)) if os.path.exists(os.path.join(HERE, "MEASURED_PEAKS.json")) else 6800.0,
                                                  "unit": "GB/s",
                                                  "note": "algorithmic bytes of all forward sub-steps of the 60 solves / forward time"},
                             "kernels_per_step": binfo.forward_kernels + binfo.adjoint_kernels,
                             "form": "one pn_batch: one launch per sub-step covers all 60 solves"},
            "moment_cell_updates_per_s": world * mcu / (step_ms / 1e3),
            "e2e": {"value": world * nsol / e2e_s, "unit": "solves/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic,
                         "kernel": "substep_kernel<double,11> (forward)",
                         "algorithmic_bytes_per_launch": bytes_step / 3,
                         "launch_us": t_launch * 1e6},
            "gpu_launches": gpu_launches,
            "clocks": clk.summary(),
            "wall_s_timed": t_wall,
        }
        if cpu:
            line["cpu_baseline"] = cpu
        print(json.dumps(line), flush=True)
    for h in handles64:
        h.close()
    batch.close()
    if dist:
        dist.barrier()
        dist.destroy_process_group()


def run_profile(args):
    """One solve of the workload (10 keV, central beam) for ncu: FP64 forward+adjoint twice, FP32 once."""
    import torch
    from pnepma_gb300 import capi, workloads
    from pnepma_gb300.problem import PN_FP32
    torch.cuda.set_device(0)
    s = workloads.config2(n_positions=1, energies=(10.0,))[0]
    rho, noa, acs = s.inputs()
    d, k = s.problem.descriptor(s.x_rays)
    h = capi.Handle(d, k)
    for _ in range(2):
        I = h.forward(rho, noa, acs)
        h.adjoint(1.0 / np.abs(I))
    s.problem.precision = PN_FP32
    d32, k32 = s.problem.descriptor(s.x_rays)
    h32 = capi.Handle(d32, k32)
    I32 = h32.forward(rho, noa, acs)
    h32.adjoint(1.0 / np.abs(I))
    torch.cuda.synchronize()
    print(json.dumps({"profile_case": s.label, "steps": s.problem.N_steps, "I": I.tolist(), "I32": I32.tolist(),
                      "fp64": h.info().forward_kernels + h.info().adjoint_kernels}))
    h.close()
    h32.close()


def run_profile_batch(args):
    """FP32 batch of 16 beam positions at 10 keV (state 160 MB > L2), forward + adjoint twice, tapes
    within 6 GiB."""
    import torch
    from pnepma_gb300 import capi, workloads
    from pnepma_gb300.problem import PN_FP32
    torch.cuda.set_device(0)
    solves = workloads.config2(n_positions=16, energies=(10.0,), precision=PN_FP32)
    descs, keep = [], []
    for s in solves:
        d, k = s.problem.descriptor(s.x_rays)
        descs.append(d)
        keep.append(k)
    b = capi.Batch(descs, keep, memory_budget=6 << 30)
    rho, noa, acs = solves[0].inputs()
    dv = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    d_rho, d_noa, d_acs = dv(rho), dv(noa), dv(acs)
    n = len(solves)
    nr = len(solves[0].x_rays)
    I = torch.zeros((n, nr), dtype=torch.float64, device="cuda")
    ib = torch.ones((n, nr), dtype=torch.float64, device="cuda")
    sz = capi.query_sizes(descs[0])
    rb = [torch.zeros(sz.n_rho, dtype=torch.float64, device="cuda") for _ in range(n)]
    nb = [torch.zeros(sz.n_noa, dtype=torch.float64, device="cuda") for _ in range(n)]
    ab = [torch.zeros(sz.n_acs, dtype=torch.float64, device="cuda") for _ in range(n)]
    for _ in range(2):
        b.forward([d_rho.data_ptr()] * n, [d_noa.data_ptr()] * n, [d_acs.data_ptr()] * n, [I[i].data_ptr() for i in range(n)])
        torch.cuda.synchronize()
        ib.copy_(1.0 / I.abs())
        b.adjoint([ib[i].data_ptr() for i in range(n)], [t.data_ptr() for t in rb], [t.data_ptr() for t in nb],
                  [t.data_ptr() for t in ab])
        torch.cuda.synchronize()
    info = b.info()
    print(json.dumps({"profile_batch": len(solves), "steps": solves[0].problem.N_steps,
                      "stride": info.checkpoint_stride, "bytes": info.device_bytes,
                      "kernels": info.forward_kernels + info.adjoint_kernels}))
    b.close()


# ------------------------------------------------------------------------------------------------
class ServedStream:
    """The served stream's requests with their descriptors and inputs, prepared before timing."""

    def __init__(self, n_requests, rate, precision):
        from pnepma_gb300 import workloads
        self.reqs = workloads.config5(n_requests=n_requests, rate=rate, precision=precision)
        self.prepared = {}
        for r in self.reqs:
            key = id(r.solves)
            if key in self.prepared:
                continue
            items, keep = [], []
            rho, noa, acs = r.solves[0].inputs()
            for s in r.solves:
                d, k = s.problem.descriptor(s.x_rays)
                keep.append(k)
                items.append((d, rho, noa, acs, np.ones(len(s.x_rays))))
            self.prepared[key] = (items, keep)

    def items(self, r):
        return self.prepared[id(r.solves)][0]


def serve_run(stream, budget, rate_scale=1.0, reqs=None):
    """Submit every request at its arrival time (scaled), wait for all; returns the measurements."""
    from pnepma_gb300 import capi
    reqs = stream.reqs if reqs is None else reqs
    with capi.Server(memory_budget=budget) as srv:
        tickets = []
        t0 = time.perf_counter()
        for r in reqs:
            due = t0 + r.arrival_s / rate_scale
            now = time.perf_counter()
            if due > now:
                time.sleep(due - now)
            tickets.append(srv.submit(stream.items(r), adjoint=True))
        for t in tickets:
            t.wait()
        wall = time.perf_counter() - t0
        infos = [t.info() for t in tickets]
        sinfo = srv.info()
    lat = np.array([i.total_ms for i in infos])
    queued = np.array([i.queued_ms for i in infos])
    solves = sum(len(r.solves) for r in reqs)
    out = {"requests": len(reqs), "solves": solves, "wall_s": wall,
           "solves_per_s": solves / wall, "requests_per_s": len(reqs) / wall,
           "offered_requests_per_s": len(reqs) / max(reqs[-1].arrival_s / rate_scale, 1e-9),
           "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                          "mean": float(np.mean(lat))},
           "queued_ms": {"p50": float(np.percentile(queued, 50)), "p99": float(np.percentile(queued, 99))},
           "waves": int(sinfo.waves_launched), "max_waves_in_flight": int(sinfo.max_waves_in_flight),
           "wave_build_ms_mean": sinfo.wave_build_us / 1e3 / max(1, sinfo.waves_launched),
           "peak_device_bytes": int(sinfo.peak_bytes)}
    by_kind = {}
    for r, l in zip(reqs, lat):
        by_kind.setdefault(r.kind, []).append(l)
    out["latency_ms_by_kind"] = {k: {"n": len(v), "p50": float(np.percentile(v, 50)),
                                     "p99": float(np.percentile(v, 99))} for k, v in sorted(by_kind.items())}
    return out


def fp64_sequential_seconds(stream):
    """FP64 plain, one solve at a time (device-pointer ABI, inputs resident): the time of one solve
    of each (kind, energy), timed with CUDA events, summed over the stream's solves."""
    import torch
    from pnepma_gb300 import capi
    from pnepma_gb300.problem import PN_FP64
    dev = torch.device("cuda", 0)
    stream_ = torch.cuda.Stream(device=dev)
    per = {}
    samples = {}
    for r in stream.reqs:
        for s in r.solves:
            key = (r.kind, s.problem.N_steps)
            samples.setdefault(key, s)
    for key, s in samples.items():
        prec = s.problem.precision
        s.problem.precision = PN_FP64
        d, k = s.problem.descriptor(s.x_rays)
        s.problem.precision = prec
        h = capi.Handle(d, k)
        rho, noa, acs = s.inputs()
        dv = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
        x, y, z = dv(rho), dv(noa), dv(acs)
        I = torch.zeros(len(s.x_rays), dtype=torch.float64, device=dev)
        ib = torch.ones(len(s.x_rays), dtype=torch.float64, device=dev)
        sz = h.sizes
        rb = torch.zeros(sz.n_rho, dtype=torch.float64, device=dev)
        nb = torch.zeros(sz.n_noa, dtype=torch.float64, device=dev)
        ab = torch.zeros(max(sz.n_acs, 1), dtype=torch.float64, device=dev)
        sp = stream_.cuda_stream
        ts = []
        for it in range(2):
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            with torch.cuda.stream(stream_):
                a.record(stream_)
                h.forward_device(x.data_ptr(), y.data_ptr(), z.data_ptr(), I.data_ptr(), sp)
                h.adjoint_device(ib.data_ptr(), rb.data_ptr(), nb.data_ptr(), ab.data_ptr(), sp)
                b.record(stream_)
            stream_.synchronize()
            ts.append(a.elapsed_time(b) / 1e3)
        per[key] = ts[-1]
        h.close()
    total = 0.0
    for r in stream.reqs:
        for s in r.solves:
            total += per[(r.kind, s.problem.N_steps)]
    return total, {f"{k[0]} {k[1]} steps": v * 1e3 for k, v in sorted(per.items())}


def run_serve(args):
    import torch
    from pnepma_gb300.problem import PN_FP32
    torch.cuda.set_device(0)
    t_prep = time.perf_counter()
    stream = ServedStream(args.serve_requests, args.serve_rate, PN_FP32)
    t_prep = time.perf_counter() - t_prep
    budget = int(args.serve_budget_gb * 1e9)
    first = {}
    for r in stream.reqs:
        first.setdefault(r.kind, r)
    serve_run(stream, budget, rate_scale=50.0, reqs=list(first.values()))   # warm-up: one request per kind
    with Clocks(0) as clk:
        full = serve_run(stream, budget)
    seq_s, per_solve_ms = fp64_sequential_seconds(stream)
    seq = full["solves"] / seq_s
    # a sustainable load: the same stream at 60 % of the measured request capacity
    scale = 0.6 * full["requests_per_s"] / args.serve_rate
    light = serve_run(stream, budget, rate_scale=scale)
    mix = {}
    for r in stream.reqs:
        mix[r.kind] = mix.get(r.kind, 0) + 1
    line = {
        "metric": "served forward+adjoint k-ratio solves/s (Poisson 1D/2D/3D request stream)",
        "value": full["solves_per_s"], "unit": "solves/s", "n_gpus": 1, "higher_is_better": True,
        "dtype": "f32 state and stencil, f64 accumulators", "data": "synthetic (seeded)",
        "config": {"workload": "config5 stream: requests of 16 positions x {10, 15} keV forward+adjoint; "
                               "1D N=7 200 cells / 2D N=11 128x64 / 3D N=5 64x64x48 at 50/40/10",
                   "requests": len(stream.reqs), "mix": mix, "rate_requests_per_s": args.serve_rate,
                   "memory_budget_bytes": budget, "host_prep_s": t_prep},
        "at_offered_rate": full,
        "at_60pct_capacity": light,
        "fp64_plain_sequential": {"solves_per_s": seq, "seconds_for_stream": seq_s,
                                  "per_solve_ms": per_solve_ms,
                                  "method": "one FP64 solve per (kind, step count) timed with CUDA events, summed"},
        "speedup_vs_fp64_plain_sequential": full["solves_per_s"] / seq,
        "clocks": clk.summary(),
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.profile:
        run_profile(args)
    elif args.profile_batch:
        run_profile_batch(args)
    elif args.serve:
        run_serve(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
