"""Benchmark: EPG voxel·pulse·state updates/s on the MRF dictionary workload.

Workload (one step): the 880-pulse MRF sequence (flip 5->60 deg over 300
pulses, 60->2 deg over 300, 280 x 2 deg; TR 10 ms; inversion at t = 0) over a
128 x 64 x 32 grid of T1 (geomspace 100-4000 ms) x T2 (geomspace 5-500 ms) x
B1 (linspace 0.6-1.4) = 262,144 atoms, nstates 20, FP32, writing the
complex64 signal AND the forward-mode Jacobian w.r.t. T1, T2 and B1 in one
fused kernel pass. Atoms with T2 >= T1 are simulated like the rest (the count
stays 262,144). Inputs are synthetic and seeded; the outputs (7.4 GB per step)
are larger than L2, and an explicit 512 MB L2 flush runs between timed steps.

Printed: one JSON line (rank 0). ``value`` is updates/s with inputs resident
on the device; ``e2e`` is the same metric through the public API with the
tissue copied in from pinned host memory and the signal and Jacobian copied
back to pinned host memory inside the timed region. ``--impl reference`` times
the reference's own CPU kernels (or, where they cannot be built, the oracle's
FP32 port of them) on the host cores instead.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

PULSES = 880
STATES = 20
GRID = (128, 64, 32)
ATOMS = GRID[0] * GRID[1] * GRID[2]
# Algorithmic FP32 FLOPs per voxel, pulse and order (FMA = 2): 18 for the
# forward (relaxation 3, rotation 15) and 42 per forward-mode tangent.
FLOPS_PER_UPDATE = 18 + 42 * 3
WORKLOAD = "mrf_dictionary_fwd_jac"


def mrf_schedule() -> np.ndarray:
    return np.concatenate(
        [np.linspace(5, 60, 300), np.linspace(60, 2, 300), np.full(280, 2.0)]
    ).astype(np.float32)


def dictionary_grid(atoms: int = ATOMS):
    """The first ``atoms`` entries of the T1 x T2 x B1 grid (all of it by default)."""
    t1 = np.geomspace(100, 4000, GRID[0]).astype(np.float32)
    t2 = np.geomspace(5, 500, GRID[1]).astype(np.float32)
    b1 = np.linspace(0.6, 1.4, GRID[2]).astype(np.float32)
    T1, T2, B1 = np.meshgrid(t1, t2, b1, indexing="ij")
    return T1.ravel()[:atoms].copy(), T2.ravel()[:atoms].copy(), B1.ravel()[:atoms].copy()


def config(extra=None):
    c = {
        "workload": WORKLOAD,
        "sequence": "MRF inversion + 880 pulses (5-60-2 deg), TR 10 ms",
        "atoms": ATOMS,
        "grid": "T1 geomspace(100,4000,128) x T2 geomspace(5,500,64) x B1 linspace(0.6,1.4,32)",
        "nstates": STATES,
        "jacobian": ["T1", "T2", "B1"],
        "outputs": "complex64 signal (262144,880) + Jacobian (262144,3,880)",
        "l2": "512 MB flush between timed steps; outputs 7.4 GB per step exceed L2",
        "parallelism": "replicas",
    }
    if extra:
        c.update(extra)
    return c


# ---- clocks -----------------------------------------------------------------


class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int) -> None:
        self.index = index
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None
            return self
        # nvidia-smi takes a moment to start: begin the timed region only once
        # it is sampling (at most 5 s).
        deadline = time.perf_counter() + 5.0
        while not self.lines and self.proc.poll() is None and time.perf_counter() < deadline:
            time.sleep(0.01)
        self.first = len(self.lines)
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.thread.join(timeout=2)

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        # The samples taken while the timed region ran (the last one taken
        # before it as well when it was shorter than the sampling period).
        first = getattr(self, "first", 0)
        lines = self.lines[first:] if len(self.lines) > first else self.lines[max(0, first - 1):]
        for line in lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for name, flag in zip(names, parts[5:9], strict=False):
                if flag.lower() in ("active", "1"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# ---- the GPU arm ------------------------------------------------------------


def fp32_peak(torch, lib, device, paired: bool = False) -> float:
    """FP32 FLOP/s of the FMA probe kernel on this GPU (best of 5); with
    ``paired`` the probe issues paired FMAs (two per instruction)."""
    import ctypes

    sms = torch.cuda.get_device_properties(device).multi_processor_count
    blocks, threads, iters = sms * 8, 256, 4096
    out = torch.zeros(blocks, device=device)
    stream = torch.cuda.current_stream().cuda_stream
    flops = ctypes.c_double()
    best = 0.0
    for _ in range(6):
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        probe = lib.tsg_probe_fp32x2 if paired else lib.tsg_probe_fp32
        rc = probe(blocks, threads, iters, out.data_ptr(), stream, ctypes.byref(flops))
        e.record()
        e.synchronize()
        if rc != 0:
            raise RuntimeError("fp32 probe failed")
        best = max(best, flops.value / (s.elapsed_time(e) * 1e-3))
    return best


def traffic_per_launch() -> float | None:
    """DRAM bytes per launch of the fused dictionary kernel, from the
    committed ncu summary (profiles/), if one has been recorded."""
    path = ROOT / "profiles" / "sweep_t12b_mrf_dictionary.md"
    if not path.exists():
        return None
    for line in path.read_text().splitlines():
        if line.startswith("dram_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1].strip())
            except ValueError:
                return None
    return None


def host_link(torch, device, d2h_bytes: int, size: int = 2 << 30) -> dict:
    """Device-to-host copy bandwidth of this machine (2 GB, best of 4) into
    page-locked memory allocated while the process runs on the CPUs of each
    NUMA node in turn, and into pageable memory; and the time the e2e call's
    copies need at the best of them (the host link's bound on that call)."""
    import glob

    nodes = {}
    for path in sorted(glob.glob("/sys/devices/system/node/node[0-9]*")):
        cpus = set()
        for part in open(path + "/cpulist").read().strip().split(","):
            if part:
                a, _, b = part.partition("-")
                cpus |= set(range(int(a), int(b or a) + 1))
        nodes[int(path.rsplit("node", 1)[1])] = cpus
    src = torch.empty(size, dtype=torch.uint8, device=device)
    src.fill_(1)

    def rate(host):
        best = 0.0
        for _ in range(4):
            s0, e0 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s0.record()
            host.copy_(src, non_blocking=True)
            e0.record()
            e0.synchronize()
            best = max(best, size / (s0.elapsed_time(e0) * 1e-3) / 1e9)
        return best

    out = {"numa_nodes": len(nodes)}
    mine = os.sched_getaffinity(0)
    for node, cpus in nodes.items():
        if not cpus & mine:
            continue
        os.sched_setaffinity(0, cpus & mine)
        try:
            buf = torch.empty(size, dtype=torch.uint8, pin_memory=True)
            buf.fill_(0)
            out[f"pinned_node{node}_gbs"] = rate(buf)
            del buf
        finally:
            os.sched_setaffinity(0, mine)
    buf = torch.empty(size, dtype=torch.uint8)
    buf.fill_(0)
    out["pageable_gbs"] = rate(buf)
    del buf, src
    best = max(v for k, v in out.items() if k.endswith("_gbs"))
    out["e2e_copy_bound_ms"] = d2h_bytes / (best * 1e9) * 1e3
    return out


def job_seconds(local_seconds: float, dist, device) -> float:
    """The job's time for N replicas: the slowest rank's (max over ranks)."""
    if dist is None:
        return local_seconds
    import torch

    t = torch.tensor([local_seconds], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_value(units_per_step: float, steps: int, world: int, seconds: float) -> float:
    """Whole-job throughput: the units every rank processed over the job's time."""
    return units_per_step * steps * world / seconds


def run_gpu(args, rank: int, world: int, dist) -> dict | None:
    import torch

    from torchsim_gb300 import _native, engine
    from torchsim_gb300.sequence import mrf_events, program_for

    local = int(os.environ.get("LOCAL_RANK", "0"))
    device = torch.device("cuda", local)
    torch.cuda.set_device(device)
    lib = _native.library()
    flip = mrf_schedule()
    events = mrf_events(flip, 10.0)
    program = program_for(events, device)
    atoms = args.atoms
    t1, t2, b1 = dictionary_grid(atoms)
    tissue = engine.tissue_maps(device, atoms, torch.from_numpy(t1), torch.from_numpy(t2), None,
                                torch.from_numpy(b1), None)
    names = ("T1", "T2", "B1")
    sig = torch.empty((atoms, PULSES), dtype=torch.complex64, device=device)
    jac = torch.empty((atoms, 3, PULSES), dtype=torch.complex64, device=device)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=device)
    tune_info = None
    if args.launch:
        launch = tuple(args.launch)
    else:
        t_tune = time.perf_counter()
        launch = engine.tuned_shape(program, tissue, STATES, names, use_cache=False)
        tune_info = {"shape": {"lanes_per_voxel": launch[0], "orders_per_lane": launch[1],
                               "warps_per_block": launch[2],
                               "min_blocks_per_sm": launch[3] if len(launch) > 3 else 0},
                     "tuning_s": time.perf_counter() - t_tune, "sample_atoms": min(32768, atoms)}

    def step():
        engine.forward_tangents(program, tissue, STATES, names, sig_out=sig, jac_out=jac,
                                launch=launch)

    for _ in range(args.warmup):
        step()
        flush.zero_()
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    with ClockSampler(local) as clocks:
        torch.cuda.synchronize()
        wall0 = time.perf_counter()
        for i in range(args.steps):
            starts[i].record()
            step()
            ends[i].record()
            flush.zero_()
        torch.cuda.synchronize()
        wall = time.perf_counter() - wall0
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends, strict=True)]
    total_s = job_seconds(sum(step_ms) * 1e-3, dist, device)
    updates = float(atoms) * PULSES * STATES
    value = job_value(updates, args.steps, world, total_s)
    kernel_s = total_s / args.steps

    # Plain form: the reference's call pattern on the GPU -- one forward pass,
    # then one forward+tangent pass per Jacobian column (torch.func.jvp per
    # property, model/_signal.py:233-268) -- through the same kernels.
    plain = None
    if rank == 0 and not args.skip_plain:
        one = torch.empty((atoms, 1, PULSES), dtype=torch.complex64, device=device)
        def plain_step():
            engine.forward(program, tissue, STATES, out=sig)
            for name in names:
                engine.forward_tangents(program, tissue, STATES, (name,), sig_out=sig,
                                        jac_out=one)
        plain_step()
        torch.cuda.synchronize()
        ps, pe = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ps.record()
        for _ in range(max(1, args.steps // 2)):
            plain_step()
        pe.record()
        pe.synchronize()
        plain_s = ps.elapsed_time(pe) * 1e-3 / max(1, args.steps // 2)
        plain = {"value": updates / plain_s, "ms_per_step": plain_s * 1e3,
                 "launches_per_step": 4,
                 "form": "forward + one forward-and-tangent pass per column (T1, T2, B1)"}
        del one

    # End to end through the public API: the call a user makes with host
    # tensors, torchsim_gb300.mrf_sim(flip, TR, T1, T2, B1=..., diff=(T1, T2,
    # B1), states=20) on CPU tensors, returning the signal and Jacobian as CPU
    # tensors; the tissue upload, the sweep and the copies back (chunked, each
    # overlapping the next chunk's sweep) are inside the timed region.
    def measure_e2e() -> dict:
        """End to end through the public API (run after the device-timed
        sections, so the host has settled from whatever ran before)."""
        import torchsim_gb300 as ts

        host_flip = torch.from_numpy(flip)
        host_t = [torch.from_numpy(a) for a in (t1, t2, b1)]

        def e2e_step():
            return ts.mrf_sim(host_flip, 10.0, host_t[0], host_t[1], B1=host_t[2],
                              diff=names, states=STATES)

        out = e2e_step()
        assert out[0].device.type == "cpu" and out[1].shape == (atoms, 3, PULSES)
        d2h = int(out[0].numel() * 8 + out[1].numel() * 8)
        del out
        # The same W untimed warm-up steps as the device-timed region: the
        # first calls after the other sections pay one-off host costs
        # (page-locked blocks, cached device buffers).
        for _ in range(max(0, args.warmup - 1)):
            out = e2e_step()
            del out
        torch.cuda.synchronize()
        n_e2e = max(1, min(args.steps, 10))
        e2e_steps = []
        t0 = time.perf_counter()
        for _ in range(n_e2e):
            t_step = time.perf_counter()
            out = e2e_step()
            del out
            torch.cuda.synchronize()
            e2e_steps.append((time.perf_counter() - t_step) * 1e3)
        e2e_s = (time.perf_counter() - t0) / n_e2e
        return {"value": updates / e2e_s, "unit": "updates/s", "ms_per_step": e2e_s * 1e3,
                "steps_ms": e2e_steps, "ms_median": statistics.median(e2e_steps),
                "h2d_bytes_per_step": 3 * atoms * 4 + PULSES * 4,
                "d2h_bytes_per_step": d2h,
                "host_link": host_link(torch, device, d2h),
                "api": "torchsim_gb300.mrf_sim(flip, 10.0, T1, T2, B1=B1, "
                       "diff=('T1','T2','B1'), states=20) with CPU tensors in and out (the "
                       "public call): tissue upload, fused sweep in chunks of ~64 MB of "
                       "output, each chunk's copy to page-locked host memory overlapping the "
                       "next chunk's sweep"}

    if rank != 0:
        return None
    peak_scalar = fp32_peak(torch, lib, device)
    peak_paired = fp32_peak(torch, lib, device, paired=True)
    peak = max(peak_scalar, peak_paired)
    flops = float(atoms) * PULSES * STATES * FLOPS_PER_UPDATE
    out_bytes = float(sig.numel() * 8 + jac.numel() * 8)
    in_bytes = 3.0 * atoms * 4
    hbm_peak = None
    peaks_path = ROOT / "MEASURED_PEAKS.json"
    if peaks_path.exists():
        hbm_peak = json.loads(peaks_path.read_text()).get("hbm_gbs")
    hbm_peak = hbm_peak or 6800.0
    achieved = flops / kernel_s / 1e12
    traffic = traffic_per_launch()
    clk = clocks.summary()
    line = {
        "metric": "EPG voxel·pulse·state updates/s (fused forward + Jacobian T1/T2/B1)",
        "value": value,
        "unit": "updates/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": kernel_s * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded grid of the named shape)",
        "config": config({"atoms": atoms} if atoms != ATOMS else None),
        "roofline": {
            "bound": "fp32",
            "achieved": achieved,
            "peak": peak / 1e12,
            "unit": "TFLOP/s",
            "frac": achieved * 1e12 / peak,
            "traffic": traffic,
            "peak_source": "measured: FP32 FMA probe kernels on this GPU in this run (max of "
                           "scalar and paired FMA)",
            "peak_scalar_fma": peak_scalar / 1e12,
            "peak_paired_fma": peak_paired / 1e12,
            "flops_per_launch": flops,
            "hbm": {"achieved_gbs": (out_bytes + in_bytes) / kernel_s / 1e9,
                    "peak_gbs": hbm_peak,
                    "frac": (out_bytes + in_bytes) / kernel_s / 1e9 / hbm_peak,
                    "algorithmic_bytes_per_launch": out_bytes + in_bytes,
                    "peak_source": "MEASURED_PEAKS.json hbm_gbs (copy bandwidth)"},
        },
        "e2e": None,
        "plain_form": plain,
        "gpu_launches": args.steps,
        "launch_shape": tune_info if tune_info else {"given": list(launch)},
        "clocks": clk,
        "wall_s_timed_region": wall,
    }
    if not args.skip_adjoint:
        line["adjoint"] = adjoint_section(torch, device)
    if not args.skip_second:
        line["second_order"] = second_order_section(torch, device, voxels=args.second_voxels,
                                                    design_step=not args.skip_design_step)
    if not args.skip_batched:
        line["batched"] = batched_section(torch, device, sequences=args.batch_sequences,
                                          shape=args.batch_shape)
        b = line["batched"]
        b_flops = float(b["updates"]) * 18.0  # relax 3 + rotate 15 per update
        b_achieved = b_flops / (b["persistent_graph_ms"] * 1e-3) / 1e12
        b["roofline"] = {"bound": "fp32", "achieved": b_achieved, "peak": peak / 1e12,
                         "unit": "TFLOP/s", "frac": b_achieved * 1e12 / peak,
                         "flops_per_launch": b_flops,
                         "flop_count": "18 per update (order x echo x voxel): relaxation 3, "
                                       "rotation 15",
                         "peak_source": "the FP32 FMA probe of this run"}
    if not args.skip_gn:
        line["gn_server"] = gn_section(torch, device, requests=args.gn_requests,
                                       cpu_sample=0 if args.skip_cpu else 4096)
    if not args.skip_match:
        line["dictionary_match"] = match_section(torch, device, voxels=args.match_voxels)
    if not args.skip_e2e:
        # Start from a clean allocator state: the sections above leave tens
        # of GB of cached device blocks and host garbage behind.
        import gc

        gc.collect()
        torch.cuda.empty_cache()
        line["e2e"] = measure_e2e()
    if not args.skip_cpu:
        line["cpu_baseline"] = cpu_baseline(args.cpu_sample)
    return line


# ---- adjoint sequence-optimisation workload ---------------------------------


def adjoint_section(torch, device, repeats: int = 5) -> dict:
    """Gradient of sum |s - target|^2 over 16,384 voxels w.r.t. 600 flips and
    600 TRs (and the tissue), nstates 20: the adjoint (trajectory or
    checkpointed, whichever the tuner finds faster) against one plain forward
    of the same sequence."""
    from torchsim_gb300 import engine
    from torchsim_gb300.sequence import mrf_events, program_for

    rng = np.random.default_rng(0)
    V, n, S = 16384, 600, 20
    t1 = np.exp(rng.uniform(np.log(100), np.log(3000), V)).astype(np.float32)
    t2 = np.minimum(np.exp(rng.uniform(np.log(10), np.log(300), V)), 0.999 * t1).astype(np.float32)
    b1 = rng.uniform(0.8, 1.2, V).astype(np.float32)
    flips = rng.uniform(5, 70, n).astype(np.float32)
    trs = rng.uniform(8, 15, n).astype(np.float32)
    ev = mrf_events(flips, trs)
    prog = program_for(ev, device)
    tissue = engine.tissue_maps(device, V, torch.from_numpy(t1), torch.from_numpy(t2), None,
                                torch.from_numpy(b1), None)
    sig = torch.empty((V, n), dtype=torch.complex64, device=device)
    seed = torch.randn((V, n), dtype=torch.complex64, device=device)
    grads = {k: torch.zeros(V, device=device) for k in ("t1_ms", "t2_ms", "b1")}
    grads["flip_rad"] = torch.zeros((1, ev.events), device=device)
    grads["duration_s"] = torch.zeros((1, ev.events), device=device)
    from torchsim_gb300 import autotune

    # Both sides tuned: the forward over every sweep shape, the adjoint over
    # launch shapes and segment lengths.
    fwd_shape, _ = autotune.tune(
        autotune.workload_key("adjoint-forward", states=S, ops=prog.ops, voxels=V),
        autotune.sweep_shapes(S, engine.FAMILY_SHAPES[0]),
        lambda shape: engine.forward(prog, tissue, S, out=sig, launch=shape), use_cache=False)
    buffers = {}

    def run_adjoint(cand):
        shape, c_req = cand[:3], cand[3]
        c, ck, ws = engine.adjoint_plan(prog, V, S, shape, c_req)
        if (shape, c) not in buffers:
            buffers.clear()
            ckpt = torch.empty(ck // 4, dtype=torch.float32, device=device)
            work = torch.empty(ws, dtype=torch.uint8, device=device)
            engine.forward_checkpointed(prog, tissue, S, c, ckpt)
            buffers[(shape, c)] = (ckpt, work)
        ckpt, work = buffers[(shape, c)]
        engine.adjoint(prog, tissue, S, seed, ckpt, c, grads, workspace=work, launch=shape)

    # Segment length 1 is trajectory mode (every op's entry state kept);
    # longer segments are checkpoints with a re-run.
    adj_cands = [(*shape, c) for shape in ((1, 20, 2), (1, 20, 4), (5, 4, 2), (5, 4, 4), (4, 6, 2),
                                           (10, 2, 4), (2, 10, 2)) for c in (1, 4, 5, 6)]
    adj_best, _ = autotune.tune(autotune.workload_key("adjoint", states=S, ops=prog.ops, voxels=V),
                                adj_cands, run_adjoint, use_cache=False)
    shape, c_req = tuple(adj_best[:3]), adj_best[3]
    c, ck, ws = engine.adjoint_plan(prog, V, S, shape, c_req)
    ckpt = torch.empty(ck // 4, dtype=torch.float32, device=device)
    work = torch.empty(ws, dtype=torch.uint8, device=device)

    def timed(fn):
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        best = 1e30
        for _ in range(repeats):
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.record()
            fn()
            e.record()
            e.synchronize()
            best = min(best, s.elapsed_time(e))
        return best

    fwd = timed(lambda: engine.forward(prog, tissue, S, out=sig, launch=fwd_shape))
    fwd_ck = timed(lambda: engine.forward_checkpointed(prog, tissue, S, c, ckpt, out=sig,
                                                       launch=fwd_shape))
    bwd = timed(lambda: engine.adjoint(prog, tissue, S, seed, ckpt, c, grads, workspace=work,
                                       launch=shape))
    del ckpt, work
    # The complex path: the same sequence with RF phases U(-40, 40) deg and
    # per-voxel B0 U(-40, 40) Hz and B1phase U(-0.5, 0.5) rad.
    cev = mrf_events(flips, trs, phases_deg=rng.uniform(-40, 40, n))
    cprog = program_for(cev, device, phased=True)
    off, keep = engine.offaxis_maps(device, V, rng.uniform(-0.5, 0.5, V).astype(np.float32),
                                    rng.uniform(-40, 40, V).astype(np.float32))
    csig = torch.empty((V, n), dtype=torch.complex64, device=device)
    tb, wb = engine.complex_adjoint_plan(cprog, V, S)
    ctraj = torch.empty(tb, dtype=torch.uint8, device=device)
    cwork = torch.empty(wb, dtype=torch.uint8, device=device)
    cgrads = {k: torch.zeros(V, device=device) for k in ("t1_ms", "t2_ms", "b1", "b1_phase_rad",
                                                         "b0_hz")}
    for k in ("flip_rad", "duration_s", "phase_rad"):
        cgrads[k] = torch.zeros((1, cev.events), device=device)
    c_fwd = timed(lambda: engine.forward_complex(cprog, tissue, S, off, out=csig))
    c_fwd_t = timed(lambda: engine.forward_complex_trajectory(cprog, tissue, S, off,
                                                              trajectory=ctraj))
    c_bwd = timed(lambda: engine.adjoint_complex(cprog, tissue, S, seed, ctraj, cgrads, off,
                                                 workspace=cwork))
    del ctraj, cwork, keep
    # One step of sequence design through the public API: flips and TRs are
    # device-resident leaves, the program is rebound on the device from them
    # (no host round trip, no compile), loss = sum |s - target|^2, backward.
    from torchsim_gb300 import MRFSimulator

    flip_leaf = torch.from_numpy(flips).to(device)
    tr_leaf = torch.from_numpy(trs).to(device)
    t1d, t2d, b1d = tissue.t1, tissue.t2, tissue.b1
    target = seed

    def design_step():
        f = flip_leaf.clone().requires_grad_(True)
        r = tr_leaf.clone().requires_grad_(True)
        s_ = MRFSimulator(flip=f, TR=r, states=S).simulate(T1=t1d, T2=t2d, B1=b1d)
        (s_ - target).abs().square().sum().backward()
        return f.grad

    for _ in range(3):
        design_step()
    torch.cuda.synchronize()
    steps_ms = []
    for _ in range(repeats):
        t0 = time.perf_counter()
        design_step()
        torch.cuda.synchronize()
        steps_ms.append((time.perf_counter() - t0) * 1e3)
    return {
        "workload": "MRF adjoint: 16384 voxels, 600 pulses (flip U(5,70) deg, TR U(8,15) ms), "
                    "nstates 20, loss sum |s - target|^2",
        "mode": "trajectory" if c == 1 else "checkpointed",
        "ops_per_checkpoint": c,
        "checkpoint_bytes": ck,
        "forward_shape": list(fwd_shape),
        # Trajectory mode up to 20 states runs one voxel per lane whatever
        # shape is requested (its warps per block are kept).
        "adjoint_shape": ([1, 10 if S <= 10 else 20, shape[2]] if c == 1 and S <= 20
                          else list(shape)),
        "forward_ms": fwd,
        "forward_with_checkpoints_ms": fwd_ck,
        "backward_ms": bwd,
        "backward_over_forward": bwd / fwd,
        "gradient_over_forward": (fwd_ck + bwd) / fwd,
        "gradient_definition": "forward with checkpoints + backward, over a plain forward (the "
                               "reference's benchmarks/anatomy.py measure: 8.4x CUDA, 4.6x CPU)",
        "forward_updates_per_s": V * n * S / (fwd * 1e-3),
        "complex": {
            "workload": "the same sequence with RF phases U(-40, 40) deg, B0 U(-40, 40) Hz, "
                        "B1phase U(-0.5, 0.5) rad per voxel (the complex path)",
            "forward_ms": c_fwd,
            "forward_with_trajectory_ms": c_fwd_t,
            "backward_ms": c_bwd,
            "backward_over_forward": c_bwd / c_fwd,
            "gradient_over_forward": (c_fwd_t + c_bwd) / c_fwd,
            "gradients": "T1, T2, B1, B1phase, B0, flip, duration, phase",
        },
        "timing": "best of 5 after 3 warm-up runs, CUDA events",
        "public_api_design_step": {
            "ms": min(steps_ms),
            "ms_median": float(np.median(steps_ms)),
            "call": "MRFSimulator(flip=f, TR=r, states=20).simulate(T1, T2, B1) with f, r "
                    "device leaves; loss sum |s - target|^2; backward (program rebound on the "
                    "device, trajectory chosen by free memory)",
            "timing": "host wall clock per step after 3 warm-up steps, synchronised",
        },
    }


# ---- second order: Cramer-Rao design gradient ---------------------------------


def second_order_section(torch, device, voxels: int = 16384, repeats: int = 5,
                         design_step: bool = True) -> dict:
    """Gradient of a Cramer-Rao design cost, sum over voxels of the bounds of
    (T1, T2, B1, M0) relative to their squares, with respect to 600 flips and
    600 TRs (nstates 20, 16,384 tissues drawn as the adjoint workload's): the
    Jacobian forward that stores the trajectory plus ONE reverse sweep over
    the three tangent directions and the M0 column, against the fused forward
    Jacobian alone and against one forward-over-reverse pass per column (the
    reference's route, sequence/_accelerators.py:1780-1800)."""
    from torchsim_gb300 import MRFSimulator, crlb, engine
    from torchsim_gb300.sequence import mrf_events, program_for

    rng = np.random.default_rng(0)
    V, n, S = voxels, 600, 20
    t1 = np.exp(rng.uniform(np.log(100), np.log(3000), V)).astype(np.float32)
    t2 = np.minimum(np.exp(rng.uniform(np.log(10), np.log(300), V)), 0.999 * t1).astype(np.float32)
    b1 = rng.uniform(0.8, 1.2, V).astype(np.float32)
    m0 = rng.uniform(0.5, 1.5, V).astype(np.float32)
    flips = rng.uniform(5, 70, n).astype(np.float32)
    trs = rng.uniform(8, 15, n).astype(np.float32)
    ev = mrf_events(flips, trs)
    prog = program_for(ev, device)
    tissue = engine.tissue_maps(device, V, torch.from_numpy(t1), torch.from_numpy(t2),
                                torch.from_numpy(m0), torch.from_numpy(b1), None)
    names = ("T1", "T2", "B1")
    mask = sum(engine.DESIGN_BITS[k] for k in names)
    seed = torch.randn((V, len(names) + 1, n), dtype=torch.complex64, device=device)
    curvature = {"flip_rad": torch.zeros((1, ev.events), device=device),
                 "duration_s": torch.zeros((1, ev.events), device=device)}

    def timed(fn):
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        best = 1e30
        for _ in range(repeats):
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.record()
            fn()
            e.record()
            e.synchronize()
            best = min(best, s.elapsed_time(e))
        return best

    jac_ms = timed(lambda: engine.forward_tangents(prog, tissue, S, (*names, "M0")))
    # Launch shape (lanes per voxel, orders per lane): forward + reverse timed
    # once each per candidate, the fastest kept.
    tuning = {}
    for shape in ((5, 4, 0), (10, 2, 0), (8, 4, 0), (16, 2, 0)):
        tb, wb = engine.design_plan(prog, V, S, mask, launch=shape)
        traj = torch.empty(tb, dtype=torch.uint8, device=device)
        work = torch.empty(wb, dtype=torch.uint8, device=device)

        def pair():
            engine.design_forward(prog, tissue, S, mask, with_m0=True, trajectory=traj,
                                  launch=shape)
            engine.design_reverse(prog, tissue, S, mask, seed, traj, work, with_m0=True,
                                  curvature=curvature, launch=shape)

        tuning[shape] = timed(pair)
        del traj, work
    shape = min(tuning, key=tuning.get)
    tb, wb = engine.design_plan(prog, V, S, mask, launch=shape)
    traj = torch.empty(tb, dtype=torch.uint8, device=device)
    work = torch.empty(wb, dtype=torch.uint8, device=device)
    fwd_ms = timed(lambda: engine.design_forward(prog, tissue, S, mask, with_m0=True,
                                                 trajectory=traj, launch=shape))
    engine.design_forward(prog, tissue, S, mask, with_m0=True, trajectory=traj, launch=shape)
    rev_ms = timed(lambda: engine.design_reverse(prog, tissue, S, mask, seed, traj, work,
                                                 with_m0=True, curvature=curvature, launch=shape))
    # One forward-over-reverse pass per column, as the reference pays.
    tb1, wb1 = engine.design_plan(prog, V, S, engine.DESIGN_BITS["T1"], launch=shape)
    traj1 = torch.empty(tb1, dtype=torch.uint8, device=device)
    work1 = torch.empty(wb1, dtype=torch.uint8, device=device)
    seeds1 = [seed[:, k:k + 1].contiguous() for k in range(len(names))]

    def per_column():
        for k, name in enumerate(names):
            bit = engine.DESIGN_BITS[name]
            engine.design_forward(prog, tissue, S, bit, trajectory=traj1, launch=shape)
            engine.design_reverse(prog, tissue, S, bit, seeds1[k], traj1, work1,
                                  curvature=curvature, launch=shape)

    per_col_ms = timed(per_column)
    del traj1, work1
    # The public route: Jacobian, Cramer-Rao cost and backward per design step.
    theta = torch.tensor(flips, device=device, requires_grad=True)
    tau = torch.tensor(trs, device=device, requires_grad=True)
    tis = {"T1": torch.from_numpy(t1).to(device), "T2": torch.from_numpy(t2).to(device),
           "B1": torch.from_numpy(b1).to(device), "M0": torch.from_numpy(m0).to(device)}
    scale = torch.stack([tis[k] for k in ("T1", "T2", "B1", "M0")], dim=-1)

    def design_step_once():
        theta.grad = None
        tau.grad = None
        _, jac = MRFSimulator(flip=theta, TR=tau, states=S).jacobian(
            ("T1", "T2", "B1", "M0"), **tis)
        (crlb(jac) / scale.square()).sum().backward()

    step_ms = timed(design_step_once) if design_step else None
    state_bytes = V * prog.ops * (len(names) + 1) * 3 * S * 4
    rec_bytes = V * ev.outputs * (len(names) + 1) * 4
    seed_bytes = V * (len(names) + 1) * n * 8
    rev_bytes = state_bytes + rec_bytes + seed_bytes
    fwd_bytes = state_bytes + rec_bytes + V * (len(names) + 2) * n * 8
    return {
        "workload": f"Cramer-Rao design gradient: {V} tissues, 600-pulse MRF (flip U(5,70) deg, "
                    "TR U(8,15) ms), nstates 20, Jacobian (T1, T2, B1, M0), cost sum CRLB/theta^2",
        "forward_jacobian_ms": jac_ms,
        "forward_with_trajectory_ms": fwd_ms,
        "reverse_ms": rev_ms,
        "gradient_over_forward_jacobian": (fwd_ms + rev_ms) / jac_ms,
        "per_column_ms": per_col_ms,
        "per_column_form": "one forward-with-trajectory + reverse pass per tangent column (the "
                           "reference's one forward-over-reverse call per column)",
        "fused_speedup_over_per_column": per_col_ms / (fwd_ms + rev_ms),
        "design_step_ms": step_ms,
        "design_step_form": "MRFSimulator.jacobian + torchsim_gb300.crlb + backward (public API)",
        "launch_shape": {"lanes_per_voxel": shape[0], "orders_per_lane": shape[1]},
        "tuning_ms": {f"{k[0]}x{k[1]}": v for k, v in tuning.items()},
        "trajectory_bytes": tb,
        "reverse_hbm": {"algorithmic_bytes": rev_bytes, "achieved_gbs": rev_bytes / rev_ms / 1e6},
        "forward_hbm": {"algorithmic_bytes": fwd_bytes, "achieved_gbs": fwd_bytes / fwd_ms / 1e6},
        "timing": "best of 5 after 3 warm-up runs, CUDA events",
    }


# ---- uneven CPMG batch in one persistent launch ------------------------------


def batched_section(torch, device, sequences: int = 512, repeats: int = 5,
                    shape: tuple[int, int, int] | None = None) -> dict:
    """512 CPMG sequences: ETL U{8..64}, refocusing U(100,180) deg per echo,
    ESP U(5,15) ms, excitation 90 deg at 90 deg phase, refocusing phase 90 deg,
    voxels per sequence round(exp(U(ln 1e3, ln 6.4e4))), T1 U(300,3000),
    T2 U(10,300), B1 U(0.7,1.3), nstates 2*ETL. One autotuned persistent launch
    replayed from a CUDA graph, against one fixed-shape launch per sequence."""
    from torchsim_gb300.batching import BatchEntry, SequenceBatch
    from torchsim_gb300.sequence import fse_events

    rng = np.random.default_rng(2)
    entries = []
    for _ in range(sequences):
        etl = int(rng.integers(8, 65))
        flips = rng.uniform(100, 180, etl).astype(np.float32)
        ev = fse_events(flips, float(rng.uniform(5, 15)), phases_deg=90.0)
        v = int(round(np.exp(rng.uniform(np.log(1e3), np.log(6.4e4)))))
        entries.append(BatchEntry(ev, 2 * etl, rng.uniform(300, 3000, v).astype(np.float32),
                                  rng.uniform(10, 300, v).astype(np.float32),
                                  rng.uniform(0.7, 1.3, v).astype(np.float32)))
    batch = SequenceBatch(entries, device)
    t0 = time.perf_counter()
    if shape is None:
        shape, timings = batch.tune(use_cache=False)
    else:
        batch.shape, timings = tuple(shape), {}
    tune_s = time.perf_counter() - t0
    batch.capture()

    def timed(fn):
        for _ in range(2):
            fn()
        torch.cuda.synchronize()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        for _ in range(repeats):
            fn()
        e.record()
        e.synchronize()
        return s.elapsed_time(e) / repeats

    graph_ms = timed(batch.run)
    plain_ms = timed(batch.run_plain)
    updates = batch.updates()
    return {
        "workload": f"{sequences} uneven CPMG sequences, {int(batch.voxels.sum())} voxels, "
                    "nstates 2*ETL, FP32 forward",
        "updates": updates,
        "persistent_graph_ms": graph_ms,
        "persistent_updates_per_s": updates / (graph_ms * 1e-3),
        "plain_per_sequence_ms": plain_ms,
        "plain_updates_per_s": updates / (plain_ms * 1e-3),
        "speedup_over_plain": plain_ms / graph_ms,
        "launches": {"persistent": 1, "plain": sequences},
        "tuned_shape": {"orders_per_lane": shape[0], "warps_per_block": shape[1],
                        "ctas_per_sm": shape[2]},
        "tuning_candidates": len(timings),
        "tuning_s": tune_s,
    }


# ---- dictionary matching on the tensor cores ----------------------------------


def match_section(torch, device, voxels: int = 65536, repeats: int = 3) -> dict:
    """Match noisy, scaled, phase-turned signals against the full MRF
    dictionary (the 262,144-atom grid x 880 pulses, simulated here by the
    forward kernel): the tensor-core screen with fused best-8 selection and
    the exact FP32 rescoring, against the reference's FP32 route (chunked
    matrix products and top-k, estimators/_dictionary.py:354-375) on a
    bounded sample of the voxels."""
    import json as _json

    from torchsim_gb300 import DictionaryMatcher, _native, engine
    from torchsim_gb300.sequence import mrf_events, program_for

    rng = np.random.default_rng(11)
    T1, T2, B1 = (torch.from_numpy(a) for a in dictionary_grid())
    A = T1.numel()
    prog = program_for(mrf_events(mrf_schedule(), 10.0), device)
    tissue = engine.tissue_maps(device, A, T1, T2, None, B1, None)
    dictionary = engine.forward(prog, tissue, STATES)
    params = torch.stack((T1, T2, B1), 1).to(device)
    del tissue
    matcher = DictionaryMatcher(dictionary=dictionary, parameters=params, query_chunk_size=voxels)
    truth = torch.from_numpy(rng.integers(0, A, voxels)).to(device)
    phase = torch.from_numpy(np.exp(1j * rng.uniform(-np.pi, np.pi, voxels)).astype(np.complex64)).to(device)
    sig = dictionary[truth] * phase[:, None]
    sigma = float(sig.abs().mean()) / 50.0
    noise = torch.randn(sig.shape, dtype=torch.complex64, device=device) * sigma
    measured = (sig + noise).contiguous()

    def timed(fn, n=repeats):
        fn()
        torch.cuda.synchronize()
        best = 1e30
        for _ in range(n):
            s0, e0 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s0.record()
            fn()
            e0.record()
            e0.synchronize()
            best = min(best, s0.elapsed_time(e0))
        return best

    match_ms = timed(lambda: matcher.match(measured))
    # The screen kernel alone, for the roofline.
    s_hat = measured / torch.linalg.vector_norm(measured, dim=-1, keepdim=True)
    queries = matcher._queries(s_hat)
    k = matcher._screen_atoms.shape[1]
    lib = _native.library()
    cands = lib.tsg_match_candidates()
    cand_s = torch.empty((voxels, cands), dtype=torch.float32, device=device)
    cand_i = torch.empty((voxels, cands), dtype=torch.int32, device=device)
    err = torch.zeros(1, dtype=torch.int32, device=device)

    def screen():
        _native.check(lib.tsg_match_screen(queries.data_ptr(), 2 * voxels,
                                           matcher._screen_atoms.data_ptr(), A, k,
                                           cand_s.data_ptr(), cand_i.data_ptr(), err.data_ptr(),
                                           torch.cuda.current_stream().cuda_stream))

    screen_ms = timed(screen)
    # Executed tensor work: every query row against every atom's hi and lo
    # rows (k contraction columns); the product it stands for is half that.
    flops = 2.0 * (2 * voxels) * A * k
    res = matcher.match(measured)
    hits = float((res.indices[:, 0] == truth).float().mean())
    # The reference's FP32 route on a bounded sample: normalized complex
    # products in chunks of 4,096 voxels x 16,384 atoms, top-1 per chunk.
    sample = min(4096, voxels)
    dn = matcher.normalized

    def reference_route():
        q = s_hat[:sample]
        best_s = torch.full((sample,), -1.0, device=device)
        best_i = torch.zeros((sample,), dtype=torch.int64, device=device)
        for start in range(0, A, 16384):
            sc = (q @ dn[start:start + 16384].mH).abs()
            v, i = sc.max(dim=1)
            better = v > best_s
            best_s = torch.where(better, v, best_s)
            best_i = torch.where(better, i + start, best_i)
        return best_i, best_s

    ref_ms = timed(reference_route, 1)
    ref_i, ref_s = reference_route()
    agree = float((ref_i == res.indices[:sample, 0]).float().mean())
    # How far below the FP32 route's best score the chosen atom scores.
    deficit = (ref_s - res.scores[:sample, 0]).clamp_min(0)
    # Against an FP64 exhaustive search of the same sample: the chosen atom's
    # own FP64 score below the FP64 best, and agreement where the FP64 best
    # and second best are further apart than 2e-6.
    profile = dictionary.imag if bool(dictionary.imag.ne(0).any()) else dictionary.real
    s64 = measured[:sample].to(torch.complex128)
    s64 = s64 / torch.linalg.vector_norm(s64, dim=-1, keepdim=True)
    top = torch.full((sample, 2), -1.0, dtype=torch.float64, device=device)
    arg = torch.zeros((sample, 2), dtype=torch.int64, device=device)
    for start in range(0, A, 16384):
        d64 = profile[start:start + 16384].to(torch.float64)
        d64 = d64 / torch.linalg.vector_norm(d64, dim=-1, keepdim=True)
        sc = torch.hypot(s64.real @ d64.T, s64.imag @ d64.T)
        v, i = torch.topk(sc, 2, dim=1)
        top, pick = torch.topk(torch.cat((top, v), 1), 2, dim=1)
        arg = torch.gather(torch.cat((arg, i + start), 1), 1, pick)
    chosen = res.indices[:sample, 0]
    d64 = profile[chosen].to(torch.float64)
    d64 = d64 / torch.linalg.vector_norm(d64, dim=-1, keepdim=True)
    own = torch.hypot((s64.real * d64).sum(-1), (s64.imag * d64).sum(-1))
    deficit64 = (top[:, 0] - own).clamp_min(0)
    separated = (top[:, 0] - top[:, 1]) > 2e-6
    peaks = _json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    peak = float(peaks.get("bf16_tflops", 1900.0))
    return {
        "workload": f"{voxels} noisy MRF signals (SNR 50, random phase) against the {A}-atom "
                    "dictionary x 880 pulses (nstates 20), top-1",
        "match_ms": match_ms,
        "matches_per_s": voxels / (match_ms * 1e-3),
        "voxel_atom_pairs_per_s": voxels * A / (match_ms * 1e-3),
        "screen_ms": screen_ms,
        "screen_tflops": flops / (screen_ms * 1e-3) / 1e12,
        "screen_peak_tflops": peak,
        "screen_peak_source": "MEASURED_PEAKS.json bf16_tflops (cuBLAS bf16 GEMM burst); the "
                              "screen runs fp16 inputs at the same dense rate",
        "screen_frac_of_measured_peak": flops / (screen_ms * 1e-3) / 1e12 / peak,
        "screen_contraction": f"{k} fp16 columns: each atom's hi and lo rows side by side",
        "true_atom_recovered": hits,
        "agreement_with_fp64_argmax": float((chosen == arg[:, 0]).float().mean()),
        "agreement_with_fp64_argmax_where_separated": {
            "value": float((chosen[separated] == arg[separated, 0]).float().mean()),
            "voxels": int(separated.sum()), "gap": 2e-6},
        "score_deficit_vs_fp64": {"max": float(deficit64.max()), "mean": float(deficit64.mean()),
                                  "sample_voxels": sample},
        "agreement_with_fp32_route": agree,
        "score_deficit_vs_fp32_route": {"max": float(deficit.max()), "mean": float(deficit.mean())},
        "reference_route_fp32": {
            "sample_voxels": sample,
            "ms": ref_ms,
            "matches_per_s": sample / (ref_ms * 1e-3),
            "form": "torch complex64 matmul in 4,096 x 16,384 chunks + max (the reference's route)",
        },
        "speedup_over_reference_route": (voxels / (match_ms * 1e-3)) / (sample / (ref_ms * 1e-3)),
    }


# ---- Gauss-Newton mapping server ---------------------------------------------


def gn_section(torch, device, requests: int = 40, rate: float = 20.0,  # noqa: C901
               cpu_sample: int = 4096) -> dict:
    """Poisson arrivals (20 req/s, seeded); each request one slice of
    round(exp(U(ln 4096, ln 262144))) voxels of the 880-pulse MRF signal at
    ground-truth T1/T2/B1 (drawn as the 1,024-voxel workload) and M0 U(0.5,1.5)
    plus complex Gaussian noise at SNR 50 (sigma = mean|s|/50); B1 known;
    unknowns (T1, T2, M0) bounded (50,5000), (2,1000), (0,5); start at the
    median of a training draw; <= 10 LM steps with FP64 3x3 solves; 120 GB
    admission budget. The continuously batched server against the same fused
    solver serving one request at a time, first come first served."""
    from torchsim_gb300 import engine
    from torchsim_gb300.recon import GaussNewton, NonlinearLeastSquares, TrustRegion
    from torchsim_gb300.sequence import mrf_events, program_for
    from torchsim_gb300.serving import GNServer, MapRequest, latency_summary, serve_plain

    rng = np.random.default_rng(4)
    program = program_for(mrf_events(mrf_schedule(), 10.0), device)
    bounds = {"T1": (50.0, 5000.0), "T2": (2.0, 1000.0), "M0": (0.0, 5.0)}
    draw_t1 = np.exp(rng.uniform(np.log(100), np.log(3000), 4096))
    draw_t2 = np.exp(rng.uniform(np.log(10), np.log(300), 4096))
    draw_m0 = rng.uniform(0.5, 1.5, 4096)
    from torchsim_gb300 import MRFSimulator

    est = NonlinearLeastSquares(MRFSimulator(flip=mrf_schedule(), TR=10.0, states=10),
                                bounds=bounds).fit(T1=draw_t1, T2=draw_t2, M0=draw_m0)
    start = est._start
    gaps = rng.exponential(1.0 / rate, requests)
    arrivals = np.cumsum(gaps) - gaps[0]
    made = []
    gen = torch.Generator(device=device).manual_seed(4)
    for i in range(requests):
        V = int(round(np.exp(rng.uniform(np.log(4096), np.log(262144)))))
        t1 = np.exp(rng.uniform(np.log(100), np.log(3000), V)).astype(np.float32)
        t2 = np.minimum(np.exp(rng.uniform(np.log(10), np.log(300), V)), 0.999 * t1).astype(np.float32)
        b1 = rng.uniform(0.8, 1.2, V).astype(np.float32)
        m0 = rng.uniform(0.5, 1.5, V).astype(np.float32)
        tissue = engine.tissue_maps(device, V, t1, t2, m0, b1, None)
        sig = engine.forward(program, tissue, 10)
        sigma = sig.abs().mean() / 50
        sig = sig + sigma * torch.complex(torch.randn(sig.shape, device=device, generator=gen),
                                          torch.randn(sig.shape, device=device, generator=gen))
        made.append((sig, torch.from_numpy(b1).to(device), float(arrivals[i]), (t1, t2, m0)))
    torch.cuda.synchronize()
    loop = GaussNewton(TrustRegion(), max_iterations=10)
    total_voxels = sum(m[0].shape[0] for m in made)

    def requests_list():
        return [MapRequest(s, b, arrival=a, id=i) for i, (s, b, a, _) in enumerate(made)]

    # Warm the kernels and the launch path of all three solvers outside the
    # measured runs: a first call pays one-off library and kernel loading
    # (seconds on a fresh machine) that would otherwise land in one arm's
    # latencies.
    from torchsim_gb300.recon import PlainGaussNewton

    warm = GNServer(program, 10, bounds, start, loop, budget_bytes=2 << 30, device=device)
    warm.serve([MapRequest(made[0][0][:4096], made[0][1][:4096], id=0)], realtime=False)
    loop.minimize_program(program, made[0][0][:4096], start, bounds, 10, b1=made[0][1][:4096])
    PlainGaussNewton(TrustRegion(), max_iterations=10).minimize_program(
        program, made[0][0][:4096], start, bounds, 10, b1=made[0][1][:4096])
    torch.cuda.synchronize()

    server = GNServer(program, 10, bounds, start, loop, budget_bytes=120 * 2**30, device=device)
    t0 = time.perf_counter()
    done = server.serve(requests_list(), realtime=True)
    torch.cuda.synchronize()
    span = time.perf_counter() - t0
    lat = latency_summary(done)
    server_stats = server.stats
    # Accuracy against the ground truth (median relative error over voxels).
    errs = []
    for r in done:
        t1, t2, m0 = made[r.id][3]
        errs.append(np.abs(r.maps["T1"].cpu().numpy() - t1) / t1)
    err = float(np.median(np.concatenate(errs)))

    plain_reqs = requests_list()
    t0 = time.perf_counter()
    plain_done = serve_plain(program, 10, bounds, start, plain_reqs, loop)
    plain_span = time.perf_counter() - t0
    plain_lat = latency_summary(plain_done)

    # Capacity: every request present at once (saturated), the server against
    # the same solver one request at a time and against the plain form laid
    # out as the reference lays it out (forward + one pass per Jacobian
    # column, Jacobian in HBM), on the first `sat` requests.
    del server, warm
    torch.cuda.empty_cache()
    sat = min(requests, 12)
    sat_vox = sum(m[0].shape[0] for m in made[:sat])
    burst = [MapRequest(s, b, arrival=0.0, id=i) for i, (s, b, a, _) in enumerate(made[:sat])]
    srv = GNServer(program, 10, bounds, start, loop, budget_bytes=120 * 2**30, device=device)
    t0 = time.perf_counter()
    sat_server_lat = latency_summary(srv.serve(burst, realtime=False))
    torch.cuda.synchronize()
    sat_server = time.perf_counter() - t0
    sat_iterations = srv.stats.iterations
    t0 = time.perf_counter()
    sat_fifo_lat = latency_summary(serve_plain(
        program, 10, bounds, start,
        [MapRequest(s, b, arrival=0.0, id=i) for i, (s, b, a, _) in enumerate(made[:sat])],
        loop))
    sat_fifo = time.perf_counter() - t0
    t0 = time.perf_counter()
    sat_plain_lat = latency_summary(serve_plain(
        program, 10, bounds, start,
        [MapRequest(s, b, arrival=0.0, id=i) for i, (s, b, a, _) in enumerate(made[:sat])],
        PlainGaussNewton(TrustRegion(), max_iterations=10)))
    sat_plain = time.perf_counter() - t0
    # The CPU baseline of the mapping workload: the reference's loop (LM,
    # TrustRegion, one forward and one tangent pass per EPG-dependent unknown
    # per step) restated over the oracle's FP32 port of its kernels, on all
    # host cores, on the first request's first `cpu_sample` voxels.
    cpu = None
    if cpu_sample > 0:
        from oracle import gn_port

        n = min(cpu_sample, made[0][0].shape[0])
        y = made[0][0][:n].cpu().numpy()
        b1_host = made[0][1][:n].cpu().numpy()
        events = mrf_events(mrf_schedule(), 10.0)
        low = np.array([bounds[k][0] for k in ("T1", "T2", "M0")])
        high = np.array([bounds[k][1] for k in ("T1", "T2", "M0")])
        threads = os.cpu_count() or 1
        t0 = time.perf_counter()
        got = gn_port.fit(events, y, np.asarray(start, np.float64), low, high, 10, b1=b1_host,
                          max_iterations=10, threads=threads)
        cpu_s = time.perf_counter() - t0
        cpu = {"maps_per_s": n / cpu_s, "seconds": cpu_s, "cores": threads, "kind": "port",
               "cpu": cpu_model(),
               "sample": f"the first request's first {n} voxels, <=10 LM steps "
                         f"({got.passes} EPG passes over the voxels still moving)",
               "form": "the reference's Levenberg-Marquardt/TrustRegion loop over the oracle's "
                       "FP32 port of its kernels: per step one forward and one tangent pass "
                       "per EPG-dependent unknown (T1, T2), FP64 3x3 solves"}
    return {
        "workload": f"{requests} requests, Poisson {rate}/s, {total_voxels} voxels, 880-pulse "
                    "MRF, nstates 10, SNR 50, <=10 LM steps, 120 GB budget",
        "cpu_baseline": cpu,
        "server": {"maps_per_s": total_voxels / span, "makespan_s": span, **lat,
                   "iterations": server_stats.iterations,
                   "launches_per_iteration": 3,
                   "host_reads_per_iteration": 1,
                   "peak_live_voxels": server_stats.peak_live_voxels,
                   "voxel_iterations": server_stats.voxel_iterations},
        "plain_one_request_at_a_time": {"maps_per_s": total_voxels / plain_span,
                                        "makespan_s": plain_span, **plain_lat},
        "saturated": {"requests": sat, "voxels": sat_vox,
                      "note": "every request arrives at time 0; latency = completion time",
                      "server": {"maps_per_s": sat_vox / sat_server, **sat_server_lat,
                                 "iterations": sat_iterations},
                      "fused_one_at_a_time": {"maps_per_s": sat_vox / sat_fifo, **sat_fifo_lat},
                      "reference_layout_plain": {"maps_per_s": sat_vox / sat_plain,
                                                 **sat_plain_lat}},
        "t1_median_relative_error": err,
    }


# ---- CPU baselines ----------------------------------------------------------


def cpu_model() -> str:
    """The host CPU's model name (lscpu's, else /proc/cpuinfo's, else the
    platform's machine type)."""
    import platform
    import subprocess

    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip() + f" ({platform.machine()})"
    except (OSError, subprocess.SubprocessError):
        pass
    return platform.machine()


def cpu_run(sample: int, threads: int):
    """Forward + one tangent pass per Jacobian column (the reference's call
    pattern, `torch.func.jvp` per property) over the first `sample` atoms of the
    grid. Runs the reference's own compiled CPU kernel where a build for this
    machine exists, else the oracle's FP32 port, whose forward is the
    reference's per-atom kernel and whose tangents are its eight-atom lane
    kernel (the layout the reference picks for these runs), bitwise the
    reference's results. Returns (seconds, kind)."""
    from oracle import oracle as O
    from torchsim_gb300.sequence import mrf_events

    t1, t2, b1 = (a[:sample].copy() for a in dictionary_grid())
    ev = mrf_events(mrf_schedule(), 10.0)
    p = O.Packed(t1, t2, ev.duration, ev.kind, ev.flip, ev.action, ev.output_index, STATES, b1=b1)
    ref = O.reference_module()
    t0 = time.perf_counter()
    if ref is not None:
        O.reference_forward(ref, p, threads)
        for column in (0, 1, 3):  # T1, T2, B1 tissue slots
            O.reference_jvp(ref, p, column, threads)
        return time.perf_counter() - t0, "reference"
    O.forward(p, "f32", threads=threads)
    for key in ("t1_ms", "t2_ms", "b1"):
        O.tangent(p, "f32", threads=threads, **{key: 1.0})
    return time.perf_counter() - t0, "port"


PORT_NOTE = ("the oracle's FP32 port: the reference's compiled kernel is built only where its "
             "sources are, and no build for this host's architecture exists here; the port "
             "runs the reference's own kernel layouts (per-atom forward, eight-atom lane "
             "tangents) and reproduces its results bit for bit")


def cpu_baseline(sample: int) -> dict:
    from oracle import oracle as O

    threads = O.cpu_threads()
    seconds, kind = cpu_run(sample, threads)
    line = {"value": float(sample) * PULSES * STATES / seconds, "unit": "updates/s",
            "cores": threads, "kind": kind, "cpu": cpu_model(),
            "sample": f"first {sample} of the {ATOMS} grid atoms, forward + 3 tangent passes "
                      f"(the reference's per-column call pattern), {seconds:.2f} s"}
    # One thread as well, on an eighth of the sample.
    one = max(8, sample // 8)
    seconds1, _ = cpu_run(one, 1)
    line["single_thread"] = {"value": float(one) * PULSES * STATES / seconds1,
                             "sample_atoms": one, "seconds": seconds1}
    if kind == "port":
        line["why_port"] = PORT_NOTE
    return line


def run_reference(args, rank: int) -> dict | None:
    if rank != 0:
        return None
    from oracle import oracle as O

    threads = O.cpu_threads()
    cpu_run(min(args.cpu_sample, 1024), threads)  # warm the pages and caches
    for _ in range(max(0, args.warmup - 1)):
        cpu_run(min(args.cpu_sample, 2048), threads)
    times = []
    kind = "port"
    for _ in range(args.steps):
        seconds, kind = cpu_run(args.cpu_sample, threads)
        times.append(seconds)
    total = sum(times)
    value = float(args.cpu_sample) * PULSES * STATES * args.steps / total
    return {
        "impl": "reference",
        "metric": "EPG voxel·pulse·state updates/s (fused forward + Jacobian T1/T2/B1)",
        "value": value,
        "unit": "updates/s",
        "n_gpus": 1,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": total / args.steps * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded grid of the named shape)",
        "config": config({"sample_atoms_per_step": args.cpu_sample}),
        "cpu_baseline": {"value": value, "unit": "updates/s", "cores": threads, "kind": kind,
                         "cpu": cpu_model(),
                         "sample": f"{args.cpu_sample} of {ATOMS} atoms per step, forward + "
                                   "3 tangent passes",
                         **({"why_port": PORT_NOTE} if kind == "port" else {})},
        "e2e": {"value": value, "unit": "updates/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }


def main() -> None:
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=60)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--cpu-sample", type=int, default=16384)
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-plain", action="store_true")
    ap.add_argument("--skip-e2e", action="store_true")
    ap.add_argument("--skip-adjoint", action="store_true")
    ap.add_argument("--skip-second", action="store_true")
    ap.add_argument("--second-voxels", type=int, default=16384)
    ap.add_argument("--skip-design-step", action="store_true",
                    help="leave out the public-API design step (torch's inverse is not "
                         "loadable under the profiler)")
    ap.add_argument("--skip-batched", action="store_true")
    ap.add_argument("--skip-gn", action="store_true")
    ap.add_argument("--skip-match", action="store_true")
    ap.add_argument("--match-voxels", type=int, default=65536)
    ap.add_argument("--gn-requests", type=int, default=40)
    ap.add_argument("--batch-sequences", type=int, default=512)
    ap.add_argument("--batch-shape", type=int, nargs=3, default=None,
                    metavar=("ORDERS", "WARPS", "CTAS_PER_SM"),
                    help="persistent launch shape of the batched section (default: autotuned)")
    ap.add_argument("--atoms", type=int, default=ATOMS,
                    help="first N grid atoms (a smaller case for profiling; default all)")
    ap.add_argument("--launch", type=int, nargs="+", metavar="N",
                    help="lanes per voxel, orders per lane, warps per block[, min blocks per SM]")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.impl == "reference":
        line = run_reference(args, rank)
        if line is not None:
            print(json.dumps(line), flush=True)
        return
    dist = None
    if world > 1:
        import torch
        import torch.distributed as tdist

        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        tdist.init_process_group("nccl")
        dist = tdist
    line = run_gpu(args, rank, world, dist)
    if line is not None:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
