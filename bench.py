"""Benchmark: BC1/BC3 + mips Mtexels/s on one GB300, learned endpoint proposal vs plain cluster fit.

Default workload (c4, the configuration the learned proposal's target is quoted on): 1024 textures,
power-of-two sizes 128..4096 per axis (80% square), 50% BC1 / 30% BC3 (alpha field, transparency) /
20% BC5 fBm normal maps, linear colour, Normal quality, full Kaiser (width 3, alpha 4, stretch 1) mip
chains, 4.68e9 texels per step, all in one batch replayed as one CUDA graph (ntg_batch), launch
shapes autotuned. A step is one replay: filter every level of every texture and encode every block.
Mtexels/s = encoded texels of all levels / step time.

  value    : the plain batched cluster fit (bit-identical to the reference), device time per step
             (CUDA events on the launching stream), inputs resident in HBM; the inputs (14 GB) are far
             larger than L2, and L2 is also flushed (256 MiB write) between steps.
  learned  : the same batch with the learned endpoint proposals: per block network -> pruned search ->
             full fit of the flagged blocks; its Mtexels/s, the ratio to plain, and per texture the
             RMSE (nvtt::rmsError on the decoded levels) against the plain fit's, at each operating
             point measured.
  e2e      : the plain batch over host buffers through ntg_batch_process_host: every step copies every
             texture in from pinned host memory and every texture's blocks out, two bindings taking
             turns so that the copies run beside the neighbouring steps' graphs.
  roofline : the dominant kernel (the BC1 cluster fit) against the FP32 rate of the clocks seen, its
             orderings counted on the device; the mip phase against measured HBM bandwidth.
  cpu_baseline : the oracle port (C restatement of the reference path) on the host cores, a bounded
             sample of the workload's textures.
  c1       : secondary key, the single 4096x4096 sRGB / Kaiser / BC3 chain (workload c1).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference] [--workload c4|c1|c0|c2|c3]
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

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "nvidia-texture-tools_gb300"))

import numpy as np  # noqa: E402

METRIC = "BC1/BC3+mips Mtexels/s, learned-proposal vs plain cluster fit at equal RMSE"
UNIT = "Mtexels/s"
FLUSH_BYTES = 256 << 20

WORKLOADS = {
    # name: (w, h, format, quality, filter, alpha_mode, in_xform, out_xform, description)
    "c1": (4096, 4096, 4, 1, 2, 1, 2, 2,
           "4096x4096 RGBA8 sRGB, Kaiser(w3,a4,s1) mips, transparency, BC3 Normal, 13 levels"),
    "c0": (512, 512, 1, 1, 0, 0, 0, 0, "512x512 RGBA8 linear, box mips, BC1 Normal, 10 levels"),
    # reduced-size variant of c1 for profiler captures (same kernels, a quarter of the texels)
    "c1_2k": (2048, 2048, 4, 1, 2, 1, 2, 2,
              "2048x2048 RGBA8 sRGB, Kaiser(w3,a4,s1) mips, transparency, BC3 Normal, 12 levels"),
}
# Batched workloads: (count, seed, kmin, kmax, filter, description). Sizes 2^k per axis with k in
# [kmin, kmax], 80% square; formats 50% BC1 / 30% BC3 (transparency) / 20% BC5 fBm normal maps;
# linear colour; Normal quality; whole chains; one graph per step (ntg_batch).
BATCHES = {
    "c2": (256, 0xC2, 6, 11, 1, "256 textures 64..2048 px (80% square), 50/30/20 BC1/BC3/BC5, Triangle mips, "
                                "one CUDA graph (ntg_batch), autotuned launch shapes"),
    "c2_small": (64, 0xC2, 6, 9, 1, "64 textures 64..512 px, 50/30/20 BC1/BC3/BC5, Triangle mips, one CUDA graph"),
    "c4": (1024, 0xC4, 7, 12, 2, "1024 textures 128..4096 px (80% square), 50/30/20 BC1/BC3/BC5, Kaiser mips, one CUDA "
                                 "graph (ntg_batch), autotuned; BC1 through the learned endpoint proposal"),
}
LEARNED_BATCHES = {"c4"}
# The learned proposals: per format, the generators (ntg.learned.generator_texture kinds) its network
# is trained on, and the operating points {format: (search, margin)} measured on the batch (search: a
# window radius, or DESCENT | moves); the line's headline is the point that keeps the most proposed
# textures within 0.5% RMSE of the plain fit, the fastest among equals.
DESCENT = 256
FORMAT_NAMES = {1: "BC1", 4: "BC3"}
PROPOSAL_TRAINING = {1: (0, 1, 2), 4: (3, 4)}
INF = float("inf")
BATCH_FRONTIER = [{1: (DESCENT | 4, INF)}, {1: (DESCENT | 8, 0.05)}, {1: (DESCENT | 4, INF), 4: (2, INF)},
                  {1: (2, INF)}]
# DRAM bytes per block of the BC1 fit: one ncu capture of k_bc1<7> over 262,144 blocks of a 2048x2048
# planar FP32 level (67,384,064 B read + 712,192 B written, profiles/k_bc1_7_cases_2048.md), per block;
# the batch's BC1 levels are planar FP32 too, so the traffic scales with the blocks
# DRAM bytes (read + write) of the 4096 x 4096 chain's mip launches (k_tile2x_u8, 6 k_tile2x, k_mip_tail)
# in one ncu capture of `bench.py --workload c1` (dram__bytes_read.sum + dram__bytes_write.sum).
C1_MIP_TRAFFIC = 191867392
BC1_TRAFFIC_PER_BLOCK = (67384064 + 712192) / 262144

# FP32 operations of one ordering of icbc's cluster fits (src/nvtt/icbc.h:2501-2540 and 2200-2240 in
# the scalar build), each multiply/add/min/max/round/reciprocal counted once: cluster_fit_four w3 1,
# cluster differences 8, alpha2 4, beta2 4, alphabeta 2, alphax 12 = 31, cluster_fit_three 14, then
# the shared solve/snap/residual: factor 4, betax 3, a 12, b 12, saturate + 5:6:5 rounding 36, e2 18,
# e1 18, metric 5, compare 1 = 109.
OPS_PER_ORDERING4 = 140
OPS_PER_ORDERING3 = 123

# FP32 operations of one cluster-split evaluation of squish's WeightedClusterFit::Compress4
# (src/nvtt/squish/weightedclusterfit.cpp:505-545) as the kernel's inner loop runs it, each
# multiply/add/min/max/floor/reciprocal counted once (no FMA contraction): w3 1, alpha2 2, beta2 3,
# alphabeta 2, factor 4, alphax 6, betax 3, a and b 24 each (two products, difference, saturating
# scale, 5:6:5 snap), residual 18, e1 21, error 2, compare 1, running sums 4 = 115.
OPS_PER_SPLIT = 115
# Instructions the inner loop issues per split (the FP32 operations plus integer, shared-memory and
# control instructions), for the issue-slot fraction reported beside the FP32 fraction.
ISSUE_PER_SPLIT = 141


def splits(count: int) -> int:
    return (count + 1) * (count + 2) * (count + 3) // 6


T_START = time.perf_counter()


def log(*a):
    print(f"[{time.perf_counter() - T_START:7.1f} s]", *a, file=sys.stderr, flush=True)


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 200 ms while the timed region runs."""

    def __init__(self, index: int):
        self.index, self.proc, self.lines = index, None, []

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except FileNotFoundError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "of measured"
    except (OSError, ValueError):
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "of fallback"


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        backend = "nccl" if args.impl != "reference" else "gloo"
        if backend == "nccl":
            import torch
            torch.cuda.set_device(local)  # one GPU per rank, before the communicator exists
        dist.init_process_group(backend=backend)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        if dist.get_backend() == "nccl":
            import torch
            dist.barrier(device_ids=[torch.cuda.current_device()])
        else:
            dist.barrier()


def max_over_ranks(world, value, device=None):
    if world <= 1:
        return value
    import torch
    import torch.distributed as dist
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def workload_texture(name):
    import ntg.synth as synth
    w, h = WORKLOADS[name][:2]
    if name.startswith("c1"):
        return synth.texture_c1(w=w, h=h)
    return synth.texture_c0(w=w, h=h)


def chain_texels(w, h):
    import ntg
    return sum(lw * lh for lw, lh in ntg.chain_levels(w, h))


# ---------------------------------------------------------------------------------------------
# CPU legs (oracle port): the reference's algorithm on the host cores

def cpu_chain(oracle, bgra, spec, threads):
    """Mips single-threaded (as the reference filters), encode on `threads` host threads."""
    w, h, fmt, quality, filt, am, ix, ox = spec[:8]
    width = {0: 0.5, 1: 1.0, 2: 3.0}[filt]
    t0 = time.perf_counter()
    _, enc = oracle.mip_chain(bgra, w, h, filt, width, 4.0, 1.0, 2, am, ix, ox, 2.2)
    t1 = time.perf_counter()
    for lv in enc:
        lw, lh = lv.shape[2], lv.shape[1]
        flat = lv.reshape(-1)
        if fmt == 1:
            oracle.bc1_image(flat, lw, lh, am, quality, threads=threads)
        elif fmt == 4:
            oracle.bc3_image(flat, lw, lh, am, quality, threads=threads)
        else:
            oracle.bc5_image(flat, lw, lh, quality, threads=threads)
    t2 = time.perf_counter()
    return t2 - t0, t1 - t0, t2 - t1


def cpu_sample(name, bgra, threads):
    """The bounded CPU sample: the full chain of the workload's texture (C1: ~10-30 s of CPU work)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    oracle = pyoracle.Oracle()
    spec = WORKLOADS[name]
    total, mips, enc = cpu_chain(oracle, bgra, spec, threads)
    texels = chain_texels(spec[0], spec[1])
    return {"value": texels / total / 1e6, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"the full {name} chain ({texels} texels): mips on 1 thread {mips:.2f} s, "
                      f"encode on {threads} threads {enc:.2f} s"}


def run_reference(args):
    """The reference arm: the reference's algorithm on the host cores, one bounded sample per step."""
    world, rank, _ = dist_setup(args)
    if rank != 0:
        return 0
    name = args.workload
    spec = list(WORKLOADS[name])
    bgra = workload_texture(name)
    # bounded sample: the top-left quadrant (up to 2048x2048) with its own full chain
    sw, sh = min(spec[0], 2048), min(spec[1], 2048)
    sample = np.ascontiguousarray(bgra[:sh, :sw])
    spec[0], spec[1] = sw, sh
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    pyoracle.build_oracle()
    oracle = pyoracle.Oracle()
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_chain(oracle, sample, spec, threads)
    times = [cpu_chain(oracle, sample, spec, threads)[0] for _ in range(args.steps)]
    texels = chain_texels(sw, sh)
    value = texels * len(times) / sum(times) / 1e6
    desc = WORKLOADS[name][8]
    why = ("the reference library itself cannot be built on this host (its source tree is absent), so its C "
           "restatement in oracle/ runs: mips on one thread as the reference filters, encode on every core")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * sum(times) / len(times),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": {"workload": desc, "texels_per_step": texels,
                                            "sample": f"top-left {sw}x{sh} quadrant with its full chain"},
            "cpu_baseline": dict({"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                                  "sample": f"{sw}x{sh} quadrant of the {name} texture per step; {why}"}, **host_cpu()),
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------------------------
# GPU leg

def split_counts(ctx, levels_flat, spec, steps_table):
    """Distinct RGB colours per block of every level after the BC3 quantiser (the squish split
    count), for the algorithmic FLOP count of the encoder. Level 0 uses the 8-bit tables."""
    import torch
    import ntg
    w, h = spec[0], spec[1]
    total_splits, off = 0, 0
    steps = torch.from_numpy(steps_table[1:].copy()).cuda()
    for lw, lh in ntg.chain_levels(w, h):
        n = lw * lh
        lv = levels_flat[off: off + 4 * n].view(4, lh, lw)
        off += 4 * n
        rgb = lv[:3]
        q = torch.searchsorted(steps, rgb.contiguous(), right=True).to(torch.int64)  # counts steps <= x
        q = torch.where(torch.isnan(rgb), torch.zeros_like(q), q)
        code = (q[0] << 16) | (q[1] << 8) | q[2]
        bh, bw = (lh + 3) // 4, (lw + 3) // 4
        # ColorBlock edge repetition for partial blocks: i % size within the block
        by = torch.arange(bh * 4, device=code.device)
        bx = torch.arange(bw * 4, device=code.device)
        yy = (by // 4) * 4 + (by % 4) % torch.clamp(lh - (by // 4) * 4, max=4)
        xx = (bx // 4) * 4 + (bx % 4) % torch.clamp(lw - (bx // 4) * 4, max=4)
        blk = code[yy][:, xx].view(bh, 4, bw, 4).permute(0, 2, 1, 3).reshape(-1, 16)
        s, _ = torch.sort(blk, dim=1)
        distinct = 1 + (s[:, 1:] != s[:, :-1]).sum(dim=1)
        cnt = distinct.to(torch.int64)
        sp = (cnt + 1) * (cnt + 2) * (cnt + 3) // 6
        sp = torch.where(cnt == 1, torch.zeros_like(sp), sp)  # single colour: table lookup, no fit
        total_splits += int(sp.sum().item())
    return total_splits


def host_cpu():
    """The host's CPU model, online cores and this process's affinity (recorded with CPU figures)."""
    model = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.split(":")[0].strip() in ("Model name", "Model"):
                model = line.split(":", 1)[1].strip()
                if not model.isdigit():
                    break
    except (OSError, subprocess.SubprocessError):
        pass
    if not model:
        import platform
        model = platform.processor() or platform.machine()
    try:
        aff = sorted(os.sched_getaffinity(0))
    except AttributeError:
        aff = list(range(os.cpu_count() or 1))
    ranges, start = [], None
    for i, c in enumerate(aff):
        if start is None:
            start = c
        if i + 1 == len(aff) or aff[i + 1] != c + 1:
            ranges.append(f"{start}-{c}" if c != start else f"{c}")
            start = None
    return {"cpu_model": model, "nproc": os.cpu_count(), "affinity": ",".join(ranges)}


def run_gpu(args):
    import torch
    import ntg
    world, rank, local = dist_setup(args)
    torch.cuda.set_device(local)
    ctx = ntg.Context(local)
    line = measure_chain(ctx, args.workload, args, world, rank, with_cpu=not args.no_cpu and world == 1)
    if rank == 0:
        print(json.dumps(line), flush=True)
    ctx.close()
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


def measure_chain(ctx, name, args, world, rank, with_cpu):
    """The single-chain workload `name` (c1, c0): device steps, phase split, e2e through the host-buffer
    C ABI, rooflines and (with_cpu) the CPU sample; returns the JSON line (rank 0; None elsewhere)."""
    import torch
    import ntg
    spec = WORKLOADS[name]
    w, h, fmt, quality, filt, am, ix, ox, desc = spec
    opt = ntg.ChainOptions.make(format=fmt, quality=quality, filter=filt, alpha_mode=am, in_xform=ix,
                                out_xform=ox, gamma=2.2)
    bgra = workload_texture(name)
    texels = chain_texels(w, h)
    d_bgra = torch.from_numpy(bgra).cuda()
    d_out = torch.empty(ntg.chain_bytes(w, h, opt), dtype=torch.uint8, device="cuda")
    flush = torch.empty(FLUSH_BYTES, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()
    for _ in range(args.warmup):
        n0 = ntg.launch_count()
        ctx.compress_chain(d_bgra, w, h, opt, out=d_out)
        launches_per_step = ntg.launch_count() - n0  # the library's own count of its kernel launches
    torch.cuda.synchronize()

    # device-resident timing: CUDA events around each step, L2 flushed in between
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    barrier(world)
    torch.cuda.synchronize()
    with ClockSampler(torch.cuda.current_device()) as clk:
        t_wall = time.perf_counter()
        for i in range(args.steps):
            flush.zero_()
            starts[i].record(stream)
            ctx.compress_chain(d_bgra, w, h, opt, out=d_out)
            ends[i].record(stream)
        torch.cuda.synchronize()
        barrier(world)
        wall = time.perf_counter() - t_wall
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    # phase split for the rooflines: phase events of the same chain, in 3 runs outside the timed region
    ctx.profile(True)
    phase = []
    for _ in range(3):
        flush.zero_()
        ctx.compress_chain(d_bgra, w, h, opt, out=d_out)
        phase.append(ctx.profile_read())
    ctx.profile(False)
    mips_ms = sum(p[0] for p in phase) / len(phase)
    enc_ms = sum(p[1] for p in phase) / len(phase)
    dev_ms = max_over_ranks(world, sum(step_ms), torch.device("cuda"))
    value = world * texels * args.steps / (dev_ms / 1000.0) / 1e6

    # end to end through the host-buffer C-ABI (ntg_compress_chains_host): every step copies its image
    # in from pinned host memory and its blocks out to pinned host memory, overlapped with the chains
    # of the neighbouring steps (two device slots)
    h_in = torch.from_numpy(bgra.reshape(-1)).pin_memory()
    h_outs = [torch.empty(d_out.numel(), dtype=torch.uint8).pin_memory() for _ in range(2)]
    in_np, outs_np = h_in.numpy(), [o.numpy() for o in h_outs]
    ctx.compress_chains_host([in_np] * 2, w, h, opt, outs=outs_np)
    barrier(world)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ctx.compress_chains_host([in_np] * args.steps, w, h, opt, outs=[outs_np[i & 1] for i in range(args.steps)])
    e2e_s = max_over_ranks(world, time.perf_counter() - t0, torch.device("cuda"))
    e2e_value = world * texels * args.steps / e2e_s / 1e6
    same = bool(np.array_equal(outs_np[(args.steps - 1) & 1], d_out.cpu().numpy()))

    line = None
    if rank == 0:
        # the filtered levels, for the encoder's operation count (outside any timing)
        levels_flat = ctx.mip_chain(d_bgra, w, h, opt)
        torch.cuda.synchronize()
        chain_ms = dev_ms / args.steps
        steps_table = ntg.host_transform_tables(ix, ox, 2.2)[3] if ox == 2 else None
        peaks, peak_src = measured_peaks()
        clocks = clk.summary()
        roof = None
        if fmt == 4 and steps_table is not None:
            nsplits = split_counts(ctx, levels_flat, spec, steps_table)
            ops = nsplits * OPS_PER_SPLIT
            sm_mhz = clocks["sm_mhz"] or 2070.0
            peak_tops = 152 * 128 * sm_mhz * 1e6 / 1e12  # one FP32 op per lane per clock (no FMA pairing)
            achieved = ops / (enc_ms / 1000.0) / 1e12
            # DRAM bytes of one encoder launch: one ncu capture of this kernel on the 2048x2048 variant
            # (22,553,856 B for 349,525 blocks), scaled by the blocks this launch encodes
            blocks = ntg.chain_bytes(w, h, opt) // 16
            traffic = 22553856.0 * blocks / 349525.0
            # thread instructions / 32 = warp instructions, against one issue per scheduler per clock
            issue = nsplits * ISSUE_PER_SPLIT / 32 / (enc_ms / 1000.0) / (152 * 4 * sm_mhz * 1e6)
            roof = {"bound": "fp32", "achieved": achieved, "peak": peak_tops, "unit": "TFLOP/s",
                    "frac": achieved / peak_tops, "traffic": traffic, "issue_slot_frac": issue,
                    "kernel": "k_bc3 (squish weighted cluster fit + DXT5A)",
                    "note": f"peak = 152 SMs x 128 FP32 lanes x median SM clock {sm_mhz:.0f} MHz (derived from the "
                            f"clocks seen; the file of measured peaks has no FP32 figure); {nsplits} splits x "
                            f"{OPS_PER_SPLIT} FP32 ops; issue_slot_frac: {ISSUE_PER_SPLIT} instructions per split (per "
                            f"thread; / 32 per warp) over 152 SMs x 4 schedulers x the clock; encoder phase {enc_ms:.3f} ms (one launch over all "
                            f"levels, CUDA events on the launching stream, mean of 3 runs); traffic: DRAM bytes of one "
                            f"ncu capture of the same kernel on the 2048x2048 variant, scaled by blocks"}
        # mip filter against HBM: algorithmic bytes = read level l-1 + write level l (FP32 planar),
        # level 0 read as BGRA8, plus the BGRA8 quantised copy each level writes for the encoder
        mip_bytes = 0
        lv = ntg.chain_levels(w, h)
        for i in range(1, len(lv)):
            src = lv[i - 1][0] * lv[i - 1][1] * (4 if i == 1 else 16)
            dst = lv[i][0] * lv[i][1] * (16 + (4 if fmt != 1 else 0))
            mip_bytes += src + dst
        hbm = peaks.get("hbm_gbs", 6800.0)
        mip_gbs = mip_bytes / (mips_ms / 1000.0) / 1e9
        # the filter's FP32 work: a 2:1 polyphase output costs 2 rows x taps x 8 (multiply and add per
        # channel, no FMA contraction) for the X pass plus taps x 8 for the Y pass
        width = {0: 0.5, 1: 1.0, 2: 3.0}[filt]
        taps = int(np.ceil(width * 2 * 2)) + 1
        outputs = sum(a * b for a, b in lv[1:])
        mip_ops = outputs * (3 * taps * 8) if not (filt == 0 and am == 0) else outputs * 4 * 4
        sm_mhz_m = clocks["sm_mhz"] or 2070.0
        fp32_peak = 152 * 128 * sm_mhz_m * 1e6
        roof_hbm = {"bound": "hbm", "achieved": mip_gbs, "peak": hbm, "unit": "GB/s", "frac": mip_gbs / hbm,
                    "traffic": C1_MIP_TRAFFIC if name == "c1" else None,
                    "kernel": "mip launches of the chain (k_tile2x_u8 / k_tile2x for the 2:1 steps, k_mip_tail for the "
                              "levels from 32x32 down)",
                    "algorithmic_bytes": mip_bytes, "ms": mips_ms, "peak_source": peak_src,
                    "fp32_ops": mip_ops, "fp32_frac": mip_ops / (mips_ms / 1000.0) / fp32_peak,
                    "note": "the Kaiser filter is FP32-bound before it is HBM-bound: 312 FP32 instructions per output "
                            "without FMA contraction; traffic: DRAM read + write of the chain's 8 mip launches in one ncu "
                            "capture (below the algorithmic bytes: each level is read back from L2 by the next step)"}
        cpu = None
        if with_cpu:
            try:
                cpu = cpu_sample(name, bgra, os.cpu_count() or 1)
            except Exception as e:  # reported, not fatal
                cpu = {"value": None, "unit": UNIT, "cores": os.cpu_count(), "kind": "port", "sample": f"failed: {e}"}
            cpu.update(host_cpu())
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": dev_ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "base_level": {"value": w * h * args.steps / (dev_ms / 1000.0) / 1e6, "unit": UNIT,
                               "texels_per_step": w * h, "note": "level-0 texels only, same device time"},
                "config": {"workload": desc, "texels_per_step": texels, "blocks_per_step": ntg.chain_bytes(w, h, opt) // 16
                           if fmt != 1 else ntg.chain_bytes(w, h, opt) // 8, "l2": "flushed (256 MiB write) between steps",
                           "method": "plain (non-learned) cluster fit", "replicas": world},
                "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(bgra.nbytes),
                        "d2h_bytes_per_step": int(d_out.numel()), "matches_device_path": same,
                        "api": "ntg_compress_chains_host: host buffers, copies overlapped with the neighbouring "
                               "steps' chains"},
                "gpu_launches": launches_per_step * args.steps,
                "clocks": clocks, "roofline": roof, "roofline_mips": roof_hbm,
                "split_ms": {"mips": mips_ms, "encode": enc_ms, "chain": chain_ms,
                             "note": "mips and encode from phase events of 3 runs outside the timed region"},
                "wall_s_timed": wall, "cpu_baseline": cpu}
    return line


# ---------------------------------------------------------------------------------------------
# Batched workloads

def batch_textures(name):
    """(w, h, format, options tuple, image) per texture of a batched workload: one seeded image per
    distinct (size, format), shared by the textures that have both (generated on every core)."""
    import ntg.synth as synth
    count, seed, kmin, kmax, filt, _ = BATCHES[name]
    out = []
    for (w, h, fmt, img) in synth.batch_workload(count, seed, kmin, kmax):
        am = 1 if fmt == 4 else 0
        out.append((w, h, fmt, (fmt, 1, filt, am, 0, 0), img))
    return out


def batch_options(o):
    import ntg
    fmt, quality, filt, am, ix, ox = o
    return ntg.ChainOptions.make(format=fmt, quality=quality, filter=filt, wrap=ntg.WRAP_MIRROR, alpha_mode=am,
                                 in_xform=ix, out_xform=ox)


def timed_launches(batch, steps, warmup, flush, stream):
    """Per-step device times (ms) of `steps` graph replays after `warmup`, L2 flushed before each."""
    import torch
    for _ in range(warmup):
        batch.launch()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    for a, b in ev:
        flush.zero_()
        a.record(stream)
        batch.launch()
        b.record(stream)
    torch.cuda.synchronize()
    return [a.elapsed_time(b) for a, b in ev]


def texture_rmse(ctx, specs, textures, outs_list):
    """Per texture: the colour RMSE (nvtt::rmsError over all levels) of each encoding in outs_list
    (a list over encodings of per-texture device blocks), as an [encodings x textures] array."""
    from ntg import learned
    r = np.zeros((len(outs_list), len(specs)))
    for i, ((w, h, fmt, o, img), tex) in enumerate(zip(specs, textures)):
        sse, n = learned.chain_sse(ctx, tex[0], w, h, tex[3], [outs[i] for outs in outs_list])
        r[:, i] = np.sqrt(np.asarray(sse) / n)
    return r


def learned_batch(ctx, batch, specs, textures, plain_out, plain_ms, args, flush, stream, world):
    """The batch with the learned endpoint proposals against the plain fit: one network per format
    trained on the GPU, timed replays at each operating point of BATCH_FRONTIER, per-texture RMSE of
    every proposed texture against the plain fit's."""
    import torch
    import ntg
    from ntg import learned
    cfg = LEARNED
    nets, training = {}, {}
    for fmt, kinds in PROPOSAL_TRAINING.items():
        t0 = time.perf_counter()
        x, t = learned.training_set(ctx, cfg["train_blocks"], seed=0x5EED + fmt, size=cfg["train_size"], kinds=kinds)
        data_s = time.perf_counter() - t0
        net = ntg.MLP(seed=0x4E4554 + fmt)
        steps = cfg["train_blocks"] // cfg["batch"]
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        losses = learned.train(net, x, t, steps=steps, batch=cfg["batch"], lr=cfg["lr"])
        train_s = time.perf_counter() - t0
        del x, t
        torch.cuda.empty_cache()
        nets[fmt] = net
        log(f"{FORMAT_NAMES[fmt]} network: data {data_s:.1f} s, training {train_s:.1f} s")
        training[FORMAT_NAMES[fmt]] = (f"Adam lr {cfg['lr']}, batch {cfg['batch']}, {steps} steps on {cfg['train_blocks']} "
                                       f"blocks of generators {list(kinds)} (seeds apart from the batch's); data "
                                       f"{data_s:.1f} s, training {train_s:.1f} s, loss {float(losses[0]):.4f} -> "
                                       f"{float(losses[-64:].mean()):.4f}")
    texels = batch.info()["texels"]
    sel = [i for i, sp in enumerate(specs) if sp[2] in nets]
    points = []
    for k, point in enumerate(BATCH_FRONTIER):
        for fmt, net in nets.items():
            r_, m_ = point.get(fmt, (None, None))
            batch.set_proposal(net if r_ is not None else None, radius=r_ or 0, margin=m_ or 0.0, format=fmt)
        ms = timed_launches(batch, args.steps if k == 0 else max(2, args.steps // 2), args.warmup, flush, stream)
        step_ms = sum(ms) / len(ms)
        stats = {FORMAT_NAMES[f]: batch.proposal_stats(format=f) for f in nets if point.get(f, (None,))[0] is not None}
        points.append({"step_ms": step_ms, "stats": stats, "outs": [textures[i][4].clone() for i in sel]})
        log(f"learned point {point}: {step_ms:.2f} ms per step")
    for fmt in nets:
        batch.set_proposal(None, format=fmt)
    rm = texture_rmse(ctx, [specs[i] for i in sel], [textures[i] for i in sel],
                      [[plain_out[i] for i in sel]] + [p["outs"] for p in points])
    log("per-texture RMSE done")
    fmts = np.array([specs[i][2] for i in sel])
    blocks = {f: sum(ntg.chain_bytes(w, h, batch_options(o)) // ntg.BLOCK_BYTES[f] for (w, h, ff, o, img) in specs if ff == f)
              for f in nets}
    frontier = []
    for k, (point, p) in enumerate(zip(BATCH_FRONTIER, points)):
        d = 100.0 * (rm[k + 1] / np.maximum(rm[0], 1e-30) - 1.0)
        gated = np.array([point.get(int(f), (None,))[0] is not None for f in fmts])
        dg = d[gated] if gated.any() else np.zeros(1)
        f_ = {"point": {FORMAT_NAMES[f]: {"search": (f"descent, {v[0] & (DESCENT - 1)} moves" if v[0] & DESCENT
                                                     else f"window, radius {v[0]}"),
                                          "margin": v[1] if v[1] != INF else "inf (no fallback)"}
                        for f, v in point.items()},
              "step_ms": p["step_ms"], "value": world * texels / (p["step_ms"] / 1000.0) / 1e6,
              "speedup_vs_plain": plain_ms / p["step_ms"], "textures_gated": int(gated.sum()),
              "textures_within_0p5pct": float(np.mean(dg <= 0.5)),
              "rmse_delta_pct_mean": float(dg.mean()), "rmse_delta_pct_max": float(dg.max()),
              "textures_bit_equal": int(sum(torch.equal(o, plain_out[i]) for o, i in zip(p["outs"], sel)))}
        for f in nets:
            name = FORMAT_NAMES[f]
            if name in p["stats"]:
                st = p["stats"][name]
                f_[name] = {"full_fit_fraction": st["full_fit"] / max(1, blocks[f]),
                            "orderings_per_kept_block": st["orderings"] / max(1, st["kept"])}
        frontier.append(f_)
        del p["outs"]
    head = max(frontier, key=lambda f: (f["textures_within_0p5pct"], f["speedup_vs_plain"]))
    fastest = max(frontier, key=lambda f: f["speedup_vs_plain"])
    for net in nets.values():
        net.close()
    return {"value": head["value"], "step_ms": head["step_ms"], "plain_step_ms": plain_ms,
            "speedup_vs_plain": head["speedup_vs_plain"], "point": head["point"],
            "textures_within_0p5pct": head["textures_within_0p5pct"], "textures_gated": head["textures_gated"],
            "rmse_delta_pct_mean": head["rmse_delta_pct_mean"], "rmse_delta_pct_max": head["rmse_delta_pct_max"],
            "fastest_point": {k: fastest[k] for k in ("point", "speedup_vs_plain", "textures_within_0p5pct",
                                                       "rmse_delta_pct_mean", "rmse_delta_pct_max")},
            "gate": "per texture, the colour RMSE over all levels (nvtt::rmsError on the decoded blocks) of the learned "
                    "encoding within 0.5% of the plain fit's (the plain fit's blocks are the reference's)",
            "target": ">= 2x the plain fit's Mtexels/s with every texture within 0.5%",
            "target_met": bool(head["textures_within_0p5pct"] >= 1.0 and head["speedup_vs_plain"] >= 2.0),
            "formats_with_proposal": [FORMAT_NAMES[f] for f in nets],
            "network": "per format an MLP 48-256-256-8, GELU (tanh form), BF16 weights/activations, FP32 accumulation "
                       "(tcgen05), trained on the GPU by the library's own kernels",
            "training": training, "frontier": frontier}


def run_gpu_batch(args):
    import torch
    import ntg
    world, rank, local = dist_setup(args)
    name = args.workload
    desc = BATCHES[name][5]
    specs = batch_textures(name)   # before the GPU context: generated by spawned processes
    log(f"{name}: {len(specs)} textures generated")
    # N GPUs: the batch's textures split across the ranks (largest first by chain texels), each rank
    # running the batch of its own part; the whole batch's work is fixed (strong scaling)
    total_texels = sum(chain_texels(sp[0], sp[1]) for sp in specs)
    base_texels = sum(sp[0] * sp[1] for sp in specs)
    if world > 1:
        from ntg import partition
        parts = partition.partition_textures([(sp[0], sp[1]) for sp in specs], world)
        specs = [specs[i] for i in parts[rank]]
        log(f"rank {rank}: {len(specs)} textures of the batch")
    torch.cuda.set_device(local)
    ctx = ntg.Context(local)
    textures, host_in = [], []
    for (w, h, fmt, o, img) in specs:
        opt = batch_options(o)
        d_in = torch.from_numpy(img.reshape(-1).view(np.uint32)).cuda()
        d_out = torch.empty(ntg.chain_bytes(w, h, opt), dtype=torch.uint8, device="cuda")
        textures.append((d_in, w, h, opt, d_out))
        host_in.append(img)
    log("inputs on the device")
    t0 = time.perf_counter()
    batch = ntg.Batch(ctx, textures)
    build_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    batch.autotune()
    tune_s = time.perf_counter() - t0
    info = batch.info()
    log(f"batch built ({build_s:.1f} s), autotuned ({tune_s:.1f} s): {info['shape']}")
    flush = torch.empty(FLUSH_BYTES, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()
    barrier(world)
    with ClockSampler(torch.cuda.current_device()) as clk:
        t_wall = time.perf_counter()
        step_ms = timed_launches(batch, args.steps, args.warmup, flush, stream)
        barrier(world)
        wall = time.perf_counter() - t_wall
    dev_ms = max_over_ranks(world, sum(step_ms), torch.device("cuda"))
    value = total_texels * args.steps / (dev_ms / 1000.0) / 1e6
    plain_out = [t[4].clone() for t in textures]
    log(f"plain: {dev_ms / args.steps:.2f} ms per step")

    # end to end: every step copies every texture in from pinned host memory, replays the graph and
    # copies every texture's blocks out, in one library call over the steps; two bindings of the batch
    # (double buffering) let a step's copies run beside the neighbouring steps' graphs
    h_in = [torch.from_numpy(img.reshape(-1).view(np.uint32)).pin_memory() for img in host_in]
    h_outs = [[torch.empty(t[4].numel(), dtype=torch.uint8).pin_memory() for t in textures] for _ in range(2)]
    bi = sum(int(x.numel()) * 4 for x in h_in)
    bo = sum(int(x.numel()) for x in h_outs[0])
    # the alternate binding's buffers live as long as the batch: its graph writes them whenever the
    # batch recaptures
    alt_in = [torch.empty_like(t[0]) for t in textures]
    alt_out = [torch.empty_like(t[4]) for t in textures]
    batch.bind_alternate(alt_in, alt_out)

    def e2e_run(n):
        # one library call over n sets of host buffers: copies in, graph, copies out per set, the two
        # bindings taking turns (ntg_batch_process_host)
        batch.process_host([(h_in, h_outs[k & 1]) for k in range(n)])
        torch.cuda.synchronize()

    e2e_run(2)
    barrier(world)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e2e_run(args.steps)
    e2e_s = max_over_ranks(world, time.perf_counter() - t0, torch.device("cuda"))
    e2e_value = total_texels * args.steps / e2e_s / 1e6
    same = all(torch.equal(y, r.cpu()) for y, r in zip(h_outs[(args.steps - 1) & 1], plain_out))
    del h_in, h_outs
    log(f"e2e: {e2e_value:.0f} Mtexels/s")

    learned_info = None
    if name in LEARNED_BATCHES and not args.no_learned and world == 1:
        try:
            learned_info = learned_batch(ctx, batch, specs, textures, plain_out, dev_ms / args.steps, args, flush,
                                         stream, world)
        except Exception as e:  # reported in the line; the plain measurement stands
            import traceback
            traceback.print_exc()
            learned_info = {"error": f"{type(e).__name__}: {e}"}
            for fmt in FORMAT_NAMES:
                try:
                    batch.set_proposal(None, format=fmt)
                except Exception:
                    pass

    line = None
    if rank == 0:
        phases, blocks = batch.time_phases()
        clocks = clk.summary()
        peaks, peak_src = measured_peaks()
        hbm = peaks.get("hbm_gbs", 6800.0)
        # mip phase against HBM: read level l-1 (BGRA8 for level 0, else FP32 planar), write level l
        # (FP32 planar, plus the BGRA8 copy the BC3/BC5 encoders read)
        mip_bytes = 0
        for (w, h, fmt, o, img) in specs:
            lv = ntg.chain_levels(w, h)
            for i in range(1, len(lv)):
                mip_bytes += lv[i - 1][0] * lv[i - 1][1] * (4 if i == 1 else 16)
                mip_bytes += lv[i][0] * lv[i][1] * (16 + (4 if fmt != 1 else 0))
        mip_gbs = mip_bytes / (phases["mips"] / 1000.0) / 1e9
        dominant = max(("bc1", "bc3", "bc5", "mips"), key=lambda k: phases[k])
        roof_mips = {"bound": "hbm", "achieved": mip_gbs, "peak": hbm, "unit": "GB/s", "frac": mip_gbs / hbm,
                     "traffic": None, "kernel": "mip launches of the batch (k_tile2x_u8, k_tile2x_f32, k_tile2x, k_poly, k_mip_tail, k_fast_down)",
                     "algorithmic_bytes": mip_bytes, "ms": phases["mips"], "peak_source": peak_src}
        roof = None
        if dominant == "bc1" and phases["bc1"] > 0:
            # the BC1 Level8 fit against the FP32 peak: orderings counted on the device by the same
            # gather / reduce_colors the encoder runs, times the FP32 operations of one ordering
            n4, n3 = batch.count_work()
            sm_mhz_b = clocks["sm_mhz"] or 2070.0
            peak_b = 152 * 128 * sm_mhz_b * 1e6
            ops = n4 * OPS_PER_ORDERING4 + n3 * OPS_PER_ORDERING3
            ach = ops / (phases["bc1"] / 1000.0)
            nb1 = blocks["bc1"]
            roof = {"bound": "fp32", "achieved": ach / 1e12, "peak": peak_b / 1e12, "unit": "TFLOP/s",
                    "frac": ach / peak_b,
                    "traffic": BC1_TRAFFIC_PER_BLOCK * nb1 if nb1 and BC1_TRAFFIC_PER_BLOCK else None,
                    "kernel": "k_bc1<7> (icbc Level8 cluster fit)",
                    "note": f"peak = 152 SMs x 128 FP32 lanes x median SM clock {sm_mhz_b:.0f} MHz; {n4} four-cluster x "
                            f"{OPS_PER_ORDERING4} + {n3} three-cluster x {OPS_PER_ORDERING3} FP32 ops over the BC1 phase "
                            f"({phases['bc1']:.3f} ms, one run outside the graph, CUDA events); traffic: DRAM bytes per "
                            f"block of one ncu capture of k_bc1<7>, times the blocks"}
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": dev_ms / args.steps, "higher_is_better": True,
                "scaling": "strong" if world > 1 else "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "base_level": {"value": base_texels * args.steps / (dev_ms / 1000.0) / 1e6, "unit": UNIT,
                               "texels_per_step": base_texels, "note": "level-0 texels only, same device time"},
                "config": {"workload": desc, "textures": BATCHES[name][0], "texels_per_step": total_texels,
                           "blocks_per_step": info["blocks"] if world == 1 else None,
                           "l2": "inputs (14 GB for c4) larger than L2, and L2 flushed (256 MiB write) between steps",
                           "method": "value: plain (non-learned) cluster fit, bit-identical to the reference; "
                                     "learned: the endpoint proposals (key 'learned', one GPU)",
                           "ranks": "one GPU" if world == 1 else f"{world} ranks, the batch's textures partitioned largest "
                                                                  "first by chain texels (ntg.partition), no exchange",
                           "launch_shape": info["shape"], "build_s": build_s, "autotune_s": tune_s,
                           "images": "one seeded image per distinct (size, format)"},
                "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": bi, "d2h_bytes_per_step": bo,
                        "matches_device_path": same,
                        "api": "ntg_batch_process_host: host buffers, two bindings taking turns, copies on their own streams"},
                "gpu_launches": info["launches"] * args.steps,
                "clocks": clocks, "roofline": roof, "roofline_mips": roof_mips,
                "phase_ms": phases, "phase_blocks": blocks, "dominant_phase": dominant,
                "graph_vs_phases_ms": {"step": dev_ms / args.steps, "sum_of_phases": sum(phases.values()),
                                       "note": "each phase run alone outside the graph; the step replays them all in "
                                               "one graph"},
                "learned": learned_info, "wall_s_timed": wall, "cpu_baseline": None}
    batch.close()
    del textures, plain_out, alt_in, alt_out
    torch.cuda.empty_cache()
    if world == 1 and name == "c4" and not args.no_c1:
        # secondary key: the single 4096x4096 chain
        try:
            c1 = measure_chain(ctx, "c1", args, world, rank, with_cpu=not args.no_cpu)
            line["c1"] = {k: c1[k] for k in ("value", "ms_per_step", "e2e", "roofline", "roofline_mips", "split_ms",
                                             "config", "cpu_baseline", "gpu_launches")}
            log(f"c1: {c1['value']:.0f} Mtexels/s")
        except Exception as e:  # reported in the line
            import traceback
            traceback.print_exc()
            line["c1"] = {"error": f"{type(e).__name__}: {e}"}
    if rank == 0:
        if not args.no_cpu and world == 1:
            try:
                line["cpu_baseline"] = cpu_batch_sample(name, specs, os.cpu_count() or 1, 20.0)
            except Exception as e:  # reported, not fatal
                line["cpu_baseline"] = {"value": None, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
                                        "sample": f"failed: {e}"}
            line["cpu_baseline"].update(host_cpu())
        print(json.dumps(line), flush=True)
    ctx.close()
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


def cpu_batch_sample(name, specs, threads, budget_s):
    """The oracle port on the host cores over the batch's textures in order until about `budget_s`
    seconds of work: whole chains, mips on one thread, encode on `threads`."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    pyoracle.build_oracle()
    oracle = pyoracle.Oracle()
    done, texels, total = 0, 0, 0.0
    for (w, h, fmt, o, img) in specs:
        spec = (w, h, fmt, o[1], o[2], o[3], o[4], o[5])
        total += cpu_chain(oracle, img, spec, threads)[0]
        texels += chain_texels(w, h)
        done += 1
        if total >= budget_s:
            break
    return {"value": texels / total / 1e6, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"the first {done} of {len(specs)} textures of {name} with their whole chains "
                      f"({texels} texels, {total:.1f} s)"}


def run_reference_batch(args):
    """The reference arm on a batch: the oracle port over a bounded sample of its textures per step."""
    world, rank, _ = dist_setup(args)
    if rank != 0:
        return 0
    name = args.workload
    specs = batch_textures(name)
    threads = os.cpu_count() or 1
    budget = args.cpu_seconds
    sample = cpu_batch_sample(name, specs, threads, budget)
    for _ in range(args.warmup - 1):
        cpu_batch_sample(name, specs, threads, budget)
    vals = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        vals.append(cpu_batch_sample(name, specs, threads, budget))
        vals[-1]["s"] = time.perf_counter() - t0
    value = statistics.mean(v["value"] for v in vals)
    why = ("the reference library itself cannot be built on this host (its source tree is absent), so its C "
           "restatement in oracle/ runs: mips on one thread as the reference filters, encode on every core")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * statistics.mean(v["s"] for v in vals),
            "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": BATCHES[name][5], "sample": sample["sample"]},
            "cpu_baseline": dict({"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                                  "sample": sample["sample"] + "; " + why}, **host_cpu()),
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------------------------
# The learned endpoint proposal (BC1): trained on seeded blocks of both generators, evaluated on a
# separate-seed 2048x2048 texture against the plain GPU cluster fit.

LEARNED = {"train_blocks": 1 << 24, "train_size": 2048, "batch": 8192, "lr": 1e-3, "eval_size": 2048,
           # headline operating point: neighbourhood radius 2, no fallback to the full fit (the network's
           # error estimate unused); the frontier below, on the same texture, includes the fallback points
           "radius": 2, "margin": float("inf"),
           # the radius / margin trade-off, measured on the same texture and reported beside the headline
           "frontier": [(1, 0.01), (1, 0.1), (1, 0.25), (1, 0.5), (1, float("inf")), (2, 0.01), (2, 0.25), (2, float("inf")),
                        (3, 0.25)]}


def run_gpu_learned(args):
    import torch
    import ntg
    from ntg import learned
    world, rank, local = dist_setup(args)
    torch.cuda.set_device(local)
    ctx = ntg.Context(local)
    cfg = LEARNED
    t0 = time.perf_counter()
    x, t = learned.training_set(ctx, cfg["train_blocks"], seed=0x5EED, size=cfg["train_size"])
    data_s = time.perf_counter() - t0
    net = ntg.MLP(seed=0x4E4554)
    steps = cfg["train_blocks"] // cfg["batch"]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    losses = learned.train(net, x, t, steps=steps, batch=cfg["batch"], lr=cfg["lr"])
    train_s = time.perf_counter() - t0
    del x, t
    size = cfg["eval_size"]
    kind = 1  # the RGBA8 generator: sRGB colour, alpha field, Kaiser mips, transparency
    img = learned.generator_texture(kind, size, 0xE7A1 + kind)
    opt = learned.generator_options(kind)
    d = torch.from_numpy(img).cuda()
    texels = chain_texels(size, size)
    plain = ctx.compress_chain(d, size, size, opt)
    out, st = ctx.compress_chain_learned(net, d, size, size, opt, radius=cfg["radius"], margin=cfg["margin"])
    flush = torch.empty(FLUSH_BYTES, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()

    def timed_steps(fn):
        for _ in range(args.warmup):
            fn()
        torch.cuda.synchronize()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
        for a, b in ev:
            flush.zero_()
            a.record(stream)
            fn()
            b.record(stream)
        torch.cuda.synchronize()
        return sum(a.elapsed_time(b) for a, b in ev) / args.steps

    with ClockSampler(torch.cuda.current_device()) as clk:
        n0 = ntg.launch_count()
        learned_ms = timed_steps(lambda: ctx.compress_chain_learned(net, d, size, size, opt, radius=cfg["radius"],
                                                                    margin=cfg["margin"], out=out, stats=False))
        # the library's kernel launches per learned chain (the timed steps and their warm-up)
        learned_launches = (ntg.launch_count() - n0) // (args.steps + args.warmup)
        plain_ms = timed_steps(lambda: ctx.compress_chain(d, size, size, opt, out=plain))
    value = texels / (learned_ms / 1000.0) / 1e6
    rmse_plain = learned.chain_rmse(ctx, d, size, size, opt, plain)
    rmse_learned = learned.chain_rmse(ctx, d, size, size, opt, out)
    same = float((out.view(-1, 8) == plain.view(-1, 8)).all(dim=1).float().mean().item())
    nb = plain.numel() // 8
    frontier = []
    for r_, m_ in cfg["frontier"]:
        o_, st_ = ctx.compress_chain_learned(net, d, size, size, opt, radius=r_, margin=m_)
        ms_ = learned.timed(lambda: ctx.compress_chain_learned(net, d, size, size, opt, radius=r_, margin=m_, out=o_,
                                                               stats=False))
        rl_ = learned.chain_rmse(ctx, d, size, size, opt, o_)
        frontier.append({"radius": r_, "margin": m_ if m_ != float("inf") else "inf", "speedup_vs_plain": plain_ms / ms_,
                         "rmse_delta_pct": 100 * (rl_ / rmse_plain - 1), "full_fit_fraction": st_["full_fit"] / (plain.numel() // 8)})
    # the network's inference kernel against the tensor-core peak (one call over every block)
    xf = ctx.chain_features(d, size, size, opt)
    y = net.infer(xf)
    infer_ms = learned.timed(lambda: net.infer(xf, out=y))
    flop = nb * 2 * (48 * 256 + 256 * 256 + 256 * 16)
    peaks, peak_src = measured_peaks()
    tflops = flop / (infer_ms / 1000.0) / 1e12
    peak = peaks.get("bf16_tflops", 1900.0)
    # end to end: host image in, blocks out, through the same call
    h_in = torch.from_numpy(img.reshape(-1)).pin_memory()
    h_out = torch.empty(out.numel(), dtype=torch.uint8).pin_memory()

    def e2e_step():
        d.view(-1).copy_(h_in, non_blocking=True)
        ctx.compress_chain_learned(net, d, size, size, opt, radius=cfg["radius"], margin=cfg["margin"], out=out,
                                   stats=False)
        h_out.copy_(out, non_blocking=True)
        torch.cuda.current_stream().synchronize()

    e2e_step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    e2e_value = texels * args.steps / (time.perf_counter() - t0) / 1e6
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": learned_ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "bf16+f32",
            "data": "synthetic",
            "config": {"workload": f"learned endpoint proposal, BC1 Normal: {size}x{size} separate-seed RGBA8 texture "
                                   "(sRGB, alpha field, Kaiser mips, transparency), whole chain",
                       "texels_per_step": texels, "blocks_per_step": nb, "l2": "flushed (256 MiB write) between steps",
                       "network": "MLP 48-256-256-8, GELU (tanh form), BF16 weights/activations, FP32 accumulation (tcgen05)",
                       "training": f"Adam lr {cfg['lr']}, batch {cfg['batch']}, {steps} steps on {cfg['train_blocks']} "
                                   f"seeded blocks of both generators; data {data_s:.1f} s, training {train_s:.1f} s, "
                                   f"loss {float(losses[0]):.4f} -> {float(losses[-64:].mean()):.4f}",
                       "radius": cfg["radius"], "margin": cfg["margin"] if cfg["margin"] != float("inf") else "inf"},
            "learned": {"chain_ms": learned_ms, "plain_chain_ms": plain_ms, "speedup_vs_plain": plain_ms / learned_ms,
                        "rmse": rmse_learned, "plain_rmse": rmse_plain, "rmse_delta_pct": 100 * (rmse_learned / rmse_plain - 1),
                        "blocks_equal_to_plain": same, "full_fit_fraction": st["full_fit"] / nb,
                        "orderings_per_block": st["orderings"] / max(1, st["kept"] + st["full_fit"]),
                        "frontier": frontier},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(img.nbytes),
                    "d2h_bytes_per_step": int(out.numel()), "matches_device_path": bool(torch.equal(h_out, out.cpu()))},
            "gpu_launches": learned_launches * args.steps, "clocks": clk.summary(),
            "roofline": {"bound": "tensor", "achieved": tflops, "peak": peak, "unit": "TFLOP/s", "frac": tflops / peak,
                         "traffic": None, "kernel": "k_mlp_infer (fused 3-layer tcgen05 inference, one call over all blocks)",
                         "flop_per_block": 2 * (48 * 256 + 256 * 256 + 256 * 16), "ms": infer_ms, "peak_source": peak_src},
            "cpu_baseline": None}
    print(json.dumps(line), flush=True)
    net.close()
    ctx.close()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ntg", choices=["ntg", "reference"])
    ap.add_argument("--workload", default="c4", choices=sorted(WORKLOADS) + sorted(BATCHES) + ["c3"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-learned", action="store_true", help="c4: skip the learned proposals' measurement")
    ap.add_argument("--no-c1", action="store_true", help="c4: skip the secondary c1 measurement")
    ap.add_argument("--cpu-seconds", type=float, default=5.0, help="CPU work per reference-arm step on batched workloads")
    args = ap.parse_args()
    if args.warmup < 3:
        log("warmup raised to 3")
        args.warmup = 3
    if args.impl == "reference":
        if args.workload == "c3":
            print(json.dumps({"impl": "reference", "unavailable": "the learned proposal has no counterpart in the "
                              "reference; its plain cluster fit is the c1/c0 reference arm"}), flush=True)
            return 0
        return run_reference_batch(args) if args.workload in BATCHES else run_reference(args)
    if args.workload == "c3":
        return run_gpu_learned(args)
    return run_gpu_batch(args) if args.workload in BATCHES else run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
