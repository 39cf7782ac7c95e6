"""Benchmark: detection-event Gbit/s of the bulk detection sampler.

Workload (one step): 2^20 shots of the rotated surface code memory-Z experiment, distance 25, 25 rounds
(1249 qubits, 15,600 detectors + 1 observable, REPEAT block kept as a loop), p = 1e-3 on all four noise
knobs, generated by the reference's generator (tests/golden/circuits/surface_rz_d25_r25.stim).  This is
one 2^20-shot chunk of the 2^24-shot streamed configuration.

  value : device-resident Gbit/s = shots x (detectors + observables) / time of the noise kernel, the frame
          kernel and the shot-major transpose, output left in HBM (CUDA events on the library's stream).
  e2e   : the same metric through the public API (CompiledDetectorSampler.sample(..., bit_packed=True,
          separate_observables=True, dets_out=, obs_out=)) into reused page-locked host arrays, device->host
          copies included (the same call into pageable arrays is reported beside it).
  other legs (same JSON line): batched (256 circuits in one launch), serving (Poisson arrivals), m2d (the
          measurements-to-detection-events converter), dem (detector-error-model sampling), feed (the decoder
          feed with postselection), cpu_baseline (the oracle port on all host cores and on one).

`--impl reference` times the CPU reference implementation of the path on the host cores: the oracle port
(oracle/stim_oracle.c, a 64-bit-word restatement of the reference's FrameSimulator) with all host threads,
on a bounded sample of the same workload per step.
"""

import argparse
import json
import math
import os
import re
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "detection-event Gbit/s at d=25 r=25 (surface_code:rotated_memory_z, p=1e-3)"
# DRAM bytes per shot of the frame kernel on this workload, dram__bytes_read.sum + dram__bytes_write.sum from
# one ncu capture of 131,072 shots (lean frame kernel, hit-list mode, 1 block x 128 threads per CTA: 155.93 +
# 218.82 MB); traffic grows with shots.
FRAME_DRAM_BYTES_PER_SHOT = 2859.1
UNIT = "Gbit/s"
E2E_WARMUP = 3
WORKLOAD = dict(family="surface_code:rotated_memory_z", distance=25, rounds=25, p=0.001)


def circuit_text():
    from stim_gb300 import workloads

    return workloads.code_circuit(WORKLOAD["family"], WORKLOAD["distance"], WORKLOAD["rounds"], WORKLOAD["p"])


def algorithmic_work(text):
    """Per-shot shared-memory frame-bit accesses and random bits, with the per-gate rules:
    1q Clifford = read 2 + write 2 (H) or 1 (S-like); CX/CZ = read 4 + write 2; other 2q = 8; M = 3;
    MR = 4; R = 2; DETECTOR with k record refs = k + 1; a noise hit = 4 (8 for DEPOLARIZE2);
    random bits = 1 per M/MR/R target plus one per qubit at the start of a shot."""
    acc = 0.0
    rbits = 0.0
    hits = 0.0
    mult = [1]
    for line in text.splitlines():
        line = line.split("#")[0].strip()
        if not line:
            continue
        if line.startswith("REPEAT"):
            mult.append(mult[-1] * int(line.split()[1]))
            continue
        if line == "}":
            mult.pop()
            continue
        m = re.match(r"([A-Z_0-9]+)(?:\(([^)]*)\))?\s*(.*)", line)
        g, args, targets = m.group(1), m.group(2), m.group(3).split()
        k = mult[-1]
        n = len(targets)
        if g in ("H", "H_YZ", "SQRT_X", "SQRT_Y"):
            acc += k * n * 4
        elif g in ("S", "S_DAG", "H_XY"):
            acc += k * n * 3
        elif g in ("CX", "CZ", "CY"):
            acc += k * (n // 2) * 6
        elif g in ("SWAP", "ISWAP"):
            acc += k * (n // 2) * 8
        elif g in ("M", "MX"):
            acc += k * n * 3
            rbits += k * n
        elif g in ("MR", "MRX"):
            acc += k * n * 4
            rbits += k * n
        elif g in ("R", "RX"):
            acc += k * n * 2
            rbits += k * n
        elif g == "DETECTOR":
            acc += k * (n + 1)
        elif g in ("X_ERROR", "Z_ERROR", "DEPOLARIZE1"):
            hits += k * n * float(args)
            acc += k * n * float(args) * 4
        elif g == "DEPOLARIZE2":
            hits += k * (n // 2) * float(args)
            acc += k * (n // 2) * float(args) * 8
    return acc, rbits, hits


def e2e_tail(times, parts):
    """Where the slow end-to-end calls (over 1.15x the median) spend their time: the sampler's own CUDA-event split
    of each call into kernels and the rest (device->host copies and the gaps between them)."""
    if not times:
        return None
    med = statistics.median(times)
    slow = [k for k, t in enumerate(times) if t > 1.15 * med]
    fast = [k for k in range(len(times)) if k not in set(slow)]

    def split(ks):
        if not ks:
            return None
        kern = statistics.mean(parts[k]["frame_ms"] + parts[k]["noise_ms"] + parts[k]["transpose_ms"] for k in ks)
        return {"kernels_ms": kern, "copy_ms": statistics.mean(parts[k]["copy_ms"] for k in ks),
                "wall_ms": 1e3 * statistics.mean(times[k] for k in ks)}

    return {"slow_calls": len(slow), "slow_call_indices": slow[:16], "slow": split(slow), "typical": split(fast)}


def _nearest_rank(values, q):
    """The q-quantile of `values` by the nearest-rank rule (the ceil(q * n)-th smallest)."""
    xs = sorted(values)
    return xs[min(len(xs) - 1, max(0, int(math.ceil(q * len(xs))) - 1))]


class quiet_gc:
    """Python's cyclic garbage collector off inside a timed loop (as the standard library's timeit does), so
    that a collection of the interpreter's objects does not land inside one timed call."""

    def __enter__(self):
        import gc

        gc.collect()
        self.was = gc.isenabled()
        gc.disable()

    def __exit__(self, *exc):
        import gc

        if self.was:
            gc.enable()


def measure_link(local, nbytes=1 << 31, reps=5):
    """Device-to-host and host-to-device rates of this GPU's host link: cudaMemcpyAsync of `nbytes` between
    HBM and page-locked host memory, best of `reps` (CUDA events on a side stream).  The device-to-host figure
    is the floor of the end-to-end step (every output byte crosses it once)."""
    import torch

    dev = torch.empty(nbytes, dtype=torch.uint8, device=f"cuda:{local}")
    dev.fill_(1)
    host = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
    host.fill_(0)
    st = torch.cuda.Stream(device=f"cuda:{local}")
    out = {}
    for name, (dst, src) in (("d2h", (host, dev)), ("h2d", (dev, host))):
        best = None
        for _ in range(reps):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            with torch.cuda.stream(st):
                a.record(st)
                dst.copy_(src, non_blocking=True)
                b.record(st)
            b.synchronize()
            ms = a.elapsed_time(b)
            best = ms if best is None else min(best, ms)
        out[name + "_gbs"] = nbytes / (best / 1e3) / 1e9
    del dev, host
    torch.cuda.empty_cache()
    return out


def noise_philox_calls(text):
    """Expected Philox4x32-10 calls per shot of the hit-list noise kernel under the random-bit contract: each
    noise instruction instance is cut into segments of 16 units x 128 shots; a segment draws one 32-bit value
    for the first gap, then per hit one more for the Pauli choice (DEPOLARIZE1/2) and one for the next gap,
    four draws per Philox call.  E[ceil(draws / 4)] under the binomial number of hits, per 128 shots, / 128."""
    from math import comb

    def calls_per_segment(trials, p, choice):
        if p <= 0:
            return 0.0
        if p >= 1:
            return math.ceil(trials * (1 + choice) / 4)
        acc, cum, h = 0.0, 0.0, 0
        while cum < 1 - 1e-12 and h <= trials:
            pr = comb(trials, h) * p ** h * (1 - p) ** (trials - h)
            acc += pr * math.ceil((1 + h * (1 + choice)) / 4)
            cum += pr
            h += 1
        return acc

    total = 0.0
    mult = [1]
    for line in text.splitlines():
        line = line.split("#")[0].strip()
        if not line:
            continue
        if line.startswith("REPEAT"):
            mult.append(mult[-1] * int(line.split()[1]))
            continue
        if line == "}":
            mult.pop()
            continue
        m = re.match(r"([A-Z_0-9]+)(?:\(([^)]*)\))?\s*(.*)", line)
        g, args, targets = m.group(1), m.group(2), m.group(3).split()
        if g in ("X_ERROR", "Y_ERROR", "Z_ERROR", "DEPOLARIZE1"):
            units, choice = len(targets), 1 if g == "DEPOLARIZE1" else 0
        elif g == "DEPOLARIZE2":
            units, choice = len(targets) // 2, 1
        elif g in ("M", "MX", "MY", "MR", "MRX", "MRY") and args:
            units, choice = len(targets), 0
        else:
            continue
        p = float(args)
        full, rest = divmod(units, 16)
        seg = full * calls_per_segment(16 * 128, p, choice) + (calls_per_segment(rest * 128, p, choice) if rest else 0)
        total += mult[-1] * seg / 128.0
    return total


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "50"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, FileNotFoundError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm = [float(r[1]) for r in self.rows if len(r) >= 9 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) >= 9 and r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            if len(r) >= 9:
                for name, v in zip(names, r[5:9]):
                    if v.lower() == "active":
                        reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


def cpu_baseline(text, D, O, chunk, threads, min_s, max_s):
    """The oracle port on the host cores: consecutive `chunk`-shot calls until at least `min_s` seconds of
    CPU work (at most `max_s`) have been timed.  Returns (Gbit/s, seconds, shots)."""
    from oracle.oracle import OracleCircuit

    c = OracleCircuit(text)
    c.sample(min(chunk, 1024), 1, threads=threads)  # warm
    shots = 0
    t0 = time.perf_counter()
    while True:
        c.sample(chunk, 2, first_shot=shots, threads=threads)
        shots += chunk
        dt = time.perf_counter() - t0
        if dt >= min_s or dt + dt / (shots // chunk) > max_s:
            break
    return shots * (D + O) / dt / 1e9, dt, shots


def _measured_hbm_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            v = json.load(f).get("hbm_gbs")
            if v:
                return float(v)
    except (OSError, ValueError):
        pass
    return 6800.0


def reference_stim():
    """The reference's own `stim` binary, built from the reference's sources with the reference's release flags
    (oracle/Makefile `ref-bench`: g++ -O3 -fno-strict-aliasing; on aarch64 the reference sets no SIMD flag, so it
    runs on 64-bit words) on first use.  The sources come from $STIM_REFERENCE_TREE or the copy staged under
    baseline/_ref.  Returns None where neither exists."""
    arch = os.uname().machine
    exe = os.path.join(ROOT, "oracle", "_ref", f"bench-{arch}", "stim")

    def runs():
        try:
            return subprocess.run([exe, "help"], capture_output=True, timeout=30).returncode == 0
        except (OSError, subprocess.TimeoutExpired):
            return False

    if os.path.isfile(exe) and runs():
        return exe
    staged = os.path.join(ROOT, "baseline", "_ref", "stim", "file_lists", "source_files_no_main")
    if not (os.environ.get("STIM_REFERENCE_TREE") or os.path.isfile(staged)):
        return None
    jobs = str(max(1, os.cpu_count() or 1))
    r = subprocess.run(["make", "-s", "-j" + jobs, "-C", os.path.join(ROOT, "oracle"), "ref-bench"],
                       capture_output=True, text=True)
    if r.returncode != 0 or not runs():
        sys.stderr.write("reference build failed:\n" + r.stderr[-2000:] + "\n")
        return None
    return exe


def reference_compiler():
    try:
        return subprocess.run(["g++", "--version"], capture_output=True, text=True).stdout.splitlines()[0]
    except (OSError, IndexError):
        return "g++"


def time_reference_detect(exe, circuit_path, shots, procs, seed0):
    """Wall time of `stim detect --shots N --seed s --out_format b8 --append_observables --out /dev/null` as
    `procs` concurrent processes with distinct seeds, `shots` shots in total (sinter-style sharding of one
    job over the host cores; procs = 1 is the single-core CLI)."""
    per = [shots // procs + (1 if i < shots % procs else 0) for i in range(procs)]
    t0 = time.perf_counter()
    ps = [subprocess.Popen([exe, "detect", "--shots", str(n), "--seed", str(seed0 + i), "--out_format", "b8",
                            "--append_observables", "--out", "/dev/null", "--in", circuit_path],
                           stdout=subprocess.DEVNULL, stderr=subprocess.PIPE) for i, n in enumerate(per) if n]
    errs = [p.communicate()[1] for p in ps]
    dt = time.perf_counter() - t0
    for p, e in zip(ps, errs):
        if p.returncode != 0:
            raise RuntimeError("reference stim failed: " + e.decode(errors="replace")[-500:])
    return dt


def _circuit_file(text):
    import tempfile

    fd, path = tempfile.mkstemp(suffix=".stim")
    with os.fdopen(fd, "w") as f:
        f.write(text)
    return path


def reference_cpu_figures(text, D, O, shots_all, shots_one, reps):
    """The reference's CLI sampler on this host: all cores (one process per core) and one core.  Returns a
    dict, or None when the reference cannot be built here."""
    exe = reference_stim()
    if exe is None:
        return None
    path = _circuit_file(text)
    try:
        cores = os.cpu_count() or 1
        time_reference_detect(exe, path, min(shots_all, 4096 * cores), cores, 1000)  # warm page cache
        all_s = [time_reference_detect(exe, path, shots_all, cores, 100 * k) for k in range(reps)]
        one_s = [time_reference_detect(exe, path, shots_one, 1, 7)]
    finally:
        os.unlink(path)
    med = statistics.median(all_s)
    return {"value": shots_all * (D + O) / med / 1e9, "unit": UNIT, "cores": cores, "kind": "reference",
            "sample": f"stim detect --out_format b8 --append_observables --out /dev/null: {shots_all} shots as "
                      f"{cores} processes (distinct seeds), median of {reps}; reference built from its own sources "
                      f"with -O3 -fno-strict-aliasing ({reference_compiler()}), "
                      f"{'64-bit words (no SIMD flag on aarch64)' if os.uname().machine == 'aarch64' else 'SSE2 128-bit words'}",
            "one_core": {"value": shots_one * (D + O) / one_s[0] / 1e9, "unit": UNIT, "cores": 1,
                         "sample": f"{shots_one} shots, one process"},
            "p50_ms": 1e3 * med, "p99_ms": 1e3 * max(all_s)}


def run_reference(args):
    """The reference arm: the reference's own CPU sampler (its `stim detect` CLI, built from its sources) on the
    host cores, one process per core, over --ref-shots shots of the main workload per step.  Falls back to the
    oracle port (oracle/stim_oracle.c) only where the reference's sources are not on this machine."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle.oracle import OracleCircuit

    text = circuit_text()
    exe = reference_stim()
    cores = os.cpu_count() or 1
    times = []
    oc = OracleCircuit(text)  # detector and observable counts (nothing of the GPU library runs in this arm)
    D, O = oc.num_detectors, oc.num_observables
    if exe is not None:
        path = _circuit_file(text)
        try:
            for k in range(args.warmup):
                time_reference_detect(exe, path, args.ref_shots, cores, 10_000 + k * cores)
            for k in range(args.steps):
                times.append(time_reference_detect(exe, path, args.ref_shots, cores, 20_000 + k * cores))
            one = time_reference_detect(exe, path, args.ref_shots // 16, 1, 7)
        finally:
            os.unlink(path)
        kind = "reference"
        simd = "64-bit words (no SIMD flag on aarch64)" if os.uname().machine == "aarch64" else "SSE2 128-bit words"
        note = (f"the reference's `stim detect --out_format b8 --append_observables --out /dev/null`, built from "
                f"its own sources with its release flags (-O3 -fno-strict-aliasing, {reference_compiler()}), "
                f"{simd}; one process per host core with distinct seeds, shots split evenly")
        extra = {"one_core": {"value": (args.ref_shots // 16) * (D + O) / one / 1e9, "unit": UNIT, "cores": 1,
                              "sample": f"{args.ref_shots // 16} shots, one process"}}
    else:
        c = oc
        for _ in range(args.warmup):
            c.sample(args.ref_shots, 0, threads=cores)
        for k in range(args.steps):
            t0 = time.perf_counter()
            c.sample(args.ref_shots, 1 + k, threads=cores)
            times.append(time.perf_counter() - t0)
        kind = "port"
        note = ("oracle port (oracle/stim_oracle.c, pthreads over 1024-shot batches, 64-bit words): the reference's "
                "sources are not on this machine")
        extra = {}
    total = sum(times)
    value = args.steps * args.ref_shots * (D + O) / total / 1e9
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64 bitwise",
        "data": "synthetic (reference-generated circuit, seeded shots)",
        "config": {"workload": "surface_code:rotated_memory_z d=25 r=25 p=1e-3", "shots_per_step": args.ref_shots,
                   "note": note},
        "cpu_baseline": dict({"value": value, "unit": UNIT, "cores": cores, "kind": kind,
                              "sample": f"{args.ref_shots} shots per step x {args.steps} steps"}, **extra),
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "p50_ms": 1e3 * statistics.median(times),
        "p99_ms": 1e3 * sorted(times)[min(len(times) - 1, int(math.ceil(0.99 * len(times))) - 1)],
    }
    print(json.dumps(line))


def run_gpu(args):
    import numpy as np
    import torch

    import stim_gb300
    from stim_gb300 import _native

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    text = circuit_text()
    circ = stim_gb300.Circuit(text)
    D, O = circ.num_detectors, circ.num_observables
    shots = args.shots
    # One stream sharded by shot range: every rank uses the same seed and samples its own blocks of it
    # (step k of rank r = global shots [(k * world + r) * shots, ...)); no collective touches the data.
    sampler = circ.compile_detector_sampler(seed=args.seed, device=local)
    shots_al = (args.shots + 127) // 128 * 128
    step_no = [0]
    sampler.set_noise_mode(args.noise_mode)
    if args.shape:
        b, t = [int(x) for x in args.shape.split(",")]
        sampler.set_launch_shape(b, t)
    elif args.autotune:
        sampler.autotune(1 << 18)  # launch shape by measurement (results never depend on it)
    drow, orow = (D + 7) // 8, (O + 7) // 8
    dets = torch.empty((shots, drow), dtype=torch.uint8, device=f"cuda:{local}")
    obs = torch.empty((shots, orow), dtype=torch.uint8, device=f"cuda:{local}")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{local}")
    L = _native.lib()
    flags = _native.BIT_PACKED

    def device_step():
        sampler.set_stream_position((step_no[0] * world + rank) * shots_al)
        step_no[0] += 1
        _native.check(L.gfs_sample_detections_device(sampler._h, shots, flags, dets.data_ptr(), drow,
                                                     obs.data_ptr(), orow))
        return sampler.last_timings()

    for _ in range(args.warmup):
        device_step()
    clocks = ClockSampler(local)
    clocks.start()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    frame_ms, noise_ms, step_ms, launches, frame_launches, noise_launches = [], [], [], 0, 0, 0
    t0 = time.perf_counter()
    for _ in range(args.steps):
        flush.zero_()  # outputs exceed L2 anyway; also evict them between steps
        t = device_step()
        frame_ms.append(t["frame_ms"])
        noise_ms.append(t["noise_ms"])
        step_ms.append(t["frame_ms"] + t["noise_ms"] + t["transpose_ms"])
        launches += t["frame_launches"] + t["noise_launches"] + t["transpose_launches"]
        frame_launches += t["frame_launches"]
        noise_launches += t["noise_launches"]
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    if world > 1:
        torch.distributed.barrier()
    clk = clocks.stop()
    dev_s = sum(step_ms) / 1e3
    if world > 1:
        tt = torch.tensor([dev_s], device=f"cuda:{local}", dtype=torch.float64)
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        dev_s = float(tt.item())
    value = world * args.steps * shots * (D + O) / dev_s / 1e9

    # End to end through the public API into host numpy arrays that the caller reuses between requests
    # (dets_out= / obs_out=, as a streaming caller does).  The headline uses page-locked arrays (numpy views of
    # torch pin_memory tensors), so the device->host copies run as DMA at the link's rate; the same call into
    # ordinary pageable numpy arrays is reported beside it.  E2E_WARMUP untimed calls touch the pages first.
    def e2e_leg(dets_arr, obs_arr):
        times, parts = [], []
        if args.e2e_steps <= 0:
            return times, parts
        with quiet_gc():
            for k in range(E2E_WARMUP + args.e2e_steps):
                t1 = time.perf_counter()
                sampler.sample(shots, bit_packed=True, separate_observables=True, dets_out=dets_arr,
                               obs_out=obs_arr)
                if k >= E2E_WARMUP:
                    times.append(time.perf_counter() - t1)
                    parts.append(sampler.last_timings())
        return times, parts

    pin_rows = shots if args.e2e_steps > 0 else 0
    pinned_dets = torch.empty((pin_rows, drow), dtype=torch.uint8, pin_memory=True).numpy()
    pinned_obs = torch.empty((pin_rows, orow), dtype=torch.uint8, pin_memory=True).numpy()
    e2e_times, e2e_parts = e2e_leg(pinned_dets, pinned_obs)
    e2e_s = sum(e2e_times)
    e2e_value = world * len(e2e_times) * shots * (D + O) / e2e_s / 1e9 if e2e_times else None
    page_times, _ = e2e_leg(np.empty((pin_rows, drow), dtype=np.uint8), np.empty((pin_rows, orow), dtype=np.uint8))
    page_value = world * len(page_times) * shots * (D + O) / sum(page_times) / 1e9 if page_times else None

    acc_bits, rbits, hits = algorithmic_work(text)
    frame_avg_s = statistics.mean(frame_ms) / 1e3
    achieved_gbs = acc_bits / 8 * shots / frame_avg_s / 1e9
    shots_per_frame_launch = shots * args.steps / max(1, frame_launches)
    smem_peak = _native.measure_smem_peak(local) / 1e9
    int_peaks = _native.measure_int_peaks(local)
    # Noise kernel: Philox calls per launch (the contract's expected count) / its CUDA-event time, against the
    # Philox probe's calls/s on the same GPU.
    philox_per_shot = noise_philox_calls(text)
    noise_avg_s = statistics.mean(noise_ms) / 1e3 * args.steps / max(1, noise_launches)
    shots_per_noise_launch = shots * args.steps / max(1, noise_launches)
    noise_achieved = philox_per_shot * shots_per_noise_launch / noise_avg_s if noise_launches else None
    link = measure_link(local)
    # Transpose: reads the detector-major rows (16 bytes per row per 128 shots) and writes the shot-major rows.
    tr_ms = statistics.mean(t - f - z for t, f, z in zip(step_ms, frame_ms, noise_ms))
    tr_bytes = shots * ((D + O) / 8 + drow + orow)
    hbm_peak = _measured_hbm_peak()

    configs = run_configs(args, local) if args.config_steps > 0 else None
    writes = run_sample_write(args, local, text) if args.write_steps > 0 else None
    batched = run_batched(args, local) if args.batched else None
    serving = run_serving_legs(args, local) if args.serve_seconds > 0 else None
    m2d = run_m2d(args, local, text) if args.m2d_steps > 0 else None
    dem = run_dem(args, local) if args.dem_steps > 0 else None
    feed = run_feed(args, local, text) if args.feed_steps > 0 else None

    if rank == 0:
        cb_value, cb_s, cb_shots = cpu_baseline(text, D, O, args.cpu_chunk, os.cpu_count() or 1, args.cpu_seconds,
                                                3 * args.cpu_seconds)
        # The same port on one core (the reference CLI's `stim detect` is single-threaded).
        cb1_value, cb1_s, cb1_shots = cpu_baseline(text, D, O, 4096, 1, min(args.cpu_seconds, 3.0),
                                                   3 * min(args.cpu_seconds, 3.0))
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * dev_s / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u32 bitwise",
            "data": "synthetic (reference-generated circuit, seeded shots)",
            "config": {"workload": "surface_code:rotated_memory_z d=25 r=25 p=1e-3", "shots_per_step": shots,
                       "detectors": D, "observables": O, "launch_shape": sampler.launch_shape(),
                       "l2": "outputs (2 GB/step) exceed L2; a 256 MiB buffer is also rewritten between steps",
                       "parallelism": f"replicas by shot range x{world}"},
            "p50_ms": statistics.median(step_ms), "p99_ms": sorted(step_ms)[-1],
            "kernel_ms": {"frame": statistics.mean(frame_ms), "noise": statistics.mean(noise_ms),
                          "transpose": tr_ms},
            "wall_ms_per_step": 1e3 * wall / args.steps,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": shots * (drow + orow),
                    "ms_per_step": 1e3 * e2e_s / max(1, len(e2e_times)),
                    "p50_ms": 1e3 * statistics.median(e2e_times) if e2e_times else None,
                    "p99_ms": 1e3 * _nearest_rank(e2e_times, 0.99) if e2e_times else None,
                    "max_ms": 1e3 * max(e2e_times) if e2e_times else None,
                    "calls": len(e2e_times),
                    "api": "CompiledDetectorSampler.sample(shots, bit_packed=True, separate_observables=True, "
                           "dets_out=, obs_out=) into reused page-locked host numpy arrays",
                    "pageable": {"value": page_value, "unit": UNIT,
                                 "p50_ms": 1e3 * statistics.median(page_times) if page_times else None,
                                 "p99_ms": 1e3 * _nearest_rank(page_times, 0.99) if page_times else None,
                                 "max_ms": 1e3 * max(page_times) if page_times else None,
                                 "api": "the same call into reused pageable numpy arrays"},
                    "link": dict(link, note="cudaMemcpyAsync of 2 GiB between HBM and page-locked host memory, "
                                                   "best of 5, measured in this run"),
                    "link_bound_ms": 1e3 * shots * (drow + orow) / (link["d2h_gbs"] * 1e9),
                    "device_ms": {k: statistics.mean(p[k] for p in e2e_parts) for k in
                                  ("frame_ms", "noise_ms", "transpose_ms", "copy_ms", "total_ms")}
                    if e2e_parts else None,
                    "tail": e2e_tail(e2e_times, e2e_parts)},
            "gpu_launches": launches,
            "roofline": {"bound": "smem", "achieved": achieved_gbs, "peak": smem_peak, "unit": "GB/s",
                         "frac": achieved_gbs / smem_peak,
                         "traffic": FRAME_DRAM_BYTES_PER_SHOT * shots_per_frame_launch,
                         "traffic_note": "DRAM bytes per frame-kernel launch (ncu per-shot figure x shots per "
                                         "launch); shared memory, not DRAM, bounds this kernel",
                         "basis": f"{acc_bits:.0f} frame-bit accesses/shot x {shots} shots per frame-kernel launch; "
                                  "peak = project shared-memory probe (gfs_measure_smem_peak)"},
            "roofline_noise": {"bound": "integer issue (Philox4x32-10)", "achieved": noise_achieved,
                               "peak": int_peaks["philox_per_s"], "unit": "Philox calls/s",
                               "frac": noise_achieved / int_peaks["philox_per_s"] if noise_achieved else None,
                               "philox_calls_per_shot": philox_per_shot, "ms_per_launch": 1e3 * noise_avg_s,
                               "shots_per_launch": shots_per_noise_launch,
                               "basis": "expected Philox calls of the random-bit contract per shot (segments of "
                                        "16 units x 128 shots: first gap draw, then per hit a choice draw for "
                                        "DEPOLARIZE1/2 and a gap draw, 4 draws per call) x shots per noise-kernel "
                                        "launch / its CUDA-event time; peak = project Philox probe "
                                        "(gfs_measure_int_peaks)"},
            "lop3_peak_ops_per_s": int_peaks["lop3_per_s"],
            "roofline_transpose": {"bound": "hbm", "achieved": tr_bytes / (tr_ms / 1e3) / 1e9, "peak": hbm_peak,
                                   "unit": "GB/s", "frac": tr_bytes / (tr_ms / 1e3) / 1e9 / hbm_peak,
                                   "basis": "detector-major rows read + shot-major rows written per step; "
                                            "peak = measured HBM copy bandwidth"},
            "cpu_baseline": {"value": cb_value, "unit": UNIT, "cores": os.cpu_count() or 1, "kind": "port",
                             "sample": f"{cb_shots} shots of the same workload in {args.cpu_chunk}-shot calls "
                                       f"({cb_s:.1f} s), oracle port (64-bit words, pthreads)",
                             "one_core": {"value": cb1_value, "unit": UNIT, "cores": 1,
                                          "sample": f"{cb1_shots} shots in 4096-shot calls ({cb1_s:.1f} s)"}},
            "clocks": clk,
            "configs": configs,
            "sample_write": writes,
            "batched": batched,
            "serving": serving,
            "m2d": m2d,
            "dem": dem,
            "feed": feed,
        }
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


def _pinned(shape):
    import torch

    return torch.empty(shape, dtype=torch.uint8, pin_memory=True).numpy()


def _median_ms(fn, steps):
    """Median wall time of `steps` calls of fn after E2E_WARMUP untimed calls (which touch the arrays' pages)."""
    times = []
    with quiet_gc():
        for k in range(E2E_WARMUP + steps):
            t0 = time.perf_counter()
            fn()
            if k >= E2E_WARMUP:
                times.append(time.perf_counter() - t0)
    return 1e3 * statistics.median(times)


def run_m2d(args, local, text):
    """Measurements to detection events (compile_m2d_converter().convert) on the main workload: the
    measurement sampler's records of `--shots` shots, converted from host arrays into host arrays reused across
    calls (host->device and device->host copies inside the timed region; chunks pipelined so that one chunk's
    copies overlap the next one's).  Headline with page-locked arrays, the same call on pageable numpy arrays
    beside it.  Reports detection-event Gbit/s out and measurement Gbit/s in, and checks the result against the
    detection sampler with the same seed."""
    import numpy as np

    import stim_gb300

    shots = args.shots
    c = stim_gb300.Circuit(text)
    D, O, M = c.num_detectors, c.num_observables, c.num_measurements
    meas_page = c.compile_sampler(seed=args.seed, device=local).sample(shots, bit_packed=True)
    conv = c.compile_m2d_converter(device=local)
    meas = _pinned(meas_page.shape)
    meas[...] = meas_page
    d, o = _pinned((shots, (D + 7) // 8)), _pinned((shots, (O + 7) // 8))

    def call(mm, dd, oo):
        conv.convert(measurements=mm, separate_observables=True, append_observables=False, bit_packed=True,
                     dets_out=dd, obs_out=oo)

    ms = _median_ms(lambda: call(meas, d, o), args.m2d_steps)
    dp, op = np.empty_like(d), np.empty_like(o)
    ms_page = _median_ms(lambda: call(meas_page, dp, op), args.m2d_steps)
    want_d, want_o = c.compile_detector_sampler(seed=args.seed, device=local).sample(
        shots, separate_observables=True, bit_packed=True)
    return {"workload": f"{shots} shots of {M} measurement bits (the measurement sampler's records) -> {D} "
                        f"detectors + {O} observables, page-locked host arrays in and out",
            "gbits": shots * (D + O) / (ms / 1e3) / 1e9, "meas_gbits_in": shots * M / (ms / 1e3) / 1e9,
            "ms": ms, "h2d_bytes": int(meas.nbytes), "d2h_bytes": int(d.nbytes + o.nbytes),
            "pageable": {"gbits": shots * (D + O) / (ms_page / 1e3) / 1e9, "ms": ms_page},
            "equals_detection_sampler": bool(np.array_equal(d, want_d) and np.array_equal(o, want_o)
                                             and np.array_equal(dp, want_d) and np.array_equal(op, want_o))}


def run_dem(args, local):
    """Detector-error-model sampling (DetectorErrorModel.compile_sampler().sample) of the main workload's
    model (the reference's analyze_errors of the same circuit: 326,897 error mechanisms), `--shots` shots
    into reused host arrays, device->host copies inside the timed region (pipelined with the next chunk's
    kernels); page-locked arrays, pageable beside them."""
    import numpy as np

    import stim_gb300
    from stim_gb300 import workloads

    shots = args.shots
    dem = stim_gb300.DetectorErrorModel(workloads.dem_d25_text())
    s = dem.compile_sampler(seed=args.seed, device=local)
    D, O = dem.num_detectors, dem.num_observables
    d, o = _pinned((shots, (D + 7) // 8)), _pinned((shots, (O + 7) // 8))
    ms = _median_ms(lambda: s.sample(shots, bit_packed=True, dets_out=d, obs_out=o), args.dem_steps)
    dp, op = np.empty_like(d), np.empty_like(o)
    ms_page = _median_ms(lambda: s.sample(shots, bit_packed=True, dets_out=dp, obs_out=op), args.dem_steps)
    return {"workload": f"{shots} shots of the d=25 r=25 p=1e-3 detector error model ({dem.num_errors} error "
                        f"mechanisms, {D} detectors, {O} observables), page-locked host arrays out",
            "gbits": shots * (D + O) / (ms / 1e3) / 1e9, "ms": ms, "d2h_bytes": int(d.nbytes + o.nbytes),
            "pageable": {"gbits": shots * (D + O) / (ms_page / 1e3) / 1e9, "ms": ms_page},
            "mean_detection_events_per_shot": float(np.unpackbits(d[:4096], axis=1).sum() / 4096)}


def run_feed(args, local, text):
    """The decoder feed (CompiledDetectorSampler.sample_for_decoder, the sampling half of sinter's
    StimThenDecodeSampler) on the main workload: `--shots` shots with the first 40 detectors postselected, kept
    rows into reused page-locked host arrays; detection events counted and discarded shots dropped on the device."""
    import numpy as np

    import stim_gb300

    shots = args.shots
    c = stim_gb300.Circuit(text)
    D, O = c.num_detectors, c.num_observables
    s = c.compile_detector_sampler(seed=args.seed, device=local)
    mask = np.zeros((D + 7) // 8, dtype=np.uint8)
    mask[:5] = 0xFF
    d, o = _pinned((shots, (D + 7) // 8)), _pinned((shots, (O + 7) // 8))
    last = {}

    def call():
        kd, ko, disc, ev = s.sample_for_decoder(shots, postselection_mask=mask, dets_out=d, obs_out=o)
        last.update(kept=kd.shape[0], discards=disc, events=ev)

    ms = _median_ms(call, args.feed_steps)
    return {"workload": f"{shots} shots, detectors 0-39 postselected, kept rows into page-locked host arrays",
            "gbits_sampled": shots * (D + O) / (ms / 1e3) / 1e9, "ms": ms, "kept": last["kept"],
            "discards": last["discards"], "detection_events_per_shot": last["events"] / shots}


def run_configs(args, local):
    """The two smaller configurations of the metric, each through the device entry point (kernels only, CUDA
    events) and the public API into page-locked host arrays (device->host copies included), beside the
    reference's own CLI sampler and the oracle port on the host cores:
      plain CPU-runnable: surface_code:rotated_memory_z d=3 r=3 p=1e-3, 65,536 shots, seed 0;
      plain GPU: surface_code:rotated_memory_x d=11 r=11, p in {1e-3, 5e-3, 0}, 2^20 shots, seeds 0..3
      (p = 0 must give no detection events)."""
    import numpy as np
    import torch

    import stim_gb300
    from oracle.oracle import OracleCircuit
    from stim_gb300 import _native, workloads

    L = _native.lib()
    dev = f"cuda:{local}"
    exe = reference_stim()
    cases = [("surface_code:rotated_memory_z", 3, 0.001, 1 << 16, [0])]
    cases += [("surface_code:rotated_memory_x", 11, p, 1 << 20, [0, 1, 2, 3]) for p in (0.001, 0.005, 0.0)]
    out = []
    for family, d, p, shots, seeds in cases:
        text = workloads.code_circuit(family, d, d, p)
        c = stim_gb300.Circuit(text)
        D, O = c.num_detectors, c.num_observables
        drow, orow = (D + 7) // 8, (O + 7) // 8
        bits = shots * (D + O)
        dd = torch.empty((shots, drow), dtype=torch.uint8, device=dev)
        od = torch.empty((shots, orow), dtype=torch.uint8, device=dev)
        hd, ho = _pinned((shots, drow)), _pinned((shots, orow))
        dev_ms, e2e_ms, events = [], [], 0
        with quiet_gc():
            for seed in seeds:
                s = c.compile_detector_sampler(seed=seed, device=local)
                for k in range(E2E_WARMUP + max(3, args.config_steps)):
                    _native.check(L.gfs_sample_detections_device(s._h, shots, _native.BIT_PACKED, dd.data_ptr(), drow,
                                                                 od.data_ptr(), orow))
                    t = s.last_timings()
                    if k >= E2E_WARMUP:
                        dev_ms.append(t["frame_ms"] + t["noise_ms"] + t["transpose_ms"])
                s = c.compile_detector_sampler(seed=seed, device=local)
                for k in range(E2E_WARMUP + max(3, args.config_steps)):
                    t0 = time.perf_counter()
                    s.sample(shots, bit_packed=True, separate_observables=True, dets_out=hd, obs_out=ho)
                    if k >= E2E_WARMUP:
                        e2e_ms.append(1e3 * (time.perf_counter() - t0))
                if p == 0:
                    events += int(np.count_nonzero(hd)) + int(np.count_nonzero(ho))
        row = {"workload": f"{family} d={d} r={d} p={p:g}, {shots} shots, seeds {seeds}",
               "detectors": D, "observables": O,
               "value": bits / (statistics.median(dev_ms) / 1e3) / 1e9,
               "e2e": {"value": bits / (statistics.median(e2e_ms) / 1e3) / 1e9,
                       "p50_ms": statistics.median(e2e_ms), "p99_ms": max(e2e_ms),
                       "d2h_bytes_per_call": shots * (drow + orow)},
               "device_ms_p50": statistics.median(dev_ms)}
        if p == 0:
            row["zero_detection_events"] = events == 0  # every seed's last end-to-end output, all bytes
        if exe is not None:
            path = _circuit_file(text)
            try:
                cores = os.cpu_count() or 1
                all_s = statistics.median(time_reference_detect(exe, path, shots, cores, 50 + 10 * k)
                                          for k in range(3))
                one_s = time_reference_detect(exe, path, min(shots, 1 << 16), 1, 5)
            finally:
                os.unlink(path)
            row["reference_cpu"] = {"value": bits / all_s / 1e9, "cores": cores,
                                    "one_core": min(shots, 1 << 16) * (D + O) / one_s / 1e9,
                                    "kind": "reference", "unit": UNIT}
        oc = OracleCircuit(text)
        t0 = time.perf_counter()
        oc.sample(shots, 1, threads=os.cpu_count() or 1)
        row["port_cpu"] = {"value": bits / (time.perf_counter() - t0) / 1e9, "cores": os.cpu_count() or 1,
                           "kind": "port", "unit": UNIT}
        out.append(row)
    return out


def run_sample_write(args, local, text):
    """sample_write (the result file formats, made on the device) of the main workload into /dev/null, so that the
    figure is the library's own rate, not the disk's: detection events with the observables appended, per format,
    median of --write-steps calls.  01 writes one byte per bit, so it samples a quarter of the shots."""
    import stim_gb300

    c = stim_gb300.Circuit(text)
    D, O = c.num_detectors, c.num_observables
    s = c.compile_detector_sampler(seed=args.seed, device=local)
    out = {}
    for fmt in ("b8", "r8", "hits", "dets", "ptb64", "01"):
        shots = args.write_shots // 4 if fmt == "01" else args.write_shots
        ms = _median_ms(lambda: s.sample_write(shots, filepath="/dev/null", format=fmt, append_observables=True),
                        args.write_steps)
        out[fmt] = {"shots": shots, "ms": ms, "gbits": shots * (D + O) / (ms / 1e3) / 1e9}
    return {"workload": f"sample_write of d=25 r=25 p=1e-3 detection events + observable, to /dev/null",
            "formats": out}


def run_batched(args, local):
    """The many-circuit workload: 256 rotated surface-code circuits (d in 3..17, rounds = d, p log-uniform in
    [1e-4, 1e-2], shots log-uniform in [2^12, 2^20], one seed each) sampled (a) in one batched persistent
    launch replayed as a CUDA graph and (b) as 256 sequential single-circuit calls, both into device
    buffers.  Aggregate detection-event Gbit/s for each, and p50/p99 of the batched call."""
    import torch

    import stim_gb300
    from stim_gb300 import _native, workloads

    wl = workloads.batched_workload(num_circuits=args.batch_circuits, seed=2024)
    circuits = [stim_gb300.Circuit(w["text"]) for w in wl]
    shots = [w["shots"] for w in wl]
    bits = sum(n * (c.num_detectors + c.num_observables) for n, c in zip(shots, circuits))
    dev = f"cuda:{local}"
    dbufs = [torch.empty((n, (c.num_detectors + 7) // 8), dtype=torch.uint8, device=dev) for n, c in zip(shots, circuits)]
    obufs = [torch.empty((n, (c.num_observables + 7) // 8), dtype=torch.uint8, device=dev) for n, c in zip(shots, circuits)]
    dptr, dstr = [b.data_ptr() for b in dbufs], [b.shape[1] for b in dbufs]
    optr, ostr = [b.data_ptr() for b in obufs], [b.shape[1] for b in obufs]

    batch = stim_gb300.BatchSampler([c.compile_detector_sampler(seed=w["seed"], device=local)
                                     for c, w in zip(circuits, wl)])
    tune_ms = batch.autotune(shots)
    for _ in range(args.warmup):
        batch.sample_device(shots, dptr, dstr, optr, ostr)
    torch.cuda.synchronize()
    # Both forms are timed the same way: host wall clock around a call that returns with its work complete
    # (sample_device synchronizes; the sequential loop is followed by a synchronize).  The batched call's CUDA
    # events (graph replay, and its frame-kernel part) are reported beside it.
    wall, times, frame = [], [], []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        batch.sample_device(shots, dptr, dstr, optr, ostr)
        wall.append(time.perf_counter() - t0)
        t = batch.last_timings()
        times.append(t["total_ms"])
        frame.append(t["frame_ms"])
    t = batch.last_timings()

    plain = [c.compile_detector_sampler(seed=w["seed"], device=local) for c, w in zip(circuits, wl)]
    L = _native.lib()

    def sequential():
        for s, n, dp, ds, op, os_ in zip(plain, shots, dptr, dstr, optr, ostr):
            _native.check(L.gfs_sample_detections_device(s._h, n, _native.BIT_PACKED, dp, ds, op, os_))

    for _ in range(args.warmup):
        sequential()
    torch.cuda.synchronize()
    seq = []
    for _ in range(max(1, args.steps // 2)):
        t0 = time.perf_counter()
        sequential()
        torch.cuda.synchronize()
        seq.append(time.perf_counter() - t0)
    seq_s = statistics.median(seq)
    bat_s = statistics.median(wall)
    return {
        "workload": f"{len(wl)} rotated surface-code memory-Z circuits, d in 3..17 (rounds = d), p log-uniform "
                    "[1e-4, 1e-2], shots log-uniform [2^12, 2^20], generator seed 2024",
        "total_shots": sum(shots), "total_bits": bits,
        "batched_gbits": bits / bat_s / 1e9, "batched_p50_ms": 1e3 * statistics.median(wall),
        "batched_p99_ms": 1e3 * max(wall), "batched_graph_ms": statistics.median(times),
        "batched_frame_ms": statistics.median(frame),
        "sequential_gbits": bits / seq_s / 1e9, "sequential_ms": 1e3 * seq_s,
        "speedup": seq_s / bat_s, "timing": "host wall clock around a completed call, both forms (median)",
        "launch_shape": batch.launch_shape(), "autotune_best_frame_ms": tune_ms,
        "graph_launches": t["graph_launches"], "graph_builds": t["graph_builds"],
        "note": "device-resident outputs; batched = one persistent frame-kernel launch + per-circuit transposes "
                "in one CUDA graph; sequential = one gfs_sample_detections_device call per circuit",
    }


def run_serving_legs(args, local):
    """The serving configuration (Poisson --serve-rate req/s for --serve-seconds s) and a sweep of lower arrival
    rates (--serve-sweep, --serve-sweep-seconds each) showing latency below saturation."""
    main = run_serving(args, local, args.serve_rate, args.serve_seconds)
    sweep = []
    for rate in [float(x) for x in args.serve_sweep.split(",") if x.strip()]:
        if args.serve_sweep_seconds > 0:
            sweep.append(run_serving(args, local, rate, args.serve_sweep_seconds))
    main["sweep"] = [{k: r[k] for k in ("rate", "seconds", "requests", "gbits", "offered_gbits", "p50_ms", "p99_ms",
                                        "wall_s", "counters")} for r in sweep]
    bounded = [r["rate"] for r in sweep if r["p99_ms"] is not None and r["p99_ms"] < 1000.0]
    main["highest_swept_rate_with_p99_under_1s"] = max(bounded) if bounded else None
    return main


def run_serving(args, local, rate, seconds):
    """Open-loop serving: Poisson arrivals at --serve-rate requests/s for --serve-seconds, each request a
    generated code circuit (repetition d 3..51, rotated surface X/Z d 3..21, color d 3..15; rounds = d;
    p log-uniform [1e-4, 1e-2] on a 16-per-decade grid; shots log-uniform [2^10, 2^22]; own seed),
    submitted to the continuous-batching server with bit-packed results in device memory.  Latency is
    measured from each request's scheduled arrival to its completion, so client back-pressure (a full
    result arena) counts against it."""
    import collections

    import torch

    import stim_gb300
    from stim_gb300 import workloads

    wl = workloads.serving_workload(rate=rate, seconds=seconds, seed=7)
    texts, dims = {}, {}
    for w in wl:
        key = (w["family"], w["distance"], w["p"])
        if key not in texts:
            t = workloads.code_circuit(w["family"], w["distance"], w["distance"], w["p"])
            c = stim_gb300.Circuit(t)
            texts[key] = t
            dims[key] = (c.num_detectors, c.num_observables)
    arena_bytes = args.serve_arena_gb << 30
    arena = torch.empty(arena_bytes, dtype=torch.uint8, device=f"cuda:{local}")
    base = arena.data_ptr()
    server = stim_gb300.Server(device=local, hbm_budget=args.serve_hbm_gb << 30, max_chunk_shots=1 << 18)
    for key, t in texts.items():  # warm the device-side circuit cache
        D, O = dims[key]
        server.submit_device(t, 0, seed=0, dets_ptr=base, dets_stride=(D + 7) // 8).result()
    outstanding = collections.deque()  # (request, start, size): results held in the arena, oldest first
    head = 0
    lat = []
    bits = 0

    def retire(block):
        while outstanding and (block or outstanding[0][0].done()):
            r = outstanding.popleft()[0]
            r.result()
            lat.append(r.latency_ms + r._client_delay_ms)
            block = False

    def alloc(size):
        # Ring allocation in the result arena; waits for the oldest request when there is no room.  The
        # strict comparisons keep head != tail while the ring is wrapped.
        nonlocal head
        if size >= arena_bytes:
            raise ValueError("request larger than the result arena")
        while True:
            if not outstanding:
                head = 0
            if not outstanding or head >= outstanding[0][1]:
                tail = outstanding[0][1] if outstanding else arena_bytes
                if head + size <= arena_bytes:
                    start = head
                    break
                if size < tail and outstanding:
                    start = 0
                    break
            elif head + size < outstanding[0][1]:
                start = head
                break
            retire(True)
        head = start + size
        return start

    t0 = time.perf_counter()
    for w in wl:
        key = (w["family"], w["distance"], w["p"])
        D, O = dims[key]
        drow, orow = (D + 7) // 8, (O + 7) // 8
        size = (w["shots"] * (drow + orow) + 255) & ~255
        now = time.perf_counter() - t0
        if now < w["t"]:
            time.sleep(w["t"] - now)
        start = alloc(size)
        sub = time.perf_counter() - t0
        r = server.submit_device(texts[key], w["shots"], seed=w["seed"], dets_ptr=base + start, dets_stride=drow,
                                 obs_ptr=base + start + w["shots"] * drow, obs_stride=orow)
        r._client_delay_ms = max(0.0, 1e3 * (sub - w["t"]))
        outstanding.append((r, start, size))
        bits += w["shots"] * (D + O)
        retire(False)
    while outstanding:
        retire(True)
    wall = time.perf_counter() - t0
    st = server.stats()
    counters = server.counters()
    server.close()
    lat.sort()
    offered = sum(w["shots"] * sum(dims[(w["family"], w["distance"], w["p"])]) for w in wl) / seconds
    return {
        "workload": f"Poisson {rate:g} req/s for {seconds:g} s; repetition d3-51, surface "
                    "X/Z d3-21, color d3-15, rounds = d, p log-uniform [1e-4, 1e-2] (16 per decade), shots "
                    "log-uniform [2^10, 2^22], per-request seed; bit-packed results in device memory",
        "rate": rate, "seconds": seconds, "counters": counters,
        "requests": len(wl), "distinct_circuits": len(texts),
        "gbits": bits / wall / 1e9, "offered_gbits": offered / 1e9,
        "p50_ms": lat[len(lat) // 2] if lat else None,
        "p99_ms": lat[min(len(lat) - 1, int(math.ceil(0.99 * len(lat))) - 1)] if lat else None,
        "wall_s": wall, "batches": st["batches"], "chunks_per_batch": st["chunks_per_batch"],
        "cache_hits": st["cache_hits"], "cache_misses": st["cache_misses"],
        "latency_basis": "scheduled arrival to completion (server completion time plus client submit delay)",
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--shots", type=int, default=1 << 20)
    ap.add_argument("--e2e-steps", type=int, default=100)
    ap.add_argument("--cpu-chunk", type=int, default=1 << 16)
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--ref-shots", type=int, default=1 << 20)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--shape", default="")
    ap.add_argument("--noise-mode", type=int, default=-1, help="-1 automatic, 0 inline, 1 hit lists")
    ap.add_argument("--autotune", type=int, default=1)
    ap.add_argument("--batched", type=int, default=1)
    ap.add_argument("--write-steps", type=int, default=3, help="timed sample_write calls per result format")
    ap.add_argument("--write-shots", type=int, default=1 << 20)
    ap.add_argument("--config-steps", type=int, default=5, help="timed calls per seed of the d=3 and d=11 legs")
    ap.add_argument("--m2d-steps", type=int, default=5)
    ap.add_argument("--dem-steps", type=int, default=5)
    ap.add_argument("--feed-steps", type=int, default=3)
    ap.add_argument("--batch-circuits", type=int, default=256)
    ap.add_argument("--serve-seconds", type=float, default=60.0)
    ap.add_argument("--serve-rate", type=float, default=2000.0)
    ap.add_argument("--serve-sweep", default="250,500,1000", help="arrival rates (req/s) of the latency sweep")
    ap.add_argument("--serve-sweep-seconds", type=float, default=8.0)
    ap.add_argument("--serve-arena-gb", type=int, default=48)
    ap.add_argument("--serve-hbm-gb", type=int, default=16)
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
