#!/usr/bin/env python
"""Benchmark of the GB300 step loop: particle-steps/s of the mixed-precision
batched form and of the plain FP64 drop-in on one workload, through
libmavi_cuda.so.

Default workload (one GPU): 512 independent 2D Lennard-Jones replicas of
uneven N (log-uniform in [1000, 65536], 7,871,648 particles in total),
density 0.6, rigid/periodic walls x rectangular/circular geometry, Maxwell
velocities at T in [0.3, 1.0], velocity Verlet dt = 1e-3, all replicas behind
one handle (see mavi.jl_gb300/workloads.py). `--workload harm_262144` (one
large soft-disk system), `lj_4194304` and `rings_64` are the other shapes. A
"step" is one whole step of the step loop (chunk rebuild -> pair forces ->
integration -> walls) of every replica.

Timing: W untimed warm-up steps, then K steps; before every timed step a
256 MiB buffer is written (L2 flush), then one step runs as a CUDA graph whose
first and last launch carry CUDA events on the library's own stream; the value
is N * K / (sum of those device times). Per-kernel device times come from the
same replays. `e2e` is measured through the C ABI with pinned host buffers,
host-timed: upload state -> one step -> download state on one handle; for a
batched workload the batch runs as eight handles of consecutive replicas
whose copies and steps overlap (uploads, steps and queued downloads of all,
then a wait on each), and the single-handle figure is kept beside it.

--impl reference: the reference's algorithm on the host cores (the CPU
restatement in oracle/, OpenMP over chunk columns like the reference's
Threaded mode), on the same workload, a bounded number of steps.

Multi-GPU (torchrun): replicas only. A batched workload of R replicas per GPU
becomes R x world replicas (the same seeded generator, continued), split
between the ranks by particle count (replicas.shard_replicas; weak scaling, no
data-path collective); a single-system workload runs one copy per rank.
value = all ranks' particle-steps / max-over-ranks time.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
import __graft_entry__ as graft  # noqa: E402

GATHER_NAMES = {0: "staged", 1: "global", 2: "columns", 3: "tiles", 4: "tiles_queue", 5: "lanes2", 6: "lanes4", 7: "split"}
METRIC = "particle-steps/s on 1 GB300, mixed+batched vs plain FP64, at ≤1e-5 rel force err"
UNIT = "particle-steps/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--workload", default="lj_batch_512")
    ap.add_argument("--gather", default="auto",
                    help="pair gather of the mixed form (auto: the autotuner's choice; a fixed one for profiling "
                         "runs, where serialised launches make the autotuner's timings meaningless)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--accuracy-steps", type=int, default=500,
                    help="steps of the energy-drift / g(r) comparison of the two forms (0: skip)")
    return ap.parse_args()


def dist_info():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def rel_force_err(f, ref):
    rms = math.sqrt(float(np.mean(np.sum(ref * ref, axis=1))))
    return float(np.max(np.linalg.norm(f - ref, axis=1)) / max(rms, 1e-300))


class Clocks:
    """nvidia-smi sampling during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        self.proc.wait()
        rows = []
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                rows.append((float(f[1]), float(f[2]), f[5], f[6], f[7], f[8]))
            except ValueError:
                continue
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[2 + k].lower() == "active"})
        loaded = [r[0] for r in rows if r[0] > 0.5 * r[1]] or [r[0] for r in rows]
        return {"sm_mhz": statistics.median(loaded), "sm_max_mhz": max(r[1] for r in rows), "reasons": reasons,
                "samples": len(rows)}


def launches_per_step(step_kind, abi, precision):
    rebin = 3   # scan, scatter, deterministic per-chunk order + permutation
    body = {abi.MAVI_STEP_NEWTON: 2, abi.MAVI_STEP_OVERDAMPED: 1, abi.MAVI_STEP_SZABO: 1, abi.MAVI_STEP_RTP: 1,
            abi.MAVI_STEP_RINGS: 3}[step_kind]   # rings: pair pass, ring terms + update + histogram, polarisation
    if step_kind == abi.MAVI_STEP_RINGS and precision == "fp64":
        body += 1                                # ring areas in the reference's operation order
    return rebin + body


def measured_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except OSError:
        return {}


class Runner:
    """One workload behind one handle: a single System, or a list of systems
    advanced together as a SystemBatch (replicas in the same launches)."""

    def __init__(self, mg, obj, step, precision):
        self.mg = mg
        self.step = step
        self.precision = precision
        if isinstance(obj, (list, tuple)):
            self.systems = list(obj)
            self.batch = mg.SystemBatch(self.systems, step)
            self.handle = self.batch.handle
        else:
            self.systems = [obj]
            self.batch = None
            self.handle = obj._ensure(step.kind if step is not None else None)
        self.kind = self.handle.step_kind
        self.num_slots = int(sum(s.num_slots for s in self.systems))

    @property
    def first(self):
        return self.systems[0]

    def forces(self):
        return self.handle.forces(False)

    def stats(self):
        return self.handle.stats()

    def host_state(self):
        """Concatenated host arrays in the layout of mavi_create."""
        st = [s.state for s in self.systems]
        pos = np.concatenate([x.pos.reshape(-1) for x in st])
        vel = None
        if st[0].kind == self.mg.abi.MAVI_STATE_SECOND_LAW and st[0].vel is not None:
            vel = np.concatenate([x.vel.reshape(-1) for x in st])
        pol = None
        if st[0].pol_array() is not None:
            pol = np.concatenate([x.pol_array() for x in st])
        return pos, vel, pol

    def oracle_forces(self, orc, nthreads):
        out = []
        for s in self.systems:
            o = orc.from_system(s, nthreads=nthreads, step_kind=self.kind)
            out.append(o.forces(orc.THREADED if nthreads > 1 else orc.SEQUENTIAL))
            o.close()
        return np.concatenate(out)

    def close(self):
        if self.batch is not None:
            self.batch.close()
        else:
            self.systems[0].close()


def time_form(mg, runner, K, W, flush, torch):
    """Device-timed steps of one workload; returns a dict of measurements."""
    abi = mg.abi
    h = runner.handle
    lib, hd = h.lib, h.handle
    h.check(lib.mavi_step(hd, W), "warm-up")

    def timed(mode, k):
        # mode 2: one event pair around each step's graph (nothing between its
        # kernels); mode 1: event pairs around every kernel group as well
        h.check(lib.mavi_profile_enable(hd, mode), "profile")
        h.check(lib.mavi_step(hd, 1), "profiled warm-up")      # captures the graph of this mode
        h.check(lib.mavi_profile_enable(hd, mode), "profile reset")
        torch.cuda.synchronize()
        ms = []
        for _ in range(k):
            flush()
            torch.cuda.synchronize()
            h.check(lib.mavi_step(hd, 1), "timed step")
            p = abi.MaviProfile()
            lib.mavi_profile_read(hd, C.byref(p))
            ms.append(p.last_step_ms)
        torch.cuda.synchronize()
        p = abi.MaviProfile()
        lib.mavi_profile_read(hd, C.byref(p))
        return ms, p

    step_ms, _ = timed(2, K)
    kb = min(K, 100)
    _, p = timed(1, kb)
    h.check(lib.mavi_profile_enable(hd, 0), "profile off")
    kinds = {abi.MAVI_KERNEL_NAMES[k]: {"ms": p.ms[k] * K / kb, "launches": int(p.launches[k]) * K // kb}
             for k in range(abi.MAVI_NUM_KERNEL_KINDS) if p.launches[k]}
    return {"total_ms": float(sum(step_ms)), "step_ms": step_ms, "kinds": kinds,
            "launches_per_step": launches_per_step(h.step_kind, abi, runner.precision),
            "kernel_breakdown_steps": kb}


def e2e_form(mg, runner, K, torch):
    """Through the C ABI with pinned host buffers: upload -> 1 step -> download."""
    h = runner.handle
    lib, hd = h.lib, h.handle
    dp = C.POINTER(C.c_double)
    bufs = []
    for a in runner.host_state():
        if a is None:
            bufs.append((None, None))
            continue
        t = torch.empty(a.shape, dtype=torch.float64, pin_memory=True)
        t.copy_(torch.from_numpy(np.ascontiguousarray(a)))
        bufs.append((t, C.cast(t.data_ptr(), dp)))
    (pt, pp), (vt, vp), (qt, qp) = bufs
    bi = sum(t.numel() * 8 for t, _ in bufs if t is not None)
    bo = bi
    for _ in range(3):
        h.check(lib.mavi_upload_state(hd, pp, vp, qp), "upload")
        h.check(lib.mavi_step(hd, 1), "step")
        h.check(lib.mavi_download_state(hd, pp, vp, qp), "download")
    t0 = time.perf_counter()
    for _ in range(K):
        h.check(lib.mavi_upload_state(hd, pp, vp, qp), "upload")
        h.check(lib.mavi_step(hd, 1), "step")
        h.check(lib.mavi_download_state(hd, pp, vp, qp), "download")
    dt = time.perf_counter() - t0
    return {"seconds": dt, "h2d": bi, "d2h": bo}


def accuracy_form(mg, runner, steps, samples, r_max, nbins):
    """From the workload's starting state (uploaded again): the total energy
    after every steps/samples steps, recorded on the device, and the
    pair-distance histogram of all replicas at the end."""
    abi = mg.abi
    h = runner.handle
    pos, vel, pol = runner.host_state()
    dp = C.POINTER(C.c_double)
    h.check(h.lib.mavi_upload_state(h.handle, pos.ctypes.data_as(dp),
                                    None if vel is None else vel.ctypes.data_as(dp),
                                    None if pol is None else pol.ctypes.data_as(dp)), "upload")
    out = {}
    if runner.kind == abi.MAVI_STEP_NEWTON:
        ke0, pe0 = h.energies(abi.MAVI_PE_STENCIL)
        ke, pe = h.energy_series(samples, steps // samples, abi.MAVI_PE_STENCIL)
        out["energy"] = np.vstack([ke0 + pe0, ke + pe])            # (samples + 1, replicas)
    else:
        h.step(steps)
    out["hist"] = h.pair_distribution(-1, r_max, nbins).astype(np.float64)
    return out


def ideal_pairs(runner, r_max, nbins):
    """Pairs an ideal gas at each replica's density puts in each annulus, summed."""
    edges = np.linspace(0.0, r_max, nbins + 1)
    shell = np.pi * (edges[1:] ** 2 - edges[:-1] ** 2)
    w = 0.0
    for sy in runner.systems:
        g = sy.space_cfg.geometry_cfg
        area = g.length * g.height if hasattr(g, "height") else math.pi * g.radius ** 2
        w += 0.5 * sy.num_slots ** 2 / area
    return shell * w


def accuracy(mg, runners, steps, samples):
    """Energy drift of both forms (velocity Verlet only: overdamped steps
    conserve nothing) and the L-inf difference of their g(r), from the same
    start; trajectories diverge chaotically, so the forms are compared on
    statistics. The g(r) bound is five standard deviations of the counting
    noise of two independent samples."""
    def chunk_side(sy):
        bb = sy.space_cfg.bounding_box()
        cc = getattr(sy.int_cfg, "chunks_cfg", None) or getattr(sy.int_cfg, "p_chunks_cfg")
        return min(bb.length / cc.num_cols, bb.height / cc.num_rows)

    r_max = math.floor(min(chunk_side(sy) for sy in runners["mixed"].systems) * 50) / 50
    nbins = max(1, int(round(r_max / 0.02)))
    res = {p: accuracy_form(mg, runners[p], steps, samples, r_max, nbins) for p in ("fp64", "mixed")}
    ideal = ideal_pairs(runners["mixed"], r_max, nbins)
    g = {p: res[p]["hist"] / ideal for p in res}
    noise = np.sqrt(res["fp64"]["hist"] + res["mixed"]["hist"]) / ideal
    out = {"steps": steps, "gr_linf": float(np.max(np.abs(g["mixed"] - g["fp64"]))),
           "gr_bins": {"r_max": r_max, "num_bins": nbins}}
    if "energy" in res["fp64"]:
        # counting noise of independent pair samples: meaningful for the
        # equilibrium (velocity-Verlet) workloads; bonded ring pairs and
        # driven overdamped states are not independent counts
        out["gr_5sigma_bound"] = float(np.max(5 * noise))
        out["gr_within_bound"] = bool(np.all(np.abs(g["mixed"] - g["fp64"]) <= 5 * noise + 1e-12))
    if "energy" in res["fp64"]:
        drift = {}
        for p in res:
            e = res[p]["energy"]
            drift[p] = (e[-1] - e[0]) / np.max(np.abs(e), axis=0)      # per replica
        out["energy_drift"] = {"fp64_max_abs": float(np.max(np.abs(drift["fp64"]))),
                               "mixed_max_abs": float(np.max(np.abs(drift["mixed"]))),
                               "max_abs_difference": float(np.max(np.abs(drift["mixed"] - drift["fp64"]))),
                               "samples": samples, "per": "replica, relative to its largest |E| in the series"}
    return out


def e2e_pipelined(mg, name, rank, world, K, torch, groups=8):
    """End to end through the C ABI for a batched workload, the way a host runs
    independent replica groups side by side: the batch as `groups` handles of
    consecutive replicas (about equal particle counts), each on its own
    stream. Every step, group by group: wait for the group's previous
    download (mavi_synchronize: the host then holds that step's result),
    upload its state from page-locked memory, step once and queue its
    download (mavi_download_state_async). A group waits only for its own
    previous step, so one group's copies overlap the other groups' steps
    across step boundaries too, and uploads overlap downloads (the host link
    moves both directions at once); after the last step every group is
    awaited inside the timed region."""
    systems, step = workload_share(name, "mixed", rank, world)
    cum = np.cumsum([s.num_slots for s in systems])
    cuts = [0] + [int(np.searchsorted(cum, cum[-1] * g / groups)) + 1 for g in range(1, groups)] + [len(systems)]
    runs = [Runner(mg, systems[a:b], step, "mixed") for a, b in zip(cuts[:-1], cuts[1:]) if b > a]
    dp = C.POINTER(C.c_double)
    sets = []
    nbytes = 0
    for r in runs:
        bufs = []
        for a in r.host_state():
            if a is None:
                bufs.append((None, None))
                continue
            t = torch.empty(a.shape, dtype=torch.float64, pin_memory=True)
            t.copy_(torch.from_numpy(np.ascontiguousarray(a)))
            bufs.append((t, C.cast(t.data_ptr(), dp)))
            nbytes += t.numel() * 8
        sets.append(bufs)

    def one_step():
        for r, ((_, pp), (_, vp), (_, qp)) in zip(runs, sets):
            h = r.handle
            h.synchronize()   # this group's previous step is back on the host
            h.check(h.lib.mavi_upload_state(h.handle, pp, vp, qp), "upload")
            h.check(h.lib.mavi_step(h.handle, 1), "step")
            h.check(h.lib.mavi_download_state_async(h.handle, pp, vp, qp), "download")

    def wait_all():
        for r in runs:
            r.handle.synchronize()

    for _ in range(3):
        one_step()
    wait_all()
    t0 = time.perf_counter()
    for _ in range(K):
        one_step()
    wait_all()
    dt = time.perf_counter() - t0
    n = sum(r.num_slots for r in runs)
    for r in runs:
        r.close()
    return {"value": n * K / dt, "h2d": nbytes, "d2h": nbytes, "groups": len(runs)}


def algorithmic_bytes(kind, precision, step_kind, abi, has_vel):
    """Algorithmic HBM bytes per particle of one launch of each kernel kind:
    the unique data the launch must read and write once (neighbour reads hit
    in L1/L2 and are not counted)."""
    mixed = precision == "mixed"
    off = 8 if mixed else 0          # int2 fixed-point chunk offset
    vel = 16 if has_vel else 0
    if kind == "force":
        if step_kind == abi.MAVI_STEP_NEWTON:
            # pass 1: r x, v, uid, rep, cell, (off) ; w x', F(t), (off')
            p1 = (16 + 16 + 4 + 4 + 4 + off) + (16 + (8 if mixed else 16) + off)
            # pass 2: r x', v, F(t), (off') ; w x, v, uid, rep, cell, (off)
            p2 = (16 + 16 + (8 if mixed else 16) + 4 + 4 + 4 + off) + (16 + 16 + 4 + 4 + 4 + off)
            return p1 + p2
        # final pass: r x, (v), uid, rep, cell, (off); w x, (v), uid, rep, cell, (off)
        return (16 + vel + 4 + 4 + 4 + off) + (16 + vel + 4 + 4 + 4 + off)
    if kind == "bin_sort":
        # r src_of, cell_at, key_of, x, (v), rep, (off); w x, (v), uid, rep, cell, slot_of, (off)
        return (4 + 4 + 4 + 16 + vel + 4 + off) + (16 + vel + 4 + 4 + 4 + 4 + off)
    if kind == "bin_scatter":
        return 4 + 4 + 4 + 4 + 4       # r cell, uid; w src_of, key_of, cell_at (the count atomics hit L2)
    if kind == "bin_scan":
        return 0                  # per chunk, not per particle (counted in the chunk term)
    if kind == "update" and step_kind == abi.MAVI_STEP_RINGS:
        # k_rings, user order: r slot_of, x, (off), cell, F; w x', (off'), cell' (user order
        # copy) and x', (off'), uid, rep, cell (sorted order, for the chunk update)
        f = 8 if mixed else 16
        return (4 + 16 + off + 4 + f) + (16 + off + 4) + (16 + off + 4 + 4 + 4)
    return 0


def ring_bytes(precision):
    """Per-ring bytes of the rings update (k_rings + k_ring_pol): ring replica,
    type, (cos, sin), velocity sum, area, angle; FP32 pairs in the mixed form."""
    v = 8 if precision == "mixed" else 16
    return (4 + 4 + v) + (v + 8) + (8 + 4 + 4 + v + v) + (8 + v)


# Flops per pair evaluation (sqrt and division count 1 each): HarmTrunc 16,
# LenJones 23, Szabo 14 (periodic minimum image included).
FLOPS_PER_PAIR = {0: 16, 1: 23, 2: 14, 3: 23, 4: 16}


def ncu_traffic(workload, precision, kernel):
    """DRAM bytes per launch of `kernel` from a committed ncu capture, or None."""
    try:
        d = json.load(open(os.path.join(ROOT, "profiles", "ncu_traffic.json")))
        e = d[workload][precision]
        return e["bytes_per_launch"] if e["kernel"] == kernel else None
    except (OSError, KeyError, ValueError):
        return None


def roofline(meas, n, precision, step_kind, abi, peaks, candidate_pairs, fma_peak, dyn_kind, has_vel,
             workload=None, num_rings=0):
    kinds = meas["kinds"]
    dom = max(kinds, key=lambda k: kinds[k]["ms"])
    avg_ms = kinds[dom]["ms"] / max(kinds[dom]["launches"], 1)
    bpp = algorithmic_bytes(dom, precision, step_kind, abi, has_vel)
    traffic_bytes = bpp * n
    if dom == "update" and step_kind == abi.MAVI_STEP_RINGS:
        traffic_bytes += ring_bytes(precision) * num_rings
    achieved = traffic_bytes / (avg_ms * 1e-3) / 1e9
    peak = peaks.get("hbm_gbs", 6800.0)
    rf = {"kernel": dom, "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
          "frac": achieved / peak, "traffic": ncu_traffic(workload, precision, dom),
          "algorithmic_bytes_per_launch": traffic_bytes,
          "avg_launch_ms": avg_ms, "peak_source": "measured" if "hbm_gbs" in peaks else "fallback"}
    if dom == "force" and candidate_pairs:
        flops_pair = FLOPS_PER_PAIR[dyn_kind]
        passes = 2 if step_kind == abi.MAVI_STEP_NEWTON else 1
        fl = 2 * candidate_pairs * flops_pair * passes   # each unordered pair is evaluated from both sides
        rf["fp_pipe"] = {"achieved_tflops": fl / (avg_ms * 1e-3) / 1e12,
                         "peak_tflops": fma_peak / 1e12 if fma_peak else None,
                         "frac": (fl / (avg_ms * 1e-3)) / fma_peak if fma_peak else None,
                         "pair_evaluations_per_launch": 2 * candidate_pairs * passes,
                         "flops_per_pair": flops_pair}
    return rf


def oracle_steps(orc, o, k, mode, kind, rng):
    """k oracle steps, drawing the step's noise on the host when it has any."""
    cnt = o.noise_count()
    o.step(k, mode, orc.noise_for(kind, cnt * k, rng) if cnt else None)


def cpu_baseline(mg, orc, runner, seconds, nthreads):
    """The reference's algorithm (oracle/, Threaded column split) on the host
    cores: whole replicas, in order, until about `seconds` of work."""
    mode = orc.THREADED if nthreads > 1 else orc.SEQUENTIAL
    done = 0
    total = 0.0
    used = 0
    steps = []
    rng = np.random.default_rng(0)
    for s in runner.systems:
        o = orc.from_system(s, nthreads=nthreads, step_kind=runner.kind)
        oracle_steps(orc, o, 1, mode, runner.kind, rng)                      # warm-up
        t0 = time.perf_counter()
        oracle_steps(orc, o, 1, mode, runner.kind, rng)
        one = time.perf_counter() - t0
        budget = max(seconds / max(len(runner.systems), 1), seconds - total) if used == 0 else seconds - total
        k = max(1, min(10000, int(budget / max(one, 1e-6))))
        noise = orc.noise_for(runner.kind, o.noise_count() * k, rng) if o.noise_count() else None
        t0 = time.perf_counter()
        o.step(k, mode, noise)
        total += time.perf_counter() - t0
        o.close()
        done += s.num_slots * k
        steps.append(k)
        used += 1
        if total >= seconds:
            break
    what = (f"{steps[0]} steps of the full workload (N={runner.num_slots})" if len(runner.systems) == 1 else
            f"{used} of {len(runner.systems)} replicas, {min(steps)}..{max(steps)} steps each")
    return {"value": done / total, "unit": UNIT, "cores": nthreads, "kind": "port",
            "sample": f"{what} after 1 warm-up step, oracle/mavi_oracle.c, "
                      f"{'Threaded column split' if nthreads > 1 else 'Sequencial'}"}


BATCHED = {"lj_batch_512": 512, "rings_64": 64}


MIXED_GATHER = "auto"   # --gather: the mixed form's pair gather


def workload_share(name, precision, rank=0, world=1):
    """The systems this rank advances (host side, no device handle yet).
    Batched workloads under torchrun: R x world replicas from the same seeded
    generator, this rank's share by particle count (replicas.shard_replicas:
    every rank derives the same partition alone; no exchange between ranks)."""
    from mavi_gb300 import replicas, workloads
    W = workloads.WORKLOADS
    if name in BATCHED and world > 1:
        obj, step = W[name](precision=precision, num_replicas=BATCHED[name] * world)
        mine = replicas.my_replicas([s.num_slots for s in obj], rank, world)
        obj = [obj[i] for i in mine]
    else:
        obj, step = W[name](precision=precision)
    if precision == "mixed" and MIXED_GATHER != "auto":
        for s in (obj if isinstance(obj, (list, tuple)) else [obj]):
            s.int_cfg.device.gather = MIXED_GATHER
    return obj, step


def build_workload(mg, name, precision, rank=0, world=1):
    obj, step = workload_share(name, precision, rank, world)
    return Runner(mg, obj, step, precision)


def run_reference_generic(args, mg, orc, workloads, nthreads):
    """The reference's algorithm (oracle/) on any workload: every replica
    advances one step per step, steps bounded to about a minute in total."""
    from mavi_gb300.system import get_step_function
    obj, step = workloads.WORKLOADS[args.workload](precision="fp64")
    systems = list(obj) if isinstance(obj, (list, tuple)) else [obj]
    kind = step.kind if step is not None else get_step_function(systems[0]).kind
    oracles = [orc.from_system(s, nthreads=nthreads, step_kind=kind) for s in systems]
    rng = np.random.default_rng(0)
    for o in oracles:
        oracle_steps(orc, o, max(args.warmup, 1), orc.THREADED, kind, rng)
    noise = [orc.noise_for(kind, o.noise_count(), rng) if o.noise_count() else None for o in oracles]
    n = sum(s.num_slots for s in systems)
    k = 0
    t0 = time.perf_counter()
    while k < args.steps:
        for o, z in zip(oracles, noise):   # one step of noise per replica, reused (timing only)
            o.step(1, orc.THREADED, z)
        k += 1
        if time.perf_counter() - t0 > 60.0:
            break
    dt = time.perf_counter() - t0
    for o in oracles:
        o.close()
    v = n * k / dt
    line = {"metric": METRIC, "value": v, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus, "steps": k,
            "warmup": args.warmup, "ms_per_step": dt / k * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": args.workload, "N": n, "replicas": len(systems)},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": nthreads, "kind": "port",
                             "sample": f"{k} steps of every replica; the reference is Julia, absent on this "
                                       f"machine: its algorithm restated in C (oracle/), Threaded column split"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def run_reference(args):
    rank, world, _ = dist_info()
    if rank != 0:
        return 0
    mg = graft.load_package()
    orc = graft.load_oracle()
    from mavi_gb300 import workloads
    nthreads = os.cpu_count() or 1
    if args.workload != "harm_262144":
        return run_reference_generic(args, mg, orc, workloads, nthreads)
    pos, L = workloads.harm_262144_initial()
    # same relaxation as the GPU arm, on the oracle (the reference's algorithm)
    sys_ = workloads.harm_system(pos, L, "fp64")
    o = orc.from_system(sys_, nthreads=nthreads, step_kind=workloads.OVERDAMPED.kind)
    o.step(200, orc.THREADED)
    relaxed, _, _ = o.state()
    o.close()
    s2 = workloads.harm_system(relaxed, L, "fp64")
    o = orc.from_system(s2, nthreads=nthreads, step_kind=workloads.OVERDAMPED.kind)
    o.step(max(args.warmup, 1), orc.THREADED)
    t1 = time.perf_counter()
    o.step(1, orc.THREADED)
    one = time.perf_counter() - t1
    k = max(1, min(args.steps, int(60.0 / max(one, 1e-6))))
    t0 = time.perf_counter()
    o.step(k, orc.THREADED)
    dt = time.perf_counter() - t0
    n = s2.num_slots
    v = n * k / dt
    line = {"metric": METRIC, "value": v, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus, "steps": k,
            "warmup": args.warmup, "ms_per_step": dt / k * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": args.workload, "N": n, "box": L, "chunks": [int(L // 2.0)] * 2,
                       "step": "overdamped", "dt": 1e-2},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": nthreads, "kind": "port",
                             "sample": f"{k} steps of the full workload; the reference is Julia, absent on this "
                                       f"machine: its algorithm restated in C (oracle/), Threaded column split"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def main():
    global MIXED_GATHER
    args = parse()
    MIXED_GATHER = args.gather
    if args.impl == "reference":
        return run_reference(args)
    rank, world, local = dist_info()
    if world > 1 and "CUDA_VISIBLE_DEVICES" not in os.environ:
        # one GPU per rank: make the rank's GPU device 0 of this process
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
    local_dev = 0 if world > 1 else local
    import torch
    torch.cuda.set_device(local_dev)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    mg = graft.load_package()
    abi = mg.abi
    lib = mg.load_library()
    peaks = measured_peaks()
    flush_buf = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def flush():
        flush_buf.fill_(1.0)

    runners = {precision: build_workload(mg, args.workload, precision, rank, world)
               for precision in ("fp64", "mixed")}

    # force accuracy at the starting state (both forms and the oracle)
    f64 = runners["fp64"].forces()
    fmx = runners["mixed"].forces()
    err = {"mixed_vs_fp64": rel_force_err(fmx, f64)}
    stats = runners["fp64"].stats()
    orc = None
    if rank == 0 and not args.no_cpu_baseline:
        orc = graft.load_oracle()
        fo = runners["fp64"].oracle_forces(orc, os.cpu_count() or 1)
        err["fp64_vs_oracle"] = rel_force_err(f64, fo)
        err["mixed_vs_oracle"] = rel_force_err(fmx, fo)

    fma = {}
    for prec, code in (("fp64", abi.MAVI_PREC_FP64), ("mixed", abi.MAVI_PREC_MIXED)):
        v = C.c_double()
        fma[prec] = v.value if lib.mavi_fma_peak(code, local_dev, C.byref(v)) == 0 else None

    meas = {}
    clk_form = {}
    for precision in ("fp64", "mixed"):
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()
        clocks = Clocks(local)      # sampled around each form's timed region
        clocks.start()
        m = time_form(mg, runners[precision], args.steps, max(args.warmup, 3), flush, torch)
        torch.cuda.synchronize()
        clk_form[precision] = clocks.stop()
        if world > 1:
            from mavi_gb300 import replicas
            m["total_ms"] = replicas.max_over_ranks(m["total_ms"], dist)   # the slowest rank sets the job time
            dist.barrier()
        meas[precision] = m

    e2e = e2e_form(mg, runners["mixed"], min(args.steps, 300), torch)
    e2e_pipe = (e2e_pipelined(mg, args.workload, rank, world, min(args.steps, 300), torch)
                if len(runners["mixed"].systems) > 1 else None)
    acc = accuracy(mg, runners, args.accuracy_steps, 5) if args.accuracy_steps >= 5 else None

    n = runners["mixed"].num_slots
    K = args.steps
    line_forms = {}
    for precision in ("fp64", "mixed"):
        m = meas[precision]
        r = runners[precision]
        v = world * n * K / (m["total_ms"] * 1e-3)
        params = abi.MaviReplicaParams()
        r.first.fill_params(params, r.kind)
        rf = roofline(m, n, precision, r.kind, abi, peaks, stats.candidate_pairs,
                      fma[precision], params.dyn.kind, getattr(r.first.state, "vel", None) is not None,
                      args.workload, sum(int(getattr(q.state, "num_rings", 0) or 0) for q in r.systems))
        line_forms[precision] = {"value": v, "ms_per_step": m["total_ms"] / K, "roofline": rf,
                                 "kernels_ms_per_step": {k: d["ms"] / K for k, d in m["kinds"].items()},
                                 "gpu_launches": m["launches_per_step"] * K}
    cpu = None
    if rank == 0 and orc is not None:
        cpu = cpu_baseline(mg, orc, runners["fp64"], args.cpu_seconds, os.cpu_count() or 1)
        one = cpu_baseline(mg, orc, runners["fp64"], max(args.cpu_seconds / 2, 1.0), 1)
        cpu["one_core"] = {"value": one["value"], "sample": one["sample"]}
    if rank == 0:
        mx = line_forms["mixed"]
        first = runners["mixed"].first
        cc = first.int_cfg.chunks_cfg if hasattr(first.int_cfg, "chunks_cfg") else None
        grid = [cc.num_rows, cc.num_cols] if cc is not None and len(runners["mixed"].systems) == 1 else None
        out = {
            "metric": METRIC, "value": mx["value"], "unit": UNIT, "n_gpus": world, "steps": K,
            "warmup": max(args.warmup, 3), "ms_per_step": mx["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 pair loop + f64 update",
            "data": "synthetic",
            "config": {"workload": args.workload, "N": n, "replicas": len(runners["mixed"].systems),
                       "form": "mixed", "chunks": grid, "total_chunks": stats.total_chunks,
                       "candidate_pairs": stats.candidate_pairs,
                       "gather": GATHER_NAMES.get(runners["mixed"].stats().gather_mode),
                       "autotuned_among": runners["mixed"].handle.pass_modes(),
                       "parallelism": (f"replicas split over {world} GPUs" if world > 1 else
                                       ("replicas" if len(runners["mixed"].systems) > 1 else "single")),
                       "l2": "flushed (256 MiB write) before every timed step"},
            "roofline": mx["roofline"],
            "cpu_baseline": cpu,
            "e2e": (
                {"value": world * e2e_pipe["value"], "unit": UNIT,
                 "h2d_bytes_per_step": e2e_pipe["h2d"], "d2h_bytes_per_step": e2e_pipe["d2h"],
                 "path": f"the batch as {e2e_pipe['groups']} handles of consecutive replicas on their own streams; "
                         "every step, group by group: wait for the group's previous download (mavi_synchronize), "
                         "upload its state (mavi_upload_state), step once (mavi_step), queue its download "
                         "(mavi_download_state_async); every group awaited after the last step; pinned host buffers",
                 "single_handle": {"value": world * n * min(K, 300) / e2e["seconds"],
                                   "path": "one handle: mavi_upload_state -> mavi_step(1) -> mavi_download_state"}}
                if e2e_pipe else
                {"value": world * n * min(K, 300) / e2e["seconds"], "unit": UNIT,
                 "h2d_bytes_per_step": e2e["h2d"], "d2h_bytes_per_step": e2e["d2h"],
                 "path": "mavi_upload_state -> mavi_step(1) -> mavi_download_state, pinned host buffers"}),
            "gpu_launches": mx["gpu_launches"],
            "clocks": clk_form["mixed"],
            "plain_fp64": {"value": line_forms["fp64"]["value"], "ms_per_step": line_forms["fp64"]["ms_per_step"],
                           "clocks": clk_form["fp64"],
                           "roofline": line_forms["fp64"]["roofline"],
                           "kernels_ms_per_step": line_forms["fp64"]["kernels_ms_per_step"],
                           "gpu_launches": line_forms["fp64"]["gpu_launches"]},
            "kernels_ms_per_step": mx["kernels_ms_per_step"],
            "speedup_mixed_vs_fp64": mx["value"] / line_forms["fp64"]["value"],
            "force_error": err,
            "energy_drift": acc.get("energy_drift") if acc else None,
            "gr_linf": acc["gr_linf"] if acc else None,
            "accuracy": acc,
            "fma_peak_tflops": {k: (v / 1e12 if v else None) for k, v in fma.items()},
        }
        print(json.dumps(out))
    for r in runners.values():
        r.close()
    if world > 1:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
