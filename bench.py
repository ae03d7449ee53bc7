"""FLIP step throughput on one GB300 (replicas on N GPUs).

Workload (default): the 256^3 dam break -- block x<0.4, y<0.6, all z, walls
on all faces, 8 particles per fluid cell from seed 0, gravity -9.8 with
dx=1/256 (9.8*256 cells/s^2 in index space), flip 0.95, CFL 1, 30 frames/s,
fp32 Jacobi PCG to relative residual 1e-5 (max 1500 iterations).  A step is
one FlipDriver::RunOneStep with dt from the CFL rule.

value: steps/s with the particle state resident in HBM, CUDA events on the
library's stream around exactly K steps (after W warm-up steps), max over
ranks.  The particle state (32.2M particles, 1.16 GB) is larger than L2.
e2e:   the same steps through the public C ABI from pinned host buffers:
upload particles (H2D), step, download particles (D2H) every step; with the
host link's measured bandwidth and the step time it allows (link_floor_ms).
roofline: the dominant kernel's algorithmic bytes / its event-timed time.
cpu_baseline: the oracle (a restatement of the reference CPU path, single
thread, as the reference runs one partition with TBB at 1 thread) timed on
the host for a bounded sample of the same workload.

--impl reference times that CPU path alone (the reference itself cannot be
built here) and prints its own line.
"""
from __future__ import annotations

import argparse
import json
import os
import platform
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "fluid-sim-lb_gb300"))
sys.path.insert(0, str(ROOT))

PEAKS = ROOT / "MEASURED_PEAKS.json"
FRAME_STEP = float(np.float32(1.0) / np.float32(30.0))

WORKLOADS = {
    "dam_break_256": dict(n=256, scene="dam_break"),
    "sphere_drop_64": dict(n=64, scene="sphere_drop"),
    "sphere_drop_128": dict(n=128, scene="sphere_drop"),
    "multidam_512": dict(n=512, scene="multidam"),
    "sphere_pool_1024": dict(n=1024, scene="sphere_pool"),
}

# Algorithmic HBM bytes per unknown (fluid cell) per launch of each PCG kernel
# (Ap is never stored; z = r/diag is recomputed):
#   pcg_spmv:   read r, p_{j-1} (8) + flags (1); write p_j (4)        = 13 B
#   pcg_update: read p_j, x, r (12) + flags (1); write x, r (8)       = 21 B
ALG_BYTES = {"pcg_spmv": 13, "pcg_update": 21, "pcg_spmv_mixed": 13, "pcg_update_mixed": 21,
             "pcg_spmv_f64": 25, "pcg_update_f64": 41,
             # single-reduction iteration (FSIM_PCG_CG1=1): read flags, x, p, r, w, s;
             # write x, p, r, w, s
             "pcg_cg1": 41,
             # resident loop: the pair's fused iteration (34 B per unknown when
             # streamed); it keeps x, r, p and the flags on chip, so its own traffic
             # is lower (the r and p mirrors written, 8 B, and the remote halo read)
             "pcg_resident": 34}
# The same iteration in the textbook formulation, where z = M^-1 r and Ap are stored:
#   Ap = A p and p.Ap:                read p, flags; write Ap                 =  9 B
#   x += a p; r -= a Ap; z; r.r, r.z: read x, p, r, Ap, flags; write x, r, z  = 29 B
#   p = z + b p:                      read z, p; write p                      = 12 B
# (fp32 vectors), keyed by the spmv kernel of the pair.
UNFUSED_BYTES = {"pcg_spmv": 50, "pcg_spmv_mixed": 50, "pcg_cg1": 50, "pcg_resident": 50}
# DRAM traffic per unknown per launch (dram__bytes_read.sum + dram__bytes_write.sum) from ncu
# captures of `bench.py --pcg-micro`.  The fp32 pair: the 256^3 dam-break system (4,021,250
# unknowns), host-launched loop (FSIM_PCG_GRAPH=0), caches NOT flushed between launches
# (--cache-control none), 20 launches in the middle of the step's solve: the steady state of
# the timed loop, where the vectors stay in L2 and DRAM mostly sees write-backs.  Scaled by
# each step's unknowns.  The MIXED pair: a capture at 1024^3 (111,452,816 unknowns, caches
# flushed; the vectors do not fit in L2 there), the size its solver is benchmarked at.
# The resident loop: one launch is a whole solve, so its DRAM bytes (48.22 MB read + 23.18 MB
# written) are divided by the solve's 779 iterations: a capture of the timed step of the
# 256^3 dam break (about 4.03 M unknowns) with the default bench settings.
NCU_TRAFFIC_PER_UNKNOWN = {"pcg_spmv": (1.4706e6 + 17.5451e6) / 4021250,
                           "pcg_update": (5.4866e6 + 19.9465e6) / 4021250,
                           "pcg_spmv_mixed": 1.5765e9 / 111452816,
                           "pcg_update_mixed": 2.3834e9 / 111452816,
                           "pcg_resident": (48.224768e6 + 23.182592e6) / 779 / 4.03e6}
NCU_TRAFFIC_SOURCE = {"pcg_spmv": "the 256^3 system, caches not flushed",
                      "pcg_update": "the 256^3 system, caches not flushed",
                      "pcg_spmv_mixed": "the 1024^3 system, caches flushed",
                      "pcg_update_mixed": "the 1024^3 system, caches flushed",
                      "pcg_resident": "the 256^3 system, one solve's launch over its 779 iterations"}
# The two launches of one PCG iteration (spmv then update) are reported as one unit: the
# split of the iteration's work between them is a design choice (the update could take
# x += alpha p or leave it), and their times are nearly equal.
PCG_PAIRS = {"pcg_spmv": "pcg_update", "pcg_update": "pcg_spmv",
             "pcg_spmv_mixed": "pcg_update_mixed", "pcg_update_mixed": "pcg_spmv_mixed",
             "pcg_spmv_f64": "pcg_update_f64", "pcg_update_f64": "pcg_spmv_f64"}
# Kernels that are a whole PCG iteration on their own.
PCG_SINGLE = {"pcg_cg1", "pcg_resident"}  # pcg_cg1 with its per-pass s re-forming (pcg_cg1_s), in loop_ms


def peaks():
    try:
        d = json.loads(PEAKS.read_text())
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, dev: int):
        self.dev = dev
        self.proc = None
        fd, name = tempfile.mkstemp(prefix="fsim_clocks_", suffix=".csv")
        os.close(fd)
        self.path = Path(name)

    def __enter__(self):
        try:
            q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.dev), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.fh.close()

    def summary(self):
        try:
            return self._summary()
        finally:
            try:
                self.path.unlink()
            except OSError:
                pass

    def _summary(self):
        if self.proc is None or not self.path.exists():
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.path.read_text().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(sm)}


def max_over_ranks(values, device=None):
    """Max of each value over the ranks of the default process group (the
    slowest replica sets the whole-job time); identity without a group."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return [float(v) for v in values]
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t.tolist()]


def whole_job_rate(world, steps, ms_max):
    """Steps/s of the whole job: every replica runs `steps` steps; the job
    takes the slowest replica's time."""
    return world * steps / (ms_max * 1e-3)


def pcg_cfg(args):
    import fsim

    prec = {"fp32": fsim.PREC_FP32, "mixed": fsim.PREC_MIXED, "fp64": fsim.PREC_FP64}[args.precision]
    return fsim.pcg_params(fsim.PCG_RELATIVE, prec, args.max_iterations, tolerance=args.tol,
                           inner_tolerance=1e-2)


def make_sim(wl, args, device):
    import fsim

    n = wl["n"]
    g, f = fsim.physical_gravity(n)
    sim = fsim.Simulation((n, n, n), fsim.BOUNDARY_BOX, g, f, 0.95, args.ppc, device=device)
    sim.seed(fsim.scene_passes(wl["scene"], n), seed=0)
    return sim


def run_gpu(args, rank, world):
    import torch

    import fsim

    device = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(device)
    if args.lib:
        fsim._lib = fsim.load_library(args.lib)  # a variant build of the library
    wl = WORKLOADS[args.workload]
    sim = make_sim(wl, args, device)
    n_particles = sim.particle_count()
    prm = pcg_cfg(args)
    stream = torch.cuda.ExternalStream(sim.stream(), device=device)

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    # warm-up steps (untimed)
    t_in_frame = 0.0
    inv = sim.cfl()

    def next_dt():
        nonlocal t_in_frame, inv
        dt, t_in_frame = fsim.compute_dt(inv, 1, FRAME_STEP, t_in_frame)
        if t_in_frame + 1e-5 >= FRAME_STEP:
            t_in_frame = 0.0
        return dt

    for _ in range(args.warmup):
        st = sim.step(next_dt(), prm)
        inv = st.next_inv_speed
    free_b, total_b = torch.cuda.mem_get_info(device)  # after warm-up: all buffers exist
    launches0 = sim.launch_count()
    iters, rows, loop_ms = [], [], []
    barrier()
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    with Clocks(device) as clk:
        ev0.record(stream)
        for _ in range(args.steps):
            st = sim.step(next_dt(), prm)
            inv = st.next_inv_speed
            iters.append(st.pcg.iterations)
            rows.append(st.pcg.n_rows)
            loop_ms.append(st.pcg.loop_ms)
        ev1.record(stream)
        torch.cuda.synchronize()
    barrier()
    ms = ev0.elapsed_time(ev1)
    launches = sim.launch_count() - launches0
    # per-kernel CUDA-event times on the library's stream (a second pass, so
    # the events do not perturb the timed steps above)
    sim.set_profiling(True)
    sim.reset_kernel_times()
    piters, prows = [], []
    t1 = torch.cuda.Event(enable_timing=True)
    t2 = torch.cuda.Event(enable_timing=True)
    t1.record(stream)
    for _ in range(max(1, min(args.steps, args.profile_steps))):
        st = sim.step(next_dt(), prm)
        inv = st.next_inv_speed
        piters.append(st.pcg.iterations)
        prows.append(st.pcg.n_rows)
    t2.record(stream)
    torch.cuda.synchronize()
    prof_ms = t1.elapsed_time(t2)
    kt = sim.kernel_times()
    sim.set_profiling(False)
    n_fluid = float(np.mean(rows)) if rows else None

    # e2e: public API with host buffers (pinned), H2D + step + D2H per step
    pos, vel, gvel = sim.download_particles()
    hp = torch.from_numpy(pos).pin_memory()
    hv = torch.from_numpy(vel).pin_memory()
    hg = torch.from_numpy(gvel).pin_memory()
    e2e_steps = max(1, min(args.steps, args.e2e_steps))
    barrier()
    torch.cuda.synchronize()
    import ctypes as C

    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    marks = [[torch.cuda.Event(enable_timing=True) for _ in range(4)] for _ in range(e2e_steps)]
    e0.record(stream)
    # (a) the three calls in sequence: upload, step, download (for the split)
    for k in range(e2e_steps):
        marks[k][0].record(stream)
        rc = sim.lib.fsim_upload_particles(sim.h, hp.data_ptr(), hv.data_ptr(), hg.data_ptr(),
                                           hp.shape[0])
        if rc:
            raise RuntimeError(sim.lib.fsim_last_error(sim.h).decode())
        marks[k][1].record(stream)
        st = sim.step(next_dt(), prm)
        inv = st.next_inv_speed
        cnt = sim.particle_count()
        marks[k][2].record(stream)
        got = C.c_int64()
        rc = sim.lib.fsim_download_particles(sim.h, hp.data_ptr(), hv.data_ptr(), hg.data_ptr(),
                                             hp.shape[0], C.byref(got))
        if rc:
            raise RuntimeError(sim.lib.fsim_last_error(sim.h).decode())
        marks[k][3].record(stream)
        if cnt < hp.shape[0]:  # particles deleted at walls: shrink the state
            hp, hv, hg = hp[:cnt], hv[:cnt], hg[:cnt]
    e1.record(stream)
    torch.cuda.synchronize()
    seq_ms = e0.elapsed_time(e1) / e2e_steps
    e2e_split = {name: sum(m[i].elapsed_time(m[i + 1]) for m in marks) / e2e_steps
                 for i, name in enumerate(("upload_ms", "step_ms", "download_ms"))}
    # (b) the headline: fsim_step_host, one call per step with the copies
    # overlapping the step (in place on the same pinned buffers).  One untimed
    # call first: its first use sets up the I/O stream and the staging buffer
    # of the early position download (one-time allocations).
    st, cnt = sim.step_host(next_dt(), prm, hp, hv, hg, out=(hp, hv, hg))
    inv = st.next_inv_speed
    if cnt < hp.shape[0]:
        hp, hv, hg = hp[:cnt], hv[:cnt], hg[:cnt]
    barrier()
    torch.cuda.synchronize()
    e0.record(stream)
    for k in range(e2e_steps):
        st, cnt = sim.step_host(next_dt(), prm, hp, hv, hg, out=(hp, hv, hg))
        inv = st.next_inv_speed
        if cnt < hp.shape[0]:
            hp, hv, hg = hp[:cnt], hv[:cnt], hg[:cnt]
    e1.record(stream)
    torch.cuda.synchronize()
    e2e_ms = e0.elapsed_time(e1) / e2e_steps
    e2e_split["sequential_calls_ms"] = seq_ms
    e2e_split.update(host_link_floor(hp, stream, device, ms / args.steps, kt,
                                     max(1, min(args.steps, args.profile_steps))))
    barrier()
    ms, e2e_ms = max_over_ranks([ms, e2e_ms], device=f"cuda:{device}")
    sim.close()
    return dict(ms=ms, kt=kt, launches=launches, iters=iters, rows=rows, loop_ms=loop_ms,
                clocks=clk.summary(),
                device_memory_gb=(total_b - free_b) / 1e9,
                piters=piters, prows=prows, prof_ms=prof_ms,
                n_particles=n_particles, n_fluid=n_fluid, e2e_ms=e2e_ms, e2e_split=e2e_split,
                e2e_bytes=36 * n_particles)


def host_link_floor(hp, stream, device, step_ms, kt, prof_steps):
    """Host link bandwidth and the end-to-end floor it sets.

    One particle array (12 B per particle, pinned) is copied each way, best
    of 3, on the library's stream.  fsim_step_host needs all three arrays on
    the device before the particle gather (P2G reads the velocities), and
    can start the velocity and PIC-velocity downloads only after G2P; only
    the advection/keying and the sort run while the uploads finish, and the
    position download overlaps the rest of the step.  So no schedule beats
        3 x upload + (device step - keys - sort) + 2 x download."""
    import torch

    flat = hp.reshape(-1)
    dbuf = torch.empty(flat.numel(), dtype=flat.dtype, device=f"cuda:{device}")
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)

    def best_ms(copy):
        best = float("inf")
        with torch.cuda.stream(stream):
            for _ in range(3):
                a.record(stream)
                copy()
                b.record(stream)
                torch.cuda.synchronize()
                best = min(best, a.elapsed_time(b))
        return best

    # blocking copies: a non-blocking one would leave an event of the library's
    # stream on the pinned block, which outlives the stream
    up = best_ms(lambda: dbuf.copy_(flat))
    down = best_ms(lambda: flat.copy_(dbuf))
    del dbuf
    nbytes = flat.numel() * flat.element_size()
    early = sum(kt[k][0] for k in ("advect_keys", "radix_sort(cub)") if k in kt) / prof_steps
    return {"link_h2d_gbs": nbytes / (up * 1e-3) / 1e9,
            "link_d2h_gbs": nbytes / (down * 1e-3) / 1e9,
            "link_floor_ms": e2e_floor_ms(up, down, step_ms, early)}


def e2e_floor_ms(up_ms, down_ms, step_ms, early_ms):
    """Critical path of fsim_step_host given one array's upload and download
    times: all three uploads, the step less the work that overlaps them,
    then the two downloads that follow G2P."""
    return 3 * up_ms + max(0.0, step_ms - early_ms) + 2 * down_ms


def roofline(res):
    """Roofline of the dominant kernel.

    When the dominant kernel is one of the two PCG launches, the unit is one
    PCG iteration (spmv + update): algorithmic bytes = both kernels' bytes per
    unknown x unknowns, and the time is the iteration loops' device time in
    the timed steps (CUDA events the library records on its stream around
    each step's loop: fsim_pcg_stats.loop_ms).  The per-kernel split comes
    from the profiled steps' per-launch events (host-launched, so slower than
    the graph loop).  Otherwise the dominant kernel's profiled event time."""
    peak, src = peaks()
    kt = res["kt"]
    if not kt:
        return None
    top = max(kt.items(), key=lambda kv: kv[1][0])
    name, (tot_ms, nl) = top
    out = {"bound": "hbm", "peak": peak, "peak_source": src, "unit": "GB/s", "traffic": None}
    pair = name in PCG_PAIRS and PCG_PAIRS[name] in kt
    if (pair or name in PCG_SINGLE) and res.get("loop_ms") and sum(res["loop_ms"]) > 0:
        # spmv, update; or the one kernel of a single-reduction iteration
        names = sorted([name, PCG_PAIRS[name]], key=lambda k: "update" in k) if pair else [name]
        per = sum(ALG_BYTES[k] for k in names)
        its, rws, lms = res["iters"], res["rows"], res["loop_ms"]
        tot_bytes = sum(per * r * it for r, it in zip(rws, its))
        loop = sum(lms)
        achieved = tot_bytes / (loop * 1e-3) / 1e9
        n_rows = float(np.mean(rws))
        loop_form = "one cooperative launch per solve" if name == "pcg_resident" else "graph loop"
        out.update(kernel="pcg_iteration (" + " + ".join(names) + ", " + loop_form + ")",
                   achieved=achieved, frac=achieved / peak, alg_bytes_per_unknown=per,
                   alg_bytes_per_launch=per * n_rows, unknowns=n_rows,
                   us_per_iteration=loop * 1e3 / max(sum(its), 1), working_launches=sum(its),
                   share_of_step=loop / res["ms"] if res["ms"] > 0 else None,
                   time_source="fsim_pcg_stats.loop_ms: CUDA events on the library stream, timed steps")
        if names[0] in UNFUSED_BYTES:
            # the same loop time, counted in the textbook formulation's bytes
            ub = UNFUSED_BYTES[names[0]]
            out["unfused_alg_bytes_per_unknown"] = ub
            out["unfused_frac"] = achieved * ub / per / peak
        if all(k in NCU_TRAFFIC_PER_UNKNOWN for k in names):
            out["traffic"] = sum(NCU_TRAFFIC_PER_UNKNOWN[k] for k in names) * n_rows
            out["traffic_source"] = (f"ncu capture ({NCU_TRAFFIC_SOURCE[names[0]]}) of "
                                     f"{' + '.join(names)}, per iteration, scaled by unknowns")
        if name == "pcg_resident":
            out["note"] = ("the resident loop keeps every vector of the iteration on chip (shared and "
                           "tensor memory); achieved counts the streamed formulation's 34 B per unknown, "
                           "so frac above 1 means the loop beats the HBM roofline of a streaming "
                           "iteration; its own DRAM traffic is `traffic`")
        pit = sum(res["piters"])
        prow = sum(r * it for r, it in zip(res["prows"], res["piters"]))
        out["per_kernel_profiled"] = {
            k: {"us_per_launch": kt[k][0] * 1e3 / max(pit, 1),
                "achieved": ALG_BYTES[k] * prow / (kt[k][0] * 1e-3) / 1e9}
            for k in names}
        return out
    out.update(kernel=name, launches=nl,
               share_of_step=tot_ms / res["prof_ms"] if res["prof_ms"] > 0 else None)
    if name in NCU_TRAFFIC_PER_UNKNOWN and res["prows"]:
        out["traffic"] = NCU_TRAFFIC_PER_UNKNOWN[name] * float(np.mean(res["prows"]))
        out["traffic_source"] = f"ncu capture ({NCU_TRAFFIC_SOURCE[name]}), scaled by unknowns"
    if name in ALG_BYTES and res["prows"]:
        alg = ALG_BYTES[name] * float(np.mean(res["prows"]))
        tot_bytes = sum(ALG_BYTES[name] * r * it for r, it in zip(res["prows"], res["piters"]))
        achieved = tot_bytes / (tot_ms * 1e-3) / 1e9
        out.update(achieved=achieved, frac=achieved / peak, alg_bytes_per_launch=alg,
                   working_launches=sum(res["piters"]))
    else:
        out.update(achieved=None, frac=None)
    return out


def host_cpu():
    """(threads, CPU model) of the host the CPU legs run on."""
    model = platform.processor() or platform.machine()
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                model = line.split(":", 1)[1].strip()
                break
    except Exception:
        pass
    return os.cpu_count() or 1, model


def oracle_steps(args, warmup, steps):
    """The oracle (the CPU restatement of the reference's single-partition
    FLIP path) on the workload: `warmup` untimed steps, then `steps` timed
    steps, each one full RunOneStep plus the CFL that sizes the next dt, with
    the dt rule of the GPU arm.  Every host thread works on the loops whose
    results do not depend on the thread count (the oracle is bit-identical
    for any thread count); the P2G write-back stays serial.  Returns
    (per-step seconds, per-step PCG iterations, particles, unknowns, threads)."""
    import fsim
    from oracle import oracle as O

    threads, _ = host_cpu()
    O.set_threads(threads)
    wl = WORKLOADS[args.workload]
    n = wl["n"]
    g, f = fsim.physical_gravity(n)
    orc = O.OracleSim((n, n, n), fsim.BOUNDARY_BOX, g, f, 0.95, 8)
    orc.seed(fsim.scene_passes(wl["scene"], n), seed=0)
    npart = orc.particle_count()
    inv, t_in = orc.cfl(), 0.0
    for _ in range(warmup):
        dt, t_in = fsim_dt(inv, t_in)
        orc.step(dt, mode=1, precision=0, max_iterations=args.max_iterations, tol=args.tol)
        inv = orc.cfl()
    secs, iters, rows = [], [], []
    for _ in range(steps):
        dt, t_in = fsim_dt(inv, t_in)
        t0 = time.perf_counter()
        st = orc.step(dt, mode=1, precision=0, max_iterations=args.max_iterations, tol=args.tol)
        inv = orc.cfl()
        secs.append(time.perf_counter() - t0)
        iters.append(st.iterations)
        rows.append(st.n_rows)
    orc.close()
    O.set_threads(1)
    return secs, iters, npart, (float(np.mean(rows)) if rows else None), threads


def pcg_compare(args, workload):
    """Mixed-precision vs FP32 PCG on one divergence (default: the 512^3
    multi-dam of the mixed-precision configuration).

    Runs one step to build the system, then solves it again with: an FP64
    PCG to relative residual 1e-12 (the reference solution x64; the GPU FP64
    path is checked against the FP64 oracle solve in tests/test_gpu_pcg.py),
    plain FP32 PCG, MIXED PCG (fp32 vectors; dot products accumulated as
    double-float pairs, about 44 significant bits, not FP64; fp64 outer
    residual replacement) and FP64 PCG at ladders of tolerances.  Each solve
    is timed with CUDA events on the library's stream; its error is
    ||x - x64|| / ||x64|| over the fluid cells.  Returns the record.
    """
    import torch

    import fsim

    wl = WORKLOADS[workload]
    sim = make_sim(wl, args, 0)
    stream = torch.cuda.ExternalStream(sim.stream(), device=0)
    st = sim.step(0.01, fsim.pcg_params(fsim.PCG_RELATIVE, fsim.PREC_FP32, 3000, tolerance=1e-5))
    rows = st.pcg.n_rows

    def solve(prm):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        stt = sim.pcg_solve(prm)
        e1.record(stream)
        torch.cuda.synchronize()
        x, act = sim.field(fsim.FIELD_PRESSURE)
        return e0.elapsed_time(e1), stt, x[act.astype(bool)].astype(np.float64)

    t_ref, st_ref, xref = solve(fsim.pcg_params(fsim.PCG_RELATIVE, fsim.PREC_FP64, 40000,
                                                tolerance=1e-12))
    nref = np.linalg.norm(xref)
    out = {"metric": "PCG time to relative error vs FP64 solution", "unit": "ms",
           "workload": workload, "unknowns": rows,
           "mixed_dots": "double-float pairs (about 44 significant bits), not FP64; "
                         "alpha and beta formed in FP64",
           "fp64_reference": {"ms": t_ref, "iterations": st_ref.iterations,
                              "rel_residual": float(np.sqrt(st_ref.rr / st_ref.bb))},
           "fp32": [], "mixed": [], "fp64": []}
    for tol in (1e-5, 1e-6, 1e-7, 1e-8):
        ms, stt, x = solve(fsim.pcg_params(fsim.PCG_RELATIVE, fsim.PREC_FP32, 40000,
                                           tolerance=tol))
        out["fp32"].append({"tol": tol, "ms": ms, "iterations": stt.iterations,
                            "status": stt.status, "error": float(np.linalg.norm(x - xref) / nref)})
    for tol, inner in ((1e-6, 1e-2), (1e-6, 1e-3), (1e-7, 1e-2), (1e-8, 1e-3), (1e-9, 1e-3)):
        ms, stt, x = solve(fsim.pcg_params(fsim.PCG_RELATIVE, fsim.PREC_MIXED, 40000,
                                           tolerance=tol, inner_tolerance=inner,
                                           max_refinements=20))
        out["mixed"].append({"tol": tol, "inner": inner, "ms": ms, "iterations": stt.iterations,
                             "refinements": stt.refinements, "status": stt.status,
                             "error": float(np.linalg.norm(x - xref) / nref)})

    for tol in (1e-5, 1e-6, 1e-7):
        ms, stt, x = solve(fsim.pcg_params(fsim.PCG_RELATIVE, fsim.PREC_FP64, 40000,
                                           tolerance=tol))
        out["fp64"].append({"tol": tol, "ms": ms, "iterations": stt.iterations,
                            "status": stt.status, "error": float(np.linalg.norm(x - xref) / nref)})

    def best(lst):
        ok = [r for r in lst if r["error"] <= 1e-6]
        return min(ok, key=lambda r: r["ms"]) if ok else None

    bf, bm, bd = best(out["fp32"]), best(out["mixed"]), best(out["fp64"])
    out["fp32_error_floor"] = min(r["error"] for r in out["fp32"])
    out["fastest_fp32_at_1e-6"] = bf
    out["fastest_mixed_at_1e-6"] = bm
    out["fastest_fp64_at_1e-6"] = bd
    out["speedup_mixed_vs_fp32"] = (bf["ms"] / bm["ms"]) if (bf and bm) else None
    out["speedup_mixed_vs_fp64"] = (bd["ms"] / bm["ms"]) if (bd and bm) else None
    # the dots' precision does not limit MIXED: it needs FP64's iteration count
    if bm and bd:
        out["iterations_mixed_vs_fp64_at_1e-6"] = [bm["iterations"], bd["iterations"]]
    sim.close()
    return out


def pcg_micro(args):
    """Per-kernel times of the PCG iteration on one step's pressure system.

    One fsim_step builds the system (fp32, relative 1e-5).  Then the same
    system is solved again with FSIM_PCG_FIXED for --micro-iters iterations:
    once per precision with the library's CUDA-event profiling on (mean time
    per launch of each kernel), and once without profiling (the graph loop;
    wall time per iteration).  Prints one JSON line.  This is the program the
    PCG ncu captures run.
    """
    import fsim

    if args.lib:
        fsim._lib = fsim.load_library(args.lib)  # a variant build of the library
    wl = WORKLOADS[args.workload]
    sim = make_sim(wl, args, 0)
    prm = fsim.pcg_params(fsim.PCG_RELATIVE, fsim.PREC_FP32, 1500, tolerance=1e-5)
    st = sim.step(0.01, prm)
    k = args.micro_iters
    out = {"workload": args.workload, "unknowns": st.pcg.n_rows, "step_iterations": st.pcg.iterations,
           "fixed_iterations": k}
    for prec, name in ((fsim.PREC_FP32, "fp32"), (fsim.PREC_MIXED, "mixed")):
        sim.set_profiling(True)
        sim.reset_kernel_times()
        sim.pcg_solve(fsim.pcg_params(fsim.PCG_FIXED, prec, k))
        sim.synchronize()
        kt = sim.kernel_times()
        sim.set_profiling(False)
        # per iteration: the host launches chunks of iterations, and launches
        # after the stop flag return at once, so the time is divided by the
        # k working launches rather than by all launches
        out[name + "_us_per_launch"] = {n: round(v[0] / k * 1e3, 2)
                                        for n, v in kt.items() if v[1] >= k // 2}
    for prec, name in ((fsim.PREC_FP32, "fp32"), (fsim.PREC_MIXED, "mixed")):
        sim.synchronize()
        t0 = time.perf_counter()
        sim.pcg_solve(fsim.pcg_params(fsim.PCG_FIXED, prec, k))
        sim.synchronize()
        out[name + "_graph_us_per_iteration"] = round((time.perf_counter() - t0) / k * 1e6, 2)
    out["pcg_graph_mode"] = os.environ.get("FSIM_PCG_GRAPH", "1")
    print(json.dumps(out), flush=True)
    sim.close()


def adjoint_check(args):
    """Differentiable rollout: gradient w.r.t. the initial particle velocity.

    The 128^3 sphere drop (walls) with the initial velocities perturbed by
    Gaussian noise (0.1 m/s, seed 1), 16 steps at dt = 1/300 s with MIXED
    PCG to 1e-9, checkpoints every 4 steps; loss 0.5 ||u_16 - u_target||^2
    with u_target from the same rollout under seed 2's noise.  The adjoint
    (fp32 forward tape, fp64 accumulation) is compared with central
    differences of the fp64 replay along 32 seeded directions at eps=1e-3
    (and the first 4 directions at smaller eps), and with the fp64 reference
    gradient.  The first 4 directions also run at eps = 1e-4, 1e-5, 1e-6,
    where the differences converge to the exact derivative.  The frozen map
    (bins, clamps, stencil sides, markers, active faces and the weight cut
    of the forward) is smooth but strongly curved (v = m / w at faces whose total
    weight sits near the 1e-5 cut), so the central differences carry a large
    eps^2 term; each direction also gets the Richardson combination
    (4 D(eps/2) - D(eps)) / 3 at eps = 1e-3, which cancels it.  Prints one
    JSON line.
    """
    import fsim

    n, steps, every, dt = args.adjoint_n, 16, 4, 1.0 / 300.0
    t0 = time.perf_counter()
    sim, ro, target, pcg = fsim.rollout_case(n, steps, every, dt)
    t_case = time.perf_counter() - t0
    adj = fsim.pcg_params(fsim.PCG_RELATIVE, fsim.PREC_FP64, 20000, tolerance=1e-12)
    t0 = time.perf_counter()
    loss = ro.forward(dt, pcg, target)
    t_fwd = time.perf_counter() - t0
    t0 = time.perf_counter()
    gv, gg = ro.backward(adj, tape=0)
    t_bwd = time.perf_counter() - t0
    gv64, gg64 = ro.backward(adj, tape=1)
    g32, g64 = gv + gg, gv64 + gg64
    theta, _ = ro.initial_velocity()
    rng = np.random.default_rng(11)
    dirs = [rng.standard_normal(theta.shape) for _ in range(args.adjoint_dirs)]
    rows = []
    t0 = time.perf_counter()
    def central(d, eps):
        lp = ro.replay_loss(theta + eps * d, theta + eps * d)
        lm = ro.replay_loss(theta - eps * d, theta - eps * d)
        return (lp - lm) / (2 * eps)

    for k, d in enumerate(dirs):
        a32, a64 = float(np.sum(g32 * d)), float(np.sum(g64 * d))
        fds = {}
        for eps in ((1e-3, 5e-4, 1e-4, 1e-5, 1e-6) if k < 4 else (1e-3, 5e-4)):
            fd = fds[eps] = central(d, eps)
            rows.append({"dir": k, "eps": eps, "fd": fd, "adj_fp32": a32, "adj_fp64": a64,
                         "rel_fp32": abs(a32 - fd) / abs(fd), "rel_fp64": abs(a64 - fd) / abs(fd)})
        # Richardson: central differences at eps and eps/2 cancel the eps^2 term
        fr = (4.0 * fds[5e-4] - fds[1e-3]) / 3.0
        rows.append({"dir": k, "eps": "1e-3 richardson", "fd": fr, "adj_fp32": a32,
                     "adj_fp64": a64, "rel_fp32": abs(a32 - fr) / abs(fr),
                     "rel_fp64": abs(a64 - fr) / abs(fr)})
    t_fd = time.perf_counter() - t0
    main = [r for r in rows if r["eps"] == 1e-3]
    rich = [r for r in rows if r["eps"] == "1e-3 richardson"]
    out = {"metric": "adjoint gradient vs central differences", "workload": f"sphere_drop_{n}",
           "particles": ro.n, "steps": steps, "checkpoint_every": every, "loss": loss,
           "directions": len(dirs),
           "max_rel_fp32_eps1e-3": max(r["rel_fp32"] for r in main),
           "median_rel_fp32_eps1e-3": float(np.median([r["rel_fp32"] for r in main])),
           "max_rel_fp64_eps1e-3": max(r["rel_fp64"] for r in main),
           "median_rel_fp64_eps1e-3": float(np.median([r["rel_fp64"] for r in main])),
           "max_rel_fp64_eps1e-3_richardson": max(r["rel_fp64"] for r in rich),
           "median_rel_fp64_eps1e-3_richardson": float(np.median([r["rel_fp64"] for r in rich])),
           "max_rel_fp32_eps1e-3_richardson": max(r["rel_fp32"] for r in rich),
           "max_rel_by_eps": {f"{e:g}": {"fp32": max(r["rel_fp32"] for r in rows if r["eps"] == e),
                                         "fp64": max(r["rel_fp64"] for r in rows if r["eps"] == e)}
                              for e in (1e-3, 5e-4, 1e-4, 1e-5, 1e-6)},
           "grad_rel_l2_fp32_vs_fp64": float(np.linalg.norm(g32 - g64) / np.linalg.norm(g64)),
           "seconds": {"scene": t_case, "forward": t_fwd, "backward": t_bwd, "fd": t_fd},
           "rows": rows}
    print(json.dumps(out), flush=True)
    ro.close()
    sim.close()


def fsim_dt(inv, t_in):
    from oracle.oracle import compute_dt

    dt, t = compute_dt(inv, 1, FRAME_STEP, t_in)
    if t + 1e-5 >= FRAME_STEP:
        t = 0.0
    return dt, t


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="dam_break_256", choices=sorted(WORKLOADS))
    ap.add_argument("--precision", default="fp32", choices=["fp32", "mixed", "fp64"])
    ap.add_argument("--tol", type=float, default=1e-5)
    ap.add_argument("--max-iterations", type=int, default=1500)
    ap.add_argument("--e2e-steps", type=int, default=10)
    ap.add_argument("--cpu-pcg-iters", type=int, default=40)
    ap.add_argument("--profile-steps", type=int, default=3)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-pcg-compare", action="store_true",
                    help="leave the 512^3 mixed-vs-FP32-vs-FP64 PCG record out of the bench line")
    ap.add_argument("--pcg-compare", action="store_true",
                    help="mixed vs FP32 PCG time to 1e-6 error (use --workload multidam_512)")
    ap.add_argument("--pcg-micro", action="store_true",
                    help="per-kernel PCG times on one step's system (fixed iteration count)")
    ap.add_argument("--micro-iters", type=int, default=300)
    ap.add_argument("--ppc", type=int, default=8,
                    help="particles per fluid cell (8 defines the workloads; fewer gives the same "
                         "pressure system in less memory, for --pcg-micro captures only)")
    ap.add_argument("--lib", default=None, help="path of a variant libfsim.so (A/B runs)")
    ap.add_argument("--adjoint-check", action="store_true",
                    help="differentiable rollout: adjoint vs central differences")
    ap.add_argument("--adjoint-n", type=int, default=128)
    ap.add_argument("--adjoint-dirs", type=int, default=32)
    args = ap.parse_args()
    if args.ppc != 8 and not args.pcg_micro:
        ap.error("--ppc changes the workload: it is for --pcg-micro only")

    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    wl = WORKLOADS[args.workload]
    config = {"workload": args.workload, "grid": wl["n"], "scene": wl["scene"],
              "pcg": f"jacobi {args.precision} relative {args.tol:g} max {args.max_iterations}",
              "cfl": 1, "flip": 0.95, "frame_rate": 30,
              "l2": "inputs larger than L2 (particle state > 129 MB)",
              "parallelism": f"replicas x{world}"}

    if args.pcg_compare:
        print(json.dumps(pcg_compare(args, args.workload)), flush=True)
        return
    if args.pcg_micro:
        pcg_micro(args)
        return
    if args.adjoint_check:
        adjoint_check(args)
        return

    if args.impl == "reference":
        if rank != 0:
            return
        # The same steps as the GPU arm: W untimed warm-up steps, then K timed
        # steps of the oracle, each a full RunOneStep (no extrapolation).
        secs, iters, npart, rows, threads = oracle_steps(args, args.warmup, args.steps)
        _, model = host_cpu()
        total = sum(secs)
        v = args.steps / total
        line = {"impl": "reference", "metric": "FLIP steps/s", "value": v, "unit": "steps/s",
                "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": config,
                "workload_stats": {"particles": npart, "fluid_cells": rows,
                                   "pcg_iters_per_step": float(np.mean(iters)),
                                   "pcg_iters": iters},
                "cpu_baseline": {"value": v, "unit": "steps/s", "cores": threads, "kind": "port",
                                 "host": model,
                                 "sample": f"steps {args.warmup + 1}-{args.warmup + args.steps} "
                                           f"of {args.workload} ({npart} particles) after "
                                           f"{args.warmup} untimed warm-up steps, each a full "
                                           f"step; the oracle's restatement of the reference "
                                           f"CPU path on {threads} host threads (its loops "
                                           f"with thread-count-independent results; the "
                                           f"P2G write-back stays on one)"},
                "e2e": {"value": v, "unit": "steps/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return

    if world > 1:
        import torch

        torch.distributed.init_process_group("nccl")
    res = run_gpu(args, rank, world)
    if rank != 0:
        return
    value = whole_job_rate(world, args.steps, res["ms"])
    line = {"metric": "FLIP steps/s", "value": value, "unit": "steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": res["ms"] / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": config,
            "workload_stats": {"particles": res["n_particles"], "fluid_cells": res["n_fluid"],
                               "pcg_iters_per_step": float(np.mean(res["iters"])),
                               "pcg_iters": res["iters"]},
            "roofline": roofline(res),
            "e2e": {"value": whole_job_rate(world, 1, res["e2e_ms"]), "unit": "steps/s",
                    "h2d_bytes_per_step": res["e2e_bytes"], "d2h_bytes_per_step": res["e2e_bytes"],
                    **{k: round(v, 3) for k, v in res["e2e_split"].items()}},
            "gpu_launches": res["launches"], "clocks": res["clocks"],
            "device_memory_gb": round(res["device_memory_gb"], 2),
            "kernels_ms": {k: round(v[0], 3) for k, v in sorted(res["kt"].items(),
                                                                key=lambda kv: -kv[1][0])}}
    if not args.no_pcg_compare:
        line["pcg_compare"] = pcg_compare(args, "multidam_512")
    if not args.no_cpu:
        secs, iters, npart, _, threads = oracle_steps(args, 0, 1)
        _, model = host_cpu()
        line["cpu_baseline"] = {"value": 1.0 / secs[0], "unit": "steps/s", "cores": threads,
                                "kind": "port", "host": model,
                                "sample": f"first step of {args.workload} ({npart} particles, "
                                          f"{iters[0]} PCG iterations), one full step of the "
                                          f"oracle on {threads} host threads; the reference arm "
                                          f"(--impl reference) times the same steps as this "
                                          f"line"}
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
