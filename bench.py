"""Benchmark: spin-flip attempts/ns of one PT cycle on one GB300.

Workload (default, the batched configuration): L=32 cubic periodic lattices, NCONF=64 disorder
configurations (PHI=2, XI=3, seeds IRINIT+k), each with a 32-replica ladder linear over
T=8.0-11.5, HOT starts; J1=1, J2=-1, Jperp=1, no dilution.  2048 lattices resident on the GPU.
One step = one PT cycle: PTSWAPEVER=5 fused FP32 sweeps of all lattices, the observable
reduction, the replica exchange and the FP64 running sums.  Synthetic inputs of the reference's
shapes (no dataset is involved).  The FP64 plain form is timed beside it on the L=24, 16-replica
PT configuration (START=STR, STRAXIS=X).

`value`, the sweep kernel's CUDA-event time behind the roofline and e2e all come from one engine
and the same timed steps (its cycle graph brackets the sweep launch with event nodes).  The
reference arm times the reference's CPU path, restated in the oracle (the Fortran program has no
toolchain here), on the same workload: every step is one whole PT cycle of every ladder.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "j1j2-public_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "spin-flip attempts/ns, FP32 batched vs FP64 plain on 1 GB300; % HBM roofline"
UNIT = "attempts/ns"
B_PER_ATTEMPT_FP32 = 11.8  # full PT cycle model: 10 B per sweep attempt + 9 B/site measure / 5
B_PER_ATTEMPT_FP64 = 21.4
L2_FLUSH_BYTES = 256 << 20
# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of one sweep-kernel launch (5 sweeps
# + measure of every lattice), from an ncu capture of the same workload
# (the kernel the tuner keeps for the workload: two lattices of one configuration per CTA)
TRAFFIC = {"batched_fp32_L32_64x32": 75683072 + 8576000}
# issue-slot utilisation and thread instructions per attempt of the same capture (the kernel is
# bound by instruction issue inside shared memory, not by DRAM)
NCU_ISSUE = {"batched_fp32_L32_64x32": {"issue_active": 0.564, "inst_per_attempt": 44.7,
                                        "binding_limit": "instruction issue (shared-memory "
                                                         "resident lattices)",
                                        "source": "profiles/sweep_fixed_fp32_L32_2048lat.md"}}

# name -> lattice-shape groups (L, nconf, nreplica), precision and options
HEADLINE = "batched_fp32_L32_64x32"  # the workload the metric is quoted on

WORKLOADS = {
    # L=32, 64 disorder configurations x 32-replica ladders (2048 lattices), FP32 sweep
    "batched_fp32_L32_64x32": dict(groups=[(32, 64, 32)], precision=1),
    # L=24, one disorder configuration, 16-replica PT ladder, FP64 sweep (plain form), stripe
    # start along x (START=STR, STRAXIS=X)
    "plain_fp64_L24_1x16": dict(groups=[(24, 1, 16)], precision=0, start="STR_X"),
    # the batched workload in the FP64 form (same seeds)
    "batched_fp64_L32_64x32": dict(groups=[(32, 64, 32)], precision=0),
    # uneven batch: L=16/24/32/48 with 128/64/32/8 configurations and 16/24/32/48 replicas
    "mixed_L16_24_32_48": dict(groups=[(16, 128, 16), (24, 64, 24), (32, 32, 32), (48, 8, 48)],
                               precision=1),
    # L=96, 5 % site vacancies, 8 configurations x 48 replicas, one Wolff update per PT cycle
    "large_L96_vac5_wolff_8x48": dict(groups=[(96, 8, 48)], precision=1, vacancies=0.05,
                                      wolff=True),
    # the same with one configuration (48 lattices): the small case for ncu captures
    "large_L96_vac5_wolff_1x48": dict(groups=[(96, 1, 48)], precision=1, vacancies=0.05,
                                      wolff=True),
    # L=16 single-temperature local Metropolis (T=9.5, one sweep + measurement per cycle), FP64
    # LOCAL: one sweep + measurement per cycle, 100 back-to-back cycles per step (a LOCAL run of
    # the reference is 10^4 + 10^4 such sweeps in one call)
    "local_fp64_L16_T9.5": dict(groups=[(16, 1, 1)], precision=0, ptswapever=1, T=9.5,
                                cycles_per_step=100),
}


def peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except OSError:
        return {}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    return ws, int(os.environ.get("RANK", "0")), int(os.environ.get("LOCAL_RANK", "0"))


def conf_base_of(rank, w):
    """First global configuration index of a rank: every rank holds the workload's full set of
    configurations, with disjoint disorder seeds (weak scaling, no data-path collective)."""
    return rank * sum(n for _, n, _ in w["groups"])


def max_over_ranks(dist, x, device):
    """Maximum of a per-rank float (the timed interval) over all ranks."""
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc is not None:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [ln for ln in out.splitlines() if ln.strip()]

    def summary(self):
        mhz, mx, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in getattr(self, "lines", []):
            f = [x.strip() for x in ln.split(",")]
            try:
                mhz.append(float(f[1]))
                mx.append(float(f[2]))
            except (ValueError, IndexError):
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        if not mhz:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(mhz), "sm_max_mhz": max(mx),
                "reasons": sorted(reasons), "samples": len(mhz)}


def workload_config(wname, w, ws=1):
    """The workload as both arms name it in their JSON line."""
    g0 = w["groups"][0]
    cfg = {"workload": wname, "L": g0[0], "H": g0[0],
           "nconf_per_gpu": sum(n for _, n, _ in w["groups"]), "nreplica": g0[2],
           "ptswapever": w.get("ptswapever", 5), "T": [w["T"]] if "T" in w else [8.0, 11.5],
           "phi": 2.0, "xi": 3.0, "start": w.get("start", "HOT"),
           "lattices_per_gpu": sum(n * r for _, n, r in w["groups"]),
           "attempts_per_step": None, "parallelism": f"confs x{ws}"}
    if len(w["groups"]) > 1:
        cfg["groups_L_nconf_nreplica"] = [list(g) for g in w["groups"]]
    if w.get("vacancies"):
        cfg["vacancies"] = w["vacancies"]
    if w.get("wolff"):
        cfg["wolff_per_cycle"] = 1
    return cfg


def make_engine(jc, w, device, conf_base=0, flags=0, irinit=1):
    """Engine of one workload: disorder of conf k from seed irinit + conf_base + k (PHI=2,
    XI=3), optional Bernoulli site vacancies from the same seed, linear ladders over
    T = 8.0-11.5 (or one temperature), HOT starts (or the workload's stripe start)."""
    ptswapever = w.get("ptswapever", 5)
    if w.get("wolff"):
        flags |= jc.FLAG_WOLFF
    eng = jc.Engine(groups=[(L, L, n, r) for L, n, r in w["groups"]], ptswapever=ptswapever,
                    precision=w["precision"], seed=irinit, conf_base=conf_base, device=device,
                    flags=flags)
    betas, k = [], 0
    for L, n, r in w["groups"]:
        b = np.full(r, 1.0 / w["T"]) if "T" in w else 1.0 / jc.ladder(r, 8.0, 11.5)
        for _ in range(n):
            seed = irinit + conf_base + k
            occu = None
            if w.get("vacancies"):
                occu = jc.setup_vacancies(seed, L, L, w["vacancies"])[0]
            eng.set_disorder(k, jc.disorder(L, L, seed, 2.0, 3.0), occu)
            betas.append(b)
            k += 1
    betas = np.concatenate(betas)
    eng.set_ladder(-1, betas)
    start, axis = (jc.START_STR, jc.AXIS_X) if w.get("start") == "STR_X" else (jc.START_HOT, 0)
    for k in range(eng.nconf):
        eng.init_spins(k, start, axis)
    eng.reset_measurements()
    return eng, betas


def attempts_per_cycle(eng):
    """Occupied sites x replicas x sweeps of one PT cycle, summed over the configurations."""
    reps = np.array([eng.nrep_of(k) for k in range(eng.nconf)], np.int64)
    return int((eng.nocc * reps).sum()) * eng.ptswapever


class L2Flush:
    """Empties L2 of a step's data before the next step: a write of a buffer twice the L2's
    size, then a read of a second one, so that the step starts cold and the lines left in L2
    are clean (the write alone leaves ~126 MB of dirty lines, whose write-back the step would
    otherwise pay)."""

    def __init__(self, torch):
        self.torch = torch
        self.w = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
        self.r = torch.zeros(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
        self.out = torch.empty((), dtype=torch.float32, device="cuda")

    def __call__(self):
        self.w.zero_()
        self.out.copy_(self.r.sum())


def time_steps(torch, eng, steps, warmup, flush, cycles=1):
    """Device time of `steps` steps of `cycles` PT cycles each: CUDA events on a dedicated
    stream that also carries the L2 flush before every step (outside the timed interval) and the
    engine's own launches, so every event, flush and cycle is ordered on one stream."""
    stream = timing_stream(torch)
    eng.set_stream(stream.cuda_stream)
    with torch.cuda.stream(stream):
        eng.run(warmup, measure=True, restart_swap_phase=True)
        stream.synchronize()
        prof0 = eng.profile()[0]
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(steps)]
        # the cycles are enqueued without waiting, so each step's closing event follows its
        # cycles directly on the stream (j1j2c_run would wait, and the event would also time the
        # host's return from that wait)
        for k in range(steps):
            flush()
            ev[k][0].record(stream)
            eng.enqueue(cycles, measure=True, restart_swap_phase=False)
            ev[k][1].record(stream)
        eng.sync()
        stream.synchronize()
    total_ms = 0.0
    for a, b in ev:
        total_ms += a.elapsed_time(b)
    return total_ms, eng.profile()[0] - prof0


_STREAM = []


def timing_stream(torch):
    """One non-default stream for every timed run (a stream handle of 0 would make the engine
    use its own stream, unordered with the events)."""
    if not _STREAM:
        _STREAM.append(torch.cuda.Stream())
    return _STREAM[0]


def time_workload(torch, jc, w, device, flush, steps, min_ms=60.0, max_steps=200):
    """Device throughput of one workload (CUDA events per step, L2 flushed between).  The value
    comes from an engine without profiling events (graph event nodes cost microseconds per
    cycle, a sizeable share of a small lattice's cycle); a second engine with them gives its own
    step time and the sweep launches' share of it, over the same number of steps.  A short
    workload gets more steps (up to max_steps), so that at least min_ms of device time is timed:
    three steps after three warm-up steps estimate the step time."""
    cycles = w.get("cycles_per_step", 1)
    eng, _ = make_engine(jc, w, device)
    est, _ = time_steps(torch, eng, 3, 3, flush, cycles)
    steps = max(steps, min(max_steps, int(np.ceil(min_ms * 3 / max(est, 1e-3)))))
    ms, _ = time_steps(torch, eng, steps, 1, flush, cycles)
    eng.close()
    eng, _ = make_engine(jc, w, device, flags=jc.FLAG_PROFILE)
    pms, prof_ms = time_steps(torch, eng, steps, 3, flush, cycles)
    att = attempts_per_cycle(eng) * cycles
    out = {"value": round(att * steps / (ms * 1e6), 4), "unit": UNIT,
           "ms_per_step": round(ms / steps, 4), "steps": steps, "attempts_per_step": att,
           "profiled_engine": {"ms_per_step": round(pms / steps, 4),
                               "sweep_ms_per_step": round(prof_ms / steps, 4)},
           "groups_L_nconf_nreplica": [list(g) for g in w["groups"]]}
    if w.get("start"):
        out["start"] = w["start"]
    if cycles > 1:
        out["cycles_per_step"] = cycles
    cfg = eng.config()
    out["block_threads"] = cfg["block_threads"]
    eng.close()
    return out


B_PER_WOLFF_SITE = 18  # spin 1 + J_eff 8 + label write/read 8 + flip 1, per cluster site


def wolff_report(torch, jc, w, device, warm=30, n=10):
    """The Wolff update alone (j1j2c_wolff, every lattice at its slot's temperature) on lattices
    equilibrated for `warm` PT cycles: device time per update (CUDA events on the engine's
    stream), flipped-cluster sites per update, sites per ns, and the streaming model of 18 bytes
    per cluster site against the measured copy bandwidth."""
    eng, _ = make_engine(jc, w, device)
    stream = timing_stream(torch)
    eng.set_stream(stream.cuda_stream)
    with torch.cuda.stream(stream):
        eng.run(warm, measure=False)
        eng.wolff()
        stream.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        sites = 0
        a.record(stream)
        for _ in range(n):
            sites += int(eng.wolff().sum())
        b.record(stream)
        stream.synchronize()
    ms = a.elapsed_time(b) / n
    eng.close()
    per = sites / n
    gbs = B_PER_WOLFF_SITE * per / (ms * 1e-3) / 1e9
    hbm = peaks().get("hbm_gbs") or 6800.0
    return {"ms_per_update": round(ms, 4), "cluster_sites_per_update": int(per),
            "sites_per_ns": round(per / (ms * 1e6), 3), "bytes_per_site": B_PER_WOLFF_SITE,
            "model_gbs": round(gbs, 1), "frac_of_hbm": round(gbs / hbm, 4),
            "equilibration_cycles": warm}


def secondary_workloads(torch, jc, device, flush, steps):
    """The other configurations of the same path, each timed alone on this GPU."""
    res = {}
    for name in ("batched_fp64_L32_64x32", "mixed_L16_24_32_48", "large_L96_vac5_wolff_8x48"):
        res[name] = time_workload(torch, jc, WORKLOADS[name], device, flush, steps)
    res["large_L96_vac5_wolff_8x48"]["wolff"] = wolff_report(
        torch, jc, WORKLOADS["large_L96_vac5_wolff_8x48"], device)
    # per-L throughput of the uneven batch: each lattice-shape group alone
    per_l = {}
    for L, n, r in WORKLOADS["mixed_L16_24_32_48"]["groups"]:
        w = dict(groups=[(L, n, r)], precision=1)
        per_l[str(L)] = time_workload(torch, jc, w, device, flush, steps)["value"]
    res["mixed_L16_24_32_48"]["per_L_alone"] = per_l
    res["local_fp64_L16_T9.5"] = time_workload(torch, jc, WORKLOADS["local_fp64_L16_T9.5"],
                                               device, flush, steps)
    return res


def precision_report(jc, eng, w, device, equil, measured):
    """The FP32 form against the FP64 form on the headline workload's seeds: (1) the flip-decision
    mismatch rate in deterministic replay (one FP64 sweep of every lattice from the FP32 run's
    current state, the FP32 decision evaluated on the same configuration and uniform); (2) per
    temperature slot and observable, the FP32 - FP64 difference of the configuration-averaged
    thermal average in units of its standard error over the configurations (both forms from the
    same starts, equil + measured PT cycles)."""
    att, mis = eng.audit_fp32(1)
    names = ("absmag", "mag2", "en", "en2", "strx_abs", "stry_abs", "nbar", "nbar2")
    cols = [jc.SUM_FIELDS.index(n) for n in names]
    avg = {}
    for prec in (0, 1):
        e, _ = make_engine(jc, dict(w, precision=prec), device)
        e.run(equil, measure=False)
        e.reset_measurements()
        e.run(measured, measure=True)
        s, nm = e.slot_sums(-1)
        avg[prec] = (s[:, cols] / nm[:, None]).reshape(e.nconf, -1, len(cols))
        e.close()
    d = avg[1] - avg[0]  # (conf, slot, observable)
    se = d.std(axis=0, ddof=1) / np.sqrt(d.shape[0])
    z = np.abs(d.mean(axis=0)) / np.where(se > 0, se, np.inf)
    return {"fp32_flip_mismatch_rate": mis / att, "attempts_audited": int(att),
            "observable_z_max": {n: round(float(z[:, j].max()), 3) for j, n in enumerate(names)},
            "z_above_2_fraction": round(float((z > 2).mean()), 4),
            "cycles": [equil, measured], "nconf": int(d.shape[0])}


def run_ours(args):
    import torch

    import j1j2cuda as jc

    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    flush = L2Flush(torch)

    wname = args.workload
    w = WORKLOADS[wname]
    if args.nconf:  # a smaller case of the same kernels (profiling captures)
        w = dict(w, groups=[(L, args.nconf, r) for L, _, r in w["groups"]])
    # `value` and e2e: the production engine (no profiling nodes in its cycle graph)
    eng, betas = make_engine(jc, w, local, conf_base=conf_base_of(rank, w), flags=args.flags)
    cycles = w.get("cycles_per_step", 1)
    attempts_per_step = attempts_per_cycle(eng) * cycles

    if ws > 1:
        dist.barrier()
    torch.cuda.synchronize()
    with Clocks(local) as clk:
        total_ms, _ = time_steps(torch, eng, args.steps, args.warmup, flush, cycles)
    torch.cuda.synchronize()
    cfg = eng.config()  # the kernel the first run's tuners kept
    # the sweep kernel's duration: an otherwise identical engine whose cycle graph brackets the
    # sweep launch with CUDA events, over as many steps (the event nodes cost ~1 % of a headline
    # cycle: they keep the swap kernel from launching into the sweep's tail); capped at the
    # production engine's step time
    engp, _ = make_engine(jc, w, local, conf_base=conf_base_of(rank, w),
                          flags=jc.FLAG_PROFILE | args.flags)
    prof_total_ms, prof_ms = time_steps(torch, engp, args.steps, args.warmup, flush, cycles)
    engp.close()
    if ws > 1:
        total_ms = max_over_ranks(dist, total_ms, "cuda")
        prof_total_ms = max_over_ranks(dist, prof_total_ms, "cuda")
        prof_ms = max_over_ranks(dist, prof_ms, "cuda")
        dist.barrier()
    steps = max(args.steps, 1)
    sweep_ms_avg = min(prof_ms / steps, total_ms / steps)  # sweep kernel, per launch
    value = attempts_per_step * args.steps * ws / (total_ms * 1e6)

    # end to end through the public API with pinned host buffers: ladder H2D, one cycle, all
    # running sums and observables D2H, every step
    def pinned(nbytes):
        return torch.empty(nbytes, dtype=torch.uint8, pin_memory=True).numpy()

    h_betas = pinned(betas.nbytes).view(np.float64)
    h_betas[:] = betas
    h_sums = pinned(eng.nentries * eng.SLOT_DTYPE.itemsize).view(eng.SLOT_DTYPE)
    h_obs = pinned(eng.nentries * 5 * 8).view(np.float64).reshape(eng.nentries, 5)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        eng.set_ladder(-1, h_betas)
        eng.run(cycles, measure=True, restart_swap_phase=False)
        sums, nm = eng.slot_sums(-1, out=h_sums)
        obs = eng.observables(-1, out=h_obs)
    e2e_s = time.perf_counter() - t0
    e2e = attempts_per_step * args.steps * ws / (e2e_s * 1e9)
    h2d = h_betas.nbytes
    d2h = h_sums.nbytes + h_obs.nbytes
    assert np.isfinite(sums).all()

    pk = peaks()
    hbm = pk.get("hbm_gbs")
    peak_src = "measured" if hbm else "fallback"
    hbm = hbm or 6800.0
    bpa = B_PER_ATTEMPT_FP32 if w["precision"] == 1 else B_PER_ATTEMPT_FP64
    achieved = attempts_per_step * bpa / (sweep_ms_avg * 1e-3) / 1e9 if sweep_ms_avg > 0 else 0.0

    prec = None  # the FP32-vs-FP64 report is defined on the headline workload (shared memory)
    if wname == HEADLINE and not args.headline_only and not args.nconf:
        prec = precision_report(jc, eng, w, local, 100, 300)

    # FP64 plain form on the L=24, 16-replica PT configuration (the 10x target's denominator)
    fp64 = time_workload(torch, jc, WORKLOADS["plain_fp64_L24_1x16"], local, flush,
                         max(4, args.steps // 4))
    extra = None
    if not args.headline_only:
        extra = secondary_workloads(torch, jc, local, flush, max(5, args.steps // 10))

    cpu = cpu_baseline(w) if (rank == 0 and not args.no_cpu) else None
    clocks = clk.summary()
    config = workload_config(wname, w, ws)
    config["attempts_per_step"] = attempts_per_step * ws
    config["l2"] = "flushed before each step (256 MB written, then 256 MB read)"
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(total_ms / args.steps, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32" if w["precision"] == 1 else "f64",
        "data": "synthetic (corr_rand_3d disorder from seeds IRINIT+k, HOT starts)",
        "config": config,
        "kernel": {"block_threads": cfg["block_threads"],
                   "sites_per_thread": cfg["sites_per_thread"], "smem_bytes": cfg["smem_bytes"]},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": hbm,
                     "unit": "GB/s", "frac": round(achieved / hbm, 4),
                     "traffic": None if args.nconf else TRAFFIC.get(wname),
                     "peak_source": peak_src, "bytes_per_attempt": bpa,
                     "sweep_kernel_ms": round(sweep_ms_avg, 4),
                     "kernel_time": "CUDA events around the sweep launch in an otherwise "
                                    "identical engine (J1J2C_FLAG_PROFILE), as many steps, "
                                    "capped at ms_per_step",
                     "profiled_engine": {"ms_per_step": round(prof_total_ms / steps, 4),
                                         "sweep_ms_per_step": round(prof_ms / steps, 4)}},
        "e2e": {"value": round(e2e, 3), "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h)},
        "fp64_plain": dict(fp64, workload="plain_fp64_L24_1x16",
                           ratio_fp32_over_fp64=round(value / fp64["value"] / ws, 2)),
        "gpu_launches": 2 * args.steps,
        "clocks": clocks,
    }
    if not args.nconf and wname in NCU_ISSUE:
        line["roofline"].update(NCU_ISSUE[wname])
    if prec is not None:
        line["precision"] = prec
    if extra is not None:
        line["workloads"] = extra
    if cpu is not None:
        line["cpu_baseline"] = cpu
    eng.close()
    if rank == 0:
        print(json.dumps(line))
    if ws > 1:
        dist.destroy_process_group()


def reference_models(w, irinit=1):
    """One oracle Model per configuration of the workload, its disorder from the oracle's numpy
    restatement of corr_rand_3d (seed irinit + k, PHI=2, XI=3) and its vacancies from the
    oracle's Setup_vacancies: nothing of the engine's library is loaded."""
    from oracle import corr3d
    from oracle import oracle as O

    models, k = [], 0
    for L, n, _ in w["groups"]:
        for _ in range(n):
            seed = irinit + k
            p = corr3d.make_corr_rand_3d(L, L, L, 3.0, seed, True, 2.0).reshape(-1)
            occu = O.setup_vacancies(seed, L, L, w["vacancies"])[0] if w.get("vacancies") else None
            models.append(O.Model(L, L, p, occu))
            k += 1
    return models


def reference_steps(w, nthreads, steps, warmup=0):
    """Seconds of each of `steps` steps (after `warmup` untimed ones) of the reference CPU path on
    the workload (one PT cycle of every ladder per step; ladders round-robin over nthreads
    threads) and the attempts per step."""
    from oracle import oracle as O

    if len(w["groups"]) != 1:
        raise ValueError("the CPU path is timed on single-shape workloads")
    L, n, nrep = w["groups"][0]
    models = reference_models(w)
    betas = 1.0 / O.ladder(nrep, 8.0, 11.5) if "T" not in w else np.full(nrep, 1.0 / w["T"])
    ptswapever = w.get("ptswapever", 5)
    cycles = w.get("cycles_per_step", 1)
    for _ in range(warmup):
        O.bench_pt_multi(models, nthreads, betas, ptswapever, cycles)
    secs = [O.bench_pt_multi(models, nthreads, betas, ptswapever, cycles) for _ in range(steps)]
    attempts = sum(int(m.N - m.nimp) for m in models) * nrep * ptswapever * cycles
    return secs, attempts


def cpu_baseline(w):
    """The oracle's restatement of the reference PT cycle (sequential site order, KISS, FP64,
    neighbour tables) on all host threads: two whole PT cycles of the workload (every ladder),
    the faster one reported."""
    nthreads = os.cpu_count() or 1
    secs, attempts = reference_steps(w, nthreads, 2)
    best = min(secs)
    return {"value": round(attempts / best / 1e9, 5), "unit": UNIT, "cores": nthreads,
            "kind": "port",
            "sample": f"the whole workload, one PT cycle of all {sum(n for _, n, _ in w['groups'])}"
                      f" ladders ({attempts} attempts) in {best:.2f} s, ladders round-robin over "
                      f"{nthreads} threads; Fortran toolchain absent"}


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    w = WORKLOADS[args.workload]
    nthreads = os.cpu_count() or 1
    secs, attempts = reference_steps(w, nthreads, args.steps, args.warmup)
    total = sum(secs)
    value = attempts * args.steps / total / 1e9
    config = workload_config(args.workload, w, ws)
    config["attempts_per_step"] = attempts
    config["l2"] = "flushed before each step (256 MB written, then 256 MB read)"
    line = {"impl": "reference", "metric": METRIC, "value": round(value, 5), "unit": UNIT,
            "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(total * 1e3 / args.steps, 2), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (corr_rand_3d disorder from seeds IRINIT+k, HOT starts)",
            "config": config,
            "cpu_baseline": {"value": round(value, 5), "unit": UNIT, "cores": nthreads,
                             "kind": "port",
                             "sample": f"every step one whole PT cycle of the workload (all "
                                       f"ladders, {attempts} attempts), ladders round-robin over "
                                       f"{nthreads} threads; the reference's sequential site "
                                       "order, KISS stream and FP64 arithmetic restated in C "
                                       "(Fortran toolchain absent)"},
            "e2e": {"value": round(value, 5), "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default=HEADLINE, choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--flags", type=int, default=0,
                    help="engine flags added to the run (e.g. 16 pins the one-launch-per-colour "
                         "HBM path; for profiling captures)")
    ap.add_argument("--nconf", type=int, default=0,
                    help="configurations per lattice shape instead of the workload's (a smaller "
                         "case for profiling captures; 0: the workload's)")
    ap.add_argument("--headline-only", action="store_true",
                    help="skip the secondary workloads (batched FP64, mixed L, L=96, local)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
