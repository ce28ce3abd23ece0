"""Particle-element steps/s of HPSim's tracking path on one GB300.

Workload (one "step"): one pass of the DTL-like lattice -- 165 DTL RF gaps
(E0 = 2.5 MV/m, phi_s = -26 deg, cubic T(beta), S(beta)) between 166 quads
(0.04 m), a full SCHEFF 32x128 space-charge solve at every gap and quad --
over 1,048,576 H- macro-particles from a 6D waterbag at 0.75 MeV.  The beam
state is restored on the device before every step; the metric is
N x elements / step time.  Synthetic seeded inputs stand in for a lattice
database and a measured input beam.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
                    [--precision fp32|fp64]

Multi-GPU: every rank runs an independent replica beam (the single-beam path
has no data-parallel exchange); value = all ranks' particle-element steps /
the slowest rank's time.
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
sys.path.insert(0, ROOT)

METRIC = "particle-element steps/s"
N_PART = 1 << 20
GAPS = 165
SURROGATE_NET = os.path.join(ROOT, "hpsim_gb300", "data", "scheff_surrogate_32x128.npz")


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--precision", default=None, choices=["fp32", "fp64"])
    p.add_argument("--particles", type=int, default=None)
    p.add_argument("--gaps", type=int, default=GAPS)
    p.add_argument("--elements", type=int, default=None,
                   help="single-beam workloads: keep only the lattice's first N elements (short profiling runs)")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--workload", default="dtl_like",
                   choices=["dtl_like", "small_fodo", "ccl_large", "batched", "ccl_batch", "surrogate_net"],
                   help="dtl_like: one 1M-particle beam through 165 DTL gaps (the headline); small_fodo: "
                        "65,536 particles in FP64 through buncher + 40 FODO elements; ccl_large: 16,777,216 "
                        "particles through 1024 CCL gaps, SCHEFF 64x256; batched: 256 beams of the "
                        "small-FODO topology in one graph launch; ccl_batch: 16 beams of 1,048,576 particles "
                        "through the CCL lattice with perturbed set points in one graph launch; surrogate_net: "
                        "the learned field surrogate's forward pass at batches of 1, 8 and 32 planes, its "
                        "layers on CUDA cores and on the tensor cores")
    p.add_argument("--beams", type=int, default=None, help="batched: 256, ccl_batch: 16")
    p.add_argument("--lockstep", action="store_true",
                   help="batches run in lockstep (one launch per kernel for all beams) instead of as per-simulator "
                        "child graphs")
    p.add_argument("--surrogate", nargs="?", const=SURROGATE_NET, default=None,
                   help="small_fodo (FP64): time the plain path, then with the learned field surrogate attached "
                        "(a network file; default the shipped 32x128 network), and report both")
    p.add_argument("--surrogate-tol", type=float, default=None,
                   help="the network's spot-check tolerance: default 0.015 for the DTL-like batch (the largest "
                        "measured that meets the 1e-3 emittance gate there), 0.02 for the small_fodo ablation")
    p.add_argument("--surrogate-kernel", choices=["tensor", "cuda"], default="cuda",
                   help="the surrogate's layers on CUDA cores (default: faster at one plane) or on the tensor cores")
    p.add_argument("--no-autotune", action="store_true",
                   help="keep the default launch shapes instead of timing candidates before the warm-up")
    p.add_argument("--shape", default=None,
                   help="contraction,deposit_blocks_per_sm,sweep_blocks_per_sm[,deposit_aggregate[,deposit_threads]]: "
                        "set this launch shape instead of tuning (reproducible profiling runs)")
    p.add_argument("--tune-elements", type=int, default=60,
                   help="the autotuner times runs over the lattice's first N elements")
    p.add_argument("--surrogate-batch", type=int, default=8,
                   help="dtl_like on one GPU: also time this many set-point-perturbed beams of the same size in one "
                        "batch launch, without and with the learned field surrogate, and report the ratio to the "
                        "plain single-beam path (0: skip)")
    return p.parse_args()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def slowest(t_local, ws, device=None):
    """The largest of the ranks' times (every rank gets it); t_local alone
    when there is one rank."""
    if ws <= 1:
        return t_local
    import torch
    import torch.distributed as dist
    x = torch.tensor([t_local], dtype=torch.float64, device=device)
    dist.all_reduce(x, op=dist.ReduceOp.MAX)
    return float(x.item())


def job_value(t_step_local, ws, particles, n_elem, device=None):
    """Whole-job throughput of ws replica beams: every rank's particle-element
    steps over the slowest rank's step time.  Returns (value, that time)."""
    t = slowest(t_step_local, ws, device)
    return ws * particles * n_elem / t, t


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [s.strip() for s in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            for k, nm in enumerate(names):
                if r[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


# beam and solver of each single-beam workload: particles, precision, W0 [MeV],
# f [MHz], SCHEFF mesh (nr, nz) and kick interval [m]
WORKLOADS = {
    "dtl_like": dict(particles=N_PART, precision="fp32", w0=0.75, freq=201.25, mesh=(32, 128), interval=0.01),
    "small_fodo": dict(particles=65536, precision="fp64", w0=0.75, freq=201.25, mesh=(32, 128), interval=0.10),
    "ccl_large": dict(particles=16777216, precision="fp32", w0=100.0, freq=805.0, mesh=(64, 256), interval=0.01),
}


def resolve(args):
    """Fill the workload's defaults into --particles and --precision."""
    spec = WORKLOADS.get(args.workload, WORKLOADS["dtl_like"])
    if args.particles is None:
        args.particles = spec["particles"] if args.workload in WORKLOADS else N_PART
    if args.precision is None:
        args.precision = spec["precision"] if args.workload in WORKLOADS else "fp32"
    return spec


def workload(args):
    from hpsim_gb300 import lattices as L
    if args.workload == "small_fodo":
        elems = L.small_fodo()
    elif args.workload == "ccl_large":
        elems = L.ccl_like()
    else:
        elems = L.dtl_like(n_gaps=args.gaps)
    return elems[:args.elements] if args.elements else elems


def describe(args, n_elem):
    spec = WORKLOADS[args.workload]
    nr, nz = spec["mesh"]
    if args.workload == "small_fodo":
        lat = f"small_fodo: buncher + 20 x (0.10 m drift, 0.05 m quad, +-18 T/m)"
    elif args.workload == "ccl_large":
        lat = f"ccl_large: 4 x 32 x 8 CCL gaps at 805 MHz from 100 MeV, doublets between tanks ({n_elem} elements)"
    else:
        lat = (f"dtl_like: {args.gaps} DTL gaps (E0 2.5 MV/m, phi_s -26 deg, T(beta) and S(beta) cubics in "
               f"u = (beta - beta_g)/beta_g with coefficients drawn +-5% about (0.85, 0.40, -1.2, 0.5) and "
               f"(0.10, -0.10, 0.3, -0.1)) + {args.gaps + 1} quads of 0.04 m at +-80 T/m (not +-45 T/m: at "
               f"+-45 T/m the 15 mA beam is lost within the first tank)")
    return (f"{lat}, {args.particles} H- particles, waterbag {spec['w0']} MeV, SCHEFF {nr}x{nz} full solve at "
            f"every element")


def beam_flags(beam):
    """loss and lloss flags of every particle (host copies)."""
    import numpy as np
    from hpsim_gb300._capi import call, uptr
    out = []
    for k in (0, 1):
        a = np.empty(beam.get_size(), dtype=np.uint32)
        call("hps_beam_get_loss", beam.handle, k, uptr(a))
        out.append(a)
    return out


def make_sim(args, elems, seed):
    from hpsim_gb300 import HPSim, lattices as L
    spec = WORKLOADS[args.workload]
    beam = HPSim.Beam(mass=939.294, charge=-1.0, current=0.015, num=args.particles, precision=args.precision)
    beam.set_waterbag(*L.waterbag_twiss(w0=spec["w0"], freq=spec["freq"]), 0.0, spec["w0"], spec["freq"], seed)
    beam.set_ref_w(spec["w0"])
    beam.set_ref_phi(0.0)
    beam.save_initial_beam()
    bl = HPSim.BeamLine(elements=elems)
    sc = HPSim.SpaceCharge(*spec["mesh"], spec["interval"], 0)
    sc.set_remesh_threshold(0.0)
    sim = HPSim.Simulator(beam, bl, sc)
    return beam, bl, sc, sim


# Compulsory bytes per particle of one launch of each profiled kernel class:
# the particle arrays it must read and write.
#   FP32 beams with SCHEFF (fused sequence per element):
#     drift / gap1 half before the kick + every statistic of the kick: 6
#       coordinates and both loss flags in (32 B), x, y, phi out (12 B);
#     quad half before the kick: 32 B in, x, x', y, y', phi out (20 B);
#     sc_stats: nothing when the half before the kick certified its
#       statistics (the loss-test and moments sweeps then return at once);
#     sc_mesh (deposit; Green's table and contraction are mesh-sized): flags,
#       x, y, phi in (20 B);
#     sc_kick (kick + element half after it): 6 coordinates and both flags in
#       (32 B), 6 coordinates out (24 B).
#   FP64 beams: one kernel per class, 8-byte coordinates.
ALG_BYTES = {
    "fp32": {"drift": 44, "gap1": 44, "quad": 52, "sc_stats": 0, "sc_mesh": 20, "sc_kick": 56,
             "gap2": 2 * 6 * 4 + 4, "other": 2 * 6 * 4 + 8, "monitor": 32},
    "fp64": {"gap2": 2 * 6 * 8 + 4, "gap1": 6 * 8 + 4 + 3 * 8, "quad": 6 * 8 + 4 + 5 * 8, "drift": 5 * 8 + 4 + 3 * 8,
             "sc_kick": 6 * 8 + 8 + 3 * 8, "sc_stats": 3 * 8 + 4 * 8 + 8 * 2, "sc_mesh": 3 * 8 + 8,
             "other": 2 * 6 * 8 + 8, "monitor": 64},
}
# Minimum traffic of a particle-element step: one read and write of the six
# coordinates plus both loss flags read (2 * 6 * s + 8 bytes).
STEP_BYTES = {"fp32": 56, "fp64": 104}
PHASE_KERNELS = {
    "fp32": {"quad": "pass_kernel_f<OpPushScStats<QuadMap>>", "gap1": "pass_kernel_f<OpPushScStats<Gap1Map>>",
             "drift": "pass_kernel_f<OpPushScStats<DriftMap>>",
             "sc_stats": "pass_kernel_f<Op32LlossScStats> (returns at once when the sweep before the kick "
                         "certified its statistics)",
             "sc_mesh": "k32_green + k32_green_deposit + k_contract_m | k_contract_tc + k_tc_reduce", "sc_kick": "k32_kick_push<QuadMap|Gap2Map|DriftMap>"},
    "fp64": {},
}


def algorithmic_bytes(phase, n, prec):
    """Compulsory bytes of one launch of a profiled kernel class."""
    return ALG_BYTES[prec].get(phase, STEP_BYTES[prec]) * n


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            pk = json.load(fh)
        return float(pk["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def load_traffic(phase, prec, n):
    """DRAM bytes per launch of a kernel class from an ncu capture at
    1048576 particles, scaled to n particles (the sweeps' traffic grows in
    proportion)."""
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as fh:
            t = json.load(fh)
        v = t.get(f"{prec}:{phase}")
        return None if v is None else v * n / 1048576
    except (OSError, ValueError):
        return None


def oracle_sim(args, elems, seed=12345):
    """The FP64 oracle's beam and simulator for the workload (waterbag of the
    same seed as the GPU beam of rank 0; set-up is not timed)."""
    from hpsim_gb300 import lattices as L
    from oracle import oracle as O
    types, params, _ = L.lattice_arrays(elems)
    spec = WORKLOADS[args.workload]
    b = O.Beam(args.particles)
    b.set_waterbag(L.waterbag_twiss(w0=spec["w0"], freq=spec["freq"]), 0.0, spec["w0"], spec["freq"], seed)
    b.set_ref_w(spec["w0"])
    b.set_ref_phi(0.0)
    sp = O.Scheff(*spec["mesh"], spec["interval"], 0)
    sp.set(remesh_threshold=0.0)
    return b, O.Sim(b, types, params, sp)


def cpu_baseline(args, elems, budget_s=12.0, min_s=10.0, impl_kind="port", keep_first=False):
    """The FP64 oracle (oracle/, OpenMP over all host cores) on a bounded
    sample of the same workload at the same particle count: passes of the
    lattice from a fresh beam, element by element, until at least min_s of
    oracle time (at most budget_s; a long lattice stops inside its first
    pass).  Beam setup is not timed.  keep_first: the first pass's monitor
    records and final loss flags are returned too (key "first"), when that
    pass covered the whole lattice."""
    from oracle import oracle as O
    O.build()
    threads = os.cpu_count() or 1
    O.lib().orc_set_threads(threads)
    done = passes = 0
    dt = 0.0
    first = None
    while True:  # at least one pass
        b, sim = oracle_sim(args, elems)
        t0 = time.perf_counter()
        stopped = False
        for i in range(len(elems)):
            sim.simulate(i, i)
            done += 1
            if dt + time.perf_counter() - t0 > budget_s:
                stopped = i + 1 < len(elems)
                break
        dt += time.perf_counter() - t0
        passes += 1
        if keep_first and passes == 1 and not stopped:
            first = (sim.mon.copy(), b.arr("loss").copy(), b.arr("lloss").copy())
        if stopped or dt > budget_s or dt >= min_s:
            break
    what = (f"{passes} passes of all {len(elems)} elements" if done == passes * len(elems)
            else f"the first {done} of {len(elems)} elements" if passes == 1
            else f"{done} element steps over {passes} passes of {len(elems)} elements")
    out = {"value": args.particles * done / dt, "unit": METRIC, "cores": threads, "kind": impl_kind,
           "sample": f"{args.particles} particles x {what}, FP64 oracle, {dt:.1f} s",
           "whole_passes": done == passes * len(elems)}
    if keep_first:
        out["first"] = first
    return out


# monitor columns (include/hps_layout.h): centroid -> its sigma, sigmas,
# emittances, synchronous particle
MON_CENTROIDS = {2: 3, 4: 5, 7: 8, 9: 10, 12: 13, 14: 15}
MON_SIGMAS = (3, 5, 8, 10, 13, 15)
MON_EMITS = {"eps_x": 6, "eps_y": 11, "eps_z": 16}
EMIT_GATE = 1e-3


def accuracy(mon, ref, loss, ref_loss, lloss, ref_lloss):
    """Per-element agreement of a GPU pass with the FP64 oracle's pass of the
    same beam: transmission (particles alive after every element), loss and
    longitudinal-loss flags of every particle, and the largest relative
    error over the elements of the emittances, the rms sizes, the centroids
    (in units of their rms size) and particle 0's energy and phase.  The
    gate: emittances within 1e-3 relative, transmission and flags exact."""
    import numpy as np
    m, r = np.asarray(mon, float), np.asarray(ref, float)

    def rel(a, b):
        ok = np.abs(b) > 0
        if not ok.any():
            return 0.0, -1
        e = np.zeros(len(b))
        e[ok] = np.abs(a[ok] - b[ok]) / np.abs(b[ok])
        k = int(np.argmax(e))
        return float(e[k]), k

    err, at = {}, {}
    for name, col in MON_EMITS.items():
        err[name], at[name] = rel(np.nan_to_num(m[:, col]), np.nan_to_num(r[:, col]))
    err["sigma"] = max(rel(m[:, c], r[:, c])[0] for c in MON_SIGMAS)
    cen = 0.0
    for a, sc in MON_CENTROIDS.items():
        sig = np.abs(r[:, sc])
        ok = sig > 0
        if ok.any():
            cen = max(cen, float(np.max(np.abs(m[ok, a] - r[ok, a]) / sig[ok])))
    err["centroid_over_sigma"] = cen
    err["w0"] = rel(m[:, 17], r[:, 17])[0]
    err["phi0"] = rel(m[:, 18], r[:, 18])[0]
    out = {"transmission_equal": bool(np.array_equal(m[:, 0], r[:, 0])),
           "good_count_equal": bool(np.array_equal(m[:, 1], r[:, 1])),
           "loss_flags_equal": bool(np.array_equal(loss, ref_loss)),
           "lloss_equal": bool(np.array_equal(lloss, ref_lloss)),
           "transmitted": int(m[-1, 0]), "elements": int(len(m)),
           "max_rel_err": err, "worst_element": at}
    out["gate"] = {"emittance_rel_max": EMIT_GATE,
                   "pass": bool(out["transmission_equal"] and out["loss_flags_equal"] and out["lloss_equal"]
                                and max(err[k] for k in MON_EMITS) <= EMIT_GATE)}
    return out


def run_reference(args):
    """The reference's CPU path (the FP64 oracle, all host cores) on the same
    workload: each step is one whole pass of the lattice over the full beam
    when the warm-up pass shows it takes at most 8 s, else a prefix of the
    lattice bounded to 8 s whose time is scaled to the whole lattice."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    elems = workload(args)
    per_step = 8.0
    for _ in range(args.warmup):
        cpu_baseline(args, elems, budget_s=per_step, min_s=0.0)
    vals, times, prefix = [], [], False
    r = None
    for _ in range(args.steps):
        r = cpu_baseline(args, elems, budget_s=per_step, min_s=0.0)
        vals.append(r["value"])
        times.append(args.particles * len(elems) / r["value"])
        prefix |= not r["whole_passes"]
    v = args.steps / sum(1.0 / x for x in vals)
    note = " (time scaled from bounded prefixes of the lattice)" if prefix else ""
    line = {"metric": METRIC, "value": v, "unit": METRIC, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000 * statistics.mean(times), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": describe(args, len(elems)) + note,
                       "particles": args.particles, "elements": len(elems), "precision": "fp64"},
            "cpu_baseline": {"value": v, "unit": METRIC, "cores": r["cores"], "kind": "port",
                             "sample": f"{args.steps} steps, each {r['sample']}"},
            "e2e": {"value": v, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def surrogate_batched(args, plain_value, local, flush, net_path, tol):
    """Surrogate + batched against plain SCHEFF on the DTL-like workload: B
    beams of the same particle count with per-beam perturbed set points
    (lattices.dtl_batch) in one batch graph launch, timed without and then
    with the learned field surrogate attached to every solver (the same
    timing as the headline: L2 flushed, CUDA events around the launch).
    Beam 0 of the surrogate run is then checked against the FP64 oracle on
    the same lattice and seed (transmission, flags, emittances).  Returns
    the record of the bench line's "surrogate_batched" key."""
    import numpy as np
    import torch
    from hpsim_gb300 import HPSim, lattices as L
    base = L.dtl_like(n_gaps=args.gaps)
    scan = L.dtl_batch(args.surrogate_batch, num=args.particles)
    spec = WORKLOADS["dtl_like"]
    objs = []
    for sb in scan:
        beam = HPSim.Beam(mass=939.294, charge=-1.0, current=0.015, num=sb.num, precision="fp32")
        beam.set_waterbag(*L.waterbag_twiss(w0=spec["w0"], freq=spec["freq"]), 0.0, spec["w0"], spec["freq"],
                          sb.seed)
        beam.set_ref_w(spec["w0"])
        beam.set_ref_phi(0.0)
        beam.save_initial_beam()
        bl = HPSim.BeamLine(elements=L.perturbed(base, sb))
        sc = HPSim.SpaceCharge(*spec["mesh"], spec["interval"], 0)
        sc.set_remesh_threshold(0.0)
        objs.append((beam, bl, sc, HPSim.Simulator(beam, bl, sc)))
    batch = HPSim.Batch([o[3] for o in objs])
    batch.set_lockstep(args.lockstep)
    n_elem = len(base)
    total = sum(sb.num for sb in scan)
    tune = None
    if not args.no_autotune:
        tune = batch.autotune(0, min(n_elem, args.tune_elements) - 1, reps=2)

    def step():
        for o in objs:
            o[0].restore_initial_beam()
        batch.simulate()
        return batch.last_time_ms()

    def timed():
        for _ in range(args.warmup):
            flush.zero_()
            step()
        ms = []
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            ms.append(step())
        return total * n_elem / (sum(ms) / len(ms) / 1000.0), sum(ms) / len(ms)

    def beam0_monitor():
        sim0 = objs[0][3]
        sim0.enable_monitor(True)
        step()
        mon = sim0.monitor.copy()
        sim0.enable_monitor(False)
        return mon

    plain_b, plain_ms = timed()
    plain_mode = batch.last_mode()
    mon_plain = beam0_monitor()
    net = np.load(net_path)
    for o in objs:
        o[2].set_surrogate(net, tol=tol)
        o[2].set_surrogate_kernel(args.surrogate_kernel)
    stats0 = [o[2].surrogate_stats() for o in objs]
    sur_b, sur_ms = timed()
    sur_mode = batch.last_mode()
    stats1 = [o[2].surrogate_stats() for o in objs]
    acc_n = sum(b[0] - a[0] for a, b in zip(stats0, stats1)) / args.steps / len(objs)
    rej_n = sum(b[1] - a[1] for a, b in zip(stats0, stats1)) / args.steps / len(objs)
    mon_sur = beam0_monitor()
    loss_sur, lloss_sur = beam_flags(objs[0][0])
    rel = lambda i: float(np.max(np.abs(np.nan_to_num(mon_sur[:, i]) / np.nan_to_num(mon_plain[:, i]) - 1.0)))  # noqa: E731
    out = {"beams": len(objs), "particles_per_beam": args.particles, "elements": n_elem,
           "lattice": "dtl_like with per-beam RF amplitude x U(0.99, 1.01), RF phase offset U(-1, +1) deg, "
                      "quad gradients x U(0.97, 1.03)",
           "network": os.path.relpath(net_path, ROOT), "tol": tol, "layers": args.surrogate_kernel,
           "launch_shape": objs[0][3].get_shape(), "autotune": tune,
           "batch_form": {"plain": plain_mode[0], "surrogate": sur_mode[0], "surrogate_why": sur_mode[1] or None},
           "plain_single_value": plain_value, "plain_batched_value": plain_b, "plain_batched_ms_per_step": plain_ms,
           "surrogate_batched_value": sur_b, "surrogate_batched_ms_per_step": sur_ms,
           "surrogate_batched_over_plain": sur_b / plain_value, "plain_batched_over_plain": plain_b / plain_value,
           "kicks_per_beam_step": n_elem, "accepted_per_beam_step": acc_n, "fallbacks_per_beam_step": rej_n,
           "fallback_rate": rej_n / max(acc_n + rej_n, 1e-30),
           "surrogate_vs_plain_beam0": {"transmission_equal": bool(np.array_equal(mon_sur[:, 0], mon_plain[:, 0])),
                                        "emittance_rel_err_max": {"x": rel(6), "y": rel(11), "z": rel(16)}},
           "target": ">= 5x the plain path at <= 1e-3 relative rms-emittance error and exact transmission"}
    return out, (scan[0], L.perturbed(base, scan[0]), mon_sur, loss_sur, lloss_sur)


def surrogate_accuracy(args, check):
    """Beam 0 of the surrogate batch against the FP64 oracle's pass of the
    same beam through the same lattice."""
    from hpsim_gb300 import lattices as L
    from oracle import oracle as O
    sb, elems, mon, loss, lloss = check
    spec = WORKLOADS["dtl_like"]
    O.build()
    O.lib().orc_set_threads(os.cpu_count() or 1)
    types, params, _ = L.lattice_arrays(elems)
    b = O.Beam(sb.num)
    b.set_waterbag(L.waterbag_twiss(w0=spec["w0"], freq=spec["freq"]), 0.0, spec["w0"], spec["freq"], sb.seed)
    b.set_ref_w(spec["w0"])
    b.set_ref_phi(0.0)
    sp = O.Scheff(*spec["mesh"], spec["interval"], 0)
    sp.set(remesh_threshold=0.0)
    sim = O.Sim(b, types, params, sp)
    sim.simulate()
    return accuracy(mon, sim.mon.copy(), loss, b.arr("loss").copy(), lloss, b.arr("lloss").copy())


def run_surrogate_net(args):
    """The surrogate network's forward pass (ten layers, random weights of the
    shipped architecture, 128 x 32 planes) at batches of 1, 8 and 32 planes,
    captured as one CUDA graph per variant and timed with CUDA events over
    max(--steps, 20) replays after --warmup: the layers on CUDA cores
    (hps_nn_conv_forward) and on the tensor cores (hps_nn_conv_forward_tiles,
    weight tiles laid out once).  value = the tensor-core forward time at
    batch 32 (ms, lower is better); the table is under "forward_ms"."""
    import ctypes as C
    import numpy as np
    import torch
    from hpsim_gb300 import HPSim, build, surrogate as S  # noqa: F401
    from hpsim_gb300._capi import call
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    build.build()
    HPSim.set_gpu(local)

    def ptr(t):
        return C.c_void_p(t.data_ptr())

    rng = np.random.default_rng(0)
    table = {}
    for B in (1, 8, 32):
        shapes = S.layer_shapes(B)
        wts = [torch.tensor(rng.normal(size=(co, ci, 3, 3)) / np.sqrt(9 * ci), dtype=torch.bfloat16, device="cuda")
               for ci, co, *_ in S.ARCH]
        bias = [torch.zeros(co, device="cuda") for _, co, *_ in S.ARCH]
        x = torch.randn(B, 2, S.NZ, S.NR, device="cuda").to(torch.bfloat16)
        acts, tiles = [], []
        for d, w in zip(shapes, wts):
            b_, ci, co, h, wd, s, u = (int(v) for v in d)
            acts.append(torch.empty(b_, co, (h * u - 1) // s + 1, (wd * u - 1) // s + 1, dtype=torch.bfloat16,
                                    device="cuda"))
            nb = C.c_uint64()
            call("hps_nn_conv_tc_tile_bytes", d.ctypes.data_as(C.POINTER(C.c_int)), C.byref(nb))
            t = torch.empty(int(nb.value), dtype=torch.uint8, device="cuda")
            call("hps_nn_conv_tc_prepare", d.ctypes.data_as(C.POINTER(C.c_int)), ptr(w), ptr(t), None)
            tiles.append(t)
        err = torch.zeros(1, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        cs = torch.cuda.Stream()

        def net(tc):
            st = C.c_void_p(cs.cuda_stream)
            cur = x
            for l, (d, w, b, a, t) in enumerate(zip(shapes, wts, bias, acts, tiles)):
                skip = acts[S.SKIP[l]] if l in S.SKIP else None
                dp = d.ctypes.data_as(C.POINTER(C.c_int))
                if tc:
                    call("hps_nn_conv_forward_tiles", dp, ptr(cur), ptr(t), ptr(b), int(S.ARCH[l][4]),
                         None if skip is None else ptr(skip), ptr(a), ptr(err), st)
                else:
                    call("hps_nn_conv_forward", dp, ptr(cur), ptr(w), ptr(b), int(S.ARCH[l][4]),
                         None if skip is None else ptr(skip), ptr(a), st)
                cur = a

        for tc in (False, True):
            g = torch.cuda.CUDAGraph()
            with torch.cuda.stream(cs):
                net(tc)  # untimed run outside the capture (kernel attributes, lazy loading)
                with torch.cuda.graph(g, stream=cs):
                    net(tc)
            for _ in range(max(3, args.warmup)):
                g.replay()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            reps = max(args.steps, 20)
            e0.record()
            for _ in range(reps):
                g.replay()
            e1.record()
            torch.cuda.synchronize()
            table[f"{'tensor' if tc else 'cuda'}_b{B}"] = e0.elapsed_time(e1) / reps
        if int(err.item()):
            raise SystemExit("surrogate_net: a tensor-core layer's pipeline wait timed out")
    if rank != 0:
        return
    line = {"metric": "surrogate network forward time, batch 32, tensor-core layers", "value": table["tensor_b32"],
            "unit": "ms", "n_gpus": 1, "steps": max(args.steps, 20), "warmup": args.warmup,
            "ms_per_step": table["tensor_b32"], "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "bf16", "data": "synthetic (random weights of the shipped architecture, random planes)",
            "config": {"workload": "surrogate_net: ten 3x3 conv layers (32-64-128-128-128 down, 128-128-64-32 up, "
                                   "2 out) on 128 x 32 planes, one CUDA graph per variant",
                       "forward_ms": {k: round(v, 4) for k, v in table.items()}},
            "e2e": None, "gpu_launches": 10}
    print(json.dumps(line), flush=True)


def run_batched(args):
    """Independent beams advanced by one graph launch per step; value = all
    beams' particle-element steps / step time.  batched: beams of uneven
    sizes with perturbed RF and quad set points on the small-FODO topology
    (lattices.batched_scan); ccl_batch: equal 1,048,576-particle beams
    through the CCL-like lattice with perturbed set points
    (lattices.ccl_batch)."""
    import torch
    from hpsim_gb300 import HPSim, build, lattices as L
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    build.build()
    HPSim.set_gpu(local)
    ccl = args.workload == "ccl_batch"
    if args.beams is None:
        args.beams = 16 if ccl else 256
    if ccl:
        scan = L.ccl_batch(args.beams)
        base = L.ccl_like()
        spec = WORKLOADS["ccl_large"]
        lattice = lambda sb: L.perturbed(base, sb)  # noqa: E731
    else:
        scan = L.batched_scan(args.beams)
        spec = WORKLOADS["small_fodo"]
        lattice = L.scan_lattice
    w0, freq = spec["w0"], spec["freq"]
    # with N ranks each GPU takes its share of the beams, balanced by particle
    # count; the beams are independent, so no collective touches the data
    if ws > len(scan):
        raise SystemExit(f"--beams {len(scan)} is fewer than the {ws} ranks: every rank needs at least one beam")
    mine = L.partition_beams([sb.num for sb in scan], ws)[rank]
    all_total = sum(sb.num for sb in scan)
    scan = [scan[i] for i in mine]
    objs = []
    for sb in scan:
        beam = HPSim.Beam(mass=939.294, charge=-1.0, current=0.015, num=sb.num, precision=args.precision)
        beam.set_waterbag(*L.waterbag_twiss(w0=w0, freq=freq), 0.0, w0, freq, sb.seed)
        beam.set_ref_w(w0)
        beam.set_ref_phi(0.0)
        beam.save_initial_beam()
        bl = HPSim.BeamLine(elements=lattice(sb))
        sc = HPSim.SpaceCharge(*spec["mesh"], spec["interval"], 0)
        sc.set_remesh_threshold(0.0)
        objs.append((beam, bl, sc, HPSim.Simulator(beam, bl, sc)))
    batch = HPSim.Batch([o[3] for o in objs])
    batch.set_lockstep(args.lockstep)
    n_elem = len(objs[0][1])
    total = sum(sb.num for sb in scan)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{local}")
    tune = None
    if not args.no_autotune:
        t0 = time.perf_counter()
        tune = batch.autotune(0, min(n_elem, args.tune_elements) - 1, reps=2)
        tune["seconds"] = time.perf_counter() - t0
        tune["elements"] = min(n_elem, args.tune_elements)

    def step():
        for o in objs:
            o[0].restore_initial_beam()
        batch.simulate()
        return batch.last_time_ms()

    for _ in range(args.warmup):
        step()
    launches0 = HPSim.kernel_launch_count()
    ms = []
    torch.cuda.synchronize()
    if ws > 1:
        torch.distributed.barrier()
    with ClockSampler(local) as clocks:
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            ms.append(step())
    torch.cuda.synchronize()
    if ws > 1:
        torch.distributed.barrier()
    launches = HPSim.kernel_launch_count() - launches0
    mode = batch.last_mode()
    t = slowest(sum(ms) / len(ms) / 1000.0, ws, device=f"cuda:{local}")
    # the same step in the other batch form, for comparison
    batch.set_lockstep(not args.lockstep)
    for _ in range(2):
        step()
    other_ms = []
    for _ in range(max(1, min(args.steps, 3))):
        flush.zero_()
        torch.cuda.synchronize()
        other_ms.append(step())
    other_mode = batch.last_mode()
    t_other = slowest(sum(other_ms) / len(other_ms) / 1000.0, ws, device=f"cuda:{local}")
    batch.set_lockstep(args.lockstep)
    # the same step with one simulate() per beam, one after another (each its
    # own graph launch), for comparison
    for o in objs:
        o[0].restore_initial_beam()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for o in objs:
        o[3].simulate()
    t_seq = slowest(time.perf_counter() - t0, ws, device=f"cuda:{local}")
    if rank != 0:
        torch.distributed.destroy_process_group()
        return
    total = all_total
    line = {"metric": METRIC, "value": total * n_elem / t, "unit": METRIC, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000 * t, "higher_is_better": True, "scaling": "strong",
            "vs_baseline": None, "dtype": "f32" if args.precision == "fp32" else "f64", "data": "synthetic",
            "config": {"workload": (f"CCL batch: {args.beams} beams of {scan[0].num} particles (total {total}), "
                                    f"CCL-like lattice ({n_elem} elements) with per-beam RF amplitude scale, "
                                    f"RF phase offset and quad scale, SCHEFF 64x256 at every element, one graph "
                                    f"launch per step") if ccl else
                                   (f"batched scan: {args.beams} beams, particles log-uniform in [16384, 524288] "
                                    f"(total {total}), small-FODO topology ({n_elem} elements) with per-beam RF "
                                    f"scale, phase offset and quad scale, SCHEFF 32x128 at every element, one "
                                    f"graph launch per step"), "beams": args.beams, "particles": total,
                       "parallelism": f"beams partitioned over {ws} GPU(s), balanced by particle count",
                       "elements": n_elem, "precision": args.precision,
                       "l2": "flushed between steps (256 MB write)",
                       "launch_shape": objs[0][3].get_shape(), "autotune": tune,
                       "batch_form": {"mode": mode[0], "why_not_lockstep": mode[1] or None}},
            "other_batch_form": {"mode": other_mode[0], "ms_per_step": 1000 * t_other,
                                 "value": all_total * n_elem / t_other},
            "sequential": {"ms_per_step": 1000 * t_seq, "value": total * n_elem / t_seq,
                           "note": "one simulate() per beam in turn, wall clock"},
            "e2e": None, "gpu_launches": int(launches), "clocks": clocks.summary()}
    print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


def main():
    args = parse()
    resolve(args)
    if args.impl == "reference":
        run_reference(args)
        return
    if args.workload in ("batched", "ccl_batch"):
        run_batched(args)
        return
    if args.workload == "surrogate_net":
        run_surrogate_net(args)
        return
    ws, rank, local = dist_env()
    import numpy as np
    import torch
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from hpsim_gb300 import HPSim, build
    build.build()
    HPSim.set_gpu(local)
    elems = workload(args)
    n_elem = len(elems)
    beam, bl, sc, sim = make_sim(args, elems, seed=12345 + rank)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{local}")
    tune = None
    if args.shape:
        sim.set_shape(dict(zip(HPSim.Simulator.SHAPE_KEYS, (int(v) for v in args.shape.split(",")))))
    elif not args.no_autotune:
        t0 = time.perf_counter()
        tune = sim.autotune(0, min(n_elem, args.tune_elements) - 1, reps=3)
        tune["seconds"] = time.perf_counter() - t0
        tune["elements"] = min(n_elem, args.tune_elements)

    def barrier():
        torch.cuda.synchronize()
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    def step():
        beam.restore_initial_beam()
        sim.simulate()
        return sim.last_time_ms()

    def monitored():
        sim.enable_monitor(True)
        step()
        mon = sim.monitor.copy()
        sim.enable_monitor(False)
        return mon

    sur = None
    if args.surrogate:
        if args.workload != "small_fodo":
            raise SystemExit("--surrogate: the field surrogate is trained for the small_fodo mesh (FP64 beams)")
        # the plain path first, timed the same way, and its moments per element
        for _ in range(args.warmup):
            flush.zero_()
            step()
        barrier()
        plain_ms = []
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            plain_ms.append(step())
        plain_value, _ = job_value(sum(plain_ms) / len(plain_ms) / 1000.0, ws, args.particles, n_elem,
                                   device=f"cuda:{local}")
        mon_plain = monitored()
        net = np.load(args.surrogate)
        tol = 0.02 if args.surrogate_tol is None else args.surrogate_tol
        sc.set_surrogate(net, tol=tol)
        sc.set_surrogate_kernel(args.surrogate_kernel)
        sur = {"network": os.path.relpath(args.surrogate, ROOT), "tol": tol, "layers": args.surrogate_kernel,
               "plain_value": plain_value, "plain_ms_per_step": sum(plain_ms) / len(plain_ms),
               "network_val_field_err_median": float(net["meta_val_median"]) if "meta_val_median" in net else None}

    for _ in range(args.warmup):
        flush.zero_()
        step()
    launches0 = HPSim.kernel_launch_count()
    sweeps0 = sc.get_counter("stat_sweeps")
    sur0 = sc.surrogate_stats() if sur else None
    barrier()
    dev_ms = []
    wall0 = time.perf_counter()
    with ClockSampler(local) as clocks:
        for _ in range(args.steps):
            flush.zero_()          # L2 flush between steps (256 MB > 129 MB L2)
            torch.cuda.synchronize()
            dev_ms.append(step())
    barrier()
    wall = time.perf_counter() - wall0
    launches = HPSim.kernel_launch_count() - launches0
    stat_sweeps = (sc.get_counter("stat_sweeps") - sweeps0) / args.steps
    value, t_step = job_value(sum(dev_ms) / len(dev_ms) / 1000.0, ws, args.particles, n_elem,
                              device=f"cuda:{local}")
    if sur:
        acc, rej, _ = sc.surrogate_stats()
        mon_sur = monitored()
        rel = lambda i: float(np.max(np.abs(mon_sur[:, i] / mon_plain[:, i] - 1.0)))  # noqa: E731
        sur.update({"gain": value / sur["plain_value"],
                    "accepted_per_step": (acc - sur0[0]) / args.steps,
                    "fallbacks_per_step": (rej - sur0[1]) / args.steps,
                    "emittance_rel_err_max": {"x": rel(6), "y": rel(11), "z": rel(16)},
                    "transmission_equal": bool(np.array_equal(mon_sur[:, 0], mon_plain[:, 0]))})

    # per-phase breakdown of one more (untimed) step: dominant kernel + roofline
    sim.profile(True)
    sim.profile_read(reset=True)
    step()
    prof = sim.profile_read(reset=True)
    sim.profile(False)
    dom = max(prof, key=lambda k: prof[k][0])
    dom_ms, dom_n = prof[dom]
    per_launch_s = dom_ms / 1000.0 / max(dom_n, 1)
    peak, peak_kind = load_peaks()
    achieved = algorithmic_bytes(dom, args.particles, args.precision) / per_launch_s / 1e9
    traffic = load_traffic(dom, args.precision, args.particles)
    # the whole step against the minimum traffic of a particle-element step
    step_gbs = value / ws * STEP_BYTES[args.precision] / 1e9

    # end to end through the public API with host buffers
    e2e = None
    if not args.no_e2e:
        n = args.particles
        pin = lambda dt: torch.empty(n, dtype=dt, pin_memory=True).numpy()  # noqa: E731
        beam.restore_initial_beam()
        host_in = {k: pin(torch.float64) for k in ("x", "xp", "y", "yp", "phi", "w")}
        for k in host_in:
            host_in[k][:] = beam._coord(k)
        loss_in, lloss_in = pin(torch.int32).view(np.uint32), pin(torch.int32).view(np.uint32)
        loss_in[:] = 0
        lloss_in[:] = 0
        host_out = {k: pin(torch.float64) for k in ("x", "xp", "y", "yp", "phi", "w")}
        loss_out = pin(torch.int32).view(np.uint32)
        from hpsim_gb300._capi import call, dptr, uptr
        ref_w, ref_phi = beam.get_ref_w(), beam.get_ref_phi()

        def e2e_step():
            call("hps_beam_set_distribution", beam.handle, *[dptr(host_in[k]) for k in host_in],
                 uptr(loss_in), uptr(lloss_in))
            beam.set_ref_w(ref_w)
            beam.set_ref_phi(ref_phi)
            sim.simulate()
            for k, c in zip(host_out, range(6)):
                call("hps_beam_get_coord", beam.handle, c, dptr(host_out[k]))
            call("hps_beam_get_loss", beam.handle, 0, uptr(loss_out))

        e2e_step()
        barrier()
        t0 = time.perf_counter()
        ek = max(1, min(args.steps, 3))
        for _ in range(ek):
            e2e_step()
        barrier()
        te_value, _ = job_value((time.perf_counter() - t0) / ek, ws, n, n_elem, device=f"cuda:{local}")
        e2e = {"value": te_value, "unit": METRIC, "h2d_bytes_per_step": n * (6 * 8 + 4 + 4),
               "d2h_bytes_per_step": n * (6 * 8 + 4)}

    # one more (untimed) pass from the initial beam with per-element records,
    # for the accuracy check against the FP64 oracle's pass of the same beam
    mon_gpu = monitored()
    loss_gpu, lloss_gpu = beam_flags(beam)

    # the headline comparison: surrogate + batched against the plain path
    sb_rec = sb_check = None
    if args.workload == "dtl_like" and args.surrogate_batch > 0 and ws == 1 and not args.surrogate:
        sb_tol = 0.015 if args.surrogate_tol is None else args.surrogate_tol
        sb_rec, sb_check = surrogate_batched(args, value, local, flush, SURROGATE_NET, sb_tol)

    if rank != 0:
        return
    cpu = acc = None
    if not args.no_cpu_baseline:
        cpu = cpu_baseline(args, elems, keep_first=True)
        first = cpu.pop("first")
        if first is not None:
            acc = accuracy(mon_gpu, first[0], loss_gpu, first[1], lloss_gpu, first[2])
            acc["oracle"] = "FP64 oracle, same waterbag seed and lattice, one whole pass"
        else:
            acc = {"skipped": "the oracle's first pass did not cover the whole lattice within its time bound"}
        cpu.pop("whole_passes", None)
    ck = clocks.summary()
    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000 * t_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32" if args.precision == "fp32" else "f64", "data": "synthetic",
        "config": {"workload": describe(args, n_elem),
                   "particles": args.particles, "elements": n_elem, "precision": args.precision,
                   "parallelism": f"replicas x{ws}", "l2": "flushed between steps (256 MB write)",
                   "wall_s": wall, "sc_kicks_per_step": n_elem,
                   "sc_uncertified_kicks_per_step": stat_sweeps,
                   "launch_shape": sim.get_shape(), "autotune": tune},
        "roofline": {"bound": "hbm", "kernel_phase": dom,
                     "kernels": PHASE_KERNELS[args.precision].get(dom, dom),
                     "bytes_per_particle": ALG_BYTES[args.precision].get(dom, STEP_BYTES[args.precision]),
                     "achieved": achieved, "peak": peak,
                     "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "launch_ms": per_launch_s * 1000.0,
                     "step": {"bytes_per_particle_element": STEP_BYTES[args.precision], "achieved": step_gbs,
                              "frac": step_gbs / peak},
                     "phases_ms_per_step": {k: round(v[0], 4) for k, v in prof.items()}},
        "cpu_baseline": cpu,
        "e2e": e2e,
        "gpu_launches": int(launches),
        "clocks": ck,
    }
    if acc is not None:
        line["accuracy"] = acc
    if sb_rec is not None:
        if not args.no_cpu_baseline:
            sb_rec["accuracy_vs_oracle_beam0"] = surrogate_accuracy(args, sb_check)
            a = sb_rec["accuracy_vs_oracle_beam0"]
            sb_rec["target_met"] = bool(sb_rec["surrogate_batched_over_plain"] >= 5.0 and a["gate"]["pass"])
        line["surrogate_batched"] = sb_rec
    if sur:
        line["surrogate"] = sur
    print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
