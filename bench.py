"""Throughput of the GEODESIC-M CUDA backend: ns/day and pair interactions/s.

Workload (one "step" = one geodesic-BAB + RATTLE step, lib.rs:292-323): the
seeded 50,000-atom synthetic system -- jittered cubic lattice (2.15 A, +-0.3
A), serpentine bond/angle/dihedral chain, 8 Lorentz-Berthelot types, charges
+-0.5 e net zero, Coulomb and scaled 1-4 pairs (LJ 1/2.0, Coulomb 1/1.2),
cutoff 10 / switch 8 / list radius 12 A (rebuild when an atom moves > 1 A),
non-periodic 10^4 A box, Maxwell-Boltzmann 300 K, dt = 2 fs -- in mixed
precision, inputs resident on the device.  The FP64 device path is timed on
the same system for the mixed/FP64 ratio.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl cuda|reference]

--impl reference times the oracle (the FP64 C restatement of the reference
CPU path, static thread strips over all host cores) on the same workload.
With torchrun and N > 1 every rank runs an independent replica ("replicas
only": the path has no exchange step) and rank 0 prints one JSON line.
"""
import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (os.path.join(ROOT, "geodesic-m_gb300"), os.path.join(ROOT, "oracle")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

N_ATOMS = 50_000
SEED = 20261203
DT_PS = 0.002
METRIC = "ns/day & pairs/s at 50k atoms: mixed vs FP64 GPU path at ≤1e-5 rel force err"
PHYS = dict(box_size=(10000.0,) * 3, periodic=False, r_cutoff=10.0, r_skin=12.0, r_switch=8.0, coulomb=True,
            scale14_lj=0.5, scale14_coul=1.0 / 1.2, max_constr_iter=100, constr_tol=1e-10)
L2_FLUSH_BYTES = 256 << 20  # > 129 MB L2
STEP_FORMS = {"graph": 0, "persistent": 1}  # gm_step_form: GM_STEP_GRAPH, GM_STEP_PERSISTENT
# DRAM bytes (read + write) per launch of the mixed pair kernel per half-list
# pair, from one ncu capture of the 50k workload at its minimised start
# (93,729,280 + 2,589,952 B for 10,067,070 pairs); traffic grows with the
# pair count, so the bench scales it to its own count
PAIR_TRAFFIC_PER_PAIR = 96_319_232 / 10_067_070
# The dominant kernel of a step in the persistent form, step_persistent_kernel:
# ncu's DRAM read + write of one launch of the 50k workload at its minimised
# start (552.3 GB/s over 197.4 us), and that launch's algorithmic bytes
# (step_kernel_bytes of 10,067,070 pairs, 50,000 atoms, 49,999 bonds, 49,998
# angles, 49,997 dihedrals and 1-4 pairs); the bench scales the traffic by
# its own algorithmic bytes
STEP_TRAFFIC_CAPTURE = 109_037_824
STEP_BYTES_CAPTURE = 58_668_176


def step_kernel_bytes(pairs, n_atoms, topo):
    """Algorithmic bytes of one persistent step launch: the pair part (one
    int32 index per half-list pair of neighbor.rs:25-43, plus per atom the
    coordinates, charge, type, force and energy of force/nonbonded.rs:20-82:
    4 P + 52 N), the bonded part (8 B of indices per bond, 12 per angle, 16
    per dihedral, 8 per 1-4 pair: one per dihedral of the chain; 24 B of force
    traffic per atom), and per atom the integrator phase's reads (position,
    velocity, force, inverse mass, build reference, slot, charge word, system:
    120 B) and writes (position, velocity, drift reference, the packed
    coordinate record, the cleared force: 128 B)."""
    nb, na, nd = len(topo.bond_i), len(topo.angle_i), len(topo.dihed_i)
    return 4 * pairs + 52 * n_atoms + 8 * nb + 12 * na + 16 * nd + 8 * nd + 24 * n_atoms + 248 * n_atoms


def ns_per_day(steps, seconds):
    return DT_PS * 1e-3 * steps / seconds * 86400.0


def replica_seed(rank):
    """Each rank's replica is its own seeded system."""
    return SEED + rank


def max_over_ranks(sec, device):
    """The timed span of the slowest rank, on every rank (one MAX all-reduce
    in whatever process group is initialised; the value itself without one)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return sec
    t = torch.tensor([sec], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_ns_per_day(world, steps, sec):
    """Whole-job throughput: world replicas of `steps` steps each in `sec`."""
    return world * ns_per_day(steps, sec)


def workload(rank=0):
    from geodesic_cuda import synth
    # the lattice is over-compressed for its sigma range: FIRE-minimise it
    # (1000 iterations, two stages) so NVE starts near 300 K instead of
    # converting ~25 kcal/mol/atom of compression energy into heat
    return synth.generate(N_ATOMS, seed=replica_seed(rank), temperature=300.0, relax_iters=1000)


def config_dict():
    """The workload, identical in both arms' lines."""
    return {"workload": "synthetic lattice chain, 50,000 atoms (2.15 A lattice, cube 79.6 A), FIRE-minimised "
                        "(1000 iterations) then MB 300 K, mixed precision, 2 fs BAB + RATTLE",
            "n_atoms": N_ATOMS, "seed": SEED, "cutoff_A": 10.0, "switch_A": 8.0, "list_radius_A": 12.0,
            "coulomb": True, "scale14": [0.5, 1 / 1.2], "periodic": False, "dt_fs": 2.0,
            "relaxation": "FIRE, 1000 iterations", "parallelism": "replicas, one system per GPU",
            "l2": "flushed between timed steps (256 MB memset outside the timed span)"}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        self.lines = []
        if self.proc:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [ln for ln in out.splitlines() if ln.strip()]

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in getattr(self, "lines", []):
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for k, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(k)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm), "span": "the whole CUDA arm (warm-up, timed steps, profiling loops)"}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            j = json.load(f)
        return float(j["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def pinned_like(a):
    """A pinned host copy (torch page-locked memory) viewed as numpy."""
    import torch
    t = torch.empty(a.shape, dtype=torch.float64, pin_memory=True)
    v = t.numpy()
    v[...] = a
    return t, v


def run_cuda(args, rank, world):
    """The CUDA arm; nvidia-smi samples the clocks over all of it."""
    import torch

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    atoms, topo, state, info = workload(rank)
    with ClockSampler(dev) as clk:
        line = _cuda_arm(args, rank, world, dev, atoms, topo, state)
    if line is not None:
        line["clocks"] = clk.summary()
    return line


def _cuda_arm(args, rank, world, dev, atoms, topo, state):
    import torch

    from geodesic_cuda import backend
    import oracle

    prec = backend.PRECISION_FP64 if args.precision == "fp64" else backend.PRECISION_MIXED
    p = backend.SimParams(precision=prec, device=dev, **PHYS)
    be = backend.CudaBackend(atoms, topo, p)
    form = STEP_FORMS[args.step_form]
    if prec == backend.PRECISION_MIXED:
        be.step_form(form)
    be.upload_state(np.ascontiguousarray(state.pos), np.ascontiguousarray(state.vel))
    be.forces_resident()
    if args.pair_shape:
        # a known launch shape instead of the autotuner (profiler runs, where
        # the autotuner's timings are distorted); the same bits either way
        sp, wb, gr = (int(x) for x in args.pair_shape.split(","))
        be.pair_shape(sp, wb, gr)
        tuned = {"split": sp, "warps_per_block": wb, "grid": gr, "set": "--pair-shape"}
    else:
        tuned = be.autotune(reps=3)  # pair kernel split / block size / grid, same bits for every choice
    be.run_resident(DT_PS, args.warmup)
    be.synchronize()
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=f"cuda:{dev}")
    c0 = be.counters()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    dev_ms = be.time_steps(DT_PS, args.steps, first_step=args.warmup, flush_ptr=flush.data_ptr(),
                           flush_bytes=L2_FLUSH_BYTES)
    t1 = time.perf_counter()
    torch.cuda.synchronize()
    c1 = be.counters()
    sec = max_over_ranks(dev_ms / 1e3, f"cuda:{dev}")
    pairs = c1["pairs"]
    result = dict(sec=sec, wall=t1 - t0, pairs=pairs, rebuilds=c1["rebuilds"] - c0["rebuilds"],
                  launches=c1["launches"] - c0["launches"])
    if rank != 0:
        return None
    if args.quick:
        return {"metric": METRIC, "value": round(aggregate_ns_per_day(world, args.steps, sec), 3), "unit": "ns/day",
                "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": round(1e3 * sec / args.steps, 5), "quick": True, "precision": args.precision,
                "half_list_pairs": pairs,
                "rebuilds": result["rebuilds"], "gpu_launches": int(result["launches"]),
                "kernel_ms": {"pair": round(be.profile("pair", 3), 5), "rebuild": round(be.profile("rebuild", 2), 5)},
                "autotuner": tuned}
    # steady state: 1,000 back-to-back steps, no flush (L2 keeps part of the
    # list), with the list rebuilds they meet (amortised per step)
    cb0 = be.counters()
    n_bb = 1000
    t_bb = be.time_steps(DT_PS, n_bb, first_step=args.warmup + args.steps) / 1e3
    reb_bb = be.counters()["rebuilds"] - cb0["rebuilds"]
    # roofline leg: 20 single flushed steps, each timed alone with the pair
    # count it ran on; the median (a step that rebuilt the list is an outlier)
    n_roof = 20
    roof = []
    for k in range(n_roof):
        pr = be.counters()["pairs"]
        ms = be.time_steps(DT_PS, 1, first_step=args.warmup + args.steps + n_bb + k, flush_ptr=flush.data_ptr(),
                           flush_bytes=L2_FLUSH_BYTES)
        roof.append((ms, pr))
    roof.sort()
    t_roof, pairs_roof = roof[n_roof // 2][0] / 1e3, roof[n_roof // 2][1]
    # the other step form on the same state, the same number of flushed steps
    other = "persistent" if args.step_form == "graph" else "graph"
    be.step_form(STEP_FORMS[other])
    be.run_resident(DT_PS, 3)
    be.synchronize()
    t_other = be.time_steps(DT_PS, args.steps, first_step=args.warmup + args.steps + n_bb + n_roof + 3,
                            flush_ptr=flush.data_ptr(), flush_bytes=L2_FLUSH_BYTES) / 1e3
    be.step_form(form)
    # roofline of the pair kernel: algorithmic bytes 4 P + 52 N per launch (one
    # int32 index per half-list pair of neighbor.rs:25-43, plus per atom the
    # coordinates, charge, type, force and energy of force/nonbonded.rs:20-82)
    # at the list it is timed on
    pairs_prof = be.counters()["pairs"]
    t_pair = be.profile("pair", 30) / 1e3
    t_bonded = be.profile("bonded", 30) / 1e3
    t_rebuild = be.profile("rebuild", 5) / 1e3
    # the other pieces of a step (CUDA events, warm): the 1-4 kernel, the list
    # build kernel alone, and the whole force evaluation (pack, then the pair
    # kernel beside the bonded and 1-4 kernels)
    t_pair14 = be.profile("pair14", 30) / 1e3
    t_build = be.profile("build", 5) / 1e3
    t_forces = be.profile("forces", 30) / 1e3
    alg_bytes = 4 * pairs_prof + 52 * N_ATOMS
    peak, peak_kind = measured_peaks()
    achieved = alg_bytes / t_pair / 1e9
    # the dominant kernel of the timed steps: in the persistent form each
    # timed graph launch is one step_persistent_kernel (plus the rebuild IF
    # node); its bytes and time from the roofline leg's state
    step_bytes = step_kernel_bytes(pairs_roof, N_ATOMS, topo)
    t_launch = t_roof
    # force / energy error of both device paths vs the FP64 oracle, at the
    # generator's raw lattice (before minimisation), at the minimised start
    # (step 0: net forces ~12x smaller than the individual terms, the hardest
    # case for FP32 pair math) and at the thermalised state after the timed
    # steps
    pos_end = np.ascontiguousarray(np.zeros((3, N_ATOMS)))
    vel_end = np.ascontiguousarray(np.zeros((3, N_ATOMS)))
    be.download_state(pos_end, vel_end)
    step_end = args.warmup + args.steps + n_bb
    op = oracle.make_params(box=PHYS["box_size"], periodic=False, r_cutoff=10.0, r_skin=12.0, r_switch=8.0,
                            n_threads=0, coulomb=True, scale14_lj=0.5, scale14_coul=1 / 1.2)
    errs = {}
    fp64_nsday = fp64_tuned = fp64_pair_ms = lattice = None
    from geodesic_cuda import synth
    raw = synth.generate(N_ATOMS, seed=SEED, temperature=300.0, relax_iters=0)[2].pos
    for label, pos_k in (("generator_lattice", np.ascontiguousarray(raw)), ("step0", np.ascontiguousarray(state.pos)),
                         (f"step{step_end}", pos_end)):
        pi_k, pj_k = oracle.neighbor_build(pos_k.copy(), atoms, topo, op, cells=True)
        ob = oracle.CpuBackend(atoms, topo, op)
        ob.set_pairs(pi_k, pj_k, pos_k)
        f_ref = ob.compute_forces(pos_k)
        e_ref = ob.potential_energy
        errs[label] = {}
        for name, prec in (("mixed", backend.PRECISION_MIXED), ("fp64", backend.PRECISION_FP64)):
            b2 = backend.CudaBackend(atoms, topo, backend.SimParams(precision=prec, device=dev, **PHYS))
            pp = pos_k.copy()
            b2.build_neighbor_list(pp)
            f = b2.compute_forces(pp).copy()
            if label == "generator_lattice" and prec == backend.PRECISION_MIXED:
                # the literal lattice (no relaxation): its pair count and the
                # mixed pair kernel's time on it, beside the timed state's
                b2.upload_state(np.ascontiguousarray(raw), np.ascontiguousarray(state.vel))
                b2.forces_resident()
                b2.autotune(reps=3)
                lattice = {"half_list_pairs": int(b2.counters()["pairs"]),
                           "pair_kernel_ms": round(b2.profile("pair", 20), 5)}
            errs[label][name] = dict(
                force_rel_l2=float(np.linalg.norm(f - f_ref) / np.linalg.norm(f_ref)),
                force_max_rel=float(np.max(np.abs(f - f_ref) / np.maximum(np.abs(f_ref), 1.0))),
                energy_rel=float(abs(b2.potential_energy() - e_ref) / abs(e_ref)))
            if prec == backend.PRECISION_FP64 and fp64_nsday is None:
                b2.upload_state(np.ascontiguousarray(state.pos), np.ascontiguousarray(state.vel))
                b2.forces_resident()
                fp64_tuned = b2.autotune(reps=3)  # the FP64 pair kernel gets the same tuning
                fp64_pair_ms = b2.profile("pair", 10)
                b2.run_resident(DT_PS, 3)
                b2.synchronize()
                n64 = max(50, min(args.steps, 300))
                s64 = b2.time_steps(DT_PS, n64, first_step=3, flush_ptr=flush.data_ptr(),
                                    flush_bytes=L2_FLUSH_BYTES) / 1e3
                fp64_nsday = ns_per_day(n64, s64)
            b2.close()
    # e2e: the public API with host buffers, one gm_steps call per step
    # (H2D of positions+velocities from pinned memory, one device step, D2H
    # of positions+velocities and the energy)
    tp, hp = pinned_like(state.pos)
    tv, hv = pinned_like(state.vel)
    be.download_state(hp, hv)
    n_e2e = max(200, min(args.steps, 500))  # host-timed calls: enough of them to average the host jitter
    be.steps(hp, hv, DT_PS, 1)
    t0 = time.perf_counter()
    for _ in range(n_e2e):
        be.steps(hp, hv, DT_PS, 1)
    t_e2e = time.perf_counter() - t0
    h2d = 6 * 8 * N_ATOMS
    d2h = 6 * 8 * N_ATOMS + 8
    # CPU baseline: the oracle on this host's cores, bounded sample
    cpu = cpu_baseline_sample(atoms, topo, state, result["rebuilds"] / max(args.steps, 1))
    steps_per_s = args.steps / sec
    line = {
        "metric": METRIC, "value": round(aggregate_ns_per_day(world, args.steps, sec), 3), "unit": "ns/day",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1e3 * sec / args.steps, 5), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "fp32 pair math, int64 fixed-point forces, fp64 state/energy",
        "data": "synthetic (seeded generator, no dataset)",
        "config": config_dict(), "replicas": world, "list_rebuilds_in_timed_region": result["rebuilds"],
        "pairs_per_s": round(world * pairs * steps_per_s, 1), "half_list_pairs": pairs,
        "literal_lattice": lattice,
        "fp64_path_ns_per_day": round(fp64_nsday, 3) if fp64_nsday else None,
        "fp64_pair_kernel": {"ms": round(fp64_pair_ms, 5) if fp64_pair_ms else None, "autotuner": fp64_tuned},
        "mixed_over_fp64": round(ns_per_day(args.steps, sec) / fp64_nsday, 2) if fp64_nsday else None,
        "steady_state": {"ns_per_day": round(ns_per_day(n_bb, t_bb), 3), "steps": n_bb,
                         "ms_per_step": round(1e3 * t_bb / n_bb, 5), "list_rebuilds": int(reb_bb),
                         "note": "back to back, no L2 flush, list rebuilds included (amortised)"},
        "step_form": args.step_form,
        "other_step_form": {"form": other, "ns_per_day": round(ns_per_day(args.steps, t_other), 3),
                            "ms_per_step": round(1e3 * t_other / args.steps, 5),
                            "note": "same flushed timing, later in the same run"},
        "errors_vs_fp64_oracle": errs,
        "kernel_ms": {"pair": round(t_pair * 1e3, 5), "bonded": round(t_bonded * 1e3, 5),
                      "pair14": round(t_pair14 * 1e3, 5), "forces": round(t_forces * 1e3, 5),
                      "list_rebuild": round(t_rebuild * 1e3, 4), "build_kernel": round(t_build * 1e3, 4)},
        "roofline": ({"bound": "hbm", "achieved": round(step_bytes / t_launch / 1e9, 1), "peak": peak, "unit": "GB/s",
                      "frac": round(step_bytes / t_launch / 1e9 / peak, 4),
                      "traffic": round(STEP_TRAFFIC_CAPTURE * step_bytes / STEP_BYTES_CAPTURE),
                      "peak_source": peak_kind, "kernel": "step_persistent_kernel", "algorithmic_bytes": step_bytes,
                      "launch_ms": round(t_launch * 1e3, 5), "half_list_pairs": pairs_roof,
                      "timing": f"median of {n_roof} single graph launches (one launch of the kernel each, CUDA "
                                f"events, L2 flushed before each), at the state after the timed steps"}
                     if args.step_form == "persistent" else
                     {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                      "frac": round(achieved / peak, 4), "traffic": round(PAIR_TRAFFIC_PER_PAIR * pairs_prof),
                      "peak_source": peak_kind, "kernel": "pair_kernel_mixed", "algorithmic_bytes": alg_bytes}),
        "pair_kernel_roofline": {"kernel": "pair_kernel_mixed", "achieved": round(achieved, 1), "unit": "GB/s",
                                 "frac": round(achieved / peak, 4),
                                 "traffic": round(PAIR_TRAFFIC_PER_PAIR * pairs_prof), "half_list_pairs": pairs_prof,
                                 "algorithmic_bytes": alg_bytes, "ms": round(t_pair * 1e3, 5),
                                 "note": "the pair kernel alone (gm_profile, 30 launches, warm): the pair items' "
                                         "work without the bonded terms and the integrator"},
        "e2e": {"value": round(ns_per_day(n_e2e, t_e2e), 3), "unit": "ns/day", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "api": "gm_steps (C ABI), one step per call, pinned host buffers"},
        "gpu_launches": int(result["launches"]),
        "autotuner": tuned,
        "cpu_baseline": cpu,
    }
    return line


def cpu_baseline_sample(atoms, topo, state, rebuilds_per_step):
    """Oracle (C restatement, static strips over all host cores) on the same
    system: five force evaluations on the reference's pair list, plus the
    reference's O(N^2) serial list build timed on the first N/4 atoms and
    scaled by 16, combined per BAB step at the GPU run's rebuild rate."""
    import oracle
    nthreads = oracle.host_threads()
    op = oracle.make_params(box=PHYS["box_size"], periodic=False, r_cutoff=10.0, r_skin=12.0, r_switch=8.0,
                            n_threads=nthreads, coulomb=True, scale14_lj=0.5, scale14_coul=1 / 1.2)
    pos = np.ascontiguousarray(state.pos)
    pi, pj = oracle.neighbor_build(pos.copy(), atoms, topo, op, cells=True)
    ob = oracle.CpuBackend(atoms, topo, op)
    ob.set_pairs(pi, pj, pos)
    ts = []
    for _ in range(5):
        t0 = time.perf_counter()
        ob.compute_forces(pos)
        ts.append(time.perf_counter() - t0)
    t_force = float(np.median(ts))
    ns = N_ATOMS // 4
    sub = _Sub(atoms, ns)
    t0 = time.perf_counter()
    oracle.neighbor_build(np.ascontiguousarray(pos[:, :ns]), sub, _sub_topo(topo, ns), op)
    t_build = (time.perf_counter() - t0) * (N_ATOMS / ns) ** 2
    t_step = t_force + t_build * rebuilds_per_step
    return {"value": round(ns_per_day(1, t_step), 4), "unit": "ns/day", "cores": nthreads, "kind": "port",
            "sample": (f"oracle CpuBackend forces {t_force:.3f} s/eval (median of 5, {nthreads} threads) + "
                       f"reference O(N^2) serial list build timed on {ns} atoms and scaled x16 ({t_build:.1f} s) "
                       f"at {rebuilds_per_step:.4f} rebuilds/step; integrator O(N) terms neglected")}


class _Sub:
    def __init__(self, atoms, n):
        self.sigma, self.epsilon, self.mass = atoms.sigma[:n], atoms.epsilon[:n], atoms.mass[:n]
        self.charge, self.element = atoms.charge[:n], atoms.element[:n]


def _sub_topo(topo, n):
    from geodesic_cuda import amber
    t = amber.BondedTopology.empty()
    keep = (topo.excl_i < n) & (topo.excl_j < n)
    t.excl_i, t.excl_j = topo.excl_i[keep], topo.excl_j[keep]
    return t


def run_reference(args):
    """Times the oracle's BAB loop (the reference CPU path restated in C, all
    host cores) on the same workload; min(K, 20) timed steps after W warm-up
    steps, reported per step."""
    import oracle
    atoms, topo, state, info = workload(0)
    nthreads = oracle.host_threads()
    op = oracle.make_params(box=PHYS["box_size"], periodic=False, r_cutoff=10.0, r_skin=12.0, r_switch=8.0,
                            n_threads=nthreads, coulomb=True, scale14_lj=0.5, scale14_coul=1 / 1.2,
                            max_constr_iter=100, constr_tol=1e-10)
    pos = np.ascontiguousarray(state.pos.copy())
    vel = np.ascontiguousarray(state.vel.copy())
    b = oracle.CpuBackend(atoms, topo, op)
    pi, pj = oracle.neighbor_build(pos.copy(), atoms, topo, op, cells=True)
    b.set_pairs(pi, pj, pos)  # the reference's pair set, without timing its O(N^2) build here
    f = b.compute_forces(pos)
    n_w = args.warmup
    n_t = max(1, min(args.steps, 200))  # ~30 ms per step: a bounded sample
    t_total, n_reb = 0.0, 0
    for k in range(n_w + n_t):
        t0 = time.perf_counter()
        oracle.half_kick(vel, f, atoms.mass, DT_PS / 2)
        b.geodesic_drift(pos, vel, DT_PS, k)
        if b.needs_rebuild(pos):
            b.build_neighbor_list(pos)  # the reference's O(N^2) serial build
            n_reb += k >= n_w
        f = b.compute_forces(pos)
        oracle.half_kick(vel, f, atoms.mass, DT_PS / 2)
        dt = time.perf_counter() - t0
        if k >= n_w:
            t_total += dt
    val = ns_per_day(n_t, t_total)
    return {"impl": "reference", "metric": METRIC, "value": round(val, 4), "unit": "ns/day", "n_gpus": 1,
            "steps": n_t, "warmup": n_w, "ms_per_step": round(1e3 * t_total / n_t, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "fp64", "data": "synthetic (seeded generator)",
            "config": config_dict(), "replicas": 1, "steps_requested": args.steps,
            "cpu_baseline": {"value": round(val, 4), "unit": "ns/day", "cores": nthreads, "kind": "port",
                             "sample": f"{n_t} BAB steps of the oracle loop after {n_w} warm-up steps "
                                       f"({n_reb} O(N^2) list rebuilds in the timed steps)"},
            "e2e": {"value": round(val, 4), "unit": "ns/day", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


# ---------------------------------------------------------------- other configs
# Each prints its own JSON line (python bench.py --config NAME); the default
# line above is the headline workload.

def _gen_one(args_):
    """Worker of the generator pool (spawned before any GPU work): one
    system with a single generator thread."""
    n, seed, relax, h = args_
    sys.path[:0] = [os.path.join(ROOT, "geodesic-m_gb300")]
    from geodesic_cuda import synth
    return synth.generate(n, seed=seed, temperature=300.0, relax_iters=relax, h_fraction=h, n_threads=1)[:3]


def _clock_ok(clk):
    return {k: clk[k] for k in ("sm_mhz", "sm_max_mhz", "reasons") if k in clk}


def _time_batch(be, args, flush, form):
    """Resident batch steps in one step form from the state the context
    holds: warm-up, then args.steps flushed timed steps."""
    from geodesic_cuda import backend
    be.step_form(form)
    be.run_resident(DT_PS, args.warmup)
    be.synchronize()
    c0 = be.counters()
    with ClockSampler(0) as clk:
        dev_ms = be.time_steps(DT_PS, args.steps, first_step=args.warmup, flush_ptr=flush.data_ptr(),
                               flush_bytes=L2_FLUSH_BYTES)
    c1 = be.counters()
    return dev_ms / 1e3, c1["rebuilds"] - c0["rebuilds"], int(c1["launches"] - c0["launches"]), clk.summary()


def run_ensemble(args):
    """The batched ensemble: 256 independent systems, N log-uniform in
    [500, 20000], per-system seeds, MB 300 K, mixed precision: one context,
    one graph launch per step for the whole batch (one persistent launch
    inside it, and the kernel graph for comparison), split from the
    autotuner; against the same systems run one by one (each in its own
    context)."""
    import multiprocessing as mp
    rng = np.random.default_rng(SEED)
    n_sys = args.systems
    sizes = np.exp(rng.uniform(np.log(500), np.log(20000), n_sys)).astype(int)
    jobs = [(int(n), SEED + 1000 + k, 200, 0.0) for k, n in enumerate(sizes)]
    t0 = time.perf_counter()
    with mp.get_context("spawn").Pool(min(os.cpu_count() or 1, 32)) as pool:
        syss = pool.map(_gen_one, jobs, chunksize=1)
    t_gen = time.perf_counter() - t0
    import torch
    from geodesic_cuda import backend
    torch.cuda.set_device(0)
    p = backend.SimParams(precision=backend.PRECISION_MIXED, **PHYS)
    pos = np.ascontiguousarray(np.concatenate([s[2].pos for s in syss], axis=1))
    vel = np.ascontiguousarray(np.concatenate([s[2].vel for s in syss], axis=1))
    be = backend.CudaBackend.ensemble([s[0] for s in syss], [s[1] for s in syss], p)
    be.upload_state(pos, vel)
    be.forces_resident()
    if args.pair_shape:
        # a known split instead of the autotuner (profiler runs)
        sp, wb, gr = (int(x) for x in args.pair_shape.split(","))
        be.pair_shape(sp, wb, gr)
        choice = {"split": sp, "warps_per_block": wb, "grid": gr, "set": "--pair-shape"}
    else:
        choice = be.autotune(reps=3)
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda:0")
    if args.quick:
        # the batch's persistent steps only (profiler runs)
        sec, reb, launches, _ = _time_batch(be, args, flush, backend.STEP_PERSISTENT)
        be.close()
        return {"metric": "aggregate ns/day of a 256-system batch (quick)", "value": round(n_sys * ns_per_day(
                args.steps, sec), 2), "unit": "ns/day", "steps": args.steps, "quick": True,
                "ms_per_step": round(1e3 * sec / args.steps, 4), "list_rebuilds_in_timed_region": reb,
                "gpu_launches": launches, "autotuner": choice}
    # the whole batch as one persistent launch per step, then the same start
    # state as the kernel graph
    sec, reb, launches, clk = _time_batch(be, args, flush, backend.STEP_PERSISTENT)
    be.upload_state(pos, vel)
    be.forces_resident()
    sec_g, reb_g, _, clk_g = _time_batch(be, args, flush, backend.STEP_GRAPH)
    batched = n_sys * ns_per_day(args.steps, sec)
    batched_graph = n_sys * ns_per_day(args.steps, sec_g)
    be.close()
    # one by one: each system alone, its own context and graph
    k1 = max(20, min(args.steps, args.single_steps))
    t_single = 0.0
    for atoms, topo, state in syss:
        b1 = backend.CudaBackend(atoms, topo, p)
        b1.upload_state(np.ascontiguousarray(state.pos), np.ascontiguousarray(state.vel))
        b1.forces_resident()
        b1.run_resident(DT_PS, args.warmup)
        b1.synchronize()
        t_single += b1.time_steps(DT_PS, k1, first_step=args.warmup, flush_ptr=flush.data_ptr(),
                                  flush_bytes=L2_FLUSH_BYTES) / 1e3 / k1
        b1.close()
    one_by_one = n_sys * ns_per_day(1, t_single)
    return {"metric": "aggregate ns/day of a 256-system batch, batched vs one by one", "value": round(batched, 2),
            "unit": "ns/day", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(1e3 * sec / args.steps, 4), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "fp32 pair math, int64 fixed-point forces, fp64 state/energy",
            "data": "synthetic (seeded generator, no dataset)",
            "config": {"workload": f"{n_sys} independent lattice-chain systems, N log-uniform in [500, 20000] "
                                   f"(total {int(sizes.sum())} atoms), per-system seeds, MB 300 K, 2 fs, "
                                   "FIRE 200 iterations", "n_systems": n_sys, "total_atoms": int(sizes.sum()),
                       "l2": "flushed between timed steps"},
            "step_form": "persistent (one cooperative launch per batch step, rebuild in the graph's IF node)",
            "one_by_one_ns_per_day": round(one_by_one, 2), "batched_over_one_by_one": round(batched / one_by_one, 2),
            "one_by_one_sample": f"{k1} timed steps per system after {args.warmup} warm-up steps, summed",
            "kernel_graph_form": {"ns_per_day": round(batched_graph, 2), "ms_per_step": round(1e3 * sec_g / args.steps, 4),
                                  "list_rebuilds_in_timed_region": reb_g, "clocks": _clock_ok(clk_g)},
            "autotuner": choice, "list_rebuilds_in_timed_region": reb,
            "gpu_launches": launches, "generation_s": round(t_gen, 1),
            "clocks": _clock_ok(clk)}


def run_warm_start(args):
    """The constrained warm-start workload: 50,000 atoms with 40 % hydrogens
    (H bonds constrained at 1.09 A), FP64 SHAKE/RATTLE to 1e-10: the network
    is trained on solver multipliers of a different seed (2,000 recorded
    steps), then the same run is timed cold and warm-started.  At 2 fs: with
    H at 1.008 amu and only the H bonds constrained this lattice fails within
    20 steps at 4 fs and within ~1,000 at 3 fs (the oracle fails the same
    way)."""
    import torch
    from geodesic_cuda import amber, backend, synth
    torch.cuda.set_device(0)
    dt = 0.002
    p = backend.SimParams(precision=backend.PRECISION_MIXED, max_constr_iter=200, constr_tol=1e-10, **{
        k: v for k, v in PHYS.items() if k not in ("max_constr_iter", "constr_tol")})

    def system(seed):
        atoms, topo, state, _ = synth.generate(N_ATOMS, seed=seed, h_fraction=0.4, temperature=300.0,
                                               relax_iters=1000)
        return atoms, amber.promote_hydrogen_bonds(topo, atoms), state
    if args.quick:
        # the evaluation system, cold, timed steps only (profiler runs)
        ev = system(SEED)
        be = backend.CudaBackend(ev[0], ev[1], p)
        be.upload_state(np.ascontiguousarray(ev[2].pos), np.ascontiguousarray(ev[2].vel))
        be.forces_resident()
        be.run_resident(dt, args.warmup)
        be.synchronize()
        c0 = be.counters()
        sec = be.time_steps(dt, args.steps, first_step=args.warmup) / 1e3
        c1 = be.counters()
        cold = {"ms_per_step": round(1e3 * sec / args.steps, 4),
                "mean_shake_iters": (c1["shake_iter_sum"] - c0["shake_iter_sum"]) / max(args.steps, 1),
                "rebuilds": c1["rebuilds"] - c0["rebuilds"]}
        # then warm-started, with a network trained briefly on this run's own
        # multipliers (profiling the warm-start kernels, not its benefit)
        be.ws_record(50, 1)
        be.run_resident(dt, 50, first_step=args.warmup + args.steps)
        be.synchronize()
        be.ws_record(0)
        be.ws_train(300, blocks=32, lr=3e-3, seed=5)
        be.ws_enable(True)
        c0 = be.counters()
        sec = be.time_steps(dt, args.steps, first_step=args.warmup + args.steps + 50) / 1e3
        c1 = be.counters()
        warm = {"ms_per_step": round(1e3 * sec / args.steps, 4),
                "mean_shake_iters": (c1["shake_iter_sum"] - c0["shake_iter_sum"]) / max(args.steps, 1)}
        return {"metric": "constrained 50k step time (quick)", "value": cold["ms_per_step"], "unit": "ms/step",
                "steps": args.steps, "quick": True, "cold": cold, "warm": warm}
    t0 = time.perf_counter()
    tr = system(SEED + 7)
    ev = system(SEED)
    t_gen = time.perf_counter() - t0
    # training data: the solver's own multipliers along a trajectory
    b = backend.CudaBackend(tr[0], tr[1], p)
    b.upload_state(np.ascontiguousarray(tr[2].pos), np.ascontiguousarray(tr[2].vel))
    b.forces_resident()
    b.ws_record(args.train_steps, 1)
    b.run_resident(dt, args.train_steps)
    b.synchronize()
    b.ws_record(0)
    n_samples = b.counters()["ws_records"] * len(tr[1].constr_i)
    t1 = time.perf_counter()
    loss = b.ws_train(args.train_iters, blocks=64, lr=3e-3, seed=11)
    t_train = time.perf_counter() - t1
    P, norm = b.ws_params()
    b.close()
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda:0")
    out = {}
    # cold and warm with the default force evaluation (the persistent
    # kernel's force phase), and cold once more with the kernel graph's pair
    # kernel beside the bonded kernel
    for name, warm in (("cold", False), ("warm", True), ("cold_kernel_graph_forces", False)):
        be = backend.CudaBackend(ev[0], ev[1], p)
        if name == "cold_kernel_graph_forces":
            be.step_form(backend.STEP_GRAPH)
        be.upload_state(np.ascontiguousarray(ev[2].pos), np.ascontiguousarray(ev[2].vel))
        be.forces_resident()
        if warm:
            be.ws_params(P, norm)
            be.ws_enable(True)
        be.run_resident(dt, args.warmup)
        be.synchronize()
        c0 = be.counters()
        with ClockSampler(0) as clk:
            sec = be.time_steps(dt, args.steps, first_step=args.warmup, flush_ptr=flush.data_ptr(),
                                flush_bytes=L2_FLUSH_BYTES) / 1e3
        c1 = be.counters()
        steps = c1["constrained_steps"] - c0["constrained_steps"]
        out[name] = dict(ns_per_day=round(dt * 1e-3 * args.steps / sec * 86400.0, 3),
                         mean_shake_iters=round((c1["shake_iter_sum"] - c0["shake_iter_sum"]) / max(steps, 1), 3),
                         mean_rattle_iters=round((c1["rattle_iter_sum"] - c0["rattle_iter_sum"]) / max(steps, 1), 3),
                         ms_per_step=round(1e3 * sec / args.steps, 4), clocks=_clock_ok(clk.summary()))
        be.close()
    return {"metric": "mean SHAKE iterations and ns/day, BF16 warm start vs cold start, equal tolerance",
            "value": out["warm"]["ns_per_day"], "unit": "ns/day", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "fp32 pair math, fp64 SHAKE/RATTLE, bf16 network", "data": "synthetic (seeded generator)",
            "config": {"workload": "50,000-atom lattice chain, 40 % H (1.008 amu, constrained 1.09 A bonds), "
                                   "2 fs, tol 1e-10", "train_seed": SEED + 7, "eval_seed": SEED,
                       "train_steps_recorded": args.train_steps, "train_samples": int(n_samples),
                       "train_iters": args.train_iters, "l2": "flushed between timed steps"},
            "cold": out["cold"], "warm": out["warm"], "cold_kernel_graph_forces": out["cold_kernel_graph_forces"],
            "warm_over_cold_ns_per_day": round(out["warm"]["ns_per_day"] / out["cold"]["ns_per_day"], 3),
            "train_loss_standardised": round(loss, 5), "train_s": round(t_train, 2), "generation_s": round(t_gen, 1)}


def run_scaled(args, n_atoms, precision, relax, steps_default):
    """The 1,000,000-atom scale test (mixed, 200 steps) and the 5,000-atom
    system (FP64, 1,000 steps): timed device steps, list rebuild and pair
    kernel bandwidth."""
    import torch
    from geodesic_cuda import backend, synth
    torch.cuda.set_device(0)
    t0 = time.perf_counter()
    atoms, topo, state, _ = synth.generate(n_atoms, seed=SEED, temperature=300.0, relax_iters=relax)
    t_gen = time.perf_counter() - t0
    p = backend.SimParams(precision=precision, **PHYS)
    be = backend.CudaBackend(atoms, topo, p)
    be.upload_state(np.ascontiguousarray(state.pos), np.ascontiguousarray(state.vel))
    be.forces_resident()
    choice = be.autotune(reps=3) if precision == backend.PRECISION_MIXED else None
    be.run_resident(DT_PS, args.warmup)
    be.synchronize()
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda:0")
    steps = args.steps if args.steps_given else steps_default
    c0 = be.counters()
    with ClockSampler(0) as clk:
        sec = be.time_steps(DT_PS, steps, first_step=args.warmup, flush_ptr=flush.data_ptr(),
                            flush_bytes=L2_FLUSH_BYTES) / 1e3
    c1 = be.counters()
    pairs = c1["pairs"]
    t_pair = be.profile("pair", 10) / 1e3
    t_reb = be.profile("rebuild", 3) / 1e3
    peak, peak_kind = measured_peaks()
    alg_pair = 4 * pairs + 52 * n_atoms
    # list build algorithmic bytes: per atom 16 B read, 8 B cell key and index,
    # 16 B sorted coordinates and 4 B offset written, plus one int32 index per
    # half-list pair (neighbor.rs:8-55's output)
    alg_list = n_atoms * 44 + 4 * pairs
    return {"metric": f"ns/day at {n_atoms} atoms", "value": round(ns_per_day(steps, sec), 3), "unit": "ns/day",
            "n_gpus": 1, "steps": steps, "warmup": args.warmup, "ms_per_step": round(1e3 * sec / steps, 4),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "fp64" if precision == backend.PRECISION_FP64 else "fp32 pair math, int64 fixed-point forces",
            "data": "synthetic (seeded generator)",
            "config": {"workload": f"synthetic lattice chain, {n_atoms} atoms, 2 fs, FIRE {relax} iterations",
                       "n_atoms": n_atoms, "l2": "flushed between timed steps"},
            "pairs_per_s": round(pairs * steps / sec, 1), "half_list_pairs": pairs,
            "list_rebuilds_in_timed_region": c1["rebuilds"] - c0["rebuilds"],
            "pair_kernel": {"ms": round(t_pair * 1e3, 4), "algorithmic_bytes": alg_pair,
                            "achieved_gbs": round(alg_pair / t_pair / 1e9, 1),
                            "frac": round(alg_pair / t_pair / 1e9 / peak, 4)},
            "list_rebuild": {"ms": round(t_reb * 1e3, 4), "algorithmic_bytes": alg_list,
                             "achieved_gbs": round(alg_list / t_reb / 1e9, 1),
                             "frac": round(alg_list / t_reb / 1e9 / peak, 4)},
            "peak_gbs": peak, "peak_source": peak_kind, "autotuner": choice,
            "gpu_launches": int(c1["launches"] - c0["launches"]), "generation_s": round(t_gen, 1),
            "clocks": _clock_ok(clk.summary())}



def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10000)
    ap.add_argument("--warmup", type=int, default=50)
    ap.add_argument("--impl", choices=["cuda", "reference"], default="cuda")
    ap.add_argument("--quick", action="store_true",
                    help="timed steps only (no error, CPU-baseline, FP64 or e2e legs); for profiler runs")
    ap.add_argument("--precision", choices=["mixed", "fp64"], default="mixed",
                    help="with --quick: the precision of the timed steps")
    ap.add_argument("--step-form", choices=["graph", "persistent"], default="persistent",
                    help="unconstrained mixed-precision steps: the kernel graph, or one persistent launch per step")
    ap.add_argument("--pair-shape", default="",
                    help="SPLIT,WARPS,GRID: the pair kernel's launch shape instead of the autotuner's choice")
    ap.add_argument("--config", default="headline",
                    choices=["headline", "ensemble", "warm_start", "scale_1m", "small_5k"],
                    help="headline: 50k atoms (the default line); the others print their own line")
    ap.add_argument("--systems", type=int, default=256, help="ensemble: number of systems")
    ap.add_argument("--single-steps", type=int, default=200, help="ensemble: timed steps per system one by one")
    ap.add_argument("--train-steps", type=int, default=2000, help="warm_start: recorded steps")
    ap.add_argument("--train-iters", type=int, default=4000, help="warm_start: Adam steps")
    argv = sys.argv[1:]
    args = ap.parse_args(argv)
    args.steps_given = any(a == "--steps" or a.startswith("--steps=") for a in argv)
    args.warmup = max(args.warmup, 3)
    if args.config != "headline":
        from geodesic_cuda import backend
        if args.config == "ensemble":
            if not args.steps_given:
                args.steps = 5000  # the batched-ensemble workload's own step count
            line = run_ensemble(args)
        elif args.config == "warm_start":
            if not args.steps_given:
                args.steps = 1000
            line = run_warm_start(args)
        elif args.config == "scale_1m":
            line = run_scaled(args, 1_000_000, backend.PRECISION_MIXED, 300, 200)
        else:
            line = run_scaled(args, 5_000, backend.PRECISION_FP64, 1000, 1000)
        print(json.dumps(line), flush=True)
        return
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        if rank != 0:
            return
        print(json.dumps(run_reference(args)), flush=True)
        return
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("nccl")
    line = run_cuda(args, rank, world)
    if rank == 0 and line is not None:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
