"""Benchmark of the batched UFF energy+gradient scorer (one JSON line on rank 0).

Workload (per GPU): one 48-atom ligand with 8 rotatable bonds against a
6,000-atom pocket in an 18 A sphere, 4,096 poses per step, energy plus the
analytic gradient with respect to the 6 rigid-body and 8 torsion DOFs
(seeded synthetic inputs; the reference publishes no benchmark data).

* ``value``: poses/s with the poses resident in HBM, device-timed with CUDA
  events on the scoring stream; L2 is flushed (256 MiB write) before every
  timed step, outside the timed interval.
* ``e2e``: the same through ``mmo_score_poses`` (C ABI, host buffers): the
  H2D copy of the poses and the D2H copy of energies, gradients and statuses
  are inside the timed interval.
* ``plain``: the one-pose-per-launch path on a sample of the same poses.
* ``roofline``: the pair-sweep kernel's algorithmic FP32 rate against the
  device's measured FP32 FMA rate.
* ``cpu_baseline``: the FP64 CPU restatement of the reference path timed on
  the host cores, energy plus central-difference gradient as the reference
  computes it (src/lds.ml:1118-1136); ``legs`` adds the same on one thread,
  the brute L x P sum and the analytic gradient.
* ``errors``: every pose of the step against the FP64 oracle (energy relative
  error, gradient per-component error).
* ``energy_only_65536``: the 65,536-pose energy-only batch on the same
  system, with its own roofline and errors on 4,096 sampled poses.

``--impl reference`` times only that CPU path (the reference itself is OCaml
and cannot be built here) and prints its own line.
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

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "poses/s (energy+grad) batched vs plain GPU at ≤1e-5 rel err vs FP64 oracle"
WORKLOAD = ("energy+gradient, 4096 poses/step, 48-atom ligand (8 torsions) vs 6000-atom pocket "
            "(18 A sphere), UFF LJ 12-6 + Coulomb eps=4, 12 A switch, intra-ligand 1-4+")
FLOPS_PAIR_GRAD = 42  # per ligand-protein pair, energy + gradient (FMA = 2)
FLOPS_PAIR_E = 26
POSES = 4096


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--poses", type=int, default=POSES)
    ap.add_argument("--cpu-sample", type=int, default=0,
                    help="poses in the CPU-baseline sample (0: about 10 s of work)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-energy-only", action="store_true",
                    help="skip the 65,536-pose energy-only measurement of the main workload")
    ap.add_argument("--no-large-pocket", action="store_true",
                    help="skip the 4,096-pose line against the 12,000-atom pocket")
    ap.add_argument("--no-tune", action="store_true",
                    help="keep the default launch plan instead of the autotuner's")
    ap.add_argument("--workload", default="poses",
                    choices=["poses", "ragged", "mc", "grid", "dock"],
                    help="poses: the energy+gradient pose batch (default); ragged: 1,024 "
                         "systems x 64 poses in one pass; mc: 512 Monte Carlo chains; "
                         "grid: per-type grids built, then the poses scored from them; dock: "
                         "exhaustive rigid docking on grids and masks")
    ap.add_argument("--systems", type=int, default=1024, help="ragged: systems in the batch")
    ap.add_argument("--mc-steps", type=int, default=10000, help="mc: steps per chain")
    return ap.parse_args()


class Clocks:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self.proc = None
        self.t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.t = threading.Thread(target=self._read, daemon=True)
        self.t.start()

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([v.strip() for v in line.split(",")])

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.t:
            self.t.join(timeout=2)
        sm = [float(r[1]) for r in self.rows if len(r) >= 9 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) >= 9 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            if len(r) >= 9:
                for n, v in zip(names, r[5:9]):
                    if v.lower() == "active":
                        reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(sm)}


def system_for_rank(rank: int, poses: int):
    from mmo_gb300 import synth

    s = synth.pose_batch(n_poses=poses, seed=1)
    if rank:
        s.poses = synth.random_poses(np.random.default_rng(1000 + 7919 * rank), poses,
                                     s.ligand.nrb, 4.0)
    return s


FD_EPS_NOTE = "central differences with the reference's steps, 0.1 A / 1 deg (lds.ml:1118-1136)"


def _fd_eps(nd):
    return np.array([0.1] * 3 + [np.pi / 180.0] * (nd - 3))


def cpu_baseline(system, sample: int, nthreads: int, gpu_E=None, use_cells=True, mode=2):
    """The oracle (FP64 restatement of the reference path) on `sample` poses:
    energy + central differences with the reference's steps (mode 2, 29
    scorings per pose) or + the analytic gradient (mode 1); the 12 A cell
    neighbour sum (the BST query of mol.ml:939) or the brute L x P sum.
    Returns (poses/s, seconds, sample, max rel E error vs GPU)."""
    from oracle import oracle as O

    nd = 6 + system.ligand.nrb
    d = system.poses[:sample]
    t0 = time.perf_counter()
    E, _, _ = O.score_batch(system.pocket, system.ligand, d, mode=mode, eps=_fd_eps(nd),
                            use_cells=use_cells, nthreads=nthreads)
    dt = time.perf_counter() - t0
    err = None
    if gpu_E is not None:
        g = gpu_E[:sample]
        err = float(np.max(np.abs(g - E) / np.maximum(np.abs(E), 1e-300)))
    return sample / dt, dt, err


def calibrate_sample(system, nthreads: int, target_s=10.0, use_cells=True, mode=2) -> int:
    from oracle import oracle as O

    nd = 6 + system.ligand.nrb
    n0 = max(nthreads, 4)
    t0 = time.perf_counter()
    O.score_batch(system.pocket, system.ligand, system.poses[:n0], mode=mode, eps=_fd_eps(nd),
                  use_cells=use_cells, nthreads=nthreads)
    per = (time.perf_counter() - t0) / n0
    return int(max(n0, min(len(system.poses), target_s / max(per, 1e-9))))


def cpu_legs(system, nthreads: int, gpu_E, target_s=10.0):
    """The CPU baselines: the reference's method (energy + central
    differences, cell-list sum) on all host threads (the headline CPU
    figure), the same on one thread (the shape of the reference's own
    per-process loop), the brute L x P sum on all threads, and the analytic
    FP64 gradient on all threads.  Each is a bounded sample of the poses."""
    legs = {}
    for name, threads, cells, mode in (("all_threads", nthreads, True, 2),
                                       ("single_thread", 1, True, 2),
                                       ("brute_all_threads", nthreads, False, 2),
                                       ("analytic_all_threads", nthreads, False, 1)):
        n = calibrate_sample(system, threads, target_s, cells, mode)
        v, dt, err = cpu_baseline(system, n, threads, gpu_E, cells, mode)
        legs[name] = {"value": v, "unit": "poses/s", "cores": threads, "sample_poses": n,
                      "seconds": dt,
                      "inter_sum": "12 A cell list" if cells else "brute L x P",
                      "gradient": FD_EPS_NOTE if mode == 2 else "analytic FP64 (reverse mode)",
                      "max_rel_err_E_gpu_vs_fp64": err}
    return legs


def errors_vs_oracle(system, E, G, nthreads: int, poses=None, flags_mc=False, dofs=None):
    """The GPU results against the FP64 oracle on the given poses, under the
    scoring contract: energies |E - E64| / |E64| (cancellation cases, where
    S = sum over pairs of w (|elec| + D p12 + 2 D p6) exceeds 100 |E64|, are
    reported apart), gradient components |G - G64| / max(|G64|, 0.01 GA)
    with GA the per-component sum of |terms| (orc_grad_scale), and the plain
    per-component relative error."""
    from oracle import oracle as O

    src = system.poses if dofs is None else dofs
    d = src if poses is None else src[poses]
    E = np.asarray(E, np.float64)
    mode = 1 if G is not None else 0
    fl = O.F_INTER | O.F_INTRA | (O.F_RECENTER if flags_mc else 0)
    E64, G64, _ = O.score_batch(system.pocket, system.ligand, d, flags=fl, mode=mode,
                                nthreads=nthreads)
    S, GA, _ = O.score_batch(system.pocket, system.ligand, d, flags=fl, mode=3,
                             nthreads=nthreads)
    rel = np.abs(E - E64) / np.abs(E64)
    cancel = S > 100.0 * np.abs(E64)
    out = {"poses": int(len(d)),
           "max_rel_err_E": float(rel[~cancel].max()) if (~cancel).any() else None,
           "max_err_E_cond": float((np.abs(E - E64) / np.maximum(np.abs(E64), S)).max()),
           "cancellation_poses": int(np.count_nonzero(cancel)),
           "tolerance_E": 1e-5}
    if G is not None:
        dG = np.abs(np.asarray(G, np.float64) - G64)
        with np.errstate(divide="ignore", invalid="ignore"):
            plain = np.where(dG == 0, 0.0, dG / np.abs(G64))
        out.update({"max_rel_err_G": float((dG / np.maximum(np.abs(G64), 0.01 * GA)).max()),
                    "max_rel_err_G_plain": float(plain.max()),
                    "frac_G_components_plain_within_1e-4": float(np.mean(plain <= 1e-4)),
                    "tolerance_G": 1e-4,
                    "G_rule": "per component, relative to max(|G64_k|, 0.01 GA_k)"})
    return out


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    nthreads = os.cpu_count() or 1
    s = system_for_rank(0, args.poses)
    # about two minutes of CPU work over all the timed steps
    budget = 120.0 / max(args.steps, 1)
    # the brute L x P sum (the reference's -ff BrL, mol.ml:822-849): on this
    # pocket it is faster than the 12 A cell list standing in for -ff Bst
    sample = args.cpu_sample or min(args.poses, calibrate_sample(s, nthreads, target_s=budget,
                                                                 use_cells=False))
    times = []
    for _ in range(max(args.warmup, 0) and 1):
        cpu_baseline(s, min(sample, nthreads), nthreads, use_cells=False)
    for _ in range(args.steps):
        _, dt, _ = cpu_baseline(s, sample, nthreads, use_cells=False)
        times.append(dt)
    v = sample * len(times) / sum(times)
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "poses/s", "n_gpus": 0,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * sum(times) / len(times), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "poses_per_step_per_gpu": args.poses,
                       "ligand_atoms": s.ligand.n, "torsions": s.ligand.nrb,
                       "pocket_atoms": s.pocket.n,
                       "precision": "fp64 (the reference computes in OCaml floats)",
                       "parallelism": "host threads over poses (the reference forks workers)"},
            "sampling": {"poses_scored_per_step": sample,
                         "note": "each step scores a bounded sample of the step's %d poses; "
                                 "value = poses scored / seconds" % args.poses,
                         "gradient": FD_EPS_NOTE,
                         "inter_sum": "brute L x P with the 12 A switch (-ff BrL, "
                                      "mol.ml:822-849; faster here than the 12 A cell list "
                                      "that stands in for the BST query of -ff Bst)"},
            "cpu_baseline": {"value": v, "unit": "poses/s", "cores": nthreads, "kind": "port",
                             "sample": "%d poses per step of the 4096-pose workload" % sample},
            "e2e": {"value": v, "unit": "poses/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "note": "FP64 C restatement of MMO's OCaml path (the OCaml toolchain is absent)"}
    print(json.dumps(line), flush=True)
    return 0


def _timed_region(torch, stream, step, steps, clocks=None):
    """CUDA-event times (ms) of `steps` calls of step() on `stream`."""
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(steps)]
    torch.cuda.synchronize()
    if clocks:
        clocks.start()
    for a, b in ev:
        a.record(stream)
        step()
        b.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop() if clocks else None
    return [a.elapsed_time(b) for a, b in ev], clk


def run_ragged(args):
    """1,024 independent ligand/pocket systems (12-80 ligand atoms, 0-15
    torsions, 2,000-8,000 pocket atoms), 64 poses each, energy and gradient of
    every pose in one pass of the system-batch kernels."""
    from mmo_gb300 import synth

    # made before CUDA starts, in spawned processes
    systems = synth.ragged_systems(args.systems, 64, seed=3, workers=os.cpu_count() or 1)
    import torch

    from mmo_gb300 import lib as L
    from mmo_gb300.ff import UFFScorer

    dev = torch.device("cuda", 0)
    sc = UFFScorer(0)
    sc.set_systems([(s.pocket, s.ligand, len(s.poses)) for s in systems])
    po, do = sc.systems_layout()
    B = int(po[-1])
    h = np.concatenate([s.poses.reshape(-1) for s in systems]).astype(np.float32)
    d = torch.from_numpy(h).to(dev)
    E = torch.empty(B, dtype=torch.float64, device=dev)
    G = torch.empty_like(d)
    st = torch.empty(B, dtype=torch.int32, device=dev)
    flags = L.F_INTER | L.F_INTRA | L.F_GRAD
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    sp = stream.cuda_stream
    tune_ms = None
    if not args.no_tune:
        tune_ms = sc.tune_systems_device(d.data_ptr(), E.data_ptr(), G.data_ptr(), st.data_ptr(),
                                         flags, sp)

    def step():
        sc.score_systems_device(d.data_ptr(), E.data_ptr(), G.data_ptr(), st.data_ptr(), flags, sp)

    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)
    for _ in range(max(args.warmup, 3)):
        step()
    sc.set_profiling(True)
    sms = []
    torch.cuda.synchronize()
    ev = []
    clocks = Clocks(0)
    clocks.start()
    for _ in range(args.steps):
        flush.zero_()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        step()
        b.record(stream)
        ev.append((a, b))
        sms.append(sc.stage_times())
    torch.cuda.synchronize()
    clk = clocks.stop()
    sc.set_profiling(False)
    ms = [a.elapsed_time(b) for a, b in ev]
    value = B * len(ms) / (sum(ms) * 1e-3)
    pairs_ev, pairs_all = sc.pair_count()
    stages = np.mean(np.array(sms), axis=0)
    # CUDA graph of the whole step
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=stream):
        step()
    for _ in range(3):
        g.replay()
    gms, _ = _timed_region(torch, stream, g.replay, args.steps)
    gval = B * len(gms) / (sum(gms) * 1e-3)
    # end to end with host buffers (page-locked, as a caller keeps them)
    h_in = torch.from_numpy(h).pin_memory().numpy()
    h_out = (torch.empty(B, dtype=torch.float64).pin_memory().numpy(),
             torch.empty(int(h.size), dtype=torch.float32).pin_memory().numpy(),
             torch.empty(B, dtype=torch.int32).pin_memory().numpy())
    e2e = []
    for k in range(args.warmup + args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t = time.perf_counter()
        Eh, Gh, sth = sc.score_systems(h_in, grad=True, out=h_out)
        if k >= args.warmup:
            e2e.append(time.perf_counter() - t)
    e2e_val = B * len(e2e) / sum(e2e)
    peak = sc.fp32_peak_tflops()
    achieved = FLOPS_PAIR_GRAD * pairs_ev / (stages[1] * 1e-3) * 1e-12
    Ls = [s.ligand.n for s in systems]
    Ps = [s.pocket.n for s in systems]
    line = {
        "metric": "poses/s (energy+grad), ragged batch of %d systems x 64 poses, one pass" %
                  len(systems),
        "value": value, "unit": "poses/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": float(np.mean(ms)), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "ragged: %d systems, ligands %d-%d atoms (mean %.1f), 0-15 "
                               "torsions, pockets %d-%d atoms (mean %.0f), 64 poses each" %
                               (len(systems), min(Ls), max(Ls), np.mean(Ls), min(Ps), max(Ps),
                                np.mean(Ps)),
                   "poses": B, "plan": dict(sc.systems_plan(), tuned_ms=tune_ms),
                   "l2": "flushed before every timed step of value and e2e (256 MiB write), not "
                         "timed; the graph line replays back to back on inputs larger than L2 "
                         "(%.0f MB of packed proteins)" % (32e-6 * sum(Ps))},
        "graph": {"value": gval, "unit": "poses/s", "ms_per_step": float(np.mean(gms))},
        "e2e": {"value": e2e_val, "unit": "poses/s", "h2d_bytes_per_step": int(h.nbytes),
                "d2h_bytes_per_step": int(Eh.nbytes + Gh.nbytes + sth.nbytes)},
        "stages_ms": {"rebuild": float(stages[0]), "sort": float(stages[3]),
                      "sweep": float(stages[1]), "finish": float(stages[2])},
        "roofline": {"bound": "fp32", "kernel": "k_sys_pairs (sweep of every system)",
                     "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak, "pairs_evaluated": pairs_ev,
                     "pairs_all": pairs_all, "flops_per_pair": FLOPS_PAIR_GRAD,
                     "ms_per_launch": float(stages[1])},
        "gpu_launches": sc.last_launches() * args.steps,
        "clocks": clk,
        "status_bits_set": int(np.count_nonzero(st.cpu().numpy())),
    }
    print(json.dumps(line), flush=True)
    sc.close()
    return 0


def run_mc(args):
    """512 Monte Carlo chains per system of the uneven batch's kind (Gaussian
    moves 5 deg / 0.3 A / 30 deg, kT 0.593, 20 gradient-descent iterations every
    50 steps), the block of steps replayed as a CUDA graph, with the reference's
    resets: a hard region of interest of 7 A about the pocket centre and a
    reset when a trial's inter energy is 0 (src/lds.ml:906-928)."""
    from mmo_gb300 import synth

    systems = [synth.ragged_system(i, seed=3, poses_per=512) for i in (1, 2, 3, 4)]
    import torch

    from mmo_gb300 import lib as L
    from mmo_gb300.ff import UFFScorer

    dev = torch.device("cuda", 0)
    prm = dict(kT=0.593, rot_step=np.radians(5.0), trans_step=0.3, tors_step=np.radians(30.0),
               move_law=L.MC_GAUSSIAN, adapt=0, flip_every=0, minimize_every=50,
               minimize_iters=20, gd_step=0.1, seed=2024, roi_center=(0.0, 0.0, 0.0),
               roi_radius=7.0, reset_on_zero_inter=1)
    runs, tot_steps, tot_s, finals = [], 0, 0.0, []
    for s in systems:
        sc = UFFScorer(0)
        sc.set_protein(s.pocket)
        sc.set_ligand(s.ligand)
        chains = len(s.poses)
        d = torch.from_numpy(s.poses).to(dev)
        E = torch.empty(chains, dtype=torch.float64, device=dev)
        acc = torch.empty(chains, dtype=torch.int32, device=dev)
        stt = torch.empty(chains, dtype=torch.int32, device=dev)
        res = torch.zeros(chains, dtype=torch.int32, device=dev)
        # warm-up run: plans, buffers and the graph of a block
        w = d.clone()
        sc.mc_run_device(chains, 100, prm, w.data_ptr(), E.data_ptr(), None, None, None, None,
                         None, True)
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        sc.mc_run_device(chains, args.mc_steps, prm, d.data_ptr(), E.data_ptr(), None, None,
                         acc.data_ptr(), stt.data_ptr(), None, True, d_resets=res.data_ptr())
        b.record()
        torch.cuda.synchronize()
        sec = a.elapsed_time(b) * 1e-3
        tot_steps += chains * args.mc_steps
        tot_s += sec
        runs.append({"system": s.name, "ligand_atoms": s.ligand.n, "torsions": s.ligand.nrb,
                     "pocket_atoms": s.pocket.n, "chains": chains,
                     "chain_steps_per_s": chains * args.mc_steps / sec,
                     "acceptance": float(acc.float().mean().item() / args.mc_steps),
                     "resets": int(res.sum().item()),
                     "chains_reset": int((res > 0).sum().item())})
        finals.append((s, d.cpu().numpy(), E.cpu().numpy()))
        sc.close()
    line = {
        "metric": "MC chain-steps/s (energy per step, 20 GD iterations every 50 steps)",
        "value": tot_steps / tot_s, "unit": "chain-steps/s", "n_gpus": 1,
        "steps": args.mc_steps, "warmup": 100, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "512 chains x %d steps on each of 4 systems of the uneven batch "
                               "(Gaussian moves 5 deg / 0.3 A / 30 deg, kT 0.593 kcal/mol)" %
                               args.mc_steps, "graph": True,
                   "resets": "hard ROI 7 A about the pocket centre, and E_inter = 0"},
        "runs": runs,
    }
    if not args.no_cpu:
        errs, skipped = [], 0
        for s, dofs, Eg in finals:
            # chains whose last frame was a reset hold E = +inf (the reference's prev_E)
            keep = np.flatnonzero(np.isfinite(Eg))[:64]
            skipped += int(np.count_nonzero(~np.isfinite(Eg)))
            er = errors_vs_oracle(s, Eg[keep], None, os.cpu_count() or 1, poses=keep,
                                  flags_mc=True, dofs=dofs)
            errs.append(er["max_rel_err_E"] or 0.0)
        line["cpu_baseline"] = {"kind": "port", "cores": os.cpu_count() or 1,
                                "final_E_max_rel_err_vs_fp64": float(max(errs)),
                                "error": "|E - E64| / |E64| (no cancellation case among them)",
                                "sample": "64 final chains per system re-scored in FP64",
                                "chains_ending_on_a_reset": skipped}
    print(json.dumps(line), flush=True)
    return 0


def run_grid(args):
    """The reference's default inter-energy path: per-type grids of the
    4,096-pose workload's system built on the GPU (0.5 A lattice over the
    protein's box plus the 36 A margin of src/lds.ml:1832, mask sphere of the
    ROI's outer radius + 24 A about the pocket centre, 48 ligand atom types),
    then the 4,096 poses scored (energy + gradient) by trilinear interpolation."""
    import torch

    from mmo_gb300 import grids as GR
    from mmo_gb300 import lib as L
    from mmo_gb300.ff import UFFScorer

    s = system_for_rank(0, args.poses)
    dev = torch.device("cuda", 0)
    sc = UFFScorer(0)
    sc.set_protein(s.pocket)
    sc.set_ligand(s.ligand)
    types, per = GR.type2id([s.ligand])
    pxyz = s.pocket.xyz()
    margin = 3.0 * GR.CHARGED_CUTOFF
    origin, dims = GR.lattice_from_box(GR.GRID_STEP, pxyz.min(axis=0) - margin,
                                       pxyz.max(axis=0) + margin)
    roi_out_radius = 10.0
    mask_c = np.zeros(3)
    mask_r = GR.roi_mask_radius(roi_out_radius)
    nelem = len({t[0] for t in types})

    def build():
        return sc.build_grids(GR.GRID_STEP, dims, origin, types, mask_center=mask_c,
                              mask_radius=mask_r, max_E=GR.MAX_E)

    sc.set_profiling(True)  # pair counts of the build (a counting variant of the kernel)
    build()
    st = sc.grid_build_stats()
    sc.set_profiling(False)
    # the fastest launch shape (1, 2 or 4 lattice points per lane; the values are the same)
    shape_ms = {}
    for kp in (1, 2, 4):
        sc.set_grid_build(kp)
        build()
        shape_ms[kp] = min(build() for _ in range(3))
    kp_best = min(shape_ms, key=shape_ms.get)
    sc.set_grid_build(kp_best)
    for _ in range(max(args.warmup, 3)):
        build()
    steps = max(1, min(args.steps, 50))
    clocks = Clocks(0)
    clocks.start()
    ms = [build() for _ in range(steps)]
    clk = clocks.stop()
    nvals = st["points"] * len(types)
    value = nvals * len(ms) / (sum(ms) * 1e-3)
    # end to end: protein upload, build and the download of every grid value
    e2e = []
    gbytes = 4 * len(types) * int(np.prod(dims))
    for k in range(2 + steps // 5):
        t = time.perf_counter()
        sc.set_protein(s.pocket)
        build()
        g = sc.grid_values()
        if k >= 2:
            e2e.append(time.perf_counter() - t)
    e2e_val = nvals * len(e2e) / sum(e2e)
    # the interpolated scoring of the 4,096 poses (energy + gradient)
    B, nd = s.poses.shape
    d_dofs = torch.from_numpy(s.poses).to(dev)
    d_E = torch.empty(B, dtype=torch.float64, device=dev)
    d_G = torch.empty((B, nd), dtype=torch.float32, device=dev)
    d_st = torch.empty(B, dtype=torch.int32, device=dev)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    sp = stream.cuda_stream
    flags = L.F_INTER | L.F_INTRA | L.F_GRAD | L.F_GRID

    def score():
        sc.score_poses_device(d_dofs.data_ptr(), B, d_E.data_ptr(), d_G.data_ptr(),
                              d_st.data_ptr(), flags, sp)

    for _ in range(max(args.warmup, 3)):
        score()
    torch.cuda.synchronize()
    sc.set_profiling(True)
    ev, stages = [], []
    for _ in range(args.steps):
        flush.zero_()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        score()
        b.record(stream)
        ev.append((a, b))
        stages.append(sc.stage_times())
    torch.cuda.synchronize()
    sc.set_profiling(False)
    sms = [a.elapsed_time(b) for a, b in ev]
    iv = B * len(sms) / (sum(sms) * 1e-3)
    stg = np.mean(np.array(stages), axis=0)
    st_bits = d_st.cpu().numpy()
    h = torch.from_numpy(s.poses).pin_memory()
    ie = []
    for k in range(args.warmup + args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t = time.perf_counter()
        Eh, Gh, sth = sc.score_poses(h.numpy(), grad=True, grid=True)
        if k >= args.warmup:
            ie.append(time.perf_counter() - t)
    ie_val = B * len(ie) / sum(ie)
    peak = sc.fp32_peak_tflops()
    # flops per (point, atom) pair of the kernel's formulation: distance from float
    # pairs, switch, electrostatics 24; the factorised vdW sums of geometric mixing 9
    # (per-element sums, 8 per element, for Lorentz-Berthelot)
    flops_pair = 24 + 9
    kernel_ms = float(np.mean(ms))
    achieved = flops_pair * st["pairs_within_cutoff"] / (kernel_ms * 1e-3) * 1e-12
    line = {
        "metric": "grid values/s (per-type UFF interaction grids, 0.5 A lattice)",
        "value": value, "unit": "values/s", "n_gpus": 1, "steps": steps,
        "warmup": max(args.warmup, 3), "ms_per_step": kernel_ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "grids of the 4096-pose workload's system: 6000-atom pocket, "
                               "%d ligand atom types (%d elements), lattice %dx%dx%d at 0.5 A "
                               "(protein box + 36 A margin), mask sphere r = %.0f A "
                               "(ROI outer radius %.0f A + 24 A)" %
                               (len(types), nelem, dims[0], dims[1], dims[2], mask_r,
                                roi_out_radius),
                   "masked_points": st["points"], "values_per_build": nvals,
                   "points_per_lane": kp_best, "shape_ms": shape_ms,
                   "grid_bytes": gbytes,
                   "l2": "each build writes %.1f GB (> L2)" % (gbytes / 1e9)},
        "e2e": {"value": e2e_val, "unit": "values/s", "h2d_bytes_per_step": int(36 * s.pocket.n),
                "d2h_bytes_per_step": gbytes,
                "what": "mmo_set_protein + mmo_build_grids + mmo_grid_values (host copy)"},
        "interp": {"metric": "poses/s (energy+grad) by grid interpolation", "value": iv,
                   "unit": "poses/s", "ms_per_step": float(np.mean(sms)),
                   "stages_ms": {"rebuild": float(stg[0]), "lookup": float(stg[1]),
                                 "finish": float(stg[2])},
                   "e2e": {"value": ie_val, "unit": "poses/s",
                           "h2d_bytes_per_step": int(s.poses.nbytes),
                           "d2h_bytes_per_step": int(Eh.nbytes + Gh.nbytes + sth.nbytes)},
                   "status_off_grid": int(np.count_nonzero(st_bits & L.S_OFF_GRID)),
                   "l2": "flushed before every timed step (256 MiB write), not timed"},
        "roofline": {"bound": "fp32", "kernel": "k_grid_build", "achieved": achieved,
                     "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                     "traffic": None,
                     "flops_per_pair": flops_pair, "pairs_within_cutoff": st["pairs_within_cutoff"],
                     "pairs_evaluated": st["pairs_evaluated"], "ms_per_launch": kernel_ms,
                     "peak_source": "measured FP32 FMA probe on this GPU (mmo_fp32_fma_peak)"},
        "gpu_launches": steps,
        "clocks": clk,
    }
    if not args.no_cpu:
        from oracle import oracle as O

        nthreads = os.cpu_count() or 1
        # every masked lattice point (the whole build), in random order
        rng = np.random.default_rng(11)
        ax = [np.arange(n) for n in dims]
        ii, jj, kk = np.meshgrid(*ax, indexing="ij")
        pts = origin + GR.GRID_STEP * np.stack([ii.ravel(), jj.ravel(), kk.ravel()], axis=1)
        pts = pts[((pts - mask_c) ** 2).sum(axis=1) < mask_r * mask_r]
        pts = pts[rng.permutation(len(pts))]
        ta = np.array([t[0] for t in types], np.int32)
        tq = np.array([t[1] for t in types])
        n0 = 256
        t0 = time.perf_counter()
        O.grid_points(s.pocket, pts[:n0], ta, tq, nthreads=nthreads)
        per = (time.perf_counter() - t0) / n0
        n = int(min(len(pts), max(n0, 30.0 / max(per, 1e-9))))
        t0 = time.perf_counter()
        ref = O.grid_points(s.pocket, pts[:n], ta, tq, nthreads=nthreads)
        dt = time.perf_counter() - t0
        # the error of the GPU values relative to max(|E|, sum of |pair terms|) on a
        # sub-sample (capped values excluded: both sides hold max_E)
        m = min(n, 20000)
        ref_s, scale = O.grid_points(s.pocket, pts[:m], ta, tq, nthreads=nthreads,
                                     with_scale=True)
        gi = np.rint((pts[:m] - origin) / GR.GRID_STEP).astype(int)
        got = g[:, gi[:, 2], gi[:, 1], gi[:, 0]].T.astype(np.float64)
        free = ref_s < GR.MAX_E
        # over values whose terms reach 1e-2 kcal/mol: near the 12 A cut-off a lone
        # switched term carries the FP32 rounding of r^2 (relative 1e-7 of 144,
        # through w = (1 - r^2/144)^2) as a relative error that grows as w -> 0
        big = free & (scale >= 1e-2)
        rel = np.where(big, np.abs(got - ref_s) /
                       np.maximum(np.maximum(np.abs(ref_s), scale), 1e-300), 0.0)
        err = float(rel.max())
        abs_err = float(np.abs(got - ref_s)[free].max())
        wk, wl = np.unravel_index(int(rel.argmax()), rel.shape)
        wp = pts[wk]
        worst = {"got": float(got[wk, wl]), "ref": float(ref_s[wk, wl]),
                 "scale": float(scale[wk, wl]), "type": int(wl),
                 "ijk": [int(v) for v in gi[wk]],
                 "mask_margin_A": float(mask_r - np.sqrt(((wp - mask_c) ** 2).sum())),
                 "nearest_atom_A": float(np.sqrt(((pxyz - wp) ** 2).sum(axis=1)).min())}
        cap_ok = bool(np.all(got[~free] == GR.MAX_E))
        line["cpu_baseline"] = {"value": n * len(types) / dt, "unit": "values/s",
                                "cores": nthreads, "kind": "port",
                                "sample": "%d of the %d masked lattice points x %d types, "
                                          "%.1f s (12 A cell-list neighbour sum per point)" %
                                          (n, len(pts), len(types), dt),
                                "max_rel_err_gpu_vs_fp64": err,
                                "error_scale": "max(|E|, sum of |pair terms|), 20000 points, "
                                               "values with terms >= 1e-2 kcal/mol",
                                "max_abs_err_kcal": abs_err,
                                "capped_values_equal": cap_ok, "worst": worst}
    print(json.dumps(line), flush=True)
    sc.close()
    return 0


def _dock_launches(poses, k, per_block=2048):
    """Kernels of one mmo_dock_exhaustive: the sweep, then the top-k merges."""
    n = -(-poses // per_block) * k
    launches = 1
    while n > k:
        n = -(-n // per_block) * k
        launches += 1
    return launches


def run_dock(args):
    """Exhaustive rigid docking (Lds.exhaustive_rigid_ligand_docking): a 24-atom
    ligand in a 6,000-atom cavity site, grids and masks built first, every pose
    of a 4 A ROI at 0.5 A x 2,000 super-Fibonacci rotations scored after the
    vdW clash test, the 64 best kept."""
    from mmo_gb300 import grids as GR
    from mmo_gb300 import synth

    site = synth.docking_site(seed=21, n_pocket=6000, r_in=8.0, r_out=20.0, n_atoms=24, n_rot=4)
    import torch

    from mmo_gb300.ff import UFFScorer

    sc = UFFScorer(0)
    sc.set_protein(site.pocket)
    sc.set_ligand(site.ligand)
    types, (lt,) = GR.type2id([site.ligand])
    pxyz = site.pocket.xyz()
    margin = 3.0 * GR.CHARGED_CUTOFF
    origin, dims = GR.lattice_from_box(GR.GRID_STEP, pxyz.min(axis=0) - margin,
                                       pxyz.max(axis=0) + margin)
    roi_c, roi_r, step, nrot, k = np.zeros(3), 4.0, 0.5, 2000, 64
    grid_ms = sc.build_grids(GR.GRID_STEP, dims, origin, types, mask_center=roi_c,
                             mask_radius=GR.roi_mask_radius(roi_r))
    t = time.perf_counter()
    sc.build_masks(site.pocket.radius)
    mask_s = time.perf_counter() - t
    const_intra = float(sc.ene_intra(site.ligand))

    def dock():
        return sc.dock_exhaustive(roi_c, roi_r, step, nrot, topk=k, const_intra=const_intra,
                                  lig_radius=site.ligand.radius)

    for _ in range(max(args.warmup, 3)):
        res = dock()
    steps = max(1, min(args.steps, 20))
    clocks = Clocks(0)
    clocks.start()
    ms, wall = [], []
    for _ in range(steps):
        torch.cuda.synchronize()
        t = time.perf_counter()
        res = dock()
        wall.append(time.perf_counter() - t)
        ms.append(res["ms"])
    clk = clocks.stop()
    poses = res["poses"]
    value = poses * len(ms) / (sum(ms) * 1e-3)
    e2e = poses * len(wall) / sum(wall)
    L = site.ligand.n
    line = {
        "metric": "poses/s (exhaustive rigid docking: vdW clash test + interpolated E_inter + "
                  "top-k)",
        "value": value, "unit": "poses/s", "n_gpus": 1, "steps": steps,
        "warmup": max(args.warmup, 3), "ms_per_step": float(np.mean(ms)),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": "%d-atom ligand, %d-atom cavity site, ROI r = %.0f A at %.1f A "
                               "(%d positions) x %d super-Fibonacci rotations = %d poses, top %d" %
                               (L, site.pocket.n, roi_r, step, res["positions"], nrot, poses, k),
                   "grids": "%dx%dx%d x %d types, built in %.2f ms" %
                            (dims[0], dims[1], dims[2], len(types), grid_ms),
                   "masks_s": mask_s, "scored": res["scored"], "clashed": res["clashed"],
                   "precision": "rotated atoms in lattice units as float pairs (FP64 once per "
                                "rotation and atom), float-pair cell fractions, FP32 trilinear "
                                "terms, compensated FP32 sum per pose",
                   "l2": "grids %.2f GB (> L2); the poses touch a small region of them, read "
                         "again by every call (not flushed)" %
                         (4.0 * len(types) * dims[0] * dims[1] * dims[2] / 1e9)},
        "e2e": {"value": e2e, "unit": "poses/s", "h2d_bytes_per_step": 8 * 9 * nrot,
                "d2h_bytes_per_step": 16 * k,
                "what": "mmo_dock_exhaustive wall time (rotations and positions uploaded, "
                        "top-k downloaded)"},
        "best": {"score": res["best_score"], "rot": res["best_rot"],
                 "pos": [float(v) for v in res["best_pos"]]},
        "gpu_launches": steps * _dock_launches(res["poses"], k),
        "clocks": clk,
    }
    if not args.no_cpu:
        from oracle import oracle as O

        g = sc.grid_values()
        vdw, _ = sc.mask_values()
        lat = O.lattice(GR.GRID_STEP, dims, origin)
        from mmo_gb300.ff import so3_rotations

        R = so3_rotations(nrot)
        n0 = 20
        t0 = time.perf_counter()
        O.dock_scores(lat, g, vdw, site.ligand, lt, site.ligand.radius, roi_c, roi_r, step,
                      R[:n0], const_intra)
        per = (time.perf_counter() - t0) / (res["positions"] * n0)
        nr = int(min(nrot, max(n0, 10.0 / max(per * res["positions"], 1e-12))))
        t0 = time.perf_counter()
        sc_cpu, _ = O.dock_scores(lat, g, vdw, site.ligand, lt, site.ligand.radius, roi_c, roi_r,
                                  step, R[:nr], const_intra)
        dt = time.perf_counter() - t0
        ok = np.isfinite(sc_cpu)
        line["cpu_baseline"] = {"value": res["positions"] * nr / dt, "unit": "poses/s", "cores": 1,
                                "kind": "port",
                                "sample": "all %d positions x the first %d rotations, %.1f s "
                                          "(one thread, as the reference's loop)" %
                                          (res["positions"], nr, dt),
                                "best_of_sample": float(sc_cpu[ok].min()) if ok.any() else None}
    print(json.dumps(line), flush=True)
    sc.close()
    return 0


def energy_only_batch(args, torch, sc, L, dev, stream, flush):
    """65,536 poses of inter + intra energy (no gradient) per step, on the
    4,096-pose workload's ligand and pocket: device-resident poses/s (L2
    flushed before every step), end to end through mmo_score_poses with
    page-locked host buffers, and the sweep's roofline at 26 flops per
    counted pair.  The autotuner picks this batch's plan first."""
    from mmo_gb300 import synth

    big = synth.pose_batch(n_poses=65536, seed=1)
    B = len(big.poses)
    sp = stream.cuda_stream
    d_dofs = torch.from_numpy(big.poses).to(dev)
    d_E = torch.empty(B, dtype=torch.float64, device=dev)
    d_st = torch.empty(B, dtype=torch.int32, device=dev)
    flags = L.F_INTER | L.F_INTRA

    def step():
        sc.score_poses_device(d_dofs.data_ptr(), B, d_E.data_ptr(), None, d_st.data_ptr(),
                              flags, sp)

    tune_ms = None
    if not args.no_tune:
        tune_ms = sc.tune_device(d_dofs.data_ptr(), B, d_E.data_ptr(), None, d_st.data_ptr(),
                                 flags, sp)
    for _ in range(3):
        flush.zero_()
        step()
    torch.cuda.synchronize()
    steps = max(5, min(args.steps, 40))
    sc.set_profiling(True)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(steps)]
    sweep_ms = []
    for a, b in ev:
        flush.zero_()
        a.record(stream)
        step()
        b.record(stream)
        sweep_ms.append(sc.stage_times()[1])
    torch.cuda.synchronize()
    sc.set_profiling(False)
    pairs_ev, pairs_all = sc.pair_count()
    ms = [a.elapsed_time(b) for a, b in ev]
    E = d_E.cpu().numpy()
    h_dofs = torch.from_numpy(big.poses).pin_memory()
    h_out = (torch.empty(B, dtype=torch.float64).pin_memory().numpy(), None,
             torch.empty(B, dtype=torch.int32).pin_memory().numpy())
    e2e = []
    for k in range(3 + min(steps, 10)):
        flush.zero_()
        torch.cuda.synchronize()
        t = time.perf_counter()
        sc.score_poses(h_dofs.numpy(), grad=False, out=h_out)
        if k >= 3:
            e2e.append(time.perf_counter() - t)
    peak = sc.fp32_peak_tflops()
    sweep = float(np.mean(sweep_ms))
    achieved = FLOPS_PAIR_E * pairs_ev / (sweep * 1e-3) * 1e-12
    return {"metric": "poses/s (energy: inter + intra, no gradient)",
            "value": B * steps / (sum(ms) * 1e-3), "unit": "poses/s",
            "ms_per_step": sum(ms) / steps, "steps": steps,
            "config": {"workload": "energy only, 65536 poses/step, 48-atom ligand (8 torsions) "
                                   "vs 6000-atom pocket, the same system as the main line",
                       "poses_per_step_per_gpu": B, "l2": "flushed before every timed step",
                       "plan": dict(sc.plan(), tuned_ms=tune_ms)},
            "e2e": {"value": B * len(e2e) / sum(e2e), "unit": "poses/s",
                    "h2d_bytes_per_step": int(big.poses.nbytes),
                    "d2h_bytes_per_step": int(B * 8 + B * 4)},
            "roofline": {"bound": "fp32", "kernel": "k_pairs_cull (cut-off pair sweep, energy)",
                         "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                         "frac": achieved / peak, "flops_per_pair": FLOPS_PAIR_E,
                         "pairs_evaluated": pairs_ev, "pairs_all": pairs_all,
                         "ms_per_launch": sweep,
                         "peak_source": "measured FP32 FMA probe on this GPU"},
            "status_bits_set": int(np.count_nonzero(d_st.cpu().numpy())),
            "E": E, "system": big}


def large_pocket_batch(args, torch, L, dev, stream, flush):
    """4,096 poses of the main line's 48-atom ligand with the gradient against a
    12,000-atom pocket (22.7 A sphere: the 6,000-atom pocket's atom density),
    above the sweep's shared-memory staging of the protein: device-resident
    poses/s (L2 flushed before every step), the stage times and the sweep's cost
    per evaluated pair, to set beside the main line's."""
    from mmo_gb300 import synth
    from mmo_gb300.ff import UFFScorer

    sysm = synth.pose_batch(n_poses=4096, seed=1, n_pocket=12000, radius=22.7)
    B = len(sysm.poses)
    sc = UFFScorer(0)
    sc.set_protein(sysm.pocket)
    sc.set_ligand(sysm.ligand)
    sp = stream.cuda_stream
    d_dofs = torch.from_numpy(sysm.poses).to(dev)
    d_E = torch.empty(B, dtype=torch.float64, device=dev)
    d_G = torch.empty(sysm.poses.shape, dtype=torch.float32, device=dev)
    d_st = torch.empty(B, dtype=torch.int32, device=dev)
    flags = L.F_INTER | L.F_INTRA | L.F_GRAD

    def step():
        sc.score_poses_device(d_dofs.data_ptr(), B, d_E.data_ptr(), d_G.data_ptr(),
                              d_st.data_ptr(), flags, sp)

    tune_ms = None
    if not args.no_tune:
        tune_ms = sc.tune_device(d_dofs.data_ptr(), B, d_E.data_ptr(), d_G.data_ptr(),
                                 d_st.data_ptr(), flags, sp)
    for _ in range(3):
        flush.zero_()
        step()
    torch.cuda.synchronize()
    steps = max(5, min(args.steps, 40))
    sc.set_profiling(True)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(steps)]
    stage = []
    for a, b in ev:
        flush.zero_()
        a.record(stream)
        step()
        b.record(stream)
        stage.append(sc.stage_times())
    torch.cuda.synchronize()
    sc.set_profiling(False)
    pairs_ev, pairs_all = sc.pair_count()
    ms = [a.elapsed_time(b) for a, b in ev]
    st = np.mean(np.array(stage), axis=0)
    out = {"metric": "poses/s (energy+grad)", "value": B * steps / (sum(ms) * 1e-3),
           "unit": "poses/s", "ms_per_step": sum(ms) / steps, "steps": steps,
           "config": {"workload": "energy+grad, 4096 poses/step, 48-atom ligand (8 torsions) vs "
                                  "12000-atom pocket (22.7 A sphere)",
                      "poses_per_step_per_gpu": B, "pocket_atoms": 12000,
                      "l2": "flushed before every timed step",
                      "plan": dict(sc.plan(), tuned_ms=tune_ms)},
           "stages_ms": dict(zip(("rebuild", "sweep", "finish", "sort"), (float(v) for v in st))),
           "pairs_evaluated": pairs_ev, "pairs_all": pairs_all,
           "sweep_ns_per_evaluated_pair": float(st[1]) * 1e6 / pairs_ev,
           "status_bits_set": int(np.count_nonzero(d_st.cpu().numpy())),
           "E": d_E.cpu().numpy(), "G": d_G.cpu().numpy(), "system": sysm}
    sc.close()
    return out


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "ragged":
        return run_ragged(args)
    if args.workload == "mc":
        return run_mc(args)
    if args.workload == "grid":
        return run_grid(args)
    if args.workload == "dock":
        return run_dock(args)

    import torch

    from mmo_gb300 import lib as L
    from mmo_gb300.ff import UFFScorer

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    s = system_for_rank(rank, args.poses)
    sc = UFFScorer(local)
    sc.set_protein(s.pocket)
    sc.set_ligand(s.ligand)
    L_atoms, P, nrb, B = s.ligand.n, s.pocket.n, s.ligand.nrb, args.poses
    nd = 6 + nrb
    flags = L.F_INTER | L.F_INTRA | L.F_GRAD

    d_dofs = torch.from_numpy(s.poses).to(dev)
    d_E = torch.empty(B, dtype=torch.float64, device=dev)
    d_G = torch.empty((B, nd), dtype=torch.float32, device=dev)
    d_st = torch.empty(B, dtype=torch.int32, device=dev)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)  # 256 MiB > L2
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    sp = stream.cuda_stream

    def step():
        sc.score_poses_device(d_dofs.data_ptr(), B, d_E.data_ptr(), d_G.data_ptr(),
                              d_st.data_ptr(), flags, sp)

    # launch plan from the autotuner (times the candidate plans on this batch)
    tune_ms = None
    if not args.no_tune:
        tune_ms = sc.tune_device(d_dofs.data_ptr(), B, d_E.data_ptr(), d_G.data_ptr(),
                                 d_st.data_ptr(), flags, sp)
    # warm-up (also builds the launch plan and scratch)
    for _ in range(max(args.warmup, 3)):
        flush.zero_()
        step()
    sc.sync(sp)
    torch.cuda.synchronize()

    # ---- device-resident batched steps ------------------------------------
    sc.set_profiling(True)
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    pair_ms, stage_ms = [], []
    clocks = Clocks(local)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    t0 = time.perf_counter()
    for k in range(args.steps):
        flush.zero_()
        starts[k].record(stream)
        step()
        ends[k].record(stream)
        stage_ms.append(sc.stage_times())  # waits for this step's events
        pair_ms.append(stage_ms[-1][1])
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    sc.set_profiling(False)
    sc.sync(sp)
    plan = sc.plan()
    launches = sc.last_launches()
    pairs_ev, pairs_all = sc.pair_count()
    # the pairs within the 12 A cutoff of the same poses: the second roofline denominator
    pairs_12 = sc.pairs_within(12.0)
    step_ms = [a.elapsed_time(b) for a, b in zip(starts, ends)]
    tot_ms = float(sum(step_ms))
    if dist:
        t = torch.tensor([tot_ms], dtype=torch.float64, device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        tot_ms = float(t.item())
    value = world * B * args.steps / (tot_ms * 1e-3)
    E_gpu = d_E.cpu().numpy()
    G_gpu = d_G.cpu().numpy()
    st = d_st.cpu().numpy()

    # ---- end to end through the C ABI with host buffers -------------------
    h_dofs = torch.from_numpy(s.poses).pin_memory()
    # page-locked result buffers, as a caller keeps them between calls
    h_out = (torch.empty(B, dtype=torch.float64).pin_memory().numpy(),
             torch.empty(tuple(s.poses.shape), dtype=torch.float32).pin_memory().numpy(),
             torch.empty(B, dtype=torch.int32).pin_memory().numpy())
    e2e_ms = []
    for k in range(args.warmup + args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t = time.perf_counter()
        E_h, G_h, st_h = sc.score_poses(h_dofs.numpy(), grad=True, out=h_out)
        if k >= args.warmup:
            e2e_ms.append((time.perf_counter() - t) * 1e3)
    e2e_tot = sum(e2e_ms)
    if dist:
        t = torch.tensor([e2e_tot], dtype=torch.float64, device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_tot = float(t.item())
    e2e_val = world * B * len(e2e_ms) / (e2e_tot * 1e-3)
    h2d = s.poses.nbytes
    d2h = E_h.nbytes + G_h.nbytes + st_h.nbytes

    # ---- plain one-pose-per-launch path on a sample ------------------------
    n_plain = min(512, B)
    plain_dev_ms, plain_e2e_ms = 0.0, 0.0
    for k in range(8):  # warm-up
        sc.score_poses_device(d_dofs[k:k + 1].data_ptr(), 1, d_E.data_ptr(), d_G.data_ptr(),
                              d_st.data_ptr(), flags, sp)
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for k in range(n_plain):
        sc.score_poses_device(d_dofs[k:k + 1].data_ptr(), 1, d_E[k:k + 1].data_ptr(),
                              d_G[k:k + 1].data_ptr(), d_st[k:k + 1].data_ptr(), flags, sp)
    ev1.record(stream)
    torch.cuda.synchronize()
    plain_dev_ms = ev0.elapsed_time(ev1)
    plain_launches = sc.last_launches()
    t = time.perf_counter()
    for k in range(n_plain):
        sc.score_poses(s.poses[k:k + 1], grad=True)
    plain_e2e_ms = (time.perf_counter() - t) * 1e3
    plain_v = n_plain / (plain_dev_ms * 1e-3)
    plain_e2e = n_plain / (plain_e2e_ms * 1e-3)

    # ---- the 65,536-pose energy-only batch (same ligand and pocket) ----------
    cfg1 = None
    if not args.no_energy_only:
        cfg1 = energy_only_batch(args, torch, sc, L, dev, stream, flush)
    # ---- 4,096 poses against a 12,000-atom pocket ----------------------------
    big = None
    if not args.no_large_pocket:
        big = large_pocket_batch(args, torch, L, dev, stream, flush)

    # ---- roofline of the pair sweep -----------------------------------------
    peak = sc.fp32_peak_tflops()
    pair_avg = float(np.mean(pair_ms))
    flops = FLOPS_PAIR_GRAD * pairs_ev
    achieved = flops / (pair_avg * 1e-3) * 1e-12
    culled = pairs_ev < pairs_all
    # DRAM bytes per launch of the sweep from the committed ncu capture of this workload
    traffic = None
    try:
        with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "profiles",
                               "traffic.json")) as f:
            tr = json.load(f).get("k_pairs_cull" if culled else "k_pairs")
        if tr and B == 4096 and P == 6000 and L_atoms == 48:
            traffic = tr["dram_bytes_per_launch"]
    except (OSError, ValueError, KeyError):
        traffic = None

    line = {
        "metric": METRIC, "value": value, "unit": "poses/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": tot_ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": WORKLOAD, "poses_per_step_per_gpu": B, "ligand_atoms": L_atoms,
                   "torsions": nrb, "pocket_atoms": P,
                   "precision": "fp32 pair terms, fp64 per-pose sums",
                   "l2": "flushed before every timed step (256 MiB write), not timed",
                   "parallelism": "dp%d (poses sharded, no collective)" % world,
                   "plan": dict(plan, tuned_ms=tune_ms)},
        "e2e": {"value": e2e_val, "unit": "poses/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h)},
        "gpu_launches": launches * args.steps,
        "plain": {"value": plain_v, "e2e": plain_e2e, "unit": "poses/s", "sample": n_plain,
                  "launches_per_pose": plain_launches},
        "batched_vs_plain": value / world / plain_v,
        "batched_vs_plain_e2e": e2e_val / world / plain_e2e,
        "roofline": {"bound": "fp32",
                     "kernel": ("k_pairs_cull (cut-off pair sweep, energy+gradient)" if culled
                                else "k_pairs (pair sweep, energy+gradient)"),
                     "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "traffic_unit": "DRAM bytes per launch (ncu capture)",
                     "peak_source": "measured FP32 FMA probe on this GPU (mmo_fp32_fma_peak)",
                     "flops_per_pair": FLOPS_PAIR_GRAD, "pairs_evaluated": pairs_ev,
                     "pairs_all": pairs_all, "flops_per_launch": flops,
                     "ms_per_launch": pair_avg,
                     "pairs_within_12A": pairs_12,
                     "frac_within_12A": FLOPS_PAIR_GRAD * pairs_12 / (pair_avg * 1e-3) * 1e-12 / peak},
        "stages_ms": dict(zip(("rebuild", "sweep", "finish", "sort"),
                              (float(v) for v in np.mean(np.array(stage_ms), axis=0)))),
        "clocks": clk,
        "wall_s_timed": wall,
        "status_bits_set": int(np.count_nonzero(st)),
    }
    if rank == 0 and not args.no_cpu:
        nthreads = os.cpu_count() or 1
        legs = cpu_legs(s, nthreads, E_gpu)
        # the faster of the two sums on all host threads (both are the
        # reference's: -ff BrL brute, -ff Bst through its 12 A neighbour query)
        key = max(("all_threads", "brute_all_threads"), key=lambda k: legs[k]["value"])
        main = legs[key]
        line["cpu_baseline"] = {"value": main["value"], "unit": "poses/s", "cores": nthreads,
                                "kind": "port",
                                "sample": "%d of the 4096 poses, %.1f s, energy + central "
                                          "differences (29 scorings/pose), %s"
                                          % (main["sample_poses"], main["seconds"],
                                             main["inter_sum"]),
                                "max_rel_err_E_gpu_vs_fp64": main["max_rel_err_E_gpu_vs_fp64"],
                                "legs": legs}
        # every pose of the step against the FP64 oracle (energy and gradient)
        line["errors"] = errors_vs_oracle(s, E_gpu, G_gpu, nthreads)
        if cfg1 is not None:
            idx = np.random.default_rng(7).choice(len(cfg1["E"]), 4096, replace=False)
            cfg1_sys = cfg1.pop("system")
            cfg1["errors"] = errors_vs_oracle(cfg1_sys, cfg1.pop("E")[idx], None, nthreads,
                                              poses=idx)
        if big is not None:
            idx = np.random.default_rng(8).choice(len(big["E"]), 256, replace=False)
            big["errors"] = errors_vs_oracle(big["system"], big["E"][idx], big["G"][idx],
                                             nthreads, poses=idx)
    if cfg1 is not None:
        cfg1.pop("E", None)
        cfg1.pop("system", None)
        line["energy_only_65536"] = cfg1
    if big is not None:
        for k in ("E", "G", "system"):
            big.pop(k, None)
        big["sweep_ns_per_evaluated_pair_main_line"] = (line["roofline"]["ms_per_launch"] * 1e6 /
                                                        line["roofline"]["pairs_evaluated"])
        line["pocket_12000"] = big
    if rank == 0:
        print(json.dumps(line), flush=True)
    sc.close()
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
