"""Throughput benchmark: attempted atom moves per second on one GB300.

Every default run measures the five workloads of the engine's configuration
set on the production path (equilibration as the warm-up, then timed
production cycles that sample E, E^2 and the histograms every cycle):

  cu55     Sutton-Chen EAM Cu55 (scripts/cu55.jl:39-48 parameters), icosahedral
           start, SphericalBC(14 bohr), 32 replicas over 200-1000 K   (headline)
  ne13     ELJEven Ne13, sphere 11 bohr, 16 replicas over 4-16 K
  npt108   bulk Ne NPT, 108 atoms fcc in CubicBC(25.2), 32 replicas over 10-40 K
  batched  256 runs of ELJEven Ne clusters, N in {13, 38, 55, 101, 147}, 16 replicas
  nn55     RuNNer NN potential on Cu55, 64 replicas over 300-900 K, delayed
           acceptance with a GPU-trained pair surrogate

The chosen form is FP32 move rows with an FP64 running total resynchronised by
a full FP64 recompute every 1000 cycles, batched as B independent PT runs
(different Philox streams) per launch with an autotuned launch shape per atom
count; the plain FP64 form is timed on the same batch.  The line's `value`,
`roofline`, `cpu_baseline` and `e2e` are the headline workload's; `workloads`
holds one record per workload.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--workload all|cu55|ne13|npt108|batched|nn55]
  python bench.py --impl reference ...   # the CPU oracle on all host cores

Under torchrun (N>1) every rank runs its own batch on its own GPU (replicas
only, weak scaling; no collective on the data path), timing is max over ranks.
"""
import argparse
import ctypes
import functools
import hashlib
import json
import math
import multiprocessing as mp
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

C_NE = [-10.5097942564988, 989.725135614556, -101383.865938807, 3918846.12841668,
        -56234083.4334278, 288738837.441765]
CU_EAM = dict(n=8.482, m=4.692, eps=0.0367493 * 0.0370, C=27.561, a=0.25 * 18.8973)
P_NE = 101325 * 3.398928944382626e-14
HEADLINE = "cu55"
ALL = ["cu55", "ne13", "npt108", "batched", "nn55"]
METRIC = "atom-moves/sec on 1 GB300, chosen vs plain FP64 form at equal Cv(T) error"

# Counters of the chosen form's cycle kernel from one ncu capture per workload
# (smsp__inst_executed over the launch's attempted moves; DRAM read + write
# bytes of the launch per run), valid for the launch shape (lanes per walker)
# and the kernel sources whose sha256 prefix is given: a changed kernel drops
# them from the line instead of reporting stale figures.
CSRC = os.path.join(ROOT, "paralleltemperingmontecarlo.jl_gb300", "csrc")
NARROW_SRC = ("ptmc_cycles32n.cu", "ptmc_fp32.cuh")
PROFILED = {
    # 760 runs x 32 replicas of Cu55, 4 lanes per walker, one 20-cycle launch
    # (26.8 M attempted moves): 2.511e9 warp instructions, 78.8 MB DRAM
    "cu55": dict(inst_per_move=93.9, lanes=4, dram_bytes_per_run=78.85e6 / 760,
                 src=NARROW_SRC, src_sha="6e43710641953936"),
}


def kernel_sha(files):
    h = hashlib.sha256()
    for f in files:
        h.update(open(os.path.join(CSRC, f), "rb").read())
    return h.hexdigest()[:16]


# --------------------------------------------------------------- workloads
@functools.lru_cache(maxsize=1)
def _cu55_ico():
    d = json.load(open(os.path.join(ROOT, "tests", "golden", "nn_cu55.json")))
    return np.array(d["ico55_nm"]) * (d["cu_lattice_nm"] * d["nm_to_bohr"])


def cu55_ico():
    return _cu55_ico().copy()


def sphere_start(N, radius, min_sep, seed):
    return _starts().sphere_start(N, radius, min_sep, seed)


def fcc(ncell, a, jitter, seed):
    return _starts().fcc_box(ncell, a, jitter, seed)


def _starts():
    import __graft_entry__ as g
    g.load_package()
    import ptmc_gb300.starts as st
    return st


def workload(name):
    """Description of one workload: replicas, temperature range, potential,
    ensemble, boundary, per-run atom counts and start configurations, chosen
    and plain-form cycles per timed step, and the algorithmic FP32 work per
    pair (ELJ 24 ops, +9 with the minimum image; EAM 17 ops + 3 MUFU)."""
    if name == "cu55":
        return dict(name="cu55_eam", R=32, T=(200.0, 1000.0), pot="eam", ens="nvt",
                    bc=("sphere", 14.0), sizes=lambda B: [55] * B,
                    start=lambda n, k: cu55_ico(), resync=1000, flops_pair=17, mufu_pair=3,
                    cycles=200, plain_cycles=20)
    if name == "ne13":
        return dict(name="ne13_eljeven", R=16, T=(4.0, 16.0), pot="elj", ens="nvt",
                    bc=("sphere", 11.0), sizes=lambda B: [13] * B,
                    start=lambda n, k: sphere_start(13, 8.0, 4.5, 1234 + k), resync=1000,
                    flops_pair=24, mufu_pair=1, cycles=200, plain_cycles=100)
    if name == "npt108":
        return dict(name="ne108_npt", R=32, T=(10.0, 40.0), pot="elj", ens="npt",
                    bc=("cubic", 25.2), sizes=lambda B: [108] * B,
                    start=lambda n, k: fcc(3, 8.4, 0.05, 7 + k), resync=1000,
                    flops_pair=33, mufu_pair=1, cycles=200, plain_cycles=20)
    if name == "nn55":
        return dict(name="nn55_runner", R=64, T=(300.0, 900.0), pot="nn", ens="nvt",
                    bc=("sphere", 14.0), sizes=lambda B: [55] * B,
                    start=lambda n, k: cu55_ico(), resync=1000,
                    # FP32 flops of one exactly evaluated move in the table-specialised
                    # kernel: 54 x 53 ordered pairs (j, k) of atoms other than the moved
                    # one at 177 (cut-off products, triangle sums, 14 exponent arguments,
                    # two cosines, powers, 2 x 26 accumulating FMAs; plus 17 MUFU), 1431
                    # unordered pairs at 138 for the moved atom's own angle, and the MLP
                    # 2 x 55 x (31 x 20 + 20 x 20 + 20)
                    flops_move=54 * 53 * 177 + 1431 * 138 + 2 * 55 * 1040, flops_pair=0, mufu_pair=0,
                    da=True, cycles=20, plain_cycles=2)
    if name == "batched":
        ns = [13, 38, 55, 101, 147]

        def sizes(B):
            return [ns[k % 5] for k in range(B)]
        return dict(name="batched_uneven_elj", R=16, T=(4.0, 16.0), pot="elj", ens="nvt",
                    bc=("sphere", None), sizes=sizes,
                    start=lambda n, k: sphere_start(n, 0.9 * n ** (1 / 3) * 3, 4.3, 500 + k),
                    resync=1000, flops_pair=24, mufu_pair=1, cycles=200, plain_cycles=20)
    raise SystemExit("unknown workload " + name)


def default_runs(name, n_sm=152):
    return {"cu55": 2 * n_sm, "ne13": 4 * n_sm, "npt108": n_sm, "batched": 256,
            "nn55": max(1, (2 * n_sm) // 64)}[name]


def nn_potential(pk):
    """88 G2/G4 functions of scripts/cu55.jl with r_c = 12 bohr, MLP 88-20-20-1
    with seeded FP32 weights; the output layer is scaled by 0.3 so that the
    exact chain accepts ~20-40 % of the default 0.1-bohr moves at 300-900 K, and
    a 3-bohr hard core (E = 100 below it) keeps atoms apart."""
    tables = json.load(open(os.path.join(ROOT, "tests", "golden", "nn_cu55.json")))
    nodes = [88, 20, 20, 1]
    return pk.RuNNerPotential(pk.RuNNerPotential.sf_table(tables, 12.0),
                              pk.RuNNerPotential.random_weights(nodes, 3, 0.3), nodes, boundary=3.0)


def train_surrogate(pk, eng, sizes, R, cycles=300, records=100000, steps=4000):
    """Delayed acceptance set-up (outside the timed region): capture `records`
    (configuration row, exact dE) pairs of the exact chain over `cycles`
    cycles, train the pair surrogate on the GPU, freeze, enable."""
    every = max(1, (cycles * sum(sizes) * R) // records)
    eng.surrogate_set(pk.PairSurrogate(2.0, 12.0, None, 12.0, 0.0), capacity=records,
                      record_every=every)
    eng.surrogate_record(True)
    t0 = time.perf_counter()
    eng.cycles_nosample(cycles)
    eng.surrogate_record(False)
    t1 = time.perf_counter()
    loss = eng.surrogate_train(steps, batch=512, lr=2e-3)
    t2 = time.perf_counter()
    rows, y = eng.surrogate_records()
    P, sur, _ = eng.surrogate_state()
    held = slice(-min(5000, len(y) // 5), None)
    corr = float(np.corrcoef(sur.eval(P, rows[held]), y[held])[0, 1])
    eng.surrogate_enable(True)
    return dict(records=int(len(y)), record_s=t1 - t0, train_s=t2 - t1, train_steps=steps,
                loss=loss, heldout_corr=corr, escale=sur.escale)


# --------------------------------------------------------------- GPU arm
def start_configs(W, B):
    """The host start configuration of every run (one per run)."""
    return [W["start"](n, r) for r, n in enumerate(W["sizes"](B))]


def make_engine(pk, W, B, precision, cycles_per_launch, seed, device, starts=None, xyz=None,
                eq_cycles=0, init=True):
    """Engine of B runs of workload W.  `starts`: per run, the slot-ordered
    states of an earlier engine (configurations and step sizes) to start from;
    `xyz`: per run, a host start configuration made beforehand; `eq_cycles`:
    MCParams.eq_cycles (ptmc_equilibrate simulates half of them)."""
    R = W["R"]
    sizes = W["sizes"](B)
    mp_ = pk.MCParams(mc_cycles=10 ** 6, eq_cycles=eq_cycles, mc_sample=1, n_traj=R,
                      n_atoms=sizes[0])
    temp = pk.TempGrid(W["T"][0], W["T"][1], R)
    if W["pot"] == "eam":
        pot = pk.EmbeddedAtomPotential(**CU_EAM)
    elif W["pot"] == "nn":
        pot = nn_potential(pk)
    else:
        pot = pk.ELJPotentialEven(C_NE)
    ens = pk.NPT(sizes[0], P_NE) if W["ens"] == "npt" else pk.NVT(sizes[0])
    eng = pk.Engine(mp_, temp, pot, ens, n_runs=B, precision=precision,
                    resync_every=W["resync"], exch_prob=1.0, seed=seed,
                    cycles_per_launch=cycles_per_launch, device=device)
    def bc_of(n):
        if W["bc"][0] == "cubic":
            return pk.CubicBC(W["bc"][1])
        return pk.SphericalBC(W["bc"][1] if W["bc"][1] else 0.9 * n ** (1 / 3) * 3 + 3.0)

    if starts is None and len(set(sizes)) == 1:  # one atom count: one call for every run
        eng.set_configs_batch(np.stack([W["start"](n, r) if xyz is None else xyz[r]
                                        for r, n in enumerate(sizes)]), bc_of(sizes[0]))
    else:
        for r, n in enumerate(sizes):
            if starts is None:
                eng.set_configs(r, pk.Config(W["start"](n, r) if xyz is None else xyz[r], bc_of(n)))
            else:
                st = starts[r]
                eng.set_configs(r, [pk.Config(x, bc_of(n)) for x in st["xyz"]],
                                max_displ=st["max_displ"])
    if init:
        eng.init()
    return eng, sizes


def fill_batch(pk, W, form, n_sm, cycles, seed, device):
    """Runs per batch and FP32 launch shape for a workload of one atom count:
    every candidate shape gets the batch that fills the GPU in whole waves
    (ptmc_occupancy x SMs), a short untimed trial of that batch, and the best
    rate wins.  Returns (runs, (C, L) or None, record)."""
    N, R = W["sizes"](1)[0], W["R"]
    probe, _ = make_engine(pk, W, 1, form, cycles, seed, device, init=False)
    if form == "fp64":
        occ = probe.occupancy(N)
        probe.close()
        return max(1, occ) * n_sm, None, {"ctas_per_sm": occ}
    shapes = [(1, 32), (1, 16)] + ([(1, 8), (1, 4)] if W["ens"] == "nvt" and N <= 64 else [])
    trials = {}
    for C, L in shapes:
        if (R // C) % (32 // L):
            continue
        occ = probe.occupancy(N, C, L)
        if occ < 1:
            continue
        B = occ * n_sm // C
        eng, sizes = make_engine(pk, W, B, form, cycles, seed, device)
        eng.set_launch_shape(N, C, L)
        eng.cycles_nosample(4)
        eng.cycles_nosample(20)
        rate = B * R * N * 20 / (eng.stats()["last_cycles_ms"] / 1e3)
        eng.close()
        trials["%d,%d" % (C, L)] = dict(ctas_per_sm=occ, runs=B, trial_rate=rate)
    probe.close()
    best = max(trials, key=lambda k: trials[k]["trial_rate"])
    C, L = (int(v) for v in best.split(","))
    return trials[best]["runs"], (C, L), {"shape": best, "trials": trials}


def flush_l2(torch, dev):
    buf = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    buf.fill_(1.0)
    torch.cuda.synchronize(dev)


class ClockSampler:
    def __init__(self, out_path, device):
        self.out_path, self.device, self.proc = out_path, device, None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(self.out_path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device),
                                          "--query-gpu=" + q, "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        try:
            rows = [r.split(",") for r in open(self.out_path).read().strip().split("\n") if r]
        except Exception:
            return None
        sm = [float(r[1]) for r in rows if len(r) >= 9 and r[1].strip().replace(".", "").isdigit()]
        if not sm:
            return None
        mx = max(float(r[2]) for r in rows if len(r) >= 9)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows if len(r) >= 9 for k in range(4)
                          if r[5 + k].strip() == "Active"})
        loaded = [s for s in sm if s > 0.5 * mx] or sm
        return {"sm_mhz": statistics.median(loaded), "sm_max_mhz": mx, "reasons": reasons,
                "samples": len(sm)}


def time_steps(torch, eng, steps, cycles, dev, production=True):
    """K timed steps; L2 flushed between steps; device time from the engine's
    own CUDA events on its stream.  A production step samples every cycle
    (ptmc_run_cycles)."""
    ms = []
    for _ in range(steps):
        flush_l2(torch, dev)
        if production:
            eng.run_cycles(cycles)
        else:
            eng.cycles_nosample(cycles)
        ms.append(eng.stats()["last_cycles_ms"])
    return ms


def _accepted(eng, B):
    return sum(int(eng.states(r)["counts"][:, 0].sum()) for r in range(B))


def combine_ranks(torch, dev_s, moves, device, world):
    """Whole-job figures of a timed segment: under torchrun every rank runs its
    own batch (replicas only, weak scaling), the job takes as long as its
    slowest rank and makes the moves of all ranks."""
    if world <= 1:
        return dev_s, float(moves)
    t = torch.tensor([dev_s], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    m = torch.tensor([float(moves)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(m)
    return float(t.item()), float(m.item())


def run_workload(args, name, pk, torch, dev, rank, world, peaks, steps, warmup, e2e_on):
    """One workload: the chosen form (and the plain FP64 form unless
    --only-chosen) timed on the production path; returns its record."""
    W = workload(name)
    if args.atoms > 0 and name == "batched":
        W["sizes"] = lambda B, n=args.atoms: [n] * B
    n_sm = torch.cuda.get_device_properties(dev).multi_processor_count
    B = args.runs or default_runs(name, n_sm)
    cycles = args.cycles or W["cycles"]
    pcycles = max(1, args.plain_cycles or W["plain_cycles"])
    seed = 1234 + 7919 * rank
    res = {}

    def timed(eng, form, sizes, cyc, k_steps, nruns=B):
        """k_steps timed production steps of `eng` (barrier + synchronize on both sides)."""
        st0 = eng.stats()
        acc0 = _accepted(eng, nruns)
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        clk = ClockSampler(os.path.join(args.outdir, "clocks_%s_%s_r%d.csv" % (name, form, rank)),
                           args.local_rank)
        with clk:
            ms = time_steps(torch, eng, k_steps, cyc, dev)
        torch.cuda.synchronize(dev)
        wall = time.perf_counter() - t0
        st1 = eng.stats()
        moves = sum(sizes) * W["R"] * cyc * k_steps
        dev_s, moves_all = combine_ranks(torch, sum(ms) / 1e3, moves, dev, world)
        acc = _accepted(eng, nruns)
        return dict(value=moves_all / dev_s, runs=nruns, ms_per_step=1e3 * dev_s / k_steps, wall=wall,
                    steps=k_steps, cycles_per_step=cyc,
                    launches=st1["kernel_launches"] - st0["kernel_launches"],
                    drift=st1["max_drift"], clocks=clk.summary(), moves=moves, sizes=sizes,
                    acceptance=(acc - acc0) / moves)

    if W.get("da"):
        # delayed acceptance: one FP32 chain is warmed up, its surrogate trained
        # on the chain's own records and the screening strength per temperature
        # slot calibrated (all untimed); then every timed form starts from that
        # chain's saved states (configurations and step sizes) on a fresh engine
        # with the same equilibration: the exact FP32 form, the chosen form (the
        # standard two-stage test, kappa = 1 on every slot: on this workload it
        # accepts more moves per second than the calibrated per-slot choice,
        # which is timed and reported beside it), and the plain FP64 form
        eng, sizes = make_engine(pk, W, B, "fp32", cycles, seed, args.local_rank,
                                 eq_cycles=2 * warmup * cycles)
        eng.cycles_nosample(cycles)
        da = train_surrogate(pk, eng, sizes, W["R"], records=args.da_records)
        trained = eng.surrogate_state()[:2]
        eng.equilibrate()
        # per-slot strengths (kappa = 0 where the model says screening does not
        # pay, from the records and a measured stage-1 cost)
        kap = eng.surrogate_calibrate(0.0, timing_cycles=cycles)
        da["kappa"] = dict(mean=float(np.mean(kap)), screened_slots=int(np.sum(kap > 0)),
                           per_slot=[round(float(k), 4) for k in kap])
        starts = [eng.states(r) for r in range(B)]
        eng.close()

        def segment(form, kappa):
            """A fresh engine from the saved states, equilibrated, then timed;
            kappa None: the exact form (no surrogate)."""
            e, _ = make_engine(pk, W, B, "fp32", cycles, seed + 2, args.local_rank,
                               starts=starts, eq_cycles=2 * warmup * cycles)
            if kappa is not None:
                e.surrogate_set(trained[1], capacity=1, params=trained[0])
                e.surrogate_set_kappa(kappa)
                e.surrogate_enable(True)
            e.equilibrate()
            s0 = e.surrogate_state()[2] if kappa is not None else None
            r = timed(e, form, sizes, cycles, steps)
            st = dict(attempted_per_s=r["value"], acceptance=r["acceptance"],
                      accepted_per_s=r["acceptance"] * r["value"])
            if kappa is not None:
                s1 = e.surrogate_state()[2]
                mv = r["moves"]
                st.update(stage1_reject_frac=(s1["stage1_rejects"] - s0["stage1_rejects"]) / mv,
                          exact_eval_frac=(s1["exact_evals"] - s0["exact_evals"]) / mv)
                if "fp32" in res:
                    # time per attempted move under screening = (r + p1) x the
                    # exact time per move, p1 = fraction evaluated exactly: r is
                    # the stage-1 cost as a fraction of an exact move; with stage
                    # 1 free (r = 0) accepted moves per second could rise at most
                    # (a / a0) / p1
                    ex, p1 = res["fp32"], st["exact_eval_frac"]
                    st.update(stage1_cost_frac=ex["value"] / r["value"] - p1,
                              accepted_gain=st["accepted_per_s"] / (ex["acceptance"] * ex["value"]),
                              accepted_gain_bound_free_stage1=((st["acceptance"] / ex["acceptance"]) / p1
                                                               if p1 > 0 else None))
            e.close()
            return r, st

        if not args.only_chosen:
            res["fp32"], st = segment("fp32", None)
            da.update(acceptance_exact=st["acceptance"], accepted_per_s_exact=st["accepted_per_s"])
        res["fp32_da"], da["kappa_1"] = segment("fp32_da", np.ones(W["R"]))
        if not args.only_chosen:
            _, da["calibrated"] = segment("fp32_da_calibrated", kap)
        res["fp32_da"]["da"] = da
        if not args.only_chosen:
            eng, _ = make_engine(pk, W, B, "fp64", pcycles, seed + 1, args.local_rank,
                                 starts=starts, eq_cycles=2 * 3 * pcycles)
            eng.equilibrate()
            res["fp64"] = timed(eng, "fp64", sizes, pcycles, 3)
            eng.close()
    else:
        forms = ["fp32"] if args.only_chosen else ["fp64", "fp32"]
        uniform = name != "batched" and not args.runs
        for form in forms:
            cyc = cycles if form == "fp32" else pcycles
            k_steps = steps if form == "fp32" else 3
            k_warm = warmup if form == "fp32" else 3
            Bf, shape, fill = B, None, None
            if args.shape and form == "fp32":
                shape = tuple(int(v) for v in args.shape.split(","))
            elif uniform:  # the batch that fills the GPU in whole waves (untimed set-up)
                t0 = time.perf_counter()
                Bf, shape, fill = fill_batch(pk, W, form, n_sm, cyc, seed, args.local_rank)
                fill["fill_s"] = round(time.perf_counter() - t0, 3)
            eng, sizes = make_engine(pk, W, Bf, form, cyc, seed, args.local_rank,
                                     eq_cycles=2 * k_warm * cyc)
            shapes = None
            t0 = time.perf_counter()
            if shape is not None:
                eng.set_launch_shape(sizes[0], *shape)
                shapes = {sizes[0]: shape}
            elif form == "fp32" and not args.no_tune:
                # launch shape per atom count, untimed set-up; the autotuner
                # restores the chain after its trials
                shapes = eng.autotune(trial_cycles=max(2, min(20, cyc // 4)),
                                      cache=os.path.join(args.outdir, "autotune_r%d.json" % rank))
            tune_s = time.perf_counter() - t0
            eng.equilibrate()           # the warm-up: k_warm steps' worth of cycles
            res[form] = timed(eng, form, sizes, cyc, k_steps, Bf)
            res[form]["fill"] = fill
            if shapes is not None:
                res[form]["launch_shapes"] = {
                    "ctas_per_run": {str(k): v[0] for k, v in sorted(shapes.items())},
                    "lanes_per_walker": {str(k): v[1] for k, v in sorted(shapes.items())},
                    "autotune_s": round(tune_s, 3)}
            eng.close()
    chosen = "fp32_da" if "fp32_da" in res else "fp32"
    ch = res[chosen]
    sizes = ch["sizes"]
    if W.get("flops_move"):
        # moves evaluated exactly (delayed acceptance: the stage-1 survivors)
        exact = (ch.get("da") or {}).get("kappa_1", {}).get("exact_eval_frac", 1.0)
        flops_launch = W["flops_move"] * exact * sum(sizes) * W["R"] * ch["cycles_per_step"]
    else:
        flops_launch = sum((W["flops_pair"] * (n - 1) + 2 * n) * n * W["R"]
                           for n in sizes) * ch["cycles_per_step"]
    # the cycle kernels are ~all of a step's device time
    achieved = flops_launch / (ch["ms_per_step"] / 1e3) / 1e12
    prof = PROFILED.get(name)
    fresh = prof is not None and prof["src_sha"] == kernel_sha(prof["src"])
    roof = {"bound": "fp32_fma", "achieved": achieved, "peak": peaks["fp32_tflops"],
            "unit": "TFLOP/s", "frac": achieved / peaks["fp32_tflops"],
            "traffic": prof["dram_bytes_per_run"] * ch["runs"] if fresh else None,
            "peak_source": "measured in-situ by ptmc_measure_peaks (FFMA chains)",
            "ops_per_pair": W["flops_pair"], "mufu_per_pair": W["mufu_pair"],
            "fp64_peak_tflops": peaks["fp64_tflops"], "mufu_peak_tops": peaks["mufu_tops"],
            "issue": issue_roof(prof if fresh else None, ch, n_sm)}
    if prof is not None and not fresh:
        roof["counters_note"] = ("ncu counters predate kernel source %s; not reported"
                                 % kernel_sha(prof["src"]))
    rec = {"workload": W["name"], "value": ch["value"], "unit": "atom-moves/s",
           "ms_per_step": ch["ms_per_step"], "steps": ch["steps"],
           "cycles_per_step": ch["cycles_per_step"], "runs": ch["runs"], "replicas": W["R"],
           "atoms": sorted(set(sizes)), "path": "production (ptmc_run_cycles: E, E^2, histograms)",
           "form": "fp32resync_batched" + ("_da" if chosen == "fp32_da" else ""),
           "launch_shapes": ch.get("launch_shapes"), "batch_fill": ch.get("fill"),
           "acceptance": ch["acceptance"],
           # largest |E_running - E_fp64| at a resync so far (null: no resync yet)
           "fp32_max_drift_eh": ch["drift"] if ch["drift"] > 0 else None,
           "gpu_launches": ch["launches"],
           "clocks": ch["clocks"], "roofline": roof,
           "plain_fp64": ({"value": res["fp64"]["value"], "ms_per_step": res["fp64"]["ms_per_step"],
                           "cycles_per_step": res["fp64"]["cycles_per_step"],
                           "runs": res["fp64"]["runs"],
                           "chosen_over_plain": ch["value"] / res["fp64"]["value"]}
                          if "fp64" in res else None),
           "fp32_exact": ({"value": res["fp32"]["value"], "ms_per_step": res["fp32"]["ms_per_step"]}
                          if chosen != "fp32" and "fp32" in res else None),
           "delayed_acceptance": ch.get("da")}
    # e2e through the public API with host buffers, one engine per step
    if e2e_on and rank == 0:
        # per step: a context from host arrays (start configurations; with delayed
        # acceptance also the trained surrogate's parameters), equilibration
        # cycles, the step's production cycles, every run's energies read back
        ts = []
        h2d = d2h = 0
        Be = ch["runs"]
        host_xyz = start_configs(W, Be)   # the step's inputs, made before the clock
        lshape = ch.get("launch_shapes") or {}
        for k in range(warmup + steps):
            torch.cuda.synchronize(dev)
            t0 = time.perf_counter()
            eng, sizes = make_engine(pk, W, Be, "fp32", cycles, 99 + k, args.local_rank,
                                     xyz=host_xyz, eq_cycles=2)
            for n, c_ in (lshape.get("ctas_per_run") or {}).items():  # the tuned launch shapes
                eng.set_launch_shape(int(n), c_, lshape["lanes_per_walker"][n])
            h2d = sum(n * 3 * 8 for n in sizes)  # start configurations (one per run)
            if W.get("da"):
                P, sur = trained
                eng.surrogate_set(sur, capacity=1, params=P)   # kappa = 1 on every slot
                eng.surrogate_enable(True)
                h2d += P.nbytes
            eng.equilibrate()
            eng.run_cycles(cycles)
            outs = [eng.energies()]  # every run's slot-ordered energies, one read
            eng.close()
            t1 = time.perf_counter()
            if k >= warmup:
                ts.append(t1 - t0)
            d2h = sum(o.nbytes for o in outs)
        rec["e2e"] = dict(value=sum(sizes) * W["R"] * cycles / statistics.mean(ts),
                          unit="atom-moves/s", h2d_bytes_per_step=h2d, d2h_bytes_per_step=d2h)
    return rec


def gpu_arm(args, rank, world, names):
    import torch
    import __graft_entry__ as g
    pk = g.load_package()
    dev = torch.device("cuda", args.local_rank)
    torch.cuda.set_device(dev)
    L = pk._capi.load()
    # measured in-situ peaks (FMA/MUFU-bound kernels)
    f32, f64, mufu = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    pk._capi.check(L.ptmc_measure_peaks(args.local_rank, ctypes.byref(f32), ctypes.byref(f64),
                                        ctypes.byref(mufu)))
    peaks = dict(fp32_tflops=f32.value, fp64_tflops=f64.value, mufu_tops=mufu.value)
    recs = {}
    for name in names:
        head = name == names[0]
        steps = args.steps if head else max(3, args.steps // 4)
        warmup = args.warmup if head else 3
        recs[name] = run_workload(args, name, pk, torch, dev, rank, world, peaks, steps, warmup,
                                  e2e_on=head and not args.no_e2e)
    return recs, peaks


# --------------------------------------------------------------- CPU oracle arm
def _cpu_worker(args_tuple):
    wname, seed, budget_s, k = args_tuple
    from oracle import oracle as orc
    W = workload(wname)
    n = W["sizes"](k + 1)[k]
    x = W["start"](n, k)
    R = W["R"]
    T, _ = orc.tempgrid(W["T"][0], W["T"][1], R)
    ens = orc.NPT if W["ens"] == "npt" else orc.NVT
    bcp = W["bc"][1] if W["bc"][1] else 0.9 * n ** (1 / 3) * 3 + 3.0
    run = orc.Run(n, R, np.stack([x] * R), T, ensemble=ens, pressure=P_NE,
                  bc=orc.BC_CUBIC if W["bc"][0] == "cubic" else orc.BC_SPHERE, bc_param=bcp,
                  exch_prob=1.0, seed=seed)
    if W["pot"] == "eam":
        E = CU_EAM
        ean = E["eps"] * E["a"] ** E["n"] / 2
        ecam = E["eps"] * E["C"] * E["a"] ** (E["m"] / 2)
        run.set_eam(E["n"], E["m"], ean, ecam)
    elif W["pot"] == "nn":
        import __graft_entry__ as g
        pot = nn_potential(g.load_package())
        run.set_nn(pot.sf, pot.weights, pot.nodes, pot.boundary)
    else:
        run.set_elj(C_NE, True)
    run.init()
    cyc, t0 = 0, time.perf_counter()
    while time.perf_counter() - t0 < budget_s:
        run.cycles(cyc + 1, 1)
        cyc += 1
    dt = time.perf_counter() - t0
    return n * R * cyc, dt, cyc


def cpu_baseline(wname, cores, budget_s):
    from oracle import oracle as orc
    orc.build()
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores) as pool:
        out = pool.map(_cpu_worker, [(wname, 1000 + k, budget_s, k) for k in range(cores)])
    moves = sum(o[0] for o in out)
    dt = max(o[1] for o in out)
    cyc = sum(o[2] for o in out)
    return moves / dt, cyc


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="all", choices=["all"] + ALL,
                    help="all: every workload, the headline (cu55) first")
    ap.add_argument("--runs", type=int, default=0, help="independent PT runs batched (0 = fill the GPU)")
    ap.add_argument("--cycles", type=int, default=0,
                    help="chosen-form MC cycles per step (0: the workload's, 200; NN: 20)")
    ap.add_argument("--plain-cycles", type=int, default=0,
                    help="plain FP64 form MC cycles per step (0: the workload's)")
    ap.add_argument("--da-records", type=int, default=100000,
                    help="delayed acceptance: (configuration, dE) records the surrogate trains on")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--outdir", default=os.path.join(tempfile.gettempdir(), "ptmc_bench"),
                    help="clock samples and the autotuner cache")
    ap.add_argument("--only-chosen", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-tune", action="store_true", help="keep one CTA per run (no autotuning)")
    ap.add_argument("--shape", default="",
                    help="C,L: force the FP32 launch shape (CTAs per run, lanes per walker); "
                         "with --runs, no batch sizing or autotuning (profiling one kernel)")
    ap.add_argument("--atoms", type=int, default=0,
                    help="batched workload: every run with this atom count (profiling one group)")
    args = ap.parse_args()
    os.makedirs(args.outdir, exist_ok=True)
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    args.local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    names = ALL if args.workload == "all" else [args.workload]
    head = names[0]
    W = workload(head)
    cores = os.cpu_count() or 1

    if args.impl == "reference":
        # the reference's CPU path on all host cores: the oracle port, a
        # restatement of the reference's hot path (no Julia here), on the
        # headline workload
        if rank != 0:
            return
        per_step = []
        for _ in range(args.warmup + args.steps):
            v, cyc = cpu_baseline(head, cores, max(2.0, args.cpu_seconds / 4))
            per_step.append(v)
        v = statistics.mean(per_step[args.warmup:])
        line = {"metric": METRIC,
                "value": v, "unit": "atom-moves/s", "n_gpus": args.gpus, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "impl": "reference",
                "config": {"workload": W["name"], "replicas": W["R"]},
                "cpu_baseline": {"value": v, "unit": "atom-moves/s", "cores": cores, "kind": "port",
                                 "sample": "each step: %d spawn workers x %.1f s of oracle cycles"
                                           % (cores, max(2.0, args.cpu_seconds / 4))},
                "e2e": {"value": v, "unit": "atom-moves/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    if world > 1:
        import torch
        torch.distributed.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    # CPU baseline first (spawned workers, before any GPU work in this process)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        v, cyc = cpu_baseline(head, cores, args.cpu_seconds)
        cpu = {"value": v, "unit": "atom-moves/s", "cores": cores, "kind": "port",
               "sample": "%d spawn workers, one %s PT run each (R=%d), %.0f s, %d cycles in total"
                         % (cores, W["name"], W["R"], args.cpu_seconds, cyc)}
    recs, peaks = gpu_arm(args, rank, world, names)
    if rank != 0:
        return
    h = recs[head]
    line = {
        "metric": METRIC,
        "value": h["value"], "unit": "atom-moves/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": h["ms_per_step"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+f64+bf16" if h["delayed_acceptance"] else "f32+f64", "data": "synthetic",
        "config": {"workload": h["workload"] + "_" + h["form"], "runs_per_gpu": h["runs"],
                   "replicas": h["replicas"], "atoms": h["atoms"],
                   "cycles_per_step": h["cycles_per_step"], "resync_every": W["resync"],
                   "exchange": "every cycle", "path": h["path"],
                   "launch_shapes": h["launch_shapes"],
                   "l2": "flushed between steps (256 MB write)"},
        "plain_fp64": h["plain_fp64"],
        "fp32_exact": h["fp32_exact"],
        "delayed_acceptance": h["delayed_acceptance"],
        "fp32_max_drift_eh": h["fp32_max_drift_eh"],
        "roofline": h["roofline"],
        "cpu_baseline": cpu,
        "e2e": h.get("e2e"),
        "gpu_launches": h["gpu_launches"],
        "clocks": h["clocks"],
        "workloads": {k: {kk: vv for kk, vv in r.items() if kk != "e2e"} for k, r in recs.items()},
    }
    print(json.dumps(line))


def issue_roof(prof, ch, n_sm):
    """The instruction-issue roofline of the cycle kernel: warp instructions
    per move (ncu, for the profiled launch shape) x moves/s against 4 issue
    slots per SM per clock at the SM clock sampled during the timed region."""
    if not prof or not ch.get("clocks"):
        return None
    shapes = (ch.get("launch_shapes") or {}).get("lanes_per_walker") or {}
    if any(v != prof["lanes"] for v in shapes.values()):
        return None  # measured for one launch shape only
    mhz = ch["clocks"]["sm_mhz"]
    ipm = prof["inst_per_move"]
    achieved = ch["value"] * ipm / 1e9
    peak = 4 * n_sm * mhz * 1e6 / 1e9
    return {"warp_inst_per_move": ipm, "achieved": achieved, "peak": peak, "unit": "G warp-inst/s",
            "frac": achieved / peak,
            "source": "ncu smsp__inst_executed, kernel source %s" % prof["src_sha"]}


if __name__ == "__main__":
    main()
