"""Benchmark: lnL evaluations/s of the p4 likelihood hot path on one GB300.

Workload (default): DNA 4-state, 64 taxa, 100,000 sites simulated under
GTR+G4 with 4 composition vectors on random node sets (seeded synthetic
data; no public dataset exists for this metric).  A step = one full lnL
evaluation: setPrams on the GPU (discrete-gamma rates, Q eigensystems,
every P deck in FP64) + fused FP32 pruning + FP64 log-sum.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

value : device throughput -- K steps, each at new branch lengths (as the
        MCMC's branch-length moves produce): parameter image copy, P decks
        for every node and category, fused pruning, result copy; CUDA events
        on the library stream, L2 flushed (256 MB write) between steps
        outside the timed events.  Eigensystems and gamma rates are cached
        by the library and recomputed only when their inputs change.
full_setprams : the same with comps, R and gamma shape also changing every
        step, so every eigensystem and gamma rate is recomputed (FP64).
e2e   : the same step through the public C ABI from host buffers:
        p4g_setBrLens (host branch lengths change every step, as an MCMC
        proposal does) + p4g_setPrams + p4g_treeLogLike, which returns lnL
        to the host; wall clock around K such calls.
batched_8_trees : 8 trees of the workload (the chains of an MCMCMC), each
        at new branch lengths every step, evaluated by p4g_batchLogLike in
        one captured CUDA graph per step; host wall clock.
mcmc  : MCMC throughput and ESS/s on the MCMC workloads (after the timed
        region; --no-mcmc skips it).
--impl reference : the reference algorithm's CPU implementation (the
        oracle's restatement of Pf/p4_node.c + Pf/p4_tree.c, FP64), pattern-
        parallel over all host cores, on the same workload.
Multi-GPU (torchrun): independent replicas, one per rank; value sums ranks
over the max-over-ranks time.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, "p4-phylogenetics_gb300"))
sys.path.insert(0, REPO)

import numpy  # noqa: E402

METRIC = ("lnL evals/sec (p4's allBrLens evaluation: new branch lengths, every P deck, "
          "pruning and log-sum per eval)")
DATA = "synthetic (seeded Yule tree + simulation under the workload's model; no public dataset)"
L2_NOTE = ("GPU arm: L2 flushed between timed steps (256 MB write); CPU arm: its working set "
           "(FP64 conditional likelihoods: 0.8 GB for the 64-taxon DNA workload, 0.5 GB for the 48-taxon "
           "protein one) exceeds the host caches")
WORKLOAD = "dna64het"
FP32_PEAK_TFLOPS = 152 * 128 * 2 * 2.07e9 / 1e12   # nominal FP32 FMA peak at max SM clock


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default=WORKLOAD)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-mcmc", action="store_true", help="skip the MCMC throughput section")
    ap.add_argument("--no-next", action="store_true",
                    help="skip the ancestral draws / Newton / simulation section")
    ap.add_argument("--clade-size", type=int, default=-1,
                    help="pin the clade-table size in leaves (0: off) instead of the first evaluation's timing")
    ap.add_argument("--shape", type=int, default=-1,
                    help="pin the pruning tile shape of the first (dim, nCat) group after the autotuner")
    ap.add_argument("--batch-shape", type=int, default=-1,
                    help="pin the 8-tree batch's tile shape instead of timing the shapes on the batch")
    ap.add_argument("--programmatic-launch", type=int, default=1, choices=[0, 1],
                    help="launch P decks and pruning with programmatic dependent launch (1, default) or plain stream order (0)")
    return ap.parse_args()


def ess_block(s, seconds):
    from p4gpu import mcmc
    out = {}
    for k in ("lnL", "treeLength", "alpha"):
        v = numpy.asarray(s[k], dtype=float)
        if len(v) > 10 and numpy.isfinite(v).all():
            ess = mcmc.effective_sample_size(v)
            out["ess_" + k] = ess
            out["ess_per_s_" + k] = ess / seconds
    return out


def run_until_ess(m, minEss=100, chunk=2000, budget=60.0, maxGens=400000):
    """Run m in chunks until every reported ESS (lnL, tree length, gamma shape)
    reaches minEss, or the time budget or generation cap is spent; returns
    (generations, seconds) of the measured run."""
    import torch
    gens, t0 = 0, time.perf_counter()
    while True:
        m.run(chunk)
        gens += chunk
        torch.cuda.synchronize()
        el = time.perf_counter() - t0
        e = ess_block(m.samples, el)
        if all(e.get("ess_" + k, 0.0) >= minEss for k in ("lnL", "treeLength", "alpha")):
            break
        if el >= budget or gens >= maxGens:
            break
    return gens, time.perf_counter() - t0


def _cpu_chain_worker(config, nChains, gens, seed, cpu, queue):
    """One process of the MCMC CPU baseline: the same sampler on the
    reference's own C core, pinned to one core."""
    try:
        if cpu is not None and hasattr(os, "sched_setaffinity"):
            os.sched_setaffinity(0, {cpu})
        from oracle import oracle
        from p4gpu import mcmc, sim
        prob = sim.make_config(config)
        m = mcmc.Mcmc(prob, nChains=nChains, chainTemp=0.1, seed=seed, sampleInterval=0,
                      evaluator=oracle.RefChainEvaluator)
        m.run(max(1, min(20, gens // 5)))    # warm-up: allocation, first full evaluations
        t0 = time.perf_counter()
        m.run(gens)
        queue.put(("ok", gens, time.perf_counter() - t0))
    except Exception as ex:
        queue.put(("error", repr(ex), 0.0))


def cpu_chains(config, nChains, gens, nProcs):
    """nProcs independent reference-likelihood runs side by side (spawned,
    pinned one per core): (generations per second of one run, aggregate)."""
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    cpus = sorted(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else [None]
    ps = [ctx.Process(target=_cpu_chain_worker, args=(config, nChains, gens, 7 + i, cpus[i % len(cpus)], q))
          for i in range(nProcs)]
    for pr in ps:
        pr.start()
    res = [q.get(timeout=1800) for _ in ps]
    for pr in ps:
        pr.join(timeout=30)
    bad = [r for r in res if r[0] != "ok"]
    if bad:
        raise RuntimeError("MCMC CPU baseline: %s" % bad[0][1])
    worst = max(r[2] for r in res)
    return gens / statistics.median(r[2] for r in res), nProcs * gens / worst


def cpu_mcmcmc_parallel(config, nChains, seconds):
    """One Metropolis-coupled run on the reference core with its chains'
    evaluations spread over nChains processes (one per core): generations
    per second over a bounded sample of about `seconds`."""
    from oracle import oracle
    from p4gpu import mcmc, sim
    prob = sim.make_config(config)
    ev = oracle.ParallelRefEvaluator(prob, nChains)
    try:
        m = mcmc.Mcmc(prob, nChains=nChains, chainTemp=0.1, seed=2, sampleInterval=0, evaluator=ev)
        m.run(3)
        gens, t0 = 0, time.perf_counter()
        while time.perf_counter() - t0 < seconds:
            m.run(2)
            gens += 2
        return gens, time.perf_counter() - t0
    finally:
        ev.close()


def mcmc_section(cpu=True):
    """MCMC throughput and ESS/s on the MCMC workloads (run after the timed
    region), each run long enough that every reported ESS reaches 100 (or a
    time budget ends it), with the same sampler on the reference's own C core
    as the CPU baseline:
      - 16-taxon DNA, single chain, p4's default proposals (eTBR included);
      - 8 chains (heat 0.1 steps) x 12 partitions on 32 taxa: the chains
        evaluated in one captured CUDA graph per generation, and one library
        call per chain (p4's chain loop);
      - the learned proposal over three seeds.
    CPU ESS/s = the GPU run's ESS per generation x the CPU's generations per
    second (same sampler, same target distribution)."""
    import torch
    from p4gpu import mcmc, pf, sim
    from p4gpu.engine import Engine
    out = {}
    ncpu = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)
    prob = sim.make_config("dna16")
    e = Engine(prob)
    pf.setPrecision(e.cTree, 1)
    e.calcLogLike()
    t0 = time.perf_counter()
    for _ in range(20):
        lnl64 = e.calcLogLike()
    fp64_ms = (time.perf_counter() - t0) / 20 * 1e3
    e.free()
    m = mcmc.Mcmc(prob, nChains=1, seed=1, sampleInterval=10)
    m.run(2000)
    for k in m.samples:
        m.samples[k] = []
    m.run(0)                        # zero the proposal counts (p4's restart semantics)
    gens, dt = run_until_ess(m, budget=40.0, chunk=10000)
    d = {"workload": "DNA 16 taxa, 1,000 sites, GTR+G4, single chain, p4's default proposals (eTBR included), "
                     "sample every 10", "fp64_single_eval_ms": fp64_ms, "fp64_lnL": lnl64, "generations": gens,
         "seconds": dt, "gens_per_s": gens / dt, "acceptance": m.acceptance()}
    d.update(ess_block(m.samples, dt))
    if cpu:
        one, agg = cpu_chains("dna16", 1, 1500, 1)
        _, aggK = cpu_chains("dna16", 1, 1500, ncpu)
        d["cpu_baseline"] = {"kind": "reference", "gens_per_s": one, "cores": 1,
                             "gens_per_s_k_cores": aggK, "k": ncpu,
                             "ess_per_s": {k: d["ess_" + k] / gens * one for k in ("lnL", "treeLength", "alpha")
                                           if "ess_" + k in d},
                             "sample": "1,500 generations of the same sampler on the reference's own C core "
                                       "(Pf/*.c compiled on this host), p4 part-granular updates; k cores: k "
                                       "independent chains, aggregate; ESS/s = the GPU run's ESS per generation "
                                       "x these generations/s"}
    out["dna16_single_chain"] = d
    prob = sim.make_config("mcmcmc32")
    note = ("8 chains (temps 0,0.1,...,0.7) x 12 partitions (8 DNA + 4 protein, 200-30,000 sites) on 32 taxa; "
            "graph = every chain x part in one captured launch sequence per generation, sequential = one "
            "library call + host sync per chain (p4's loop)")
    out["mcmcmc32_note"] = note
    essPerGen = {}
    for ev in ("graph", "sequential"):
        m = mcmc.Mcmc(prob, nChains=8, chainTemp=0.1, seed=2, sampleInterval=10, evaluator=ev)
        m.run(200)
        for k in m.samples:
            m.samples[k] = []
        m.run(0)
        if ev == "graph":
            n, dt = run_until_ess(m, budget=75.0, chunk=2000)
        else:
            n, dt = 600, None
            t0 = time.perf_counter()
            m.run(n)
            torch.cuda.synchronize()
            dt = time.perf_counter() - t0
        d = {"generations": n, "seconds": dt, "gens_per_s": n / dt, "lnL_evals_per_s": 8 * n / dt,
             "swap_accepts": [int(x) for x in m.swapAccepts], "acceptance": m.acceptance()}
        if ev == "graph":
            d.update(ess_block(m.samples, dt))
            essPerGen = {k: d["ess_" + k] / n for k in ("lnL", "treeLength", "alpha") if "ess_" + k in d}
        else:
            d["ess_per_s_from_graph_ess_per_gen"] = {k: v * n / dt for k, v in essPerGen.items()}
        out["mcmcmc32_8chains_12parts_" + ev] = d
    if cpu:
        gk, dk = cpu_mcmcmc_parallel("mcmcmc32", 8, 15.0)
        one, _ = cpu_chains("mcmcmc32", 8, 3, 1)
        out["mcmcmc32_8chains_12parts_graph"]["cpu_baseline"] = {
            "kind": "reference", "gens_per_s": one, "cores": 1, "gens_per_s_8_cores": gk / dk, "k": 8,
            "ess_per_s": {k: v * one for k, v in essPerGen.items()},
            "ess_per_s_8_cores": {k: v * gk / dk for k, v in essPerGen.items()},
            "sample": "the same 8-chain sampler on the reference's own C core with p4's part-granular updates: "
                      "3 generations on 1 core, and %d generations with the 8 chains' evaluations on 8 "
                      "processes (one per core); ESS/s = the GPU graph run's ESS per generation x these "
                      "generations/s" % gk}
    out["dna32het6_learned"] = learned_seeds((5, 6, 7))
    return out


def learned_seeds(seeds):
    """The learned proposal's gain over several seeds: per seed the ratio of
    min-ESS/s (learned / plain chain from the same burned-in state), with the
    mean and spread."""
    runs = [learned_section(seed=s) for s in seeds]
    ratios = [r["min_ess_per_s_ratio"] for r in runs]
    return {"seeds": list(seeds), "runs": runs, "min_ess_per_s_ratio": ratios,
            "ratio_mean": statistics.mean(ratios), "ratio_min": min(ratios), "ratio_max": max(ratios),
            "asdsf_learned_vs_plain": [r["asdsf_learned_vs_plain"] for r in runs]}


def learned_section(nBurn=20000, nSample=20000, weight=0.5, seed=5):
    """The learned proposal on the 32-taxon, 50,000-site, 6-composition DNA
    workload: a plain chain burns in for nBurn generations while its states
    are recorded, the network is trained on them (GPU kernels) and kappa is
    tuned, everything is frozen; then the learned chain and a plain chain
    both start from the burned-in state and run nSample generations each."""
    import torch
    from p4gpu import mcmc, sim
    from p4gpu.learned import LearnedProposal
    prob = sim.make_config("dna32het6")
    m = mcmc.Mcmc(prob, nChains=1, seed=seed, sampleInterval=1)
    lp = LearnedProposal(m, hidden=128, seed=seed, blockSize=4)
    m.learned = lp
    t0 = time.perf_counter()
    for _ in range(nBurn):
        m.step()
        lp.record(m.coldChain().cur)
    t1 = time.perf_counter()
    losses = lp.fit(steps=2000, batch=256, lr=1e-3)
    t2 = time.perf_counter()
    kappa = lp.tune_kappa(m, gensPer=200)
    lp.freeze()
    start = m.coldChain().cur.copy()
    res = {"workload": "DNA 32 taxa, 50,000 sites, GTR+G4, 6 compositions; 3-layer MLP (128 hidden, BF16 "
                       "weights) trained on the first %d burn-in states" % nBurn, "seed": seed,
           "burn_seconds": t1 - t0, "train_seconds": t2 - t1, "train_steps": len(losses), "kappa": kappa,
           "learned_weight": weight}
    chains = {}
    for name in ("plain", "learned"):
        mm = mcmc.Mcmc(prob, nChains=1, seed=seed + 6, sampleInterval=1, startState=start.copy())
        if name == "learned":
            mm.learned = lp
            mm.prob.learned = weight
            mm._makeProposals()
        mm.run(200)
        for k in mm.samples:
            mm.samples[k] = []
        a0, p0 = lp.nAccepted, lp.nProposed
        t0 = time.perf_counter()
        mm.run(nSample)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        d = {"generations": nSample, "seconds": dt, "gens_per_s": nSample / dt}
        d.update(ess_block(mm.samples, dt))
        d["min_ess_per_s"] = min(d.get("ess_per_s_" + k, float("inf")) for k in ("lnL", "treeLength", "alpha"))
        if name == "learned":
            d["learned_acceptance"] = (lp.nAccepted - a0) / max(1, lp.nProposed - p0)
        res[name] = d
        chains[name] = mm.samples
    res["asdsf_learned_vs_plain"] = mcmc.asdsf(chains["plain"]["splits"], chains["learned"]["splits"])
    res["min_ess_per_s_ratio"] = res["learned"]["min_ess_per_s"] / max(res["plain"]["min_ess_per_s"], 1e-12)
    return res


def max_over_ranks(vals, ws, device):
    """Per-rank timings -> the slowest rank's (the replicas run side by side,
    so the job takes as long as its slowest replica)."""
    import torch
    t = torch.tensor(vals, dtype=torch.float64, device=device)
    if ws > 1:
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return t.tolist()


def replica_value(units_per_rank, ws, seconds):
    """Whole-job throughput: units every rank processed / the max-over-ranks time."""
    return ws * units_per_rank / seconds


def describe(problem, nPatterns=None):
    """The workload in words: states, taxa, sites (-> patterns), model, seed."""
    parts = problem.parts
    kind = "DNA 4-state" if all(sp.dim == 4 for sp in parts) else \
        ("protein 20-state" if all(sp.dim == 20 for sp in parts) else "DNA + protein")
    sites = sum(sp.nChar for sp in parts)
    comps = max(sp.comps.shape[0] for sp in parts)
    s = "%s, %d taxa, %d sites" % (kind, problem.nTax, sites)
    if nPatterns is not None:
        s += " -> %d patterns" % nPatterns
    s += ", %d part%s, +G%d, %d composition%s per part on random node sets (workload %s, seeded)" % (
        len(parts), "s" if len(parts) > 1 else "", parts[0].nCat, comps, "s" if comps > 1 else "", problem.name)
    return s


def workload_config(problem, nGpus=1):
    """The config dict both arms print: the workload, its pattern count (the
    oracle's compression, identical to the library's), the L2 policy."""
    from oracle import oracle
    nPat = 0
    for sp in problem.parts:
        nPat += oracle.make_patterns(oracle.encode_part(sp, problem.nTax))[0].shape[1]
    return {"workload": describe(problem, nPat), "l2": L2_NOTE,
            "parallelism": "replicas x %d" % nGpus if nGpus > 1 else "single GPU"}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    return int(os.environ.get("RANK", "0")), int(os.environ.get("LOCAL_RANK", "0")), ws


# ---------------------------------------------------------------- work model
def algorithmic_flops(problem):
    """FP32 flops of one fused pruning pass: per pattern, every internal child
    edge costs nCat*D*(2D-1) (a D x D matvec, first term a multiply), every
    further child factor nCat*D multiplies, the root nCat*D*2."""
    t = problem.tree
    total = 0
    for sp in problem.parts:
        D, C = sp.dim, sp.nCat
        per = 0
        for v in range(t.nNodes):
            if t.isLeaf[v] and v != t.root:
                continue
            kids = list(t.children(v))
            per += sum(C * D * (2 * D - 1) for k in kids if not t.isLeaf[k])
            per += (len(kids) - 1) * C * D
        per += 2 * C * D
        total += per * npat_of(sp)
    return total


_NPAT = {}


def npat_of(sp):
    return _NPAT[id(sp)]


def fused_bytes(problem):
    """HBM bytes the fused kernel must move per pass: one code byte per taxon
    per pattern, the FP64 pattern weight and the invariant mask."""
    return sum((problem.tree.nLeaves + 8 + 4) * npat_of(sp) for sp in problem.parts)


def algorithmic_bytes(problem):
    """Algorithmic bytes of one pruning pass of the per-node method: per
    pattern, every internal node's FP32 conditional likelihoods written once
    and read once more through its parent edge (plus a 4-byte scaler each),
    one code byte per leaf edge and the 4-byte pattern weight:
    P * [(N_int + E_int + 1) * (D*C*4 + 4) + E_leaf + 4]
    (8,500 B per pattern for 64 taxa, D = 4, C = 4)."""
    t = problem.tree
    nInt = sum(1 for v in range(t.nNodes) if not t.isLeaf[v] or v == t.root)
    eInt = sum(1 for v in range(t.nNodes) if not t.isLeaf[v] and v != t.root)
    eLeaf = sum(1 for v in range(t.nNodes) if t.isLeaf[v] and v != t.root)
    total = 0
    for sp in problem.parts:
        total += npat_of(sp) * ((nInt + eInt + 1) * (sp.dim * sp.nCat * 4 + 4) + eLeaf + 4)
    return total


# ---------------------------------------------------------------- clocks
class ClockSampler(object):
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.p = None
        self.lines = []

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                                       "--format=csv,noheader,nounits", "-lms", "100"],
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.p = None

    def _read(self):
        for line in self.p.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        sm, mx, reasons, power = [], None, set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
                power.append(float(f[3]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm),
                "power_w_max": max(power) if power else None}


# ---------------------------------------------------------------- CPU baseline
def share_problem(problem, share, nShares, spi):
    """The workload restricted to the sites whose pattern falls in one share
    (patterns k with k % nShares == share).  Compressed again, those sites give
    exactly that share of the patterns with their counts, so the shares'
    lnLs add up to the whole workload's."""
    from p4gpu import sim
    sp = problem.parts[0]
    sites = numpy.nonzero(spi % nShares == share)[0]
    seqs = [numpy.frombuffer(q.encode(), numpy.uint8)[sites].tobytes().decode() for q in sp.sequences]
    part = sim.PartSpec(sp.dataType, seqs, sp.comps, sp.rmats, sp.gammaShapes, sp.nCat, sp.compNums,
                        sp.rMatrixNums, sp.gdasrvNums, sp.pInvar, sp.relRate, sp.equates)
    return sim.Problem(problem.tree, [part], problem.name)


def brlen_sets(problem, seed, n=8):
    """The branch-length vectors the timed steps cycle through (both arms)."""
    rng = numpy.random.default_rng(seed)
    base = problem.tree.brLen.copy()
    return [numpy.ascontiguousarray(base * numpy.exp(rng.normal(0, 0.05, base.shape))) for _ in range(n)]


def _cpu_worker(config, share, nShares, cpu, nEvals, seconds, barrier, queue):
    """One process of the CPU arm: the reference core (or, where it is not
    built, the oracle's restatement) over one share of the patterns, pinned
    to one core; times p4's allBrLens evaluation (new branch lengths, every
    P deck, full pruning, log-sum)."""
    try:
        if cpu is not None and hasattr(os, "sched_setaffinity"):
            os.sched_setaffinity(0, {cpu})
        from oracle import oracle
        from p4gpu import sim
        problem = sim.make_config(config)
        sp = problem.parts[0]
        _, _, spi = oracle.make_patterns(oracle.encode_part(sp, problem.nTax))
        sub = share_problem(problem, share, nShares, spi)
        bls = brlen_sets(problem, 0)
        if oracle.have_ref():
            kind = "reference"
            r = oracle.RefTree(sub)
            r.logLike()                                  # setPrams: eigensystems, gamma rates
            def ev(i):
                return r.allBrLensLogLike(bls[i % len(bls)])
        else:
            kind = "port"
            def ev(i):
                return oracle.port_loglike64(sub, brLen=bls[i % len(bls)])[0]
        ev(0)                                            # warm-up
        barrier.wait()
        times, lnl = [], None
        t0 = time.perf_counter()
        i = 0
        while (nEvals and i < nEvals) or (not nEvals and time.perf_counter() - t0 < seconds):
            t1 = time.perf_counter()
            v = ev(i)
            times.append(time.perf_counter() - t1)
            if i % len(bls) == 0:
                lnl = v
            i += 1
        queue.put((share, kind, times, lnl, sub.parts[0].nChar))
    except Exception as ex:    # reported by the parent
        queue.put((share, "error", repr(ex), None, 0))
        try:
            barrier.abort()
        except Exception:
            pass


def run_cpu_arm(config, nShares, nProcs, nEvals=0, seconds=0.0, timeout=900):
    """Run shares 0..nProcs-1 of nShares in nProcs pinned processes (spawned,
    so no CUDA state is inherited); returns per-share (kind, eval times, lnL
    at the first branch-length set)."""
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    barrier = ctx.Barrier(nProcs)
    queue = ctx.Queue()
    cpus = sorted(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else [None] * nProcs
    procs = [ctx.Process(target=_cpu_worker,
                         args=(config, k, nShares, cpus[k % len(cpus)], nEvals, seconds, barrier, queue))
             for k in range(nProcs)]
    for pr in procs:
        pr.start()
    out = {}
    try:
        for _ in range(nProcs):
            share, kind, times, lnl, nSites = queue.get(timeout=timeout)
            if kind == "error":
                raise RuntimeError("CPU arm worker %d: %s" % (share, times))
            out[share] = (kind, times, lnl, nSites)
    finally:
        for pr in procs:
            pr.join(timeout=30)
            if pr.is_alive():
                pr.terminate()
    return out


def cpu_baseline(config, seconds):
    """The reference core on ONE core, on a bounded sample of the workload:
    share 0 of 8 of the patterns evaluated for `seconds`; the whole
    workload's rate is the share's rate / 8 (the shares are round-robin
    over the patterns, so each holds 1/8 of the work)."""
    res = run_cpu_arm(config, 8, 1, seconds=seconds)
    kind, times, _, nSites = res[0]
    per = statistics.median(times) * 8
    return {"value": 1.0 / per, "unit": "evals/s", "cores": 1, "kind": kind,
            "sample": "%d allBrLens evaluations (new branch lengths, every P deck, full pruning + log-sum) "
                      "of 1/8 of the patterns (%d sites) on 1 pinned core, median time x 8" % (len(times), nSites)}


def reference_arm(args):
    rank, _, ws = dist_env()
    if rank != 0:
        return
    from p4gpu import sim
    problem = sim.make_config(args.config)
    nProcs = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)
    # size the steps: one evaluation per step per process, about 1 s of work per step at most
    probe = run_cpu_arm(args.config, nProcs, nProcs, nEvals=2)
    one = max(statistics.median(t[1]) for t in probe.values())
    per_step = max(1, int(1.0 / max(one, 1e-6)))
    res = run_cpu_arm(args.config, nProcs, nProcs, nEvals=(args.warmup + args.steps) * per_step)
    kind = res[0][0]
    # step i of every process ran at the same time; the step takes as long as its slowest process
    steps = []
    for i in range(args.warmup, args.warmup + args.steps):
        steps.append(max(sum(res[k][1][i * per_step:(i + 1) * per_step]) for k in res) / per_step)
    ms = 1e3 * statistics.mean(steps)
    value = 1e3 / ms
    lnl = sum(res[k][2] for k in res)
    line = {"metric": METRIC, "value": value, "unit": "evals/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": DATA,
            "impl": "reference",
            "config": workload_config(problem, args.gpus),
            "cpu_baseline": {"value": value, "unit": "evals/s", "cores": nProcs, "kind": kind,
                             "sample": "%d steps of %d evaluation(s) each: p4's allBrLens evaluation "
                                       "(p4_calculateBigPDecks of every node + p4_treeLogLike) by the %s, "
                                       "the patterns split round-robin over %d processes pinned one per core; "
                                       "a step takes as long as its slowest process"
                                       % (args.steps, per_step,
                                          "reference's own C core (Pf/*.c compiled on this host)"
                                          if kind == "reference" else "oracle's FP64 restatement", nProcs)},
            "e2e": {"value": value, "unit": "evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "lnL": lnl}
    print(json.dumps(line))


# ---------------------------------------------------------------- our arm
def main():
    args = parse()
    if args.impl == "reference":
        reference_arm(args)
        return
    rank, local, ws = dist_env()
    import torch
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
        torch.cuda.set_device(local)
    else:
        torch.cuda.set_device(0)
    from p4gpu import pf, sim
    from p4gpu import _lib
    if not os.path.exists(_lib.LIB_PATH):
        import build as _b
        _b.build()
    pf._L().p4g_init(torch.cuda.current_device())
    pf.setProgrammaticLaunch(args.programmatic_launch)
    problem = sim.make_config(args.config)
    from p4gpu.engine import Engine
    eng = Engine(problem)
    for p, sp in enumerate(problem.parts):
        _NPAT[id(sp)] = eng.nPatterns(p)
    info = pf.treeInfo(eng.cTree)
    if args.clade_size >= 0:
        pf.setCladeSize(eng.cTree, args.clade_size)
    lnl0 = eng.calcLogLike()
    stream = torch.cuda.ExternalStream(pf.getStream())
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    def flush_l2():
        with torch.cuda.stream(stream):
            flush.zero_()

    bls = brlen_sets(problem, rank)
    # two model-value sets to alternate between for the full-recompute steps
    sp0 = problem.parts[0]
    alt = []
    for k in range(2):
        r2 = numpy.random.default_rng(100 + k)
        comps = [sim._fix(c * numpy.exp(r2.normal(0, 0.01, c.shape))) for c in sp0.comps]
        rv = sim.upper_of(sp0.rmats[0]) * numpy.exp(r2.normal(0, 0.01, sp0.dim * (sp0.dim - 1) // 2))
        alt.append((comps, rv / rv.sum(), sp0.gammaShapes[0] * (1.0 + 0.01 * (k + 1))))

    def set_model(k):
        comps, rv, a = alt[k % 2]
        for c, val in enumerate(comps):
            eng.setComp(0, c, val)
        eng.setRMatrix(0, 0, rv)
        eng.setGamma(0, 0, a)

    # warm-up (includes the tile-shape autotuner on the first evaluation)
    for i in range(max(3, args.warmup)):
        pf.setBrLens(eng.cTree, bls[i % 8])
        pf.treeLogLikeAsync(eng.cTree, 1)
        pf.treeLogLikeWait(eng.cTree)
    if args.shape >= 0:
        pf.setPruneShape(eng.cTree, 0, args.shape)
    shape, tile = pf.getPruneShape(eng.cTree, 0)
    clocks = ClockSampler(local)
    clocks.start()

    # ---- value: device-timed full steps, L2 flushed between steps
    def barrier():
        torch.cuda.synchronize()
        if ws > 1:
            torch.distributed.barrier()
    barrier()
    nfull = max(10, args.steps // 4)
    nEvents = max(args.steps, nfull)
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(nEvents)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(nEvents)]
    for i in range(args.steps):
        flush_l2()
        pf.setBrLens(eng.cTree, bls[i % 8])
        starts[i].record(stream)
        pf.treeLogLikeAsync(eng.cTree, 1)
        ends[i].record(stream)
    lnl_dev = pf.treeLogLikeWait(eng.cTree)
    barrier()
    step_ms = [s.elapsed_time(e) for s, e in zip(starts[:args.steps], ends[:args.steps])]
    ms = statistics.mean(step_ms)

    # ---- full setPrams: every eigensystem and gamma rate recomputed each step
    for i in range(nfull):
        flush_l2()
        set_model(i)
        pf.setBrLens(eng.cTree, bls[i % 8])
        starts[i].record(stream)
        pf.treeLogLikeAsync(eng.cTree, 1)
        ends[i].record(stream)
        pf.treeLogLikeWait(eng.cTree)   # the host values change each step
    torch.cuda.synchronize()
    full_ms = statistics.mean(s.elapsed_time(e) for s, e in zip(starts[:nfull], ends[:nfull]))
    set_model(0)
    for c, val in enumerate(sp0.comps):
        eng.setComp(0, c, val)
    eng.setRMatrix(0, 0, sim.upper_of(sp0.rmats[0]))
    eng.setGamma(0, 0, sp0.gammaShapes[0])

    # ---- dominant kernel alone (pruning + result copy), L2 flushed
    k_ms = []
    for i in range(args.steps):
        flush_l2()
        starts[i].record(stream)
        pf.treeLogLikeAsync(eng.cTree, 0)
        ends[i].record(stream)
    pf.treeLogLikeWait(eng.cTree)
    torch.cuda.synchronize()
    k_ms = [s.elapsed_time(e) for s, e in zip(starts[:args.steps], ends[:args.steps])]
    prune_ms = statistics.mean(k_ms)
    nClades = pf.treeInfo(eng.cTree).get("nClade", 0)   # before the batch below (batches use none)
    cl = 1 if nClades else 0

    # ---- the plain FP64 GPU path (per-node launches), same steps, L2 flushed
    pf.setPrecision(eng.cTree, 1)
    for _ in range(3):
        pf.treeLogLikeAsync(eng.cTree, 1)
        lnl64 = pf.treeLogLikeWait(eng.cTree)
    n64 = max(10, args.steps // 10)
    f64_ms = []
    for i in range(n64):
        flush_l2()
        pf.setBrLens(eng.cTree, bls[i % 8])
        starts[i].record(stream)
        pf.treeLogLikeAsync(eng.cTree, 1)
        ends[i].record(stream)
        pf.treeLogLikeWait(eng.cTree)
    torch.cuda.synchronize()
    f64_ms = statistics.mean(s.elapsed_time(e) for s, e in zip(starts[:n64], ends[:n64]))
    # both paths at one parameter point
    pf.setBrLens(eng.cTree, bls[0])
    pf.treeLogLikeAsync(eng.cTree, 1)
    lnl64 = pf.treeLogLikeWait(eng.cTree)
    pf.setPrecision(eng.cTree, 0)
    pf.treeLogLikeAsync(eng.cTree, 1)
    lnl32 = pf.treeLogLikeWait(eng.cTree)

    # ---- e2e: public C ABI from host buffers, branch lengths change each step
    barrier()
    t0 = time.perf_counter()
    for i in range(args.steps):
        pf.setBrLens(eng.cTree, bls[i % 8])
        pf.p4_setPrams(eng.cTree, -1)
        pf.p4_treeLogLike(eng.cTree, 0)
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0

    # ---- 8 trees per launch sequence (the chains of an MCMCMC, p4g_batchLogLike):
    # new branch lengths for every tree each step, lnL of all 8 back on the host
    nb = 8
    others = [Engine(problem, shared=(eng.cData, eng.cParts)) for _ in range(nb - 1)]
    trees = [eng] + others
    if args.batch_shape >= 0:   # the batch takes the first tree's shapes; no timing on the batch
        pf.setPruneShape(eng.cTree, 0, args.batch_shape)
        pf.setAutotune(False)
    batch = pf.Batch([x.cTree for x in trees], clades=True)   # fixed topology: clade tables pay
    for r in range(3):
        for i, x in enumerate(trees):
            pf.setBrLens(x.cTree, bls[(i + r) % 8])
        batch.logLike()
    pf.setAutotune(True)
    nbSteps = max(20, args.steps // 4)
    t0 = time.perf_counter()
    for r in range(nbSteps):
        for i, x in enumerate(trees):
            pf.setBrLens(x.cTree, bls[(i + r) % 8])
        lnlBatch = batch.logLike()
    batch_s = time.perf_counter() - t0
    batch.free()
    for x in others:
        x.free()
    ck = clocks.stop()
    # the roofline denominator: measured FP32 FMA throughput, with the SM clock sampled meanwhile
    pk = ClockSampler(local)
    pk.start()
    time.sleep(0.3)
    tf, tf_ms = pf.fp32FmaPeak(40000)
    pck = pk.stop()
    fp32_peak = {"tflops": tf, "ms": tf_ms, "sm_mhz": pck.get("sm_mhz")}

    # max over ranks
    ms, e2e_s, prune_ms = max_over_ranks([ms, e2e_s, prune_ms], ws, "cuda")
    if rank != 0:
        return
    value = replica_value(1.0, ws, ms * 1e-3)
    e2e = replica_value(args.steps, ws, e2e_s)
    flops = algorithmic_flops(problem)
    abytes = algorithmic_bytes(problem)
    fbytes = fused_bytes(problem)
    traffic = read_traffic(args.config)
    tflops = flops / (prune_ms * 1e-3) / 1e12
    kname = ("k_prune_tc" if (sp0.dim == 20 and shape == 3) else "k_prune")
    if kname == "k_prune":
        roof = {"bound": "fp32", "achieved": tflops,
                "peak": fp32_peak["tflops"], "unit": "TFLOP/s", "frac": tflops / fp32_peak["tflops"],
                "traffic": traffic,
                "peak_source": "measured FP32 FMA throughput on this GPU (p4g_fp32FmaPeak, CUDA events, SM clock "
                               "%s MHz sampled during the probe), frac of measured" % fp32_peak["sm_mhz"],
                "binding_resource": "FP32 issue and latency on the CUDA cores (ncu: issue active < 45 %, long-"
                                    "scoreboard stalls on the clade-table gathers, 14-15 warps per SM for one "
                                    "tree); the kernel keeps every conditional likelihood on chip, so HBM does "
                                    "not bind it"}
    else:   # split-TF32 tensor-core kernel: TF32 dense runs at half the measured bf16 rate
        tf32 = measured_peak("bf16_tflops", 1900.0) / 2.0
        roof = {"bound": "tensor", "achieved": tflops, "peak": tf32, "unit": "TFLOP/s", "frac": tflops / tf32,
                "traffic": traffic,
                "peak_source": "measured bf16 dense GEMM throughput (MEASURED_PEAKS bf16_tflops, burst) / 2 = "
                               "TF32 dense; flops counted once per split-TF32 product (the tensor pipe issues 3 "
                               "MMAs for each), frac of measured",
                "fp32_equivalent": {"peak": fp32_peak["tflops"], "frac": tflops / fp32_peak["tflops"],
                                    "note": "the same flops against the measured FP32 FMA throughput"},
                "binding_resource": "latency between the four warpgroups' MMA issue, commit wait and TMEM read-"
                                    "back (ncu: tensor pipe active ~3 %, issue active ~31 %, long-scoreboard and "
                                    "barrier stalls); the leaf gathers and products run on the CUDA cores"}
    roof.update({
            "kernel": "%s<D=%d,nCat=%d> fused pruning + root log-sum (tile shape %d: %d patterns "
                      "per block, %s), %s, incl. the 12 B result copy"
                      % (kname, sp0.dim, sp0.nCat, shape, tile, "pinned" if args.shape >= 0 else "autotuned",
                         "with the clade-table launch (%d clades)" % nClades if nClades else "no clade tables"),
            "kernel_ms": prune_ms, "flops_per_launch": flops,
            "flops_note": "algorithmic flops of the per-pattern method: per pattern every internal child "
                          "edge nCat*D*(2D-1), every further child factor nCat*D, the root 2*nCat*D (clade "
                          "tables skip part of this work, so the kernel executes fewer)",
            "nominal_peak_tflops": FP32_PEAK_TFLOPS,
            "bytes_avoided": {"per_node_method_bytes_per_launch": abytes,
                              "fused_min_bytes_per_launch": fbytes,
                              "note": "the per-node method's FP32 CL traffic P*[(N_int+E_int+1)*(D*C*4+4)+"
                                      "E_leaf+4], which the fused kernel never moves (its DRAM traffic, `traffic` "
                                      "from the committed ncu summary, is the tip codes, weights and clade-table "
                                      "entries); not an HBM fraction"},
            "hbm_of_measured": {"achieved_gbs": (traffic or fbytes) / (prune_ms * 1e-3) / 1e9,
                                "peak_gbs": measured_peak("hbm_gbs", 6684.5),
                                "frac": (traffic or fbytes) / (prune_ms * 1e-3) / 1e9
                                / measured_peak("hbm_gbs", 6684.5)}})
    line = {"metric": METRIC, "value": value, "unit": "evals/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 (pruning) / f64 (setPrams, log-sum)",
            "data": DATA,
            "config": workload_config(problem, ws),
            "e2e": {"value": e2e, "unit": "evals/s", "h2d_bytes_per_step": info["h2dBytes"],
                    "d2h_bytes_per_step": info["d2hBytes"],
                    "path": "p4g_setBrLens + p4g_setPrams + p4g_treeLogLike (host lnL each step); h2d = the "
                            "branch lengths, which the P-deck kernel reads from the pinned host image (the "
                            "parameter image is copied only when other values change)"},
            "gpu_launches": args.steps * (2 + 1 + 2 + 3 * cl) + nfull * (3 + cl)
            + n64 * (1 + problem.tree.nNodes - problem.tree.nLeaves + 1) + nbSteps * 3,
            "gpu_launches_note": "value step: k_pdeck + k_prune (+ the clade-table k_prune when clade tables "
                                 "are on); prune-only: k_prune (+ clade tables); e2e: k_pdeck + k_prune "
                                 "(+ clade tables); full step adds k_gammaEig; FP64 step: k_pdeck + one "
                                 "k_node64 per internal node + k_root64; batched step (graph): k_gammaEig + "
                                 "k_pdeck + k_prune",
            "full_setprams": {"value": 1e3 / full_ms, "unit": "evals/s", "ms_per_step": full_ms,
                              "note": "comps, R, gamma shape and branch lengths all change every step: every "
                                      "eigensystem (FP64 Jacobi) and gamma rate set is recomputed"},
            "programmatic_launch": bool(args.programmatic_launch),
            "roofline": roof, "fp32_peak_probe": fp32_peak, "clocks": ck, "lnL": lnl_dev, "lnL_first": lnl0,
            "plain_fp64_gpu": {"value": 1e3 / f64_ms, "unit": "evals/s", "ms_per_step": f64_ms,
                               "speedup_fp32_over_fp64": f64_ms / ms, "lnL": lnl64, "lnL_fp32_same_point": lnl32,
                               "rel_dlnL_fp32_vs_fp64": abs(lnl32 - lnl64) / abs(lnl64),
                               "path": "per-node FP64 kernels, reference loop structure, no scaling"},
            "batched_8_trees": {"value": nb * nbSteps / batch_s, "unit": "evals/s", "trees": nb,
                                "steps": nbSteps, "ms_per_step": 1e3 * batch_s / nbSteps,
                                "speedup_over_plain_fp64_gpu": (nb * nbSteps / batch_s) / (1e3 / f64_ms),
                                "path": "p4g_batchLogLike with clade tables: 8 trees (new branch lengths each) in one captured "
                                        "CUDA graph per step, lnL of all 8 to the host; host wall clock"}}
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(args.config, args.cpu_seconds)
    if not args.no_next and ws == 1:
        line["draws_and_ml"] = draws_and_ml_section(problem)
    if not args.no_mcmc and ws == 1:
        line["mcmc"] = mcmc_section(cpu=not args.no_cpu_baseline)
    print(json.dumps(line))


def draws_cpu_baseline(problem, seconds=3.0):
    """The oracle's restatements of the draws on the host (kind "port", one
    thread): the simulation (numpy, by sites) of the whole alignment, and the
    ancestral draw of a bounded sample of sites on the port's FP64 root CLs."""
    from oracle import oracle
    decks = [oracle.port_pdecks(problem, p) for p in range(len(problem.parts))]
    t0 = time.perf_counter()
    oracle.port_simulate(problem, 5, decks)
    sim_s = time.perf_counter() - t0
    sp = problem.parts[0]
    cl = oracle.port_root_cl(problem, 0)
    u = oracle.philox_uniforms(7, 0, sp.nChar)
    prep = oracle.draw_anc_prep(problem, 0)
    n = 0
    step = max(1, sp.nChar // 200)
    t0 = time.perf_counter()
    while time.perf_counter() - t0 < seconds and n < sp.nChar:
        oracle.port_draw_anc(problem, 0, cl, u, sites=range(n, min(sp.nChar, n + step)), prep=prep)
        n += step
    draw_rate = min(n, sp.nChar) / (time.perf_counter() - t0)
    states = sum(q.nChar for q in problem.parts) * problem.tree.nNodes
    return {"kind": "port", "cores": 1,
            "simulation_node_states_per_s": states / sim_s,
            "ancestral_draw_sites_per_s": draw_rate,
            "sample": "whole-alignment simulation (numpy, by sites); ancestral draws of %d sites "
                      "(Python loop over the sites on the port's FP64 root CLs)" % n}


def draws_and_ml_section(problem):
    """The consumers of the likelihood path on the same workload, on the GPU
    (host wall clock per call, median of 5 after one warm-up): ancestral-state
    draws of every site (p4_drawAncState), Newton optimisation of every branch
    length (one p4_newtAround(1e-5, 1e-7)), simulation of a new alignment
    (p4_simulate), in that order (the simulation replaces the data)."""
    from p4gpu import pf
    from p4gpu.engine import Engine
    eng = Engine(problem)
    lnl0 = eng.calcLogLike()
    sp = problem.parts[0]

    def med(f, n=5):
        f()
        ts = []
        for _ in range(n):
            t0 = time.perf_counter()
            f()
            ts.append(time.perf_counter() - t0)
        return statistics.median(ts)

    sites = sum(q.nChar for q in problem.parts)
    draw_s = med(lambda: pf.drawAncStates(eng.cTree, 0, sp.nChar, None, 7))
    cpu = draws_cpu_baseline(problem)
    t0 = time.perf_counter()
    pf.p4_newtAround(eng.cTree, 1.0e-5, 1.0e-7)
    newt_s = time.perf_counter() - t0
    lnl1 = eng.calcLogLike()

    def sim_and_compress():
        pf.simulate(eng.cTree, 5)
        for cp in eng.cParts:
            pf.makePatternsDevice(cp)
            pf.setGlobalInvarSitesVec(cp)
    sim_s = med(sim_and_compress)
    states = sites * problem.tree.nNodes
    eng.free()
    return {"cpu_baseline": cpu,
            "ancestral_draws": {"seconds": draw_s, "sites_per_s": sp.nChar / draw_s,
                                "path": "p4g_drawAncStates: setPrams + FP32 pruning with root partials + "
                                        "k_drawAnc, draws to the host"},
            "newton_branch_lengths": {"seconds": newt_s, "lnL_before": lnl0, "lnL_after": lnl1,
                                      "path": "p4g_newtAround(1e-5, 1e-7): FP64 cl/cl2 and Newton sums on "
                                              "the GPU, the reference's control flow on the host"},
            "simulation": {"seconds": sim_s, "node_states_per_s": states / sim_s,
                           "path": "p4g_simulate (setPrams, Philox stream, k_simRoot/k_simRank/k_simMutate, "
                                   "leaf states to the host) + makePatternsDevice + setGlobalInvarSitesVec "
                                   "per part: a new compressed alignment, ready to evaluate"}}


def measured_peak(key, default):
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)[key])
    except (OSError, KeyError, ValueError):
        return default


TRAFFIC_PROFILES = {"dna64het": "prune_dna4_dna64het.md", "prot48het": "prune_tc_prot20_prot48het.md"}


def read_traffic(workload):
    """DRAM bytes per launch of the workload's pruning kernel from its
    committed ncu summary (a line 'dram_bytes_per_launch: N'), or None."""
    if workload not in TRAFFIC_PROFILES:
        return None
    path = os.path.join(REPO, "profiles", TRAFFIC_PROFILES[workload])
    try:
        for ln in open(path):
            if ln.strip().startswith("dram_bytes_per_launch:"):
                return float(ln.split(":", 1)[1].split()[0])
    except OSError:
        pass
    return None


if __name__ == "__main__":
    main()
