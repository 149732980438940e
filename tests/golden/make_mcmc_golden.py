"""Posterior summaries of the reference-likelihood MCMC on the 16-taxon DNA
workload, the fixture the GPU sampler is compared with.

    python tests/golden/make_mcmc_golden.py [REFERENCE_PF_DIR]

Runs the project's sampler (p4gpu.mcmc.Mcmc: p4's default proposal mixture,
eTBR included, p4's tuner) with the reference's own C likelihood core as its
evaluator (oracle.RefChainEvaluator: every proposed state pushed into a
reference tree and evaluated by p4_setPrams + p4_treeLogLike).  Two
independent runs of NGEN generations from the simulating tree, sampled every
SAMPLE_INTERVAL, the first BURN generations discarded.  Stored per run: the
mean, variance and ESS (p4's estimator) of lnL, tree length and gamma shape,
the split frequencies, and the proposal acceptance rates.
"""
import multiprocessing as mp
import os
import sys

import numpy

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "p4-phylogenetics_gb300"))
sys.path.insert(0, REPO)

WORKLOAD = "dna16"
NGEN = 120000
BURN = 20000
SAMPLE_INTERVAL = 10
SEEDS = (101, 202)
OUT = os.path.join(HERE, "mcmc", "dna16_reference.npz")


def run(seed):
    from oracle import oracle
    from p4gpu import mcmc, sim
    prob = sim.make_config(WORKLOAD)
    m = mcmc.Mcmc(prob, nChains=1, seed=seed, sampleInterval=SAMPLE_INTERVAL,
                  evaluator=oracle.RefChainEvaluator(prob))
    m.run(NGEN)
    keep = [i for i, g in enumerate(m.samples["gen"]) if g >= BURN]
    out = {}
    for k in ("lnL", "treeLength", "alpha"):
        v = numpy.asarray(m.samples[k], float)[keep]
        out[k] = (float(v.mean()), float(v.var()), float(mcmc.effective_sample_size(v)), len(v))
    freqs = mcmc.split_frequencies([m.samples["splits"][i] for i in keep])
    return seed, out, freqs, m.acceptance()


def main():
    from oracle import oracle
    refdir = sys.argv[1] if len(sys.argv) > 1 else os.environ.get(oracle.REF_ENV)
    if refdir:
        oracle.build(ref=True, refdir=refdir)
    if not oracle.have_ref():
        sys.exit("usage: make_mcmc_golden.py REFERENCE_PF_DIR (or set %s)" % oracle.REF_ENV)
    with mp.get_context("spawn").Pool(len(SEEDS)) as pool:
        res = pool.map(run, SEEDS)
    z = {"workload": WORKLOAD, "ngen": NGEN, "burn": BURN, "sampleInterval": SAMPLE_INTERVAL}
    for r, (seed, out, freqs, acc) in enumerate(res):
        z["run%d_seed" % r] = seed
        for k, (mean, var, ess, n) in out.items():
            z["run%d_%s" % (r, k)] = numpy.array([mean, var, ess, n])
        masks = sorted(freqs)
        z["run%d_split_masks" % r] = numpy.array(masks, numpy.int64)
        z["run%d_split_freqs" % r] = numpy.array([freqs[m] for m in masks])
        names = sorted(acc)
        z["run%d_acc_names" % r] = numpy.array(names)
        z["run%d_acc" % r] = numpy.array([acc[a] if acc[a] is not None else numpy.nan for a in names])
        print("run %d (seed %d): %s acceptance %s" % (r, seed, out, acc))
    numpy.savez_compressed(OUT, **z)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
