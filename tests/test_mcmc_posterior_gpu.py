"""The GPU sampler targets p4's posterior: a chain evaluated on the GPU
(FP32 pruning, CUDA-graph batch evaluator) with p4's default proposal mixture
-- eTBR included -- against two chains of the same proposal code whose
likelihood is the reference's own C core (tests/golden/mcmc/dna16_reference.npz,
written by tests/golden/make_mcmc_golden.py).

The runs are independent (different seeds), so agreement is statistical:
  - posterior means of lnL, tree length and gamma shape agree within 4 Monte
    Carlo standard errors, se = sqrt(var_gpu/ESS_gpu + var_ref/ESS_ref) with
    p4's ESS estimator (the reference side pools its two runs);
  - split frequencies agree: ASDSF (p4/func.py:3428, splits >= 0.1) below 0.01
    against each reference run;
  - every proposal of the mixture, eTBR included, was tried and accepted.
"""
import math
import os

import numpy
import pytest

from conftest import GOLDEN
from p4gpu import mcmc, sim

pytestmark = pytest.mark.gpu

FIXTURE = os.path.join(GOLDEN, "mcmc", "dna16_reference.npz")
SEED = 303


def ref_run(z, r):
    freqs = dict(zip((int(m) for m in z["run%d_split_masks" % r]), z["run%d_split_freqs" % r]))
    stats = {k: z["run%d_%s" % (r, k)] for k in ("lnL", "treeLength", "alpha")}
    return stats, freqs


@pytest.fixture(scope="module")
def gpu_chain(lib):
    z = numpy.load(FIXTURE)
    prob = sim.make_config(str(z["workload"]))
    m = mcmc.Mcmc(prob, nChains=1, seed=SEED, sampleInterval=int(z["sampleInterval"]))
    m.run(int(z["ngen"]))
    keep = [i for i, g in enumerate(m.samples["gen"]) if g >= int(z["burn"])]
    return m, keep, z


def test_posterior_means_match_reference_chain(gpu_chain):
    m, keep, z = gpu_chain
    runs = [ref_run(z, r) for r in (0, 1)]
    for k in ("lnL", "treeLength", "alpha"):
        v = numpy.asarray(m.samples[k], float)[keep]
        ess = mcmc.effective_sample_size(v)
        assert ess > 20, (k, ess)          # a sanity floor; the comparison below uses the ESS
        se_gpu2 = v.var() / ess
        means = [s[k][0] for s, _ in runs]
        se_ref2 = sum(s[k][1] / s[k][2] for s, _ in runs) / 4.0      # mean of the two runs
        se = math.sqrt(se_gpu2 + se_ref2)
        assert abs(v.mean() - numpy.mean(means)) < 4.0 * se, (k, v.mean(), means, se)


def test_split_frequencies_match_reference_chain(gpu_chain):
    m, keep, z = gpu_chain
    f_gpu = mcmc.split_frequencies([m.samples["splits"][i] for i in keep])
    for r in (0, 1):
        _, f_ref = ref_run(z, r)
        d = mcmc.asdsf_of_frequencies(f_gpu, f_ref)
        assert d < 0.01, (r, d)


def test_every_default_proposal_moves(gpu_chain):
    m, _, _ = gpu_chain
    acc = m.acceptance()
    for name in ("local", "eTBR", "allBrLens", "allCompsDir.0", "allRMatricesDir.0", "gdasrv.0"):
        assert acc.get(name) is not None and acc[name] > 0.0, (name, acc)
    etbr = next(p for p in m.proposals if p.name == "eTBR")
    assert sum(etbr.nTopologyChanges) > 0
