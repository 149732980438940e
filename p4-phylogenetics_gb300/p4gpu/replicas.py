"""Independent MCMC replicas, one per process and GPU: the multi-GPU form of
this path.  Runs share nothing while they sample (no collective on the data
path); at the end each rank's split sets and parameter traces are gathered to
rank 0, which compares the runs as p4 compares runs: the average standard
deviation of split frequencies (p4/func.py:3428-3468, generalised from two
runs to N: for every split supported at >= minimumProportion in some run, the
n-1 standard deviation of its frequency across the runs; the mean over
splits) and the per-run means and ESS of lnL, tree length and Gamma shape.

Launch: one process per GPU under torchrun (RANK/WORLD_SIZE from the
environment, MASTER_ADDR=127.0.0.1), process group "nccl" on GPUs or "gloo"
for host-only use.
"""
import math

import numpy

from . import mcmc


def asdsf_runs(splitSetsPerRun, minimumProportion=0.1):
    """ASDSF over N runs (N >= 2); equals mcmc.asdsf for two runs."""
    freqs = [mcmc.split_frequencies(s) for s in splitSetsPerRun]
    keys = set()
    for f in freqs:
        keys |= {k for k, v in f.items() if v >= minimumProportion}
    if not keys or len(freqs) < 2:
        return 0.0
    sds = []
    for k in keys:
        v = numpy.array([f.get(k, 0.0) for f in freqs])
        sds.append(math.sqrt(v.var(ddof=1)))
    return float(sum(sds) / len(sds))


def summary(samples):
    out = {}
    for q in ("lnL", "treeLength", "alpha"):
        v = numpy.asarray(samples[q], dtype=float)
        if len(v) > 10 and numpy.isfinite(v).all():
            out[q] = {"mean": float(v.mean()), "ess": float(mcmc.effective_sample_size(v))}
    return out


def run_replica(problem, nGens, seed, rank=None, **mcmcKw):
    """One run on this process; the seed is offset by the rank so that the
    replicas are independent."""
    import torch.distributed as dist
    if rank is None:
        rank = dist.get_rank() if dist.is_available() and dist.is_initialized() else 0
    m = mcmc.Mcmc(problem, seed=seed + 1000 * rank, **mcmcKw)
    m.run(nGens)
    return m


def gather_and_compare(samples, minimumProportion=0.1, group=None):
    """Gather every rank's samples to rank 0 and compare the runs; returns
    the comparison on rank 0 and None elsewhere."""
    import torch.distributed as dist
    payload = {"splits": [sorted(s) for s in samples["splits"]], "summary": summary(samples)}
    ws = dist.get_world_size(group)
    got = [None] * ws
    dist.all_gather_object(got, payload, group=group)
    if dist.get_rank(group) != 0:
        return None
    splitRuns = [[frozenset(s) for s in g["splits"]] for g in got]
    return {"runs": ws, "asdsf": asdsf_runs(splitRuns, minimumProportion),
            "summaries": [g["summary"] for g in got]}
