"""The multi-GPU form of the path -- independent replicas, one per process --
on the CPU: two gloo ranks each run an MCMC (the oracle stands in for the GPU
library's lnL, test infrastructure only), then rank 0 gathers and compares the
runs; and the bench's max-over-ranks timing and whole-job throughput."""
import json
import os
import socket
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, ws, port, outPath):
    for p in (os.path.join(REPO, "p4-phylogenetics_gb300"), REPO, os.path.join(REPO, "tests")):
        sys.path.insert(0, p)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    from conftest import golden_files
    from oracle import oracle as port
    from p4gpu import replicas, sim
    from test_mcmc_gpu import problem_of_state
    import bench

    prob, _ = sim.load_problem(golden_files()[0])

    class PortEvaluator(object):
        def evaluate(self, states):
            return [port.port_loglike64(problem_of_state(prob, st))[0] for st in states]

    m = replicas.run_replica(prob, 200, seed=3, nChains=1, sampleInterval=2, evaluator=PortEvaluator())
    res = replicas.gather_and_compare(m.samples)
    t = bench.max_over_ranks([1.0 + rank, 5.0 - rank], ws, "cpu")
    if rank == 0:
        with open(outPath, "w") as f:
            json.dump({"res": res, "max": t, "lnL": [x for x in m.samples["lnL"]][:3]}, f)
    dist.destroy_process_group()


def test_two_replicas_gather_and_compare(tmp_path, lib):
    import torch.multiprocessing as mp
    out = str(tmp_path / "r.json")
    mp.spawn(_worker, args=(2, _port(), out), nprocs=2, join=True)
    d = json.load(open(out))
    assert d["max"] == [2.0, 5.0]
    res = d["res"]
    assert res["runs"] == 2 and len(res["summaries"]) == 2
    assert 0.0 <= res["asdsf"] < 1.0
    # different seeds per rank: the runs are not copies of each other
    assert res["summaries"][0]["lnL"]["mean"] != res["summaries"][1]["lnL"]["mean"]


def test_asdsf_runs_matches_two_run_formula():
    sys.path.insert(0, os.path.join(REPO, "p4-phylogenetics_gb300"))
    from p4gpu import mcmc, replicas
    a = [frozenset({1, 2}), frozenset({1, 4}), frozenset({1, 2})]
    b = [frozenset({1, 2}), frozenset({2, 4}), frozenset({1, 4})]
    assert abs(replicas.asdsf_runs([a, b]) - mcmc.asdsf(a, b)) < 1e-15
    assert replicas.asdsf_runs([a, a, a]) == 0.0


def test_replica_throughput_is_whole_job():
    sys.path.insert(0, REPO)
    import bench
    assert bench.replica_value(100, 4, 2.0) == 200.0
