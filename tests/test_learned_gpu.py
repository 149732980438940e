"""The learned-proposal network's GPU kernels against the FP64 CPU oracle,
and the learned proposal inside the MCMC."""
import numpy
import pytest

from conftest import golden_files
from p4gpu import mcmc, sim
from p4gpu.learned import LearnedProposal, Network

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mlp_ref():
    from oracle import mlp_ref
    return mlp_ref


@pytest.mark.parametrize("dIn,H,d,B,masked", [(7, 16, 5, 3, False), (80, 128, 80, 64, False),
                                              (33, 128, 20, 200, False), (66, 128, 33, 128, True)])
def test_forward_and_gradients_match_oracle(lib, mlp_ref, dIn, H, d, B, masked):
    net = Network(dIn, H, 2 * d, maxBatch=256, seed=3)
    rng = numpy.random.default_rng(dIn)
    p = net.params()
    # a trained-like state: perturb all weights so nothing is trivially zero
    p = (p + 0.05 * rng.standard_normal(p.shape)).astype(numpy.float32)
    net.set_params(p)
    x = rng.standard_normal((B, dIn)).astype(numpy.float32)
    t = rng.standard_normal((B, d)).astype(numpy.float32)
    if masked:   # NaN targets are left out of the loss (block-conditional training)
        t[rng.random((B, d)) < 0.7] = numpy.nan
    y = net.forward(x)
    yr, _ = mlp_ref.forward(p, x, dIn, H, 2 * d)
    numpy.testing.assert_allclose(y, yr, rtol=0, atol=2e-5 * (1 + numpy.abs(yr).max()))
    loss, g = net.gradients(x, t)
    lr, gr = mlp_ref.loss_and_grads(p, x, t, dIn, H, 2 * d)
    assert abs(loss - lr) <= 1e-4 * (1 + abs(lr))
    scale = numpy.abs(gr).max()
    numpy.testing.assert_allclose(g, gr, rtol=0, atol=1e-4 * scale)
    net.free()


def test_training_reduces_loss(lib):
    rng = numpy.random.default_rng(0)
    d = 6
    net = Network(d, 32, 2 * d, maxBatch=512, seed=1)
    A = rng.standard_normal((d, d)) * 0.3
    X = rng.standard_normal((4000, d))
    T = X @ A.T + 0.2 * rng.standard_normal((4000, d))    # displacement depends on x
    losses = [net.train_step(X[i:i + 256], T[i:i + 256], 3e-3) for i in range(0, 3744, 16)]
    assert numpy.mean(losses[-10:]) < numpy.mean(losses[:10]) - 0.5
    net.free()


def test_learned_move_is_exact_bookkeeping(lib, port):
    """Ratios of the learned move: reverse(forward(x)) returns to x, and the
    recorded lnL of the chain stays the exact lnL of its state."""
    prob, _ = sim.load_problem(golden_files()[0])
    m = mcmc.Mcmc(prob, nChains=1, seed=9, sampleInterval=0)
    lp = LearnedProposal(m, hidden=32, seed=2)
    m.learned = lp
    for _ in range(400):
        m.step()
        lp.record(m.coldChain().cur)
    lp.fit(steps=200, batch=128)
    lp.freeze(kappa=0.5)
    m.prob.learned = 1.0
    m._makeProposals()
    m.run(200)
    assert lp.nProposed > 10
    st = m.coldChain().cur
    x = lp.to_x(st)
    st2 = st.copy()
    assert lp.from_x(x, st2)
    numpy.testing.assert_allclose(lp.to_x(st2), x, rtol=0, atol=1e-9)
    from test_mcmc_gpu import problem_of_state
    ref, _ = port.port_loglike64(problem_of_state(prob, st))
    assert abs(m.coldChain().curLogLike - ref) <= 1e-6 * abs(ref)


def test_learned_proposal_against_plain(lib):
    """What the trained proposal gains, measured: from the same burned-in
    state, the chain with the learned move in p4's mixture against p4's plain
    mixture, 10,000 generations each.  Printed: ESS per 10,000 generations of
    lnL, tree length and gamma shape for both.  Asserted: the learned move is
    accepted often enough to matter (> 5 %), and both chains sample the same
    posterior: the learned chain's split frequencies agree with the plain
    chain's (ASDSF below 0.01, p4's usual convergence threshold; a second
    plain chain's is printed beside it), and the means of tree length and
    shape agree within 4 Monte Carlo standard errors."""
    prob, _ = sim.load_problem(golden_files()[0])       # 16 taxa, 1,000 sites, GTR+G4
    m = mcmc.Mcmc(prob, nChains=1, seed=5, sampleInterval=1)
    lp = LearnedProposal(m, hidden=128, seed=5, blockSize=4)
    m.learned = lp
    for _ in range(6000):
        m.step()
        lp.record(m.coldChain().cur)
    lp.fit(steps=1500, batch=256)
    lp.tune_kappa(m, gensPer=200)
    lp.freeze()
    start = m.coldChain().cur.copy()
    out = {}
    for name in ("plain", "plain2", "learned"):
        mm = mcmc.Mcmc(prob, nChains=1, seed=11 if name != "plain2" else 12, sampleInterval=1,
                       startState=start.copy())
        if name == "learned":
            mm.learned = lp
            mm.prob.learned = 0.5
            mm._makeProposals()
            a0, p0 = lp.nAccepted, lp.nProposed
        mm.run(10000)
        out[name] = mm.samples
    acc = (lp.nAccepted - a0) / max(1, lp.nProposed - p0)
    ess = {k: {q: mcmc.effective_sample_size(out[k][q]) for q in ("lnL", "treeLength", "alpha")} for k in out}
    print("ESS per 10,000 generations", ess, "learned acceptance", acc)
    assert acc > 0.05
    dLearned = mcmc.asdsf(out["plain"]["splits"], out["learned"]["splits"])
    dPlain = mcmc.asdsf(out["plain"]["splits"], out["plain2"]["splits"])
    print("ASDSF learned-plain", dLearned, "plain-plain", dPlain)
    assert dLearned < 0.01 and dPlain < 0.01
    for q in ("treeLength", "alpha"):
        a, b = numpy.asarray(out["plain"][q]), numpy.asarray(out["learned"][q])
        se = numpy.hypot(a.std() / numpy.sqrt(ess["plain"][q]), b.std() / numpy.sqrt(ess["learned"][q]))
        assert abs(a.mean() - b.mean()) <= 4.0 * se, (q, a.mean(), b.mean(), se)
