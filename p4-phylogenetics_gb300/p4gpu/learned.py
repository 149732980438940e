"""Learned joint proposal for the MCMC: an MLP trained during burn-in on the
chain's own samples, then frozen, proposing joint moves of branch lengths,
compositions and gamma shapes, with an exact Metropolis-Hastings correction.
No counterpart in p4 (its proposals are hand-made); p4's proposals stay in
the mixture.

Coordinates.  x (fixed dimension d) holds
  * log branch length of every edge, edges ordered by their unordered node
    pair (so re-rooting, which moves a length from one node to another,
    leaves the coordinates alone);
  * additive log-ratio of every composition, log(pi_i / pi_last), i < dim-1;
  * log gamma shape of every part that has one.
At the end of burn-in the recorded states give a mean m and covariance
C = L L^T of x, and the model works in whitened coordinates
z = L^-1 (x - m), where the posterior's linear correlations (tree length
against gamma shape, neighbouring branches, composition coordinates) are
gone.

Network.  A block-conditional density: the input is (z with a block B of
coordinates zeroed, the 0/1 mask of B) and the output is (mu, s) for every
coordinate; trained on the recorded states with random blocks, scoring only
the coordinates of B (NaN targets elsewhere), it learns the posterior
conditional N(mu_B(z_-B), exp(2 s_B(z_-B))) of a block given the rest.

Move.  Pick a block B uniformly at random, evaluate the network once at
(z_-B, mask) and move the block by an autoregressive step towards that
conditional:
    z'_B = mu + (1 - kappa) (z_B - mu) + sqrt(2 kappa - kappa^2) sigma eps,
where mu is clipped to [-MU_MAX, MU_MAX] and sigma = exp(s) to
[SIG_MIN, SIG_MAX]: in whitened units the conditional of a Gaussian posterior
is N(0, 1), so the network is a bounded correction to that (a burn-in chain
is strongly autocorrelated, and an unbounded fit memorises its trajectory:
conditionals far narrower than the posterior's).  With useNet=False the move
uses N(0, 1) itself.
The step is reversible with respect to N(mu, sigma^2) and mu, sigma depend
only on z_-B, which the move leaves alone, so
    log q(z | z') - log q(z' | z) = log N(z_B; mu, sigma) - log N(z'_B; mu, sigma).
kappa = 1 draws the block from the learned conditional; smaller kappa stays
closer to the current state.

Hastings ratio in the model parameters theta (branch lengths, simplex
compositions, shapes): the ratio above plus
log|dx/dtheta|(theta) - log|dx/dtheta|(theta') (|dz/dx| = |L^-1| cancels),
with log|dx/dtheta| = -sum log b - sum over comps of sum_i log pi_i
- sum log alpha.  Priors: exponential(lambda) branch lengths and
exponential(1) shapes (p4's defaults), flat Dirichlet compositions.  The
network, m, L, block size and kappa are frozen before sampling, so the chain
targets the exact posterior.
"""
import ctypes
import math

import numpy

from . import _lib
from ._lib import check, fptr
from .var import var


class Network(object):
    """The library's MLP (BF16 weights, FP32 accumulate, Adam), as a Python object."""

    def __init__(self, dIn, hidden, dOut, maxBatch=1024, seed=0):
        self.dIn, self.hidden, self.dOut, self.maxBatch = dIn, hidden, dOut, maxBatch
        self.h = _lib.handle(_lib.load().p4g_mlpNew(dIn, hidden, dOut, maxBatch, seed), "mlpNew")
        n = ctypes.c_int(0)
        check(_lib.load().p4g_mlpNumParams(self.h, ctypes.byref(n)), "mlpNumParams")
        self.nParams = n.value

    def params(self):
        out = numpy.zeros(self.nParams, numpy.float32)
        check(_lib.load().p4g_mlpGetParams(self.h, fptr(out)), "mlpGetParams")
        return out

    def set_params(self, p):
        p = numpy.ascontiguousarray(p, numpy.float32)
        check(_lib.load().p4g_mlpSetParams(self.h, fptr(p)), "mlpSetParams")

    def forward(self, x):
        x = numpy.ascontiguousarray(numpy.atleast_2d(x), numpy.float32)
        y = numpy.zeros((x.shape[0], self.dOut), numpy.float32)
        check(_lib.load().p4g_mlpForward(self.h, fptr(x), x.shape[0], fptr(y)), "mlpForward")
        return y

    def gradients(self, x, t):
        x = numpy.ascontiguousarray(x, numpy.float32)
        t = numpy.ascontiguousarray(t, numpy.float32)
        g = numpy.zeros(self.nParams, numpy.float32)
        loss = ctypes.c_float(0.0)
        check(_lib.load().p4g_mlpGradients(self.h, fptr(x), fptr(t), x.shape[0], fptr(g), ctypes.byref(loss)),
              "mlpGradients")
        return loss.value, g

    def train_step(self, x, t, lr):
        x = numpy.ascontiguousarray(x, numpy.float32)
        t = numpy.ascontiguousarray(t, numpy.float32)
        loss = ctypes.c_float(0.0)
        check(_lib.load().p4g_mlpTrainStep(self.h, fptr(x), fptr(t), x.shape[0], float(lr), ctypes.byref(loss)),
              "mlpTrainStep")
        return loss.value

    def free(self):
        if self.h:
            _lib.load().p4g_mlpFree(self.h)
            self.h = None


class LearnedProposal(object):
    """blockSize: whitened coordinates moved per proposal (None: all)."""

    MU_MAX, SIG_MIN, SIG_MAX = 0.5, 0.5, 2.0

    def __init__(self, mcmc, hidden=128, seed=0, blockSize=4, useNet=True, mode="rw"):
        self.mcmc = mcmc
        prob = mcmc.problem
        self.nNodes = prob.tree.nNodes
        self.comps = [(p, c, sp.dim) for p, sp in enumerate(prob.parts) for c in range(sp.comps.shape[0])]
        self.compParts = [(p, sp.comps.shape[0], sp.dim) for p, sp in enumerate(prob.parts) if sp.comps.shape[0]]
        self.gammas = [p for p, sp in enumerate(prob.parts) if sp.nCat > 1 and len(sp.gammaShapes)]
        self.d = (self.nNodes - 1) + sum(dim - 1 for (_, _, dim) in self.comps) + len(self.gammas)
        self.blockSize = self.d if not blockSize else min(int(blockSize), self.d)
        self.hidden = hidden
        self.useNet = useNet
        self.mode = mode
        self.net = Network(2 * self.d, hidden, 2 * self.d, maxBatch=1024, seed=seed) if useNet else None
        if self.net is not None:
            # start from the whitened Gaussian: output biases mu = 0, s = 0
            w = self.net.params()
            w[-self.d:] = 0.0
            self.net.set_params(w)
        self.mean = numpy.zeros(self.d)
        self.L = numpy.eye(self.d)
        self.Linv = numpy.eye(self.d)
        self.kappa = 1.0
        self.frozen = False
        self.history = []
        self.nProposed = 0
        self.nAccepted = 0
        self.sumJump = 0.0

    # ---------------------------------------------------------- transforms
    def edges(self, st):
        """Non-root nodes (each stores the length of the edge to its parent),
        ordered by the edge's unordered node pair."""
        v = numpy.arange(self.nNodes)
        v = v[v != st.root]
        par = numpy.asarray(st.parent)[v]
        key = numpy.minimum(v, par) * self.nNodes + numpy.maximum(v, par)
        return v[numpy.argsort(key, kind="stable")]

    def to_x(self, st):
        out = [numpy.log(numpy.asarray(st.brLen, dtype=float)[self.edges(st)])]
        for (p, nc, dim) in self.compParts:
            pi = st.parts[p].comps
            out.append(numpy.log(pi[:, :-1] / pi[:, -1:]).ravel())
        for p in self.gammas:
            out.append([math.log(st.parts[p].gamma[0])])
        return numpy.concatenate(out)

    def from_x(self, x, st):
        """Write x into state st; returns False if outside the parameter bounds."""
        e = self.edges(st)
        k = len(e)
        b = numpy.exp(x[:k])
        if b.min() < var.BRLEN_MIN or b.max() > var.BRLEN_MAX:
            return False
        st.brLen[e] = b
        for (p, nc, dim) in self.compParts:
            a = numpy.zeros((nc, dim))
            a[:, :-1] = x[k:k + nc * (dim - 1)].reshape(nc, dim - 1)
            a = numpy.exp(a - a.max(axis=1, keepdims=True))
            pi = a / a.sum(axis=1, keepdims=True)
            if pi.min() < var.PIVEC_MIN:
                return False
            rows = numpy.arange(nc)
            pi[rows, numpy.argmax(pi, axis=1)] += 1.0 - pi.sum(axis=1)
            st.parts[p].comps[:] = pi
            k += nc * (dim - 1)
        for p in self.gammas:
            a = math.exp(x[k])
            if not (var.GAMMA_SHAPE_MIN <= a <= var.GAMMA_SHAPE_MAX):
                return False
            st.parts[p].gamma[0] = a
            k += 1
        return True

    def _brLens(self, st):
        b = numpy.asarray(st.brLen, dtype=float)
        return b[numpy.arange(self.nNodes) != st.root]

    def log_jacobian(self, st):
        """log |dx/dtheta| at theta."""
        j = -float(numpy.log(self._brLens(st)).sum())
        for (p, nc, dim) in self.compParts:
            j -= float(numpy.log(st.parts[p].comps).sum())
        for p in self.gammas:
            j -= math.log(st.parts[p].gamma[0])
        return j

    def log_prior(self, st):
        lp = -self.mcmc.brLenPriorLambda * float(self._brLens(st).sum())
        for p in self.gammas:
            lp -= st.parts[p].gamma[0]
        return lp

    # ---------------------------------------------------------- density
    def to_z(self, x):
        return self.Linv @ (x - self.mean)

    def from_z(self, z):
        return self.mean + self.L @ z

    def conditional(self, z, B):
        """(mu, sigma) of the learned conditional of block B given the rest."""
        if not self.useNet:
            return numpy.zeros(len(B)), numpy.ones(len(B))
        mask = numpy.zeros(self.d)
        mask[B] = 1.0
        inp = numpy.concatenate([z * (1.0 - mask), mask])
        y = self.net.forward(inp[None, :])[0].astype(numpy.float64)
        sig = numpy.clip(numpy.exp(numpy.clip(y[self.d:], -12.0, 6.0)), self.SIG_MIN, self.SIG_MAX)
        return numpy.clip(y[: self.d][B], -self.MU_MAX, self.MU_MAX), sig[B]

    @staticmethod
    def _lognormal(z, mu, sig):
        r = (z - mu) / sig
        return float(-numpy.log(sig).sum() - 0.5 * (r * r).sum())

    # ---------------------------------------------------------- mcmc hooks
    def record(self, st):
        if not self.frozen:
            self.history.append(self.to_x(st))

    def propose(self, mcmc, ch, st, tuning):
        """Apply the learned move to state st (a copy of ch.cur); sets the
        chain's ratios and changed fields."""
        z = self.to_z(self.to_x(ch.cur))
        B = numpy.arange(self.d) if self.blockSize >= self.d else \
            mcmc.rng.choice(self.d, size=self.blockSize, replace=False)
        mu, sig = self.conditional(z, B)
        zp = z.copy()
        if self.mode == "rw":
            # random walk scaled by the learned conditional sd: sigma depends on
            # z_-B only, so the move is symmetric
            zp[B] = z[B] + self.kappa * sig * mcmc.rng.standard_normal(len(B))
            lq = 0.0
        else:
            k = self.kappa
            zp[B] = mu + (1.0 - k) * (z[B] - mu) + math.sqrt(2.0 * k - k * k) * sig * mcmc.rng.standard_normal(len(B))
            lq = self._lognormal(z[B], mu, sig) - self._lognormal(zp[B], mu, sig)
        if not self.from_x(self.from_z(zp), st):
            return False
        ch.logProposalRatio = lq + self.log_jacobian(ch.cur) - self.log_jacobian(st)
        ch.logPriorRatio = self.log_prior(st) - self.log_prior(ch.cur)
        ch.changed = {"brLen"} | {("comps", p) for (p, _, _) in self.comps} | {("gamma", p) for p in self.gammas}
        ch.learnedJump = float(((zp - z) ** 2).sum())
        self.nProposed += 1
        return True

    # ---------------------------------------------------------- training
    def fit(self, steps=1500, batch=256, lr=1e-3, seed=0, burnFrac=0.5, thin=10, check=50, patience=5):
        """Whiten the recorded cold-chain states from the later part of burn-in
        and train the block-conditional network on every `thin`-th of them (a
        random block per row, of the move's block size).  A fifth of those
        states is held out: training stops when their loss has not improved
        for `patience` checks (every `check` steps), and the best weights are
        kept, so the network moves away from the whitened Gaussian only as
        far as it generalises."""
        H = numpy.array(self.history)
        H = H[int(len(H) * burnFrac):]
        n = len(H)
        if n < 50:
            raise ValueError("not enough recorded states to train on")
        self.mean = H.mean(0)
        C = numpy.cov(H.T).reshape(self.d, self.d)
        C += numpy.eye(self.d) * (1e-6 * max(float(numpy.trace(C)) / self.d, 1e-12))
        self.L = numpy.linalg.cholesky(C)
        self.Linv = numpy.linalg.inv(self.L)
        Z = ((H - self.mean) @ self.Linv.T)[::max(1, int(thin))]
        n = len(Z)
        rng = numpy.random.default_rng(seed)
        losses = []
        if not self.useNet:
            self.trainLosses = losses
            return losses
        b = self.blockSize

        def masked(rows):
            keys = rng.random((len(rows), self.d))
            mask = (keys <= numpy.sort(keys, axis=1)[:, b - 1:b]).astype(numpy.float64)   # b random coords per row
            return numpy.concatenate([rows * (1.0 - mask), mask], axis=1), numpy.where(mask > 0, rows, numpy.nan)

        perm = rng.permutation(n)
        nVal = max(1, n // 5)
        val, train = Z[perm[:nVal]], Z[perm[nVal:]]
        vIn, vT = masked(numpy.repeat(val, max(1, 1024 // nVal), axis=0)[:1024])
        best = self.net.gradients(vIn, vT)[0]
        bestW = self.net.params()
        self.valLosses = [best]
        bad = 0
        for i in range(steps):
            inp, tgt = masked(train[rng.integers(len(train), size=batch)])
            losses.append(self.net.train_step(inp, tgt, lr))
            if (i + 1) % check == 0:
                v = self.net.gradients(vIn, vT)[0]
                self.valLosses.append(v)
                if v < best:
                    best, bestW, bad = v, self.net.params(), 0
                else:
                    bad += 1
                    if bad >= patience:
                        break
        self.net.set_params(bestW)
        self.trainLosses = losses
        return losses

    def tune_kappa(self, mcmc, gensPer=200, kappas=None):
        """Pick kappa during burn-in by the expected squared whitened jump
        (the mean of the accepted ||z' - z||^2 per proposal), running the chain
        with learned moves only."""
        saved = dict(mcmc.prob)
        for k in list(mcmc.prob):
            mcmc.prob[k] = 0.0
        mcmc.prob["learned"] = 1.0
        mcmc._makeProposals()
        if kappas is None:
            kappas = (2.4, 1.6, 1.0, 0.6, 0.35) if self.mode == "rw" else (1.0, 0.5, 0.25, 0.1)
        best, bestScore = self.kappa, -1.0
        self.kappaScores = {}
        for kap in kappas:
            self.kappa = kap
            p0, j0 = self.nProposed, self.sumJump
            mcmc.run(gensPer)
            score = (self.sumJump - j0) / max(1, self.nProposed - p0)
            self.kappaScores[kap] = score
            if score > bestScore:
                best, bestScore = kap, score
        self.kappa = best
        mcmc.prob.clear()
        mcmc.prob.update(saved)
        mcmc._makeProposals()
        return best

    def freeze(self, kappa=None):
        if kappa is not None:
            self.kappa = float(kappa)
        self.frozen = True
        self.history = []
