"""Learned joint proposal for the MCMC: an MLP trained during burn-in on the
chain's own samples, then frozen, proposing joint moves of branch lengths,
compositions and gamma shapes (a random block of those coordinates per
move), with an exact Metropolis-Hastings correction.  No counterpart in p4
(its proposals are hand-made); p4's proposals stay in the mixture.

Transformed space x (fixed dimension d):
  * log branch length of every node except the current root (node order);
  * additive log-ratio of every composition, log(pi_i / pi_last), i < dim-1;
  * log gamma shape of every part that has one.
The network maps the standardised state z = (x - m) / sd to (mu, s) and the
proposal is x' ~ N(x + sd * mu, diag((kappa * sd * exp(s))^2)).  It is
trained as a conditional density of the chain's lag-k moves: the loss is the
negative log density of (x_{t+k} - x_t) / sd under N(mu(z_t), exp(2 s(z_t))).

Hastings ratio in the model parameters theta (branch lengths, simplex
compositions, shapes):
  log q(x | x') - log q(x' | x) + log|dx/dtheta|(theta) - log|dx/dtheta|(theta')
with log|dx/dtheta| = -sum log b - sum over comps of sum_i log pi_i
- sum log alpha.  Priors: exponential(lambda) branch lengths and exponential(1)
shapes (as p4's defaults), flat Dirichlet compositions.  The network and
kappa are frozen before sampling, so the chain targets the exact posterior.
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
    def __init__(self, mcmc, hidden=128, seed=0, blockSize=8):
        self.mcmc = mcmc
        self.blockSize = blockSize
        prob = mcmc.problem
        self.nNodes = prob.tree.nNodes
        self.comps = [(p, c, sp.dim) for p, sp in enumerate(prob.parts) for c in range(sp.comps.shape[0])]
        self.gammas = [p for p, sp in enumerate(prob.parts) if sp.nCat > 1 and len(sp.gammaShapes)]
        self.d = (self.nNodes - 1) + sum(dim - 1 for (_, _, dim) in self.comps) + len(self.gammas)
        self.hidden = hidden
        self.net = Network(self.d, hidden, 2 * self.d, maxBatch=1024, seed=seed)
        self.mean = numpy.zeros(self.d)
        self.sd = numpy.ones(self.d)
        self.kappa = 1.0
        self.frozen = False
        self.history = []
        self.nProposed = 0
        self.nAccepted = 0

    # ---------------------------------------------------------- transforms
    def to_x(self, st):
        out = numpy.empty(self.d)
        k = 0
        for v in range(self.nNodes):
            if v == st.root:
                continue
            out[k] = math.log(st.brLen[v])
            k += 1
        for (p, c, dim) in self.comps:
            pi = st.parts[p].comps[c]
            out[k:k + dim - 1] = numpy.log(pi[:-1] / pi[-1])
            k += dim - 1
        for p in self.gammas:
            out[k] = math.log(st.parts[p].gamma[0])
            k += 1
        return out

    def from_x(self, x, st):
        """Write x into state st; returns False if outside the parameter bounds."""
        k = 0
        for v in range(self.nNodes):
            if v == st.root:
                continue
            b = math.exp(x[k])
            if not (var.BRLEN_MIN <= b <= var.BRLEN_MAX):
                return False
            st.brLen[v] = b
            k += 1
        for (p, c, dim) in self.comps:
            a = numpy.concatenate([x[k:k + dim - 1], [0.0]])
            a = numpy.exp(a - a.max())
            pi = a / a.sum()
            if pi.min() < var.PIVEC_MIN:
                return False
            pi[numpy.argmax(pi)] += 1.0 - pi.sum()
            st.parts[p].comps[c] = pi
            k += dim - 1
        for p in self.gammas:
            a = math.exp(x[k])
            if not (var.GAMMA_SHAPE_MIN <= a <= var.GAMMA_SHAPE_MAX):
                return False
            st.parts[p].gamma[0] = a
            k += 1
        return True

    def log_jacobian(self, st):
        """log |dx/dtheta| at theta."""
        j = -sum(math.log(st.brLen[v]) for v in range(self.nNodes) if v != st.root)
        for (p, c, dim) in self.comps:
            j -= float(numpy.log(st.parts[p].comps[c]).sum())
        for p in self.gammas:
            j -= math.log(st.parts[p].gamma[0])
        return j

    def log_prior(self, st):
        lam = self.mcmc.brLenPriorLambda
        lp = -lam * sum(st.brLen[v] for v in range(self.nNodes) if v != st.root)
        for p in self.gammas:
            lp -= st.parts[p].gamma[0]
        return lp

    # ---------------------------------------------------------- density
    def _gauss(self, x):
        y = self.net.forward(((x - self.mean) / self.sd)[None, :])[0].astype(numpy.float64)
        mu = y[: self.d] * self.sd
        s = numpy.clip(y[self.d:], -12.0, 6.0)
        sig = self.kappa * self.sd * numpy.exp(s)
        return mu, sig

    @staticmethod
    def _logq(xto, xfrom, mu, sig):
        r = (xto - xfrom - mu) / sig
        return float(-numpy.log(sig).sum() - 0.5 * (r * r).sum())

    # ---------------------------------------------------------- mcmc hooks
    def record(self, st):
        if not self.frozen:
            self.history.append(self.to_x(st))

    def propose(self, mcmc, ch, st, tuning):
        """Apply the learned move to state st (a copy of ch.cur); sets the
        chain's ratios and changed fields.  A block of `blockSize`
        coordinates, chosen uniformly at random (so the reverse move picks
        the same block with the same probability), moves jointly; the rest
        stay.  Only the block enters the proposal densities."""
        x = self.to_x(ch.cur)
        mu, sig = self._gauss(x)
        B = mcmc.rng.choice(self.d, size=min(self.blockSize, self.d), replace=False)
        xp = x.copy()
        xp[B] = x[B] + mu[B] + sig[B] * mcmc.rng.standard_normal(len(B))
        if not self.from_x(xp, st):
            return False
        mu2, sig2 = self._gauss(xp)
        fwd = self._logq(xp[B], x[B], mu[B], sig[B])
        rev = self._logq(x[B], xp[B], mu2[B], sig2[B])
        ch.logProposalRatio = rev - fwd + self.log_jacobian(ch.cur) - self.log_jacobian(st)
        ch.logPriorRatio = self.log_prior(st) - self.log_prior(ch.cur)
        ch.changed = {"brLen"} | {("comps", p) for (p, _, _) in self.comps} | {("gamma", p) for p in self.gammas}
        self.nProposed += 1
        return True

    # ---------------------------------------------------------- training
    def fit(self, lagMin=20, lagMax=None, steps=1500, batch=256, lr=1e-3, seed=0, burnFrac=0.5):
        """Train on the recorded cold-chain states from the later part of
        burn-in: pairs (x_t, x_{t+k}) with k uniform in [lagMin, lagMax], so
        the network learns where the chain goes over many generations."""
        H = numpy.array(self.history)
        H = H[int(len(H) * burnFrac):]
        n = len(H)
        lagMax = lagMax or max(lagMin + 1, n // 4)
        if n <= lagMax + 10:
            raise ValueError("not enough recorded states to train on")
        self.mean = H.mean(0)
        self.sd = H.std(0) + 1e-6
        Z = (H - self.mean) / self.sd
        rng = numpy.random.default_rng(seed)
        losses = []
        for i in range(steps):
            t0 = rng.integers(n - lagMax, size=batch)
            k = rng.integers(lagMin, lagMax + 1, size=batch)
            losses.append(self.net.train_step(Z[t0], Z[t0 + k] - Z[t0], lr))
        self.trainLosses = losses
        return losses

    def tune_kappa(self, mcmc, gensPer=200, kappas=(1.0, 0.7, 0.5, 0.35, 0.25, 0.18, 0.12)):
        """Pick the proposal scale during burn-in by expected squared jump
        (acceptance x kappa^2), running the chain with learned moves only."""
        saved = dict(mcmc.prob)
        for k in list(mcmc.prob):
            mcmc.prob[k] = 0.0
        mcmc.prob["learned"] = 1.0
        mcmc._makeProposals()
        best, bestScore = self.kappa, -1.0
        for kap in kappas:
            self.kappa = kap
            a0 = self.nAccepted
            p0 = self.nProposed
            mcmc.run(gensPer)
            acc = (self.nAccepted - a0) / max(1, self.nProposed - p0)
            score = acc * kap * kap
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
