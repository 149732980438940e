"""The MCMC's output files and checkpoints, in p4's formats.

  mcmc_likes_<runNum>          '%11i %f' per sample: gen+1, the cold chain's
                               lnL (Mcmc._writeSample, p4/mcmc.py:3209-3214)
  mcmc_trees_<runNum>.nex      Nexus: taxa block, a trees block with a
                               translate table, the '[&&p4 models ...]'
                               comment for heterogeneous models, then one
                               '  tree t_<gen+1> = [&U] <newick>;' per sample
                               (p4/mcmc.py:2422-2481, 3231-3253); 'end;'
                               closes the block after every run() and is
                               removed again when the next run() starts
                               (p4/mcmc.py:2711-2741)
  mcmc_prams_<runNum>          the parameter profile as '#' comments, a
                               'genPlus1' header line, then per sample gen+1
                               and every free parameter (Model.writePramsProfile,
                               writePramsHeaderLine, writePramsLine,
                               p4/model.py:511-720)
  mcmc_pramsProfile_<runNum>.py  the column layout (p4/model.py:626-632)
  mcmc_checkPoint_<runNum>.<gen+1>  a pickle of the run's host state
                               (Mcmc.checkPoint, p4/mcmc.py:3516-3642)

A checkpoint holds what the GPU state is derived from: the tree and model
(the data are detached, as p4 detaches them, and re-attached on restart),
every chain's parameter state, lnL and temperature, the proposals' tunings
and counts, the swap counts and the random-number generator's state.  The
GPU buffers are rebuilt from those on restart (p4gpu.func.unPickleMcmc).
"""
import glob
import math
import os
import pickle
import re

from .p4exceptions import P4Error

CHECKPOINT_VERSION = 1


def _names(runNum):
    return ("mcmc_likes_%i" % runNum, "mcmc_trees_%i.nex" % runNum, "mcmc_prams_%i" % runNum,
            "mcmc_pramsProfile_%i.py" % runNum)


def nexus_name(name):
    """A taxon name as Nexus needs it: single-quoted (quotes doubled) when it
    holds anything but letters, digits, '_' and '.' (func.nexusFixNameIfQuotesAreNeeded)."""
    if re.fullmatch(r"[A-Za-z0-9_.]+", name):
        return name
    return "'" + name.replace("'", "''") + "'"


def check_new_run(m):
    """A new run refuses to overwrite an earlier run's checkpoints
    (p4/mcmc.py:862-876)."""
    if any(f.startswith("mcmc_checkPoint_%i." % m.runNum) for f in os.listdir(os.getcwd())):
        raise P4Error("runNum is set to %i, and there is at least one mcmc_checkPoint_%i.xxx file in this "
                      "directory.  This is a new Mcmc, and I am refusing to over-write existing files.  Maybe you "
                      "want to re-start from the latest mcmc_checkPoint_%i file?" % (m.runNum, m.runNum, m.runNum))


# ----------------------------------------------------------------- free parameters
def free_parameters(m):
    """Per part, the changeable parameters the run samples, in p4's column
    order: relRate, comps, R matrices, gamma shapes, pInvar."""
    out = []
    pr = m.prob
    for p, sp in enumerate(m.problem.parts):
        cols = []
        if m.freeRelRates:
            cols.append(("relRate", 1))
        if pr.allCompsDir and sp.comps.shape[0]:
            cols += [("comp", sp.dim)] * sp.comps.shape[0]
        if pr.allRMatricesDir:
            cols += [("rMatrix", sp.dim * (sp.dim - 1) // 2)] * sp.rmats.shape[0]
        if pr.gdasrv and sp.nCat > 1:
            cols += [("gdasrv", 1)] * len(sp.gammaShapes)
        if m.freePInvar[p]:
            cols.append(("pInvar", 1))
        out.append(cols)
    return out


def n_free_prams(m):
    """Free parameters (p4's count): dim-1 per comp, k-1 per R matrix of k
    rates (normalised to sum 1), one per gamma shape and pInvar, nParts-1
    relative rates."""
    n = 0
    for cols in free_parameters(m):
        for kind, k in cols:
            if kind in ("comp", "rMatrix"):
                n += k - 1
            elif kind != "relRate":
                n += 1
    if m.freeRelRates:
        n += len(m.problem.parts) - 1
    return n


def write_prams_profile(m, flob):
    """Model.writePramsProfile (p4/model.py:511-635) and the
    mcmc_pramsProfile_<runNum>.py file."""
    spacer1, spacer2 = " " * 23, " " * 12
    flob.write("# Model.writePramsProfile() runNum %i\n# \n" % m.runNum)
    flob.write("# There are %i free parameters in this model.\n" % n_free_prams(m))
    flob.write("# The parameters sampled at a given gen+1 are written on one line.\n")
    flob.write("# The first number is gen+1, followed by any changeable model parameters.\n")
    flob.write("# The number of changeable model parameters may be more than the \n")
    flob.write("#  number of free model parameters, eg for DNA composition, there are\n")
    flob.write("#  3 free parameters, but 4 changeable parameters.\n")
    flob.write("# The column number or column range for each parameter or\n")
    flob.write("#  parameter set is given twice-- the first is zero-based \n")
    flob.write("#  numbering, and the second is one-based numbering.\n")
    flob.write("# Numbers in square brackets are the number of parameters listed.\n# \n")
    flob.write("#   0-based 1-based\n#   ------- -------\n")
    nParts = len(m.problem.parts)
    flob.write("#%s%i data partitions\n" % (spacer1, nParts))
    if nParts > 1 and m.freeRelRates:
        flob.write("#%sRelative rates are set and free.\n" % spacer1)
    pramsList = []
    z, o = 1, 2
    nPrams = 0
    for p, cols in enumerate(free_parameters(m)):
        flob.write("#%sData Partition %i\n" % (spacer1, p))
        pramsList.append([])
        for kind, k in cols:
            if k == 1:
                flob.write("#   %7i %7i %s%s[1]\n" % (z, o, spacer2, kind))
            else:
                flob.write("#   %7s %7s %s%s[%i]\n" % ("%i-%i" % (z, z + k - 1), "%i-%i" % (o, o + k - 1), spacer2,
                                                      kind, k))
            pramsList[p].append([kind, k])
            nPrams += k
            z += k
            o += k
    flob.write("# \n# %i changeable prams in all.\n# \n" % nPrams)
    with open(_names(m.runNum)[3], "w") as f:
        f.write("# This file, 'mcmc_pramsProfile_%i.py', is used by func.summarizeMcmcPrams() and "
                "PosteriorSamples\n" % m.runNum)
        f.write("pramsProfile = %s\n" % pramsList)
        f.write("nPrams = %i\n" % nPrams)


def write_prams_header(m, flob):
    """'genPlus1' and the column names (Model.writePramsHeaderLine,
    p4/model.py:688-720)."""
    flob.write("genPlus1")
    for p, cols in enumerate(free_parameters(m)):
        counters = {}
        for kind, k in cols:
            i = counters.get(kind, 0)
            counters[kind] = i + 1
            if kind == "relRate":
                flob.write("\trelRate.%i" % p)
            elif kind in ("comp", "rMatrix"):
                for j in range(k):
                    flob.write("\t%s.%i.%i.%i" % (kind, p, i, j))
            elif kind == "gdasrv":
                flob.write("\tgdasrv.%i.%i" % (p, i))
            else:
                flob.write("\tpInvar.%i" % p)
    flob.write("\n")


def write_prams_line(m, st, flob):
    """One sample's values (Model.writePramsLine, p4/model.py:637-671):
    relRates, gamma shapes '\\t%12.6f', comps, R rates, pInvar '\\t%10.8f'."""
    pr = m.prob
    for p, ps in enumerate(st.parts):
        sp = m.problem.parts[p]
        if m.freeRelRates:
            flob.write("\t%12.6f" % ps.relRate)
        if pr.allCompsDir and sp.comps.shape[0]:
            for c in ps.comps:
                for v in c:
                    flob.write("\t%10.8f" % v)
        if pr.allRMatricesDir:
            for r in ps.rvals:
                for v in r:
                    flob.write("\t%10.8f" % v)
        if pr.gdasrv and sp.nCat > 1:
            for g in ps.gamma:
                flob.write("\t%12.6f" % g)
        if m.freePInvar[p]:
            flob.write("\t%10.8f" % ps.pInvar)
    flob.write("\n")


# ----------------------------------------------------------------- sample files
class SampleFiles(object):
    """The open sample files of one run() call."""

    def __init__(self, m):
        self.likesName, self.treesName, self.pramsName, _ = _names(m.runNum)
        tree = m.tree
        self.translation = {name: i + 1 for i, name in enumerate(tree.taxNames)}
        self.writePrams = m.writePrams and n_free_prams(m) > 0
        if m.gen < 0:
            if os.path.isfile(self.treesName):
                raise P4Error("The file '%s' already exists." % self.treesName)
            with open(self.treesName, "w") as f:
                f.write("#nexus\n\nbegin taxa;\n  dimensions ntax=%s;\n  taxlabels" % tree.nTax)
                for name in tree.taxNames:
                    f.write(" %s" % nexus_name(name))
                f.write(";\nend;\n\nbegin trees;\n  translate\n")
                for i, name in enumerate(tree.taxNames):
                    f.write("    %3i %s%s\n" % (i + 1, nexus_name(name), "," if i < tree.nTax - 1 else ""))
                f.write("  ;\n")
                model = tree.model
                if model.isHet:
                    f.write("  [&&p4 models p%i" % model.nParts)
                    for p, mp in enumerate(model.parts):
                        f.write(" c%i.%i r%i.%i g%i.%i" % (p, mp.nComps, p, mp.nRMatrices, p, mp.nGdasrvs))
                    f.write("]\n")
                f.write("  [Tree numbers are gen+1]\nend;\n")
            self.likes = open(self.likesName, "w")
            if self.writePrams:
                self.prams = open(self.pramsName, "w")
                write_prams_profile(m, self.prams)
                write_prams_header(m, self.prams)
            else:
                self.prams = None
        else:
            self.likes = open(self.likesName, "a")
            self.prams = open(self.pramsName, "a") if self.writePrams else None
        # every run() -- the first too -- reopens the trees block (p4/mcmc.py:2711-2741)
        strip_trailing_end(self.treesName)
        self.trees = open(self.treesName, "a")

    def sample(self, m):
        ch = m.coldChain()
        st = ch.cur
        self.likes.write("%11i %f\n" % (m.gen + 1, ch.curLogLike))
        self.trees.write("  tree t_%i = [&U] " % (m.gen + 1))
        m.tree.writeNewick(self.trees, self.translation, m.tree.model.isHet, brLen=st.brLen, parent=st.parent,
                           leftChild=st.leftChild, sibling=st.sibling, root=st.root)
        if self.prams is not None:
            self.prams.write("%12i" % (m.gen + 1))
            write_prams_line(m, st, self.prams)

    def flush(self):
        for f in (self.likes, self.trees, self.prams):
            if f is not None:
                f.flush()

    def finish(self):
        self.trees.write("end;\n\n")
        for f in (self.likes, self.trees, self.prams):
            if f is not None:
                f.close()


def strip_trailing_end(path):
    """Remove the 'end;' that closes the tree file's trees block, so that a
    continuing run appends its trees inside the block (p4/mcmc.py:2711-2741)."""
    with open(path, "r+b") as f:
        f.seek(0, 2)
        size = f.tell()
        pos = -1
        while -pos <= size:
            f.seek(pos, 2)
            if f.read(1) == b";":
                break
            pos -= 1
        pos -= 3
        f.seek(pos, 2)
        if f.read(4) != b"end;":
            raise P4Error("Failed to find and remove the 'end;' at the end of the tree file %s." % path)
        f.seek(pos, 2)
        f.truncate()


# ----------------------------------------------------------------- checkpoints
def _proposal_record(p):
    return {k: getattr(p, k) for k in ("name", "pNum", "weight", "tuning", "tnNSamples", "tnNAccepts",
                                       "nProposals", "nAcceptances", "nAborts", "nTopologyChanges")}


def check_point(m):
    """Mcmc.checkPoint: recompute, compare within 0.01, pickle; returns the
    file name."""
    lnls = m.recomputeLogLikes()
    for i, (ch, l) in enumerate(zip(m.chains, lnls)):
        if math.fabs(ch.curLogLike - l) > 0.01:
            print("Mcmc.checkPoint(), chainNum %i. Bad likelihood calculation just before writing the checkpoint. "
                  "Old curTree.logLike %g, new curTree.logLike %g, diff %g"
                  % (i, ch.curLogLike, l, math.fabs(ch.curLogLike - l)))
    if m.files is not None:
        m.files.flush()
    data, m.tree.data = m.tree.data, None
    try:
        d = {"version": CHECKPOINT_VERSION, "runNum": m.runNum, "gen": m.gen, "nChains": m.nChains,
             "chainTemp": m.chainTemp, "chainTemps": list(m.chainTemps), "sampleInterval": m.sampleInterval,
             "checkPointInterval": m.checkPointInterval, "writePrams": m.writePrams, "prob": dict(m.prob),
             "brLenPriorLambda": m.brLenPriorLambda, "doTuning": m.doTuning, "freePInvar": list(m.freePInvar),
             "freeRelRates": m.freeRelRates, "tree": m.tree,
             "chains": [{"cur": ch.cur, "curLogLike": ch.curLogLike, "tempNum": ch.tempNum} for ch in m.chains],
             "proposals": [_proposal_record(p) for p in m.proposals],
             "swapAttempts": list(m.swapAttempts), "swapAccepts": list(m.swapAccepts),
             "rng": m.rng.bit_generator.state, "samples": m.samples}
        fName = "mcmc_checkPoint_%i.%i" % (m.runNum, m.gen + 1)
        with open(fName, "wb") as f:
            pickle.dump(d, f, pickle.HIGHEST_PROTOCOL)
    finally:
        m.tree.data = data
    return fName


def latest_checkpoint(runNum):
    ff = glob.glob("mcmc_checkPoint_%i.*" % runNum)
    nums = []
    for f in ff:
        try:
            nums.append((int(f.rsplit(".", 1)[1]), f))
        except ValueError:
            pass
    if not nums:
        raise P4Error("Can't find any checkpoints for runNum %i.  Got the right runNum?" % runNum)
    return max(nums)[1]


def restore(fName, theData, evaluator="graph", verbose=True):
    """An Mcmc ready to continue from a checkpoint file: the tree and model it
    holds with theData attached, the library state rebuilt, every chain's lnL
    recomputed and required to agree with the checkpointed one within 0.01."""
    from .mcmc import Mcmc, McmcProposalProbs
    if verbose:
        print("...unpickling Mcmc in %s" % fName)
    with open(fName, "rb") as f:
        d = pickle.load(f)
    if d.get("version") != CHECKPOINT_VERSION:
        raise P4Error("%s: checkpoint version %r, expected %d" % (fName, d.get("version"), CHECKPOINT_VERSION))
    tree = d["tree"]
    tree.data = theData
    m = Mcmc(tree, nChains=d["nChains"], runNum=d["runNum"], sampleInterval=d["sampleInterval"],
             checkPointInterval=d["checkPointInterval"], writePrams=d["writePrams"], chainTemp=d["chainTemp"],
             prob=McmcProposalProbs(**d["prob"]), startState=d["chains"][0]["cur"],
             brLenPriorLambda=d["brLenPriorLambda"], tune=d["doTuning"], freeRelRates=d["freeRelRates"],
             freePInvar=d["freePInvar"], evaluator=evaluator, writeFiles=True, _restart=True)
    m.chainTemps = list(d["chainTemps"])
    for ch, rec in zip(m.chains, d["chains"]):
        ch.cur = rec["cur"].copy()
        ch.tempNum = rec["tempNum"]
    byKey = {(r["name"], r["pNum"]): r for r in d["proposals"]}
    for p in m.proposals:
        r = byKey.get((p.name, p.pNum))
        if r is None:
            continue
        for k, v in r.items():
            if k not in ("name", "pNum"):
                setattr(p, k, list(v) if isinstance(v, list) else v)
    m.swapAttempts = list(d["swapAttempts"])
    m.swapAccepts = list(d["swapAccepts"])
    m.rng.bit_generator.state = d["rng"]
    m.gen = d["gen"]
    m.samples = d["samples"]
    lnls = m.recomputeLogLikes()
    for i, (rec, l) in enumerate(zip(d["chains"], lnls)):
        if math.fabs(rec["curLogLike"] - l) > 0.01:
            raise P4Error("restart from %s, chain %i: recomputed lnL %g differs from the checkpointed %g by %g "
                          "(more than 0.01)" % (fName, i, l, rec["curLogLike"], math.fabs(rec["curLogLike"] - l)))
    for ch, l in zip(m.chains, lnls):
        ch.curLogLike = l
    return m
