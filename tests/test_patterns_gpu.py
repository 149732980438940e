"""Site-pattern compression on the GPU (p4g_makePatternsDevice) against the
host's makePatterns, which the CPU tests pin to the reference's
Pf/part.c:317-449 output: patterns, counts and the site -> pattern index
must be identical, including first-occurrence order."""
import numpy
import pytest

from conftest import golden_files, golden_ids
from p4gpu import pf, sim

pytestmark = pytest.mark.gpu


def both(nTax, seqs, sp):
    eq = sp.equateSymbols()
    out = []
    for device in (False, True):
        cp = pf.newPart(nTax, len(seqs[0]), eq, len(eq), sp.symbols, sp.dim)
        if eq:
            pf.pokeEquatesTable(cp, sp.equatesTable())
        pf.pokeSequences(cp, "".join(seqs))
        (pf.makePatternsDevice if device else pf.makePatterns)(cp)
        pf.setGlobalInvarSitesVec(cp)
        pats, cnt, spi = pf.getPatterns(cp, nTax, len(seqs[0]))
        vec, arr = pf.getInvarSites(cp, sp.dim, pats.shape[1])
        out.append((pats, cnt, spi, vec, arr))
        pf.freePart(cp)
    return out


def check_same(a, b):
    for x, y in zip(a, b):
        assert x.shape == y.shape and numpy.array_equal(x, y)


@pytest.mark.parametrize("path", golden_files(), ids=golden_ids())
def test_device_patterns_equal_host_on_fixtures(lib, path):
    prob, z = sim.load_problem(path)
    for p, sp in enumerate(prob.parts):
        host, dev = both(prob.nTax, sp.sequences, sp)
        check_same(host, dev)
        assert numpy.array_equal(dev[0], z["p%d_ref_patterns" % p])   # the reference's own output


@pytest.mark.parametrize("name", ["dna64het", "prot48het"])
def test_device_patterns_full_size(lib, name):
    prob = sim.make_config(name)
    sp = prob.parts[0]
    host, dev = both(prob.nTax, sp.sequences, sp)
    check_same(host, dev)
    assert dev[1].sum() == sp.nChar


def test_device_patterns_edge_cases(lib):
    prob, _ = sim.load_problem(golden_files()[0])
    sp = prob.parts[0]
    n = prob.nTax
    rng = numpy.random.default_rng(7)
    cases = [
        ["a"] * n,                                              # one site
        ["acgt" * 50] * n,                                      # every column constant within itself
        ["a" * 300] * n,                                        # one pattern only
        ["".join(rng.choice(list("acgt-?nrykm"), 2000)) for _ in range(n)],   # gaps and ambiguity codes
        ["".join(rng.choice(list("acgt"), 50000)) for _ in range(n)],          # nearly all distinct
    ]
    for seqs in cases:
        host, dev = both(n, seqs, sp)
        check_same(host, dev)
