"""libp4gpu host-side checks that need no GPU: the C ABI loads and exports
every symbol include/p4gpu.h declares, and the host parts of the data path
(char coding, pattern compression, invariant sites, discrete gamma) match
the reference's outputs bit for bit."""
import os
import re

import numpy
import pytest

from conftest import REPO, golden_files, golden_ids
from p4gpu import P4Error, pf, sim


def header_symbols():
    txt = open(os.path.join(REPO, "include", "p4gpu.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(p4g_[A-Za-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol(lib):
    syms = header_symbols()
    assert len(syms) > 40
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing


def test_binding_covers_header(lib):
    from p4gpu import _lib
    assert sorted(_lib.exported_symbols()) == header_symbols()


@pytest.fixture(params=golden_files(), ids=golden_ids())
def golden(request):
    return sim.load_problem(request.param)


def _cpart(prob, p):
    sp = prob.parts[p]
    eq = sp.equateSymbols()
    cp = pf.newPart(prob.nTax, sp.nChar, eq, len(eq), sp.symbols, sp.dim)
    if eq:
        pf.pokeEquatesTable(cp, sp.equatesTable())
    pf.pokeSequences(cp, "".join(sp.sequences))
    pf.makePatterns(cp)
    pf.setGlobalInvarSitesVec(cp)
    return cp


def test_library_patterns_bitexact_vs_reference(golden, lib):
    prob, z = golden
    for p, sp in enumerate(prob.parts):
        k = "p%d_" % p
        cp = _cpart(prob, p)
        pats, cnt, spi = pf.getPatterns(cp, prob.nTax, sp.nChar)
        vec, arr = pf.getInvarSites(cp, sp.dim, pats.shape[1])
        assert numpy.array_equal(pats, z[k + "ref_patterns"])
        assert numpy.array_equal(cnt, z[k + "ref_counts"])
        assert numpy.array_equal(spi, z[k + "ref_seqPosIdx"])
        assert numpy.array_equal(vec, z[k + "ref_invVec"])
        assert numpy.array_equal(arr, z[k + "ref_invArr"])
        pf.freePart(cp)


def test_library_gamma_rates_vs_reference(golden, lib):
    prob, z = golden
    for p, sp in enumerate(prob.parts):
        if sp.nCat == 1:
            continue
        for g, a in enumerate(sp.gammaShapes):
            f = numpy.zeros(sp.nCat)
            r = numpy.zeros(sp.nCat)
            pf.gdasrvCalcRates_np(sp.nCat, a, f, r)
            numpy.testing.assert_allclose(r, z["p%d_ref_gammaRates" % p][g], rtol=1e-14, atol=0)
            assert numpy.all(f == 1.0 / sp.nCat)


def test_unknown_character_raises(lib):
    cp = pf.newPart(2, 3, "", 0, "acgt", 4)
    with pytest.raises(P4Error, match="neither a symbol"):
        pf.pokeSequences(cp, "acgtxa")


def test_pattern_edge_cases(lib):
    # one site; all-identical columns; every column distinct
    for seqs in (["a", "c", "g"], ["aaaa", "aaaa", "aaaa"], ["acgt", "cgta", "gtac"]):
        cp = pf.newPart(len(seqs), len(seqs[0]), "", 0, "acgt", 4)
        pf.pokeSequences(cp, "".join(seqs))
        pf.makePatterns(cp)
        n = pf.partPatternCount(cp)
        pats, cnt, spi = pf.getPatterns(cp, len(seqs), len(seqs[0]))
        cols = ["".join(s[i] for s in seqs) for i in range(len(seqs[0]))]
        uniq = list(dict.fromkeys(cols))
        assert n == len(uniq) and cnt.sum() == len(cols)
        assert [uniq.index(c) for c in cols] == list(spi)


def test_bad_model_values_raise_before_device_work(lib):
    prob, _ = sim.load_problem(golden_files()[0])
    from p4gpu.engine import Engine
    e = Engine(prob)
    e.compVals[0][0][:] = [0.5, 0.5, 0.1, 0.0]   # sum != 1, below PIVEC_MIN
    with pytest.raises(P4Error, match="PIVEC_MIN|sum to 1"):
        e.setPrams()
