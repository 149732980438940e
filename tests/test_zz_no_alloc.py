"""p4g_treeLogLikeNoAlloc (evaluation inside the library's fixed device
array, no allocation) against p4g_setPrams + p4g_treeLogLike on the same
tree, called through the C ABI.

Tolerance: |dlnL| <= 1e-6 |lnL|, the FP32-pruning tolerance of the parity
tests (the two entry points may use different pruning tile shapes, so the
per-tile partial sums are added in a different order).  Two no-allocation
calls in a row on the same values agree exactly: the array is shared by every
call, and a counter or flag left set by the first call would show up in the
second.
"""
import ctypes

import numpy
import pytest

from conftest import golden_files, golden_ids
from p4gpu import _lib, sim
from p4gpu.engine import Engine

pytestmark = pytest.mark.gpu

LNL_RTOL = 1e-6
P4G_EUNSUPPORTED = 7


def no_alloc(lib, e):
    out = ctypes.c_double(0.0)
    rc = lib.p4g_treeLogLikeNoAlloc(e.cTree, ctypes.byref(out))
    assert rc == 0, _lib.last_error()
    return out.value, numpy.array(e.partLikes, copy=True)


def check_pair(lib, e):
    ref = e.calcLogLike()
    refParts = numpy.array(e.partLikes, copy=True)
    a, pa = no_alloc(lib, e)
    b, pb = no_alloc(lib, e)
    assert abs(a - ref) <= LNL_RTOL * abs(ref), (a, ref)
    numpy.testing.assert_allclose(pa, refParts, rtol=LNL_RTOL)
    assert a == b and numpy.array_equal(pa, pb), (a, b)
    return ref


@pytest.fixture(params=golden_files(), ids=golden_ids())
def golden(request, lib):
    return sim.load_problem(request.param)


def test_no_alloc_matches_tree_loglike(lib, golden):
    prob, _ = golden
    e = Engine(prob)
    check_pair(lib, e)
    # new branch lengths and a new gamma shape: both entry points follow
    rng = numpy.random.default_rng(5)
    brLen = prob.tree.brLen * rng.uniform(0.7, 1.4, size=prob.tree.nNodes)
    e.setBrLens(brLen)
    for p, sp in enumerate(prob.parts):
        if len(sp.gammaShapes):
            e.setGamma(p, 0, float(sp.gammaShapes[0]) * 1.5)
    check_pair(lib, e)
    e.free()


@pytest.mark.parametrize("name", ["dna64het", "mcmcmc32"])
def test_no_alloc_full_size(lib, name):
    """64 taxa x 100k DNA sites with 4 compositions; 12 DNA and protein parts
    on 32 taxa."""
    prob = sim.make_config(name)
    e = Engine(prob)
    check_pair(lib, e)
    e.free()


def test_no_alloc_rejects_oversize(lib):
    """16 taxa x 1.1M distinct patterns need about 18 MiB of tip codes alone,
    beyond the fixed array: a clear error, and the library still works."""
    prob, _ = sim.load_problem(golden_files()[0])
    sp = prob.parts[0]
    rng = numpy.random.default_rng(3)
    nSites = 1100000
    acgt = numpy.frombuffer(b"acgt", numpy.uint8)
    sp.sequences = [acgt[rng.integers(0, 4, size=nSites)].tobytes().decode()
                    for _ in range(len(sp.sequences))]
    e = Engine(prob)
    out = ctypes.c_double(0.0)
    rc = lib.p4g_treeLogLikeNoAlloc(e.cTree, ctypes.byref(out))
    assert rc == P4G_EUNSUPPORTED
    msg = _lib.last_error()
    assert "P4G_NOALLOC_SCRATCH_BYTES" in msg and "bytes of scratch" in msg, msg
    e.free()
    prob2, z = sim.load_problem(golden_files()[0])
    e2 = Engine(prob2)
    a, _ = no_alloc(lib, e2)
    ref = float(z["ref_lnL"])
    assert abs(a - ref) <= LNL_RTOL * abs(ref)
    e2.free()
