"""p4g_treeLogLikeNoAlloc (evaluation inside the library's fixed device
array, no allocation) against p4g_setPrams + p4g_treeLogLike on the same
tree and against the reference's stored lnL, called through the C ABI.

The callers this entry point serves cannot allocate device memory: code
running inside a program whose device memory belongs to another allocator
(a framework's caching pool, or an arena reserved up front for a fixed
budget), where cudaMalloc fails once the pool holds the memory and where a
cudaMalloc / cudaFree would synchronise the whole device.  So besides the
values, the tests check that a tree evaluated only through this entry point
gets no device memory of its own, that the device's free memory does not
drop across a call, and that the call succeeds while another allocation
holds nearly all of the device's free memory.

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


def device_bytes(lib, e):
    tb, db = ctypes.c_longlong(-1), ctypes.c_longlong(-1)
    assert lib.p4g_treeDeviceBytes(e.cTree, ctypes.byref(tb), ctypes.byref(db)) == 0, _lib.last_error()
    return tb.value, db.value


def check_pair(lib, e):
    ref = e.calcLogLike()
    refParts = numpy.array(e.partLikes, copy=True)
    a, pa = no_alloc(lib, e)
    b, pb = no_alloc(lib, e)
    assert abs(a - ref) <= LNL_RTOL * abs(ref), (a, ref)
    numpy.testing.assert_allclose(pa, refParts, rtol=LNL_RTOL)
    assert a == b and numpy.array_equal(pa, pb), (a, b)
    return a


@pytest.fixture(params=golden_files(), ids=golden_ids())
def golden(request, lib):
    return sim.load_problem(request.param)


def test_no_alloc_matches_tree_loglike(lib, golden):
    prob, z = golden
    e = Engine(prob)
    a = check_pair(lib, e)
    ref = float(z["ref_lnL"])
    assert abs(a - ref) <= LNL_RTOL * abs(ref), (a, ref)
    numpy.testing.assert_allclose(e.partLikes, z["ref_partLikes"], rtol=LNL_RTOL)
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


def test_no_alloc_fresh_tree_allocates_nothing(lib):
    """A tree evaluated only through the no-allocation entry point: its own
    device state and its data's device copies are never created, and the
    device's free memory does not drop across a call (after one warm-up call,
    which loads the library's code on the device if nothing did before)."""
    torch = pytest.importorskip("torch")
    prob, z = sim.load_problem([f for f in golden_files() if f.endswith("dna64het_small.npz")][0])
    e = Engine(prob)
    assert device_bytes(lib, e) == (0, 0)
    a, _ = no_alloc(lib, e)
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        b, _ = no_alloc(lib, e)
        assert b == a
    free1, _ = torch.cuda.mem_get_info()
    assert free1 >= free0, (free0, free1)
    assert device_bytes(lib, e) == (0, 0)
    ref = float(z["ref_lnL"])
    assert abs(a - ref) <= LNL_RTOL * abs(ref), (a, ref)
    e.free()


def test_no_alloc_under_memory_pressure(lib):
    """With another allocation holding all but about 512 MiB of the device's
    free memory, a 2 GiB cudaMalloc (through torch) fails while the
    no-allocation evaluation still succeeds with the same result."""
    torch = pytest.importorskip("torch")
    prob, z = sim.load_problem(golden_files()[0])
    e = Engine(prob)
    a0, _ = no_alloc(lib, e)
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    free, _ = torch.cuda.mem_get_info()
    headroom = 512 << 20
    hog = None
    size = free - headroom
    while hog is None and size > (1 << 30):
        try:
            hog = torch.empty(size, dtype=torch.uint8, device="cuda")
        except torch.cuda.OutOfMemoryError:
            size -= 256 << 20
    assert hog is not None
    try:
        with pytest.raises(torch.cuda.OutOfMemoryError):
            torch.empty(2 << 30, dtype=torch.uint8, device="cuda")
        a, _ = no_alloc(lib, e)
        assert a == a0, (a, a0)
        ref = float(z["ref_lnL"])
        assert abs(a - ref) <= LNL_RTOL * abs(ref), (a, ref)
    finally:
        del hog
        torch.cuda.empty_cache()
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
