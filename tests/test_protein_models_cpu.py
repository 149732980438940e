"""The library's empirical protein rate matrices (p4g_newRMatrix with specs
101-120, p4g_getBigR) against the reference's own: the compiled reference
core fills each matrix with its p4_newRMatrix (Pf/p4_model.c:345-450), and
every one of the 400 values must be identical.  Host-only: no GPU."""
import numpy
import pytest

from p4gpu import P4Error, func, pf, var

SPECS = [101, 102, 103, 104, 105, 106, 107, 110, 111, 112, 113, 114, 115, 116, 117, 118, 119, 120]


@pytest.fixture(scope="module")
def ref():
    from oracle import oracle
    if not oracle.have_ref():
        pytest.skip("reference core not built")
    return oracle


def test_tables_equal_reference(lib, ref):
    for spec in SPECS:
        a = numpy.zeros((20, 20), numpy.double)
        pf.getBigR(spec, a)
        b = ref.ref_bigR(spec)
        assert numpy.array_equal(a, b), spec
        off = ~numpy.eye(20, dtype=bool)
        assert numpy.array_equal(a[off], a.T[off]), spec   # symmetric off the diagonal
        assert (a[off] >= 0).all() and a.max() > 0, spec


def test_names_cover_the_table(lib):
    assert sorted(var.rMatrixProteinSpecNumberForNameDict.values()) == SPECS
    up = func.getProteinEmpiricalModelRMatrix("wag")
    full = func.getProteinEmpiricalModelRMatrix("wag", upperTriangle=False)
    assert len(up) == 190
    assert up == [full[i][j] for i in range(19) for j in range(i + 1, 20)]


def test_other_specs_refused(lib):
    a = numpy.zeros((20, 20), numpy.double)
    for spec in (0, 1, 5, 20, 100, 108, 109, 121):
        with pytest.raises(P4Error):
            pf.getBigR(spec, a)


def test_empirical_spec_needs_twenty_states(lib):
    m = pf.p4_newModel(1, 0, 0, 0, 1, var._rMatrixNormalizeTo1, *var.bounds())
    bq = numpy.ones((1, 1), numpy.int32)
    pf.p4_newModelPart(m, 0, 4, 1, 1, 0, 1, 0, bq)
    with pytest.raises(P4Error):
        pf.p4_newRMatrix(m, 0, 0, 0, 106)
    pf.p4_freeModel(m)
