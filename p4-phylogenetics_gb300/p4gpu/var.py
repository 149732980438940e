"""Global settings, mirroring p4's ``var`` singleton (p4/var.py).

The bounds live in one-element numpy arrays that the C side aliases by
pointer, as in the reference (p4/var.py:287-305).
"""
import numpy


class Var(object):
    def __init__(self):
        self._rMatrixNormalizeTo1 = numpy.array([1], numpy.int32)
        self._PIVEC_MIN = numpy.array([1.0e-13])
        self._PIVEC_MAX = numpy.array([0.999])
        self._RATE_MIN = numpy.array([1.0e-13])
        self._RATE_MAX = numpy.array([0.9999999])
        self._GAMMA_SHAPE_MIN = numpy.array([0.1])
        self._GAMMA_SHAPE_MAX = numpy.array([300.0])
        self._PINVAR_MIN = numpy.array([0.0])
        self._PINVAR_MAX = numpy.array([0.99])
        self._RELRATE_MIN = numpy.array([1.0e-8])
        self._RELRATE_MAX = numpy.array([1.0e8])
        self._KAPPA_MIN = numpy.array([0.000001])
        self._KAPPA_MAX = numpy.array([100.0])
        self._BRLEN_MIN = numpy.array([1.0e-8])
        self._BRLEN_MAX = numpy.array([3.0])
        self._newtAndBrentPowellOptPassLimit = numpy.array([50], numpy.int32)
        self.GAP_CODE = -1
        self.QMARK_CODE = -2
        self.N_LIKE = -3
        self.EQUATES_BASE = -64
        self.NO_ORDER = -10000
        self.doMcmcSp = True
        self.mcmc_swapVector = True
        self.warnReadNoFile = True
        # the empirical protein rate matrices the library carries, by p4's
        # names and spec numbers (p4/var.py:239-262, Pf/defines.h)
        self.rMatrixProteinSpecs = ['cpREV', 'd78', 'jtt', 'mtREV24', 'mtmam', 'wag', 'blosum62',
                                    'rtRev', 'tmjtt94', 'tmlg99', 'lg', 'hivb', 'mtart', 'mtzoa',
                                    'gcpREV', 'stmtREV', 'vt', 'pmb']
        self.rMatrixProteinSpecNumberForNameDict = dict(zip(
            self.rMatrixProteinSpecs,
            [101, 102, 103, 104, 105, 106, 107, 110, 111, 112, 113, 114, 115, 116, 117, 118, 119, 120]))

    def bounds(self):
        """The 14 bound arrays in p4_newModel's argument order (Pf/pfmodule.c:1484)."""
        return [self._PINVAR_MIN, self._PINVAR_MAX, self._KAPPA_MIN, self._KAPPA_MAX,
                self._GAMMA_SHAPE_MIN, self._GAMMA_SHAPE_MAX, self._PIVEC_MIN, self._PIVEC_MAX,
                self._RATE_MIN, self._RATE_MAX, self._RELRATE_MIN, self._RELRATE_MAX,
                self._BRLEN_MIN, self._BRLEN_MAX]

    def _g(name):
        return property(lambda self: self.__dict__["_" + name][0],
                        lambda self, v: self.__dict__["_" + name].__setitem__(0, v))

    PIVEC_MIN = _g("PIVEC_MIN")
    PIVEC_MAX = _g("PIVEC_MAX")
    RATE_MIN = _g("RATE_MIN")
    RATE_MAX = _g("RATE_MAX")
    GAMMA_SHAPE_MIN = _g("GAMMA_SHAPE_MIN")
    GAMMA_SHAPE_MAX = _g("GAMMA_SHAPE_MAX")
    PINVAR_MIN = _g("PINVAR_MIN")
    PINVAR_MAX = _g("PINVAR_MAX")
    RELRATE_MIN = _g("RELRATE_MIN")
    RELRATE_MAX = _g("RELRATE_MAX")
    KAPPA_MIN = _g("KAPPA_MIN")
    KAPPA_MAX = _g("KAPPA_MAX")
    BRLEN_MIN = _g("BRLEN_MIN")
    BRLEN_MAX = _g("BRLEN_MAX")
    rMatrixNormalizeTo1 = _g("rMatrixNormalizeTo1")
    del _g


var = Var()
