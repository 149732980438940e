"""p4's func-module entry points for the MCMC and the protein models (p4/func.py)."""
import numpy

from . import mcmcio, pf
from .var import var


def unPickleMcmc(runNum, theData, verbose=True, evaluator="graph"):
    """func.unPickleMcmc (p4/func.py:2144): the latest checkpoint of run
    runNum (mcmc_checkPoint_<runNum>.<gen+1> in the working directory), with
    theData attached, ready for Mcmc.run to continue.  Every chain's lnL is
    recomputed on restart and must agree with the checkpointed value within
    0.01 (p4's check, p4/mcmc.py:3603-3612)."""
    return mcmcio.restore(mcmcio.latest_checkpoint(int(runNum)), theData, evaluator=evaluator, verbose=verbose)


def getProteinEmpiricalModelRMatrix(spec, upperTriangle=True):
    """func.getProteinEmpiricalModelRMatrix (p4/func.py:3708): the 20x20
    exchangeability matrix of an empirical protein model by p4's name (one of
    var.rMatrixProteinSpecs), or its upper triangle as a list, row by row."""
    assert spec in var.rMatrixProteinSpecs, "spec should be one of var.rMatrixProteinSpecs"
    a = numpy.zeros((20, 20), dtype=numpy.double)
    pf.getBigR(var.rMatrixProteinSpecNumberForNameDict[spec], a)
    if upperTriangle:
        return [a[i][j] for i in range(19) for j in range(i + 1, 20)]
    return a
