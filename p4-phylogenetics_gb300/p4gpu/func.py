"""p4's func-module entry points for the MCMC (p4/func.py)."""
from . import mcmcio


def unPickleMcmc(runNum, theData, verbose=True, evaluator="graph"):
    """func.unPickleMcmc (p4/func.py:2144): the latest checkpoint of run
    runNum (mcmc_checkPoint_<runNum>.<gen+1> in the working directory), with
    theData attached, ready for Mcmc.run to continue.  Every chain's lnL is
    recomputed on restart and must agree with the checkpointed value within
    0.01 (p4's check, p4/mcmc.py:3603-3612)."""
    return mcmcio.restore(mcmcio.latest_checkpoint(int(runNum)), theData, evaluator=evaluator, verbose=verbose)
