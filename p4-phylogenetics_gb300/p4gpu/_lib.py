"""ctypes binding of libp4gpu.so (the C ABI declared in include/p4gpu.h).

The library is the only compute path: if it is not built, importing this
module raises, and nothing falls back to a CPU implementation.
"""
import ctypes
import os

from .p4exceptions import P4Error

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libp4gpu.so")

c_int, c_double, c_void_p, c_char_p = ctypes.c_int, ctypes.c_double, ctypes.c_void_p, ctypes.c_char_p
P_int = ctypes.POINTER(ctypes.c_int)
P_double = ctypes.POINTER(ctypes.c_double)
P_float = ctypes.POINTER(ctypes.c_float)
P_uint = ctypes.POINTER(ctypes.c_uint)
P_uchar = ctypes.POINTER(ctypes.c_ubyte)

STATUS = {0: "P4G_OK", 1: "P4G_EINVAL", 2: "P4G_ENOMEM", 3: "P4G_ECUDA", 4: "P4G_ENONPOS",
          5: "P4G_ETIMEOUT", 6: "P4G_ESTATE", 7: "P4G_EUNSUPPORTED", 8: "P4G_ENUMERIC"}

# name -> (restype, argtypes); restype None means int status
_SIGS = {
    "p4g_lastError": (c_char_p, []),
    "p4g_version": (c_char_p, []),
    "p4g_init": (None, [c_int]),
    "p4g_setStream": (None, [c_void_p]),
    "p4g_getStream": (c_void_p, []),
    "p4g_newData": (c_void_p, [c_int, c_int]),
    "p4g_freeData": (None, [c_void_p]),
    "p4g_pokePartInData": (None, [c_void_p, c_void_p, c_int]),
    "p4g_newPart": (c_void_p, [c_int, c_int, c_char_p, c_int, c_char_p, c_int]),
    "p4g_freePart": (None, [c_void_p]),
    "p4g_pokeEquatesTable": (None, [c_void_p, c_char_p]),
    "p4g_pokeSequences": (None, [c_void_p, c_char_p]),
    "p4g_makePatterns": (None, [c_void_p]),
    "p4g_partPatternCount": (None, [c_void_p, P_int]),
    "p4g_setGlobalInvarSitesVec": (None, [c_void_p]),
    "p4g_getPatterns": (None, [c_void_p, P_int, P_int, P_int]),
    "p4g_getInvarSites": (None, [c_void_p, P_int, P_int]),
    "p4g_getSiteLikes": (None, [c_void_p, P_double]),
    "p4g_newModel": (c_void_p, [c_int, c_int, c_int, c_int, c_int, P_int] + [P_double] * 14),
    "p4g_freeModel": (None, [c_void_p]),
    "p4g_newModelPart": (None, [c_void_p, c_int, c_int, c_int, c_int, c_int, c_int, c_int, P_int]),
    "p4g_newComp": (None, [c_void_p, c_int, c_int, c_int, P_double]),
    "p4g_newRMatrix": (None, [c_void_p, c_int, c_int, c_int, c_int]),
    "p4g_getBigR": (None, [c_int, P_double]),
    "p4g_newGdasrv": (c_void_p, [c_void_p, c_int, c_int, c_int, c_int, P_double, P_double, P_double]),
    "p4g_gdasrvCalcRates": (None, [c_void_p]),
    "p4g_gdasrvCalcRates_np": (None, [c_int, c_double, P_double, P_double]),
    "p4g_setRMatrixBigR": (None, [c_void_p, c_int, c_int, c_int, c_int, c_double]),
    "p4g_setKappa": (None, [c_void_p, c_int, c_int, c_double]),
    "p4g_setPInvarVal": (None, [c_void_p, c_int, c_double]),
    "p4g_setRelRateVal": (None, [c_void_p, c_int, c_double]),
    "p4g_newTree": (c_void_p, [c_int, c_int, P_int, P_int, P_int, P_double, c_void_p, c_void_p]),
    "p4g_freeTree": (None, [c_void_p]),
    "p4g_newNode": (c_void_p, [c_int, c_void_p, c_int, c_int, c_int]),
    "p4g_setNodeRelation": (None, [c_void_p, c_int, c_int]),
    "p4g_setTreeRoot": (None, [c_void_p, c_void_p]),
    "p4g_setBrLen": (None, [c_void_p, c_double]),
    "p4g_setCompNum": (None, [c_void_p, c_int, c_int]),
    "p4g_setRMatrixNum": (None, [c_void_p, c_int, c_int]),
    "p4g_setGdasrvNum": (None, [c_void_p, c_int, c_int]),
    "p4g_setPrams": (None, [c_void_p, c_int]),
    "p4g_treeLogLike": (None, [c_void_p, c_int, P_double]),
    "p4g_partLogLike": (None, [c_void_p, c_void_p, c_int, c_int, P_double]),
    "p4g_treeLogLikeNoAlloc": (None, [c_void_p, P_double]),
    "p4g_makePatternsDevice": (None, [c_void_p]),
    "p4g_getSiteRates": (None, [c_void_p, c_void_p, c_int, P_double, P_int]),
    "p4g_symbolSequences": (None, [c_void_p, ctypes.c_char_p]),
    "p4g_newtSetup": (None, [c_void_p]),
    "p4g_newtAround": (None, [c_void_p, c_double, c_double]),
    "p4g_newtAndBrentPowellOpt": (None, [c_void_p]),
    "p4g_getBrLens": (None, [c_void_p, P_double]),
    "p4g_drawAncStates": (None, [c_void_p, c_int, P_double, ctypes.c_ulonglong, P_int]),
    "p4g_simulate": (None, [c_void_p, P_double, ctypes.c_longlong, ctypes.c_ulonglong, ctypes.c_void_p]),
    "p4g_simulateRef": (None, [c_void_p, c_void_p, P_double, ctypes.c_ulonglong, P_double, ctypes.c_longlong,
                               ctypes.c_ulonglong, ctypes.c_void_p]),
    "p4g_tensorSelfTest": (None, [c_int, P_double]),
    "p4g_calculateBigPDecks": (None, [c_void_p]),
    "p4g_calculateAllBigPDecksAllParts": (None, [c_void_p]),
    "p4g_copyModelPrams": (None, [c_void_p, c_void_p]),
    "p4g_copyBigPDecks": (None, [c_void_p, c_void_p, c_int]),
    "p4g_copyCondLikes": (None, [c_void_p, c_void_p, c_int]),
    "p4g_treeLogLikeBatch": (None, [ctypes.POINTER(c_void_p), c_int, c_int, P_double]),
    "p4g_setPrecision": (None, [c_void_p, c_int]),
    "p4g_setBrLens": (None, [c_void_p, P_double]),
    "p4g_setAutotune": (None, [c_int]),
    "p4g_newBatch": (c_void_p, [ctypes.POINTER(c_void_p), c_int]),
    "p4g_freeBatch": (None, [c_void_p]),
    "p4g_batchSetGraph": (None, [c_void_p, c_int]),
    "p4g_batchSetClades": (None, [c_void_p, c_int]),
    "p4g_batchLogLike": (None, [c_void_p, P_double]),
    "p4g_getPruneShape": (None, [c_void_p, c_int, P_int, P_int]),
    "p4g_setPruneShape": (None, [c_void_p, c_int, c_int]),
    "p4g_setCladeSize": (None, [c_void_p, c_int]),
    "p4g_setGraphs": (None, [c_void_p, c_int]),
    "p4g_setCladeShape": (None, [c_void_p, c_int, c_int]),
    "p4g_setTopology": (None, [c_void_p, P_int, P_int, P_int, c_int]),
    "p4g_setRMatrixUpper": (None, [c_void_p, c_int, c_int, P_double]),
    "p4g_treeLogLikeAsync": (None, [c_void_p, c_int]),
    "p4g_treeLogLikeWait": (None, [c_void_p, P_double]),
    "p4g_treeInfo": (None, [c_void_p, ctypes.POINTER(ctypes.c_longlong)]),
    "p4g_setProgrammaticLaunch": (None, [c_int]),
    "p4g_getFreePrams": (None, [c_void_p, P_double, c_int, P_int]),
    "p4g_fp32FmaPeak": (None, [c_int, P_double, P_double]),
    "p4g_treeDeviceBytes": (None, [c_void_p, ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_longlong)]),
    "p4g_mlpNew": (c_void_p, [c_int, c_int, c_int, c_int, ctypes.c_ulonglong]),
    "p4g_mlpFree": (None, [c_void_p]),
    "p4g_mlpNumParams": (None, [c_void_p, P_int]),
    "p4g_mlpGetParams": (None, [c_void_p, P_float]),
    "p4g_mlpSetParams": (None, [c_void_p, P_float]),
    "p4g_mlpForward": (None, [c_void_p, P_float, c_int, P_float]),
    "p4g_mlpGradients": (None, [c_void_p, P_float, P_float, c_int, P_float, P_float]),
    "p4g_mlpTrainStep": (None, [c_void_p, P_float, P_float, c_int, ctypes.c_float, P_float]),
    "p4g_getPDeck": (None, [c_void_p, c_int, c_int, P_double]),
    "p4g_getDecks32": (None, [c_void_p, c_int, P_float, P_float, P_int]),
    "p4g_getCompactCodes": (None, [c_void_p, P_uchar, P_uint]),
    "p4g_getPatternLikes": (None, [c_void_p, c_int, P_float, P_int, P_double]),
    "p4g_getGammaRates": (None, [c_void_p, c_int, c_int, P_double]),
}

_lib = None


def load(path=None):
    """Load libp4gpu.so; raise if it is missing (build() must run first)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise ImportError("libp4gpu.so is not built (%s); run __graft_entry__.build() or "
                          "python p4-phylogenetics_gb300/build.py" % path)
    lib = ctypes.CDLL(path)
    for name, (res, args) in _SIGS.items():
        f = getattr(lib, name)
        f.restype = res if res is not None else c_int
        f.argtypes = args
    _lib = lib
    return lib


def exported_symbols():
    return list(_SIGS)


def last_error():
    return (load().p4g_lastError() or b"").decode(errors="replace")


def check(rc, what=""):
    if rc != 0:
        raise P4Error("%s failed: %s: %s" % (what, STATUS.get(rc, rc), last_error()))


def handle(ptr, what=""):
    if not ptr:
        raise P4Error("%s failed: %s" % (what, last_error()))
    return ptr


def dptr(a):
    return a.ctypes.data_as(P_double)


def iptr(a):
    return a.ctypes.data_as(P_int)


def fptr(a):
    return a.ctypes.data_as(P_float)


def uptr(a):
    return a.ctypes.data_as(P_uint)


def ucptr(a):
    return a.ctypes.data_as(P_uchar)
