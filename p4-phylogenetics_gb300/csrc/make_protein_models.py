"""Write p4g_protein_models.inc: the exchangeabilities of the empirical
protein rate matrices p4 ships, as the library's table.

    python make_protein_models.py [PF_DIR]

PF_DIR is p4's Pf source directory (default $P4_REFERENCE_PF).  The values
are read from its Pf/proteinModels.c (one function per matrix, every entry
r[i][j] of the 20x20 matrix assigned once; text inside comments is
ignored, so the commented-out PAML variant of mtArt is not taken) and the
spec numbers from Pf/defines.h, mapped as p4_newRMatrix maps them
(Pf/p4_model.c:366-430).  These are published data (cpREV, Dayhoff 78, JTT,
mtREV24, mtMam, WAG, BLOSUM62, rtREV, tmJTT94, tmLG99, LG, HIVb, mtArt,
mtZoa, gcpREV, stmtREV, VT, PMB) that must be identical to p4's for the
likelihoods to be.  The script checks that each matrix is complete, records
whether it is symmetric off the diagonal (all of p4's are; its stmtREV table
has a nonzero diagonal, which Q does not use), and writes every value with
enough digits to give back the same double.  tests/test_protein_models_cpu.py
compares the compiled table with the matrices of the compiled reference.
"""
import os
import re
import sys

# function in Pf/proteinModels.c -> spec constant in Pf/defines.h, in the
# order p4_newRMatrix tests them
MATRICES = [
    ("cpREVRMatrix", "RMATRIX_CPREV"), ("d78RMatrix", "RMATRIX_D78"), ("jttRMatrix", "RMATRIX_JTT"),
    ("mtREV24RMatrix", "RMATRIX_MTREV24"), ("mtmamRMatrix", "RMATRIX_MTMAM"), ("wagRMatrix", "RMATRIX_WAG"),
    ("rtRevRMatrix", "RMATRIX_RTREV"), ("tmjtt94RMatrix", "RMATRIX_TMJTT94"),
    ("tmlg99RMatrix", "RMATRIX_TMLG99"), ("lgRMatrix", "RMATRIX_LG"),
    ("blosum62RMatrix", "RMATRIX_BLOSUM62_A"), ("hivbRMatrix", "RMATRIX_HIVB"),
    ("mtartRMatrix", "RMATRIX_MTART"), ("mtzoaRMatrix", "RMATRIX_MTZOA"),
    ("gcpREVRMatrix", "RMATRIX_GCPREV"), ("stmtREVRMatrix", "RMATRIX_STMTREV"),
    ("vtRMatrix", "RMATRIX_VT"), ("pmbRMatrix", "RMATRIX_PMB"),
]
DIM = 20


def strip_comments(text):
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    return re.sub(r"//[^\n]*", " ", text)


def spec_numbers(defines):
    out = {}
    for m in re.finditer(r"#define\s+(RMATRIX_\w+)\s+(\d+)", strip_comments(defines)):
        out[m.group(1)] = int(m.group(2))
    return out


def matrices(source):
    src = strip_comments(source)
    out = {}
    for m in re.finditer(r"void\s+(\w+)\s*\(\s*double\s*\*\*\s*r\s*\)\s*\{(.*?)\n\}", src, flags=re.S):
        name, body = m.group(1), m.group(2)
        if name in out:
            raise SystemExit("%s defined twice outside comments" % name)
        r = [[None] * DIM for _ in range(DIM)]
        for a in re.finditer(r"r\[\s*(\d+)\]\[\s*(\d+)\]\s*=\s*([-+0-9.eE]+)\s*;", body):
            i, j = int(a.group(1)), int(a.group(2))
            if r[i][j] is not None:
                raise SystemExit("%s: r[%d][%d] assigned twice" % (name, i, j))
            r[i][j] = float(a.group(3))
        out[name] = r
    return out


def check(name, r):
    """Every entry assigned; returns whether the off-diagonal part is symmetric."""
    sym = True
    for i in range(DIM):
        for j in range(DIM):
            if r[i][j] is None:
                raise SystemExit("%s: r[%d][%d] not assigned" % (name, i, j))
            if i != j and r[i][j] != r[j][i]:
                sym = False
    return sym


def main():
    pf = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("P4_REFERENCE_PF")
    if not pf:
        raise SystemExit("usage: make_protein_models.py PF_DIR (or set P4_REFERENCE_PF)")
    specs = spec_numbers(open(os.path.join(pf, "defines.h")).read())
    mats = matrices(open(os.path.join(pf, "proteinModels.c")).read())
    syms = [check(fn, mats[fn]) for fn, _ in MATRICES]
    lines = ["// Generated by make_protein_models.py from p4's Pf/proteinModels.c and",
             "// Pf/defines.h: the 20x20 exchangeability matrices (row-major, as p4 fills",
             "// them) of the empirical protein models p4 ships, by spec number, and",
             "// whether each is symmetric off the diagonal.  Do not edit.",
             "static const int kProteinSpecs[%d] = {%s};" % (len(MATRICES),
                                                            ", ".join(str(specs[s]) for _, s in MATRICES)),
             "static const int kProteinSymmetric[%d] = {%s};" % (len(MATRICES), ", ".join(str(int(x)) for x in syms)),
             "static const double kProteinR[%d][%d] = {" % (len(MATRICES), DIM * DIM)]
    for fn, sp in MATRICES:
        r = mats[fn]
        vals = [repr(r[i][j]) for i in range(DIM) for j in range(DIM)]
        lines.append("    // %s (%s = %d)" % (fn, sp, specs[sp]))
        lines.append("    {")
        for k in range(0, len(vals), DIM):
            lines.append("        " + ", ".join(vals[k:k + DIM]) + ",")
        lines.append("    },")
    lines.append("};")
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "p4g_protein_models.inc")
    with open(out, "w") as f:
        f.write("\n".join(lines) + "\n")
    print("wrote %s (%d matrices)" % (out, len(MATRICES)))


if __name__ == "__main__":
    main()
