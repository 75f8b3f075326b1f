"""Generate ``dop853_tableau.h``: the Dormand-Prince 8(5,3) Butcher tableau as C macros.

The coefficients are the published DOP853 table of Hairer, Norsett & Wanner
("Solving Ordinary Differential Equations I", 2nd ed., sec. II.10; the dop853
code of Hairer & Wanner).  SciPy ships the same table as decimal literals in
``scipy/integrate/_ivp/dop853_coefficients.py`` (BSD licence); this script reads
that module's *values* (and, for the three ``bhh`` embedded-3rd-order weights
that SciPy only stores folded into ``E3``, the literal text of those lines) and
writes them out with ``repr`` so every double round-trips exactly.

Both the CUDA kernels and the CPU oracle include the generated header, so the
two sides use bit-identical constants.  Run:

    python numbacs_gb300/csrc/gen_dop853_tableau.py > numbacs_gb300/csrc/dop853_tableau.h
"""
import ast
import inspect
import sys

import scipy.integrate._ivp.dop853_coefficients as dc


def _bhh_literals():
    """Return the three literals subtracted from E3 (bhh1, bhh2, bhh3)."""
    tree = ast.parse(inspect.getsource(dc))
    vals = {}
    for node in ast.walk(tree):
        if (isinstance(node, ast.AugAssign) and isinstance(node.op, ast.Sub)
                and isinstance(node.target, ast.Subscript)
                and isinstance(node.target.value, ast.Name) and node.target.value.id == "E3"):
            idx = ast.literal_eval(node.target.slice)
            vals[idx] = float(ast.literal_eval(node.value))
    return vals[0], vals[8], vals[11]


def main(out=sys.stdout):
    A, B, C, E5 = dc.A, dc.B, dc.C, dc.E5
    bhh1, bhh2, bhh3 = _bhh_literals()
    w = out.write
    w("/* Generated by gen_dop853_tableau.py -- do not edit.\n")
    w(" * Dormand-Prince 8(5,3) tableau (Hairer, Norsett & Wanner, dop853).\n")
    w(" * Stage numbering is 1-based as in the published table: stage s uses\n")
    w(" * DP853_A_s_j (j < s) and time offset DP853_C_s; B_j are the 8th-order\n")
    w(" * weights, E5_j the 5th-order error weights, BHH1..3 the 3rd-order ones. */\n")
    w("#ifndef NBCS_DOP853_TABLEAU_H\n#define NBCS_DOP853_TABLEAU_H\n\n")
    for s in range(2, 13):
        w("#define DP853_C_%d (%r)\n" % (s, float(C[s - 1])))
    w("\n")
    for s in range(2, 13):
        for j in range(1, s):
            w("#define DP853_A_%d_%d (%r)\n" % (s, j, float(A[s - 1, j - 1])))
    w("\n")
    for j in range(1, 13):
        w("#define DP853_B_%d (%r)\n" % (j, float(B[j - 1])))
    w("\n")
    for j in range(1, 13):
        w("#define DP853_E5_%d (%r)\n" % (j, float(E5[j - 1])))
    w("\n#define DP853_BHH1 (%r)\n#define DP853_BHH2 (%r)\n#define DP853_BHH3 (%r)\n"
      % (bhh1, bhh2, bhh3))
    # dense output (the dop853 code's contd8): stage 13 is the derivative at
    # the step's end, stages 14..16 the three extra stages (DP853_A_s_j,
    # DP853_C_s), and DP853_D_r_j (r = 4..7, as the code's d4j..d7j) the
    # weights of the interpolant's coefficients 4..7 over stages j = 1..16
    w("\n")
    for s in range(14, 17):
        w("#define DP853_C_%d (%r)\n" % (s, float(C[s - 1])))
        for j in range(1, s):
            w("#define DP853_A_%d_%d (%r)\n" % (s, j, float(A[s - 1, j - 1])))
    for r in range(4, 8):
        for j in range(1, 17):
            w("#define DP853_D_%d_%d (%r)\n" % (r, j, float(dc.D[r - 4, j - 1])))
    w("\n#endif /* NBCS_DOP853_TABLEAU_H */\n")


if __name__ == "__main__":
    main()
