"""Extracts the reference's golden vectors for the cc-TPFA hot path into small fixtures.

Run with the DuMux source tree named by the environment variable DUMUX_REFERENCE
(python make_golden.py with DUMUX_REFERENCE=<path to the DuMux tree>); the GPU host has
no such tree, so the extracted values are committed:
  onep_lens_p.txt          cell field "p" of test/references/test_1p_cc-reference.vtu
                           (test_1p_incompressible_tpfa[_numdiff], 10x10 lens, 100 cells)
  pcsw_brookscorey.txt     test/references/test_pcsw_brookscorey-reference.dat
                           (regularised Brooks-Corey pc(sw) at linspace(0,1,100),
                           pe=1e4, lambda=2, Swr=Snr=0.1, pcLowSwe=0.01)
  pcsw_vangenuchten.txt    test/references/test_pcsw_vangenuchten-reference.dat
                           (regularised Van Genuchten pc(sw) at linspace(0,1,100), alpha=6.66e-5,
                           n=3.652, l=0.5, Swr=Snr=0.1, thresholds 0.01/0.99/0.1/0.9;
                           test/material/fluidmatrixinteractions/2p/test_material_2p_vangenuchten.cc)
  twop_lens_tpfa.txt       cell fields S_napl, p_aq, p_napl, pc of
                           test/references/test_2p_incompressible_cc-reference.vtu (48x32 2p
                           Van Genuchten lens, output 7 = t 3000 s; the reference's
                           test_2p_incompressible_tpfa and _tpfa_analytic compare with it)
"""
import os
import re
import sys

REFERENCE = os.environ.get("DUMUX_REFERENCE")
HERE = os.path.dirname(os.path.abspath(__file__))


def main():
    if not REFERENCE:
        sys.exit("set DUMUX_REFERENCE to the DuMux source tree")
    vtu = open(os.path.join(REFERENCE, "test/references/test_1p_cc-reference.vtu")).read()
    m = re.search(r'Name="p"[^>]*>(.*?)</DataArray>', vtu, re.S)
    vals = m.group(1).split()
    assert len(vals) == 100
    with open(os.path.join(HERE, "onep_lens_p.txt"), "w") as f:
        f.write("# cell field p of test/references/test_1p_cc-reference.vtu (Float32, ascii)\n")
        f.write("\n".join(vals) + "\n")
    dat = open(os.path.join(REFERENCE, "test/references/test_pcsw_brookscorey-reference.dat")).read().split()
    assert len(dat) == 100
    with open(os.path.join(HERE, "pcsw_brookscorey.txt"), "w") as f:
        f.write("# test/references/test_pcsw_brookscorey-reference.dat\n")
        f.write("\n".join(dat) + "\n")
    dat = open(os.path.join(REFERENCE, "test/references/test_pcsw_vangenuchten-reference.dat")).read().split()
    assert len(dat) == 100
    with open(os.path.join(HERE, "pcsw_vangenuchten.txt"), "w") as f:
        f.write("# test/references/test_pcsw_vangenuchten-reference.dat\n")
        f.write("\n".join(dat) + "\n")
    vtu = open(os.path.join(REFERENCE, "test/references/test_2p_incompressible_cc-reference.vtu")).read()
    fields = ["S_napl", "p_aq", "p_napl", "pc"]
    cols = []
    for name in fields:
        m = re.search(r'Name="%s"[^>]*>(.*?)</DataArray>' % name, vtu, re.S)
        vals = m.group(1).split()
        assert len(vals) == 1536, (name, len(vals))
        cols.append(vals)
    with open(os.path.join(HERE, "twop_lens_tpfa.txt"), "w") as f:
        f.write("# cell fields of test/references/test_2p_incompressible_cc-reference.vtu (Float32, ascii)\n")
        f.write("# " + " ".join(fields) + "\n")
        for row in zip(*cols):
            f.write(" ".join(row) + "\n")
    print("wrote fixtures to", HERE)


if __name__ == "__main__":
    sys.exit(main())
