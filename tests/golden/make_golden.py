"""Extracts the reference's golden vectors for the cc-TPFA hot path into small fixtures.

Run in a container that has the DuMux source tree at REFERENCE (default
/root/reference); the GPU host does not, so the extracted values are committed:
  onep_lens_p.txt          cell field "p" of test/references/test_1p_cc-reference.vtu
                           (test_1p_incompressible_tpfa[_numdiff], 10x10 lens, 100 cells)
  pcsw_brookscorey.txt     test/references/test_pcsw_brookscorey-reference.dat
                           (regularised Brooks-Corey pc(sw) at linspace(0,1,100),
                           pe=1e4, lambda=2, Swr=Snr=0.1, pcLowSwe=0.01)
"""
import os
import re
import sys

REFERENCE = os.environ.get("DUMUX_REFERENCE", "/root/reference")
HERE = os.path.dirname(os.path.abspath(__file__))


def main():
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
    print("wrote fixtures to", HERE)


if __name__ == "__main__":
    sys.exit(main())
