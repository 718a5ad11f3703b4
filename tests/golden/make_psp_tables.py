"""Write the radial tables of the pseudopotentials used by the test systems to small .npz
fixtures (tests/golden/psp_<El>.npz), read with the library's own psp8 reader
(sparc_gb300/psp8.py), so that set-up runs where the .psp8 files are not available.

usage: python tests/golden/make_psp_tables.py [--ref /path/to/SPARC]
"""
import argparse
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", ".."))

from oracle.refpath import reference_root  # noqa: E402
from sparc_gb300.psp8 import read_psp8, save_tables  # noqa: E402

FILES = {"Si": "14_Si_4_1.9_1.9_pbe_n_v1.0.psp8", "Al": "13_Al_3_1.9_1.9_pbe_n_v1.0.psp8",
         "C": "06_C_4_1.2_1.2_pbe_n_v1.0.psp8"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=reference_root(),
                    help="reference tree (default: $SPARC_REFERENCE, else /root/reference)")
    args = ap.parse_args()
    for el, fn in FILES.items():
        tab = read_psp8(os.path.join(args.ref, "psps", fn), el)
        out = os.path.join(HERE, f"psp_{el}.npz")
        save_tables(tab, out)
        print("wrote", out, os.path.getsize(out), "bytes")


if __name__ == "__main__":
    main()
