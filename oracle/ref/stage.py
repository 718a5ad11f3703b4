"""Stage the reference sources next to the oracle build so a machine without the reference
tree (the GPU host) can build the oracle and the accelerated SPARC from them.

Test infrastructure only. Copies <reference>/src and the pseudopotentials the test systems use
into oracle/_ref/stage/, which git ignores (the copy is never committed) and which travels with
the working tree to the GPU host. oracle/refpath.py finds the staged copy when the reference
tree itself is absent.

usage: python oracle/ref/stage.py [--ref /path/to/SPARC]
"""
import argparse
import os
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", ".."))

from oracle.refpath import STAGE, reference_root  # noqa: E402

PSPS = ("14_Si_4_1.9_1.9_pbe_n_v1.0.psp8", "13_Al_3_1.9_1.9_pbe_n_v1.0.psp8")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=reference_root(),
                    help="reference tree (default: $SPARC_REFERENCE, else /root/reference)")
    args = ap.parse_args()
    src = os.path.join(args.ref, "src")
    if not os.path.isdir(src):
        raise SystemExit(f"no reference sources under {args.ref}")
    if os.path.abspath(args.ref) == os.path.abspath(STAGE):
        raise SystemExit("the reference given is the staged copy itself")
    if os.path.isdir(STAGE):
        shutil.rmtree(STAGE)
    shutil.copytree(src, os.path.join(STAGE, "src"),
                    ignore=shutil.ignore_patterns("*.o", "*.a", "*.so", "sparc"))
    os.makedirs(os.path.join(STAGE, "psps"))
    for fn in PSPS:
        shutil.copy2(os.path.join(args.ref, "psps", fn), os.path.join(STAGE, "psps", fn))
    print("staged", STAGE)


if __name__ == "__main__":
    main()
