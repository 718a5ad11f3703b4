"""Where the reference SPARC source tree lies (test infrastructure only).

One setting for every recipe, fixture script and test that reads the reference sources: the
environment variable SPARC_REFERENCE, default /root/reference (the read-only checkout of the
build container). Machines without the tree (the GPU host) simply see it missing, and what
needs it is skipped there; the committed fixtures under tests/golden stand in for it.
"""
import os

DEFAULT = "/root/reference"


def reference_root():
    """The reference tree's root directory (it may not exist on this machine)."""
    return os.environ.get("SPARC_REFERENCE", DEFAULT)


def reference_present():
    """True when the reference sources are on this machine."""
    return os.path.isdir(os.path.join(reference_root(), "src"))


def psps_dir():
    """The reference's pseudopotential folder."""
    return os.path.join(reference_root(), "psps")
