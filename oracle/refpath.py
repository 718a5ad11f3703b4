"""Where the reference SPARC source tree lies (test infrastructure only).

One setting for every recipe, fixture script and test that reads the reference sources: the
environment variable SPARC_REFERENCE; without it the read-only checkout of the build
container (/root/reference) when present, else the staged copy under oracle/_ref/stage made by
oracle/ref/stage.py (git-ignored; it travels with the working tree to hosts without the
reference tree). Where neither exists, what needs the sources is skipped; the committed
fixtures under tests/golden stand in for them.
"""
import os

DEFAULT = "/root/reference"
STAGE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_ref", "stage")


def reference_root():
    """The reference tree's root directory (it may not exist on this machine)."""
    env = os.environ.get("SPARC_REFERENCE")
    if env:
        return env
    if os.path.isdir(os.path.join(DEFAULT, "src")):
        return DEFAULT
    if os.path.isdir(os.path.join(STAGE, "src")):
        return STAGE
    return DEFAULT


def reference_present():
    """True when the reference sources are on this machine."""
    return os.path.isdir(os.path.join(reference_root(), "src"))


def psps_dir():
    """The reference's pseudopotential folder."""
    return os.path.join(reference_root(), "psps")
