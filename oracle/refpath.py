"""Where the recipes under oracle/ find the reference tree they compile from.

The BBPP_REFERENCE environment variable names it; without it the recipes look
at the read-only checkout of the build container.  The GPU machine has no
reference tree: there the recipes are skipped and the artefacts they built
(oracle/_ref) are used as they are.  Test infrastructure only.
"""
import os

CONTAINER_CHECKOUT = "/root/reference"


def tree():
    """The reference tree's root directory."""
    return os.environ.get("BBPP_REFERENCE") or CONTAINER_CHECKOUT


def src():
    return os.path.join(tree(), "src")


def present():
    """True when the reference sources the recipes need are readable here."""
    return os.path.isfile(os.path.join(src(), "solver_kernel.cu"))
