"""Test infrastructure only: the oracle (a CPU restatement of the reference's algorithm) and
drivers over the reference's own sources.  The product never imports this package."""
from __future__ import annotations

import os
import subprocess

_HERE = os.path.dirname(os.path.abspath(__file__))
STAGE = os.path.join(_HERE, "_ref", "stage")


def _default_root() -> str:
    r = subprocess.run(["make", "-s", "--no-print-directory", "-C", _HERE, "print-ref"],
                       capture_output=True, text=True, check=True)
    return r.stdout.strip()


def reference_root() -> str:
    """The reference tree: the REF environment variable, else oracle/Makefile's default (the one
    place that default is written); where neither exists, the copy `make -C oracle stage` left in
    oracle/_ref/stage (git-ignored; it travels with the working tree to the GPU host)."""
    r = _default_root()
    if not os.path.isdir(os.path.join(r, "src")) and os.path.isdir(os.path.join(STAGE, "src")):
        return STAGE
    return r


def reference_present() -> bool:
    return os.path.isdir(os.path.join(reference_root(), "src"))


def make_args() -> list[str]:
    """the REF= argument for oracle/Makefile targets that build from the reference"""
    return ["REF=" + reference_root()]
