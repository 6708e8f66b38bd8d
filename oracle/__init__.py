"""Test infrastructure only: the oracle (a CPU restatement of the reference's algorithm) and
drivers over the reference's own sources.  The product never imports this package."""
from __future__ import annotations

import os
import subprocess

_HERE = os.path.dirname(os.path.abspath(__file__))


def reference_root() -> str:
    """The reference tree: the REF environment variable, else oracle/Makefile's default --
    the one place that default is written."""
    r = subprocess.run(["make", "-s", "--no-print-directory", "-C", _HERE, "print-ref"],
                       capture_output=True, text=True, check=True)
    return r.stdout.strip()


def reference_present() -> bool:
    return os.path.isdir(os.path.join(reference_root(), "src"))
