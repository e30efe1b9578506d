"""ORACLE -- test infrastructure only.

Stages the reference's sources into ``baseline/_ref/src`` (kept out of the repository's history, but copied with the
working tree to the machines that run the tests and the benchmark), so that those machines can compile the
reference's own CPU path (``oracle/Makefile ref``) and its CUDA path (``oracle/Makefile refcuda``) from them.  The reference is only ever read from its checkout here; every other
file takes the staged copy (or ``MRAY_REFERENCE_SRC``).  Nothing is copied into the repository's history.
"""
from __future__ import annotations

import filecmp
import os
import shutil

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
STAGED = os.path.join(ROOT, "baseline", "_ref", "src")
CHECKOUT = "/root/reference/src"


def reference_src() -> str | None:
    """The reference's source directory: MRAY_REFERENCE_SRC, else the staged copy; None when neither exists."""
    env = os.environ.get("MRAY_REFERENCE_SRC")
    if env:
        return env if os.path.isdir(env) else None
    return STAGED if os.path.isdir(STAGED) else None


def _same_tree(a: str, b: str) -> bool:
    cmp = filecmp.dircmp(a, b)
    if cmp.left_only or cmp.right_only or cmp.diff_files or cmp.funny_files:
        return False
    return all(_same_tree(os.path.join(a, d), os.path.join(b, d)) for d in cmp.common_dirs)


def stage() -> str | None:
    """Copy the checkout into baseline/_ref/src when the checkout exists here; returns the staged path."""
    if os.path.isdir(CHECKOUT):
        if not (os.path.isdir(STAGED) and _same_tree(CHECKOUT, STAGED)):
            if os.path.isdir(STAGED):
                shutil.rmtree(STAGED)
            shutil.copytree(CHECKOUT, STAGED)
            lic = os.path.join(os.path.dirname(CHECKOUT), "LICENSE.txt")
            if os.path.exists(lic):
                shutil.copy(lic, os.path.join(os.path.dirname(STAGED), "LICENSE.txt"))
    return STAGED if os.path.isdir(STAGED) else None


if __name__ == "__main__":
    print(stage())
