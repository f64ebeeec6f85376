"""Install recipe of the reference package for the timed CPU baseline (test infrastructure).

The reference COV3D is pure Python / PyTorch, so "building" it is copying its ``cov3d``
package, unmodified, to ``oracle/_ref/cov3d`` (git-ignored; it travels with the repository
copy to machines that lack the reference tree).  ``oracle/ref_step.py`` imports it from there
through ``oracle/ref_shim.py`` and times the reference's own covariance-SGD step on the host
cores.  Nothing of it is committed.

    python oracle/build_ref.py /path/to/reference
"""

import os
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
PKG = os.path.join(OUT, "cov3d")


def installed():
    return os.path.exists(os.path.join(PKG, "covar_sgd.py"))


def build(reference_root, force=False):
    """Copy ``<reference_root>/cov3d/*.py`` to ``oracle/_ref/cov3d``; returns the package dir,
    or None when the reference tree is absent."""
    src = os.path.join(reference_root, "cov3d")
    if not os.path.isdir(src):
        return PKG if installed() else None
    if installed() and not force:
        newest = max(os.path.getmtime(os.path.join(src, f)) for f in os.listdir(src) if f.endswith(".py"))
        if os.path.getmtime(os.path.join(PKG, "covar_sgd.py")) >= newest:
            return PKG
    os.makedirs(OUT, exist_ok=True)
    if os.path.isdir(PKG):
        shutil.rmtree(PKG)
    shutil.copytree(src, PKG, ignore=shutil.ignore_patterns("__pycache__", "*.pyc"))
    return PKG


if __name__ == "__main__":
    if len(sys.argv) < 2:
        sys.exit("usage: build_ref.py /path/to/reference")
    print(build(sys.argv[1], force=True))
