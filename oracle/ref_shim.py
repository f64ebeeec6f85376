"""Import shim that lets the reference COV3D package (pure Python / PyTorch) import on a
machine without its heavy third-party dependencies.

Test infrastructure only.  Used by ``tests/golden/make_golden.py`` (fixtures from the
reference run in float64) and by ``oracle/ref_step.py``, the timed CPU baseline of
``bench.py`` that runs the reference's own torch step from the copy ``oracle/build_ref.py``
makes under ``oracle/_ref/``.  The product package never imports it.

What it does:

* serves placeholder modules for packages that the reference imports at module scope
  but that the discretized hot path never calls (ASPIRE, cuFINUFFT/FINUFFT, cryoDRGN,
  mrcfile, pandas, starfile, colorlog, matplotlib, umap, seaborn, recovar; tqdm and
  scikit-learn only where they are not installed, tqdm as a pass-through progress bar);
* restates ``aspire.utils.grid_2d`` / ``grid_3d`` from their mathematical definition
  (normalised grid ``ceil(arange(-n/2, n/2)) / (n/2)``), because ``poses.py:197-215``,
  ``fsc_utils.py:43-47`` and ``mean.py:412-414`` do call them.
"""

import importlib.abc
import importlib.machinery
import sys
import types

import numpy as np

STUB_ROOTS = {
    "aspire",
    "cufinufft",
    "finufft",
    "cryodrgn",
    "mrcfile",
    "pandas",
    "starfile",
    "colorlog",
    "matplotlib",
    "umap",
    "seaborn",
    "recovar",
}


def _grid_1d_values(n, shifted, normalized, dtype):
    grid = np.ceil(np.arange(-n / 2, n / 2, dtype=dtype))
    if shifted and n % 2 == 0:
        grid = np.arange(-n / 2 + 1 / 2, n / 2 + 1 / 2, dtype=dtype)
    if normalized:
        if shifted and n % 2 == 0:
            grid = grid / (n / 2 - 1 / 2)
        else:
            grid = grid / (n / 2)
    return grid.astype(dtype)


def grid_2d(n, shifted=False, normalized=True, indexing="yx", dtype=np.float32):
    g = _grid_1d_values(n, shifted, normalized, dtype)
    a, b = np.meshgrid(g, g, indexing="ij")
    if indexing == "yx":
        y, x = a, b
    else:
        x, y = a, b
    r = np.sqrt(x * x + y * y)
    phi = np.arctan2(y, x)
    return {"x": x, "y": y, "r": r, "phi": phi}


def grid_3d(n, shifted=False, normalized=True, indexing="zyx", dtype=np.float32):
    g = _grid_1d_values(n, shifted, normalized, dtype)
    a, b, c = np.meshgrid(g, g, g, indexing="ij")
    if indexing == "zyx":
        z, y, x = a, b, c
    else:
        x, y, z = a, b, c
    r = np.sqrt(x * x + y * y + z * z)
    phi = np.arctan2(y, x)
    theta = np.arccos(np.divide(z, r, out=np.zeros_like(r), where=r > 0))
    return {"x": x, "y": y, "z": z, "r": r, "phi": phi, "theta": theta}


class _PlaceholderMeta(type):
    """Attribute access on a placeholder class (``plt.figure`` after ``from matplotlib import
    pyplot as plt``) yields another placeholder."""

    def __getattr__(cls, name):
        if name.startswith("__"):
            raise AttributeError(name)
        return _Placeholder()


class _Placeholder(metaclass=_PlaceholderMeta):
    """Stands in for any class or function of a missing package."""

    def __init__(self, *args, **kwargs):
        pass

    def __call__(self, *args, **kwargs):
        return _Placeholder()

    def __getattr__(self, name):
        return _Placeholder()

    def __class_getitem__(cls, item):
        return cls


class _StubModule(types.ModuleType):
    def __getattr__(self, name):
        if name.startswith("__"):
            raise AttributeError(name)
        placeholder = type(name, (_Placeholder,), {})
        setattr(self, name, placeholder)
        return placeholder


class _StubLoader(importlib.abc.Loader):
    def create_module(self, spec):
        mod = _StubModule(spec.name)
        mod.__path__ = []
        return mod

    def exec_module(self, module):
        if module.__name__ == "aspire.utils":
            module.grid_2d = grid_2d
            module.grid_3d = grid_3d
        if module.__name__ == "tqdm":
            module.tqdm = _Progress


class _StubFinder(importlib.abc.MetaPathFinder):
    def find_spec(self, fullname, path, target=None):
        if fullname.split(".")[0] in STUB_ROOTS:
            return importlib.machinery.ModuleSpec(fullname, _StubLoader(), is_package=True)
        return None


class _Progress:
    """Stand-in for ``tqdm.tqdm`` where tqdm is not installed: iterates what it wraps and
    ignores progress updates."""

    def __init__(self, iterable=None, *args, **kwargs):
        self.iterable = iterable

    def __iter__(self):
        return iter(self.iterable if self.iterable is not None else ())

    def update(self, *args, **kwargs):
        pass

    def set_description(self, *args, **kwargs):
        pass

    def close(self):
        pass


# optional packages the reference imports at module scope and the timed / fixture paths do
# not need: stubbed only where they are not installed (the GPU machines lack them)
OPTIONAL_ROOTS = {"tqdm", "sklearn"}


def _installed(name):
    import importlib.util

    return importlib.util.find_spec(name) is not None


def install(reference_root):
    """Put the stub finder first on ``sys.meta_path`` and the reference on ``sys.path``."""
    for name in OPTIONAL_ROOTS:
        if name not in STUB_ROOTS and not _installed(name):
            STUB_ROOTS.add(name)
    if not any(isinstance(f, _StubFinder) for f in sys.meta_path):
        sys.meta_path.insert(0, _StubFinder())
    if reference_root not in sys.path:
        sys.path.insert(0, reference_root)
