"""Import the HermesPy reference package from a source checkout with stub modules.

The reference's hot path (fading channel, OFDM waveform, LS estimation, QAM
mapping, BER evaluation) is pure numpy/scipy, but its package imports a few
heavy optional dependencies at module level (``sparse``, ``numba``, ``ray``,
``h5py``, ``matplotlib``). This helper installs minimal stand-ins for them so
that ``hermespy.modem``, ``hermespy.channel`` and ``hermespy.simulation``
import, then puts the checkout on ``sys.path``.

Only the fixture generator and the optional reference-cross-check tests use
this module; it is never imported by the engine.
"""

from __future__ import annotations

import os
import sys
import types
from unittest.mock import MagicMock

import numpy as np

ENV = "HERMESPY_REFERENCE"


def reference_path(path: str | None = None) -> str:
    """The checkout to import: ``path`` if given, else the ``HERMESPY_REFERENCE``
    environment variable; raises with a usage hint when neither is set."""

    path = path or os.environ.get(ENV)
    if not path:
        raise SystemExit(f"no HermesPy checkout given: pass its path or set {ENV}=<path to the source tree>")
    return path


class _DenseSparse(np.ndarray):
    """Dense stand-in for ``sparse.GCXS`` / ``sparse.COO`` arrays."""

    @classmethod
    def from_numpy(cls, array, *args, **kwargs):  # noqa: D401 - mirrors sparse API
        return np.asarray(array).view(cls)

    def todense(self):
        return np.asarray(self)

    @property
    def nnz(self):
        return int(np.count_nonzero(np.asarray(self)))


def _install_stubs() -> None:
    if "sparse" not in sys.modules:
        sparse = types.ModuleType("sparse")
        sparse.GCXS = _DenseSparse
        sparse.COO = _DenseSparse
        sparse.SparseArray = _DenseSparse

        def _asnumpy(a, *args, **kwargs):
            return np.asarray(a)

        sparse.asnumpy = _asnumpy
        sparse.einsum = np.einsum
        sys.modules["sparse"] = sparse

    if "numba" not in sys.modules:
        numba = types.ModuleType("numba")

        def jit(*args, **kwargs):
            if len(args) == 1 and callable(args[0]) and not kwargs:
                return args[0]

            def deco(fn):
                return fn

            return deco

        numba.jit = jit
        numba.njit = jit
        numba.vectorize = jit
        numba.prange = range
        numba.complex128 = numba.float64 = numba.int64 = MagicMock()
        sys.modules["numba"] = numba

    if not any(isinstance(f, _MockFinder) for f in sys.meta_path):
        sys.meta_path.insert(0, _MockFinder(("ray", "h5py", "matplotlib", "mpl_toolkits")))


class _MockModule(types.ModuleType):
    """Module whose every missing attribute is a MagicMock."""

    def __init__(self, name):
        super().__init__(name)
        self.__path__ = []  # behave like a package so submodules resolve

    def __getattr__(self, item):
        if item.startswith("__"):
            raise AttributeError(item)
        value = MagicMock(name=f"{self.__name__}.{item}")
        setattr(self, item, value)
        return value


class _MockLoader:
    def create_module(self, spec):
        return _MockModule(spec.name)

    def exec_module(self, module):
        return None


class _MockFinder:
    """Meta-path finder that serves stub packages for optional plotting/cluster deps."""

    def __init__(self, roots):
        self.roots = roots

    def find_spec(self, fullname, path=None, target=None):
        import importlib.machinery

        if fullname.split(".")[0] in self.roots:
            return importlib.machinery.ModuleSpec(fullname, _MockLoader(), is_package=True)
        return None


def import_reference(path: str | None = None):
    """Return the ``hermespy`` package from ``path`` (or ``$HERMESPY_REFERENCE``;
    raises ImportError if the checkout is absent)."""

    path = reference_path(path)
    os.environ[ENV] = path  # worker processes of the fixture generators import the same checkout
    if not os.path.isdir(os.path.join(path, "hermespy")):
        raise ImportError(f"HermesPy reference not found under {path}")
    _install_stubs()
    if path not in sys.path:
        sys.path.insert(0, path)
    import hermespy  # noqa: F401
    import hermespy.modem  # noqa: F401
    import hermespy.channel  # noqa: F401
    import hermespy.simulation  # noqa: F401

    return hermespy
