"""Reader and writer of the reference's ``.kmc`` files.

A ``.kmc`` file is a pickled dict of a ``kmc_dn`` object's list, tuple,
int, float and ndarray attributes (saveSelf, kmc_dopant_networks.py:943-963).
Unpickling arbitrary data can run code, so ``read_kmc`` only admits the
globals numpy needs to rebuild arrays and scalars; anything else raises
``pickle.UnpicklingError``.
"""
from __future__ import annotations

import importlib
import pickle

__all__ = ["read_kmc", "write_kmc"]

_ALLOWED = {
    ("numpy.core.multiarray", "_reconstruct"), ("numpy._core.multiarray", "_reconstruct"),
    ("numpy.core.multiarray", "scalar"), ("numpy._core.multiarray", "scalar"),
    ("numpy", "ndarray"), ("numpy", "dtype"),
}


class _Restricted(pickle.Unpickler):
    def find_class(self, module, name):
        if (module, name) not in _ALLOWED:
            raise pickle.UnpicklingError(f"global {module}.{name} is not allowed in a .kmc file")
        return getattr(importlib.import_module(module), name)


def read_kmc(path):
    with open(path, "rb") as f:
        d = _Restricted(f).load()
    if not isinstance(d, dict):
        raise pickle.UnpicklingError(".kmc file does not hold an attribute dict")
    return d


def write_kmc(path, attrs):
    with open(path, "wb") as f:
        pickle.dump(dict(attrs), f)
