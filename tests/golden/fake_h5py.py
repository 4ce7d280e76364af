"""An in-memory stand-in for the part of h5py that the HDF5 writers use.

Test infrastructure: h5py is not installed in this container or on the GPU
machines, so the layout written by ``SimulationResult.save_to_hdf`` (groups,
attributes, datasets) is recorded here instead.  ``make_golden_hdf.py`` records
what the reference writes, ``tests/test_hdf_export.py`` what this package
writes, and the two records are compared.

Semantics kept from h5py: ``File(path, mode)`` is a context manager over one
store per path; ``create_group`` makes intermediate groups and raises
ValueError when the group exists; ``f[path]`` returns a group with ``attrs``
(a dict) and ``create_dataset(name, data=...)``; ``del f[path]`` removes a
group and everything under it.
"""
from __future__ import annotations

import numpy as np

STORES: dict = {}  # file path -> {group path: {"attrs": {}, "datasets": {}}}


def _norm(path: str) -> str:
    return "/".join(p for p in str(path).split("/") if p)


class Group:
    def __init__(self, store, path):
        self._store = store
        self._path = path

    @property
    def attrs(self):
        return self._store[self._path]["attrs"]

    def create_dataset(self, name, data=None):
        self._store[self._path]["datasets"][name] = np.array(data, copy=True)


class File:
    def __init__(self, path, mode="a"):
        self.path = str(path)
        if mode == "w" or self.path not in STORES:
            STORES[self.path] = {"": {"attrs": {}, "datasets": {}}}
        self.store = STORES[self.path]

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        return False

    def close(self):
        pass

    def create_group(self, path):
        p = _norm(path)
        if p in self.store:
            raise ValueError(f"Unable to create group (name already exists): {p}")
        parts = p.split("/")
        for k in range(1, len(parts) + 1):
            self.store.setdefault("/".join(parts[:k]), {"attrs": {}, "datasets": {}})
        return Group(self.store, p)

    def __getitem__(self, path):
        p = _norm(path)
        if p not in self.store:
            raise KeyError(p)
        return Group(self.store, p)

    def __contains__(self, path):
        return _norm(path) in self.store

    def __delitem__(self, path):
        p = _norm(path)
        for key in [k for k in self.store if k == p or k.startswith(p + "/")]:
            del self.store[key]


def snapshot(path) -> dict:
    """The recorded store of one file: {group: (attrs, datasets)}."""
    return STORES[str(path)]
