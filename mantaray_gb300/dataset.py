"""Result container: xarray.Dataset when xarray is installed, else a small
stand-in with the parts of the xarray interface the reference's callers use
(`ds.sizes[...]`, `ds.kx`, `ds["x"]`, `ds.attrs`, `.coords`, `.data_vars`,
`.dims`), all backed by numpy arrays.
"""

from __future__ import annotations

from typing import Dict, Sequence, Tuple

import numpy as np

try:  # pragma: no cover - exercised only where xarray is installed
    import xarray as _xr
except Exception:  # noqa: BLE001
    _xr = None


class Variable(np.ndarray):
    """A numpy array that remembers its dimension names."""

    dims: Tuple[str, ...] = ()

    def __new__(cls, data, dims: Sequence[str]):
        obj = np.asarray(data).view(cls)
        obj.dims = tuple(dims)
        return obj

    def __array_finalize__(self, obj):
        self.dims = getattr(obj, "dims", ())

    @property
    def values(self) -> np.ndarray:
        return np.asarray(self)


class Dataset:
    """Minimal xarray.Dataset stand-in (no xarray in this environment)."""

    def __init__(self, data_vars: Dict[str, Tuple[Sequence[str], np.ndarray]], coords=(), attrs=None):
        self._vars: Dict[str, Variable] = {}
        self._coords = set(coords)
        self.attrs = dict(attrs or {})
        for name, (dims, data) in data_vars.items():
            self._vars[name] = Variable(data, dims)

    @property
    def sizes(self) -> Dict[str, int]:
        out: Dict[str, int] = {}
        for v in self._vars.values():
            for d, n in zip(v.dims, v.shape):
                out[d] = n
        return out

    dims = sizes

    @property
    def coords(self):
        return {k: v for k, v in self._vars.items() if k in self._coords}

    @property
    def data_vars(self):
        return {k: v for k, v in self._vars.items() if k not in self._coords}

    def set_coords(self, names):
        self._coords.update([names] if isinstance(names, str) else names)
        return self

    def __getitem__(self, name):
        return self._vars[name]

    def __setitem__(self, name, value):
        if isinstance(value, tuple):
            dims, data = value
        else:
            data = np.asarray(value)
            dims = (name,)
        self._vars[name] = Variable(data, dims)

    def __contains__(self, name):
        return name in self._vars

    def __getattr__(self, name):
        vars_ = self.__dict__.get("_vars", {})
        if name in vars_:
            return vars_[name]
        raise AttributeError(name)

    def __repr__(self):
        dims = ", ".join(f"{k}: {v}" for k, v in self.sizes.items())
        return f"<mantaray_gb300.Dataset ({dims}) vars={list(self._vars)}>"


def make_dataset(data_vars, coords, attrs, index_coords=None):
    """Builds an xarray.Dataset when available, else the stand-in."""
    if _xr is not None:  # pragma: no cover
        ds = _xr.Dataset(data_vars={k: (list(d), v) for k, (d, v) in data_vars.items()}, attrs=attrs)
        ds = ds.set_coords(list(coords))
        for k, v in (index_coords or {}).items():
            ds[k] = v
        return ds
    ds = Dataset(data_vars, coords=coords, attrs=attrs)
    for k, v in (index_coords or {}).items():
        ds[k] = ((k,), np.asarray(v))
    return ds
