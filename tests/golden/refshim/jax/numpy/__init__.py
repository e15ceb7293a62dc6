"""``jax.numpy`` stand-in: numpy functions whose array results carry ``.at``."""

from __future__ import annotations

import types as _types

import numpy as _np


class _AtItem:
    def __init__(self, arr, idx):
        self._arr = arr
        self._idx = idx

    def set(self, value):
        out = _np.array(self._arr, copy=True)
        out[self._idx] = _np.asarray(value)
        return _wrap(out)

    def add(self, value):
        out = _np.array(self._arr, copy=True)
        out[self._idx] += _np.asarray(value)
        return _wrap(out)

    def multiply(self, value):
        out = _np.array(self._arr, copy=True)
        out[self._idx] *= _np.asarray(value)
        return _wrap(out)

    def get(self):
        return _wrap(_np.asarray(self._arr)[self._idx])


class _At:
    def __init__(self, arr):
        self._arr = arr

    def __getitem__(self, idx):
        return _AtItem(self._arr, idx)


class _JArray(_np.ndarray):
    """ndarray subclass with JAX's functional ``.at`` update syntax."""

    @property
    def at(self):
        return _At(self)

    def block_until_ready(self):
        return self


def _wrap(x):
    if isinstance(x, _np.ndarray) and not isinstance(x, _JArray):
        return x.view(_JArray)
    if isinstance(x, tuple) and not hasattr(x, "_fields"):
        return tuple(_wrap(e) for e in x)
    if isinstance(x, list):
        return [_wrap(e) for e in x]
    return x


def _wrapped(fn):
    def call(*args, **kwargs):
        return _wrap(fn(*args, **kwargs))

    call.__name__ = getattr(fn, "__name__", "fn")
    call.__doc__ = getattr(fn, "__doc__", None)
    return call


ndarray = _JArray


def array(obj, dtype=None, copy=True, **kwargs):
    return _wrap(_np.array(obj, dtype=dtype, copy=True))


def asarray(obj, dtype=None, **kwargs):
    return _wrap(_np.array(obj, dtype=dtype, copy=True))


def einsum(*operands, **kwargs):
    kwargs.setdefault("optimize", True)
    kwargs.pop("precision", None)
    return _wrap(_np.einsum(*operands, **kwargs))


def _make_sub(name, src):
    mod = _types.ModuleType(f"jax.numpy.{name}")
    for attr in dir(src):
        if attr.startswith("_"):
            continue
        obj = getattr(src, attr)
        setattr(mod, attr, _wrapped(obj) if callable(obj) else obj)
    return mod


fft = _make_sub("fft", _np.fft)
linalg = _make_sub("linalg", _np.linalg)


def __getattr__(name):
    obj = getattr(_np, name)
    if callable(obj) and not isinstance(obj, type):
        return _wrapped(obj)
    return obj
