"""Run J-UBIK's own ``convolve.py``, ``response.py`` and ``utils.py`` without JAX.

Test infrastructure, used only by ``make_ref_fixtures.py`` in a checkout that
holds the reference sources.  JAX, jaxlib and NIFTy.re are not installed, but
the reference's patch convolution and readout touch only a small part of them.
This module registers numpy-backed stand-ins for that part in ``sys.modules``
and then loads the reference's source files, unmodified, from their own paths:

* ``jax.numpy``            -> numpy (``pad``, ``arange``, ``meshgrid``, ``fft``, ...)
* ``jax.lax.dynamic_slice`` -> a slice whose start indices are clamped to
  ``[0, operand_size - slice_size]``, the documented JAX behaviour
* ``jax.vmap``              -> a loop over the mapped axis, results stacked
* ``jax.linear_transpose`` -> the exact transpose of a linear map that is a
  gather with zero fill (each output element is one input element or 0), as
  ``slice_patches`` is: the map is evaluated on the input's element numbers to
  find its index table, the gather form is verified on a random input, and the
  transpose scatter-adds through that table.  Other maps raise.
* ``nifty.re.Vector``      -> a holder of the ``tree`` dict
* ``jubik.data.Domain``    -> the reference's own class, taken from
  ``jubik/data.py`` by its syntax tree (that module imports the whole sky-model
  stack).

JAX on the CPU computes FFTs with pocketfft, as numpy does; with x64 enabled
(``jubik/enforce_float64.py``) both work in float64/complex128.
"""
from __future__ import annotations

import ast
import importlib.util
import os
import sys
import types

import numpy as np


# ---------------------------------------------------------------- jax stand-in
def _dynamic_slice(operand, start_indices, slice_sizes):
    operand = np.asarray(operand)
    if len(start_indices) != operand.ndim or len(slice_sizes) != operand.ndim:
        raise ValueError("dynamic_slice: one start index and size per axis")
    idx = []
    for s, z, n in zip(start_indices, slice_sizes, operand.shape):
        s = int(np.clip(int(s), 0, n - int(z)))  # JAX clamps the start into range
        idx.append(slice(s, s + int(z)))
    return operand[tuple(idx)]


def _vmap(fun, in_axes=0, out_axes=0):
    if out_axes != 0:
        raise NotImplementedError("stand-in vmap maps onto output axis 0 only")

    def mapped(*args):
        axes = in_axes if isinstance(in_axes, (tuple, list)) else (in_axes,) * len(args)
        sizes = {np.shape(a)[ax] for a, ax in zip(args, axes) if ax is not None}
        if len(sizes) != 1:
            raise ValueError("vmap: mapped axes differ in size")
        (n,) = sizes
        outs = []
        for i in range(n):
            call = [a if ax is None else np.take(np.asarray(a), i, axis=ax)
                    for a, ax in zip(args, axes)]
            outs.append(np.asarray(fun(*call)))
        return np.stack(outs, axis=0)

    return mapped


def _linear_transpose(fun, *primals):
    if len(primals) != 1:
        raise NotImplementedError("stand-in linear_transpose takes one primal")
    shape = np.shape(primals[0])
    size = int(np.prod(shape)) if shape else 1
    if size >= 2 ** 52:
        raise ValueError("too many elements for an exact index table")
    numbers = (np.arange(size, dtype=np.float64) + 1.0).reshape(shape)
    table = np.asarray(fun(numbers))
    src = table.astype(np.int64)
    probe = np.random.default_rng(20240917).standard_normal(shape)
    flat = np.concatenate([[0.0], probe.reshape(-1)])
    if not (np.array_equal(src, table) and src.min() >= 0 and src.max() <= size and
            np.array_equal(np.asarray(fun(probe)), flat[src])):
        raise NotImplementedError("stand-in linear_transpose covers zero-filled gathers only")

    def transposed(cot):
        out = np.zeros(size + 1, dtype=np.result_type(np.asarray(cot).dtype, np.float64))
        np.add.at(out, src.reshape(-1), np.asarray(cot).reshape(-1))
        return (out[1:].reshape(shape),)

    return transposed


class _Config:
    def update(self, name, value):  # jax.config.update("jax_enable_x64", True)
        self.__dict__[name] = value


def _module(name, **attrs):
    m = types.ModuleType(name)
    m.__dict__.update(attrs)
    return m


class Vector:
    """``nifty.re.Vector``: a pytree holder with a ``tree`` attribute."""

    def __init__(self, tree):
        self.tree = tree


class _Model:  # only used in the reference's signatures
    def __init__(self, *a, **k):
        raise NotImplementedError("nifty.re.Model is not part of the stand-in")


def install():
    """Register the stand-in modules (idempotent); returns the ``jax`` module."""
    if "jax" in sys.modules and getattr(sys.modules["jax"], "__standin__", False):
        return sys.modules["jax"]
    jnp = _module("jax.numpy", ndarray=np.ndarray)
    jnp.__getattr__ = lambda name: getattr(np, name)  # everything else is numpy's
    lax = _module("jax.lax", dynamic_slice=_dynamic_slice)
    jax = _module("jax", numpy=jnp, lax=lax, vmap=_vmap, linear_transpose=_linear_transpose,
                  config=_Config(), __standin__=True)
    jax.__path__ = []
    jre = _module("nifty.re", Vector=Vector, Model=_Model)
    nifty = _module("nifty", re=jre)
    nifty.__path__ = []
    sys.modules.update({"jax": jax, "jax.numpy": jnp, "jax.lax": lax, "nifty": nifty,
                        "nifty.re": jre})
    return jax


# ---------------------------------------------------------------- reference loader
def _class_from_source(path, name):
    """Source of the top-level class ``name`` in the file at ``path``."""
    with open(path) as f:
        src = f.read()
    for node in ast.parse(src).body:
        if isinstance(node, ast.ClassDef) and node.name == name:
            return ast.get_source_segment(src, node)
    raise LookupError(f"class {name} not found in {path}")


def load_reference(root):
    """A ``jubik`` package whose ``convolve``, ``response`` and ``utils`` modules
    are the reference's own files under ``root/jubik``; its top level exports
    what the reference's tests use."""
    install()
    pkgdir = os.path.join(root, "jubik")
    pkg = _module("jubik")
    pkg.__path__ = [pkgdir]
    sys.modules["jubik"] = pkg
    data = _module("jubik.data", NamedTuple=__import__("typing").NamedTuple)
    exec("from typing import NamedTuple\n" + _class_from_source(os.path.join(pkgdir, "data.py"),
                                                                 "Domain"), data.__dict__)
    data.Domain.__module__ = "jubik.data"
    sys.modules["jubik.data"] = data
    pkg.data = data
    mods = {}
    for name in ("convolve", "response", "utils"):
        spec = importlib.util.spec_from_file_location(f"jubik.{name}",
                                                      os.path.join(pkgdir, f"{name}.py"))
        mod = importlib.util.module_from_spec(spec)
        sys.modules[spec.name] = mod
        spec.loader.exec_module(mod)
        setattr(pkg, name, mod)
        mods[name] = mod
    c, r, u = mods["convolve"], mods["response"], mods["utils"]
    pkg.__dict__.update(Domain=data.Domain, convolve=c.convolve, slice_patches=c.slice_patches,
                        linpatch_convolve=c.linpatch_convolve, integrate=c.integrate,
                        build_exposure_function=r.build_exposure_function,
                        build_readout_function=r.build_readout_function,
                        coord_center=u.coord_center)
    return pkg
