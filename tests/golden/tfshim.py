"""A numpy stand-in for the small part of the TensorFlow 2 API that madflow's
phase-space, wavefunction, parameter and mock-up matrix-element modules use.

It exists for one purpose: to execute madflow's own Python source (which
imports ``tensorflow`` and ``pdfflow``, neither installed in this image) so
that golden input/output vectors can be generated from the reference code
itself.  It is used only by ``make_golden.py`` in this directory.

Semantics kept from TensorFlow because the reference relies on them:

* ``tf.convert_to_tensor`` / ``tf.cast`` of a *Python* float goes through
  float32 (TensorFlow's default dtype for Python floats), Python ints through
  int32, Python complex through complex128.  numpy arrays and numpy scalars
  keep their dtype.  This is what makes ``float_me(np.pi)`` equal to
  float32(pi) and ``float_me(sqrt(0.5))`` equal to 0.7071067690849304 in the
  reference.
* ``pdfflow.configflow.float_me(x) = tf.cast(x, DTYPE)`` and
  ``int_me(x) = tf.cast(x, DTYPEINT)`` (pdfflow's published configflow; the
  package is not vendored in the reference).
* ``tf.where`` / ``tf.cond`` select; both branches of ``tf.where`` are
  evaluated (numpy does the same).
* ``tf.while_loop`` runs the body while the condition holds, at most
  ``maximum_iterations`` times.
"""
import builtins
import sys
import types

import numpy as np

float64 = np.float64
float32 = np.float32
int32 = np.int32
int64 = np.int64
complex128 = np.complex128
complex64 = np.complex64
bool_ = np.bool_


def _dt(dtype):
    return np.dtype(dtype)


def convert_to_tensor(x, dtype=None, name=None):
    if isinstance(x, np.ndarray):
        out = x
    elif isinstance(x, np.generic):
        out = np.asarray(x)
    elif isinstance(x, bool):
        out = np.asarray(x, dtype=np.bool_)
    elif isinstance(x, builtins.int):
        out = np.asarray(x, dtype=np.int32)
    elif isinstance(x, builtins.float):
        out = np.asarray(x, dtype=np.float32)
    elif isinstance(x, builtins.complex):
        out = np.asarray(x, dtype=np.complex128)
    elif isinstance(x, (list, tuple)):
        items = [convert_to_tensor(i) for i in x]
        kinds = {i.dtype for i in items}
        if len(kinds) == 1:
            out = np.stack(items) if items else np.asarray([], dtype=np.float32)
        else:
            out = np.stack([np.asarray(i, dtype=np.result_type(*kinds)) for i in items])
    else:
        out = np.asarray(x)
    if dtype is not None:
        out = out.astype(_dt(dtype))
    return out


def cast(x, dtype, name=None):
    t = convert_to_tensor(x)
    d = _dt(dtype)
    if np.iscomplexobj(t) and d.kind != "c":
        t = t.real
    return np.asarray(t.astype(d))


def constant(value, dtype=None, shape=None, name=None):
    if dtype is None:
        return convert_to_tensor(value)
    return np.asarray(np.asarray(value).astype(_dt(dtype)))


class TensorSpec:
    def __init__(self, shape=None, dtype=None, name=None):
        self.shape = shape
        self.dtype = dtype


class _Function:
    """``tf.function`` replacement: a transparent wrapper (descriptor-aware)."""

    def __init__(self, fn, input_signature=None):
        self.python_function = fn
        self.input_signature = input_signature

    def __call__(self, *args, **kwargs):
        return self.python_function(*args, **kwargs)

    def __get__(self, obj, objtype=None):
        if obj is None:
            return self
        return _Bound(self.python_function, self.input_signature, obj)


class _Bound:
    def __init__(self, fn, sig, obj):
        self.python_function = fn
        self.input_signature = sig
        self._obj = obj

    def __call__(self, *args, **kwargs):
        return self.python_function(self._obj, *args, **kwargs)


def function(fn=None, input_signature=None, **kwargs):
    if fn is None:
        return lambda f: _Function(f, input_signature)
    return _Function(fn, input_signature)


def executing_eagerly():
    return True


def _arr(x):
    return x if isinstance(x, np.ndarray) else convert_to_tensor(x)


def stack(values, axis=0, name=None):
    vals = [_arr(v) for v in values]
    shapes = {v.shape for v in vals}
    if len(shapes) > 1:  # TF requires equal shapes; broadcast scalars for convenience
        target = np.broadcast_shapes(*shapes)
        vals = [np.broadcast_to(v, target) for v in vals]
    return np.stack(vals, axis=axis)


def concat(values, axis, name=None):
    return np.concatenate([_arr(v) for v in values], axis=axis)


def where(condition, x=None, y=None, name=None):
    if x is None and y is None:
        return np.argwhere(_arr(condition)).astype(np.int64)
    return np.where(_arr(condition), _arr(x), _arr(y))


def cond(pred, true_fn, false_fn, name=None):
    return true_fn() if bool(pred) else false_fn()


def while_loop(cond_fn, body, loop_vars, parallel_iterations=10, maximum_iterations=None, **kw):
    loop_vars = tuple(loop_vars)
    it = 0
    while bool(cond_fn(*loop_vars)):
        if maximum_iterations is not None and it >= maximum_iterations:
            break
        loop_vars = tuple(body(*loop_vars))
        it += 1
    return loop_vars


def reduce_sum(x, axis=None, keepdims=False, name=None):
    if isinstance(x, (list, tuple)):
        x = stack(x)
    return np.sum(_arr(x), axis=axis, keepdims=keepdims)


def reduce_prod(x, axis=None, keepdims=False, name=None):
    return np.prod(_arr(x), axis=axis, keepdims=keepdims)


def reduce_all(x, axis=None, keepdims=False, name=None):
    if isinstance(x, (list, tuple)):
        x = stack(x)
    return np.all(_arr(x), axis=axis, keepdims=keepdims)


def _unary(fn):
    def f(x, name=None):
        return fn(_arr(x))

    return f


sqrt = _unary(np.sqrt)
square = _unary(np.square)
exp = _unary(np.exp)


def pow(x, y, name=None):  # noqa: A001 - mirrors tf.pow
    x = _arr(x)
    if isinstance(y, (builtins.int, builtins.float)):
        return np.power(x, np.asarray(y, dtype=x.dtype))
    return np.power(x, _arr(y))


def ones_like(x, dtype=None, name=None):
    x = _arr(x)
    return np.ones_like(x, dtype=_dt(dtype) if dtype is not None else x.dtype)


def zeros_like(x, dtype=None, name=None):
    x = _arr(x)
    return np.zeros_like(x, dtype=_dt(dtype) if dtype is not None else x.dtype)


def zeros(shape, dtype=np.float32, name=None):
    return np.zeros(np.asarray(shape).astype(int).tolist() if not isinstance(shape, builtins.int) else builtins.int(shape), dtype=_dt(dtype))


def ones(shape, dtype=np.float32, name=None):
    return np.ones(shape, dtype=_dt(dtype))


def reshape(x, shape, name=None):
    return np.reshape(_arr(x), shape)


def expand_dims(x, axis, name=None):
    return np.expand_dims(_arr(x), axis)


def transpose(x, perm=None, name=None):
    return np.transpose(_arr(x), perm)


def shape(x, out_type=np.int32, name=None):
    return np.asarray(_arr(x).shape, dtype=_dt(out_type))


def boolean_mask(x, mask, axis=None, name=None):
    x = _arr(x)
    m = _arr(mask).astype(bool)
    if axis in (None, 0):
        return x[m]
    return np.compress(m, x, axis=axis)


def logical_and(x, y, name=None):
    return np.logical_and(_arr(x), _arr(y))


def einsum(eq, *ops):
    return np.einsum(eq, *[_arr(o) for o in ops])


def gather(params, indices, axis=0, name=None):
    return np.take(_arr(params), _arr(indices), axis=axis)


def scatter_nd(indices, updates, shape, name=None):
    out = np.zeros(tuple(np.asarray(shape).tolist()), dtype=_arr(updates).dtype)
    idx = _arr(indices)
    out[tuple(idx.T)] = _arr(updates)
    return out


def pad(x, paddings, mode="CONSTANT", constant_values=0, name=None):
    return np.pad(_arr(x), np.asarray(paddings), constant_values=constant_values)


def complex(real, imag, name=None):  # noqa: A001 - mirrors tf.complex
    r = _arr(real).astype(np.float64)
    i = _arr(imag).astype(np.float64)
    return (r + 1j * i).astype(np.complex128)


def _lgamma(x):
    from math import lgamma as _lg

    x = _arr(x)
    return np.vectorize(_lg, otypes=[x.dtype])(x)


math = types.ModuleType("tensorflow.math")
math.sqrt = sqrt
math.sin = _unary(np.sin)
math.cos = _unary(np.cos)
math.cosh = _unary(np.cosh)
math.sinh = _unary(np.sinh)
math.log = _unary(np.log)
math.exp = exp
math.lgamma = _lgamma
math.minimum = lambda x, y, name=None: np.minimum(_arr(x), _arr(y))
math.maximum = lambda x, y, name=None: np.maximum(_arr(x), _arr(y))
math.abs = _unary(np.abs)
math.sign = _unary(np.sign)
math.real = _unary(np.real)
math.imag = _unary(np.imag)
math.conj = _unary(np.conj)
math.reduce_all = reduce_all
math.reduce_sum = reduce_sum
math.square = square

random = types.ModuleType("tensorflow.random")
_rng = {"gen": np.random.default_rng(4)}


def _set_seed(seed):
    _rng["gen"] = np.random.default_rng(seed)


def _uniform(shape, minval=0, maxval=None, dtype=np.float32, seed=None, name=None):
    maxval = 1.0 if maxval is None else maxval
    return _rng["gen"].uniform(minval, maxval, size=tuple(shape)).astype(_dt(dtype))


random.set_seed = _set_seed
random.uniform = _uniform


def _batch_dot(x, y, axes=None):
    # keras.backend.batch_dot(x[b,n,k], y[b,j,k], axes=2) -> out[b,n,j] = sum_k x*y
    assert axes == 2
    return np.einsum("bnk,bjk->bnj", _arr(x), _arr(y))


keras = types.ModuleType("tensorflow.keras")
keras.backend = types.SimpleNamespace(batch_dot=_batch_dot)
config = types.SimpleNamespace(list_physical_devices=lambda kind=None: [])


def install():
    """Register the stand-ins as ``tensorflow``, ``tensorflow.math`` and
    ``pdfflow.configflow`` in ``sys.modules``."""
    this = sys.modules[__name__]
    tf_mod = types.ModuleType("tensorflow")
    for k, v in vars(this).items():
        if not k.startswith("__") and k not in ("install", "sys", "types"):
            setattr(tf_mod, k, v)
    tf_mod.math = math
    sys.modules["tensorflow"] = tf_mod
    sys.modules["tensorflow.math"] = math

    pdf_mod = types.ModuleType("pdfflow")
    cfg = types.ModuleType("pdfflow.configflow")
    cfg.DTYPE = np.float64
    cfg.DTYPEINT = np.int32
    cfg.run_eager = lambda flag=True: None
    cfg.float_me = lambda x: cast(x, np.float64)
    cfg.int_me = lambda x: cast(x, np.int32)
    cfg.fzero = cfg.float_me(0.0)
    cfg.fone = cfg.float_me(1.0)
    cfg.izero = cfg.int_me(0)
    cfg.ione = cfg.int_me(1)
    pdf_mod.configflow = cfg
    sys.modules["pdfflow"] = pdf_mod
    sys.modules["pdfflow.configflow"] = cfg
    return tf_mod
