"""JAX custom calls of the C ABI (XLA typed FFI): the drop-in for the
reference's jit boundary.

The reference jits its step (``jax.jit(self._step)``,
solver/simulation/step_handlers.py:304-315; ``step_pure``'s
``static_argnames`` jit, solver/pure_functions/step.py:49).  Registering the
library's handlers ``aj_ffi_prepare`` / ``aj_ffi_step`` as XLA FFI targets lets
that jitted code call the GB300 kernels on its own device arrays and stream:

    from aerojax_gb300 import jax_ffi
    jax_ffi.register()                          # once per process
    ws = jax_ffi.prepare(mask, sdf, cfg)        # when the geometry changes
    u, v, p, ws = jax_ffi.step(u, v, mask, p_guess, ws, cfg)

``cfg`` is a StepConfig; its AjStepParams bytes travel as the handlers'
``params`` attribute.  The workspace is an XLA-owned uint8 buffer returned by
``prepare`` and aliased through ``step`` (input 4 -> output 3), so XLA treats
the scratch as written.  jax is imported only when these functions are
called; the library itself does not need it.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .params import StepConfig


def params_bytes(cfg: StepConfig) -> np.ndarray:
    """The AjStepParams of a StepConfig as the uint8 array attribute."""
    from .solver import make_params
    p = make_params(cfg)
    return np.frombuffer(bytes(p), dtype=np.uint8).copy()


def workspace_bytes(cfg: StepConfig) -> int:
    from .solver import make_params
    p = make_params(cfg)
    n = int(_lib.lib().aj_workspace_size(ctypes.byref(p)))
    if n == 0:
        raise ValueError("aj_workspace_size rejected the configuration")
    return n


def _jax():
    try:
        import jax
    except ImportError as e:   # pragma: no cover - jax is absent in this image
        raise RuntimeError("aerojax_gb300.jax_ffi needs jax (jax.ffi)") from e
    return jax


def register(platform: str = "CUDA") -> None:
    """Registers aj_prepare / aj_step as XLA FFI targets."""
    jax = _jax()
    L = _lib.lib()
    for name, fn in (("aj_prepare", L.aj_ffi_prepare), ("aj_step", L.aj_ffi_step)):
        jax.ffi.register_ffi_target(name, jax.ffi.pycapsule(fn), platform=platform)


def prepare(mask, sdf, cfg: StepConfig):
    """Workspace for cfg prepared for this geometry (sdf may be None)."""
    jax = _jax()
    import jax.numpy as jnp
    if sdf is None:
        sdf = jnp.zeros((0,), jnp.float32)
    out = jax.ShapeDtypeStruct((workspace_bytes(cfg),), jnp.uint8)
    return jax.ffi.ffi_call("aj_prepare", out)(mask, sdf, params=params_bytes(cfg))


def step(u, v, mask, p_guess, workspace, cfg: StepConfig):
    """One projection step inside jit; returns (u, v, p, workspace)."""
    jax = _jax()
    import jax.numpy as jnp
    if p_guess is None:
        p_guess = jnp.zeros((0,), jnp.float32)
    outs = (jax.ShapeDtypeStruct(u.shape, jnp.float32), jax.ShapeDtypeStruct(v.shape, jnp.float32),
            jax.ShapeDtypeStruct(mask.shape, jnp.float32),
            jax.ShapeDtypeStruct(workspace.shape, jnp.uint8))
    return jax.ffi.ffi_call("aj_step", outs, input_output_aliases={4: 3})(
        u, v, mask, p_guess, workspace, params=params_bytes(cfg))
