"""The JAX side of the drop-in: voltax's sparse.jacobian / factor / solve /
spsolve as XLA FFI custom calls into libvxg (voltax/sparse.py:220-249,
543-621).

Where jax (with jax.ffi) and the shim library ``libvxg_xla.so`` exist, a
voltax maintainer replaces ``voltax.sparse.factor`` and ``voltax.sparse.solve``
by `factor` and `solve` below; ``spsolve``'s ``custom_vjp`` and ``_root``'s
``filter_custom_vjp`` (voltax/analysis.py:269-288) then run the GB300 kernels
for the forward solve and the transposed adjoint solve with no other change.
`spsolve` here is the same custom VJP written against these calls.

Import cost: nothing is imported from jax until a function is called, so
this module is safe to import where jax is absent (`available()` says so).
"""

from __future__ import annotations

import ctypes as C
import functools
from pathlib import Path

from . import _lib as L

XLA_LIB = Path(__file__).resolve().parent / "_lib" / "libvxg_xla.so"
TARGETS = ("vxg_eval", "vxg_factor", "vxg_solve")


def available() -> bool:
    """True when jax with jax.ffi is importable and libvxg_xla.so is built."""
    try:
        import jax  # noqa: F401
        from jax import ffi  # noqa: F401
    except ImportError:
        return False
    return XLA_LIB.exists()


@functools.lru_cache(maxsize=1)
def register() -> None:
    """Register the three handlers as CUDA FFI targets (once)."""
    import jax
    shim = C.CDLL(str(XLA_LIB))
    L.load()  # the handlers call into libvxg.so
    for name in TARGETS:
        jax.ffi.register_ffi_target(name, jax.ffi.pycapsule(getattr(shim, name + "_ffi")),
                                    platform="CUDA")


class Topology:
    """A vxg handle for one structure and plan, with its buffer sizes."""

    def __init__(self, circuit, st, plan):
        from .runtime import Tables
        self.tables = Tables(circuit, st, plan)
        lib = L.load()
        h = C.c_void_p()
        L.check(lib.vxg_create(C.byref(self.tables.descriptor()), C.byref(h)), "vxg_create")
        self.handle = h.value
        self.S, self.nnz = st.size, st.nnz

    def sizes(self, batch: int, precision: int) -> tuple[int, int]:
        lib = L.load()
        fb, wb = C.c_size_t(), C.c_size_t()
        L.check(lib.vxg_factor_size(self.handle, batch, precision, C.byref(fb)),
                "vxg_factor_size")
        L.check(lib.vxg_workspace_size(self.handle, batch, precision, C.byref(wb)),
                "vxg_workspace_size")
        return fb.value, wb.value


def factor(topo: Topology, data, precision: int = L.VXG_F64):
    """Factors of the CSR values `data` (batch x nnz, float64) as one uint8
    buffer (replaces voltax.sparse.factor)."""
    import jax
    import jax.numpy as jnp
    register()
    batch = data.shape[0] if data.ndim == 2 else 1
    fb, wb = topo.sizes(batch, precision)
    out = (jax.ShapeDtypeStruct((fb,), jnp.uint8), jax.ShapeDtypeStruct((wb,), jnp.uint8))
    fac, _ = jax.ffi.ffi_call("vxg_factor", out)(
        data, handle=topo.handle, batch=batch, precision=precision)
    return fac


def solve(topo: Topology, factors, data, b, transpose: bool = False,
          precision: int = L.VXG_F64, refine: int = 2):
    """x = A^-1 b or A^-T b from `factor` (replaces voltax.sparse.solve)."""
    import jax
    import jax.numpy as jnp
    register()
    batch = b.shape[0] if b.ndim == 2 else 1
    _, wb = topo.sizes(batch, precision)
    out = (jax.ShapeDtypeStruct(b.shape, jnp.float64), jax.ShapeDtypeStruct((wb,), jnp.uint8))
    x, _ = jax.ffi.ffi_call("vxg_solve", out)(
        factors, data, b, handle=topo.handle, batch=batch, precision=precision,
        transpose=int(bool(transpose)), refine=refine if precision == L.VXG_F32 else 0)
    return x


def spsolve(topo: Topology, data, b, precision: int = L.VXG_F64):
    """x = A^-1 b with voltax's custom VJP (voltax/sparse.py:598-621): the
    backward pass reuses the forward factors for one transposed solve,
    gb = A^-T g, and gdata = -gb[rows] * x[indices]."""
    import jax
    import jax.numpy as jnp
    rows = jnp.asarray(topo.tables.rows)
    cols = jnp.asarray(topo.tables.indices)

    @jax.custom_vjp
    def _solve(data, b):
        return solve(topo, factor(topo, data, precision), data, b, precision=precision)

    def fwd(data, b):
        fac = factor(topo, data, precision)
        x = solve(topo, fac, data, b, precision=precision)
        return x, (fac, data, x)

    def bwd(res, g):
        fac, data, x = res
        gb = solve(topo, fac, data, g, transpose=True, precision=precision)
        return -gb[..., rows] * x[..., cols], gb

    _solve.defvjp(fwd, bwd)
    return _solve(data, b)
