"""Damped Newton, gmin stepping, DC, transient and adjoints (oracle).

Restates voltax/analysis.py:

* `newton`        -- ``_newton`` (:208-233): ``dz = J^-1 (-r)``,
  ``scale = min(1, max_dv / (max|dz_nodes| + 1e-300))``, converged when
  ``|dz| <= atol + rtol |z_new|`` elementwise, ``scale == 1`` and finite.
* `gmin_stepping` -- ``_gmin_stepping`` (:236-266): a direct attempt of
  ``direct_steps`` iterations, else gmin stepped log-uniformly from
  ``gmin_start`` down to ``gmin``, each stage warm-started.
* `dc`, `transient` -- (:410-480) with the residuals and stamped Jacobians of
  (:325-378), the linear systems solved by the block-LDU factorization of
  `oracle.lu`.
* `dc_adjoint`    -- ``_root_bwd`` (:282-288): ``J^T lam = g`` at the root,
  ``dL/dp = -lam^T dF/dp``; here returned as ``lam`` (the per-parameter VJP
  is formed by the caller with torch autograd of `oracle.stamp`).
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import lu, stamp


@dataclass(frozen=True)
class Options:
    max_steps: int = 100
    rtol: float = 1e-6
    atol: float = 1e-9
    max_dv: float = 1.0
    gmin: float = 1e-12
    gmin_steps: int = 10
    gmin_start: float = 1e-2
    direct_steps: int = 25


class System:
    """One circuit instance with its structure and padded plan."""

    def __init__(self, circuit, st, plan, b: int = 0):
        self.c, self.st, self.b = circuit, st, b
        self.pp = lu.from_plan(plan, st) if not isinstance(plan, lu.PaddedPlan) else plan
        self.nv = circuit.layout.n_nodes
        self.S = circuit.layout.size

    def solve(self, data, rhs, transpose=False):
        return lu.solve(self.pp, lu.factor(self.pp, data), rhs, transpose)

    # residual / Jacobian pairs ------------------------------------------------
    def dc_pair(self, t, gmin):
        c, st, b = self.c, self.st, self.b

        def res(z):
            return stamp.dc_residual(c, z, t, gmin, b)

        def jac(z):
            return stamp.add_gmin(stamp.jacobian(c, st, z, t, 1.0, 0.0, b), st, self.nv, gmin)
        return res, jac

    def step_pair(self, method, z_prev, t_prev, t, gmin):
        c, st, b = self.c, self.st, self.b
        cf = 1.0 if method == "be" else 0.5
        cq = 1.0 / (t - t_prev)

        def res(z):
            if method == "be":
                return stamp.be_residual(c, z, z_prev, t_prev, t, gmin, b)
            return stamp.trap_residual(c, z, z_prev, t_prev, t, gmin, b)

        def jac(z):
            return stamp.add_gmin(stamp.jacobian(c, st, z, t, cf, cq, b), st, self.nv, gmin)
        return res, jac


def newton(sys: System, res, jac, z0, opts: Options, max_steps=None):
    """Returns ``(z, converged, iterations)``."""
    max_steps = opts.max_steps if max_steps is None else max_steps
    z = np.array(z0, dtype=np.float64)
    done = False
    k = 0
    while k < max_steps and not done:
        r = res(z)
        dz = sys.solve(jac(z), -r)
        dv = np.abs(dz[: sys.nv])
        dv_max = dv.max() if len(dv) else 0.0
        scale = min(1.0, opts.max_dv / (dv_max + 1e-300))
        z_new = z + scale * dz
        small = bool(np.all(np.abs(dz) <= opts.atol + opts.rtol * np.abs(z_new)))
        done = small and scale == 1.0 and bool(np.all(np.isfinite(z_new)))
        z = z_new
        k += 1
    return z, done, k


def gmin_stepping(sys: System, t, guess, opts: Options):
    if opts.gmin_steps == 0:
        res, jac = sys.dc_pair(t, opts.gmin)
        return newton(sys, res, jac, guess, opts)
    gmins = np.concatenate([[opts.gmin], np.logspace(np.log10(opts.gmin_start),
                                                     np.log10(opts.gmin), opts.gmin_steps)])
    steps = [opts.direct_steps] + [opts.max_steps] * opts.gmin_steps
    z, ok, total = np.array(guess, np.float64), False, 0
    k = 0
    while k <= opts.gmin_steps and not (ok and k == 1):
        res, jac = sys.dc_pair(t, gmins[k])
        start = guess if k == 1 else z
        z, ok, it = newton(sys, res, jac, start, opts, steps[k])
        total += it
        k += 1
    return z, ok, total


def dc(sys: System, t=0.0, guess=None, opts: Options = Options()):
    guess = np.zeros(sys.S) if guess is None else guess
    return gmin_stepping(sys, t, guess, opts)


def transient(sys: System, ts, ic="dc", method="be", opts: Options = Options()):
    """Returns ``(z (T, S), converged (T,), iterations (T,))``."""
    ts = np.asarray(ts, np.float64)
    if isinstance(ic, str):
        if ic == "dc":
            z0 = dc(sys, ts[0], opts=opts)[0]
        elif ic == "zero":
            z0 = np.zeros(sys.S)
        else:
            raise ValueError(f"ic must be 'dc', 'zero' or an array, got {ic!r}")
    else:
        z0 = np.asarray(ic, np.float64)
    zs, oks, its = [z0], [True], [0]
    z = z0
    for t_prev, t in zip(ts[:-1], ts[1:]):
        res, jac = sys.step_pair(method, z, t_prev, t, opts.gmin)
        z, ok, it = newton(sys, res, jac, z, opts)
        zs.append(z)
        oks.append(ok)
        its.append(it)
    return np.stack(zs), np.array(oks), np.array(its)


def dc_adjoint(sys: System, z, g, t=0.0, opts: Options = Options()):
    """``lam`` with ``J(z)^T lam = g`` (voltax/analysis.py:282-288)."""
    _, jac = sys.dc_pair(t, opts.gmin)
    return sys.solve(jac(z), g, transpose=True)


def ac(sys: System, freqs, z_op, t=0.0):
    """Small-signal AC (voltax/analysis.py:494-524): ``(G + j 2 pi f C) z = -b``
    with dense complex LAPACK solves; ``G``, ``C`` the stamped Jacobians of
    f and q at the operating point ``z_op``, ``b`` the sources' stimulus."""
    c, st = sys.c, sys.st
    n = st.size
    G = np.zeros((n, n))
    Cm = np.zeros((n, n))
    rows = np.repeat(np.arange(n), np.diff(st.indptr))
    G[rows, st.indices] = stamp.jacobian(c, st, z_op, t, 1.0, 0.0, sys.b)
    Cm[rows, st.indices] = stamp.jacobian(c, st, z_op, t, 0.0, 1.0, sys.b)
    b = _ac_stimulus(c)
    return np.stack([np.linalg.solve(G + 2j * np.pi * f * Cm, -b) for f in freqs])


def _ac_stimulus(c):
    """voltax/circuit.py:204-207 with sources.py:85-115: a voltage source
    adds ``-ac e^{j phase}`` to its branch equation, a current source drives
    ``ac e^{j phase}`` from p to n."""
    b = np.zeros(c.layout.size, dtype=complex)
    for name, n, k, off in c.layout.groups:
        el = c.elements[name]
        if type(el).__name__ not in ("VoltageSource", "CurrentSource") or n == 0:
            continue
        ac = np.broadcast_to(np.asarray(el.ac, dtype=float), (n,))
        ph = np.broadcast_to(np.asarray(el.ac_phase, dtype=float), (n,))
        phasor = ac * np.exp(1j * np.pi / 180.0 * ph)
        if type(el).__name__ == "VoltageSource":
            b[off + np.arange(n) * k] -= phasor
        else:
            nodes = np.asarray(el.nodes, dtype=np.int64).reshape(n, -1)
            for col, sgn in ((0, 1.0), (1, -1.0)):
                for d in range(n):
                    if nodes[d, col] >= 0:
                        b[nodes[d, col]] += sgn * phasor[d]
    return b
