"""Device physics in torch float64 on the CPU (oracle).

Each element group becomes a `GroupModel` with ``currents(v, x, t) -> (I,
F)`` and ``charges(v, x) -> (Q, P)`` written exactly as voltax writes them:

* Resistor            voltax/elements/passive.py:37-38
* Capacitor           voltax/elements/passive.py:58-59
* Conductance         voltax/elements/behavioral.py:78-99
* VoltageSource       voltax/elements/sources.py:85-87
* CurrentSource       voltax/elements/sources.py:110-112
* Level1MOSFET        voltax/elements/mosfet.py:208-257
* Diode               voltax/elements/semiconductor.py:17-70
* Inductor            voltax/elements/passive.py:62-87
* VCCS                voltax/elements/controlled.py:46-60
* BJT                 voltax/elements/semiconductor.py:73-135
* VCVS, CCCS, CCVS    voltax/elements/controlled.py:27-98
* Transformer         voltax/elements/passive.py:90-129
* CoupledInductors    the non-local element of voltax tests/test_sparse.py:90-113
                      (``local = False``: a full mutual-inductance matrix)
* IdealOpAmp, OpAmp   voltax/elements/opamp.py:13-103
* Switch              voltax/elements/switch.py:14-50
* EKVMOSFET           voltax/elements/mosfet.py:127-205 (softplus is
                      ``logaddexp(x, 0)`` as in ``jax.nn.softplus``)
* Constant/Step/Pulse voltax/signals.py:58-114

`local_jacobian` forms each device's ``(T+K) x (T+K)`` block of
``cf * d(I,F)/du + cq * d(Q,P)/du`` by forward-mode AD, one seed per local
unknown, as voltax/sparse.py:200-249 does with ``jax.jvp``.
"""

from __future__ import annotations

import math

import numpy as np
import torch

F64 = torch.float64


def _np(x):
    if isinstance(x, torch.Tensor):
        return x.detach().cpu().to(F64)
    return torch.as_tensor(np.asarray(x, dtype=np.float64))


def _inst(x, b):
    """Instance `b` of a parameter that may carry a leading instance axis."""
    x = _np(x)
    return x[b] if x.ndim == 2 else x


def softplus(x):
    return torch.logaddexp(x, torch.zeros_like(x))


def signal_value(sig, t, b):
    """Waveform value per device (voltax/signals.py:58-114)."""
    name = type(sig).__name__
    g = lambda f: _inst(getattr(sig, f), b)  # noqa: E731
    t = torch.as_tensor(t, dtype=F64)
    if name == "Constant":
        return g("value")
    if name == "Step":
        v0, v1, delay, rise = g("v0"), g("v1"), g("delay"), g("rise")
        frac = torch.clamp((t - delay) / rise, 0.0, 1.0)
        return v0 + (v1 - v0) * frac
    if name == "Pulse":
        v1, v2, delay = g("v1"), g("v2"), g("delay")
        rise, fall, width, period = g("rise"), g("fall"), g("width"), g("period")
        tc = torch.remainder(t - delay, period)
        up = torch.clamp(tc / (rise + 1e-30), 0.0, 1.0)
        t_fall_end = rise + width + fall
        down = torch.clamp((t_fall_end - tc) / (fall + 1e-30), 0.0, 1.0)
        value = v1 + (v2 - v1) * torch.minimum(up, down)
        return torch.where(t < delay, v1, value)
    raise NotImplementedError(name)


def _jmax(a, b):
    """max with the derivative split 1/2 : 1/2 at a tie (jnp.maximum)."""
    return torch.where(a > b, a, torch.where(a < b, b, 0.5 * (a + b)))


def _jmin(a, b):
    return torch.where(a < b, a, torch.where(a > b, b, 0.5 * (a + b)))


def _explin(u, u_max=40.0):
    """exp(u), continued linearly above u_max (semiconductor.py:17-24)."""
    e = torch.exp(_jmin(u, torch.full_like(u, u_max)))
    return torch.where(u > u_max, e * (1.0 + u - u_max), e)


class GroupModel:
    """One element group of one circuit instance."""

    def __init__(self, el, b: int = 0):
        self.el, self.b = el, b
        self.name = type(el).__name__
        self.T = len(el.terminals)
        self.K = el.n_internal
        self.has_charges = self.name in ("Capacitor", "EKVMOSFET", "Level1MOSFET", "Diode",
                                         "Inductor", "BJT", "Transformer", "OpAmp",
                                         "CoupledInductors")

    # ---------------------------------------------------------------- physics
    def currents(self, v, x, t):
        el, b, name = self.el, self.b, self.name
        if name == "Resistor":
            i = (v[..., 0] - v[..., 1]) * torch.exp(-_inst(el.log_r, b))
            return torch.stack([i, -i], -1), None
        if name == "Conductance":
            th = _inst(el.theta, b)
            if el.transform == "log":
                g = torch.exp(th)
            elif el.transform == "softplus":
                g = el.g_min + softplus(th)
            elif el.transform == "sigmoid":
                g = el.g_min + (el.g_max - el.g_min) * torch.sigmoid(th)
            else:
                g = th
            i = g * (v[..., 0] - v[..., 1])
            return torch.stack([i, -i], -1), None
        if name == "Capacitor":
            return None, None
        if name == "CoupledInductors":  # through(i), -(v_p - v_n)
            i = x[..., 0]
            return torch.stack([i, -i], -1), (-(v[..., 0] - v[..., 1]))[..., None]
        if name == "VoltageSource":
            i = x[..., 0]
            val = signal_value(el.value, t, b)
            return torch.stack([i, -i], -1), ((v[..., 0] - v[..., 1]) - val)[..., None]
        if name == "CurrentSource":
            i = torch.broadcast_to(signal_value(el.value, t, b), v.shape[:1])
            return torch.stack([i, -i], -1), None
        if name == "Diode":
            i = self._diode_current(v[..., 0] - v[..., 1])
            return torch.stack([i, -i], -1), None
        if name == "BJT":  # semiconductor.py:119-128
            s = 1.0 if el.polarity == "npn" else -1.0
            vbe, vbc, i_f, i_r = self._bjt_junctions(v, s)
            early = 1.0 + (vbe - vbc) * _inst(el.inv_vaf, b)
            ic = (i_f - i_r) * early - i_r * torch.exp(-_inst(el.log_br, b))
            ib = i_f * torch.exp(-_inst(el.log_bf, b)) + i_r * torch.exp(-_inst(el.log_br, b))
            return s * torch.stack([ic, ib, -ic - ib], -1), None
        if name == "Inductor":  # passive.py:62-87
            i = x[..., 0]
            rs = _inst(el.rs, b)
            return torch.stack([i, -i], -1), (rs * i - (v[..., 0] - v[..., 1]))[..., None]
        if name == "IdealOpAmp":  # opamp.py:28-32
            i = x[..., 0]
            z = torch.zeros_like(i)
            return torch.stack([z, z, -i], -1), (v[..., 0] - v[..., 1])[..., None]
        if name == "OpAmp":  # opamp.py:93-100
            st = x[..., 0]
            rout = torch.exp(_inst(el.log_rout, b))
            a0 = torch.exp(_inst(el.log_a0, b))
            vmin, vmax = _inst(el.vmin, b), _inst(el.vmax, b)
            mid, half = 0.5 * (vmax + vmin), 0.5 * (vmax - vmin)
            u_ = a0 * (v[..., 0] - v[..., 1])
            clip = mid + half * torch.tanh((u_ - mid) / half)
            i_out = (v[..., 2] - st) / rout
            z = torch.zeros_like(i_out)
            return torch.stack([z, z, i_out], -1), (st - clip)[..., None]
        if name == "Switch":  # switch.py:39-50
            on = torch.sigmoid((v[..., 2] - v[..., 3] - _inst(el.vth, b)) / _inst(el.vwidth, b))
            lroff, lron = _inst(el.log_roff, b), _inst(el.log_ron, b)
            g = torch.exp(-lroff + on * (lroff - lron))
            i = g * (v[..., 0] - v[..., 1])
            z = torch.zeros_like(i)
            return torch.stack([i, -i, z, z], -1), None
        if name == "VCVS":  # controlled.py:27-43
            i = x[..., 0]
            z = torch.zeros_like(i)
            f = (v[..., 0] - v[..., 1]) - _inst(el.gain, b) * (v[..., 2] - v[..., 3])
            return torch.stack([i, -i, z, z], -1), f[..., None]
        if name == "CCCS":  # controlled.py:63-79
            i_s = x[..., 0]
            i = _inst(el.gain, b) * i_s
            return torch.stack([i, -i, i_s, -i_s], -1), (v[..., 2] - v[..., 3])[..., None]
        if name == "CCVS":  # controlled.py:82-98
            i, i_s = x[..., 0], x[..., 1]
            f = torch.stack([(v[..., 0] - v[..., 1]) - _inst(el.r, b) * i_s,
                             v[..., 2] - v[..., 3]], -1)
            return torch.stack([i, -i, i_s, -i_s], -1), f
        if name == "Transformer":  # passive.py:120-123
            i1, i2 = x[..., 0], x[..., 1]
            f = -torch.stack([v[..., 0] - v[..., 1], v[..., 2] - v[..., 3]], -1)
            return torch.stack([i1, -i1, i2, -i2], -1), f
        if name == "VCCS":  # controlled.py:46-60
            i = _inst(el.gm, b) * (v[..., 2] - v[..., 3])
            z = torch.zeros_like(i)
            return torch.stack([i, -i, z, z], -1), None
        if name in ("EKVMOSFET", "Level1MOSFET"):
            s = self._sign()
            vd, vg, vs, vb = (s * v[..., k] for k in range(4))
            ids = (self._drain_current(vd, vg, vs, vb) if name == "EKVMOSFET"
                   else self._l1_current(vd, vg, vs, vb))
            zero = torch.zeros_like(ids)
            return s * torch.stack([ids, zero, -ids, zero], -1), None
        raise NotImplementedError(name)

    def charges(self, v, x):
        el, b, name = self.el, self.b, self.name
        if name == "Capacitor":
            q = torch.exp(_inst(el.log_c, b)) * (v[..., 0] - v[..., 1])
            return torch.stack([q, -q], -1), None
        if name == "EKVMOSFET":
            p = el.process
            s = self._sign()
            vd, vg, vs, vb = (s * v[..., k] for k in range(4))
            i_f, i_r = self._inversion(vd, vg, vs, vb)
            xf, xr = torch.sqrt(0.25 + i_f), torch.sqrt(0.25 + i_r)
            w, l = torch.exp(_inst(el.log_w, b)), torch.exp(_inst(el.log_l, b))
            cox, n, vt = torch.exp(_np(p.log_cox)), _np(p.n), _np(p.vt)
            c_ox = cox * w * l
            scale = c_ox * n * vt
            ssum = xf + xr
            q_d = -scale * ((4 / 15) * (3 * xr**3 + 6 * xr**2 * xf + 4 * xr * xf**2
                                        + 2 * xf**3) / ssum**2 - 0.5)
            q_s = -scale * ((4 / 15) * (3 * xf**3 + 6 * xf**2 * xr + 4 * xf * xr**2
                                        + 2 * xr**3) / ssum**2 - 0.5)
            q_i = q_d + q_s
            q_b = -(n - 1) / n * (c_ox * (vg - vb) + q_i)
            q_g = -(q_i + q_b)
            intrinsic = torch.stack([q_d, q_g, q_s, q_b], -1)
            cov = torch.exp(_np(p.log_cov)) * w
            q_gs, q_gd = cov * (vg - vs), cov * (vg - vd)
            overlap = torch.stack([-q_gd, q_gs + q_gd, -q_gs, torch.zeros_like(q_gs)], -1)
            return s * (intrinsic + overlap), None
        if name == "BJT":  # semiconductor.py:130-135
            s = 1.0 if el.polarity == "npn" else -1.0
            vbe, vbc, i_f, i_r = self._bjt_junctions(v, s)
            q_be = _inst(el.tf, b) * i_f + _inst(el.cje, b) * vbe
            q_bc = _inst(el.tr, b) * i_r + _inst(el.cjc, b) * vbc
            return s * torch.stack([-q_bc, q_be + q_bc, -q_be], -1), None
        if name == "Diode":  # q = tt i + cj v (semiconductor.py:68-70)
            vd = v[..., 0] - v[..., 1]
            q = _inst(el.tt, b) * self._diode_current(vd) + _inst(el.cj, b) * vd
            return torch.stack([q, -q], -1), None
        if name == "Inductor":
            return None, (torch.exp(_inst(el.log_l, b)) * x[..., 0])[..., None]
        if name == "OpAmp":  # opamp.py:102-103: tau x on the state row
            tau = torch.exp(_inst(el.log_a0, b)) / (2 * math.pi * torch.exp(_inst(el.log_gbw, b)))
            return None, (tau * x[..., 0])[..., None]
        if name == "CoupledInductors":  # M = k sqrt(l l^T) (1 - I) + diag(l)
            ll = torch.exp(_inst(el.log_l, b))
            root = torch.sqrt(ll)
            n = ll.shape[0]
            M = el.k * torch.outer(root, root) * (1 - torch.eye(n, dtype=F64)) + torch.diag(ll)
            return None, (M @ x[..., 0])[..., None]
        if name == "Transformer":  # passive.py:125-129
            i1, i2 = x[..., 0], x[..., 1]
            l1, l2 = torch.exp(_inst(el.log_l1, b)), torch.exp(_inst(el.log_l2, b))
            m = _inst(el.k, b) * torch.sqrt(l1 * l2)
            return None, torch.stack([l1 * i1 + m * i2, m * i1 + l2 * i2], -1)
        if name == "Level1MOSFET":  # overlap charges only (mosfet.py:255-257)
            s = self._sign()
            vd, vg, vs, vb = (s * v[..., k] for k in range(4))
            w = torch.exp(_inst(el.log_w, b))
            cov = torch.exp(_np(el.process.log_cov)) * w
            q_gs, q_gd = cov * (vg - vs), cov * (vg - vd)
            overlap = torch.stack([-q_gd, q_gs + q_gd, -q_gs, torch.zeros_like(q_gs)], -1)
            return s * overlap, None
        return None, None

    def _sign(self):
        return 1.0 if self.el.polarity == "n" else -1.0

    def _inversion(self, vd, vg, vs, vb):
        el, b = self.el, self.b
        p = el.process
        vth, n, vt = _np(p.vth), _np(p.n), _np(p.vt)
        vp = (vg - vb - vth - _inst(el.dvth, b)) / n
        i_f = softplus((vp - (vs - vb)) / (2 * vt)) ** 2
        i_r = softplus((vp - (vd - vb)) / (2 * vt)) ** 2
        return i_f, i_r

    def _bjt_junctions(self, v, s):
        el, b = self.el, self.b
        vc, vb, ve = (s * v[..., k] for k in range(3))
        vbe, vbc = vb - ve, vb - vc
        i_s, vt = torch.exp(_inst(el.log_is, b)), _inst(el.vt, b)
        return vbe, vbc, i_s * (_explin(vbe / vt) - 1.0), i_s * (_explin(vbc / vt) - 1.0)

    def _diode_current(self, vd):
        """is (explin(vd / (n vt)) - 1), explin linear above 40
        (semiconductor.py:17-24, 62-63)."""
        el, b = self.el, self.b
        u = vd / (_inst(el.n, b) * _inst(el.vt, b))
        return torch.exp(_inst(el.log_is, b)) * (_explin(u) - 1.0)

    # Level 1 (mosfet.py:229-253). jnp.maximum / jnp.minimum give each side
    # half the derivative at a tie; _jmax / _jmin do the same under torch AD.
    def _l1_threshold(self, vsb):
        el, b = self.el, self.b
        p = el.process
        phi, gamma = _np(p.phi), _np(p.gamma)
        sphi = torch.sqrt(torch.as_tensor(phi, dtype=F64))
        zero = torch.zeros_like(vsb)
        reverse = torch.sqrt(phi + _jmax(vsb, zero))
        forward = _jmax(sphi + _jmin(vsb, zero) / (2 * sphi), zero)
        root = torch.where(vsb >= 0, reverse, forward)
        return _np(p.vth) + _inst(el.dvth, b) + gamma * (root - sphi)

    def _l1_forward(self, vgs, vds, vth):
        el, b = self.el, self.b
        p, sm = el.process, el.smooth
        k = torch.exp(_np(p.log_kp)) * torch.exp(_inst(el.log_w, b)) / torch.exp(
            _inst(el.log_l, b))
        if sm > 0:
            vov = sm * softplus((vgs - vth) / sm)
        else:
            vov = _jmax(vgs - vth, torch.zeros_like(vgs))
        vde = _jmin(vds, vov)
        return k * (vov - 0.5 * vde) * vde * (1.0 + _np(p.lam) * vds)

    def _l1_current(self, vd, vg, vs, vb):
        vds = vd - vs
        zero = torch.zeros_like(vds)
        fwd = self._l1_forward(vg - vs, _jmax(vds, zero), self._l1_threshold(vs - vb))
        rev = self._l1_forward(vg - vd, _jmax(-vds, zero), self._l1_threshold(vd - vb))
        return fwd - rev

    def _drain_current(self, vd, vg, vs, vb):
        el, b = self.el, self.b
        p = el.process
        i_f, i_r = self._inversion(vd, vg, vs, vb)
        w, l = torch.exp(_inst(el.log_w, b)), torch.exp(_inst(el.log_l, b))
        n, vt, lam = _np(p.n), _np(p.vt), _np(p.lam)
        i_spec = 2 * n * torch.exp(_np(p.log_kp)) * (w / l) * vt**2
        vds = vd - vs
        soft_abs = torch.sqrt(vds * vds + 1e-3 * 1e-3) - 1e-3
        return i_spec * (i_f - i_r) * (1.0 + lam * soft_abs)

    # ------------------------------------------------------------ local blocks
    def outputs(self, u, t, cf, cq):
        """``cf * currents + cq * charges`` of all devices, ``u`` (N, T+K)."""
        n, T, k = u.shape[0], self.T, self.K

        def part(A, B):
            A = torch.zeros((n, T), dtype=F64) if A is None else torch.broadcast_to(A, (n, T))
            B = torch.zeros((n, k), dtype=F64) if (B is None or k == 0) else B
            return torch.cat([A, B], 1)

        v, x = u[:, :T], u[:, T:]
        out = torch.zeros((n, T + k), dtype=F64)
        if cf != 0:
            out = out + cf * part(*self.currents(v, x, t))
        if cq != 0:
            out = out + cq * part(*self.charges(v, x))
        return out

    def group_jacobian(self, u, t, cf, cq):
        """A non-local group's ``(N m, N m)`` block ``d out / d u`` over all
        its unknowns, device-major (voltax/sparse.py:245-247's jacfwd)."""
        n, m = u.shape
        flat = lambda uu: self.outputs(uu.reshape(n, m), t, cf, cq).reshape(-1)  # noqa: E731
        return torch.func.jacfwd(flat)(u.reshape(-1))

    def local_jacobian(self, u, t, cf, cq):
        """``(N, m, m)`` blocks ``d out[d, i] / d u[d, j]`` by forward-mode AD
        (one seed per local unknown, all devices at once)."""
        n, m = u.shape
        cols = []
        for j in range(m):
            seed = torch.zeros((n, m), dtype=F64)
            seed[:, j] = 1.0
            _, tan = torch.func.jvp(lambda uu: self.outputs(uu, t, cf, cq), (u,), (seed,))
            cols.append(tan)
        return torch.stack(cols, -1)  # (N, out i, in j)
