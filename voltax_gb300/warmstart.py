"""Learned Newton warm start for batched DC operating points.

voltax starts every DC Newton solve from the caller's guess or from zeros
(voltax/analysis.py:410-431); far from the root the damping (``max_dv``)
and gmin stepping (voltax/analysis.py:236-266) make that tens of
iterations. Here a small MLP, trained on operating points the solver itself
produced, predicts each instance's node voltages from its parameter vector,
and Newton starts there:

* `WarmStartMLP` -- inputs -> hidden -> hidden -> node voltages, GELU on the
  hidden layers, BF16 weights and activations, FP32 accumulation. Forward,
  backward, loss and Adam all run in libvxg's own kernels (``vxg_mlp_*``);
  this class only owns the buffers and the schedule. Inputs and targets are
  standardised per column; the last layer writes the de-normalised
  prediction straight into the Newton state.
* `dc` -- the DC analysis from the predicted guess: the direct Newton
  attempt (``direct_steps`` iterations) from the prediction; instances it
  does not converge fall back to the plain path, i.e. the direct attempt
  and gmin stepping from the default guess (zeros), as `analysis.dc` does.
  Iteration counts include the failed warm attempt.
* `solve_dataset` -- operating points of a parameter set by the plain
  solver, in chunks (the training data).
"""

from __future__ import annotations

import dataclasses
import math

import numpy as np
import torch

from . import _lib as L
from .analysis import Options, Solution, _Call
from .runtime import cuda_device, stream_ptr


def _p(t: torch.Tensor | None, off: int = 0) -> int | None:
    if t is None:
        return None
    return t.data_ptr() + off * t.element_size()


class WarmStartMLP:
    """``n_in -> hidden -> hidden -> n_out`` MLP (GELU, BF16 weights)."""

    def __init__(self, n_in: int, n_out: int, hidden: int = 512, seed: int = 0,
                 device: torch.device | None = None):
        self.lib = L.load()
        self.dev = cuda_device() if device is None else torch.device(device)
        self.dims = (n_in, hidden, hidden, n_out)
        # one flat FP32 master buffer: W1 b1 W2 b2 W3 b3, each W at a
        # multiple of 8 elements (16-byte aligned BF16 copies)
        self.offsets = []
        o = 0
        for i in range(3):
            N, K = self.dims[i + 1], self.dims[i]
            self.offsets.append((o, o + N * K))
            o = (o + N * K + N + 7) // 8 * 8
        self.n_params = o
        rng = np.random.default_rng(seed)
        w = np.zeros(o, np.float32)
        for i, (ow, _) in enumerate(self.offsets):
            N, K = self.dims[i + 1], self.dims[i]
            a = math.sqrt(3.0 / K)  # variance 1 / fan_in
            w[ow:ow + N * K] = rng.uniform(-a, a, N * K)
        f32 = dict(dtype=torch.float32, device=self.dev)
        self.w = torch.from_numpy(w).to(self.dev)
        self.wb = torch.empty(o, dtype=torch.bfloat16, device=self.dev)
        self.g = torch.zeros(o, **f32)
        self.m = torch.zeros(o, **f32)
        self.v = torch.zeros(o, **f32)
        self.step = 0
        self.x_mean = torch.zeros(n_in, **f32)
        self.x_istd = torch.ones(n_in, **f32)
        self.y_mean = torch.zeros(n_out, **f32)
        self.y_std = torch.ones(n_out, **f32)
        self.loss = torch.zeros(1, **f32)
        self._scratch = torch.zeros(256, **f32)
        self._bufs: dict[int, dict] = {}
        self._check(self.lib.vxg_mlp_adam(o, _p(self.w), _p(self.wb), None, None, None, 0.0,
                                          0.0, 0.0, 0.0, 0, stream_ptr()), "vxg_mlp_adam")

    # ------------------------------------------------------------ plumbing
    @staticmethod
    def _check(status, what):
        L.check(status, what)

    def layers(self) -> list[tuple[np.ndarray, np.ndarray]]:
        """The FP32 master weights as ``[(W (out, in), b (out,)), ...]``."""
        w = self.w.cpu().numpy()
        out = []
        for i, (ow, ob) in enumerate(self.offsets):
            N, K = self.dims[i + 1], self.dims[i]
            out.append((w[ow:ow + N * K].reshape(N, K).copy(), w[ob:ob + N].copy()))
        return out

    def grads(self) -> list[tuple[np.ndarray, np.ndarray]]:
        g = self.g.cpu().numpy()
        out = []
        for i, (ow, ob) in enumerate(self.offsets):
            N, K = self.dims[i + 1], self.dims[i]
            out.append((g[ow:ow + N * K].reshape(N, K).copy(), g[ob:ob + N].copy()))
        return out

    def set_normalization(self, X, V):
        """Per-column mean / standard deviation of inputs and targets
        (columns that do not vary get a unit scale)."""
        X = torch.as_tensor(X, dtype=torch.float64)
        V = torch.as_tensor(V, dtype=torch.float64)
        xs = X.std(0)
        ys = V.std(0)
        self.x_mean.copy_(X.mean(0).float())
        self.x_istd.copy_(torch.where(xs > 1e-12, 1.0 / xs, torch.ones_like(xs)).float())
        self.y_mean.copy_(V.mean(0).float())
        self.y_std.copy_(torch.where(ys > 1e-12, ys, torch.ones_like(ys)).float())

    def _buffers(self, M: int, train: bool) -> dict:
        key = (M, train)
        if key not in self._bufs:
            n_in, H, _, N = self.dims
            bf = dict(dtype=torch.bfloat16, device=self.dev)
            f32 = dict(dtype=torch.float32, device=self.dev)
            b = {"x": torch.empty((M, n_in), **bf), "h1": torch.empty((M, H), **bf),
                 "h2": torch.empty((M, H), **bf)}
            if train:
                b.update(pre1=torch.empty((M, H), **f32), pre2=torch.empty((M, H), **f32),
                         y=torch.empty((M, N), **f32), dy=torch.empty((M, N), **bf),
                         d2=torch.empty((M, H), **bf), d1=torch.empty((M, H), **bf))
            self._bufs[key] = b
        return self._bufs[key]

    def _linear(self, i, M, x, act, pre=None, y=None, yf=None, z=None, ldz=0):
        N, K = self.dims[i + 1], self.dims[i]
        ow, ob = self.offsets[i]
        scale = _p(self.y_std) if z is not None else None
        shift = _p(self.y_mean) if z is not None else None
        self._check(self.lib.vxg_mlp_linear(M, N, K, _p(x), _p(self.wb, ow), _p(self.w, ob), act,
                                            _p(pre), _p(y), _p(yf), scale, shift, _p(z), ldz,
                                            stream_ptr()), "vxg_mlp_linear")

    # ------------------------------------------------------------- forward
    def forward(self, x: torch.Tensor, rows: torch.Tensor | None = None, train=False):
        """Normalised outputs (FP32) of the rows of x (float64, device)."""
        M = int(rows.numel()) if rows is not None else int(x.shape[0])
        b = self._buffers(M, True)
        self._forward(x, rows, b, M, train=True)
        return b["y"][:M]

    def _forward(self, x, rows, b, M, train, z=None):
        n_in = self.dims[0]
        self._check(self.lib.vxg_mlp_normalize(M, n_in, _p(x), x.stride(0), _p(rows),
                                               _p(self.x_mean), _p(self.x_istd), _p(b["x"]),
                                               stream_ptr()), "vxg_mlp_normalize")
        G, N0 = L.VXG_ACT_GELU, L.VXG_ACT_NONE
        self._linear(0, M, b["x"], G, pre=b.get("pre1") if train else None, y=b["h1"])
        self._linear(1, M, b["h1"], G, pre=b.get("pre2") if train else None, y=b["h2"])
        if z is None:
            self._linear(2, M, b["h2"], N0, yf=b["y"])
        else:
            self._linear(2, M, b["h2"], N0, z=z, ldz=z.stride(0))

    def predict_into(self, x: torch.Tensor, z: torch.Tensor, chunk: int = 16384) -> None:
        """Write the predicted node voltages of each row of x into z[:, :n_out]."""
        x = torch.as_tensor(x, dtype=torch.float64, device=self.dev).contiguous()
        assert z.dtype == torch.float64 and z.is_contiguous() and z.shape[0] == x.shape[0]
        for s in range(0, x.shape[0], chunk):
            M = min(chunk, x.shape[0] - s)
            b = self._buffers(min(chunk, x.shape[0]), False)
            self._forward(x[s:s + M], None, b, M, train=False, z=z[s:s + M])

    # ------------------------------------------------------------ training
    def train_step(self, x: torch.Tensor, t: torch.Tensor, rows: torch.Tensor, lr: float,
                   beta1=0.9, beta2=0.999, eps=1e-8) -> None:
        """One Adam step on the minibatch `rows` of (x, t): t holds the
        normalised targets (float32). The loss lands in ``self.loss``."""
        lib, s = self.lib, stream_ptr()
        M = int(rows.numel())
        n_in, H, _, N = self.dims
        b = self._buffers(M, True)
        self._forward(x, rows, b, M, train=True)
        self._check(lib.vxg_mlp_mse(M, N, _p(b["y"]), _p(t), _p(rows), _p(b["dy"]),
                                    _p(self.loss), _p(self._scratch), s), "vxg_mlp_mse")
        self.backward(b, M)
        self.step += 1
        self._check(lib.vxg_mlp_adam(self.n_params, _p(self.w), _p(self.wb), _p(self.g),
                                     _p(self.m), _p(self.v), lr, beta1, beta2, eps, self.step,
                                     s), "vxg_mlp_adam")

    def backward(self, b: dict, M: int) -> None:
        """Gradients into ``self.g`` from the output gradient in b["dy"]."""
        lib, s = self.lib, stream_ptr()
        n_in, H, _, N = self.dims
        (w1, c1), (w2, c2), (w3, c3) = self.offsets
        g = self.g
        self._check(lib.vxg_mlp_linear_dw(M, N, H, _p(b["dy"]), _p(b["h2"]), _p(g, w3), _p(g, c3),
                                          s), "vxg_mlp_linear_dw")
        self._check(lib.vxg_mlp_linear_dx(M, N, H, _p(b["dy"]), _p(self.wb, w3), _p(b["pre2"]),
                                          _p(b["d2"]), s), "vxg_mlp_linear_dx")
        self._check(lib.vxg_mlp_linear_dw(M, H, H, _p(b["d2"]), _p(b["h1"]), _p(g, w2), _p(g, c2),
                                          s), "vxg_mlp_linear_dw")
        self._check(lib.vxg_mlp_linear_dx(M, H, H, _p(b["d2"]), _p(self.wb, w2), _p(b["pre1"]),
                                          _p(b["d1"]), s), "vxg_mlp_linear_dx")
        self._check(lib.vxg_mlp_linear_dw(M, H, n_in, _p(b["d1"]), _p(b["x"]), _p(g, w1),
                                          _p(g, c1), s), "vxg_mlp_linear_dw")

    def fit(self, X, V, epochs: int = 30, batch: int = 1024, lr: float = 2e-3,
            lr_final: float = 2e-5, seed: int = 0, log=None) -> list[float]:
        """Train on parameter rows X (n, n_in) and operating points V
        (n, n_out); cosine learning-rate decay from lr to lr_final. Returns
        the mean minibatch loss of each epoch (normalised units)."""
        X = torch.as_tensor(X, dtype=torch.float64).to(self.dev).contiguous()
        V = torch.as_tensor(V, dtype=torch.float64).to(self.dev)
        self.set_normalization(X, V)
        T = ((V - self.y_mean.double()) / self.y_std.double()).float().contiguous()
        n = X.shape[0]
        per_epoch = max(n // batch, 1)
        total = epochs * per_epoch
        rng = np.random.default_rng(seed)
        history = []
        acc = torch.zeros(1, dtype=torch.float32, device=self.dev)
        k = 0
        for ep in range(epochs):
            perm = torch.from_numpy(rng.permutation(n).astype(np.int64)).to(self.dev)
            acc.zero_()
            for i in range(per_epoch):
                rows = perm[i * batch:(i + 1) * batch] if n >= batch else perm
                cur = lr_final + 0.5 * (lr - lr_final) * (1 + math.cos(math.pi * k / total))
                self.train_step(X, T, rows, cur)
                acc += self.loss
                k += 1
            history.append(float(acc) / per_epoch)
            if log:
                log(f"epoch {ep}: loss {history[-1]:.3e}")
        return history


# ---------------------------------------------------------------------------
# Analyses
# ---------------------------------------------------------------------------


def dc(circuit, params, model: WarmStartMLP, t: float = 0.0,
       options: Options = Options()) -> Solution:
    """DC operating points of a batched circuit from the MLP's prediction,
    with plain Newton from the default guess as the fallback."""
    call = _Call(circuit, options)
    eng, o = call.eng, options
    if eng.n_seg != 1:
        raise ValueError("the warm start needs one instance per batch row")
    B, S = call.B, eng.S
    z = torch.zeros((B, S), dtype=torch.float64, device=eng.device)
    model.predict_into(params, z)
    if call.fused:
        call.o = dataclasses.replace(o, gmin_steps=0, max_steps=o.direct_steps)
        try:  # the direct attempt alone
            z_out, conv, iters = call.fused_run(L.VXG_MODE_DC, np.array([float(t)]), z, True)
        finally:
            call.o = o
        z, conv, total = z_out[0], conv[0], iters[0].clone()
        failed = conv == 0
        if bool(failed.any()):
            zero = torch.zeros_like(z)
            zf, cf, itf = call.fused_run(L.VXG_MODE_DC, np.array([float(t)]), zero, True)
            z = torch.where(failed[:, None], zf[0], z)
            conv = torch.where(failed, cf[0], conv)
            total = total + torch.where(failed, itf[0], torch.zeros_like(total))
    else:
        conv, iters = call.newton(L.VXG_MODE_DC, z, t, gmin=o.gmin, max_steps=o.direct_steps)
        total = iters.clone()
        failed = (conv == 0).to(torch.int32)
        if bool(failed.any()):
            z = torch.where(failed.bool()[:, None], torch.zeros_like(z), z).contiguous()
            steps = o.direct_steps if o.gmin_steps else None
            cd, itd = call.newton(L.VXG_MODE_DC, z, t, gmin=o.gmin, max_steps=steps, mask=failed)
            total = total + torch.where(failed.bool(), itd, torch.zeros_like(itd))
            conv = torch.where(failed.bool(), cd, conv)
            still = (failed.bool() & (cd == 0)).to(torch.int32)
            if o.gmin_steps and bool(still.any()):
                z = torch.where(still.bool()[:, None], torch.zeros_like(z), z).contiguous()
                gmins = np.logspace(np.log10(o.gmin_start), np.log10(o.gmin), o.gmin_steps)
                for g in gmins:
                    ck, ik = call.newton(L.VXG_MODE_DC, z, t, gmin=float(g), mask=still)
                    total = total + torch.where(still.bool(), ik, torch.zeros_like(ik))
                    conv = torch.where(still.bool(), ck, conv)
    return Solution(torch.as_tensor(t, dtype=torch.float64), z, conv.bool(), circuit.layout,
                    total)


def solve_dataset(make_circuit, X: np.ndarray, chunk: int = 20000,
                  options: Options = Options(), t: float = 0.0):
    """Operating points of every parameter row of X by the plain solver
    (default guess, gmin stepping), `chunk` instances per batched solve.
    Returns (V (n, n_nodes) float64 on the GPU, converged, iterations)."""
    from . import analysis
    V, conv, iters = [], [], []
    for s in range(0, len(X), chunk):
        c = make_circuit(X[s:s + chunk])
        sol = analysis.dc(c, t=t, options=options)
        nv = c.layout.n_nodes
        V.append(sol.z.reshape(-1, sol.z.shape[-1])[:, :nv])
        conv.append(sol.converged.reshape(-1))
        iters.append(sol.iterations.reshape(-1))
    return torch.cat(V), torch.cat(conv), torch.cat(iters)
