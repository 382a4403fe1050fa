"""The generic engine's Newton loop runs on the device (a CUDA graph whose
conditional WHILE node repeats one Newton iteration), with its counters in
the caller's workspace:

* two threads calling vxg_newton on ONE handle, each with its own stream,
  workspace and buffers, get exactly the results of serial calls;
* the iteration limit is honoured (max_steps 1 stops after one iteration), and
  a repeated call (a cached graph) reproduces the first bit for bit.
"""

import ctypes as C
import threading

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

import voltax_gb300 as vx  # noqa: E402
from voltax_gb300 import _lib as L  # noqa: E402
from voltax_gb300 import workloads  # noqa: E402
from voltax_gb300.analysis import _Call  # noqa: E402


def _newton(call, z, conv, iters, ws, stream, max_steps=None):
    o = call.o.native(max_steps, refine=call.refine)
    L.check(call.eng.lib.vxg_newton(
        call.eng.handle, call.B, call.params, L.VXG_MODE_DC, 0.0, 0.0, None, None,
        call.o.gmin, C.byref(o), z.data_ptr(), conv.data_ptr(), iters.data_ptr(), None,
        ws.data_ptr(), stream), "vxg_newton")


def _buffers(call):
    dev = call.eng.device
    n = C.c_size_t()
    L.check(call.eng.lib.vxg_workspace_size(call.eng.handle, call.B, call.prec, C.byref(n)),
            "vxg_workspace_size")
    return (torch.zeros((call.B, call.eng.S), dtype=torch.float64, device=dev),
            torch.zeros(call.n_inst, dtype=torch.int32, device=dev),
            torch.zeros(call.n_inst, dtype=torch.int32, device=dev),
            torch.empty(n.value, dtype=torch.uint8, device=dev))


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_two_threads_on_one_handle_match_serial_calls(precision):
    opts = vx.Options(engine="generic", precision=precision)
    calls = [_Call(workloads.power_grid(40, seed=s), opts) for s in (1, 2)]
    assert calls[0].eng.handle == calls[1].eng.handle  # one topology, one handle
    serial = []
    for call in calls:
        z, conv, iters, ws = _buffers(call)
        _newton(call, z, conv, iters, ws, torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        serial.append((z.clone(), conv.clone(), iters.clone()))
        assert bool(conv.all()) and int(iters.max()) >= 2
    out = [None, None]
    errors = []

    def worker(k):
        try:
            call = calls[k]
            stream = torch.cuda.Stream()
            with torch.cuda.stream(stream):
                z, conv, iters, ws = _buffers(call)
                for _ in range(4):
                    z.zero_()
                    _newton(call, z, conv, iters, ws, stream.cuda_stream)
            stream.synchronize()
            out[k] = (z, conv, iters)
        except Exception as e:  # reported on the main thread
            errors.append(e)

    threads = [threading.Thread(target=worker, args=(k,)) for k in (0, 1)]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    assert not errors, errors
    for k in (0, 1):
        assert torch.equal(out[k][0], serial[k][0]), f"thread {k}: states differ"
        assert torch.equal(out[k][1], serial[k][1]) and torch.equal(out[k][2], serial[k][2])


def test_iteration_limit_and_cached_graph():
    call = _Call(workloads.power_grid(30, seed=3), vx.Options(engine="generic"))
    z, conv, iters, ws = _buffers(call)
    s = torch.cuda.current_stream().cuda_stream
    z.zero_()
    _newton(call, z, conv, iters, ws, s, max_steps=1)
    torch.cuda.synchronize()
    assert int(iters.max()) == 1 and not bool(conv.all())  # the first step moves ~1 V
    z.zero_()
    _newton(call, z, conv, iters, ws, s, max_steps=2)
    torch.cuda.synchronize()
    assert int(iters.max()) <= 2
    results = []
    for _ in range(2):  # the second call launches the cached graph
        z.zero_()
        _newton(call, z, conv, iters, ws, s)
        torch.cuda.synchronize()
        results.append((z.clone(), iters.clone()))
        assert bool(conv.all())
    assert torch.equal(results[0][0], results[1][0])
    assert torch.equal(results[0][1], results[1][1])
    ref = vx.dc(workloads.power_grid(30, seed=3), options=vx.Options(engine="generic"))
    np.testing.assert_array_equal(results[0][0][0].cpu().numpy(), ref.z.cpu().numpy())
