"""The device-buffer entry points order themselves with the caller's stream: a solve or matvec called right after a
caller queued the fill of its inputs behind a long kernel on torch's default stream (the legacy default stream) or on
a stream of its own given to adda_gb300_set_stream reads the filled inputs, not what the buffer held before, and gives
the result of the same call made after a full synchronisation."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
SLEEP_CYCLES = 20_000_000  # about 10 ms of a bounded busy-wait kernel before the fill


def make_case():
    import torch

    import adda_gb300 as A
    s = A.Setup(grid=12, shape="box", m=1.3 + 0.05j, dpl=12.0)
    ctx = A.Context.from_setup(s, nrhs_max=2)
    e = torch.from_numpy(np.ascontiguousarray(np.stack(s.einc)).view(np.float64)).cuda()
    rng = np.random.default_rng(3)
    x0 = torch.from_numpy((rng.standard_normal((2, 3 * s.n)) + 1j * rng.standard_normal((2, 3 * s.n))).view(
        np.float64)).cuda()
    return s, ctx, e, x0


def solve_from(ctx, e, d_x):
    return ctx.solve_device(e.data_ptr(), 2, d_x.data_ptr(), None, method="qmr", prec="fp64", eps=1e-300,
                            maxiter=3, init="x0")


@pytest.mark.parametrize("own_stream", [False, True], ids=["default_stream", "set_stream"])
def test_solve_device_reads_inputs_filled_on_the_callers_stream(own_stream):
    import torch
    s, ctx, e, x0 = make_case()
    want = x0.clone()
    torch.cuda.synchronize()
    solve_from(ctx, e, want)
    torch.cuda.synchronize()
    stream = torch.cuda.Stream() if own_stream else torch.cuda.default_stream()
    ctx.set_stream(stream if own_stream else None)
    got = torch.full_like(x0, 7.0)
    torch.cuda.synchronize()
    with torch.cuda.stream(stream):
        torch.cuda._sleep(SLEEP_CYCLES)
        got.copy_(x0)
    solve_from(ctx, e, got)
    torch.cuda.synchronize()
    assert torch.equal(got, want)
    ctx.close()


def test_matvec_device_orders_with_the_callers_stream():
    import torch

    import adda_gb300 as A
    s, ctx, e, x0 = make_case()
    y_want = torch.empty_like(x0)
    torch.cuda.synchronize()
    rc = ctx.L.adda_gb300_matvec_device(ctx.h, A.PREC["fp64"], 2, ctypes.c_void_p(x0.data_ptr()),
                                        ctypes.c_void_p(y_want.data_ptr()), None, 0)
    assert rc == 0
    torch.cuda.synchronize()
    x = torch.full_like(x0, 7.0)
    y = torch.empty_like(x0)
    torch.cuda.synchronize()
    torch.cuda._sleep(SLEEP_CYCLES)
    x.copy_(x0)
    rc = ctx.L.adda_gb300_matvec_device(ctx.h, A.PREC["fp64"], 2, ctypes.c_void_p(x.data_ptr()),
                                        ctypes.c_void_p(y.data_ptr()), None, 0)
    assert rc == 0
    y2 = y.clone()  # queued on the default stream after the call: sees the matvec's result
    torch.cuda.synchronize()
    assert torch.equal(y2, y_want)
    ctx.close()
