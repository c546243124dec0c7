"""Tile shapes of the matvec kernels: every FP32 shape the autotuner can pick (register-K2b threads 64/128/256 x
z-FFT y-lines 8/16/32 x x-FFT y-lines 4/8) gives the oracle's matvec on lattices whose y axis takes the register K2b
with 8 and with 16 lanes per line (y axes of 64, 256 and 512), and so does the generic K2b with 2, 4 and 8 pairs per block; axes longer than 512 (600 along each axis, 1024 along x) run with the narrow
tiles the library picks for them, in FP64 and FP32, against the oracle; an unsupported shape is refused; and the
tuner leaves a shape the build holds."""
import itertools

import numpy as np
import pytest

from helpers import oracle_for, rel

pytestmark = pytest.mark.gpu

TUNER = list(itertools.product((4, 8), (8, 16, 32), (64, 128, 256)))  # (w1, w2, threads); pairs stay 8


def box_setup(box, m=1.3 + 0.05j, dpl=12.0):
    """a fully occupied box with the reference's grid (fftFit of twice the box, z even)"""
    import adda_gb300 as A
    s = A.Setup(grid=box[0], shape="box", pars=(box[1] / box[0], box[2] / box[0]), m=m, dpl=dpl)
    assert tuple(s.box) == tuple(box), (s.box, box)
    return s


def check_matvec(s, ctx, o, precs=("fp64", "fp32")):
    x = np.random.default_rng(9).standard_normal((2, 3 * s.n)) + 1j * np.random.default_rng(10).standard_normal(
        (2, 3 * s.n))
    for her in (False, True):
        ys = {p: ctx.matvec(x, p, her)[0] for p in precs}
        for r in range(2):
            o.set_cc(s.cc[r].reshape(1, 3))
            yr, _ = o.matvec(x[r], her)
            if "fp64" in ys:
                assert rel(ys["fp64"][r], yr) < 1e-13
            if "fp32" in ys:
                assert rel(ys["fp32"][r], yr) < 5e-6


@pytest.mark.parametrize("box", [(32, 32, 32), (8, 128, 8), (4, 256, 4)],
                         ids=["grid64_lanes8", "gridY256_lanes16", "gridY512_lanes16"])
def test_every_tuner_shape_matches_oracle(box):
    import adda_gb300 as A
    s = box_setup(box)
    o = oracle_for(s)
    ctx = A.Context.from_setup(s, nrhs_max=2)
    for w1, w2, nt in TUNER:
        ctx.set_fft_shape((w1, w2, 8, nt))
        assert ctx.fft_shape() == (w1, w2, 8, nt)
        check_matvec(s, ctx, o, precs=("fp32",))
    o.close()
    ctx.close()


@pytest.mark.parametrize("box", [(300, 4, 6), (4, 300, 6), (4, 6, 300), (512, 2, 2)],
                         ids=["x600", "y600", "z600", "x1024"])
def test_long_axes_match_oracle(box):
    import adda_gb300 as A
    s = box_setup(box)
    assert max(s.grid) > 512
    o = oracle_for(s)
    ctx = A.Context.from_setup(s, nrhs_max=2)
    for prec in ("fp64", "fp32"):
        w1, w2, pairs, _ = ctx.fft_shape(prec)
        if s.grid[0] > 512:
            assert w1 == 1
        if s.grid[1] > 512:
            assert pairs == 1
    check_matvec(s, ctx, o)
    res = ctx.solve(np.stack(s.einc), prec="fp64", eps=1e-8)
    o.set_cc(s.cc[0].reshape(1, 3))
    assert rel(res["p"][0], o.solve(s.einc[0], eps=1e-8)["p"]) < 1e-7
    o.close()
    ctx.close()


@pytest.mark.parametrize("pairs", [2, 4, 8])
def test_generic_k2b_pairs_match_oracle(pairs):
    """the generic K2b (y axis not 64/128/256: here 40) with every pair count the tuner can pick"""
    import adda_gb300 as A
    s = box_setup((16, 20, 12))
    o = oracle_for(s)
    ctx = A.Context.from_setup(s, nrhs_max=2)
    ctx.set_fft_shape((8, 16, pairs, 128))
    check_matvec(s, ctx, o, precs=("fp32",))
    o.close()
    ctx.close()


def test_shape_refused_and_tuned_shape_is_built():
    import adda_gb300 as A
    s = box_setup((32, 32, 32))
    ctx = A.Context.from_setup(s, nrhs_max=2)
    with pytest.raises(A.AddaError):
        ctx.set_fft_shape((3, 16, 8, 128))           # 3 y-lines per block: not built
    with pytest.raises(A.AddaError):
        ctx.set_fft_shape((1, 16, 8, 128))           # narrow tiles: only for axes longer than 512
    ctx.close()
    ctx = A.Context.from_setup(s, nrhs_max=2)
    ctx.time_matvec("fp32", 2, iters=1)              # the first FP32 matvec tunes the shape
    w1, w2, pairs, nt = ctx.fft_shape()
    assert (w1, w2, nt) in TUNER and pairs == 8
    ctx.close()
