"""The FP32 transforms add and subtract complex float2 values with Blackwell's packed add/sub.rn.f32x2; a library
built with -DADDA_NO_F32X2 does the same sums with scalar round-to-nearest adds. Both must give the same bits: the
FP32 matvec (power-of-two grids through the register K2b, grids with radices 3/5/7 through the shared-memory
transforms, the her variant) and a mixed-precision solve are compared bit for bit between the two builds. Both
contexts get the same FP32 tile shape: the tuner picks it per context by timing, and the y-lines per K3 block set
the partition of the fused reductions (the sums of |y|^2 would differ in their last bits otherwise)."""
SHAPE = (8, 16, 8, 128)
import numpy as np
import pytest

from helpers import case, setup_for
from test_gpu_parity import random_vec

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def scalar_lib(tmp_path_factory):
    import adda_gb300 as A
    path = A.build(force=True, out=str(tmp_path_factory.mktemp("scalar_sums")), defines=["ADDA_NO_F32X2"])
    return A.load_library(path)


SETUPS = {
    "sphere128_grid256": lambda: __import__("adda_gb300").Setup(grid=128, m=1.33 + 0.01j, dpl=15),
    "c1_grid32": lambda: setup_for(case("c1_qmr")["setup"]),
    "ell24": lambda: setup_for(case("ell24")["setup"]),
    "grid10_radix5": lambda: setup_for(case("grid10")["setup"]),
    "grid18_radix3": lambda: setup_for(case("grid18")["setup"]),
    "box12": lambda: setup_for(case("box12")["setup"]),
}


@pytest.mark.parametrize("name", list(SETUPS))
def test_fp32_matvec_bit_identical(name, scalar_lib):
    import adda_gb300 as A
    s = SETUPS[name]()
    packed = A.Context.from_setup(s, nrhs_max=2)
    scalar = A.Context.from_setup(s, nrhs_max=2, library=scalar_lib)
    packed.set_fft_shape(SHAPE)
    scalar.set_fft_shape(SHAPE)
    x = random_vec(s.n, 2, 5)
    for her in (False, True):
        y1, ip1 = packed.matvec(x, "fp32", her)
        y2, ip2 = scalar.matvec(x, "fp32", her)
        assert np.array_equal(y1.view(np.uint64), y2.view(np.uint64)), (name, her)
        assert np.array_equal(ip1, ip2)
    packed.close()
    scalar.close()


def test_mixed_solve_bit_identical(scalar_lib):
    import adda_gb300 as A
    s = setup_for(case("ell24")["setup"])
    res = []
    for L in (None, scalar_lib):
        ctx = A.Context.from_setup(s, nrhs_max=2, library=L)
        ctx.set_fft_shape(SHAPE)
        res.append(ctx.solve(np.stack(s.einc), prec="mixed", eps=1e-8))
        ctx.close()
    assert [st["niter"] for st in res[0]["stats"]] == [st["niter"] for st in res[1]["stats"]]
    assert np.array_equal(res[0]["x"].view(np.uint64), res[1]["x"].view(np.uint64))
