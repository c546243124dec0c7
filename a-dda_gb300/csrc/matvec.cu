// matvec.cu - host side of the matvec (setup, partial-sum reduction) and its FP64 instantiation; the kernels are in
// matvec_kernels.cuh, the FP32 instantiations in matvec_f32.cu (compiled in parallel).
#include "matvec_kernels.cuh"

namespace adda {

int matvec_setup_f32(adda_gb300_ctx *c); // matvec_f32.cu

namespace {

// sum per-RHS partials (fixed order): out[r*4 + 0..2]
__global__ void reduce_partials_k(const double *partial, size_t nblk, double *out)
{
	__shared__ double red[32];
	const int r = blockIdx.x;
	double s[3] = {0, 0, 0};
	for (size_t b = threadIdx.x; b < nblk; b += blockDim.x)
		for (int j = 0; j < 3; j++) s[j] += partial[((size_t)r * nblk + b) * 4 + j];
	for (int j = 0; j < 3; j++) {
		double v = mv::block_sum(s[j], red);
		if (threadIdx.x == 0) out[r * 4 + j] = v;
	}
}

} // namespace

size_t matvec_partial_blocks(const adda_gb300_ctx *c, bool dbl)
{
	// K3 grid: ceil(bY/w1) x bZ blocks per RHS
	const int w = c->shape[dbl ? 0 : 1].w1;
	return (size_t)((c->bY + w - 1) / w) * c->bZ;
}

// the default tile shape of one arithmetic, narrowed per kernel where an axis longer than 512 would overflow the
// shared memory of a block
template <typename T> static bool choose_shape(adda_gb300_ctx *c, MvShape &s)
{
	if (mv::tile_smem<T>(c->gX, 3 * s.w1) > mv::SMEM_CAP && mv::static_len(c->gX) == 0) s.w1 = 1;
	if (mv::tile_smem<T>(c->gZ, s.w2) > mv::SMEM_CAP && mv::static_len(c->gZ) == 0) s.w2 = 2;
	if (!mv::use_k2b_reg<T>(c->gY) && !c->surface &&
		2 * sizeof(typename CxT<T>::type) * (size_t)c->gY * tile_ls(3 * s.pairs) > mv::SMEM_CAP &&
		mv::static_len(c->gY) == 0)
		s.pairs = 1;
	return mv::shape_fits<T>(c, s);
}

int matvec_setup(adda_gb300_ctx *c)
{
	if (!choose_shape<double>(c, c->shape[0]) || !choose_shape<float>(c, c->shape[1])) {
		set_error(c->surface ? "FFT grid too large for the shared-memory tiles (surface mode: at most 1024 per axis)"
			: "FFT grid too large for the shared-memory tiles (at most 2048 per axis)");
		return ADDA_GB300_EINVAL;
	}
	int rc = mv::set_attrs_tv<double, double2>();
	if (rc || (rc = mv::setup_yz<double>()) || (rc = mv::setup_yz<float>())) return rc;
	return matvec_setup_f32(c);
}

bool matvec_shape_ok(const adda_gb300_ctx *c, bool f32, const MvShape &s)
{
	return mv::shape_instantiated(f32, c->gX, c->gZ, c->gY, s) &&
		(f32 ? mv::shape_fits<float>(c, s) : mv::shape_fits<double>(c, s));
}

bool matvec_k2b_reg(const adda_gb300_ctx *c)
{
	return mv::use_k2b_reg<float>(c->gY);
}

int matvec_set_shape(adda_gb300_ctx *c, bool f32, const MvShape &s)
{
	if (!matvec_shape_ok(c, f32, s)) {
		set_error("set_fft_shape: this tile shape is not built for these axis lengths or does not fit shared memory");
		return ADDA_GB300_EINVAL;
	}
	c->shape[f32 ? 1 : 0] = s;
	return ADDA_GB300_OK;
}

template <typename T, typename V>
int matvec_run(adda_gb300_ctx *c, int R, const V *arg, V *res, int her, const MvEpi &epi, const int *done)
{
	return mv::launch_matvec<T, V>(c, R, arg, res, her, epi, done);
}

template int matvec_run<double, double2>(adda_gb300_ctx *, int, const double2 *, double2 *, int, const MvEpi &,
	const int *);

int reduce_partials(adda_gb300_ctx *c, int R, const double *partial, size_t nblk, double *out)
{
	reduce_partials_k<<<R, 256, 0, c->stream>>>(partial, nblk, out);
	ADDA_LAUNCHED();
	return ADDA_GB300_OK;
}

} // namespace adda
