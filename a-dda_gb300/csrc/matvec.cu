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
	// K3 grid: ceil(bY/W1) x bZ blocks per RHS
	const int w = dbl ? mv::Tiles<double>::W1 : mv::Tiles<float>::W1;
	return (size_t)((c->bY + w - 1) / w) * c->bZ;
}

int matvec_setup(adda_gb300_ctx *c)
{
	const size_t cap = 216 * 1024;
	if (mv::smem_k1<double>(c->gX) > cap || mv::smem_k2<double>(c->gZ) > cap || mv::smem_k2b<double>(c->gY) > cap ||
		mv::smem_k1<float>(c->gX) > cap || mv::smem_k2<float>(c->gZ) > cap || mv::smem_k2b<float>(c->gY) > cap) {
		set_error("FFT grid too large for the shared-memory tiles (maximum 512 per axis)");
		return ADDA_GB300_EINVAL;
	}
	int rc = mv::set_attrs_tv<double, double2>();
	if (rc) return rc;
	return matvec_setup_f32(c);
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
