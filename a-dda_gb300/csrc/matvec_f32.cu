// matvec_f32.cu - FP32-arithmetic instantiations of the matvec kernels (float2, double2 and double-float dipole
// vectors).
#include "matvec_kernels.cuh"

namespace adda {

int matvec_setup_f32(adda_gb300_ctx *c)
{
	(void)c;
	int rc = mv::set_attrs_tv<float, float2>();
	if (rc) return rc;
	rc = mv::set_attrs_tv<float, double2>();
	if (rc) return rc;
	return mv::set_attrs_tv<float, dd2>();
}

template <typename T, typename V>
int matvec_run(adda_gb300_ctx *c, int R, const V *arg, V *res, int her, const MvEpi &epi, const int *done)
{
	return mv::launch_matvec<T, V>(c, R, arg, res, her, epi, done);
}

template int matvec_run<float, float2>(adda_gb300_ctx *, int, const float2 *, float2 *, int, const MvEpi &,
	const int *);
template int matvec_run<float, double2>(adda_gb300_ctx *, int, const double2 *, double2 *, int, const MvEpi &,
	const int *);
template int matvec_run<float, dd2>(adda_gb300_ctx *, int, const dd2 *, dd2 *, int, const MvEpi &, const int *);

} // namespace adda
