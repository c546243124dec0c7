// matvec_yz.cu - the y/z stage of the matvec (K2a z-FFT, K2b y-FFT + D product, K2c inverse z-FFT) for FP64 and
// FP32 arithmetic: these kernels never touch the dipole vectors, so they are compiled once here (in parallel with
// the K1/K3 translation units) for every tile shape the build holds.
#define ADDA_MATVEC_YZ_TU
#include "matvec_kernels.cuh"

namespace adda {
namespace mv {

template int launch_yz<float>(adda_gb300_ctx *, MvGeom<float>, int, const MvShape &, cudaStream_t);
template int launch_yz<double>(adda_gb300_ctx *, MvGeom<double>, int, const MvShape &, cudaStream_t);
template int setup_yz<float>();
template int setup_yz<double>();

} // namespace mv
} // namespace adda
