// noalloc.cu - an allocation-free variant of the cross-section reduction (adda_gb300_cross_sections_noalloc).
//
// Who needs it: callers that cannot call cudaMalloc at the point where they want the cross sections -- code running
// inside a framework that owns all device memory through its own pool allocator (a cudaMalloc behind its back
// fragments or over-commits the pool it manages), or a plugin whose host forbids device allocation after start-up.
// The context-based adda_gb300_cross_sections gets its per-block partial sums from the context's solver work
// buffers (allocated on first use); this variant keeps them in one file-scope __device__ array instead, so a call
// only launches two kernels and allocates nothing. It applies the free-space plane-wave formulas (ExtCross with the
// forward amplitude, AbsCross); it is not valid for a particle near a substrate.
//
// The array (g_noalloc_scratch, 1 MiB) is part of the library image: every GPU that loads the library holds it until
// the process exits. Its device address is looked up with cudaGetSymbolAddress by the first call on each device
// (with that device current); make that first call before any stream capture. A failed lookup is not remembered:
// the next call tries again. All calls share the array and it keeps the last call's contents, so calls that
// overlap on the GPU (different streams, or different host threads on the same device) race and must be
// serialised by the caller; each call rewrites every slot it reads before reading it.
#include "ctx.cuh"

#include <cmath>
#include <mutex>

namespace {

constexpr int NOALLOC_BLOCKS = 256;                                  // partial sums per RHS
constexpr int NOALLOC_MAX_RHS = ADDA_GB300_NOALLOC_MAX_RHS;          // 64
constexpr int NOALLOC_SLOTS = 8;                                     // 6 (complex 3-vector) + 1 (absorption) + pad
constexpr size_t NOALLOC_DOUBLES = (size_t)NOALLOC_MAX_RHS * NOALLOC_BLOCKS * NOALLOC_SLOTS; // 131072 = 1 MiB

__device__ __align__(256) double g_noalloc_scratch[NOALLOC_DOUBLES];

constexpr int MAX_DEVICES = 64;
double *g_ptr[MAX_DEVICES];
std::mutex g_mutex;

// per-dipole sums of one RHS: sum_j P_j exp(-i kd n.pos_j) (CalcFieldFree, crosssec.c:506-586) and
// sum_j sum_c (-Im(1/cc) - 2k^3/3)|P_jc|^2 (AbsCross, crosssec.c:866-882)
__global__ void __launch_bounds__(256) cross_partials(double *scratch, const double2 *P, const uint16_t *pos,
	const double2 *cc, int per_dip, int nmat, const uint8_t *mat, size_t N, const double *prop, double kd, double k3)
{
	const int r = blockIdx.y;
	const double n0 = prop[3 * r], n1 = prop[3 * r + 1], n2 = prop[3 * r + 2];
	double s[7] = {0, 0, 0, 0, 0, 0, 0};
	for (size_t d = blockIdx.x * (size_t)blockDim.x + threadIdx.x; d < N; d += (size_t)gridDim.x * blockDim.x) {
		const double ph = -kd * (n0 * pos[3 * d] + n1 * pos[3 * d + 1] + n2 * pos[3 * d + 2]);
		double sn, cs;
		sincos(ph, &sn, &cs);
		for (int c = 0; c < 3; c++) {
			const double2 p = P[((size_t)r * N + d) * 3 + c];
			s[2 * c] += p.x * cs - p.y * sn;
			s[2 * c + 1] += p.x * sn + p.y * cs;
			const int m = mat ? mat[d] : 0;
			if (!per_dip && m >= nmat) { // a material index without a polarisability: Cabs of this RHS becomes NaN
				s[6] = nan("");
				continue;
			}
			const double2 a = per_dip ? cc[((size_t)r * N + d) * 3 + c] : cc[((size_t)r * nmat + m) * 3 + c];
			const double mult = a.y / (a.x * a.x + a.y * a.y) - 2 * k3 / 3; // -Im(1/cc) - 2k^3/3
			s[6] += mult * (p.x * p.x + p.y * p.y);
		}
	}
	__shared__ double sh[7][8];
	const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
	for (int j = 0; j < 7; j++) {
		double v = s[j];
		for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
		if (lane == 0) sh[j][wid] = v;
	}
	__syncthreads();
	if (threadIdx.x == 0) {
		double *o = scratch + ((size_t)r * NOALLOC_BLOCKS + blockIdx.x) * NOALLOC_SLOTS;
		for (int j = 0; j < 7; j++) {
			double v = 0;
			for (int w = 0; w < 8; w++) v += sh[j][w];
			o[j] = v;
		}
	}
}

// one thread per RHS: fixed-order sum of the partials, then ExtCross (crosssec.c:811-822) and AbsCross (:915)
__global__ void cross_finish(const double *scratch, int R, const double *prop, const double *incpol, double k,
	double gridspace, int bX, int bY, int bZ, double *cext, double *cabs)
{
	const int r = blockIdx.x * blockDim.x + threadIdx.x;
	if (r >= R) return;
	double sm[7] = {0, 0, 0, 0, 0, 0, 0};
	for (int b = 0; b < NOALLOC_BLOCKS; b++)
		for (int j = 0; j < 7; j++) sm[j] += scratch[((size_t)r * NOALLOC_BLOCKS + b) * NOALLOC_SLOTS + j];
	const double *n = prop + 3 * r, *e = incpol + 3 * r;
	double dre = 0, dim = 0;
	for (int i = 0; i < 3; i++) {
		dre += sm[2 * i] * n[i];
		dim += sm[2 * i + 1] * n[i];
	}
	const double r0[3] = {-gridspace * (bX - 1) / 2.0, -gridspace * (bY - 1) / 2.0, -gridspace * (bZ - 1) / 2.0};
	const double ph0 = -k * (r0[0] * n[0] + r0[1] * n[1] + r0[2] * n[2]);
	const double k3 = k * k * k;
	double sn, cs;
	sincos(ph0, &sn, &cs);
	const double ar = k3 * sn, ai = -k3 * cs; // -i k^3 exp(i ph0)
	double sumc = 0;
	for (int i = 0; i < 3; i++) {
		const double tr = sm[2 * i] - dre * n[i], ti = sm[2 * i + 1] - dim * n[i];
		sumc += (ar * tr - ai * ti) * e[i];
	}
	const double PI = 3.14159265358979323846;
	cext[r] = sumc * 4 * PI / (k * k);
	cabs[r] = 4 * PI * k * sm[6];
}

int fail(const char *msg, cudaError_t e = cudaSuccess)
{
	adda::set_error(e != cudaSuccess ? std::string(msg) + ": " + cudaGetErrorString(e) : std::string(msg));
	return e != cudaSuccess ? ADDA_GB300_ECUDA : ADDA_GB300_EINVAL;
}

} // namespace

extern "C" int adda_gb300_cross_sections_noalloc(int nrhs, size_t ndip, const void *d_pvec, const uint16_t *d_position,
	const uint8_t *d_material, const void *d_cc, int nmat, int per_dipole, int boxX, int boxY, int boxZ,
	double gridspace, double wavenum, const double *d_prop, const double *d_incpol, double *d_cext, double *d_cabs,
	void *stream)
{
	if (nrhs < 1 || nrhs > NOALLOC_MAX_RHS)
		return fail("cross_sections_noalloc: nrhs must be 1..ADDA_GB300_NOALLOC_MAX_RHS (64): the static scratch "
			"holds 256 partial sums for at most 64 right-hand sides");
	if (!d_pvec || !d_position || !d_cc || !d_prop || !d_incpol || !d_cext || !d_cabs || (!per_dipole && !d_material
		&& nmat != 1) || (!per_dipole && nmat < 1) || !(gridspace > 0) || !(wavenum > 0) || boxX < 1 || boxY < 1 ||
		boxZ < 1)
		return fail("cross_sections_noalloc: invalid arguments");
	int dev = 0;
	cudaError_t e = cudaGetDevice(&dev);
	if (e != cudaSuccess) return fail("cross_sections_noalloc: cudaGetDevice", e);
	if (dev < 0 || dev >= MAX_DEVICES) return fail("cross_sections_noalloc: device ordinal out of range");
	double *scratch = nullptr;
	{
		// the device address of the static array, looked up on the first call on this device (retried after a
		// failure); host code must not pass g_noalloc_scratch itself, which names a host-side stand-in
		std::lock_guard<std::mutex> lock(g_mutex);
		if (!g_ptr[dev]) {
			void *p = nullptr;
			e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
			if (e != cudaSuccess) return fail("cross_sections_noalloc: cudaGetSymbolAddress", e);
			g_ptr[dev] = static_cast<double *>(p);
		}
		scratch = g_ptr[dev];
	}
	cudaStream_t st = static_cast<cudaStream_t>(stream);
	const dim3 grid(NOALLOC_BLOCKS, nrhs);
	cross_partials<<<grid, 256, 0, st>>>(scratch, static_cast<const double2 *>(d_pvec), d_position,
		static_cast<const double2 *>(d_cc), per_dipole, nmat, per_dipole ? nullptr : d_material, ndip, d_prop,
		wavenum * gridspace, wavenum * wavenum * wavenum);
	cross_finish<<<(nrhs + 63) / 64, 64, 0, st>>>(scratch, nrhs, d_prop, d_incpol, wavenum, gridspace, boxX, boxY,
		boxZ, d_cext, d_cabs);
	adda::count_launch(2);
	e = cudaGetLastError();
	if (e != cudaSuccess) return fail("cross_sections_noalloc: kernel launch", e);
	return ADDA_GB300_OK;
}
