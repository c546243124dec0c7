// ctx.cuh - the device context behind adda_gb300_ctx and the internal interfaces between the library's .cu files.
#pragma once

#include "adda_gb300.h"
#include "common.cuh"

#include <atomic>
#include <string>
#include <vector>

namespace adda {

void set_error(const std::string &msg);
extern std::atomic<unsigned long long> g_launches;
inline void count_launch(unsigned long long k = 1) { g_launches.fetch_add(k, std::memory_order_relaxed); }

#define ADDA_CUDA(call)                                                                                          \
	do {                                                                                                         \
		cudaError_t e_ = (call);                                                                                 \
		if (e_ != cudaSuccess) {                                                                                 \
			::adda::set_error(std::string(#call) + ": " + cudaGetErrorString(e_));                               \
			return ADDA_GB300_ECUDA;                                                                             \
		}                                                                                                        \
	} while (0)

#define ADDA_LAUNCHED()                                                                                          \
	do {                                                                                                         \
		::adda::count_launch();                                                                                  \
		cudaError_t e_ = cudaGetLastError();                                                                     \
		if (e_ != cudaSuccess) {                                                                                 \
			::adda::set_error(std::string("kernel launch: ") + cudaGetErrorString(e_));                          \
			return ADDA_GB300_ECUDA;                                                                             \
		}                                                                                                        \
	} while (0)

// Krylov epilogue of the last matvec kernel: per-block partial sums written to partial[(rhs*nblk + blk)*4 + 0..2]
enum MvEpiMode {
	EPI_NONE = 0,
	EPI_NORM = 1,        // s0 = sum |y|^2
	EPI_DOT_ARG = 2,     // s1 = sum x*y        (bilinear, x = argument)       -- QMR_CS alpha (iterative.c:967)
	EPI_DOT_U_CONJ = 4,  // s1 = sum y*conj(u)                                 -- BiCGStab v.r~ (iterative.c:694)
	EPI_DOT_ARG_CONJ = 8 // s1 = sum x*conj(y)  (x = argument)                 -- BiCGStab s.t (iterative.c:712)
};

struct MvEpi {
	int mode;
	const void *u;     // vector for EPI_DOT_U_CONJ (same precision as the matvec)
	double *partial;   // per-block partial sums
};

struct SolverWork; // solver.cu

// tile shape of the matvec kernels (per arithmetic): y-lines per K1/K3 block, y-lines per K2a/K2c block, (kz, RHS)
// pairs per generic K2b block, threads per register-K2b block
struct MvShape {
	int w1, w2, pairs, nt;
};

} // namespace adda

struct adda_gb300_ctx {
	int device = 0;
	cudaStream_t stream = nullptr;
	int bX = 0, bY = 0, bZ = 0, gX = 0, gY = 0, gZ = 0, DsY = 0, DsZ = 0;
	size_t N = 0;
	int Rmax = 1;
	int interaction = 0; // enum adda_gb300_inter
	double nloc_rp = 0;  // Gaussian width of the non-local interaction
	std::vector<double> int_tables; // IGT_SO / SO: the integral tables t1..t10 back to back
	double2 so_m = {0, 0};          // SO: refractive index of the second-order terms
	// particle near a substrate: reflected interaction R~, layout [gX][gZ][gY/2+1][6]
	int surface = 0, refl = 0, msub_inf = 0;
	double zsum_shift = 0;
	double2 msub = {0, 0};
	std::vector<double2> refl_host;   // SOM table or HOST tensor (see enum adda_gb300_refl)
	double2 *R64 = nullptr;
	float2 *R32 = nullptr;
	double gridspace = 0, k = 0;
	// lattice (host and device). A group context (adda_gb300_create_group) holds P particles in one box: particle q's
	// arrays are slot q of each lattice array (stride lat_stride = N, the largest particle; line starts stride
	// bZ*bY+1), and RHS r belongs to particle r / rpp. A single lattice: P = 1, rpp = Rmax.
	int P = 1, rpp = 1;
	size_t lat_stride = 0;
	std::vector<uint16_t> pos;
	std::vector<uint8_t> mat;
	uint32_t *d_line_start = nullptr; // [bZ*bY+1]: index of the first dipole of x-line (y,z), lines z-major
	uint32_t *d_xy = nullptr;         // [N]: x | y<<16
	uint8_t *d_mat = nullptr;
	uint16_t *d_pos = nullptr;        // [N][3] (cross sections)
	// FFT plans: [0] for double, [1] for float (the float plans may use radix 16)
	adda::FftPlan px[2], py[2], pz[2];
	double2 *tw64[3] = {nullptr, nullptr, nullptr};
	float2 *tw32[3] = {nullptr, nullptr, nullptr};
	// interaction matrix, reduced layout [gX][DsZ][DsY][6]
	double2 *D64 = nullptr;
	float2 *D32 = nullptr;
	bool dready = false;
	// polarisabilities per RHS: material mode [Rmax][nmat][3], dipole mode [Rmax][N][3]
	int per_dip = 0, nmat = 0;
	std::vector<int> cc_set;          // per RHS: 1 once set
	double2 *cc64 = nullptr, *ccs64 = nullptr;
	float2 *ccs32 = nullptr;
	// matvec work
	void *Xf = nullptr;               // [R][gX][3][bZ][bY] after the X transform
	void *Tz = nullptr;               // [R][CK][3][gZ][bY] chunk of x-slabs after the Z transform
	void *TzR = nullptr;              // surface: the same chunk transformed along z with the inverse sign
	// the odd chunks' buffers and stream: two chunks of the y/z stage run at once (one's K2a/K2b/K2c filling the
	// other's tail), joined before K3 by events (also inside a stream capture)
	void *Tz2 = nullptr, *TzR2 = nullptr;
	cudaStream_t stream2 = nullptr;
	cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
	// the caller's stream the device-buffer entry points order themselves with (legacy default stream unless set)
	cudaStream_t order = cudaStreamLegacy;
	cudaEvent_t ev_in = nullptr, ev_out = nullptr;
	int CK64 = 1, CK32 = 1;           // x-slabs per chunk (sized to stay resident in L2)
	int CK32max = 1;                  // largest FP32 chunk the Tz buffer holds
	bool chunk_fixed = false;         // chunk size set by the environment: no tuning
	bool chunk_tuned = false;         // FP32 chunk size measured (tune_chunks)
	adda::MvShape shape[2] = {{4, 8, 4, 128}, {8, 16, 8, 128}}; // [0] FP64, [1] FP32 tile shapes
	bool shape_fixed = false;         // FP32 shape set by the caller or the environment: not tuned
	double *partial = nullptr;        // epilogue partial sums
	size_t partial_len = 0;
	double *d_red = nullptr;          // reduced per-RHS results [Rmax][4]
	// staging for the host-pointer matvec
	void *vin = nullptr, *vout = nullptr;
	// solver
	adda::SolverWork *sw = nullptr;
	// last solve leaves polarisations here (FP64) for the cross sections
	double2 *pvec64 = nullptr;
	int last_nrhs = 0;
	double last_solve_ms = 0;
};

namespace adda {

// plan.cpp-equivalent helpers (api.cu)
FftPlan make_plan(int n, int max_radix);

// dmatrix.cu
int dmatrix_build(adda_gb300_ctx *c);

// matvec.cu
int matvec_setup(adda_gb300_ctx *c); // tile shapes, kernel attributes
int matvec_set_shape(adda_gb300_ctx *c, bool f32, const MvShape &s); // a tile shape the build holds and that fits
bool matvec_shape_ok(const adda_gb300_ctx *c, bool f32, const MvShape &s);
bool matvec_k2b_reg(const adda_gb300_ctx *c); // the FP32 matvec uses the register K2b (its thread count is tunable)
size_t matvec_partial_blocks(const adda_gb300_ctx *c, bool dbl); // partial-sum blocks per RHS of the epilogue
// T = FFT/D arithmetic (float or double), V = dipole-vector type (float2 or double2)
template <typename T, typename V>
int matvec_run(adda_gb300_ctx *c, int R, const V *arg, V *res, int her, const MvEpi &epi, const int *done);
int reduce_partials(adda_gb300_ctx *c, int R, const double *partial, size_t nblk, double *out);

// solver.cu
int solver_solve(adda_gb300_ctx *c, const adda_gb300_solve_params *sp, int nrhs, const double *einc, double *xvec,
	double *pvec, adda_gb300_rhs_stats *stats, double *resid_hist, int hist_cap);
int solver_solve_dev(adda_gb300_ctx *c, const adda_gb300_solve_params *sp, int nrhs, const double2 *d_einc,
	double2 *d_xvec, double2 *d_pvec, adda_gb300_rhs_stats *stats);
void solver_free(adda_gb300_ctx *c);
int cross_sections(adda_gb300_ctx *c, int nrhs, const double *prop, const double *incpol, double *cext, double *cabs);
int cross_sections_beam(adda_gb300_ctx *c, int nrhs, const double *einc, double inc_scale, double *cext,
	double *cabs);
size_t solver_chpoint_size(const adda_gb300_ctx *c, int method);
int solver_chpoint_save(adda_gb300_ctx *c, int rhs, void *buf, size_t size);
int solver_chpoint_load(adda_gb300_ctx *c, int rhs, const void *buf, size_t size);
int scattered_fields(adda_gb300_ctx *c, int nrhs, int ndir, const double *dirs, double *ebuff);
int vjp_chi(adda_gb300_ctx *c, const adda_gb300_solve_params *sp, int rhs, const double prop[3], const double incpol[3],
	const double *dinv_alpha, double *grad_cext, double *grad_cabs);

} // namespace adda
