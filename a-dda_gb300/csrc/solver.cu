// solver.cu - device-resident Krylov solvers (IterativeSolver, src/iterative.c:1398-1530) and cross sections.
//
// Every vector, scalar and reduction stays on the GPU. One iteration is a fixed kernel sequence:
//   QMR_CS (iterative.c:956-1029):   matvec(v) + [alpha = v.Av fused in its epilogue] -> qmr_s1 -> qmr_v1
//                                    [v~ update + |v~|^2, v~.v~] -> qmr_s2 -> qmr_v2 [p, x, v, r updates + |r|^2]
//                                    -> progress
//   BiCGStab (iterative.c:673-720):  bs_s0 -> bs_v1 [p] -> matvec(p) [v.r~*] -> bs_s1 -> bs_v2 [s, |s|^2] -> bs_s2
//                                    -> matvec(s) [|t|^2, s.t*] -> bs_s3 -> bs_v3 [x, r, |r|^2, r.r~*] -> progress
// Scalar kernels run one block per right-hand side: they sum the deterministic per-block partials of the previous
// kernel in a fixed order and update that RHS's FP64 recurrence scalars (including the breakdown tests and the
// stagnation counter of ProgressReport, iterative.c:282-318). Several RHS iterate in lockstep; a converged RHS is
// frozen by its done flag. check_every iterations are captured once as a CUDA graph and replayed; the host reads
// the done flags only between graph launches.
//
// MIXED precision: the Krylov iterations run with the FP32 matvec on double-float vectors (dd2: pairs of floats,
// about 48 significant bits, all arithmetic on the FP32 pipes; MIXED_F64VEC: double2 vectors, MIXED_F32VEC: float2);
// scalars stay FP64 and reductions end in FP64. An outer loop recomputes the true residual b - A.x with the FP64
// matvec (the reference's ResidualNorm2, iterative.c:322-338), accumulates x in FP64 and restarts the inner solve
// on the residual until the FP64 relative residual meets eps.
//
// One deliberate difference from the reference: when IF_AUTO picks x_0 = 0, the reference reuses A.b from the
// initial-field test for the first iteration (matvec_ready, iterative.c:962-965, 691); here the first iteration
// always computes its matvec. The iterates agree to rounding.
#include "ctx.cuh"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <type_traits>
#include <vector>

namespace adda {

struct RhsState {
	double inprodR, inprodRp1, epsB, resid_scale;
	int niter, counter, done, status, half, mc, maxiter, x0zero;
	int it0;  // niter when the current Krylov run started (role parity of the swapped QMR_CS / CSYM buffers)
	double prev_err; // last reported relative residual (ProgressReport's prev_err, kept in checkpoints)
	int full; // BiCGStab: no half-step exit
	// QMR_CS
	double c_old, c_new, om_old, om_new;
	double2 beta, tautilda, s_old, s_new, alpha, theta, eta, zetat;
	// BiCGStab, BiCG_CS (ro, balpha), CGNR (real parts of ro, balpha)
	double2 ro_old, ro_new, omega, balpha;
	// CSYM: beta_(k+1) = |w| (real); tau, c, s, theta, eta share the QMR_CS fields, gamma is kept in zetat
	double cs_beta;
	// QMR_CS_2: ro_k, theta_(k-1), c_(k-1); eps_(k-1), eta_(k-1), beta_k; delta_k = v_k.v_k
	double q2_ro, q2_theta, q2_c;
	double2 q2_eps, q2_eta, q2_beta, q2_delta;
	// BCGS2: rho_0, rho_1, alpha; the convex-combination coefficients y0[1], y0[2]
	double2 b2_rho0, b2_rho1, b2_alpha, b2_y1, b2_y2;
	// coefficients for the vector kernels
	double2 k0, k1, k2, k3, kib, kr;
	double d0;
	double temp; // |b|^2
};

struct SolverWork {
	int R = 0;
	size_t n3 = 0;
	// FP64 vectors [R][3N]
	double2 *x64 = nullptr, *r64 = nullptr, *b64 = nullptr, *av64 = nullptr;
	// Krylov work vectors, stored as double2 (the float solver uses the first half of each)
	double2 *kv[8] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
	RhsState *st = nullptr;
	int *done = nullptr;   // mirror of st[r].done for the matvec early exit
	double *hist = nullptr;
	int hist_cap = 0;
	double *vpart = nullptr; // vector-kernel partials [R][nbv][4]
	int nbv = 0;
	double *xpart = nullptr; // cross-section partials
	int *h_done = nullptr;   // pinned
	// iteration checkpoints: the state of the last FP64 solve (valid until the next solve) and loaded states
	int chp_valid = 0, chp_method = -1, chp_R = 0;
	std::vector<std::vector<unsigned char>> chp_pend;
	// cached graph
	cudaGraphExec_t gexec = nullptr;
	int g_method = -1, g_dbl = -1, g_R = -1, g_K = -1;
	unsigned long long g_nodes = 0;
};

namespace {

constexpr int NT = 256;

__device__ __forceinline__ double2 dc(double a, double b) { return make_double2(a, b); }
__device__ __forceinline__ double2 dmul(double2 a, double2 b) { return dc(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
__device__ __forceinline__ double2 dadd(double2 a, double2 b) { return dc(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 dsub(double2 a, double2 b) { return dc(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 dscal(double2 a, double s) { return dc(a.x * s, a.y * s); }
__device__ __forceinline__ double2 dconj(double2 a) { return dc(a.x, -a.y); }
__device__ __forceinline__ double dabs(double2 a) { return hypot(a.x, a.y); }
__device__ __forceinline__ double2 ddiv(double2 a, double2 b)
{
	// a/b with scaling against overflow (Smith's method)
	if (fabs(b.x) >= fabs(b.y)) {
		const double r = b.y / b.x, d = b.x + b.y * r;
		return dc((a.x + a.y * r) / d, (a.y - a.x * r) / d);
	}
	const double r = b.x / b.y, d = b.x * r + b.y;
	return dc((a.x * r + a.y) / d, (a.y * r - a.x) / d);
}
__device__ __forceinline__ double2 dinv(double2 b) { return ddiv(dc(1, 0), b); }
__device__ __forceinline__ double2 dsqrt(double2 z)
{
	const double a = z.x, b = z.y;
	const double t = sqrt(0.5 * (hypot(a, b) + fabs(a)));
	if (t == 0) return dc(0, 0);
	if (a >= 0) return dc(t, b / (2 * t));
	return dc(fabs(b) / (2 * t), copysign(t, b));
}

// a loop-invariant complex coefficient in the arithmetic of the vector type C (prepared for the packed double-float
// products when C is dd2)
template <typename C> struct CoefOf {
	typedef C T;
	static __device__ __forceinline__ C make(double2 k) { return from_d2<C>(k); }
};
template <> struct CoefOf<dd2> {
	typedef dd2k T;
	static __device__ __forceinline__ dd2k make(double2 k) { return make_dd2k(from_d2<dd2>(k)); }
};
template <typename C> __device__ __forceinline__ typename CoefOf<C>::T cof(double2 k) { return CoefOf<C>::make(k); }

// block sum of up to 4 values; result valid in thread 0
__device__ __forceinline__ void block_sum4(double v[4], int nv)
{
	__shared__ double sh[4][NT / 32];
	const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
	for (int j = 0; j < nv; j++) {
		double s = v[j];
		for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
		if (lane == 0) sh[j][wid] = s;
	}
	__syncthreads();
	if (threadIdx.x == 0)
		for (int j = 0; j < nv; j++) {
			double s = 0;
			for (int w = 0; w < NT / 32; w++) s += sh[j][w];
			v[j] = s;
		}
	__syncthreads();
}

__device__ __forceinline__ void write_part(double *part, int nbv, double v[4], int nv)
{
	block_sum4(v, nv);
	if (threadIdx.x == 0) {
		double *o = part + ((size_t)blockIdx.y * nbv + blockIdx.x) * 4;
		for (int j = 0; j < nv; j++) o[j] = v[j];
	}
}

// the same from double-float accumulators
__device__ __forceinline__ void write_part(double *part, int nbv, DF a[4], int nv)
{
	double v[4];
	for (int j = 0; j < 4; j++) v[j] = acc_val(a[j]);
	write_part(part, nbv, v, nv);
}

// sum partials of RHS r in a fixed order (all threads participate); result in thread 0
__device__ __forceinline__ void sum_part(const double *part, size_t nblk, int r, double out[4], int nv)
{
	double v[4] = {0, 0, 0, 0};
	for (size_t b = threadIdx.x; b < nblk; b += blockDim.x)
		for (int j = 0; j < nv; j++) v[j] += part[((size_t)r * nblk + b) * 4 + j];
	block_sum4(v, nv);
	for (int j = 0; j < nv; j++) out[j] = v[j];
}

#define VLOOP(n3) for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < (n3); i += (size_t)gridDim.x * blockDim.x)

// ---------------- initialisation ----------------

// b = S.E (nMult_mat, linalg.c:549); partial |b|^2. E, b FP64.
__global__ void __launch_bounds__(NT) k_mult_cc(const double2 *E, double2 *b, const double2 *ccs, int per_dip, int nmat,
	const uint8_t *mat, size_t N, double *part, int nbv, int rpp, size_t lst)
{
	const int r = blockIdx.y;
	mat += (size_t)(r / rpp) * lst; // RHS r's particle (group contexts)
	const size_t n3 = 3 * N;
	double v[4] = {0, 0, 0, 0};
	VLOOP(n3) {
		const size_t d = i / 3;
		const int comp = (int)(i % 3);
		const double2 s = per_dip ? ccs[((size_t)r * N + d) * 3 + comp] : ccs[((size_t)r * nmat + mat[d]) * 3 + comp];
		const double2 e = E[(size_t)r * n3 + i];
		const double2 y = dmul(s, e);
		b[(size_t)r * n3 + i] = y;
		v[0] += y.x * y.x + y.y * y.y;
	}
	write_part(part, nbv, v, 1);
}

__global__ void s_init(RhsState *st, int *done, const double *part, int nbv, double eps, int maxiter, int mc,
	double *hist, int hist_cap, int zero_init)
{
	const int r = blockIdx.x;
	double s[4];
	sum_part(part, nbv, r, s, 1);
	if (threadIdx.x) return;
	RhsState &S = st[r];
	memset(&S, 0, sizeof(S));
	S.temp = s[0];
	S.resid_scale = 1 / s[0];
	S.epsB = eps * eps * s[0];
	S.maxiter = maxiter;
	S.mc = mc;
	S.niter = 1;
	S.it0 = 1;
	S.counter = 0;
	S.status = 0;
	if (zero_init) {
		S.inprodR = s[0];
		S.prev_err = sqrt(S.resid_scale * S.inprodR);
		if (hist_cap > 0) hist[(size_t)r * hist_cap] = S.prev_err;
		S.done = !(S.inprodR > S.epsB && S.niter <= S.maxiter);
		done[r] = S.done;
	}
}

// x0 / r0 from b (CalcInitField, iterative.c:1349-1379): zero -> x=0,r=b ; inc -> x=b,r=b-Ab ; auto -> choose
template <typename C>
__global__ void __launch_bounds__(NT) k_init_field(RhsState *st, int *done, const C *b, const C *Ab, C *x, C *r,
	size_t n3, int mode, double *part, int nbv, int stage)
{
	const int rr = blockIdx.y;
	const C *bb = b + rr * n3;
	if (stage == 0) { // r = b - Ab, partial |r|^2
		typename AccOf<C>::T v[4] = {};
		VLOOP(n3) {
			const C d = csub(bb[i], Ab[rr * n3 + i]);
			r[rr * n3 + i] = d;
			acc_abs2(v[0], d);
		}
		write_part(part, nbv, v, 1);
	}
	else { // choose x0 per RHS: st.x0zero holds 1 for x0=0
		const bool zero = st[rr].x0zero != 0;
		VLOOP(n3) {
			if (zero) {
				x[rr * n3 + i] = C{};
				r[rr * n3 + i] = bb[i];
			}
			else x[rr * n3 + i] = bb[i];
		}
	}
}

__global__ void s_init_choose(RhsState *st, int *done, const double *part, int nbv, int mode, double *hist,
	int hist_cap)
{
	const int r = blockIdx.x;
	double s[4];
	sum_part(part, nbv, r, s, 1);
	if (threadIdx.x) return;
	RhsState &S = st[r];
	S.inprodR = s[0];
	S.x0zero = 0;
	if (mode == ADDA_IF_AUTO && S.temp < S.inprodR) {
		S.inprodR = S.temp;
		S.x0zero = 1; // x0 = 0
	}
	S.prev_err = sqrt(S.resid_scale * S.inprodR);
	if (hist_cap > 0) hist[(size_t)r * hist_cap] = S.prev_err;
	S.done = !(S.inprodR > S.epsB && S.niter <= S.maxiter);
	done[r] = S.done;
}

// reductions for the method initialisation: slot 0 = |a|^2; slots 1,2 = sum a.u (mode 0, bilinear) or
// sum a.conj(u) (mode 1) -- the same slots the iteration kernels use for these dot products
template <typename C>
__global__ void __launch_bounds__(NT) k_dot(const C *a, const C *u, size_t n3, int mode, double *part, int nbv)
{
	const int r = blockIdx.y;
	typename AccOf<C>::T v[4] = {};
	VLOOP(n3) {
		const C x = a[r * n3 + i], y = u[r * n3 + i];
		acc_abs2(v[0], x);
		if (mode == 0) acc_cmul(v[1], v[2], x, y);
		else acc_cmulc(v[1], v[2], x, y);
	}
	write_part(part, nbv, v, 3);
}

template <typename C> __global__ void __launch_bounds__(NT) k_copy(C *dst, const C *src, size_t n3, const int *done)
{
	const int r = blockIdx.y;
	if (done && done[r]) return;
	VLOOP(n3) dst[r * n3 + i] = src[r * n3 + i];
}

// QMR_CS PHASE_INIT (iterative.c:939-954): beta = sqrt(r.r), omega = |r|/|beta|, v = r/beta, tau~ = omega*beta
__global__ void qmr_s_init(RhsState *st, const double *part, int nbv)
{
	const int r = blockIdx.x;
	double s[4];
	sum_part(part, nbv, r, s, 3);
	if (threadIdx.x) return;
	RhsState &S = st[r];
	S.om_old = 0;
	S.beta = dsqrt(dc(s[1], s[2]));
	S.om_new = sqrt(S.inprodR) / dabs(S.beta);
	S.kib = dinv(S.beta);
	S.tautilda = dscal(S.beta, S.om_new);
	S.c_new = S.c_old = 1;
	S.s_new = S.s_old = dc(0, 0);
}

template <typename C> __global__ void __launch_bounds__(NT) qmr_v_init(const RhsState *st, C *v, const C *r, size_t n3)
{
	const int rr = blockIdx.y;
	if (st[rr].done) return;
	const auto k = cof<C>(st[rr].kib);
	VLOOP(n3) v[rr * n3 + i] = cmul(k, r[rr * n3 + i]);
}

// ---------------- QMR_CS iteration ----------------

__global__ void qmr_s1(RhsState *st, int *done, const double *part, size_t nblk)
{
	const int r = blockIdx.x;
	if (st[r].done) return;
	double s[4];
	sum_part(part, nblk, r, s, 3);
	if (threadIdx.x) return;
	RhsState &S = st[r];
	if (1 / (S.om_new * S.om_new) < 1e-10) { // iterative.c:958-960
		S.status = ADDA_GB300_EBREAKDOWN;
		S.done = 1;
		done[r] = 1;
		return;
	}
	const double2 alpha = dc(s[1], s[2]);
	S.alpha = alpha;
	S.theta = dscal(dmul(dconj(S.s_old), S.beta), S.om_old);
	S.eta = dadd(dscal(S.beta, S.c_old * S.c_new * S.om_old), dscal(dmul(alpha, dconj(S.s_new)), S.om_new));
	S.zetat = dsub(dscal(alpha, S.c_new * S.om_new), dscal(dmul(S.s_new, S.beta), S.c_old * S.om_old));
	S.k0 = (S.niter == 1) ? dc(0, 0) : dc(-S.beta.x, -S.beta.y);
	S.k1 = dc(-alpha.x, -alpha.y);
	S.om_old = S.om_new;
}

// v~ = k0*v~ + k1*v + A.v ; partials sum re^2, im^2, re*im (nDotProdSelf_conj_Norm2, linalg.c:127)
template <typename C>
__global__ void __launch_bounds__(NT) qmr_v1(const RhsState *st, C *vt, const C *v, const C *Av, size_t n3,
	double *part, int nbv)
{
	const int r = blockIdx.y;
	if (st[r].done) return;
	const auto k0 = cof<C>(st[r].k0), k1 = cof<C>(st[r].k1);
	typename AccOf<C>::T s[4] = {};
	VLOOP(n3) {
		const size_t j = r * n3 + i;
		const C y = cadd(cadd(cmul(k0, vt[j]), cmul(k1, v[j])), Av[j]);
		vt[j] = y;
		acc_sq3(s, y);
	}
	write_part(part, nbv, s, 3);
}

__global__ void qmr_s2(RhsState *st, const double *part, int nbv)
{
	const int r = blockIdx.x;
	if (st[r].done) return;
	double s[4];
	sum_part(part, nbv, r, s, 3);
	if (threadIdx.x) return;
	RhsState &S = st[r];
	const double nrm = s[0] + s[1];
	S.beta = dsqrt(dc(s[0] - s[1], 2 * s[2]));
	S.om_new = sqrt(nrm) / dabs(S.beta);
	const double zt2 = S.zetat.x * S.zetat.x + S.zetat.y * S.zetat.y;
	const double zabs = sqrt(zt2 + nrm);
	const double zt = sqrt(zt2);
	const double2 zeta = (zt < 1e-40) ? dc(zabs, 0) : dscal(S.zetat, zabs / zt);
	S.c_old = S.c_new;
	S.c_new = zt / zabs;
	S.s_old = S.s_new;
	S.s_new = ddiv(dscal(S.beta, S.om_new), zeta);
	const double2 t4 = dinv(zeta);
	if (S.niter == 1) {
		S.k0 = dc(0, 0);
		S.k1 = dc(0, 0);
	}
	else {
		const double2 t2 = dmul(dc(-S.eta.x, -S.eta.y), t4);
		S.k1 = t2;
		S.k0 = (S.niter == 2) ? dc(0, 0) : dmul(dc(-S.theta.x, -S.theta.y), t4);
	}
	S.k2 = t4;
	const double2 tau = dscal(S.tautilda, S.c_new);
	S.tautilda = dmul(dc(-S.s_new.x, -S.s_new.y), S.tautilda);
	S.k3 = tau;
	S.kib = dinv(S.beta);
	S.d0 = S.s_new.x * S.s_new.x + S.s_new.y * S.s_new.y;
	S.kr = dscal(S.tautilda, S.c_new / S.om_new);
}

// p_old = k0*p_old + k1*p_new + k2*v (becomes p_new); x += k3*p; v~ *= 1/beta (becomes v); r = d0*r + kr*v;
// partial |r|^2
template <typename C>
__global__ void __launch_bounds__(NT) qmr_v2(const RhsState *st, C *po, const C *pn, const C *v, C *vt, C *x, C *rv,
	size_t n3, double *part, int nbv)
{
	const int r = blockIdx.y;
	if (st[r].done) return;
	const RhsState &S = st[r];
	const auto k0 = cof<C>(S.k0), k1 = cof<C>(S.k1), k2 = cof<C>(S.k2), k3 = cof<C>(S.k3), kib = cof<C>(S.kib),
		kr = cof<C>(S.kr);
	const auto d0 = rof<C>(S.d0);
	typename AccOf<C>::T s[4] = {};
	VLOOP(n3) {
		const size_t j = r * n3 + i;
		const C p = cadd(cadd(cmul(k0, po[j]), cmul(k1, pn[j])), cmul(k2, v[j]));
		po[j] = p;
		x[j] = cadd(x[j], cmul(k3, p));
		const C vn = cmul(vt[j], kib);
		vt[j] = vn;
		const C rn = cadd(cscale(rv[j], d0), cmul(kr, vn));
		rv[j] = rn;
		acc_abs2(s[0], rn);
	}
	write_part(part, nbv, s, 1);
}

// ProgressReport (iterative.c:282-306) + loop condition (iterative.c:1467); partial |r|^2 in slot 0 unless half
// mode 0: |r|^2 from partial slot 0; 1: BiCGStab (also the next ro, half-step exit); 2: inprodRp1 already set by the
// method's scalar kernel (CSYM's |tau|^2)
__global__ void s_progress(RhsState *st, int *done, const double *part, int nbv, double *hist, int hist_cap, int mode)
{
	const int r = blockIdx.x;
	if (st[r].done) return;
	double s[4];
	sum_part(part, nbv, r, s, 2);
	if (threadIdx.x) return;
	RhsState &S = st[r];
	const bool bcgs = mode == 1;
	if (!S.half && mode != 2) S.inprodRp1 = s[0];
	if (bcgs && !S.half) S.ro_old = S.ro_new; // the next bs_s0 sums the r.r~* partials of bs_v3 itself
	if (S.inprodRp1 <= S.inprodR) {
		S.inprodR = S.inprodRp1;
		S.counter = 0;
	}
	else S.counter++;
	S.prev_err = sqrt(S.resid_scale * S.inprodRp1);
	if (S.niter < hist_cap) hist[(size_t)r * hist_cap + S.niter] = S.prev_err;
	S.niter++;
	S.done = !(S.inprodR > S.epsB && S.niter <= S.maxiter && S.counter <= S.mc);
	done[r] = S.done;
}

// ---------------- BiCGStab iteration ----------------

// ro_new = r.r~* (partial slots 1,2 of the previous bs_v3, or of the initial k_dot for the first iteration)
__global__ void bs_s0(RhsState *st, int *done, const double *part, int nbv)
{
	const int r = blockIdx.x;
	if (st[r].done) return;
	double s[4];
	sum_part(part, nbv, r, s, 3);
	if (threadIdx.x) return;
	RhsState &S = st[r];
	const double2 ro = dc(s[1], s[2]);
	S.ro_new = ro;
	if (S.niter == 1) {
		S.k0 = dc(0, 0);
		S.k1 = dc(0, 0);
		return;
	}
	const double2 t1 = dmul(ro, S.balpha), t2 = dmul(S.ro_old, S.omega);
	if (dabs(t2) / dabs(t1) < 1e-10) { // iterative.c:682-684
		S.status = ADDA_GB300_EBREAKDOWN;
		S.done = 1;
		done[r] = 1;
		return;
	}
	const double2 beta = ddiv(t1, t2);
	S.k0 = beta;
	const double2 bo = dmul(beta, S.omega);
	S.k1 = dc(-bo.x, -bo.y);
}

// p = k0*p + k1*v + r
template <typename C>
__global__ void __launch_bounds__(NT) bs_v1(const RhsState *st, C *p, const C *v, const C *rv, size_t n3)
{
	const int r = blockIdx.y;
	if (st[r].done) return;
	const auto k0 = cof<C>(st[r].k0), k1 = cof<C>(st[r].k1);
	VLOOP(n3) {
		const size_t j = r * n3 + i;
		p[j] = cadd(cadd(cmul(k0, p[j]), cmul(k1, v[j])), rv[j]);
	}
}

// alpha = ro_new / (v.r~*) (matvec epilogue slot 1,2)
__global__ void bs_s1(RhsState *st, int *done, const double *part, size_t nblk)
{
	const int r = blockIdx.x;
	if (st[r].done) return;
	double s[4];
	sum_part(part, nblk, r, s, 3);
	if (threadIdx.x) return;
	RhsState &S = st[r];
	const double2 t = dc(s[1], s[2]);
	if (dabs(t) / dabs(S.ro_new) < 1e-10) { // iterative.c:695-697
		S.status = ADDA_GB300_EBREAKDOWN;
		S.done = 1;
		done[r] = 1;
		return;
	}
	S.balpha = ddiv(S.ro_new, t);
	S.k0 = dc(-S.balpha.x, -S.balpha.y);
}

// s = k0*v + r ; partial |s|^2
template <typename C>
__global__ void __launch_bounds__(NT) bs_v2(const RhsState *st, C *sv, const C *v, const C *rv, size_t n3,
	double *part, int nbv)
{
	const int r = blockIdx.y;
	if (st[r].done) return;
	const auto k0 = cof<C>(st[r].k0);
	typename AccOf<C>::T s[4] = {};
	VLOOP(n3) {
		const size_t j = r * n3 + i;
		const C y = cadd(cmul(k0, v[j]), rv[j]);
		sv[j] = y;
		acc_abs2(s[0], y);
	}
	write_part(part, nbv, s, 1);
}

__global__ void bs_s2(RhsState *st, const double *part, int nbv)
{
	const int r = blockIdx.x;
	if (st[r].done) return;
	double s[4];
	sum_part(part, nbv, r, s, 1);
	if (threadIdx.x) return;
	RhsState &S = st[r];
	S.inprodRp1 = s[0];
	S.half = (S.inprodRp1 < S.epsB && !S.full) ? 1 : 0; // converged at the half step (iterative.c:703-707)
}

// omega = s.t* / |t|^2 (matvec epilogue: slot 0 = |t|^2, slots 1,2 = s.t*)
__global__ void bs_s3(RhsState *st, const double *part, size_t nblk)
{
	const int r = blockIdx.x;
	if (st[r].done) return;
	double s[4];
	sum_part(part, nblk, r, s, 3);
	if (threadIdx.x) return;
	RhsState &S = st[r];
	if (!S.half) S.omega = dscal(dc(s[1], s[2]), 1 / s[0]);
}

// x += alpha*p (+ omega*s); r = -omega*t + s; partials |r|^2, r.r~*
template <typename C>
__global__ void __launch_bounds__(NT) bs_v3(const RhsState *st, C *x, const C *p, const C *sv, const C *t, C *rv,
	const C *rt, size_t n3, double *part, int nbv)
{
	const int r = blockIdx.y;
	if (st[r].done) return;
	const RhsState &S = st[r];
	const auto a = cof<C>(S.balpha), om = cof<C>(S.omega), mom = cof<C>(dc(-S.omega.x, -S.omega.y));
	const bool half = S.half != 0;
	typename AccOf<C>::T s[4] = {};
	VLOOP(n3) {
		const size_t j = r * n3 + i;
		if (half) {
			x[j] = cadd(x[j], cmul(a, p[j]));
			continue;
		}
		x[j] = cadd(x[j], cadd(cmul(a, p[j]), cmul(om, sv[j])));
		const C y = cadd(cmul(mom, t[j]), sv[j]);
		rv[j] = y;
		acc_abs2(s[0], y);
		acc_cmulc(s[1], s[2], y, rt[j]);
	}
	write_part(part, nbv, s, 3);
}

// ---------------- BiCG_CS (COCG), iterative.c:490-637 ----------------

// ro_new = r.r (slots 1,2 of the previous r update or of the initial k_dot); breakdown |rT.r|/(r.r) (:559-560);
// beta = ro_new/ro_old for p = beta*p + r (:566-569)
__global__ void bg_s0(RhsState *st, int *done, const double *part, int nbv)
{
	const int r = blockIdx.x;
	if (st[r].done) return;
	double s[4];
	sum_part(part, nbv, r, s, 3);
	if (threadIdx.x) return;
	RhsState &S = st[r];
	S.ro_new = dc(s[1], s[2]);
	if (dabs(S.ro_new) / S.inprodR < 1e-10) {
		S.status = ADDA_GB300_EBREAKDOWN;
		S.done = 1;
		done[r] = 1;
		return;
	}
	S.k0 = (S.niter == 1) ? dc(0, 0) : ddiv(S.ro_new, S.ro_old);
}

// p = r (first iteration) or p = k0*p + r
template <typename C> __global__ void __launch_bounds__(NT) bg_v1(const RhsState *st, C *p, const C *rv, size_t n3)
{
	const int r = blockIdx.y;
	if (st[r].done) return;
	const bool first = st[r].niter == 1;
	const auto k0 = cof<C>(st[r].k0);
	VLOOP(n3) {
		const size_t j = r * n3 + i;
		p[j] = first ? rv[j] : cadd(cmul(k0, p[j]), rv[j]);
	}
}

// mu = p.Ap (matvec epilogue slots 1,2); breakdown |pT.A.p|/(rT.r) (:594-595); alpha = ro_new/mu
__global__ void bg_s1(RhsState *st, int *done, const double *part, size_t nblk)
{
	const int r = blockIdx.x;
	if (st[r].done) return;
	double s[4];
	sum_part(part, nblk, r, s, 3);
	if (threadIdx.x) return;
	RhsState &S = st[r];
	const double2 mu = dc(s[1], s[2]);
	if (dabs(mu) / dabs(S.ro_new) < 1e-10) {
		S.status = ADDA_GB300_EBREAKDOWN;
		S.done = 1;
		done[r] = 1;
		return;
	}
	S.balpha = ddiv(S.ro_new, mu);
	S.ro_old = S.ro_new;
}

// x += alpha*p; r -= alpha*Ap; partials |r|^2 and r.r
template <typename C>
__global__ void __launch_bounds__(NT) bg_v2(const RhsState *st, C *x, const C *p, C *rv, const C *Av, size_t n3,
	double *part, int nbv)
{
	const int r = blockIdx.y;
	if (st[r].done) return;
	const auto a = cof<C>(st[r].balpha), ma = cof<C>(dc(-st[r].balpha.x, -st[r].balpha.y));
	typename AccOf<C>::T s[4] = {};
	VLOOP(n3) {
		const size_t j = r * n3 + i;
		x[j] = cadd(x[j], cmul(a, p[j]));
		const C y = cadd(rv[j], cmul(ma, Av[j]));
		rv[j] = y;
		acc_abs2(s[0], y);
		acc_cmul(s[1], s[2], y, y);
	}
	write_part(part, nbv, s, 3);
}

// ---------------- CGNR, iterative.c:729-769 ----------------

// ro_new = |A^H r|^2 (epilogue slot 0 of the her matvec); beta = ro_new/ro_old
__global__ void cg_s0(RhsState *st, const double *part, size_t nblk)
{
	const int r = blockIdx.x;
	if (st[r].done) return;
	double s[4];
	sum_part(part, nblk, r, s, 1);
	if (threadIdx.x) return;
	RhsState &S = st[r];
	S.ro_new = dc(s[0], 0);
	S.k0 = dc(S.niter == 1 ? 0 : s[0] / S.ro_old.x, 0);
}

// p = A^H r (first iteration) or p = beta*p + A^H r
template <typename C> __global__ void __launch_bounds__(NT) cg_v1(const RhsState *st, C *p, const C *ahr, size_t n3)
{
	const int r = blockIdx.y;
	if (st[r].done) return;
	const bool first = st[r].niter == 1;
	const auto beta = rof<C>(st[r].k0.x);
	VLOOP(n3) {
		const size_t j = r * n3 + i;
		p[j] = first ? ahr[j] : cadd(cscale(p[j], beta), ahr[j]);
	}
}

// alpha = ro_new / |A.p|^2 (epilogue slot 0)
__global__ void cg_s1(RhsState *st, const double *part, size_t nblk)
{
	const int r = blockIdx.x;
	if (st[r].done) return;
	double s[4];
	sum_part(part, nblk, r, s, 1);
	if (threadIdx.x) return;
	RhsState &S = st[r];
	S.balpha = dc(S.ro_new.x / s[0], 0);
	S.ro_old = S.ro_new;
}

// x += alpha*p; r -= alpha*Ap (real alpha); partial |r|^2
template <typename C>
__global__ void __launch_bounds__(NT) cg_v2(const RhsState *st, C *x, const C *p, C *rv, const C *Av, size_t n3,
	double *part, int nbv)
{
	const int r = blockIdx.y;
	if (st[r].done) return;
	const auto a = rof<C>(st[r].balpha.x), ma = rof<C>(-st[r].balpha.x);
	typename AccOf<C>::T s[4] = {};
	VLOOP(n3) {
		const size_t j = r * n3 + i;
		x[j] = cadd(x[j], cscale(p[j], a));
		const C y = cadd(rv[j], cscale(Av[j], ma));
		rv[j] = y;
		acc_abs2(s[0], y);
	}
	write_part(part, nbv, s, 1);
}

// ---------------- CSYM, iterative.c:773-892 ----------------

// PHASE_INIT: tau = |r_0|, c_0 = 1, c_-1 = 0, s_0 = s_-1 = 0; q_1 = r_0(*)/tau (cs_init_v)
__global__ void cs_init_s(RhsState *st)
{
	const int r = blockIdx.x;
	if (threadIdx.x || st[r].done) return;
	RhsState &S = st[r];
	const double tau = sqrt(S.inprodR);
	S.tautilda = dc(tau, 0);
	S.kib = dc(1 / tau, 0);
	S.c_new = 1;
	S.c_old = 0;
	S.s_new = S.s_old = dc(0, 0);
	S.cs_beta = 0;
}

// a = conj(a) * kib.x (nMultSelf_conj)
template <typename C> __global__ void __launch_bounds__(NT) cs_conj_scale(const RhsState *st, C *a, size_t n3)
{
	const int r = blockIdx.y;
	if (st[r].done) return;
	const auto k = rof<C>(st[r].kib.x);
	VLOOP(n3) {
		const size_t j = r * n3 + i;
		a[j] = cscale(cconj(a[j]), k);
	}
}

// alpha = q.Aq (epilogue slots 1,2); eta, gamma, theta (:819-824); w coefficients k0 = -alpha, k1 = -beta
__global__ void cs_s1(RhsState *st, const double *part, size_t nblk)
{
	const int r = blockIdx.x;
	if (st[r].done) return;
	double s[4];
	sum_part(part, nblk, r, s, 3);
	if (threadIdx.x) return;
	RhsState &S = st[r];
	const double2 alpha = dc(s[1], s[2]);
	const double beta = S.cs_beta;
	S.eta = dadd(dc(S.c_old * S.c_new * beta, 0), dmul(alpha, dconj(S.s_new)));
	S.zetat = dsub(dscal(alpha, S.c_new), dscal(S.s_new, S.c_old * beta)); // gamma
	S.theta = dscal(dconj(S.s_old), beta);
	S.k0 = dc(-alpha.x, -alpha.y);
	S.k1 = dc(-beta, 0);
}

// w = -beta*q_old(*) - alpha*q_new(*) + Aq (q_0 = 0 in the first iteration), stored in q_old; partial |w|^2
template <typename C>
__global__ void __launch_bounds__(NT) cs_v1(const RhsState *st, C *qo, const C *qn, const C *Av, size_t n3, double *part,
	int nbv)
{
	const int r = blockIdx.y;
	if (st[r].done) return;
	const bool first = st[r].niter == 1;
	const auto k0 = cof<C>(st[r].k0);
	const auto k1 = rof<C>(st[r].k1.x);
	typename AccOf<C>::T s[4] = {};
	VLOOP(n3) {
		const size_t j = r * n3 + i;
		C w = cadd(cmul(k0, cconj(qn[j])), Av[j]);
		if (!first) w = cadd(cscale(cconj(qo[j]), k1), w);
		qo[j] = w;
		acc_abs2(s[0], w);
	}
	write_part(part, nbv, s, 1);
}

// beta_(k+1) = |w|; Givens rotation c_k, s_k, 1/ksi_k (:832-862); p and x coefficients; tau_(k+1) = -s_k*tau_k and
// |r_k| = |tau_(k+1)|
__global__ void cs_s2(RhsState *st, int *done, const double *part, int nbv)
{
	const int r = blockIdx.x;
	if (st[r].done) return;
	double s[4];
	sum_part(part, nbv, r, s, 1);
	if (threadIdx.x) return;
	RhsState &S = st[r];
	const double beta = sqrt(s[0]);
	S.cs_beta = beta;
	S.c_old = S.c_new;
	S.s_old = S.s_new;
	const double2 gamma = S.zetat;
	double g = dabs(gamma);
	double2 invksi;
	if (g == 0) {
		if (beta == 0) { // singular interaction matrix (iterative.c:845)
			S.status = ADDA_GB300_EBREAKDOWN;
			S.done = 1;
			done[r] = 1;
			return;
		}
		S.c_new = 0;
		S.s_new = dc(1, 0);
		invksi = dc(1 / beta, 0);
	}
	else {
		if (g < beta) {
			g = g / beta;
			S.c_new = g / sqrt(1 + g * g);
		}
		else {
			g = beta / g;
			S.c_new = 1 / sqrt(1 + g * g);
		}
		invksi = ddiv(dc(S.c_new, 0), gamma);
		S.s_new = dscal(invksi, beta);
	}
	// p_out = k2*p_old + k1*p_new + k3*q_new (terms absent in the first two iterations); x += kr*p_out
	S.k3 = invksi;
	S.k1 = (S.niter >= 2) ? dmul(dc(-S.eta.x, -S.eta.y), invksi) : dc(0, 0);
	S.k2 = (S.niter >= 3) ? dmul(dc(-S.theta.x, -S.theta.y), invksi) : dc(0, 0);
	S.kr = dscal(S.tautilda, S.c_new);
	S.kib = dc(1 / beta, 0);
	S.tautilda = dmul(dc(-S.s_new.x, -S.s_new.y), S.tautilda);
	S.inprodRp1 = S.tautilda.x * S.tautilda.x + S.tautilda.y * S.tautilda.y;
}

// p_out (into the p_old buffer) = k2*p_old + k1*p_new + k3*q_new; x += kr*p_out; q_old = w(*)/beta
template <typename C>
__global__ void __launch_bounds__(NT) cs_v2(const RhsState *st, C *po, const C *pn, const C *qn, C *qo, C *x, size_t n3)
{
	const int r = blockIdx.y;
	if (st[r].done) return;
	const RhsState &S = st[r];
	const int it = S.niter;
	const auto k1 = cof<C>(S.k1), k2 = cof<C>(S.k2), k3 = cof<C>(S.k3), kr = cof<C>(S.kr);
	const auto kib = rof<C>(S.kib.x);
	VLOOP(n3) {
		const size_t j = r * n3 + i;
		C pv = cmul(k3, qn[j]);
		if (it >= 2) pv = cadd(cmul(k1, pn[j]), pv);
		if (it >= 3) pv = cadd(cmul(k2, po[j]), pv);
		po[j] = pv;
		x[j] = cadd(x[j], cmul(kr, pv));
		qo[j] = cscale(cconj(qo[j]), kib);
	}
}

// ---------------- QMR_CS_2, iterative.c:1038-1132 ----------------

// PHASE_INIT: ro_1 = |r_0|, v~_1 = r_0 (copied by the caller), c_0 = eps_0 = 1, theta_0 = 0, eta_0 = -1; delta_1 from
// the r.r partials (slots 1,2 of k_dot) as (r.r)/ro_1^2, i.e. v_1.v_1 with v_1 = v~_1/ro_1
__global__ void q2_init_s(RhsState *st, const double *part, int nbv)
{
	const int r = blockIdx.x;
	double s[4];
	sum_part(part, nbv, r, s, 3);
	if (threadIdx.x || st[r].done) return;
	RhsState &S = st[r];
	S.q2_ro = sqrt(S.inprodR);
	S.q2_c = 1;
	S.q2_eps = dc(1, 0);
	S.q2_theta = 0;
	S.q2_eta = dc(-1, 0);
	S.q2_delta = dscal(dc(s[1], s[2]), 1 / S.inprodR);
}

// resumed from a checkpoint: delta_k = v_k.v_k with v_k = v~_k/ro_k, from the v~.v~ partials (slots 1,2 of k_dot)
__global__ void q2_resume_s(RhsState *st, const double *part, int nbv)
{
	const int r = blockIdx.x;
	double s[4];
	sum_part(part, nbv, r, s, 3);
	if (threadIdx.x || st[r].done) return;
	RhsState &S = st[r];
	S.q2_delta = dscal(dc(s[1], s[2]), 1 / (S.q2_ro * S.q2_ro));
}

// delta_k test (:1086-1089); p coefficient -ro_k*delta_k/eps_(k-1) (:1091-1094); v scale 1/ro_k
__global__ void q2_s0(RhsState *st, int *done)
{
	const int r = blockIdx.x;
	if (threadIdx.x || st[r].done) return;
	RhsState &S = st[r];
	if (dabs(S.q2_delta) < 1e-10) {
		S.status = ADDA_GB300_EBREAKDOWN;
		S.done = 1;
		done[r] = 1;
		return;
	}
	S.kib = dc(1 / S.q2_ro, 0);
	S.k0 = (S.niter == 1) ? dc(0, 0) : dscal(ddiv(S.q2_delta, S.q2_eps), -S.q2_ro);
}

// v = v~/ro_k; p = v (first iteration) or p = k0*p + v
template <typename C> __global__ void __launch_bounds__(NT) q2_v1(const RhsState *st, C *v, C *p, size_t n3)
{
	const int r = blockIdx.y;
	if (st[r].done) return;
	const bool first = st[r].niter == 1;
	const auto ir = rof<C>(st[r].kib.x);
	const auto k0 = cof<C>(st[r].k0);
	VLOOP(n3) {
		const size_t j = r * n3 + i;
		const C vv = cscale(v[j], ir);
		v[j] = vv;
		p[j] = first ? vv : cadd(cmul(k0, p[j]), vv);
	}
}

// eps_k = p.Ap (epilogue slots 1,2); beta_k = eps_k/delta_k; test |eps_k| (:1104-1107)
__global__ void q2_s1(RhsState *st, int *done, const double *part, size_t nblk)
{
	const int r = blockIdx.x;
	if (st[r].done) return;
	double s[4];
	sum_part(part, nblk, r, s, 3);
	if (threadIdx.x) return;
	RhsState &S = st[r];
	S.q2_eps = dc(s[1], s[2]);
	S.q2_beta = ddiv(S.q2_eps, S.q2_delta);
	if (dabs(S.q2_eps) < 1e-10) {
		S.status = ADDA_GB300_EBREAKDOWN;
		S.done = 1;
		done[r] = 1;
		return;
	}
	S.k1 = dc(-S.q2_beta.x, -S.q2_beta.y);
}

// v~_(k+1) = A.p_k - beta_k*v_k (in place); partials |v~|^2 and v~.v~
template <typename C>
__global__ void __launch_bounds__(NT) q2_v2(const RhsState *st, C *v, const C *Av, size_t n3, double *part, int nbv)
{
	const int r = blockIdx.y;
	if (st[r].done) return;
	const auto k1 = cof<C>(st[r].k1);
	typename AccOf<C>::T s[4] = {};
	VLOOP(n3) {
		const size_t j = r * n3 + i;
		const C y = cadd(cmul(k1, v[j]), Av[j]);
		v[j] = y;
		acc_abs2(s[0], y);
		acc_cmul(s[1], s[2], y, y);
	}
	write_part(part, nbv, s, 3);
}

// ro_(k+1) = |v~_(k+1)|; theta_k, c_k, |s_k|^2, eta_k (:1111-1120); coefficients of d, x, r; delta_(k+1)
__global__ void q2_s2(RhsState *st, const double *part, int nbv)
{
	const int r = blockIdx.x;
	if (st[r].done) return;
	double s[4];
	sum_part(part, nbv, r, s, 3);
	if (threadIdx.x) return;
	RhsState &S = st[r];
	const double ro_new = sqrt(s[0]);
	const double theta_new = ro_new / (S.q2_c * dabs(S.q2_beta));
	const double th2 = theta_new * theta_new;
	const double c_new = 1 / sqrt(1 + th2);
	const double sabs2 = th2 / (1 + th2);
	const double cr = c_new / S.q2_c;
	S.q2_eta = ddiv(dscal(S.q2_eta, -S.q2_ro * cr * cr), S.q2_beta);
	const double tc = S.q2_theta * c_new;
	S.d0 = (S.niter == 1) ? 0 : tc * tc; // d = d0*d + eta*p
	S.k2 = S.q2_eta;
	S.kr = dc(-S.q2_eta.x, -S.q2_eta.y); // r = sabs2*r - eta*v~
	S.k3 = dc(sabs2, 0);
	S.q2_delta = dscal(dc(s[1], s[2]), 1 / s[0]); // v_(k+1).v_(k+1) with v_(k+1) = v~_(k+1)/ro_(k+1)
	S.q2_ro = ro_new;
	S.q2_theta = theta_new;
	S.q2_c = c_new;
}

// d = eta*p (first iteration) or d0*d + eta*p; x += d; r = sabs2*r - eta*v~; partial |r|^2
template <typename C>
__global__ void __launch_bounds__(NT) q2_v3(const RhsState *st, C *d, const C *p, C *x, C *rv, const C *v, size_t n3,
	double *part, int nbv)
{
	const int r = blockIdx.y;
	if (st[r].done) return;
	const RhsState &S = st[r];
	const bool first = S.niter == 1;
	const auto eta = cof<C>(S.k2), me = cof<C>(S.kr);
	const auto d0 = rof<C>(S.d0), sa = rof<C>(S.k3.x);
	typename AccOf<C>::T s[4] = {};
	VLOOP(n3) {
		const size_t j = r * n3 + i;
		const C dv = first ? cmul(eta, p[j]) : cadd(cscale(d[j], d0), cmul(eta, p[j]));
		d[j] = dv;
		x[j] = cadd(x[j], dv);
		const C y = cadd(cscale(rv[j], sa), cmul(me, v[j]));
		rv[j] = y;
		acc_abs2(s[0], y);
	}
	write_part(part, nbv, s, 1);
}

// ---------------- BCGS2 = BiCGstab(2), iterative.c:340-487 ----------------
// r_0..2 in r, v1, v3; u_0..2 in v2, Av, v4; r~_0 in p. Four matvecs per iteration.

__global__ void b2_init_s(RhsState *st)
{
	const int r = blockIdx.x;
	if (threadIdx.x || st[r].done) return;
	st[r].b2_rho0 = dc(-1, 0);
	st[r].b2_alpha = dc(0, 0);
}

// rho1 = r_j.r~0 (slots 1,2 of part); 1/|beta| test (:402-405); beta = alpha*rho1/rho0; rho0 = rho1
__global__ void b2_s_beta(RhsState *st, int *done, const double *part, size_t nblk, int j)
{
	const int r = blockIdx.x;
	if (st[r].done) return;
	double s[4];
	sum_part(part, nblk, r, s, 3);
	if (threadIdx.x) return;
	RhsState &S = st[r];
	const double2 rho1 = dc(s[1], s[2]);
	if (S.niter == 1 && j == 0) S.k0 = dc(0, 0);
	else {
		if (dabs(S.b2_rho0) / (dabs(rho1) * dabs(S.b2_alpha)) < 1e-10) {
			S.status = ADDA_GB300_EBREAKDOWN;
			S.done = 1;
			done[r] = 1;
			return;
		}
		const double2 beta = ddiv(dmul(S.b2_alpha, rho1), S.b2_rho0);
		S.k0 = dc(-beta.x, -beta.y);
	}
	S.b2_rho0 = rho1;
	S.b2_rho1 = rho1;
}

// u_i = r_i - beta*u_i for i <= j (u_0 = r_0 in the very first step)
template <typename C>
__global__ void __launch_bounds__(NT) b2_vu(const RhsState *st, C *u0, const C *r0, C *u1, const C *r1, size_t n3, int j)
{
	const int r = blockIdx.y;
	if (st[r].done) return;
	const bool copy = st[r].niter == 1 && j == 0;
	const auto k0 = cof<C>(st[r].k0);
	VLOOP(n3) {
		const size_t q = r * n3 + i;
		u0[q] = copy ? r0[q] : cadd(cmul(k0, u0[q]), r0[q]);
		if (j == 1) u1[q] = cadd(cmul(k0, u1[q]), r1[q]);
	}
}

// sigma = u_(j+1).r~0 (matvec epilogue slots 1,2); test (:411-414); alpha = rho1/sigma
__global__ void b2_s_alpha(RhsState *st, int *done, const double *part, size_t nblk)
{
	const int r = blockIdx.x;
	if (st[r].done) return;
	double s[4];
	sum_part(part, nblk, r, s, 3);
	if (threadIdx.x) return;
	RhsState &S = st[r];
	const double2 sigma = dc(s[1], s[2]);
	if (dabs(sigma) / dabs(S.b2_rho1) < 1e-10) {
		S.status = ADDA_GB300_EBREAKDOWN;
		S.done = 1;
		done[r] = 1;
		return;
	}
	S.b2_alpha = ddiv(S.b2_rho1, sigma);
}

// x += alpha*u_0; r_i -= alpha*u_(i+1) for i <= j; for j = 1 also the partial |r_0|^2 (Z_00, slot 0)
template <typename C>
__global__ void __launch_bounds__(NT) b2_vx(const RhsState *st, C *x, const C *u0, C *r0, const C *u1, C *r1,
	const C *u2, size_t n3, int j, double *part, int nbv)
{
	const int r = blockIdx.y;
	if (st[r].done) return;
	const auto a = cof<C>(st[r].b2_alpha), ma = cof<C>(dc(-st[r].b2_alpha.x, -st[r].b2_alpha.y));
	typename AccOf<C>::T s[4] = {};
	VLOOP(n3) {
		const size_t q = r * n3 + i;
		x[q] = cadd(x[q], cmul(a, u0[q]));
		const C y = cadd(r0[q], cmul(ma, u1[q]));
		r0[q] = y;
		if (j == 1) {
			r1[q] = cadd(r1[q], cmul(ma, u2[q]));
			acc_abs2(s[0], y);
		}
	}
	if (j == 1) write_part(part, nbv, s, 1);
}

// Gram entries Z_11, Z_22, Z_10 = r_0.r_1*, Z_20 = r_0.r_2*, Z_21 = r_1.r_2* (8 slots of xpart)
template <typename C>
__global__ void __launch_bounds__(NT) b2_gram(const RhsState *st, const C *r0, const C *r1, const C *r2, size_t n3,
	double *xpart, int nbv)
{
	const int r = blockIdx.y;
	if (st[r].done) return;
	typename AccOf<C>::T s[8] = {};
	VLOOP(n3) {
		const size_t q = r * n3 + i;
		const C a = r0[q], b = r1[q], c = r2[q];
		acc_abs2(s[0], b);
		acc_abs2(s[1], c);
		acc_cmulc(s[2], s[3], a, b);
		acc_cmulc(s[4], s[5], a, c);
		acc_cmulc(s[6], s[7], b, c);
	}
	double v[8];
	for (int k = 0; k < 8; k++) v[k] = acc_val(s[k]);
	block_sum4(v, 4);
	block_sum4(v + 4, 4);
	if (threadIdx.x == 0) {
		double *o = xpart + ((size_t)blockIdx.y * nbv + blockIdx.x) * 8;
		for (int k = 0; k < 8; k++) o[k] = v[k];
	}
}

// convex polynomial part (:427-480): minimal-residual combination of r_0..2 from the Gram matrix; y0[1], y0[2],
// omega = y0[2], |r|^2 = y0.Z.y0, rho0 *= -omega
__global__ void b2_s_final(RhsState *st, const double *vpart, const double *xpart, int nbv)
{
	const int r = blockIdx.x;
	if (st[r].done) return;
	__shared__ double sh[8][NT / 32];
	double v[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
	for (int b = threadIdx.x; b < nbv; b += blockDim.x) {
		v[0] += vpart[((size_t)r * nbv + b) * 4];
		for (int k = 0; k < 8; k++) v[1 + k] += xpart[((size_t)r * nbv + b) * 8 + k];
	}
	double tot[9];
	for (int k = 0; k < 9; k++) {
		double x = v[k];
		for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
		__syncthreads();
		if ((threadIdx.x & 31) == 0) sh[0][threadIdx.x >> 5] = x;
		__syncthreads();
		tot[k] = 0;
		for (int w = 0; w < NT / 32; w++) tot[k] += sh[0][w];
	}
	if (threadIdx.x) return;
	RhsState &S = st[r];
	double2 Z[3][3];
	Z[0][0] = dc(tot[0], 0);
	Z[1][1] = dc(tot[1], 0);
	Z[2][2] = dc(tot[2], 0);
	Z[1][0] = dc(tot[3], tot[4]);
	Z[2][0] = dc(tot[5], tot[6]);
	Z[2][1] = dc(tot[7], tot[8]);
	Z[0][1] = dconj(Z[1][0]);
	Z[0][2] = dconj(Z[2][0]);
	Z[1][2] = dconj(Z[2][1]);
	double2 y0[3] = {dc(-1, 0), ddiv(Z[1][0], Z[1][1]), dc(0, 0)};
	const double2 yl[3] = {dc(0, 0), ddiv(Z[1][2], Z[1][1]), dc(-1, 0)};
	double2 zy0[3], zyl[3];
	for (int i = 0; i < 3; i++) {
		zy0[i] = zyl[i] = dc(0, 0);
		for (int j = 0; j < 3; j++) {
			zy0[i] = dadd(zy0[i], dmul(Z[i][j], y0[j]));
			zyl[i] = dadd(zyl[i], dmul(Z[i][j], yl[j]));
		}
	}
	double d = 0;
	for (int i = 0; i < 3; i++) d += dmul(zy0[i], dconj(y0[i])).x;
	const double kappa0 = sqrt(d);
	d = 0;
	for (int i = 0; i < 3; i++) d += dmul(zyl[i], dconj(yl[i])).x;
	const double kappal = sqrt(d);
	double2 varrho = dc(0, 0);
	for (int i = 0; i < 3; i++) varrho = dadd(varrho, dmul(zy0[i], dconj(yl[i])));
	varrho = dscal(varrho, 1 / (kappa0 * kappal));
	d = dabs(varrho);
	const double2 hatgamma = dscal(varrho, (d > 0.7 ? d : 0.7) / d);
	const double2 t = dscal(hatgamma, -kappa0 / kappal);
	for (int i = 0; i < 3; i++) y0[i] = dadd(y0[i], dmul(t, yl[i]));
	const double2 omega = y0[2];
	S.b2_y1 = y0[1];
	S.b2_y2 = y0[2];
	for (int i = 0; i < 3; i++) {
		zy0[i] = dc(0, 0);
		for (int j = 0; j < 3; j++) zy0[i] = dadd(zy0[i], dmul(Z[i][j], y0[j]));
	}
	d = 0;
	for (int i = 0; i < 3; i++) d += dmul(zy0[i], dconj(y0[i])).x;
	S.inprodRp1 = d;
	S.b2_rho0 = dmul(S.b2_rho0, dc(-omega.x, -omega.y));
}

// u_0 -= y1*u_1 + y2*u_2; x += y1*r_0 + y2*r_1; r_0 -= y1*r_1 + y2*r_2; partial r_0.r~0 for the next iteration
template <typename C>
__global__ void __launch_bounds__(NT) b2_vfinal(const RhsState *st, C *u0, const C *u1, const C *u2, C *x, C *r0,
	const C *r1, const C *r2, const C *rt, size_t n3, double *part, int nbv)
{
	const int r = blockIdx.y;
	if (st[r].done) return;
	const auto y1 = cof<C>(st[r].b2_y1), y2 = cof<C>(st[r].b2_y2);
	const auto my1 = cof<C>(dc(-st[r].b2_y1.x, -st[r].b2_y1.y)), my2 = cof<C>(dc(-st[r].b2_y2.x, -st[r].b2_y2.y));
	typename AccOf<C>::T s[4] = {};
	VLOOP(n3) {
		const size_t q = r * n3 + i;
		u0[q] = cadd(cadd(u0[q], cmul(my1, u1[q])), cmul(my2, u2[q]));
		const C a = r0[q], b = r1[q];
		x[q] = cadd(cadd(x[q], cmul(y1, a)), cmul(y2, b));
		const C y = cadd(cadd(a, cmul(my1, b)), cmul(my2, r2[q]));
		r0[q] = y;
		acc_cmulc(s[1], s[2], y, rt[q]);
	}
	write_part(part, nbv, s, 3);
}

// ---------------- FP64 helpers for the refinement loop and the results ----------------

// x64 (+)= d (float or double), depending on accumulate
template <typename C>
__global__ void __launch_bounds__(NT) k_accum(double2 *x64, const C *d, size_t n3, int accumulate, const int *skip)
{
	const int r = blockIdx.y;
	if (skip && skip[r]) return;
	VLOOP(n3) {
		const double2 v = to_d2(d[r * n3 + i]);
		x64[r * n3 + i] = accumulate ? make_double2(x64[r * n3 + i].x + v.x, x64[r * n3 + i].y + v.y) : v;
	}
}

// r64 = b64 - Ax64; partial |r|^2; also the copy of r64 (in the inner solver's vector type) for the next inner solve
template <typename C>
__global__ void __launch_bounds__(NT) k_resid64(const double2 *b, const double2 *Ax, double2 *r64, C *rf,
	size_t n3, double *part, int nbv)
{
	const int r = blockIdx.y;
	double s[4] = {0, 0, 0, 0};
	VLOOP(n3) {
		const size_t j = r * n3 + i;
		const double2 d = make_double2(b[j].x - Ax[j].x, b[j].y - Ax[j].y);
		r64[j] = d;
		rf[j] = from_d2<C>(d);
		s[0] += d.x * d.x + d.y * d.y;
	}
	write_part(part, nbv, s, 1);
}

template <typename C> __global__ void __launch_bounds__(NT) k_from64(C *dst, const double2 *src, size_t n)
{
	for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
		dst[i] = from_d2<C>(src[i]);
}

// p = S.x (iterative.c:1527)
__global__ void __launch_bounds__(NT) k_pvec(const double2 *x, double2 *p, const double2 *ccs, int per_dip, int nmat,
	const uint8_t *mat, size_t N, int rpp, size_t lst)
{
	const int r = blockIdx.y;
	mat += (size_t)(r / rpp) * lst; // RHS r's particle (group contexts)
	const size_t n3 = 3 * N;
	VLOOP(n3) {
		const size_t d = i / 3;
		const int comp = (int)(i % 3);
		const double2 s = per_dip ? ccs[((size_t)r * N + d) * 3 + comp] : ccs[((size_t)r * nmat + mat[d]) * 3 + comp];
		p[(size_t)r * n3 + i] = dmul(s, x[(size_t)r * n3 + i]);
	}
}

// cross-section sums per RHS: sum_j P_j exp(-i kd n.pos_j) (CalcFieldFree, crosssec.c:506-586) and
// sum_j sum_c (-Im(1/cc) - 2k^3/3)|P_jc|^2 (AbsCross, crosssec.c:866-882)
__global__ void __launch_bounds__(NT) k_cross(const double2 *P, const uint16_t *pos, const double2 *cc, int per_dip,
	int nmat, const uint8_t *mat, size_t N, const double *prop, double kd, double k3, double *part, int nbv, int rpp,
	size_t lst)
{
	const int r = blockIdx.y;
	mat += (size_t)(r / rpp) * lst; // RHS r's particle (group contexts)
	pos += (size_t)(r / rpp) * lst * 3;
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
			const double2 a = per_dip ? cc[((size_t)r * N + d) * 3 + c] : cc[((size_t)r * nmat + mat[d]) * 3 + c];
			const double im_inv = -a.y / (a.x * a.x + a.y * a.y); // Im(1/cc)
			const double mult = -im_inv - 2 * k3 / 3;
			s[6] += mult * (p.x * p.x + p.y * p.y);
		}
	}
	__shared__ double sh[7][NT / 32];
	const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
	for (int j = 0; j < 7; j++) {
		double v = s[j];
		for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
		if (lane == 0) sh[j][wid] = v;
	}
	__syncthreads();
	if (threadIdx.x == 0) {
		double *o = part + ((size_t)r * nbv + blockIdx.x) * 8;
		for (int j = 0; j < 7; j++) {
			double v = 0;
			for (int w = 0; w < NT / 32; w++) v += sh[j][w];
			o[j] = v;
		}
	}
}

// general-beam cross-section sums per RHS: sum_j Im(P_j . conj(Einc_j)) (ExtCross, crosssec.c:823-830) and the AbsCross
// sum of k_cross
__global__ void __launch_bounds__(NT) k_cross_beam(const double2 *P, const double2 *E, const double2 *cc, int per_dip,
	int nmat, const uint8_t *mat, size_t N, double k3, double *part, int nbv, int rpp, size_t lst)
{
	const int r = blockIdx.y;
	mat += (size_t)(r / rpp) * lst; // RHS r's particle (group contexts)
	double s[2] = {0, 0};
	for (size_t d = blockIdx.x * (size_t)blockDim.x + threadIdx.x; d < N; d += (size_t)gridDim.x * blockDim.x) {
		for (int c = 0; c < 3; c++) {
			const size_t j = ((size_t)r * N + d) * 3 + c;
			const double2 p = P[j], e = E[j];
			s[0] += p.y * e.x - p.x * e.y;
			const double2 a = per_dip ? cc[((size_t)r * N + d) * 3 + c] : cc[((size_t)r * nmat + mat[d]) * 3 + c];
			const double im_inv = -a.y / (a.x * a.x + a.y * a.y);
			s[1] += (-im_inv - 2 * k3 / 3) * (p.x * p.x + p.y * p.y);
		}
	}
	__shared__ double sh[2][NT / 32];
	const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
	for (int j = 0; j < 2; j++) {
		double v = s[j];
		for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
		if (lane == 0) sh[j][wid] = v;
	}
	__syncthreads();
	if (threadIdx.x == 0) {
		double *o = part + ((size_t)r * nbv + blockIdx.x) * 8;
		for (int j = 0; j < 2; j++) {
			double v = 0;
			for (int w = 0; w < NT / 32; w++) v += sh[j][w];
			o[j] = v;
		}
	}
}

// scattering amplitudes (CalcFieldFree, crosssec.c:506-596), first stage: per block partial sums of
// P_j exp(-i kd n.pos_j) for direction blockIdx.y and RHS blockIdx.z (6 doubles: Re/Im of the 3 components)
__global__ void __launch_bounds__(NT) k_field(const double2 *P, const uint16_t *pos, size_t N, const double *dirs,
	double kd, double *part, int rpp, size_t lst)
{
	const int d = blockIdx.y, r = blockIdx.z, nb = gridDim.x;
	pos += (size_t)(r / rpp) * lst * 3; // RHS r's particle (group contexts)
	const double n0 = dirs[3 * d], n1 = dirs[3 * d + 1], n2 = dirs[3 * d + 2];
	double s[6] = {0, 0, 0, 0, 0, 0};
	for (size_t j = blockIdx.x * (size_t)NT + threadIdx.x; j < N; j += (size_t)nb * NT) {
		const double ph = -kd * (n0 * pos[3 * j] + n1 * pos[3 * j + 1] + n2 * pos[3 * j + 2]);
		double sn, cs;
		sincos(ph, &sn, &cs);
		for (int c = 0; c < 3; c++) {
			const double2 p = P[((size_t)r * N + j) * 3 + c];
			s[2 * c] += p.x * cs - p.y * sn;
			s[2 * c + 1] += p.x * sn + p.y * cs;
		}
	}
	block_sum4(s, 4);
	block_sum4(s + 4, 2);
	if (threadIdx.x == 0) {
		double *o = part + (((size_t)r * gridDim.y + d) * nb + blockIdx.x) * 6;
		for (int k = 0; k < 6; k++) o[k] = s[k];
	}
}

// second stage, one thread per (direction, RHS): fixed-order sum of the block partials, (I - nn), and the factor
// (-i k^3) exp(-i k r0.n) with r0 the centre offset of the box's first dipole (make_particle.c:2305-2308)
__global__ void k_field_fin(const double *part, int nb, int ndir, int R, const double *dirs, double k, double gs,
	int bX, int bY, int bZ, double2 *out)
{
	const int t = blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= ndir * R) return;
	const int r = t / ndir, d = t % ndir;
	const double n[3] = {dirs[3 * d], dirs[3 * d + 1], dirs[3 * d + 2]};
	double2 sum[3] = {dc(0, 0), dc(0, 0), dc(0, 0)};
	const double *p = part + ((size_t)r * ndir + d) * nb * 6;
	for (int b = 0; b < nb; b++)
		for (int c = 0; c < 3; c++) sum[c] = dadd(sum[c], dc(p[b * 6 + 2 * c], p[b * 6 + 2 * c + 1]));
	const double2 dpr = dadd(dadd(dscal(sum[0], n[0]), dscal(sum[1], n[1])), dscal(sum[2], n[2]));
	const double r0[3] = {-gs * (bX - 1) / 2.0, -gs * (bY - 1) / 2.0, -gs * (bZ - 1) / 2.0};
	double sn, cs;
	sincos(-k * (r0[0] * n[0] + r0[1] * n[1] + r0[2] * n[2]), &sn, &cs);
	const double k3 = k * k * k;
	const double2 amp = dc(sn * k3, -cs * k3); // -i k^3 (cs + i sn)
	for (int c = 0; c < 3; c++) out[((size_t)r * ndir + d) * 3 + c] = dmul(amp, dsub(sum[c], dscal(dpr, n[c])));
}

// adjoint right-hand sides for the VJP (written as "incident fields" E so that the solver's b = S.E gives the scaled
// system): E0_j = c_j incpol with c_j = (4pi/k^2)(-i k^3) exp(-i k r0.n) exp(-i kd n.pos_j)  (d Cext/d P_j), and
// E1_j = conj(mu_j P_j) with mu_jc = -Im(1/alpha_jc) - 2k^3/3  (half the gradient of Cabs/(4 pi k) w.r.t. conj P)
__global__ void __launch_bounds__(NT) k_adj_rhs(double2 *E, const double2 *P, const uint16_t *pos, const double2 *cc,
	int per_dip, int nmat, const uint8_t *mat, size_t N, double n0, double n1, double n2, double e0, double e1,
	double e2, double kd, double k, double ph0)
{
	const double PI = 3.14159265358979323846;
	const double k3 = k * k * k;
	for (size_t d = blockIdx.x * (size_t)blockDim.x + threadIdx.x; d < N; d += (size_t)gridDim.x * blockDim.x) {
		const double ph = ph0 - kd * (n0 * pos[3 * d] + n1 * pos[3 * d + 1] + n2 * pos[3 * d + 2]);
		double sn, cs;
		sincos(ph, &sn, &cs);
		// c = (4pi/k^2) * (-i k^3) * exp(i ph) = 4 pi k (sin ph - i cos ph)
		const double cr = 4 * PI * k * sn, ci = -4 * PI * k * cs;
		const double ev[3] = {e0, e1, e2};
		for (int c = 0; c < 3; c++) {
			E[d * 3 + c] = make_double2(cr * ev[c], ci * ev[c]);
			const double2 a = per_dip ? cc[d * 3 + c] : cc[(size_t)mat[d] * 3 + c];
			const double mu = a.y / (a.x * a.x + a.y * a.y) - 2 * k3 / 3;
			const double2 p = P[d * 3 + c];
			E[(N + d) * 3 + c] = make_double2(mu * p.x, -mu * p.y);
		}
	}
}

// per-dipole gradients from the forward P and the adjoint solutions lambda (extinction) and nu (absorption)
__global__ void __launch_bounds__(NT) k_vjp_grad(const double2 *P, const double2 *lam, const double2 *nu,
	const double2 *f, size_t N, double k, double *gext, double *gabs)
{
	const double PI = 3.14159265358979323846;
	for (size_t d = blockIdx.x * (size_t)blockDim.x + threadIdx.x; d < N; d += (size_t)gridDim.x * blockDim.x) {
		double lr = 0, li = 0, nr = 0, ni = 0, p2 = 0;
		for (int c = 0; c < 3; c++) {
			const double2 p = P[d * 3 + c], l = lam[d * 3 + c], v = nu[d * 3 + c];
			lr += l.x * p.x - l.y * p.y;
			li += l.x * p.y + l.y * p.x;
			nr += v.x * p.x - v.y * p.y;
			ni += v.x * p.y + v.y * p.x;
			p2 += p.x * p.x + p.y * p.y;
		}
		const double2 fd = f[d];
		// dF/dchi = -f sum(lambda P); dCext/dRe = Re, dCext/dIm = -Im
		const double gr = -(fd.x * lr - fd.y * li), gi = -(fd.x * li + fd.y * lr);
		gext[2 * d] = gr;
		gext[2 * d + 1] = -gi;
		// dCabs/dRe chi = 4pi k (-Im f |P|^2 - 2 Re(f s)); dCabs/dIm chi = 4pi k (-Re f |P|^2 + 2 Im(f s)), s = sum nu P
		const double fsr = fd.x * nr - fd.y * ni, fsi = fd.x * ni + fd.y * nr;
		gabs[2 * d] = 4 * PI * k * (-fd.y * p2 - 2 * fsr);
		gabs[2 * d + 1] = 4 * PI * k * (-fd.x * p2 + 2 * fsi);
	}
}

} // namespace

// =====================================================================================================================

static int ensure_work(adda_gb300_ctx *c, int R, int hist_cap)
{
	SolverWork *w = c->sw;
	if (!w) {
		w = c->sw = new SolverWork();
		const size_t n3 = 3 * c->N;
		const size_t Rm = c->Rmax;
		w->n3 = n3;
		const size_t vb = sizeof(double2) * Rm * std::max<size_t>(n3, 1);
		ADDA_CUDA(cudaMalloc(&w->x64, vb));
		ADDA_CUDA(cudaMalloc(&w->r64, vb));
		ADDA_CUDA(cudaMalloc(&w->b64, vb));
		ADDA_CUDA(cudaMalloc(&w->av64, vb));
		for (int i = 0; i < 8; i++) ADDA_CUDA(cudaMalloc(&w->kv[i], vb));
		ADDA_CUDA(cudaMalloc(&w->st, sizeof(RhsState) * Rm));
		ADDA_CUDA(cudaMalloc(&w->done, sizeof(int) * Rm));
		ADDA_CUDA(cudaMallocHost(&w->h_done, sizeof(int) * Rm));
		w->nbv = (int)std::max<size_t>(1, std::min<size_t>(152 * 8, (n3 + 4 * NT - 1) / (4 * NT)));
		ADDA_CUDA(cudaMalloc(&w->vpart, sizeof(double) * Rm * w->nbv * 4));
		ADDA_CUDA(cudaMalloc(&w->xpart, sizeof(double) * Rm * w->nbv * 8));
		if (!c->pvec64) ADDA_CUDA(cudaMalloc(&c->pvec64, vb));
		if (c->P > 1) {
			// group contexts: the vectors of a smaller particle are padded to the largest particle's length; the gather
			// writes only real dipoles, so the padding starts at zero and every update keeps it there
			void *bufs[] = {w->x64, w->r64, w->b64, w->av64, w->kv[0], w->kv[1], w->kv[2], w->kv[3], w->kv[4], w->kv[5],
				w->kv[6], w->kv[7], c->pvec64};
			for (void *b : bufs) ADDA_CUDA(cudaMemset(b, 0, vb));
		}
	}
	if (hist_cap > w->hist_cap) {
		if (w->hist) cudaFree(w->hist);
		w->hist = nullptr;
		if (w->gexec) cudaGraphExecDestroy(w->gexec); // the cached graph holds the old pointer
		w->gexec = nullptr;
		ADDA_CUDA(cudaMalloc(&w->hist, sizeof(double) * c->Rmax * hist_cap));
		w->hist_cap = hist_cap;
	}
	if (!w->hist) {
		ADDA_CUDA(cudaMalloc(&w->hist, sizeof(double) * c->Rmax * 1));
		w->hist_cap = 1;
	}
	w->R = R;
	return ADDA_GB300_OK;
}

void solver_free(adda_gb300_ctx *c)
{
	SolverWork *w = c->sw;
	if (!w) return;
	if (w->gexec) cudaGraphExecDestroy(w->gexec);
	void *b[] = {w->x64, w->r64, w->b64, w->av64, w->st, w->done, w->hist, w->vpart, w->xpart};
	for (void *p : b)
		if (p) cudaFree(p);
	for (int i = 0; i < 8; i++)
		if (w->kv[i]) cudaFree(w->kv[i]);
	if (w->h_done) cudaFreeHost(w->h_done);
	delete w;
	c->sw = nullptr;
}

// Krylov vector roles inside kv[] (as typed pointers)
template <typename C> struct KV {
	C *x, *r, *p, *Av, *v1, *v2, *v3, *v4;
};

template <typename C> static KV<C> kvec(SolverWork *w)
{
	KV<C> k;
	k.x = (C *)w->kv[0];
	k.r = (C *)w->kv[1];
	k.p = (C *)w->kv[2];
	k.Av = (C *)w->kv[3];
	k.v1 = (C *)w->kv[4];
	k.v2 = (C *)w->kv[5];
	k.v3 = (C *)w->kv[6];
	k.v4 = (C *)w->kv[7];
	return k;
}

static int matvecs_per_iter(int method)
{
	return (method == ADDA_ITER_BICGSTAB || method == ADDA_ITER_CGNR) ? 2 : (method == ADDA_ITER_BCGS2) ? 4 : 1;
}

// enqueue one Krylov iteration; parity selects the QMR_CS vector roles (v<->v~, p_new<->p_old swap each iteration).
// T = matvec arithmetic, C = complex type of the Krylov vectors.
template <typename T, typename C>
static int enqueue_iter(adda_gb300_ctx *c, SolverWork *w, int method, int R, int parity)
{
	const bool dbl = sizeof(T) == 8;
	KV<C> k = kvec<C>(w);
	const size_t n3 = w->n3;
	const dim3 gv(w->nbv, R);
	const size_t nblk = matvec_partial_blocks(c, dbl);
	cudaStream_t s = c->stream;
	int rc;
	if (method == ADDA_ITER_QMR_CS) {
		C *v = parity ? k.v2 : k.v1, *vt = parity ? k.v1 : k.v2;
		C *pn = parity ? k.v3 : k.p, *po = parity ? k.p : k.v3;
		MvEpi e{EPI_DOT_ARG, nullptr, c->partial};
		if ((rc = matvec_run<T>(c, R, v, k.Av, 0, e, w->done))) return rc;
		qmr_s1<<<R, NT, 0, s>>>(w->st, w->done, c->partial, nblk);
		ADDA_LAUNCHED();
		qmr_v1<C><<<gv, NT, 0, s>>>(w->st, vt, v, k.Av, n3, w->vpart, w->nbv);
		ADDA_LAUNCHED();
		qmr_s2<<<R, NT, 0, s>>>(w->st, w->vpart, w->nbv);
		ADDA_LAUNCHED();
		qmr_v2<C><<<gv, NT, 0, s>>>(w->st, po, pn, v, vt, k.x, k.r, n3, w->vpart, w->nbv);
		ADDA_LAUNCHED();
		s_progress<<<R, NT, 0, s>>>(w->st, w->done, w->vpart, w->nbv, w->hist, w->hist_cap, 0);
		ADDA_LAUNCHED();
	}
	else if (method == ADDA_ITER_BICG_CS) {
		bg_s0<<<R, NT, 0, s>>>(w->st, w->done, w->vpart, w->nbv);
		ADDA_LAUNCHED();
		bg_v1<C><<<gv, NT, 0, s>>>(w->st, k.p, k.r, n3);
		ADDA_LAUNCHED();
		MvEpi e{EPI_DOT_ARG, nullptr, c->partial};
		if ((rc = matvec_run<T>(c, R, k.p, k.Av, 0, e, w->done))) return rc;
		bg_s1<<<R, NT, 0, s>>>(w->st, w->done, c->partial, nblk);
		ADDA_LAUNCHED();
		bg_v2<C><<<gv, NT, 0, s>>>(w->st, k.x, k.p, k.r, k.Av, n3, w->vpart, w->nbv);
		ADDA_LAUNCHED();
		s_progress<<<R, NT, 0, s>>>(w->st, w->done, w->vpart, w->nbv, w->hist, w->hist_cap, 0);
		ADDA_LAUNCHED();
	}
	else if (method == ADDA_ITER_CGNR) {
		MvEpi e1{EPI_NORM, nullptr, c->partial};
		if ((rc = matvec_run<T>(c, R, k.r, k.Av, 1, e1, w->done))) return rc; // A^H r
		cg_s0<<<R, NT, 0, s>>>(w->st, c->partial, nblk);
		ADDA_LAUNCHED();
		cg_v1<C><<<gv, NT, 0, s>>>(w->st, k.p, k.Av, n3);
		ADDA_LAUNCHED();
		MvEpi e2{EPI_NORM, nullptr, c->partial};
		if ((rc = matvec_run<T>(c, R, k.p, k.Av, 0, e2, w->done))) return rc;
		cg_s1<<<R, NT, 0, s>>>(w->st, c->partial, nblk);
		ADDA_LAUNCHED();
		cg_v2<C><<<gv, NT, 0, s>>>(w->st, k.x, k.p, k.r, k.Av, n3, w->vpart, w->nbv);
		ADDA_LAUNCHED();
		s_progress<<<R, NT, 0, s>>>(w->st, w->done, w->vpart, w->nbv, w->hist, w->hist_cap, 0);
		ADDA_LAUNCHED();
	}
	else if (method == ADDA_ITER_BCGS2) {
		C *r0 = k.r, *r1 = k.v1, *r2 = k.v3, *u0 = k.v2, *u1 = k.Av, *u2 = k.v4, *rt = k.p;
		for (int j = 0; j < 2 && !rc; j++) {
			// rho1 of j = 0 comes from the previous b2_vfinal (or the init k_dot), of j = 1 from the r_1 matvec
			if (j == 0) b2_s_beta<<<R, NT, 0, s>>>(w->st, w->done, w->vpart, w->nbv, 0);
			else b2_s_beta<<<R, NT, 0, s>>>(w->st, w->done, c->partial, nblk, 1);
			ADDA_LAUNCHED();
			b2_vu<C><<<gv, NT, 0, s>>>(w->st, u0, r0, u1, r1, n3, j);
			ADDA_LAUNCHED();
			MvEpi eu{EPI_DOT_U_CONJ, rt, c->partial};
			if ((rc = matvec_run<T>(c, R, j ? u1 : u0, j ? u2 : u1, 0, eu, w->done))) return rc;
			b2_s_alpha<<<R, NT, 0, s>>>(w->st, w->done, c->partial, nblk);
			ADDA_LAUNCHED();
			b2_vx<C><<<gv, NT, 0, s>>>(w->st, k.x, u0, r0, u1, r1, u2, n3, j, w->vpart, w->nbv);
			ADDA_LAUNCHED();
			MvEpi er{j ? (int)EPI_NONE : (int)EPI_DOT_U_CONJ, rt, c->partial};
			if ((rc = matvec_run<T>(c, R, j ? r1 : r0, j ? r2 : r1, 0, er, w->done))) return rc;
		}
		b2_gram<C><<<gv, NT, 0, s>>>(w->st, r0, r1, r2, n3, w->xpart, w->nbv);
		ADDA_LAUNCHED();
		b2_s_final<<<R, NT, 0, s>>>(w->st, w->vpart, w->xpart, w->nbv);
		ADDA_LAUNCHED();
		b2_vfinal<C><<<gv, NT, 0, s>>>(w->st, u0, u1, u2, k.x, r0, r1, r2, rt, n3, w->vpart, w->nbv);
		ADDA_LAUNCHED();
		s_progress<<<R, NT, 0, s>>>(w->st, w->done, w->vpart, w->nbv, w->hist, w->hist_cap, 2);
		ADDA_LAUNCHED();
	}
	else if (method == ADDA_ITER_QMR_CS_2) {
		// v in v1, d in v2
		q2_s0<<<R, 32, 0, s>>>(w->st, w->done);
		ADDA_LAUNCHED();
		q2_v1<C><<<gv, NT, 0, s>>>(w->st, k.v1, k.p, n3);
		ADDA_LAUNCHED();
		MvEpi e{EPI_DOT_ARG, nullptr, c->partial};
		if ((rc = matvec_run<T>(c, R, k.p, k.Av, 0, e, w->done))) return rc;
		q2_s1<<<R, NT, 0, s>>>(w->st, w->done, c->partial, nblk);
		ADDA_LAUNCHED();
		q2_v2<C><<<gv, NT, 0, s>>>(w->st, k.v1, k.Av, n3, w->vpart, w->nbv);
		ADDA_LAUNCHED();
		q2_s2<<<R, NT, 0, s>>>(w->st, w->vpart, w->nbv);
		ADDA_LAUNCHED();
		q2_v3<C><<<gv, NT, 0, s>>>(w->st, k.v2, k.p, k.x, k.r, k.v1, n3, w->vpart, w->nbv);
		ADDA_LAUNCHED();
		s_progress<<<R, NT, 0, s>>>(w->st, w->done, w->vpart, w->nbv, w->hist, w->hist_cap, 0);
		ADDA_LAUNCHED();
	}
	else if (method == ADDA_ITER_CSYM) {
		// q_k and p_k swap buffers every iteration (q in r/v1, p in p/v2)
		C *qn = parity ? k.v1 : k.r, *qo = parity ? k.r : k.v1;
		C *pn = parity ? k.v2 : k.p, *po = parity ? k.p : k.v2;
		MvEpi e{EPI_DOT_ARG, nullptr, c->partial};
		if ((rc = matvec_run<T>(c, R, qn, k.Av, 0, e, w->done))) return rc;
		cs_s1<<<R, NT, 0, s>>>(w->st, c->partial, nblk);
		ADDA_LAUNCHED();
		cs_v1<C><<<gv, NT, 0, s>>>(w->st, qo, qn, k.Av, n3, w->vpart, w->nbv);
		ADDA_LAUNCHED();
		cs_s2<<<R, NT, 0, s>>>(w->st, w->done, w->vpart, w->nbv);
		ADDA_LAUNCHED();
		cs_v2<C><<<gv, NT, 0, s>>>(w->st, po, pn, qn, qo, k.x, n3);
		ADDA_LAUNCHED();
		s_progress<<<R, NT, 0, s>>>(w->st, w->done, w->vpart, w->nbv, w->hist, w->hist_cap, 2);
		ADDA_LAUNCHED();
	}
	else {
		C *v = k.v1, *sv = k.v2, *rt = k.v3;
		bs_s0<<<R, NT, 0, s>>>(w->st, w->done, w->vpart, w->nbv);
		ADDA_LAUNCHED();
		bs_v1<C><<<gv, NT, 0, s>>>(w->st, k.p, v, k.r, n3);
		ADDA_LAUNCHED();
		MvEpi e1{EPI_DOT_U_CONJ, rt, c->partial};
		if ((rc = matvec_run<T>(c, R, k.p, v, 0, e1, w->done))) return rc;
		bs_s1<<<R, NT, 0, s>>>(w->st, w->done, c->partial, nblk);
		ADDA_LAUNCHED();
		bs_v2<C><<<gv, NT, 0, s>>>(w->st, sv, v, k.r, n3, w->vpart, w->nbv);
		ADDA_LAUNCHED();
		bs_s2<<<R, NT, 0, s>>>(w->st, w->vpart, w->nbv);
		ADDA_LAUNCHED();
		MvEpi e2{EPI_NORM | EPI_DOT_ARG_CONJ, nullptr, c->partial};
		if ((rc = matvec_run<T>(c, R, sv, k.Av, 0, e2, w->done))) return rc;
		bs_s3<<<R, NT, 0, s>>>(w->st, c->partial, nblk);
		ADDA_LAUNCHED();
		bs_v3<C><<<gv, NT, 0, s>>>(w->st, k.x, k.p, sv, k.Av, k.r, rt, n3, w->vpart, w->nbv);
		ADDA_LAUNCHED();
		s_progress<<<R, NT, 0, s>>>(w->st, w->done, w->vpart, w->nbv, w->hist, w->hist_cap, 1);
		ADDA_LAUNCHED();
	}
	return ADDA_GB300_OK;
}

// Krylov solve of A.x = b on the typed vectors (b given in k.r on entry for zero init, or in bsrc). Runs until all
// RHS are done. Returns via st on the device.
// resume: the method's PHASE_INIT is replaced by a loaded checkpoint (iteration state already in place);
// chp_time > 0: stop once that many seconds have passed since t0 (checked between graph launches), *stopped = true
template <typename T, typename C>
static int krylov(adda_gb300_ctx *c, SolverWork *w, int method, int R, int K, unsigned long long *iters_run,
	bool resume = false, double chp_time = 0, std::chrono::steady_clock::time_point t0 = {}, bool *stopped = nullptr)
{
	// graph key: arithmetic and vector type
	const int mode = (sizeof(T) == 8 ? 0 : 1) + (sizeof(C) == 8 ? 2 : 0) + (std::is_same<C, dd2>::value ? 4 : 0);
	KV<C> k = kvec<C>(w);
	const size_t n3 = w->n3;
	const dim3 gv(w->nbv, R);
	cudaStream_t s = c->stream;
	// method initialisation (PHASE_INIT)
	if (resume) {}
	else if (method == ADDA_ITER_QMR_CS) {
		k_dot<C><<<gv, NT, 0, s>>>(k.r, k.r, n3, 0, w->vpart, w->nbv);
		ADDA_LAUNCHED();
		qmr_s_init<<<R, NT, 0, s>>>(w->st, w->vpart, w->nbv);
		ADDA_LAUNCHED();
		qmr_v_init<C><<<gv, NT, 0, s>>>(w->st, k.v1, k.r, n3);
		ADDA_LAUNCHED();
	}
	else if (method == ADDA_ITER_BICGSTAB) {
		k_copy<C><<<gv, NT, 0, s>>>(k.v3, k.r, n3, nullptr);
		ADDA_LAUNCHED();
		// r.r~* for the first iteration's bs_s0 (slots 1,2)
		k_dot<C><<<gv, NT, 0, s>>>(k.r, k.v3, n3, 1, w->vpart, w->nbv);
		ADDA_LAUNCHED();
	}
	else if (method == ADDA_ITER_BICG_CS) {
		// r.r for the first iteration's bg_s0 (slots 1,2)
		k_dot<C><<<gv, NT, 0, s>>>(k.r, k.r, n3, 0, w->vpart, w->nbv);
		ADDA_LAUNCHED();
	}
	else if (method == ADDA_ITER_BCGS2) {
		// r~0 = r_0 (in p), rho0 = -1; r_0.r~0 for the first b2_s_beta (slots 1,2)
		k_copy<C><<<gv, NT, 0, s>>>(k.p, k.r, n3, nullptr);
		ADDA_LAUNCHED();
		b2_init_s<<<R, 32, 0, s>>>(w->st);
		ADDA_LAUNCHED();
		k_dot<C><<<gv, NT, 0, s>>>(k.r, k.p, n3, 1, w->vpart, w->nbv);
		ADDA_LAUNCHED();
	}
	else if (method == ADDA_ITER_QMR_CS_2) {
		k_copy<C><<<gv, NT, 0, s>>>(k.v1, k.r, n3, nullptr);
		ADDA_LAUNCHED();
		k_dot<C><<<gv, NT, 0, s>>>(k.r, k.r, n3, 0, w->vpart, w->nbv);
		ADDA_LAUNCHED();
		q2_init_s<<<R, NT, 0, s>>>(w->st, w->vpart, w->nbv);
		ADDA_LAUNCHED();
	}
	else if (method == ADDA_ITER_CSYM) {
		// tau_1 = |r_0|, q_1 = r_0(*)/tau_1 in place (r is q_1)
		cs_init_s<<<R, 32, 0, s>>>(w->st);
		ADDA_LAUNCHED();
		cs_conj_scale<C><<<gv, NT, 0, s>>>(w->st, k.r, n3);
		ADDA_LAUNCHED();
	}
	// graph of K iterations (K even keeps the QMR_CS roles periodic)
	if (!w->gexec || w->g_method != method || w->g_dbl != mode || w->g_R != R || w->g_K != K) {
		if (w->gexec) cudaGraphExecDestroy(w->gexec);
		w->gexec = nullptr;
		cudaGraph_t g;
		const unsigned long long before = g_launches.load();
		ADDA_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
		int rc = ADDA_GB300_OK;
		for (int it = 0; it < K && !rc; it++) rc = enqueue_iter<T, C>(c, w, method, R, it & 1);
		cudaGraph_t gtmp = nullptr;
		cudaError_t ec = cudaStreamEndCapture(s, &gtmp);
		if (rc) {
			if (gtmp) cudaGraphDestroy(gtmp);
			return rc;
		}
		if (ec != cudaSuccess) {
			set_error(std::string("graph capture: ") + cudaGetErrorString(ec));
			return ADDA_GB300_ECUDA;
		}
		g = gtmp;
		ADDA_CUDA(cudaGraphInstantiate(&w->gexec, g, 0));
		cudaGraphDestroy(g);
		w->g_nodes = g_launches.load() - before; // kernels per graph launch (counted during capture)
		g_launches.fetch_sub(w->g_nodes);        // capture itself launched nothing
		w->g_method = method;
		w->g_dbl = mode;
		w->g_R = R;
		w->g_K = K;
	}
	unsigned long long n = 0;
	for (;;) {
		ADDA_CUDA(cudaMemcpyAsync(w->h_done, w->done, sizeof(int) * R, cudaMemcpyDeviceToHost, s));
		ADDA_CUDA(cudaStreamSynchronize(s));
		bool all = true;
		for (int r = 0; r < R; r++) all = all && w->h_done[r];
		if (all) break;
		if (chp_time > 0 && n > 0 &&
			std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count() >= chp_time) {
			if (stopped) *stopped = true;
			break;
		}
		ADDA_CUDA(cudaGraphLaunch(w->gexec, s));
		count_launch(w->g_nodes);
		n += K;
	}
	if (iters_run) *iters_run = n;
	return ADDA_GB300_OK;
}

// FP64 residual at which the mixed solver's refinement stops. A solution that only just meets eps carries a
// cross-section error of several times eps/10 (the 128^3 sphere at eps 1e-5: 6e-6 in Cabs, FP64 and the reference
// alike); the measured margins bring mixed solves within 1e-6 of the converged cross sections there: QMR_CS at
// 0.3 eps (2e-7, 5 % more iterations), BiCGStab, whose cross sections converge less regularly, at 0.1 eps (7e-7);
// so do the inner solves with FP32 Krylov vectors (MIXED_F32VEC: at 0.3 eps a 32^3 sphere's QMR_CS solve ended 1.005e-6
// off the converged Cext), which therefore stop at 0.1 eps too.
static double final_eps_of(const adda_gb300_solve_params *sp)
{
	if (sp->final_eps > 0) return std::min(sp->final_eps, sp->eps);
	const bool erratic = sp->method == ADDA_ITER_BICGSTAB || sp->method == ADDA_ITER_BCGS2 ||
		sp->precision == ADDA_PREC_MIXED_F32VEC;
	return (erratic ? 0.1 : 0.3) * sp->eps;
}

// MIXED / MIXED_F32VEC: FP32 matvec (and, for float2, FP32 Krylov vectors) inside FP64 iterative refinement
template <typename C>
static int solve_mixed(adda_gb300_ctx *c, const adda_gb300_solve_params *sp, int R, adda_gb300_rhs_stats *st_out,
	int mc, int K)
{
	SolverWork *w = c->sw;
	const size_t n3 = w->n3;
	cudaStream_t s = c->stream;
	const dim3 gv(w->nbv, R);
	int rc;
	std::vector<RhsState> hs(R);
	{
		KV<C> k = kvec<C>(w);
		const int maxref = sp->max_refine > 0 ? sp->max_refine : 10;
		// outer FP64 bookkeeping per RHS
		std::vector<double> temp(R), inprod64(R, 0.0), epsB64(R);
		std::vector<int> odone(R, 0), iters(R, 0), nmv32(R, 0), nmv64(R, 0), nref(R, 0), status(R, 0);
		// |b|^2 from the k_mult_cc partials
		ADDA_CUDA(cudaMemsetAsync(c->d_red, 0, sizeof(double) * 4 * R, s));
		if ((rc = reduce_partials(c, R, w->vpart, w->nbv, c->d_red))) return rc;
		std::vector<double> red(4 * R);
		ADDA_CUDA(cudaMemcpyAsync(red.data(), c->d_red, sizeof(double) * 4 * R, cudaMemcpyDeviceToHost, s));
		ADDA_CUDA(cudaStreamSynchronize(s));
		// the refinement drives the FP64 residual to final_eps (below eps, for the accuracy of the cross sections);
		// the solve succeeds at eps
		const double target = final_eps_of(sp);
		for (int r = 0; r < R; r++) {
			temp[r] = red[4 * r];
			epsB64[r] = target * target * temp[r];
		}
		// inner right-hand side: b (step 0) in float, kept in k.v3
		k_from64<C><<<(int)std::min<size_t>((R * n3 + NT - 1) / NT, 8192), NT, 0, s>>>(k.v3, w->b64, R * n3);
		ADDA_LAUNCHED();
		double inner_eps0 = sp->inner_eps > 0 ? sp->inner_eps : 0.5 * target;
		int *d_odone = w->done; // reused below as skip flags after the inner solve (copied from host)
		// caller-supplied x_0 (staged in x64): start like a refinement step from r = b - A.x_0 in FP64
		const bool x0mode = sp->init_field == ADDA_IF_X0;
		if (x0mode) {
			MvEpi e{EPI_NONE, nullptr, c->partial};
			if ((rc = matvec_run<double>(c, R, w->x64, w->av64, 0, e, nullptr))) return rc;
			k_resid64<C><<<gv, NT, 0, s>>>(w->b64, w->av64, w->r64, k.v3, n3, w->vpart, w->nbv);
			ADDA_LAUNCHED();
			if ((rc = reduce_partials(c, R, w->vpart, w->nbv, c->d_red))) return rc;
			ADDA_CUDA(cudaMemcpyAsync(red.data(), c->d_red, sizeof(double) * 4 * R, cudaMemcpyDeviceToHost, s));
			ADDA_CUDA(cudaStreamSynchronize(s));
			for (int r = 0; r < R; r++) {
				inprod64[r] = red[4 * r];
				nmv64[r]++;
				if (inprod64[r] <= epsB64[r]) odone[r] = 1;
			}
		}
		for (int step = 0; step <= maxref; step++) {
			const bool refine = step > 0 || x0mode; // the inner solve corrects an FP64 residual
			if (step == 0 && x0mode) {
				bool all = true;
				for (int r = 0; r < R; r++) all = all && odone[r];
				if (all) break;
			}
			// an RHS whose inner solves used up maxiter stops refining (reported as maxiter below)
			if (step > 0) {
				bool all = true;
				for (int r = 0; r < R; r++) {
					if (!odone[r] && iters[r] >= sp->maxiter) odone[r] = 1;
					all = all && odone[r];
				}
				if (all) break;
			}
			// inner solve: A d = rhs (rhs float in k.v3 on entry); init per the user's field mode at step 0
			std::vector<double> eps_in(R);
			for (int r = 0; r < R; r++) {
				if (!refine) eps_in[r] = inner_eps0;
				else {
					const double rho = sqrt(epsB64[r] / std::max(inprod64[r], 1e-300));
					eps_in[r] = std::min(0.5, std::max(0.5 * rho, 2e-6));
				}
			}
			// scalar init with |rhs|^2 (float rhs -> FP64 reduction)
			{
				KV<C> kk = k;
				k_dot<C><<<gv, NT, 0, s>>>(kk.v3, kk.v3, n3, 1, w->vpart, w->nbv);
				ADDA_LAUNCHED();
				// per-RHS eps differs: run s_init per RHS block with its own eps via a small host loop
				for (int r = 0; r < R; r++) {
					// s_init reads partial row r only when launched with gridDim 1 and offset pointer
					const int left = std::max(1, sp->maxiter - iters[r]);
					s_init<<<1, NT, 0, s>>>(w->st + r, w->done + r, w->vpart + (size_t)r * w->nbv * 4, w->nbv,
						eps_in[r], left, mc, w->hist + (size_t)r * w->hist_cap, 0, 1);
					ADDA_LAUNCHED();
				}
			}
			const int zero = refine || sp->init_field == ADDA_IF_ZERO;
			if (zero) {
				ADDA_CUDA(cudaMemsetAsync(k.x, 0, sizeof(C) * R * n3, s));
				k_copy<C><<<gv, NT, 0, s>>>(k.r, k.v3, n3, nullptr);
				ADDA_LAUNCHED();
			}
			else {
				MvEpi e{EPI_NONE, nullptr, c->partial};
				if ((rc = matvec_run<float>(c, R, k.v3, k.Av, 0, e, nullptr))) return rc;
				k_init_field<C><<<gv, NT, 0, s>>>(w->st, w->done, k.v3, k.Av, k.x, k.r, n3, sp->init_field, w->vpart,
					w->nbv, 0);
				ADDA_LAUNCHED();
				s_init_choose<<<R, NT, 0, s>>>(w->st, w->done, w->vpart, w->nbv, sp->init_field, w->hist, 0);
				ADDA_LAUNCHED();
				k_init_field<C><<<gv, NT, 0, s>>>(w->st, w->done, k.v3, k.Av, k.x, k.r, n3, sp->init_field, w->vpart,
					w->nbv, 1);
				ADDA_LAUNCHED();
			}
			// freeze RHS whose FP64 residual already meets eps
			for (int r = 0; r < R; r++) w->h_done[r] = odone[r];
			ADDA_CUDA(cudaMemcpyAsync(w->done, w->h_done, sizeof(int) * R, cudaMemcpyHostToDevice, s));
			// stale done flags from init must be OR-ed: mark st.done too
			ADDA_CUDA(cudaStreamSynchronize(s));
			std::vector<RhsState> tmp(R);
			ADDA_CUDA(cudaMemcpy(tmp.data(), w->st, sizeof(RhsState) * R, cudaMemcpyDeviceToHost));
			for (int r = 0; r < R; r++) {
				if (odone[r]) tmp[r].done = 1;
				w->h_done[r] = tmp[r].done;
			}
			ADDA_CUDA(cudaMemcpy(w->st, tmp.data(), sizeof(RhsState) * R, cudaMemcpyHostToDevice));
			ADDA_CUDA(cudaMemcpy(w->done, w->h_done, sizeof(int) * R, cudaMemcpyHostToDevice));
			unsigned long long it = 0;
			if ((rc = krylov<float, C>(c, w, sp->method, R, K, &it))) return rc;
			ADDA_CUDA(cudaMemcpyAsync(hs.data(), w->st, sizeof(RhsState) * R, cudaMemcpyDeviceToHost, s));
			ADDA_CUDA(cudaStreamSynchronize(s));
			for (int r = 0; r < R; r++) {
				if (odone[r]) continue;
				iters[r] += hs[r].niter - 1;
				nmv32[r] += matvecs_per_iter(sp->method) * (hs[r].niter - 1) + (zero ? 0 : 1);
				if (hs[r].status) status[r] = hs[r].status;
				nref[r]++;
			}
			// x64 (+)= d for the RHS still active
			for (int r = 0; r < R; r++) w->h_done[r] = odone[r];
			ADDA_CUDA(cudaMemcpyAsync(d_odone, w->h_done, sizeof(int) * R, cudaMemcpyHostToDevice, s));
			k_accum<C><<<gv, NT, 0, s>>>(w->x64, k.x, n3, refine ? 1 : 0, d_odone);
			ADDA_LAUNCHED();
			// true residual in FP64: r64 = b - A64.x64, |r64|^2; float copy into k.v3 for the next inner solve. The
			// RHS that had finished before this step keep their x64, so their A64.x64 in av64 is still current: the
			// matvec skips them
			MvEpi e{EPI_NONE, nullptr, c->partial};
			if ((rc = matvec_run<double>(c, R, w->x64, w->av64, 0, e, d_odone))) return rc;
			k_resid64<C><<<gv, NT, 0, s>>>(w->b64, w->av64, w->r64, k.v3, n3, w->vpart, w->nbv);
			ADDA_LAUNCHED();
			if ((rc = reduce_partials(c, R, w->vpart, w->nbv, c->d_red))) return rc;
			ADDA_CUDA(cudaMemcpyAsync(red.data(), c->d_red, sizeof(double) * 4 * R, cudaMemcpyDeviceToHost, s));
			ADDA_CUDA(cudaStreamSynchronize(s));
			bool all = true;
			for (int r = 0; r < R; r++) {
				if (odone[r]) continue;
				nmv64[r]++;
				inprod64[r] = red[4 * r];
				if (inprod64[r] <= epsB64[r] || status[r]) odone[r] = 1;
				all = all && odone[r];
			}
			if (all) break;
		}
		for (int r = 0; r < R; r++) {
			adda_gb300_rhs_stats *st = st_out;
			st[r].niter = iters[r];
			st[r].status = status[r];
			st[r].resid = sqrt(inprod64[r] / temp[r]);
			// maxiter reached on the way to final_eps after the residual met eps: converged
			if (st[r].status == ADDA_GB300_EMAXITER && st[r].resid <= sp->eps) st[r].status = ADDA_GB300_OK;
			if (!st[r].status && !(st[r].resid <= sp->eps)) st[r].status = ADDA_GB300_EMAXITER;
			st[r].refinements = nref[r];
			st[r].matvecs_fp32 = nmv32[r];
			st[r].matvecs_fp64 = nmv64[r];
		}
	}
	return ADDA_GB300_OK;
}

static int check_params(const adda_gb300_solve_params *sp)
{
	if (sp->method < ADDA_ITER_QMR_CS || sp->method > ADDA_ITER_BCGS2 ||
		(sp->precision != ADDA_PREC_FP64 && sp->precision != ADDA_PREC_MIXED &&
			sp->precision != ADDA_PREC_MIXED_F32VEC && sp->precision != ADDA_PREC_MIXED_F64VEC) || !(sp->eps > 0) || sp->maxiter < 0 ||
			(sp->init_field != ADDA_IF_AUTO && sp->init_field != ADDA_IF_ZERO && sp->init_field != ADDA_IF_INC &&
			sp->init_field != ADDA_IF_X0 && sp->init_field != ADDA_IF_CHPOINT) || !(sp->chp_time >= 0) ||
			!(sp->final_eps >= 0)) {
		set_error("solve: unsupported parameters");
		return ADDA_GB300_EINVAL;
	}
	return ADDA_GB300_OK;
}

// ---------------- iteration checkpoints: the reference's chp.<ringid> format (iterative.c:165-278) ----------------

// index of each ADDA_ITER_* method in the reference's params table (iterative.c:118-125, alphabetical) and the
// number of its own vectors
constexpr int kChpInd[7] = {5, 2, 1, 3, 4, 6, 0};
constexpr int kChpVec[7] = {3, 3, 0, 0, 2, 2, 1};
constexpr size_t kChpHead = sizeof(int) + sizeof(size_t) + 2 * sizeof(int) + 3 * sizeof(double);

struct ChpScalar {
	void *p;
	size_t size;
};

// the method's scalars in the order of its PHASE_VARS (iterative.c:383-386,520-521,661-664,741-742,796-803,
// 919-928,1060-1066); the reference's doublecomplex is a double2
static int chp_scalars(RhsState &S, int method, ChpScalar out[8])
{
	int n = 0;
	auto D = [&](double &v) { out[n++] = {&v, sizeof(double)}; };
	auto Z = [&](double2 &v) { out[n++] = {&v, sizeof(double2)}; };
	switch (method) {
		case ADDA_ITER_QMR_CS:
			D(S.om_old); D(S.om_new); D(S.c_old); D(S.c_new); Z(S.beta); Z(S.tautilda); Z(S.s_old); Z(S.s_new);
			break;
		case ADDA_ITER_BICGSTAB: Z(S.ro_old); Z(S.omega); Z(S.balpha); break;
		case ADDA_ITER_BICG_CS: Z(S.ro_old); break;
		case ADDA_ITER_CGNR: D(S.ro_old.x); break;
		case ADDA_ITER_CSYM: D(S.cs_beta); D(S.c_old); D(S.c_new); Z(S.tautilda); Z(S.s_old); Z(S.s_new); break;
		case ADDA_ITER_QMR_CS_2: D(S.q2_c); D(S.q2_theta); D(S.q2_ro); Z(S.q2_eps); Z(S.q2_eta); break;
		default: Z(S.b2_rho0); Z(S.b2_alpha); break;
	}
	return n;
}

// kv[] buffer of each file vector (xvec, rvec, pvec, then the method's own) for the state before iteration niter.
// The reference stores buffers, not roles: QMR_CS and CSYM swap their pointers every iteration and sort them out on
// load by the parity of niter (odd; iterative.c:809-812,935-938). P is the parity of this solver's own buffer roles
// (iterations run since it0); half: BiCGStab stopped at its half step, where the residual is s.
static int chp_buffers(int method, int P, int odd, int half, int idx[6])
{
	enum { X = 0, RV = 1, PV = 2, V1 = 4, V2 = 5, V3 = 6 };
	idx[0] = X;
	idx[1] = RV;
	idx[2] = PV;
	switch (method) {
		case ADDA_ITER_QMR_CS: { // v = vec1, v~ = vec2, p_new = vec3, p_old = pvec for odd niter
			const int v = P ? V2 : V1, vt = P ? V1 : V2, pn = P ? V3 : PV, po = P ? PV : V3;
			idx[2] = odd ? po : pn;
			idx[3] = odd ? v : vt;
			idx[4] = odd ? vt : v;
			idx[5] = odd ? pn : po;
			return 6;
		}
		case ADDA_ITER_BICGSTAB: // v, s, r~
			if (half) idx[1] = V2;
			idx[3] = V1;
			idx[4] = V2;
			idx[5] = V3;
			return 6;
		case ADDA_ITER_CSYM: { // q_new = rvec, q_old = vec1, p_new = vec2, p_old = pvec for odd niter
			const int qn = P ? V1 : RV, qo = P ? RV : V1, pn = P ? V2 : PV, po = P ? PV : V2;
			idx[1] = odd ? qn : qo;
			idx[2] = odd ? po : pn;
			idx[3] = odd ? qo : qn;
			idx[4] = odd ? pn : po;
			return 5;
		}
		case ADDA_ITER_QMR_CS_2: // v, d
			idx[3] = V1;
			idx[4] = V2;
			return 5;
		case ADDA_ITER_BCGS2: // u_0 (r~_0 is pvec)
			idx[3] = V2;
			return 4;
		default: return 3; // BiCG_CS, CGNR: p is pvec
	}
}

static size_t chp_size(int method, size_t n3)
{
	RhsState S;
	ChpScalar sc[8];
	const int ns = chp_scalars(S, method, sc);
	size_t b = kChpHead;
	for (int i = 0; i < ns; i++) b += sc[i].size;
	return b + (3 + kChpVec[method]) * sizeof(double2) * n3;
}

// the solve on device-resident data: d_einc [R][3N] FP64; leaves x in w->x64 and p = S.x in c->pvec64
static int solve_core_impl(adda_gb300_ctx *c, const adda_gb300_solve_params *sp, int R, const double2 *d_einc,
	adda_gb300_rhs_stats *stats);

static int solve_core(adda_gb300_ctx *c, const adda_gb300_solve_params *sp, int R, const double2 *d_einc,
	adda_gb300_rhs_stats *stats)
{
	cudaEvent_t e0, e1;
	ADDA_CUDA(cudaEventCreate(&e0));
	ADDA_CUDA(cudaEventCreate(&e1));
	ADDA_CUDA(cudaEventRecord(e0, c->stream));
	int rc = solve_core_impl(c, sp, R, d_einc, stats);
	if (!rc) {
		cudaEventRecord(e1, c->stream);
		cudaEventSynchronize(e1);
		float ms = 0;
		cudaEventElapsedTime(&ms, e0, e1);
		c->last_solve_ms = ms;
	}
	cudaEventDestroy(e0);
	cudaEventDestroy(e1);
	return rc;
}

static int solve_core_impl(adda_gb300_ctx *c, const adda_gb300_solve_params *sp, int R, const double2 *d_einc,
	adda_gb300_rhs_stats *stats)
{
	SolverWork *w = c->sw;
	int rc;
	const size_t n3 = w->n3;
	cudaStream_t s = c->stream;
	const dim3 gv(w->nbv, R);
	const auto t0 = std::chrono::steady_clock::now();
	const bool resume = sp->init_field == ADDA_IF_CHPOINT;
	w->chp_valid = 0;
	if (resume) {
		if (sp->precision != ADDA_PREC_FP64) {
			set_error("solve: resuming from a checkpoint needs ADDA_PREC_FP64");
			return ADDA_GB300_EINVAL;
		}
		for (int r = 0; r < R; r++) {
			if ((int)w->chp_pend.size() <= r || w->chp_pend[r].empty()) {
				set_error("solve: no checkpoint loaded for right-hand side " + std::to_string(r));
				return ADDA_GB300_ESTATE;
			}
			int ind;
			std::memcpy(&ind, w->chp_pend[r].data(), sizeof(int));
			if (ind != kChpInd[sp->method] || w->chp_pend[r].size() != chp_size(sp->method, n3)) {
				set_error("solve: the checkpoint is for different iterative method"); // iterative.c:239
				return ADDA_GB300_EINVAL;
			}
		}
	}
	// stagnation limits per method (iterative.c:118-125)
	const int mc = (sp->method == ADDA_ITER_BICGSTAB) ? 30000
		: (sp->method == ADDA_ITER_CGNR || sp->method == ADDA_ITER_CSYM) ? 10
		: (sp->method == ADDA_ITER_BCGS2) ? 15000 : 50000;
	int K = sp->check_every > 0 ? sp->check_every : 8;
	if (K % 2) K++;
	std::vector<adda_gb300_rhs_stats> st(R);
	for (auto &x : st) memset(&x, 0, sizeof(x));
	std::vector<RhsState> hs(R);
	// b = S.Einc in FP64
	k_mult_cc<<<gv, NT, 0, s>>>(d_einc, w->b64, c->ccs64, c->per_dip, c->nmat, c->d_mat, c->N, w->vpart, w->nbv, c->rpp,
		c->lat_stride);
	ADDA_LAUNCHED();
	ADDA_CUDA(cudaMemsetAsync(w->hist, 0, sizeof(double) * R * w->hist_cap, s));
	for (int i = 0; i < 8; i++) ADDA_CUDA(cudaMemsetAsync(w->kv[i], 0, sizeof(double2) * R * n3, s));
	if (sp->precision == ADDA_PREC_FP64) {
		typedef double2 C;
		KV<C> k = kvec<C>(w);
		const int zero = sp->init_field == ADDA_IF_ZERO;
		if (!resume) {
			s_init<<<R, NT, 0, s>>>(w->st, w->done, w->vpart, w->nbv, sp->eps, sp->maxiter, mc, w->hist, w->hist_cap,
				zero);
			ADDA_LAUNCHED();
		}
		if (resume) { // LoadIterChpoint (iterative.c:222-278) in place of CalcInitField and PHASE_INIT
			std::vector<int> dn(R);
			std::vector<double> h0(R);
			for (int r = 0; r < R; r++) {
				const unsigned char *q = w->chp_pend[r].data() + sizeof(int) + sizeof(size_t);
				RhsState &S = hs[r];
				std::memset(&S, 0, sizeof(S));
				std::memcpy(&S.niter, q, sizeof(int));
				std::memcpy(&S.counter, q + 4, sizeof(int));
				std::memcpy(&S.inprodR, q + 8, sizeof(double));
				std::memcpy(&S.prev_err, q + 16, sizeof(double));
				std::memcpy(&S.resid_scale, q + 24, sizeof(double));
				q += 32;
				ChpScalar sc[8];
				const int ns = chp_scalars(S, sp->method, sc);
				for (int i = 0; i < ns; i++) {
					std::memcpy(sc[i].p, q, sc[i].size);
					q += sc[i].size;
				}
				S.epsB = sp->eps * sp->eps / S.resid_scale; // iterative.c:270
				S.temp = 1 / S.resid_scale;
				S.inprodRp1 = S.prev_err * S.prev_err / S.resid_scale;
				S.maxiter = sp->maxiter;
				S.mc = mc;
				S.it0 = S.niter;
				S.full = sp->full_steps != 0;
				S.done = !(S.inprodR > S.epsB && S.niter <= S.maxiter && S.counter <= S.mc);
				dn[r] = S.done;
				h0[r] = S.prev_err;
				int idx[6];
				const int nv = chp_buffers(sp->method, 0, S.niter & 1, 0, idx);
				for (int v = 0; v < nv; v++, q += sizeof(double2) * n3)
					ADDA_CUDA(cudaMemcpyAsync(w->kv[idx[v]] + (size_t)r * n3, q, sizeof(double2) * n3,
						cudaMemcpyHostToDevice, s));
				if (S.niter - 1 < w->hist_cap)
					ADDA_CUDA(cudaMemcpyAsync(w->hist + (size_t)r * w->hist_cap + S.niter - 1, &h0[r], sizeof(double),
						cudaMemcpyHostToDevice, s));
			}
			ADDA_CUDA(cudaMemcpyAsync(w->st, hs.data(), sizeof(RhsState) * R, cudaMemcpyHostToDevice, s));
			ADDA_CUDA(cudaMemcpyAsync(w->done, dn.data(), sizeof(int) * R, cudaMemcpyHostToDevice, s));
			ADDA_CUDA(cudaStreamSynchronize(s));
			for (int r = 0; r < R; r++) w->chp_pend[r].clear(); // a checkpoint is loaded once
			// dot products the first resumed iteration takes from the previous one's fused update
			if (sp->method == ADDA_ITER_BICGSTAB) k_dot<C><<<gv, NT, 0, s>>>(k.r, k.v3, n3, 1, w->vpart, w->nbv);
			else if (sp->method == ADDA_ITER_BICG_CS) k_dot<C><<<gv, NT, 0, s>>>(k.r, k.r, n3, 0, w->vpart, w->nbv);
			else if (sp->method == ADDA_ITER_BCGS2) k_dot<C><<<gv, NT, 0, s>>>(k.r, k.p, n3, 1, w->vpart, w->nbv);
			else if (sp->method == ADDA_ITER_QMR_CS_2) {
				k_dot<C><<<gv, NT, 0, s>>>(k.v1, k.v1, n3, 0, w->vpart, w->nbv);
				ADDA_LAUNCHED();
				q2_resume_s<<<R, NT, 0, s>>>(w->st, w->vpart, w->nbv);
			}
			ADDA_LAUNCHED();
		}
		else if (zero) {
			k_copy<C><<<gv, NT, 0, s>>>(k.r, w->b64, n3, nullptr);
			ADDA_LAUNCHED();
		}
		else if (sp->init_field == ADDA_IF_X0) {
			// x_0 from the caller (staged in x64): r_0 = b - A.x_0 (InitFieldfromE, iterative.c:1335-1337)
			k_copy<C><<<gv, NT, 0, s>>>(k.x, w->x64, n3, nullptr);
			ADDA_LAUNCHED();
			MvEpi e{EPI_NONE, nullptr, c->partial};
			if ((rc = matvec_run<double>(c, R, k.x, k.Av, 0, e, nullptr))) return rc;
			k_init_field<C><<<gv, NT, 0, s>>>(w->st, w->done, w->b64, k.Av, k.x, k.r, n3, sp->init_field, w->vpart,
				w->nbv, 0);
			ADDA_LAUNCHED();
			s_init_choose<<<R, NT, 0, s>>>(w->st, w->done, w->vpart, w->nbv, sp->init_field, w->hist, w->hist_cap);
			ADDA_LAUNCHED();
		}
		else {
			MvEpi e{EPI_NONE, nullptr, c->partial};
			if ((rc = matvec_run<double>(c, R, w->b64, k.Av, 0, e, nullptr))) return rc;
			k_init_field<C><<<gv, NT, 0, s>>>(w->st, w->done, w->b64, k.Av, k.x, k.r, n3, sp->init_field, w->vpart,
				w->nbv, 0);
			ADDA_LAUNCHED();
			s_init_choose<<<R, NT, 0, s>>>(w->st, w->done, w->vpart, w->nbv, sp->init_field, w->hist, w->hist_cap);
			ADDA_LAUNCHED();
			k_init_field<C><<<gv, NT, 0, s>>>(w->st, w->done, w->b64, k.Av, k.x, k.r, n3, sp->init_field, w->vpart,
				w->nbv, 1);
			ADDA_LAUNCHED();
		}
		unsigned long long iters = 0;
		bool stopped = false;
		if (!resume && sp->full_steps) { // BiCGStab without the half-step exit (-chp_type always)
			std::vector<RhsState> h(R);
			ADDA_CUDA(cudaMemcpyAsync(h.data(), w->st, sizeof(RhsState) * R, cudaMemcpyDeviceToHost, s));
			ADDA_CUDA(cudaStreamSynchronize(s));
			for (auto &x : h) x.full = 1;
			ADDA_CUDA(cudaMemcpyAsync(w->st, h.data(), sizeof(RhsState) * R, cudaMemcpyHostToDevice, s));
			ADDA_CUDA(cudaStreamSynchronize(s));
		}
		if ((rc = krylov<double, double2>(c, w, sp->method, R, K, &iters, resume, sp->chp_time, t0, &stopped)))
			return rc;
		ADDA_CUDA(cudaMemcpyAsync(hs.data(), w->st, sizeof(RhsState) * R, cudaMemcpyDeviceToHost, s));
		ADDA_CUDA(cudaStreamSynchronize(s));
		ADDA_CUDA(cudaMemcpyAsync(w->x64, k.x, sizeof(double2) * R * n3, cudaMemcpyDeviceToDevice, s));
		for (int r = 0; r < R; r++) {
			st[r].niter = hs[r].niter - 1;
			st[r].status = hs[r].status;
			if (!st[r].status && stopped && !hs[r].done) st[r].status = ADDA_GB300_CHPOINT;
			else if (!st[r].status && hs[r].inprodR > hs[r].epsB)
				st[r].status = (hs[r].niter > hs[r].maxiter) ? ADDA_GB300_EMAXITER : ADDA_GB300_ESTAGNATION;
			st[r].resid = sqrt(hs[r].resid_scale * hs[r].inprodR);
			const int mpi = matvecs_per_iter(sp->method);
			st[r].matvecs_fp64 = (zero || resume ? 0 : 1) + mpi * (hs[r].niter - hs[r].it0);
		}
		w->chp_valid = 1;
		w->chp_method = sp->method;
		w->chp_R = R;
	}
	else if (sp->precision == ADDA_PREC_MIXED) {
		if ((rc = solve_mixed<dd2>(c, sp, R, st.data(), mc, K))) return rc;
	}
	else if (sp->precision == ADDA_PREC_MIXED_F64VEC) {
		if ((rc = solve_mixed<double2>(c, sp, R, st.data(), mc, K))) return rc;
	}
	else {
		if ((rc = solve_mixed<float2>(c, sp, R, st.data(), mc, K))) return rc;
	}
	// polarisations p = S.x (FP64) stay on the device (iterative.c:1527)
	k_pvec<<<gv, NT, 0, s>>>(w->x64, c->pvec64, c->ccs64, c->per_dip, c->nmat, c->d_mat, c->N, c->rpp, c->lat_stride);
	ADDA_LAUNCHED();
	c->last_nrhs = R;
	if (stats)
		for (int r = 0; r < R; r++) stats[r] = st[r];
	return ADDA_GB300_OK;
}

size_t solver_chpoint_size(const adda_gb300_ctx *c, int method)
{
	if (method < ADDA_ITER_QMR_CS || method > ADDA_ITER_BCGS2) return 0;
	return chp_size(method, 3 * c->N);
}

// SaveIterChpoint (iterative.c:165-218) for one right-hand side of the last FP64 solve
int solver_chpoint_save(adda_gb300_ctx *c, int rhs, void *buf, size_t size)
{
	SolverWork *w = c->sw;
	if (!w || !w->chp_valid || rhs < 0 || rhs >= w->chp_R) {
		set_error("chpoint_save: no FP64 solver state for that right-hand side");
		return ADDA_GB300_ESTATE;
	}
	const int m = w->chp_method;
	const size_t n3 = w->n3, need = chp_size(m, n3);
	if (!buf || size < need) {
		set_error("chpoint_save: buffer smaller than adda_gb300_chpoint_size");
		return ADDA_GB300_EINVAL;
	}
	cudaStream_t s = c->stream;
	RhsState S;
	ADDA_CUDA(cudaMemcpyAsync(&S, w->st + rhs, sizeof(S), cudaMemcpyDeviceToHost, s));
	ADDA_CUDA(cudaStreamSynchronize(s));
	if (S.status == ADDA_GB300_EBREAKDOWN) {
		set_error("chpoint_save: the solve of that right-hand side broke down");
		return ADDA_GB300_ESTATE;
	}
	unsigned char *o = (unsigned char *)buf;
	const int ind = kChpInd[m];
	const size_t rows = n3;
	auto put = [&](const void *p, size_t n) {
		std::memcpy(o, p, n);
		o += n;
	};
	put(&ind, sizeof(int));
	put(&rows, sizeof(size_t));
	put(&S.niter, sizeof(int));
	put(&S.counter, sizeof(int));
	put(&S.inprodR, sizeof(double));
	put(&S.prev_err, sizeof(double));
	put(&S.resid_scale, sizeof(double));
	ChpScalar sc[8];
	const int ns = chp_scalars(S, m, sc);
	for (int i = 0; i < ns; i++) put(sc[i].p, sc[i].size);
	int idx[6];
	const int nv = chp_buffers(m, (S.niter - S.it0) & 1, S.niter & 1, m == ADDA_ITER_BICGSTAB && S.half, idx);
	for (int v = 0; v < nv; v++, o += sizeof(double2) * n3)
		ADDA_CUDA(cudaMemcpyAsync(o, w->kv[idx[v]] + (size_t)rhs * n3, sizeof(double2) * n3, cudaMemcpyDeviceToHost, s));
	ADDA_CUDA(cudaStreamSynchronize(s));
	return ADDA_GB300_OK;
}

// LoadIterChpoint's checks (iterative.c:238-266); the state is applied by the next solve with ADDA_IF_CHPOINT
int solver_chpoint_load(adda_gb300_ctx *c, int rhs, const void *buf, size_t size)
{
	if (rhs < 0 || rhs >= c->Rmax || !buf || size < kChpHead) {
		set_error("chpoint_load: invalid arguments");
		return ADDA_GB300_EINVAL;
	}
	int rc = ensure_work(c, 1, 1);
	if (rc) return rc;
	SolverWork *w = c->sw;
	int ind;
	size_t rows;
	std::memcpy(&ind, buf, sizeof(int));
	std::memcpy(&rows, (const unsigned char *)buf + sizeof(int), sizeof(size_t));
	int m = -1;
	for (int i = 0; i < 7; i++)
		if (kChpInd[i] == ind) m = i;
	if (m < 0) {
		set_error("chpoint_load: unknown iterative method index in the checkpoint");
		return ADDA_GB300_EINVAL;
	}
	if (rows != w->n3) {
		set_error("chpoint_load: the checkpoint is for different vector size");
		return ADDA_GB300_EINVAL;
	}
	const size_t need = chp_size(m, w->n3);
	if (size != need) {
		set_error(size < need ? "chpoint_load: failed reading the checkpoint (too short)"
		                      : "chpoint_load: the checkpoint is too long");
		return ADDA_GB300_EINVAL;
	}
	if ((int)w->chp_pend.size() < c->Rmax) w->chp_pend.resize(c->Rmax);
	w->chp_pend[rhs].assign((const unsigned char *)buf, (const unsigned char *)buf + size);
	return ADDA_GB300_OK;
}

int solver_solve(adda_gb300_ctx *c, const adda_gb300_solve_params *sp, int R, const double *einc, double *xvec,
	double *pvec, adda_gb300_rhs_stats *stats, double *resid_hist, int hist_cap)
{
	int rc = check_params(sp);
	if (rc) return rc;
	if ((rc = ensure_work(c, R, std::max(hist_cap, 1)))) return rc;
	SolverWork *w = c->sw;
	const size_t n3 = w->n3;
	cudaStream_t s = c->stream;
	// stage Einc in the FP64 matvec output buffer (consumed by the first kernel of the solve)
	ADDA_CUDA(cudaMemcpyAsync(w->av64, einc, sizeof(double2) * R * n3, cudaMemcpyHostToDevice, s));
	if (sp->init_field == ADDA_IF_X0) {
		if (!xvec) {
			set_error("solve: init_field X0 needs x_0 in xvec");
			return ADDA_GB300_EINVAL;
		}
		ADDA_CUDA(cudaMemcpyAsync(w->x64, xvec, sizeof(double2) * R * n3, cudaMemcpyHostToDevice, s));
	}
	if ((rc = solve_core(c, sp, R, w->av64, stats))) return rc;
	if (xvec) ADDA_CUDA(cudaMemcpyAsync(xvec, w->x64, sizeof(double2) * R * n3, cudaMemcpyDeviceToHost, s));
	if (pvec) ADDA_CUDA(cudaMemcpyAsync(pvec, c->pvec64, sizeof(double2) * R * n3, cudaMemcpyDeviceToHost, s));
	if (resid_hist && hist_cap > 0) {
		if (sp->precision == ADDA_PREC_FP64)
			ADDA_CUDA(cudaMemcpy2DAsync(resid_hist, sizeof(double) * hist_cap, w->hist, sizeof(double) * w->hist_cap,
				sizeof(double) * hist_cap, R, cudaMemcpyDeviceToHost, s));
		else memset(resid_hist, 0, sizeof(double) * R * hist_cap);
	}
	ADDA_CUDA(cudaStreamSynchronize(s));
	return ADDA_GB300_OK;
}

int solver_solve_dev(adda_gb300_ctx *c, const adda_gb300_solve_params *sp, int R, const double2 *d_einc,
	double2 *d_xvec, double2 *d_pvec, adda_gb300_rhs_stats *stats)
{
	int rc = check_params(sp);
	if (rc) return rc;
	if ((rc = ensure_work(c, R, 1))) return rc;
	SolverWork *w = c->sw;
	const size_t n3 = w->n3;
	cudaStream_t s = c->stream;
	if (sp->init_field == ADDA_IF_X0) {
		if (!d_xvec) {
			set_error("solve_device: init_field X0 needs x_0 in d_xvec");
			return ADDA_GB300_EINVAL;
		}
		ADDA_CUDA(cudaMemcpyAsync(w->x64, d_xvec, sizeof(double2) * R * n3, cudaMemcpyDeviceToDevice, s));
	}
	if ((rc = solve_core(c, sp, R, d_einc, stats))) return rc;
	if (d_xvec) ADDA_CUDA(cudaMemcpyAsync(d_xvec, w->x64, sizeof(double2) * R * n3, cudaMemcpyDeviceToDevice, s));
	if (d_pvec) ADDA_CUDA(cudaMemcpyAsync(d_pvec, c->pvec64, sizeof(double2) * R * n3, cudaMemcpyDeviceToDevice, s));
	ADDA_CUDA(cudaStreamSynchronize(s));
	return ADDA_GB300_OK;
}

int vjp_chi(adda_gb300_ctx *c, const adda_gb300_solve_params *sp, int rhs, const double prop[3], const double incpol[3],
	const double *dinv_alpha, double *grad_cext, double *grad_cabs)
{
	int rc = check_params(sp);
	if (rc) return rc;
	if (c->Rmax < 2 || !c->pvec64 || rhs < 0 || rhs >= c->last_nrhs) {
		set_error("vjp_chi: needs nrhs_max >= 2 and a previous solve covering the requested RHS");
		return ADDA_GB300_ESTATE;
	}
	if ((rc = ensure_work(c, 2, 1))) return rc;
	SolverWork *w = c->sw;
	const size_t n3 = w->n3, N = c->N;
	cudaStream_t s = c->stream;
	const int last = c->last_nrhs;
	const size_t per = c->per_dip ? 3 * N : (size_t)c->nmat * 3;
	// keep the forward polarisations and the cc of slots 0,1; slots 0,1 get the forward RHS's cc
	double2 *save_p = nullptr, *save_cc = nullptr, *dF = nullptr;
	double *dg = nullptr;
	float2 *save_cc32 = nullptr;
	ADDA_CUDA(cudaMalloc(&save_p, sizeof(double2) * n3 * last));
	ADDA_CUDA(cudaMalloc(&save_cc, sizeof(double2) * per * 4));
	ADDA_CUDA(cudaMalloc(&save_cc32, sizeof(float2) * per * 2));
	ADDA_CUDA(cudaMalloc(&dF, sizeof(double2) * N));
	ADDA_CUDA(cudaMalloc(&dg, sizeof(double) * 4 * N));
	ADDA_CUDA(cudaMemcpyAsync(save_p, c->pvec64, sizeof(double2) * n3 * last, cudaMemcpyDeviceToDevice, s));
	ADDA_CUDA(cudaMemcpyAsync(save_cc, c->cc64, sizeof(double2) * per * 2, cudaMemcpyDeviceToDevice, s));
	ADDA_CUDA(cudaMemcpyAsync(save_cc + 2 * per, c->ccs64, sizeof(double2) * per * 2, cudaMemcpyDeviceToDevice, s));
	ADDA_CUDA(cudaMemcpyAsync(save_cc32, c->ccs32, sizeof(float2) * per * 2, cudaMemcpyDeviceToDevice, s));
	const std::vector<int> cc_set_saved = c->cc_set;
	for (int slot = 0; slot < 2; slot++)
		if (slot != rhs) {
			ADDA_CUDA(cudaMemcpyAsync(c->cc64 + per * slot, c->cc64 + per * rhs, sizeof(double2) * per,
				cudaMemcpyDeviceToDevice, s));
			ADDA_CUDA(cudaMemcpyAsync(c->ccs64 + per * slot, c->ccs64 + per * rhs, sizeof(double2) * per,
				cudaMemcpyDeviceToDevice, s));
			ADDA_CUDA(cudaMemcpyAsync(c->ccs32 + per * slot, c->ccs32 + per * rhs, sizeof(float2) * per,
				cudaMemcpyDeviceToDevice, s));
		}
	c->cc_set[0] = c->cc_set[1] = 1;
	// adjoint right-hand sides into the staging buffer of the solve
	const double kd = c->k * c->gridspace;
	const double r0[3] = {-c->gridspace * (c->bX - 1) / 2.0, -c->gridspace * (c->bY - 1) / 2.0,
		-c->gridspace * (c->bZ - 1) / 2.0};
	const double ph0 = -c->k * (r0[0] * prop[0] + r0[1] * prop[1] + r0[2] * prop[2]);
	const double2 *ccr = c->cc64 + per * rhs;
	const int gN = (int)std::max<size_t>(1, std::min<size_t>((N + NT - 1) / NT, 152 * 16));
	const size_t lq = (size_t)(rhs / c->rpp) * c->lat_stride; // the RHS's particle (group contexts)
	k_adj_rhs<<<gN, NT, 0, s>>>(w->av64, save_p + n3 * rhs, c->d_pos + 3 * lq, ccr, c->per_dip, c->nmat, c->d_mat + lq, N,
		prop[0],
		prop[1], prop[2], incpol[0], incpol[1], incpol[2], kd, c->k, ph0);
	ADDA_LAUNCHED();
	adda_gb300_rhs_stats st[2];
	adda_gb300_solve_params asp = *sp;
	// no caller x_0, no checkpoint and no time limit for the adjoint systems
	if (asp.init_field == ADDA_IF_X0 || asp.init_field == ADDA_IF_CHPOINT) asp.init_field = ADDA_IF_AUTO;
	asp.chp_time = 0;
	rc = solve_core(c, &asp, 2, w->av64, st);
	if (!rc) {
		ADDA_CUDA(cudaMemcpyAsync(dF, dinv_alpha, sizeof(double2) * N, cudaMemcpyHostToDevice, s));
		k_vjp_grad<<<gN, NT, 0, s>>>(save_p + n3 * rhs, c->pvec64, c->pvec64 + n3, dF, N, c->k, dg, dg + 2 * N);
		ADDA_LAUNCHED();
		ADDA_CUDA(cudaMemcpyAsync(grad_cext, dg, sizeof(double) * 2 * N, cudaMemcpyDeviceToHost, s));
		ADDA_CUDA(cudaMemcpyAsync(grad_cabs, dg + 2 * N, sizeof(double) * 2 * N, cudaMemcpyDeviceToHost, s));
		for (int r = 0; r < 2; r++)
			if (st[r].status) {
				set_error("vjp_chi: the adjoint solve did not converge");
				rc = st[r].status;
			}
	}
	// restore the forward state
	ADDA_CUDA(cudaMemcpyAsync(c->pvec64, save_p, sizeof(double2) * n3 * last, cudaMemcpyDeviceToDevice, s));
	ADDA_CUDA(cudaMemcpyAsync(c->cc64, save_cc, sizeof(double2) * per * 2, cudaMemcpyDeviceToDevice, s));
	ADDA_CUDA(cudaMemcpyAsync(c->ccs64, save_cc + 2 * per, sizeof(double2) * per * 2, cudaMemcpyDeviceToDevice, s));
	ADDA_CUDA(cudaMemcpyAsync(c->ccs32, save_cc32, sizeof(float2) * per * 2, cudaMemcpyDeviceToDevice, s));
	ADDA_CUDA(cudaStreamSynchronize(s));
	c->cc_set = cc_set_saved;
	c->last_nrhs = last;
	cudaFree(save_p);
	cudaFree(save_cc);
	cudaFree(save_cc32);
	cudaFree(dF);
	cudaFree(dg);
	return rc;
}

int scattered_fields(adda_gb300_ctx *c, int R, int ndir, const double *dirs, double *ebuff)
{
	constexpr int kMaxDir = 32768; // directions per launch (grid y extent)
	if (ndir > kMaxDir) {
		std::vector<double> part((size_t)R * kMaxDir * 6);
		for (int d0 = 0; d0 < ndir; d0 += kMaxDir) {
			const int nd = std::min(kMaxDir, ndir - d0);
			int rc = scattered_fields(c, R, nd, dirs + 3 * (size_t)d0, part.data());
			if (rc) return rc;
			for (int r = 0; r < R; r++)
				std::memcpy(ebuff + ((size_t)r * ndir + d0) * 6, part.data() + (size_t)r * nd * 6,
					sizeof(double) * 6 * nd);
		}
		return ADDA_GB300_OK;
	}
	const size_t N = c->N;
	cudaStream_t s = c->stream;
	// blocks per (direction, RHS): at least 8 dipoles a thread, at most 128 blocks
	const int nb = (int)std::max<size_t>(1, std::min<size_t>(128, (N + 8 * NT - 1) / (8 * NT)));
	double *d_dirs = nullptr, *d_part = nullptr;
	double2 *d_out = nullptr;
	ADDA_CUDA(cudaMalloc(&d_dirs, sizeof(double) * 3 * ndir));
	ADDA_CUDA(cudaMalloc(&d_part, sizeof(double) * 6 * (size_t)nb * ndir * R));
	ADDA_CUDA(cudaMalloc(&d_out, sizeof(double2) * 3 * (size_t)ndir * R));
	int rc = ADDA_GB300_OK;
	if (cudaMemcpyAsync(d_dirs, dirs, sizeof(double) * 3 * ndir, cudaMemcpyHostToDevice, s) != cudaSuccess)
		rc = ADDA_GB300_ECUDA;
	if (!rc && N) {
		k_field<<<dim3(nb, ndir, R), NT, 0, s>>>(c->pvec64, c->d_pos, N, d_dirs, c->k * c->gridspace, d_part, c->rpp,
			c->lat_stride);
		if (cudaGetLastError() != cudaSuccess) rc = ADDA_GB300_ECUDA;
		else count_launch();
	}
	if (!rc) {
		if (!N) cudaMemsetAsync(d_part, 0, sizeof(double) * 6 * (size_t)nb * ndir * R, s);
		k_field_fin<<<(ndir * R + 127) / 128, 128, 0, s>>>(d_part, nb, ndir, R, d_dirs, c->k, c->gridspace, c->bX,
			c->bY, c->bZ, d_out);
		if (cudaGetLastError() != cudaSuccess) rc = ADDA_GB300_ECUDA;
		else count_launch();
	}
	if (!rc && (cudaMemcpyAsync(ebuff, d_out, sizeof(double2) * 3 * (size_t)ndir * R, cudaMemcpyDeviceToHost, s) !=
					cudaSuccess ||
				   cudaStreamSynchronize(s) != cudaSuccess))
		rc = ADDA_GB300_ECUDA;
	if (rc) set_error(std::string("scattered_fields: ") + cudaGetErrorString(cudaGetLastError()));
	cudaFree(d_dirs);
	cudaFree(d_part);
	cudaFree(d_out);
	return rc;
}

int cross_sections(adda_gb300_ctx *c, int R, const double *prop, const double *incpol, double *cext, double *cabs)
{
	int rc = ensure_work(c, R, 1);
	if (rc) return rc;
	SolverWork *w = c->sw;
	cudaStream_t s = c->stream;
	double *d_prop = c->d_red; // needs 3*R doubles: use the reduction scratch if large enough, else allocate
	double *tmp = nullptr;
	if ((size_t)3 * R > 4 * (size_t)c->Rmax) {
		ADDA_CUDA(cudaMalloc(&tmp, sizeof(double) * 3 * R));
		d_prop = tmp;
	}
	ADDA_CUDA(cudaMemcpyAsync(d_prop, prop, sizeof(double) * 3 * R, cudaMemcpyHostToDevice, s));
	const dim3 g(w->nbv, R);
	const double kd = c->k * c->gridspace, k3 = c->k * c->k * c->k;
	k_cross<<<g, NT, 0, s>>>(c->pvec64, c->d_pos, c->cc64, c->per_dip, c->nmat, c->d_mat, c->N, d_prop, kd, k3,
		w->xpart, w->nbv, c->rpp, c->lat_stride);
	ADDA_LAUNCHED();
	std::vector<double> part((size_t)R * w->nbv * 8);
	ADDA_CUDA(cudaMemcpyAsync(part.data(), w->xpart, sizeof(double) * part.size(), cudaMemcpyDeviceToHost, s));
	ADDA_CUDA(cudaStreamSynchronize(s));
	if (tmp) cudaFree(tmp);
	const double PI = 3.14159265358979323846;
	for (int r = 0; r < R; r++) {
		double sm[7] = {0, 0, 0, 0, 0, 0, 0};
		for (int b = 0; b < w->nbv; b++)
			for (int j = 0; j < 7; j++) sm[j] += part[((size_t)r * w->nbv + b) * 8 + j];
		const double *n = prop + 3 * r, *e = incpol + 3 * r;
		// tbuff = sum - n (n.sum); ebuff = -i k^3 exp(-i k r0.n) tbuff; Cext = 4pi/k^2 Re(ebuff.e)
		double dre = 0, dim = 0;
		for (int i = 0; i < 3; i++) {
			dre += sm[2 * i] * n[i];
			dim += sm[2 * i + 1] * n[i];
		}
		const double r0[3] = {-c->gridspace * (c->bX - 1) / 2.0, -c->gridspace * (c->bY - 1) / 2.0,
			-c->gridspace * (c->bZ - 1) / 2.0};
		const double ph0 = -c->k * (r0[0] * n[0] + r0[1] * n[1] + r0[2] * n[2]);
		const double k3v = c->k * c->k * c->k;
		// amp = -i * exp(i ph0) * k^3 = k^3 (sin ph0 - i cos ph0)
		const double ar = k3v * sin(ph0), ai = -k3v * cos(ph0);
		double sumc = 0;
		for (int i = 0; i < 3; i++) {
			const double tr = sm[2 * i] - dre * n[i], ti = sm[2 * i + 1] - dim * n[i];
			sumc += (ar * tr - ai * ti) * e[i];
		}
		if (cext) cext[r] = sumc * 4 * PI / (c->k * c->k);
		if (cabs) cabs[r] = 4 * PI * c->k * sm[6];
	}
	return ADDA_GB300_OK;
}

int cross_sections_beam(adda_gb300_ctx *c, int R, const double *einc, double inc_scale, double *cext, double *cabs)
{
	int rc = ensure_work(c, R, 1);
	if (rc) return rc;
	SolverWork *w = c->sw;
	cudaStream_t s = c->stream;
	double2 *d_e = nullptr;
	const size_t n = (size_t)R * c->N * 3;
	ADDA_CUDA(cudaMalloc(&d_e, sizeof(double2) * std::max<size_t>(n, 1)));
	cudaError_t e = cudaMemcpyAsync(d_e, einc, sizeof(double2) * n, cudaMemcpyHostToDevice, s);
	std::vector<double> part((size_t)R * w->nbv * 8);
	if (e == cudaSuccess) {
		const dim3 g(w->nbv, R);
		k_cross_beam<<<g, NT, 0, s>>>(c->pvec64, d_e, c->cc64, c->per_dip, c->nmat, c->d_mat, c->N,
			c->k * c->k * c->k, w->xpart, w->nbv, c->rpp, c->lat_stride);
		count_launch();
		e = cudaGetLastError();
	}
	if (e == cudaSuccess) e = cudaMemcpyAsync(part.data(), w->xpart, sizeof(double) * part.size(),
		cudaMemcpyDeviceToHost, s);
	if (e == cudaSuccess) e = cudaStreamSynchronize(s);
	cudaFree(d_e);
	if (e != cudaSuccess) {
		set_error(std::string("cross_sections_beam: ") + cudaGetErrorString(e));
		return ADDA_GB300_ECUDA;
	}
	const double PI = 3.14159265358979323846;
	for (int r = 0; r < R; r++) {
		double s0 = 0, s1 = 0;
		for (int b = 0; b < w->nbv; b++) {
			s0 += part[((size_t)r * w->nbv + b) * 8];
			s1 += part[((size_t)r * w->nbv + b) * 8 + 1];
		}
		if (cext) cext[r] = s0 * 4 * PI * c->k * inc_scale;
		if (cabs) cabs[r] = 4 * PI * c->k * s1 * inc_scale;
	}
	return ADDA_GB300_OK;
}

} // namespace adda
