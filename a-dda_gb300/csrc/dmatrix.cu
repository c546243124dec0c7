// dmatrix.cu - the interaction matrix D = -FFT(G)/Ngrid on the GPU in FP64 (InitDmatrix, src/fft.c:918-1416).
//
//   1. green_fill      : point-dipole Green's tensor (interaction.c:290-331), optionally with the FCD corrections
//                        (interaction.c:335-411), for every lattice offset
//                        (i in (-bX,bX), j in [0,bY), k in [0,bZ)), stored per component as [k][j][i mod gX]
//   2. fft_lines (x)   : forward FFT along x of every (component, k, j) line
//   3. per component   : slice_fill mirrors the (j,k) quarter into the full (y,z) plane of every kx with the
//                        parities of the tensor components (xy,yz odd in y; xz,yz odd in z; fft.c:1275-1290),
//                        fft_lines along z then y, and d_extract keeps y<=gY/2, z<=gZ/2 scaled by -1/Ngrid into the
//                        reduced layout [x][z][y][6] (fft.c:144-150, 1310-1314)
//   4. an FP32 copy for the single-precision matvec.
//   5. surface mode (InitRmatrix, src/fft.c:818-887): refl_fill evaluates the reflected tensor for every in-plane
//      offset and height sum k in [0, 2bZ-1) (image dipole on the GPU, plus the Sommerfeld integrals of a host table,
//      or the caller's own tensor), the same x/z/y transforms follow with the y mirror only (heights are not
//      mirrored), and r_extract keeps y <= gY/2 and every z: R = -FFT(GR)/Ngrid in [x][z][y][6].
// This runs once per particle; it is written for clarity over speed (it costs a few FP64 3-D FFTs).
#include "ctx.cuh"

#include <cmath>
#include <vector>

namespace adda {

namespace {

// cosine and sine integrals for x > 0: power series up to x = 2, above it the continued fraction of the exponential
// integral E1(ix) = -Ci(x) + i(Si(x) - pi/2) (Abramowitz & Stegun 5.2.23) by the modified Lentz method
__device__ void cisi_d(double x, double &ci, double &si)
{
	if (x <= 2) {
		double sc = 0, ss = 0, term = 1; // x^n / n!
		for (int n = 1; n < 60; n++) {
			term *= x / n;
			const double sg = ((n >> 1) & 1) ? -1.0 : 1.0;
			if (n & 1) ss += sg * term / n;
			else sc += sg * term / n;
			if (term < 1e-18) break;
		}
		ci = 0.57721566490153286061 + log(x) + sc;
		si = ss;
		return;
	}
	// complex arithmetic on (re, im) pairs; z = i x
	double br = 1, bi = x;                       // b = z + 1
	double dr, di;                               // d = 1/b
	{
		const double m = br * br + bi * bi;
		dr = br / m;
		di = -bi / m;
	}
	double cr = 1e300, ci2 = 0, hr = dr, hi = di; // c, h
	for (int i = 1; i < 10000; i++) {
		const double a = -(double)i * i;
		br += 2;
		// d = 1/(a d + b)
		const double tr = a * dr + br, ti = a * di + bi, m = tr * tr + ti * ti;
		dr = tr / m;
		di = -ti / m;
		// c = b + a/c
		const double cm = cr * cr + ci2 * ci2;
		const double qr = br + a * cr / cm, qi = bi - a * ci2 / cm;
		cr = qr;
		ci2 = qi;
		// del = c d; h *= del
		const double er = cr * dr - ci2 * di, ei = cr * di + ci2 * dr;
		const double nr = hr * er - hi * ei, ni = hr * ei + hi * er;
		hr = nr;
		hi = ni;
		if (fabs(er - 1) + fabs(ei) < 1e-16) break;
	}
	double sn, cs;
	sincos(x, &sn, &cs);
	// E1(ix) = h exp(-ix)
	const double e1r = hr * cs + hi * sn, e1i = hi * cs - hr * sn;
	ci = -e1r;
	si = 1.57079632679489661923 + e1i;
}

// the scaled lower incomplete gamma function f = g(s, x)/x^s = exp(-x) sum_k Gamma(s) x^k / Gamma(s+k+1), by its
// series (converges fast for x <= 1; the reference's gamma_scaled, interaction.c:603-621)
__device__ double gamma_scaled(double s, double x, double expmx)
{
	double ap = s, del = 1 / s, sum = del;
	for (int it = 0; it < 200; it++) {
		ap += 1;
		del *= x / ap;
		sum += del;
		if (fabs(del) <= fabs(sum) * 2.220446049250313e-16) break;
	}
	return sum * expmx;
}

// 2/(sqrt(2 pi) d Rp) times the integral of exp(-(x+t)^2/(2 Rp^2)) over t in [-d/2, d/2] (AverageGaussCube,
// interaction.c:625-635), through erf or erfc so that no digits are lost
__device__ double average_gauss_cube(double x, double d, double rp)
{
	x = fabs(x);
	const double y = x / (1.4142135623730950488 * rp), z = d / (2 * 1.4142135623730950488 * rp);
	const double dif = (x < 1) ? erf(y + z) - erf(y - z) : erfc(y - z) - erfc(y + z);
	return dif / d;
}

// ---- the tabulated terms IGT_SO and SO (InterTerm_igt_so_int, InterTerm_so_int; interaction.c:431-579, 711-941) ----

constexpr int TAB_RMAX = 10, TAB_SIZE = 142;
// start of t1..t10 in the flat table array (values per entry 1, 6, 3, 18, 6, 36, 1, 6, 1, 6)
__constant__ int TAB_OFF[10] = {0, 142, 994, 1420, 3976, 4828, 9940, 10082, 10934, 11076};

struct IgtTables {
	const double *t;  // the flat tables (device)
	const int *index; // [TAB_RMAX+1][TAB_RMAX+1]: entry of (i, j, 0), i >= j
	double2 m;        // SO: refractive index of the m^2 terms
};

__device__ __forceinline__ double2 zmul(double2 a, double2 b)
{
	return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// g holds the point-dipole tensor of offset (i,j,k) on entry. Pairs with kd*rn^2 < 1 and rn <= 10 take the tabulated
// integrals of the Green's tensor over the two cubes: the offset is mapped onto i >= j >= k >= 0 (a sign per axis,
// the axes ordered by decreasing coordinate with the reference's tie order) and each component (mu,nu) reads the
// table entries of the mapped axes; SO adds its orientation-averaged m^2 term. Other pairs: the point-dipole tensor
// times 1 - kd^2/24 (SO: 1 - (1+m^2) kd^2/24) plus, for kr < 1, the median correction
// (-1 + ikr) 7/(64 rn^4) [qq(33 q4 - 7 - 12(q_mu^2 + q_nu^2)) + delta(1 - 3 q4 + 4 q_mu^2)] exp(ikr)/r^3.
__device__ void green_igt(double2 g[6], int i, int j, int k, double rn, const double q[3], const double qm[6], double kr,
	double kd, double2 ev, bool so, const IgtTables &tb)
{
	const int cmu[6] = {0, 0, 0, 1, 1, 2}, cnu[6] = {0, 1, 2, 1, 2, 2};
	const double kr2 = kr * kr, kd2 = kd * kd;
	const double2 m2 = zmul(tb.m, tb.m);
	if (kr * rn < 1 && rn <= TAB_RMAX) {
		int v[3] = {i, j, k};
		double s[3], qa[3];
		for (int a = 0; a < 3; a++) {
			s[a] = v[a] < 0 ? -1 : 1;
			v[a] = abs(v[a]);
			qa[a] = q[a] * s[a];
		}
		int o0, o1, o2; // axis of the largest, middle and smallest coordinate
		if (v[0] >= v[1]) {
			if (v[0] >= v[2]) { o0 = 0; if (v[1] >= v[2]) { o1 = 1; o2 = 2; } else { o1 = 2; o2 = 1; } }
			else { o0 = 2; o1 = 0; o2 = 1; }
		}
		else {
			if (v[0] >= v[2]) { o0 = 1; o1 = 0; o2 = 2; }
			else { o2 = 0; if (v[1] >= v[2]) { o0 = 1; o1 = 2; } else { o0 = 2; o1 = 1; } }
		}
		int rank[3];
		rank[o0] = 0; rank[o1] = 1; rank[o2] = 2;
		const double qp0 = qa[o0], qp1 = qa[o1], qp2 = qa[o2];
		const int e0 = tb.index[v[o0] * (TAB_RMAX + 1) + v[o1]] + v[o2];
		const double *t = tb.t;
		const double *t3 = t + TAB_OFF[2] + 3 * e0, *t5 = t + TAB_OFF[4] + 6 * e0;
		const double t3q = qp0 * t3[0] + qp1 * t3[1] + qp2 * t3[2];
		const double t5tr = t5[0] + t5[2] + t5[5];
		for (int a = 0; a < 6; a++) {
			const int mu = cmu[a], nu = cnu[a];
			const bool diag = mu == nu;
			const double sig = s[mu] * s[nu];
			const int r1 = rank[mu], r2 = rank[nu];
			const int e2 = 6 * e0 + r1 + r2 + ((r1 == 2 || r2 == 2) ? 1 : 0); // symmetric order xx,xy,yy,xz,yz,zz
			const double *t4 = t + TAB_OFF[3] + 3 * e2, *t6 = t + TAB_OFF[5] + 6 * e2;
			const double t4q = qp0 * t4[0] + qp1 * t4[1] + qp2 * t4[2];
			const double t6tr = t6[0] + t6[2] + t6[5];
			// kd^2 [sig (3 (I10/2 + I8) - 2 t4q - t6tr) + (kr/24) qq (kr + 3i) + delta (2 t3q + t5tr - (kr/24)(kr + i)
			//       - I9/2 - I7)] + sig I2 (3 - 3i kr - kr^2) + delta I1 (-1 + i kr + kr^2)
			double br = sig * (3 * (t[TAB_OFF[9] + e2] / 2 + t[TAB_OFF[7] + e2]) - 2 * t4q - t6tr) + kr * kr * qm[a] / 24;
			double bi = kr * 3 * qm[a] / 24;
			if (diag) {
				br += 2 * t3q + t5tr - kr * kr / 24 - t[TAB_OFF[8] + e0] / 2 - t[TAB_OFF[6] + e0];
				bi -= kr / 24;
			}
			br *= kd2;
			bi *= kd2;
			const double i2 = sig * t[TAB_OFF[1] + e2];
			br += i2 * (3 - kr2);
			bi -= i2 * 3 * kr;
			if (diag) {
				const double i1 = t[TAB_OFF[0] + e0];
				br += i1 * (kr2 - 1);
				bi += i1 * kr;
			}
			g[a] = zmul(ev, make_double2(br, bi));
			if (so) { // (kd^2/2) m^2 [delta t5tr/3 - sig t6tr + (kr/12)((kr + 3i) qq - delta (kr + i))]
				double cr = kr * (kr * qm[a]) / 12 - sig * t6tr, ci = kr * 3 * qm[a] / 12;
				if (diag) {
					cr += t5tr / 3 - kr * kr / 12;
					ci -= kr / 12;
				}
				const double2 w = zmul(zmul(ev, m2), make_double2(kd2 / 2 * cr, kd2 / 2 * ci));
				g[a] = make_double2(g[a].x + w.x, g[a].y + w.y);
			}
		}
		return;
	}
	const double2 f = so ? make_double2(1 - (1 + m2.x) * kd2 / 24, -m2.y * kd2 / 24) : make_double2(1 - kd2 / 24, 0);
	for (int a = 0; a < 6; a++) g[a] = zmul(g[a], f);
	if (kr < 1) {
		const double q2[3] = {q[0] * q[0], q[1] * q[1], q[2] * q[2]};
		const double q4 = q2[0] * q2[0] + q2[1] * q2[1] + q2[2] * q2[2];
		const double invrn4 = 1 / (rn * rn * rn * rn);
		const double2 em = zmul(ev, make_double2(-1, kr));
		for (int a = 0; a < 6; a++) {
			const int mu = cmu[a], nu = cnu[a];
			double tt = qm[a] * (33 * q4 - 7 - 12 * (q2[mu] + q2[nu]));
			if (mu == nu) tt += 1 - 3 * q4 + 4 * q2[mu];
			tt *= 7 * invrn4 / 64;
			g[a] = make_double2(g[a].x + em.x * tt, g[a].y + em.y * tt);
		}
	}
}

__global__ void green_fill(double2 *G, int bX, int bY, int bZ, int gX, double gridspace, double k, int inter,
	double rp, IgtTables tb)
{
	const size_t lines = (size_t)bZ * bY;
	const size_t total = lines * gX;
	for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
		const int xp = (int)(t % gX);
		const size_t jk = t / gX;
		const int j = (int)(jk % bY), kk = (int)(jk / bY);
		int i;
		bool valid = true;
		if (xp < bX) i = xp;
		else if (xp > gX - bX) i = xp - gX;
		else { i = 0; valid = false; }
		if (i == 0 && j == 0 && kk == 0) valid = false;
		double2 g[6];
		if (valid) {
			double q0 = i, q1 = j, q2 = kk;
			const double rn = sqrt(q0 * q0 + q1 * q1 + q2 * q2);
			const double invrn = 1.0 / rn;
			q0 *= invrn; q1 *= invrn; q2 *= invrn;
			const double rr = rn * gridspace;
			const double invr3 = 1 / (rr * rr * rr);
			const double kr = k * rr, kr2 = kr * kr;
			const double t1 = 3 - kr2, t2 = -3 * kr, t3 = kr2 - 1;
			double sn, cs;
			sincos(kr, &sn, &cs);
			const double evr = invr3 * cs, evi = invr3 * sn;
			const double qm[6] = {q0 * q0, q0 * q1, q0 * q2, q1 * q1, q1 * q2, q2 * q2};
#pragma unroll
			for (int a = 0; a < 6; a++) {
				double re, im;
				if (a == 0 || a == 3 || a == 5) {
					re = t1 * qm[a] + t3;
					im = kr + t2 * qm[a];
				}
				else {
					re = t1 * qm[a];
					im = t2 * qm[a];
				}
				g[a] = make_double2(re * evr - im * evi, re * evi + im * evr);
			}
			if (inter == ADDA_INT_NLOC || inter == ADDA_INT_NLOC_AV) {
				// static non-local interaction of two Gaussian densities (InterTerm_nloc_both, interaction.c:637-703):
				// G = t1 (3 qq - I) - t2 I with t1 = 4/(3 sqrt(pi) R^3) g(5/2, R^2/(2Rp^2)) and t2 = (4pi/3) h(R), h
				// the Gaussian (or its cube average)
				double t1, t2 = 0;
				if (rp == 0) t1 = invr3; // no lattice offset lies inside the cube around 0
				else {
					const double invrp3 = 1 / (rp * rp * rp), sx = 0.70710678118654752440 * rr / rp, x = sx * sx;
					const double expmx = exp(-x);
					const double sqrt2_9pi = 0.26596152026762178529, sqrt_pi = 1.7724538509055160273;
					if (x > 1) // g(5/2, x) by upward recursion from erf
						t1 = 4 / (3 * sqrt_pi) * (0.75 * sqrt_pi * erf(sx) - sx * (1.5 + x) * expmx) * invr3;
					else t1 = sqrt2_9pi * x * gamma_scaled(2.5, x, expmx) * invrp3;
					if (inter == ADDA_INT_NLOC_AV)
						t2 = 0.52359877559829887308 * average_gauss_cube(q0 * rr, gridspace, rp) *
							average_gauss_cube(q1 * rr, gridspace, rp) * average_gauss_cube(q2 * rr, gridspace, rp);
					else t2 = expmx * invrp3 * sqrt2_9pi;
				}
#pragma unroll
				for (int a = 0; a < 6; a++) {
					double re = 3 * t1 * qm[a];
					if (a == 0 || a == 3 || a == 5) re -= t1 + t2;
					g[a] = make_double2(re, 0);
				}
			}
			else if (inter == ADDA_INT_IGT_SO || inter == ADDA_INT_SO) {
				const double q[3] = {q0, q1, q2};
				green_igt(g, i, j, kk, rn, q, qm, kr, k * gridspace, make_double2(evr, evi), inter == ADDA_INT_SO, tb);
			}
			else if (inter) {
				// FCD corrections of the real part (InterTerm_fcd / _fcd_st, interaction.c:335-411): k_F = pi/d
				const double kfr = 3.14159265358979323846 * rn;
				double sf, cf;
				sincos(kfr, &sf, &cf);
				if (inter == 2) {
					double cI, sI;
					cisi_d(kfr, cI, sI);
					const double brd = 2 / (3 * 3.14159265358979323846) * (3 * sI + kfr * cf - 4 * sf);
					for (int a = 0; a < 6; a++) g[a] = make_double2(g[a].x * brd, g[a].y * brd);
				}
				else {
					double ci1, si1, ci2, si2;
					cisi_d(kfr + kr, ci1, si1);
					cisi_d(kfr - kr, ci2, si2);
					const double cI = ci1 - ci2, sI = 3.14159265358979323846 - si1 - si2;
					const double ipi = 0.31830988618379067154;
					const double g0 = ipi * (evi * cI + evr * sI);
					const double g2 = ipi * (kr * (evr * cI - evi * sI) + 2.0 / 3 * invr3 * (kfr * cf - 4 * sf)) - g0;
					const double tt = g0 * kr2;
#pragma unroll
					for (int a = 0; a < 6; a++) {
						double brd = qm[a] * (tt + 3 * g2);
						if (a == 0 || a == 3 || a == 5) brd -= tt + g2;
						g[a].x += brd;
					}
				}
			}
		}
		else
			for (int a = 0; a < 6; a++) g[a] = make_double2(0, 0);
		for (int a = 0; a < 6; a++) G[(size_t)a * total + t] = g[a];
	}
}

// Generic batched FFT of lines: element e of line (o, l) at data[o*od + l*ls + e*es]. Blocks: x = tile of TL lines
// in l, y = o. Either es == 1 (contiguous lines) or ls == 1 (adjacent lines); tiles are loaded along that axis.
template <typename C>
__global__ void __launch_bounds__(256) fft_lines(C *data, FftPlan p, const C *__restrict__ tw, int inv, size_t es,
	size_t ls, int nl_inner, size_t od, int TL)
{
	extern __shared__ __align__(16) unsigned char smem_raw[];
	const int LS = tile_ls(TL);
	C *a = reinterpret_cast<C *>(smem_raw);
	C *b = a + (size_t)p.n * LS;
	const int n = p.n;
	const int l0 = blockIdx.x * TL;
	const int tl = min(TL, nl_inner - l0);
	C *base = data + blockIdx.y * od + (size_t)l0 * ls;
	const bool contig = (es == 1);
	for (int t = threadIdx.x; t < n * TL; t += blockDim.x) {
		int e, l;
		if (contig) { l = t / n; e = t % n; }
		else { e = t / TL; l = t % TL; }
		a[e * LS + l] = (l < tl) ? base[(size_t)l * ls + (size_t)e * es] : cx<C>(0, 0);
	}
	__syncthreads();
	C *o = fft_tile<C>(a, b, p, TL, LS, tw, inv != 0);
	for (int t = threadIdx.x; t < n * TL; t += blockDim.x) {
		int e, l;
		if (contig) { l = t / n; e = t % n; }
		else { e = t / TL; l = t % TL; }
		if (l < tl) base[(size_t)l * ls + (size_t)e * es] = o[e * LS + l];
	}
}

__global__ void slice_fill(double2 *S, const double2 *Ga, int bY, int bZ, int gX, int gY, int gZ, double sy,
	double sz)
{
	const size_t total = (size_t)gX * gY * gZ;
	for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
		const int z = (int)(t % gZ);
		const size_t xy = t / gZ;
		const int y = (int)(xy % gY), x = (int)(xy / gY);
		int j, kk;
		double s = 1;
		if (y < bY) j = y;
		else if (y > gY - bY) { j = gY - y; s *= sy; }
		else j = -1;
		if (z < bZ) kk = z;
		else if (z > gZ - bZ) { kk = gZ - z; s *= sz; }
		else kk = -1;
		double2 v = make_double2(0, 0);
		if (j >= 0 && kk >= 0) {
			const double2 g = Ga[((size_t)kk * bY + j) * gX + x];
			v = make_double2(s * g.x, s * g.y);
		}
		S[t] = v;
	}
}

__global__ void d_extract(double2 *D, const double2 *S, int a, int gX, int gY, int gZ, int DsY, int DsZ, double invN)
{
	const size_t total = (size_t)gX * DsZ * DsY;
	for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
		const int y = (int)(t % DsY);
		const size_t xz = t / DsY;
		const int z = (int)(xz % DsZ), x = (int)(xz / DsZ);
		const double2 v = S[((size_t)x * gY + y) * gZ + z];
		D[t * 6 + a] = make_double2(-invN * v.x, -invN * v.y);
	}
}

// reflected Green's tensor of offset (i, j) and height sum k (lattice units, the probe minus the image of the source):
// ReflParams + ReflTerm_core (interaction.c:1092-1134: the point-dipole term scaled by the normal-incidence reflection
// coefficient rcn, z components inverted), for SOM plus CombineSomTensor of the table's four integrals at
// rho = |(i,j)| (interaction.c:1229-1301); HOST copies the caller's tensor. Stored per component as [k][j][i mod gX].
__global__ void refl_fill(double2 *G, int bX, int bY, int bZ, int gX, double gridspace, double k, double zshift,
	double2 rcn, int refl, const double2 *data)
{
	const int nk = 2 * bZ - 1;
	const size_t total = (size_t)nk * bY * gX;
	for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
		const int x = (int)(t % gX);
		const size_t l = t / gX;
		const int j = (int)(l % bY), kk = (int)(l / bY);
		double2 g[6];
		for (int a = 0; a < 6; a++) g[a] = make_double2(0, 0);
		const bool inside = x < bX || x > gX - bX;
		const int i = x < bX ? x : x - gX;
		if (inside && refl == ADDA_REFL_HOST) {
			const double2 *v = data + (((size_t)kk * bY + j) * (2 * bX - 1) + (i + bX - 1)) * 6;
			for (int a = 0; a < 6; a++) g[a] = v[a];
		}
		else if (inside && !(i == 0 && j == 0 && kk + zshift == 0)) {
			// (the zero distance itself is left 0: no pair of dipoles above the substrate has that height sum)
			const double q0 = i, q1 = j, q2 = kk + zshift;
			double rr = sqrt(q0 * q0 + q1 * q1 + q2 * q2);
			const double inv = 1 / rr, v0 = q0 * inv, v1 = q1 * inv, v2 = q2 * inv;
			const double qm[6] = {v0 * v0, v0 * v1, v0 * v2, v1 * v1, v1 * v2, v2 * v2};
			rr *= gridspace;
			const double invr3 = 1 / (rr * rr * rr), kr = k * rr, kr2 = kr * kr;
			const double t1 = 3 - kr2, t2 = -3 * kr, t3 = kr2 - 1;
			double sn, cs;
			sincos(kr, &sn, &cs);
			const double2 sc = make_double2(invr3 * (rcn.x * cs - rcn.y * sn), invr3 * (rcn.x * sn + rcn.y * cs));
			for (int a = 0; a < 6; a++) {
				double re, im;
				if (a == 0 || a == 3 || a == 5) {
					re = t1 * qm[a] + t3;
					im = kr + t2 * qm[a];
				}
				else {
					re = t1 * qm[a];
					im = t2 * qm[a];
				}
				g[a] = make_double2(re * sc.x - im * sc.y, re * sc.y + im * sc.x);
			}
			g[2] = make_double2(-g[2].x, -g[2].y);
			g[4] = make_double2(-g[4].x, -g[4].y);
			g[5] = make_double2(-g[5].x, -g[5].y);
			if (refl == ADDA_REFL_SOM) {
				const double2 *v = data + (((size_t)kk * bY + j) * bX + (i < 0 ? -i : i)) * 4;
				const double2 Irv = v[0], Izv = v[1], Irh = v[2], Iph = v[3];
				const double rho = hypot((double)i, (double)j);
				if (rho == 0) {
					g[0] = make_double2(g[0].x + Irh.x, g[0].y + Irh.y);
					g[3] = make_double2(g[3].x + Irh.x, g[3].y + Irh.y);
				}
				else {
					const double xr = i / rho, yr = j / rho;
					const double a2 = xr * xr, b2 = yr * yr, ab = xr * yr;
					g[0] = make_double2(g[0].x + a2 * Irh.x - b2 * Iph.x, g[0].y + a2 * Irh.y - b2 * Iph.y);
					g[1] = make_double2(g[1].x + ab * (Irh.x + Iph.x), g[1].y + ab * (Irh.y + Iph.y));
					g[2] = make_double2(g[2].x + xr * Irv.x, g[2].y + xr * Irv.y);
					g[3] = make_double2(g[3].x + b2 * Irh.x - a2 * Iph.x, g[3].y + b2 * Irh.y - a2 * Iph.y);
					g[4] = make_double2(g[4].x + yr * Irv.x, g[4].y + yr * Irv.y);
				}
				g[5] = make_double2(g[5].x + Izv.x, g[5].y + Izv.y);
			}
		}
		for (int a = 0; a < 6; a++) G[(size_t)a * total + t] = g[a];
	}
}

// the (j, k) half-plane of one reflected component into the full (y, z) plane of every kx: y mirrored with the
// component's parity (xy and yz odd in y, fft.c:859-865), heights k < nk at z = k, zero elsewhere
__global__ void slice_fill_r(double2 *S, const double2 *Ga, int bY, int nk, int gX, int gY, int gZ, double sy)
{
	const size_t total = (size_t)gX * gY * gZ;
	for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
		const int z = (int)(t % gZ);
		const size_t xy = t / gZ;
		const int y = (int)(xy % gY), x = (int)(xy / gY);
		int j;
		double s = 1;
		if (y < bY) j = y;
		else if (y > gY - bY) { j = gY - y; s = sy; }
		else j = -1;
		double2 v = make_double2(0, 0);
		if (j >= 0 && z < nk) {
			const double2 g = Ga[((size_t)z * bY + j) * gX + x];
			v = make_double2(s * g.x, s * g.y);
		}
		S[t] = v;
	}
}

__global__ void r_extract(double2 *Rm, const double2 *S, int a, int gX, int gY, int gZ, int RsY, double invN)
{
	const size_t total = (size_t)gX * gZ * RsY;
	for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
		const int y = (int)(t % RsY);
		const size_t xz = t / RsY;
		const int z = (int)(xz % gZ), x = (int)(xz / gZ);
		const double2 v = S[((size_t)x * gY + y) * gZ + z];
		Rm[t * 6 + a] = make_double2(-invN * v.x, -invN * v.y);
	}
}

__global__ void to_f32(float2 *dst, const double2 *src, size_t n)
{
	for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x)
		dst[t] = make_float2((float)src[t].x, (float)src[t].y);
}

int grid_for(size_t n)
{
	size_t g = (n + 255) / 256;
	if (g > 152 * 64) g = 152 * 64;
	if (g < 1) g = 1;
	return (int)g;
}

// FFT of all lines described by (es, ls, nl_inner, od, nouter) with the FP64 plan p
int fft_lines_run(adda_gb300_ctx *c, double2 *data, const FftPlan &p, const double2 *tw, bool inv, size_t es,
	size_t ls, int nl_inner, size_t od, int nouter)
{
	int TL = 16;
	while (TL > 1 && 2 * sizeof(double2) * (size_t)p.n * tile_ls(TL) > 200 * 1024) TL /= 2;
	const size_t smem = 2 * sizeof(double2) * (size_t)p.n * tile_ls(TL);
	ADDA_CUDA(cudaFuncSetAttribute(fft_lines<double2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
	dim3 g((nl_inner + TL - 1) / TL, nouter);
	fft_lines<double2><<<g, 256, smem, c->stream>>>(data, p, tw, inv ? 1 : 0, es, ls, nl_inner, od, TL);
	ADDA_LAUNCHED();
	return ADDA_GB300_OK;
}

int rmatrix_build(adda_gb300_ctx *c)
{
	const int bX = c->bX, bY = c->bY, bZ = c->bZ, gX = c->gX, gY = c->gY, gZ = c->gZ;
	const int nk = 2 * bZ - 1, RsY = gY / 2 + 1;
	const size_t lines = (size_t)nk * bY;
	const size_t gsz = lines * gX;
	const size_t ssz = (size_t)gX * gY * gZ;
	const size_t rlen = (size_t)gX * gZ * RsY * 6;
	double2 *G = nullptr, *S = nullptr, *data = nullptr;
	int rc = ADDA_GB300_OK;
	if (cudaMalloc(&G, sizeof(double2) * 6 * gsz) != cudaSuccess ||
		cudaMalloc(&S, sizeof(double2) * ssz) != cudaSuccess ||
		(!c->refl_host.empty() && cudaMalloc(&data, sizeof(double2) * c->refl_host.size()) != cudaSuccess)) {
		cudaFree(G);
		cudaFree(S);
		set_error("cannot allocate the R-matrix build buffers");
		return ADDA_GB300_ENOMEM;
	}
	// surfRCn, interaction.c:1411
	double2 rcn = make_double2(-1, 0);
	if (!c->msub_inf) {
		const double mr = c->msub.x, mi = c->msub.y;
		const double m2r = mr * mr - mi * mi, m2i = 2 * mr * mi;
		const double nr = 1 - m2r, ni = -m2i, dr = 1 + m2r, di = m2i, dd = dr * dr + di * di;
		rcn = make_double2((nr * dr + ni * di) / dd, (ni * dr - nr * di) / dd);
	}
	const double invN = 1.0 / (gX * ((double)gY * gZ));
	do {
		if (data && cudaMemcpyAsync(data, c->refl_host.data(), sizeof(double2) * c->refl_host.size(),
				cudaMemcpyHostToDevice, c->stream) != cudaSuccess) { rc = ADDA_GB300_ECUDA; break; }
		refl_fill<<<grid_for(gsz), 256, 0, c->stream>>>(G, bX, bY, bZ, gX, c->gridspace, c->k, c->zsum_shift, rcn,
			c->refl, data);
		count_launch();
		if (cudaGetLastError() != cudaSuccess) { rc = ADDA_GB300_ECUDA; break; }
		if ((rc = fft_lines_run(c, G, c->px[0], c->tw64[0], false, 1, gX, (int)(6 * lines), 0, 1))) break;
		for (int a = 0; a < 6 && !rc; a++) {
			const double sy = (a == 1 || a == 4) ? -1 : 1;
			slice_fill_r<<<grid_for(ssz), 256, 0, c->stream>>>(S, G + (size_t)a * gsz, bY, nk, gX, gY, gZ, sy);
			count_launch();
			if (cudaGetLastError() != cudaSuccess) { rc = ADDA_GB300_ECUDA; break; }
			if ((rc = fft_lines_run(c, S, c->pz[0], c->tw64[2], false, 1, gZ, gX * gY, 0, 1))) break;
			if ((rc = fft_lines_run(c, S, c->py[0], c->tw64[1], false, gZ, 1, gZ, (size_t)gY * gZ, gX))) break;
			r_extract<<<grid_for((size_t)gX * gZ * RsY), 256, 0, c->stream>>>(c->R64, S, a, gX, gY, gZ, RsY, invN);
			count_launch();
			if (cudaGetLastError() != cudaSuccess) { rc = ADDA_GB300_ECUDA; break; }
		}
		if (rc) break;
		to_f32<<<grid_for(rlen), 256, 0, c->stream>>>(c->R32, c->R64, rlen);
		count_launch();
		if (cudaGetLastError() != cudaSuccess) { rc = ADDA_GB300_ECUDA; break; }
		if (cudaStreamSynchronize(c->stream) != cudaSuccess) { rc = ADDA_GB300_ECUDA; break; }
	} while (0);
	if (rc == ADDA_GB300_ECUDA) set_error(std::string("R-matrix build: ") + cudaGetErrorString(cudaGetLastError()));
	cudaFree(G);
	cudaFree(S);
	cudaFree(data);
	return rc;
}

} // namespace

int dmatrix_build(adda_gb300_ctx *c)
{
	const int bX = c->bX, bY = c->bY, bZ = c->bZ, gX = c->gX, gY = c->gY, gZ = c->gZ;
	const size_t lines = (size_t)bZ * bY;
	const size_t gsz = lines * gX;
	const size_t ssz = (size_t)gX * gY * gZ;
	const size_t dlen = (size_t)gX * c->DsZ * c->DsY * 6;
	double2 *G = nullptr, *S = nullptr;
	int rc = ADDA_GB300_OK;
	if (cudaMalloc(&G, sizeof(double2) * 6 * gsz) != cudaSuccess ||
		cudaMalloc(&S, sizeof(double2) * ssz) != cudaSuccess) {
		cudaFree(G);
		set_error("cannot allocate the D-matrix build buffers");
		return ADDA_GB300_ENOMEM;
	}
	const double invN = 1.0 / (gX * ((double)gY * gZ));
	// IGT_SO / SO: the integral tables and the entry index of (i, j, 0) (ReadTables, interaction.c:1051-1061: row
	// (i, j) holds k = 0..min(j, floor(sqrt(RMAX^2 - i^2 - j^2))))
	IgtTables tb{nullptr, nullptr, c->so_m};
	double *d_tabs = nullptr;
	int *d_index = nullptr;
	if (!c->int_tables.empty()) {
		std::vector<int> index((TAB_RMAX + 1) * (TAB_RMAX + 1), 0);
		int next = 0;
		for (int i = 1; i <= TAB_RMAX; i++)
			for (int j = 0; j <= i && i * i + j * j <= TAB_RMAX * TAB_RMAX; j++) {
				index[i * (TAB_RMAX + 1) + j] = next;
				next += std::min(j, (int)std::floor(std::sqrt((double)(TAB_RMAX * TAB_RMAX - i * i - j * j)))) + 1;
			}
		if (next != TAB_SIZE || cudaMalloc(&d_tabs, sizeof(double) * c->int_tables.size()) != cudaSuccess ||
			cudaMalloc(&d_index, sizeof(int) * index.size()) != cudaSuccess ||
			cudaMemcpyAsync(d_tabs, c->int_tables.data(), sizeof(double) * c->int_tables.size(),
				cudaMemcpyHostToDevice, c->stream) != cudaSuccess ||
			cudaMemcpyAsync(d_index, index.data(), sizeof(int) * index.size(), cudaMemcpyHostToDevice, c->stream) !=
				cudaSuccess ||
			cudaStreamSynchronize(c->stream) != cudaSuccess) {
			cudaFree(G);
			cudaFree(S);
			cudaFree(d_tabs);
			cudaFree(d_index);
			set_error("cannot stage the integral tables of the interaction term");
			return ADDA_GB300_ENOMEM;
		}
		tb.t = d_tabs;
		tb.index = d_index;
	}
	do {
		green_fill<<<grid_for(gsz), 256, 0, c->stream>>>(G, bX, bY, bZ, gX, c->gridspace, c->k, c->interaction,
			c->nloc_rp, tb);
		count_launch();
		if (cudaGetLastError() != cudaSuccess) { rc = ADDA_GB300_ECUDA; break; }
		// x transform of all 6*bZ*bY lines (contiguous, length gX)
		if ((rc = fft_lines_run(c, G, c->px[0], c->tw64[0], false, 1, gX, (int)(6 * lines), 0, 1))) break;
		for (int a = 0; a < 6 && !rc; a++) {
			const double sy = (a == 1 || a == 4) ? -1 : 1, sz = (a == 2 || a == 4) ? -1 : 1;
			slice_fill<<<grid_for(ssz), 256, 0, c->stream>>>(S, G + (size_t)a * gsz, bY, bZ, gX, gY, gZ, sy, sz);
			count_launch();
			if (cudaGetLastError() != cudaSuccess) { rc = ADDA_GB300_ECUDA; break; }
			// z transform: lines (x,y) contiguous of length gZ
			if ((rc = fft_lines_run(c, S, c->pz[0], c->tw64[2], false, 1, gZ, gX * gY, 0, 1))) break;
			// y transform: element stride gZ, lines z adjacent, outer x
			if ((rc = fft_lines_run(c, S, c->py[0], c->tw64[1], false, gZ, 1, gZ, (size_t)gY * gZ, gX))) break;
			d_extract<<<grid_for((size_t)gX * c->DsZ * c->DsY), 256, 0, c->stream>>>(c->D64, S, a, gX, gY, gZ,
				c->DsY, c->DsZ, invN);
			count_launch();
			if (cudaGetLastError() != cudaSuccess) { rc = ADDA_GB300_ECUDA; break; }
		}
		if (rc) break;
		to_f32<<<grid_for(dlen), 256, 0, c->stream>>>(c->D32, c->D64, dlen);
		count_launch();
		if (cudaGetLastError() != cudaSuccess) { rc = ADDA_GB300_ECUDA; break; }
		if (cudaStreamSynchronize(c->stream) != cudaSuccess) { rc = ADDA_GB300_ECUDA; break; }
	} while (0);
	if (rc == ADDA_GB300_ECUDA) set_error(std::string("D-matrix build: ") + cudaGetErrorString(cudaGetLastError()));
	cudaFree(G);
	cudaFree(S);
	cudaFree(d_tabs);
	cudaFree(d_index);
	if (!rc && c->surface) rc = rmatrix_build(c);
	if (!rc) c->dready = true;
	return rc;
}

} // namespace adda
