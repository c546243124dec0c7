/* adda_oracle.c - CPU restatement of ADDA's FFT-accelerated DDA matvec, D-matrix, Krylov solvers and cross sections.
 *
 * TEST INFRASTRUCTURE (oracle): the checker for the GPU product and the timed CPU baseline, nothing else. Every
 * function names the reference code it restates (ADDA 1.3b6, paths relative to the reference project). The data
 * layouts follow the reference's own where the reference fixes them (the reduced D layout of fft.c:144-150); the
 * rest is organised for clarity and OpenMP parallelism.
 */
#include "adda_oracle.h"
#include "cfft.h"

#include <complex.h>
#include <math.h>
#include <omp.h>
#include <stdlib.h>
#include <string.h>

typedef double complex cplx;

#define OR_MAXMAT 256

struct or_ctx {
	int bX, bY, bZ, gX, gY, gZ;
	size_t n;            // number of non-void dipoles
	uint16_t *pos;       // [n][3] grid coordinates
	uint8_t *mat;        // [n] material index
	double gridspace, k;
	int inter;           // 0 point dipoles, 1 FCD, 2 static FCD, 3 non-local, 4 non-local (cube-averaged),
	                     // 5 IGT_SO, 6 SO (tabulated integrals)
	double rp;           // Gaussian width of the non-local interaction
	double *tabs;        // IGT_SO / SO: the ten integral tables t1..t10 back to back (OR_TAB_TOTAL doubles)
	int tab_index[OR_TAB_RMAX + 1][OR_TAB_RMAX + 1];
	cplx so_m;           // SO: the refractive index in the second-order terms (ref_index[0])
	size_t DsY, DsZ;     // reduced D sizes (fft.c:955-963)
	cplx *D;             // [gX][DsZ][DsY][6]
	int per_dip, nmat;
	cplx cc[OR_MAXMAT][3], ccs[OR_MAXMAT][3];
	cplx *ccd, *ccsd;    // per-dipole [n][3] (cc and its root)
	cfft_plan px, py, pz;
	cplx *X;             // expanded grid after the X transform: [3][bZ][bY][gX]
	int nthreads;
	// particle near a substrate (src/interaction.c:1082-1345, src/fft.c:818-887)
	int surf;
	double zshift;       // ZsumShift: distance from the lowest dipole layer to its image (lattice units)
	cplx rcn;            // surfRCn: reflection coefficient at normal incidence
	cplx *somt;          // Sommerfeld integrals [2bZ-1][bY][bX][4] (NULL: image-dipole relation)
	size_t RsY;          // reduced R size along y (gY/2+1)
	cplx *R;             // [gX][gZ][RsY][6]
};

/* fftFit, src/fft.c:528-562 (FFTW3 branch, weird_nprocs=false): smallest even x' >= x divisible by divis whose prime
 * factors are 2,3,5,7 and at most one factor of 11 or 13 */
int or_fftfit(int x, int divis)
{
	for (;; x++) {
		if (x % 2 || x % divis) continue;
		int y = x;
		while (y % 2 == 0) y /= 2;
		while (y % 3 == 0) y /= 3;
		while (y % 5 == 0) y /= 5;
		while (y % 7 == 0) y /= 7;
		if (y % 11 == 0) y /= 11;
		else if (y % 13 == 0) y /= 13;
		if (y == 1) return x;
	}
}

or_ctx *or_create(int bX, int bY, int bZ, int gX, int gY, int gZ, size_t n, const uint16_t *position,
	const uint8_t *material, double gridspace, double wavenum, int nthreads)
{
	or_ctx *c = calloc(1, sizeof(*c));
	c->bX = bX; c->bY = bY; c->bZ = bZ;
	c->gX = gX; c->gY = gY; c->gZ = gZ;
	c->n = n;
	c->pos = malloc(sizeof(uint16_t) * 3 * n);
	c->mat = malloc(n ? n : 1);
	memcpy(c->pos, position, sizeof(uint16_t) * 3 * n);
	if (material) memcpy(c->mat, material, n);
	else memset(c->mat, 0, n);
	c->gridspace = gridspace;
	c->k = wavenum;
	c->nthreads = nthreads > 0 ? nthreads : omp_get_max_threads();
	cfft_plan_init(&c->px, gX);
	cfft_plan_init(&c->py, gY);
	cfft_plan_init(&c->pz, gZ);
	c->X = malloc(sizeof(cplx) * 3 * (size_t)bZ * bY * gX);
	return c;
}

void or_free(or_ctx *c)
{
	if (!c) return;
	cfft_plan_free(&c->px);
	cfft_plan_free(&c->py);
	cfft_plan_free(&c->pz);
	free(c->pos); free(c->mat); free(c->D); free(c->X); free(c->ccd); free(c->ccsd); free(c->somt); free(c->R);
	free(c->tabs);
	free(c);
}

/* Point-dipole Green's tensor for integer offset (i,j,k) in units of the lattice spacing:
 * InterParams + InterTerm_core + InterTerm_poi, src/interaction.c:159-181, 290-331 (non-SSE3 branch).
 * Component order xx,xy,xz,yy,yz,zz. */
static void green_poi(const or_ctx *c, int i, int j, int k, cplx g[6])
{
	double q[3] = {i, j, k};
	double rn = sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2]);
	double invrn = 1.0 / rn;
	for (int a = 0; a < 3; a++) q[a] *= invrn;
	double rr = rn * c->gridspace;
	double invr3 = 1 / (rr * rr * rr);
	double kr = c->k * rr, kr2 = kr * kr;
	double qm[6] = {q[0] * q[0], q[0] * q[1], q[0] * q[2], q[1] * q[1], q[1] * q[2], q[2] * q[2]};
	double t1 = 3 - kr2, t2 = -3 * kr, t3 = kr2 - 1;
	cplx ev = invr3 * (cos(kr) + I * sin(kr));
	for (int a = 0; a < 6; a++) {
		if (a == 0 || a == 3 || a == 5) g[a] = ((t1 * qm[a] + t3) + I * (kr + t2 * qm[a])) * ev;
		else g[a] = (t1 + I * t2) * qm[a] * ev;
	}
}

/* Ci(x) = gamma + ln x + sum_k (-1)^k x^(2k)/(2k (2k)!), Si(x) = sum_k (-1)^k x^(2k+1)/((2k+1)(2k+1)!) for x <= 3;
 * for larger x from the exponential integral E1(ix) = -Ci(x) + i(Si(x) - pi/2) (Abramowitz & Stegun 5.2.23), whose
 * continued fraction E1(z) = exp(-z)/(z+1- 1/(z+3- 4/(z+5- ...))) is evaluated by the modified Lentz method */
void or_cisi(double x, double *ci, double *si)
{
	const double euler = 0.57721566490153286061;
	if (x <= 3) {
		double sc = 0, ss = 0, term = 1; // term = x^n / n!
		for (int n = 1; n < 80; n++) {
			term *= x / n;
			if (n % 2) ss += ((n / 2) % 2 ? -1 : 1) * term / n;
			else sc += ((n / 2) % 2 ? -1 : 1) * term / n;
			if (term < 1e-18 * (fabs(ss) + fabs(sc) + 1)) break;
		}
		*ci = euler + log(x) + sc;
		*si = ss;
		return;
	}
	const cplx z = I * x;
	cplx b = z + 1, cc = 1e300, d = 1 / b, h = d;
	for (int i = 1; i < 10000; i++) {
		const double a = -(double)i * i;
		b += 2;
		d = 1 / (a * d + b);
		cc = b + a / cc;
		const cplx del = cc * d;
		h *= del;
		if (cabs(del - 1) < 1e-16) break;
	}
	h *= cos(x) - I * sin(x); // E1(ix)
	*ci = -creal(h);
	*si = M_PI / 2 + cimag(h);
}

void or_set_interaction(or_ctx *c, int relation)
{
	c->inter = relation;
}

void or_set_nloc_rp(or_ctx *c, double rp)
{
	c->rp = rp;
}

/* Non-local interaction of two Gaussian dipole densities of width Rp, static (InterTerm_nloc_both,
 * src/interaction.c:637-703): G = t1 (3 qq - I) - t2 I, t1 = 4/(3 sqrt(pi) R^3) g(5/2, x), x = R^2/(2 Rp^2), from
 * erf by g(1/2,x) = sqrt(pi) erf(sqrt x), g(s+1,x) = s g(s,x) - exp(-x) x^s for x > 1 and from the series of
 * g(5/2,x)/x^(5/2) below (gamma_scaled, :603-621); t2 = (4pi/3) h(R), the Gaussian exp(-x)/((2pi)^(3/2) Rp^3) or, for
 * nloc_av, its average over the cube around the dipole (product of three erf differences, AverageGaussCube :625-635) */
static double gauss_cube(const or_ctx *c, double x)
{
	x = fabs(x);
	const double y = x / (M_SQRT2 * c->rp), z = c->gridspace / (2 * M_SQRT2 * c->rp);
	return ((x < 1) ? erf(y + z) - erf(y - z) : erfc(y - z) - erfc(y + z)) / c->gridspace;
}

static void green_nloc(const or_ctx *c, int i, int j, int k, cplx g[6])
{
	const double rn = sqrt((double)i * i + (double)j * j + (double)k * k);
	const double q[3] = {i / rn, j / rn, k / rn};
	const double rr = rn * c->gridspace, invr3 = 1 / (rr * rr * rr);
	double t1, t2 = 0;
	if (c->rp == 0) t1 = invr3;
	else {
		const double x = rr * rr / (2 * c->rp * c->rp), sx = sqrt(x), e = exp(-x), irp3 = 1 / pow(c->rp, 3);
		if (x > 1) {
			const double g12 = sqrt(M_PI) * erf(sx);                    // g(1/2, x)
			const double g32 = 0.5 * g12 - e * sx;                       // g(3/2, x)
			const double g52 = 1.5 * g32 - e * x * sx;                   // g(5/2, x)
			t1 = 4 / (3 * sqrt(M_PI)) * g52 * invr3;
		}
		else {
			double term = 1 / 2.5, sum = term; // g(5/2,x)/x^(5/2) = exp(-x) sum_n x^n / ((5/2)(7/2)...(5/2+n))
			for (int n = 1; n < 200 && term > sum * 1e-17; n++) {
				term *= x / (2.5 + n);
				sum += term;
			}
			t1 = 4 / (3 * sqrt(M_PI)) * e * sum * x * pow(2 * c->rp * c->rp, -1.5); // g52/R^3 = f x (2Rp^2)^(-3/2)
		}
		if (c->inter == 4)
			t2 = M_PI / 6 * gauss_cube(c, q[0] * rr) * gauss_cube(c, q[1] * rr) * gauss_cube(c, q[2] * rr);
		else t2 = e * irp3 * sqrt(2 / (9 * M_PI));
	}
	const double qm[6] = {q[0] * q[0], q[0] * q[1], q[0] * q[2], q[1] * q[1], q[1] * q[2], q[2] * q[2]};
	for (int a = 0; a < 6; a++) g[a] = 3 * t1 * qm[a] - ((a == 0 || a == 3 || a == 5) ? t1 + t2 : 0);
}

/* FCD corrections of the point-dipole term, InterTerm_fcd / InterTerm_fcd_st, src/interaction.c:335-411
 * (Gay-Balmaz & Martin 2002, Piller 1998): with k_F = pi/d, kfr = pi*|q| */
static void green_fcd(const or_ctx *c, int i, int j, int k, cplx g[6])
{
	green_poi(c, i, j, k, g);
	const double rn = sqrt((double)i * i + (double)j * j + (double)k * k);
	const double rr = rn * c->gridspace, invr3 = 1 / (rr * rr * rr), kr = c->k * rr, kr2 = kr * kr;
	const double kfr = M_PI * rn;
	const double ce = cos(kfr), se = sin(kfr);
	if (c->inter == 2) {
		double ci, si;
		or_cisi(kfr, &ci, &si);
		const double brd = 2 / (3 * M_PI) * (3 * si + kfr * ce - 4 * se);
		for (int a = 0; a < 6; a++) g[a] *= brd;
		return;
	}
	const cplx ev = invr3 * (cos(kr) + I * sin(kr));
	double ci1, si1, ci2, si2;
	or_cisi(kfr + kr, &ci1, &si1);
	or_cisi(kfr - kr, &ci2, &si2);
	const double ci = ci1 - ci2, si = M_PI - si1 - si2;
	const double g0 = (cimag(ev) * ci + creal(ev) * si) / M_PI;
	const double g2 = (kr * (creal(ev) * ci - cimag(ev) * si) + 2.0 / 3 * invr3 * (kfr * ce - 4 * se)) / M_PI - g0;
	const double t = g0 * kr2;
	const double q[3] = {i / rn, j / rn, k / rn};
	const double qm[6] = {q[0] * q[0], q[0] * q[1], q[0] * q[2], q[1] * q[1], q[1] * q[2], q[2] * q[2]};
	for (int a = 0; a < 6; a++) {
		double brd = qm[a] * (t + 3 * g2);
		if (a == 0 || a == 3 || a == 5) brd -= t + g2;
		g[a] += brd;
	}
}

/* ---------------- tabulated interaction terms (IGT_SO, SO) ---------------- */

// values per table entry of t1..t10
static const int tab_mult[10] = {1, 6, 3, 18, 6, 36, 1, 6, 1, 6};

void or_set_tables(or_ctx *c, const double *tables, double m_re, double m_im)
{
	free(c->tabs);
	c->tabs = malloc(sizeof(double) * OR_TAB_TOTAL);
	memcpy(c->tabs, tables, sizeof(double) * OR_TAB_TOTAL);
	c->so_m = m_re + I * m_im;
	/* ReadTables, src/interaction.c:1051-1061: entry (i,j,k) with i >= j >= k >= 0 and i^2+j^2+k^2 <= RMAX^2 sits at
	 * tab_index[i][j] + k; row (i, j) holds k = 0..min(j, floor(sqrt(RMAX^2 - i^2 - j^2))) */
	const int R2 = OR_TAB_RMAX * OR_TAB_RMAX;
	int next = 0;
	for (int i = 1; i <= OR_TAB_RMAX; i++)
		for (int j = 0; j <= i && i * i + j * j <= R2; j++) {
			c->tab_index[i][j] = next;
			int kmax = (int)floor(sqrt((double)(R2 - i * i - j * j)));
			next += (kmax < j ? kmax : j) + 1;
		}
}

static const double *tab_of(const or_ctx *c, int n) // t<n>, n = 1..10
{
	size_t off = 0;
	for (int t = 0; t < n - 1; t++) off += (size_t)OR_TAB_SIZE * tab_mult[t];
	return c->tabs + off;
}

/* InterTerm_igt_so_int / InterTerm_so_int, src/interaction.c:431-579 and 711-941 (SO with its fixed
 * orientation-averaged form, inter_avg = true: no Gc1/Gf1/Gm1 terms). Close pairs (kd*rn^2 < 1, rn <= 10): the
 * tabulated Green's tensor integrals, after mapping the offset onto i >= j >= k >= 0 (signs flipped per axis,
 * coordinates sorted in the reference's order); SO adds the m^2 term Gc2. Other pairs: the point-dipole tensor
 * times 1 - kd^2/24 (SO: 1 - (1+m^2) kd^2/24), plus the median correction Gm0 where kr < 1. Component order
 * xx,xy,xz,yy,yz,zz; the tables' symmetric-matrix order is xx,xy,yy,xz,yz,zz. */
static void green_igt(const or_ctx *c, int i, int j, int k, cplx g[6])
{
	green_poi(c, i, j, k, g);
	const int so = c->inter == 6;
	const double rn = sqrt((double)i * i + (double)j * j + (double)k * k);
	const double q[3] = {i / rn, j / rn, k / rn};
	const double qm[6] = {q[0] * q[0], q[0] * q[1], q[0] * q[2], q[1] * q[1], q[1] * q[2], q[2] * q[2]};
	const int cmu[6] = {0, 0, 0, 1, 1, 2}, cnu[6] = {0, 1, 2, 1, 2, 2};
	const double rr = rn * c->gridspace, invr3 = 1 / (rr * rr * rr), kr = c->k * rr, kr2 = kr * kr;
	const double kd = c->k * c->gridspace, kd2 = kd * kd;
	const cplx ev = invr3 * (cos(kr) + I * sin(kr));
	const cplx m2 = c->so_m * c->so_m;
	if (kr * rn < 1 && rn <= OR_TAB_RMAX) {
		int v[3] = {i, j, k}, sg[3];
		double qa[3];
		for (int a = 0; a < 3; a++) {
			sg[a] = v[a] < 0 ? -1 : 1;
			v[a] *= sg[a];
			qa[a] = q[a] * sg[a];
		}
		// ord[n] = the axis of the n-th largest coordinate, ties resolved like the reference
		int ord[3];
		if (v[0] >= v[1]) {
			if (v[0] >= v[2]) {
				ord[0] = 0;
				if (v[1] >= v[2]) { ord[1] = 1; ord[2] = 2; }
				else { ord[1] = 2; ord[2] = 1; }
			}
			else { ord[0] = 2; ord[1] = 0; ord[2] = 1; }
		}
		else {
			if (v[0] >= v[2]) { ord[0] = 1; ord[1] = 0; ord[2] = 2; }
			else {
				ord[2] = 0;
				if (v[1] >= v[2]) { ord[0] = 1; ord[1] = 2; }
				else { ord[0] = 2; ord[1] = 1; }
			}
		}
		int inv[3], vp[3];
		double qp[3];
		for (int a = 0; a < 3; a++) {
			inv[ord[a]] = a;
			qp[a] = qa[ord[a]];
			vp[a] = v[ord[a]];
		}
		const int e0 = c->tab_index[vp[0]][vp[1]] + vp[2];
		const double *t1 = tab_of(c, 1), *t2 = tab_of(c, 2), *t3 = tab_of(c, 3) + 3 * e0, *t5 = tab_of(c, 5) + 6 * e0;
		const double *t4 = tab_of(c, 4), *t6 = tab_of(c, 6), *t7 = tab_of(c, 7), *t8 = tab_of(c, 8);
		const double *t9 = tab_of(c, 9), *t10 = tab_of(c, 10);
		const double t3q = qp[0] * t3[0] + qp[1] * t3[1] + qp[2] * t3[2];
		const double t5tr = t5[0] + t5[2] + t5[5];
		for (int a = 0; a < 6; a++) {
			const int mu = cmu[a], nu = cnu[a], diag = mu == nu;
			const double sig = sg[mu] * sg[nu];
			const int m1 = inv[mu], n1 = inv[nu];
			const int e2 = 6 * e0 + m1 + n1 + ((m1 == 2 || n1 == 2) ? 1 : 0);
			const double *t4e = t4 + 3 * e2, *t6e = t6 + 6 * e2;
			const double t4q = qp[0] * t4e[0] + qp[1] * t4e[1] + qp[2] * t4e[2];
			const double t6tr = t6e[0] + t6e[2] + t6e[5];
			// Gc0: kd^2 [sig(3(I10/2 + I8) - 2 t4q - t6tr) + kr qq (kr + 3i)/24 + delta(2 t3q + t5tr - kr(kr + i)/24
			//      - I9/2 - I7)] + sig I2 (3 - 3ikr - kr^2) + delta I1 (-1 + ikr + kr^2), times exp(ikr)/r^3
			cplx br = sig * (3 * (t10[e2] / 2 + t8[e2]) - 2 * t4q - t6tr) + (kr / 24) * qm[a] * (kr + 3 * I);
			if (diag) br += 2 * t3q + t5tr - (kr / 24) * (kr + I) - t9[e0] / 2 - t7[e0];
			br *= kd2;
			br += sig * t2[e2] * (3 - 3 * I * kr - kr2);
			if (diag) br += t1[e0] * (-1 + I * kr + kr2);
			g[a] = ev * br;
			if (so) { // Gc2 with <a_mu a_nu> = delta/3: (kd^2/2) m^2 [delta t5tr/3 - sig t6tr - kr(delta(kr + i) -
				      // qq(kr + 3i))/12]
				cplx b2 = -(kr + 3 * I) * qm[a];
				if (diag) b2 += kr + I;
				b2 = -b2 * kr / 12 - sig * t6tr;
				if (diag) b2 += t5tr / 3;
				g[a] += ev * (kd2 / 2) * m2 * b2;
			}
		}
		return;
	}
	const cplx f = so ? 1 - (1 + m2) * kd2 / 24 : 1 - kd2 / 24;
	for (int a = 0; a < 6; a++) g[a] *= f;
	if (kr < 1) { // Gm0 = exp(ikr)/r^3 (-1 + ikr) (7/(64 rn^4)) [qq(33 q4 - 7 - 12(q_mu^2 + q_nu^2)) + delta(1 - 3q4 + 4q_mu^2)]
		const double q2[3] = {q[0] * q[0], q[1] * q[1], q[2] * q[2]};
		const double q4 = q2[0] * q2[0] + q2[1] * q2[1] + q2[2] * q2[2];
		const double invrn4 = 1 / (rn * rn * rn * rn);
		for (int a = 0; a < 6; a++) {
			const int mu = cmu[a], nu = cnu[a];
			double t = qm[a] * (33 * q4 - 7 - 12 * (q2[mu] + q2[nu]));
			if (mu == nu) t += 1 - 3 * q4 + 4 * q2[mu];
			t *= 7 * invrn4 / 64;
			g[a] += ev * (-1 + I * kr) * t;
		}
	}
}

size_t or_dmatrix_len(const or_ctx *c)
{
	return (size_t)c->gX * c->DsZ * c->DsY * 6;
}

static void init_rmatrix(or_ctx *c);

/* InitDmatrix, src/fft.c:918-1322 (sequential, reduced_FFT): D = -FFT(G)/Ngrid, stored for y<=gY/2, z<=gZ/2 only;
 * the remaining octants follow from the reflection symmetries of G (components xy,yz odd in y; xz,yz odd in z). */
void or_init_dmatrix(or_ctx *c)
{
	const int bX = c->bX, bY = c->bY, bZ = c->bZ, gX = c->gX, gY = c->gY, gZ = c->gZ;
	c->DsY = gY / 2 + 1;
	c->DsZ = gZ / 2 + 1;
	free(c->D);
	c->D = calloc(or_dmatrix_len(c), sizeof(cplx));
	const double invN = 1.0 / (gX * ((double)gY * gZ));
	const size_t lines = (size_t)bZ * bY;
	cplx *G = calloc(6 * lines * gX, sizeof(cplx)); // [comp][k][j][x mod gX]
	#pragma omp parallel for num_threads(c->nthreads) schedule(dynamic)
	for (int k = 0; k < bZ; k++)
		for (int j = 0; j < bY; j++)
			for (int i = 1 - bX; i < bX; i++) {
				if (!i && !j && !k) continue;
				cplx g[6];
				if (c->inter >= 5) green_igt(c, i, j, k, g);
				else if (c->inter >= 3) green_nloc(c, i, j, k, g);
				else if (c->inter) green_fcd(c, i, j, k, g);
				else green_poi(c, i, j, k, g);
				size_t idx = ((size_t)k * bY + j) * gX + (i < 0 ? i + gX : i);
				for (int a = 0; a < 6; a++) G[a * lines * gX + idx] = g[a];
			}
	for (int a = 0; a < 6; a++) {
		cplx *Ga = G + a * lines * gX;
		const double sy = (a == 1 || a == 4) ? -1 : 1, sz = (a == 2 || a == 4) ? -1 : 1;
		#pragma omp parallel num_threads(c->nthreads)
		{
			cplx *work = malloc(sizeof(cplx) * (gX > gY ? (gX > gZ ? gX : gZ) : (gY > gZ ? gY : gZ)));
			cplx *s = malloc(sizeof(cplx) * (size_t)gY * gZ); // [y][z]
			#pragma omp for
			for (size_t l = 0; l < lines; l++) cfft_exec(&c->px, Ga + l * gX, work, -1);
			#pragma omp for
			for (int x = 0; x < gX; x++) {
				memset(s, 0, sizeof(cplx) * (size_t)gY * gZ);
				for (int j = 0; j < bY; j++)
					for (int k = 0; k < bZ; k++) s[(size_t)j * gZ + k] = Ga[((size_t)k * bY + j) * gX + x];
				for (int j = 1; j < bY; j++) // mirror along y (fft.c:1276-1282)
					for (int k = 0; k < bZ; k++) s[(size_t)(gY - j) * gZ + k] = sy * s[(size_t)j * gZ + k];
				for (int j = 1 - bY; j < bY; j++) { // mirror along z (fft.c:1283-1289)
					size_t row = (size_t)(j < 0 ? j + gY : j) * gZ;
					for (int k = 1; k < bZ; k++) s[row + gZ - k] = sz * s[row + k];
				}
				for (int y = 0; y < gY; y++) cfft_exec(&c->pz, s + (size_t)y * gZ, work, -1);
				cfft_exec_strided(&c->py, s, gZ, 1, (size_t)gZ, -1);
				for (size_t z = 0; z < c->DsZ; z++)
					for (size_t y = 0; y < c->DsY; y++)
						c->D[(((size_t)x * c->DsZ + z) * c->DsY + y) * 6 + a] = -invN * s[y * gZ + z];
			}
			free(work);
			free(s);
		}
	}
	free(G);
	if (c->surf) init_rmatrix(c);
}

void or_get_dmatrix(const or_ctx *c, double *out)
{
	memcpy(out, c->D, sizeof(cplx) * or_dmatrix_len(c));
}

/* surfRCn, src/interaction.c:1411: (1 - msub^2)/(1 + msub^2), -1 for a perfectly reflecting substrate */
void or_set_surface(or_ctx *c, double zsum_shift, double msub_re, double msub_im, int msub_inf,
	const double *som_table)
{
	const cplx m = msub_re + I * msub_im;
	c->surf = 1;
	c->zshift = zsum_shift;
	c->rcn = msub_inf ? -1 : (1 - m * m) / (1 + m * m);
	free(c->somt);
	c->somt = NULL;
	if (som_table) {
		const size_t len = (size_t)4 * (2 * c->bZ - 1) * c->bY * c->bX;
		c->somt = malloc(sizeof(cplx) * len);
		memcpy(c->somt, som_table, sizeof(cplx) * len);
	}
}

/* Reflected Green's tensor for the lattice offset (i, j) and height sum k (lattice units, probe minus image of the
 * source): ReflParams + ReflTerm_core (image dipole scaled by surfRCn, z components inverted),
 * src/interaction.c:1092-1134, plus with a Sommerfeld table CombineSomTensor of the four integrals at rho = |(i,j)|,
 * src/interaction.c:1229-1301. Component order xx,xy,xz,yy,yz,zz. */
static void green_refl(const or_ctx *c, int i, int j, int k, cplx g[6])
{
	const double q[3] = {i, j, k + c->zshift};
	double rr = sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2]);
	const double qv[3] = {q[0] / rr, q[1] / rr, q[2] / rr};
	const double qm[6] = {qv[0] * qv[0], qv[0] * qv[1], qv[0] * qv[2], qv[1] * qv[1], qv[1] * qv[2], qv[2] * qv[2]};
	rr *= c->gridspace;
	const double invr3 = 1 / (rr * rr * rr), kr = c->k * rr, kr2 = kr * kr;
	const double t1 = 3 - kr2, t2 = -3 * kr, t3 = kr2 - 1;
	const cplx scale = c->rcn * (invr3 * (cos(kr) + I * sin(kr)));
	for (int a = 0; a < 6; a++) {
		if (a == 0 || a == 3 || a == 5) g[a] = ((t1 * qm[a] + t3) + I * (kr + t2 * qm[a])) * scale;
		else g[a] = (t1 + I * t2) * qm[a] * scale;
	}
	g[2] = -g[2];
	g[4] = -g[4];
	g[5] = -g[5];
	if (c->somt) {
		const int iT = i < 0 ? -i : i, jT = j < 0 ? -j : j;
		const cplx *v = c->somt + 4 * (((size_t)k * c->bY + jT) * c->bX + iT);
		const cplx Irv = v[0], Izv = v[1], Irh = v[2], Iph = v[3];
		const double x = i, y = j, rho = hypot(x, y);
		if (rho == 0) {
			g[0] += Irh;
			g[3] += Irh;
			g[5] += Izv;
		}
		else {
			const double xr = x / rho, yr = y / rho;
			g[0] += xr * xr * Irh - yr * yr * Iph;
			g[1] += xr * yr * (Irh + Iph);
			g[2] += xr * Irv;
			g[3] += yr * yr * Irh - xr * xr * Iph;
			g[4] += yr * Irv;
			g[5] += Izv;
		}
	}
}

size_t or_rmatrix_len(const or_ctx *c)
{
	return c->surf ? (size_t)c->gX * c->gZ * (c->gY / 2 + 1) * 6 : 0;
}

void or_get_rmatrix(const or_ctx *c, double *out)
{
	if (c->R) memcpy(out, c->R, sizeof(cplx) * or_rmatrix_len(c));
}

/* InitRmatrix, src/fft.c:818-887 (sequential, reduced_FFT): R = -FFT(GR)/Ngrid with GR(i,j,k) for i in (-bX,bX),
 * j in [0,bY) mirrored to negative y (xy and yz odd in y), height sums k in [0, 2bZ-1) placed at z = k without
 * mirroring; stored for y <= gY/2 and every z. */
static void init_rmatrix(or_ctx *c)
{
	const int bX = c->bX, bY = c->bY, bZ = c->bZ, gX = c->gX, gY = c->gY, gZ = c->gZ;
	const int nk = 2 * bZ - 1;
	c->RsY = gY / 2 + 1;
	free(c->R);
	c->R = calloc(or_rmatrix_len(c), sizeof(cplx));
	const double invN = 1.0 / (gX * ((double)gY * gZ));
	const size_t lines = (size_t)nk * bY;
	cplx *G = calloc(6 * lines * gX, sizeof(cplx)); // [comp][k][j][x mod gX]
	#pragma omp parallel for num_threads(c->nthreads) schedule(dynamic)
	for (int k = 0; k < nk; k++)
		for (int j = 0; j < bY; j++)
			for (int i = 1 - bX; i < bX; i++) {
				cplx g[6];
				green_refl(c, i, j, k, g);
				size_t idx = ((size_t)k * bY + j) * gX + (i < 0 ? i + gX : i);
				for (int a = 0; a < 6; a++) G[a * lines * gX + idx] = g[a];
			}
	for (int a = 0; a < 6; a++) {
		cplx *Ga = G + a * lines * gX;
		const double sy = (a == 1 || a == 4) ? -1 : 1;
		#pragma omp parallel num_threads(c->nthreads)
		{
			cplx *work = malloc(sizeof(cplx) * (gX > gY ? (gX > gZ ? gX : gZ) : (gY > gZ ? gY : gZ)));
			cplx *s = malloc(sizeof(cplx) * (size_t)gY * gZ); // [y][z]
			#pragma omp for
			for (size_t l = 0; l < lines; l++) cfft_exec(&c->px, Ga + l * gX, work, -1);
			#pragma omp for
			for (int x = 0; x < gX; x++) {
				memset(s, 0, sizeof(cplx) * (size_t)gY * gZ);
				for (int j = 0; j < bY; j++)
					for (int k = 0; k < nk; k++) s[(size_t)j * gZ + k] = Ga[((size_t)k * bY + j) * gX + x];
				for (int j = 1; j < bY; j++) // mirror along y (fft.c:859-865)
					for (int k = 0; k < nk; k++) s[(size_t)(gY - j) * gZ + k] = sy * s[(size_t)j * gZ + k];
				for (int y = 0; y < gY; y++) cfft_exec(&c->pz, s + (size_t)y * gZ, work, -1);
				cfft_exec_strided(&c->py, s, gZ, 1, (size_t)gZ, -1);
				for (size_t z = 0; z < (size_t)gZ; z++)
					for (size_t y = 0; y < c->RsY; y++)
						c->R[(((size_t)x * gZ + z) * c->RsY + y) * 6 + a] = -invN * s[y * gZ + z];
			}
			free(work);
			free(s);
		}
	}
	free(G);
}

/* InitCC, src/calculator.c:266-289: cc_sqrt = csqrt(cc) */
void or_set_cc_mat(or_ctx *c, int nmat, const double *cc)
{
	const cplx *in = (const cplx *)cc;
	c->per_dip = 0;
	c->nmat = nmat;
	for (int m = 0; m < nmat && m < OR_MAXMAT; m++)
		for (int a = 0; a < 3; a++) {
			c->cc[m][a] = in[3 * m + a];
			c->ccs[m][a] = csqrt(in[3 * m + a]);
		}
}

void or_set_cc_dip(or_ctx *c, const double *cc)
{
	const cplx *in = (const cplx *)cc;
	c->per_dip = 1;
	free(c->ccd); free(c->ccsd);
	c->ccd = malloc(sizeof(cplx) * 3 * c->n);
	c->ccsd = malloc(sizeof(cplx) * 3 * c->n);
	for (size_t i = 0; i < 3 * c->n; i++) {
		c->ccd[i] = in[i];
		c->ccsd[i] = csqrt(in[i]);
	}
}

static inline cplx ccs_of(const or_ctx *c, size_t i, int a)
{
	return c->per_dip ? c->ccsd[3 * i + a] : c->ccs[c->mat[i]][a];
}

static inline cplx cc_of(const or_ctx *c, size_t i, int a)
{
	return c->per_dip ? c->ccd[3 * i + a] : c->cc[c->mat[i]][a];
}

/* MatVec, src/matvec.c:128-425 (FFT mode, sequential): y = x + S.D.S.x with S = diag(cc_sqrt); her => A^H via
 * conjugation of input and output. inprod (if not NULL) receives |y|^2. */
void or_matvec(or_ctx *c, const double *argv, double *resv, double *inprod, int her)
{
	const cplx *arg = (const cplx *)argv;
	cplx *res = (cplx *)resv;
	const int bY = c->bY, bZ = c->bZ, gX = c->gX, gY = c->gY, gZ = c->gZ;
	const size_t plane = (size_t)bZ * bY * gX;
	const size_t DsY = c->DsY, DsZ = c->DsZ;
	cplx *X = c->X;
	memset(X, 0, sizeof(cplx) * 3 * plane);
	// scatter S.x onto the expanded grid (matvec.c:205-212)
	for (size_t i = 0; i < c->n; i++) {
		size_t idx = ((size_t)c->pos[3 * i + 2] * bY + c->pos[3 * i + 1]) * gX + c->pos[3 * i];
		for (int a = 0; a < 3; a++) {
			cplx v = arg[3 * i + a];
			if (her) v = conj(v);
			X[a * plane + idx] = ccs_of(c, i, a) * v;
		}
	}
	#pragma omp parallel num_threads(c->nthreads)
	{
		int gmax = gX > gY ? (gX > gZ ? gX : gZ) : (gY > gZ ? gY : gZ);
		cplx *work = malloc(sizeof(cplx) * gmax);
		cplx *col = malloc(sizeof(cplx) * 3 * gY);
		cplx *s = malloc(sizeof(cplx) * 3 * (size_t)gY * gZ); // [comp][y][z]
		// surface: the same slab transformed along z with the opposite sign (height sums instead of differences,
		// fft.c:396-399 planZRf), then along y (matvec.c:249, fft.c:366-367)
		cplx *sR = c->surf ? malloc(sizeof(cplx) * 3 * (size_t)gY * gZ) : NULL;
		cplx *colR = c->surf ? malloc(sizeof(cplx) * 3 * gY) : NULL;
		#pragma omp for
		for (size_t l = 0; l < 3 * (size_t)bZ * bY; l++) cfft_exec(&c->px, X + l * gX, work, -1);
		#pragma omp for schedule(dynamic)
		for (int x = 0; x < gX; x++) {
			memset(s, 0, sizeof(cplx) * 3 * (size_t)gY * gZ);
			for (int a = 0; a < 3; a++)
				for (int y = 0; y < bY; y++)
					for (int z = 0; z < bZ; z++)
						s[((size_t)a * gY + y) * gZ + z] = X[a * plane + ((size_t)z * bY + y) * gX + x];
			if (sR) {
				memcpy(sR, s, sizeof(cplx) * 3 * (size_t)gY * gZ);
				for (int a = 0; a < 3; a++)
					for (int y = 0; y < bY; y++) cfft_exec(&c->pz, sR + ((size_t)a * gY + y) * gZ, work, 1);
			}
			for (int a = 0; a < 3; a++)
				for (int y = 0; y < bY; y++) cfft_exec(&c->pz, s + ((size_t)a * gY + y) * gZ, work, -1);
			for (int z = 0; z < gZ; z++) {
				for (int a = 0; a < 3; a++) {
					cplx *ln = col + a * gY;
					for (int y = 0; y < gY; y++) ln[y] = s[((size_t)a * gY + y) * gZ + z];
					cfft_exec(&c->py, ln, work, -1);
					if (sR) {
						cplx *lr = colR + a * gY;
						for (int y = 0; y < gY; y++) lr[y] = sR[((size_t)a * gY + y) * gZ + z];
						cfft_exec(&c->py, lr, work, -1);
					}
				}
				// D~.X~ with the reduced-FFT sign flips (matvec.c:271-305)
				for (int y = 0; y < gY; y++) {
					size_t yy = (size_t)y < DsY ? (size_t)y : (size_t)(gY - y);
					size_t zz = (size_t)z < DsZ ? (size_t)z : (size_t)(gZ - z);
					const cplx *f = c->D + (((size_t)x * DsZ + zz) * DsY + yy) * 6;
					cplx m[6] = {f[0], f[1], f[2], f[3], f[4], f[5]};
					if ((size_t)y >= DsY) {
						m[1] = -m[1];
						if ((size_t)z >= DsZ) m[2] = -m[2];
						else m[4] = -m[4];
					}
					else if ((size_t)z >= DsZ) {
						m[2] = -m[2];
						m[4] = -m[4];
					}
					cplx v0 = col[y], v1 = col[gY + y], v2 = col[2 * gY + y];
					col[y] = m[0] * v0 + m[1] * v1 + m[2] * v2;
					col[gY + y] = m[1] * v0 + m[3] * v1 + m[4] * v2;
					col[2 * gY + y] = m[2] * v0 + m[4] * v1 + m[5] * v2;
					if (sR) { // yv += R~.X'~ with R's reduced-y signs (matvec.c:288-302, cReflMatrVec cmplx.h:391-401)
						const size_t ry = (size_t)y < c->RsY ? (size_t)y : (size_t)(gY - y);
						const cplx *r = c->R + (((size_t)x * gZ + z) * c->RsY + ry) * 6;
						cplx q[6] = {r[0], r[1], r[2], r[3], r[4], r[5]};
						if ((size_t)y >= c->RsY) {
							q[1] = -q[1];
							q[4] = -q[4];
						}
						const cplx u0 = colR[y], u1 = colR[gY + y], u2 = colR[2 * gY + y];
						col[y] += q[0] * u0 + q[1] * u1 + q[2] * u2;
						col[gY + y] += q[1] * u0 + q[3] * u1 + q[4] * u2;
						col[2 * gY + y] += -q[2] * u0 - q[4] * u1 + q[5] * u2;
					}
				}
				for (int a = 0; a < 3; a++) {
					cplx *ln = col + a * gY;
					cfft_exec(&c->py, ln, work, 1);
					for (int y = 0; y < bY; y++) s[((size_t)a * gY + y) * gZ + z] = ln[y];
				}
			}
			for (int a = 0; a < 3; a++)
				for (int y = 0; y < bY; y++) cfft_exec(&c->pz, s + ((size_t)a * gY + y) * gZ, work, 1);
			for (int a = 0; a < 3; a++)
				for (int y = 0; y < bY; y++)
					for (int z = 0; z < bZ; z++)
						X[a * plane + ((size_t)z * bY + y) * gX + x] = s[((size_t)a * gY + y) * gZ + z];
		}
		#pragma omp for
		for (size_t l = 0; l < 3 * (size_t)bZ * bY; l++) cfft_exec(&c->px, X + l * gX, work, 1);
		free(work); free(col); free(s); free(sR); free(colR);
	}
	// gather y = x + S.X (matvec.c:352-364)
	double sum = 0;
	for (size_t i = 0; i < c->n; i++) {
		size_t idx = ((size_t)c->pos[3 * i + 2] * bY + c->pos[3 * i + 1]) * gX + c->pos[3 * i];
		for (int a = 0; a < 3; a++) {
			cplx v = arg[3 * i + a];
			if (her) v = conj(v);
			cplx r = v + ccs_of(c, i, a) * X[a * plane + idx];
			sum += creal(r) * creal(r) + cimag(r) * cimag(r);
			res[3 * i + a] = her ? conj(r) : r;
		}
	}
	if (inprod) *inprod = sum;
}

/* ---------------- BLAS-1 restated from src/linalg.c ---------------- */

static double nnorm2(const cplx *a, size_t n)
{
	double s = 0;
	for (size_t i = 0; i < n; i++) s += creal(a[i]) * creal(a[i]) + cimag(a[i]) * cimag(a[i]);
	return s;
}

static cplx ndot(const cplx *a, const cplx *b, size_t n) // sum a*conj(b), linalg.c:75-88
{
	cplx s = 0;
	for (size_t i = 0; i < n; i++) s += a[i] * conj(b[i]);
	return s;
}

static cplx ndot_conj(const cplx *a, const cplx *b, size_t n) // sum a*b, linalg.c:92-105
{
	cplx s = 0;
	for (size_t i = 0; i < n; i++) s += a[i] * b[i];
	return s;
}

/* ---------------- iterative solvers, src/iterative.c ---------------- */

typedef struct {
	or_ctx *c;
	size_t n;                 // 3*N
	cplx *x, *r, *p, *Av, *v1, *v2, *v3, *v4;
	double inprodR, inprodRp1, epsB;
	int niter, counter, matvec_ready, complete;
	int full; // no exit at BiCGStab's half step: checkpoints of type always (iterative.c:703)
} solver;

static void mv(solver *s, const cplx *in, cplx *out, double *ipr)
{
	or_matvec(s->c, (const double *)in, (double *)out, ipr, 0);
}

/* QMR_CS, src/iterative.c:898-1032 (Freund 1992). Returns OR_OK or OR_EBREAKDOWN. */
typedef struct {
	double c_old, c_new, om_old, om_new;
	cplx beta, tautilda, s_old, s_new;
	cplx *v, *vt, *pn, *po;
} qmr_state;

static void qmr_init(solver *s, qmr_state *q)
{
	const size_t n = s->n;
	q->v = s->v1; q->vt = s->v2; q->pn = s->p; q->po = s->v3;
	q->om_old = 0.0;
	q->beta = csqrt(ndot_conj(s->r, s->r, n));
	q->om_new = sqrt(s->inprodR) / cabs(q->beta);
	cplx t = 1 / q->beta;
	for (size_t i = 0; i < n; i++) q->v[i] = t * s->r[i];
	q->tautilda = q->om_new * q->beta;
	q->c_new = q->c_old = 1.0;
	q->s_new = q->s_old = 0.0;
}

static int qmr_iter(solver *s, qmr_state *q)
{
	const size_t n = s->n;
	if (1 / (q->om_new * q->om_new) < 1e-10) return OR_EBREAKDOWN;
	if (s->niter == 1 && s->matvec_ready) {
		cplx t = 1 / q->beta;
		for (size_t i = 0; i < n; i++) s->Av[i] *= t;
	}
	else mv(s, q->v, s->Av, NULL);
	cplx alpha = ndot_conj(q->v, s->Av, n);
	cplx ma = -alpha;
	if (s->niter == 1) for (size_t i = 0; i < n; i++) q->vt[i] = ma * q->v[i] + s->Av[i];
	else {
		cplx mb = -q->beta;
		for (size_t i = 0; i < n; i++) q->vt[i] = mb * q->vt[i] + ma * q->v[i] + s->Av[i];
	}
	cplx theta = conj(q->s_old) * q->om_old * q->beta;
	cplx eta = q->c_old * q->c_new * q->om_old * q->beta;
	eta += alpha * conj(q->s_new) * q->om_new;
	cplx zetat = q->c_new * q->om_new * alpha - q->s_new * q->c_old * q->om_old * q->beta;
	q->om_old = q->om_new;
	double b0 = 0, b1 = 0, b2 = 0; // nDotProdSelf_conj_Norm2, linalg.c:127-145
	for (size_t i = 0; i < n; i++) {
		b0 += creal(q->vt[i]) * creal(q->vt[i]);
		b1 += cimag(q->vt[i]) * cimag(q->vt[i]);
		b2 += creal(q->vt[i]) * cimag(q->vt[i]);
	}
	double nrm = b0 + b1;
	q->beta = csqrt(b0 - b1 + I * 2 * b2);
	q->om_new = sqrt(nrm) / cabs(q->beta);
	double zt2 = creal(zetat) * creal(zetat) + cimag(zetat) * cimag(zetat);
	double zabs = sqrt(zt2 + nrm);
	double zt = sqrt(zt2);
	cplx zeta = (zt < 1e-40) ? (cplx)zabs : (zabs / zt) * zetat;
	q->c_old = q->c_new;
	q->c_new = zt / zabs;
	q->s_old = q->s_new;
	q->s_new = q->om_new * q->beta / zeta;
	cplx t4 = 1 / zeta;
	if (s->niter == 1) for (size_t i = 0; i < n; i++) q->pn[i] = t4 * q->v[i];
	else {
		cplx t2 = -eta * t4;
		if (s->niter == 2) for (size_t i = 0; i < n; i++) q->po[i] = t2 * q->pn[i] + t4 * q->v[i];
		else {
			cplx t1 = -theta * t4;
			for (size_t i = 0; i < n; i++) q->po[i] = t1 * q->po[i] + t2 * q->pn[i] + t4 * q->v[i];
		}
		cplx *tmp = q->po; q->po = q->pn; q->pn = tmp;
	}
	cplx tau = q->c_new * q->tautilda;
	q->tautilda = -q->s_new * q->tautilda;
	for (size_t i = 0; i < n; i++) s->x[i] += tau * q->pn[i];
	cplx ib = 1 / q->beta;
	for (size_t i = 0; i < n; i++) q->vt[i] *= ib;
	cplx *tmp = q->v; q->v = q->vt; q->vt = tmp;
	double sa2 = creal(q->s_new) * creal(q->s_new) + cimag(q->s_new) * cimag(q->s_new);
	cplx t1 = (q->c_new / q->om_new) * q->tautilda;
	double sum = 0;
	for (size_t i = 0; i < n; i++) {
		s->r[i] = sa2 * s->r[i] + t1 * q->v[i];
		sum += creal(s->r[i]) * creal(s->r[i]) + cimag(s->r[i]) * cimag(s->r[i]);
	}
	s->inprodRp1 = sum;
	return OR_OK;
}

/* BiCGStab, src/iterative.c:640-724 */
typedef struct {
	cplx ro_old, omega, alpha;
	cplx *v, *sv, *rt;
} bcgs_state;

static int bcgs_iter(solver *s, bcgs_state *b)
{
	const size_t n = s->n;
	cplx ro_new = ndot(s->r, b->rt, n);
	if (s->niter == 1) memcpy(s->p, s->r, sizeof(cplx) * n);
	else {
		cplx t1 = ro_new * b->alpha, t2 = b->ro_old * b->omega;
		if (cabs(t2) / cabs(t1) < 1e-10) return OR_EBREAKDOWN;
		cplx beta = t1 / t2;
		cplx mbo = -beta * b->omega;
		for (size_t i = 0; i < n; i++) s->p[i] = beta * s->p[i] + mbo * b->v[i] + s->r[i];
	}
	if (s->niter == 1 && s->matvec_ready) memcpy(b->v, s->Av, sizeof(cplx) * n);
	else mv(s, s->p, b->v, NULL);
	cplx t1 = ndot(b->v, b->rt, n);
	if (cabs(t1) / cabs(ro_new) < 1e-10) return OR_EBREAKDOWN;
	b->alpha = ro_new / t1;
	cplx ma = -b->alpha;
	double sum = 0;
	for (size_t i = 0; i < n; i++) {
		b->sv[i] = ma * b->v[i] + s->r[i];
		sum += creal(b->sv[i]) * creal(b->sv[i]) + cimag(b->sv[i]) * cimag(b->sv[i]);
	}
	s->inprodRp1 = sum;
	if (s->inprodRp1 < s->epsB && !s->full) {
		for (size_t i = 0; i < n; i++) s->x[i] += b->alpha * s->p[i];
		s->complete = 0;
	}
	else {
		double den;
		mv(s, b->sv, s->Av, &den);
		b->omega = ndot(b->sv, s->Av, n) / den;
		for (size_t i = 0; i < n; i++) s->x[i] += b->alpha * s->p[i] + b->omega * b->sv[i];
		cplx mo = -b->omega;
		sum = 0;
		for (size_t i = 0; i < n; i++) {
			s->r[i] = mo * s->Av[i] + b->sv[i];
			sum += creal(s->r[i]) * creal(s->r[i]) + cimag(s->r[i]) * cimag(s->r[i]);
		}
		s->inprodRp1 = sum;
		b->ro_old = ro_new;
	}
	return OR_OK;
}

/* BiCG_CS (COCG), src/iterative.c:490-637 */
static int bicg_iter(solver *s, cplx *ro_old)
{
	const size_t n = s->n;
	cplx ro_new = ndot_conj(s->r, s->r, n);
	const double abs_ro = cabs(ro_new);
	if (abs_ro / s->inprodR < 1e-10) return OR_EBREAKDOWN;
	if (s->niter == 1) memcpy(s->p, s->r, sizeof(cplx) * n);
	else {
		cplx beta = ro_new / *ro_old;
		for (size_t i = 0; i < n; i++) s->p[i] = beta * s->p[i] + s->r[i];
	}
	if (!(s->niter == 1 && s->matvec_ready)) mv(s, s->p, s->Av, NULL);
	cplx mu = ndot_conj(s->p, s->Av, n);
	if (cabs(mu) / abs_ro < 1e-10) return OR_EBREAKDOWN;
	cplx alpha = ro_new / mu;
	for (size_t i = 0; i < n; i++) s->x[i] += alpha * s->p[i];
	cplx ma = -alpha;
	double sum = 0;
	for (size_t i = 0; i < n; i++) {
		s->r[i] += ma * s->Av[i];
		sum += creal(s->r[i]) * creal(s->r[i]) + cimag(s->r[i]) * cimag(s->r[i]);
	}
	s->inprodRp1 = sum;
	*ro_old = ro_new;
	return OR_OK;
}

/* CGNR, src/iterative.c:729-769: CG on A^H A x = A^H b, real recurrence scalars */
static int cgnr_iter(solver *s, double *ro_old)
{
	const size_t n = s->n;
	double ro_new, den;
	if (s->niter == 1) or_matvec(s->c, (const double *)s->r, (double *)s->p, &ro_new, 1);
	else {
		or_matvec(s->c, (const double *)s->r, (double *)s->Av, &ro_new, 1);
		const double beta = ro_new / *ro_old;
		for (size_t i = 0; i < n; i++) s->p[i] = beta * s->p[i] + s->Av[i];
	}
	mv(s, s->p, s->Av, &den);
	const double alpha = ro_new / den;
	for (size_t i = 0; i < n; i++) s->x[i] += alpha * s->p[i];
	double sum = 0;
	for (size_t i = 0; i < n; i++) {
		s->r[i] += -alpha * s->Av[i];
		sum += creal(s->r[i]) * creal(s->r[i]) + cimag(s->r[i]) * cimag(s->r[i]);
	}
	s->inprodRp1 = sum;
	*ro_old = ro_new;
	return OR_OK;
}

/* CSYM (Bunse-Gerstner & Stover), src/iterative.c:773-892; q_k lives in r (q_new) and v1 (q_old), p_k in p / v2 */
typedef struct {
	double beta, c_old, c_new;
	cplx tau, s_old, s_new;
	cplx *q_new, *q_old, *p_new, *p_old;
} csym_state;

static void csym_init(solver *s, csym_state *q)
{
	q->q_new = s->r; q->q_old = s->v1; q->p_new = s->p; q->p_old = s->v2;
	q->tau = sqrt(s->inprodR);
	const double t = 1 / creal(q->tau);
	for (size_t i = 0; i < s->n; i++) q->q_new[i] = t * conj(q->q_new[i]);
	q->c_new = 1;
	q->c_old = 0;
	q->s_new = q->s_old = 0;
	q->beta = 0;
}

static int csym_iter(solver *s, csym_state *q)
{
	const size_t n = s->n;
	mv(s, q->q_new, s->Av, NULL);
	cplx alpha = ndot_conj(q->q_new, s->Av, n);
	cplx eta = q->c_old * q->c_new * q->beta + alpha * conj(q->s_new);
	cplx gamma = q->c_new * alpha - q->c_old * q->s_new * q->beta;
	cplx theta = q->beta * conj(q->s_old);
	cplx ma = -alpha;
	double dtmp = 0;
	if (s->niter == 1)
		for (size_t i = 0; i < n; i++) {
			q->q_old[i] = ma * conj(q->q_new[i]) + s->Av[i];
			dtmp += creal(q->q_old[i]) * creal(q->q_old[i]) + cimag(q->q_old[i]) * cimag(q->q_old[i]);
		}
	else
		for (size_t i = 0; i < n; i++) {
			q->q_old[i] = -q->beta * conj(q->q_old[i]) + ma * conj(q->q_new[i]) + s->Av[i];
			dtmp += creal(q->q_old[i]) * creal(q->q_old[i]) + cimag(q->q_old[i]) * cimag(q->q_old[i]);
		}
	q->beta = sqrt(dtmp);
	q->c_old = q->c_new;
	q->s_old = q->s_new;
	cplx invksi;
	double ag = cabs(gamma);
	if (ag == 0) {
		if (q->beta == 0) return OR_EBREAKDOWN; // singular interaction matrix (iterative.c:845)
		q->c_new = 0;
		q->s_new = 1;
		invksi = 1 / q->beta;
	}
	else {
		if (ag < q->beta) {
			ag = ag / q->beta;
			q->c_new = ag / sqrt(1 + ag * ag);
		}
		else {
			ag = q->beta / ag;
			q->c_new = 1 / sqrt(1 + ag * ag);
		}
		invksi = q->c_new / gamma;
		q->s_new = q->beta * invksi;
	}
	if (s->niter == 1)
		for (size_t i = 0; i < n; i++) q->p_new[i] = invksi * q->q_new[i];
	else {
		cplx t1 = -eta * invksi;
		if (s->niter == 2)
			for (size_t i = 0; i < n; i++) q->p_old[i] = t1 * q->p_new[i] + invksi * q->q_new[i];
		else {
			cplx t2 = -theta * invksi;
			for (size_t i = 0; i < n; i++) q->p_old[i] = t2 * q->p_old[i] + t1 * q->p_new[i] + invksi * q->q_new[i];
		}
		cplx *tp = q->p_old; q->p_old = q->p_new; q->p_new = tp;
	}
	cplx t1 = q->c_new * q->tau;
	for (size_t i = 0; i < n; i++) s->x[i] += t1 * q->p_new[i];
	const double ib = 1 / q->beta;
	for (size_t i = 0; i < n; i++) q->q_old[i] = ib * conj(q->q_old[i]);
	cplx *tq = q->q_old; q->q_old = q->q_new; q->q_new = tq;
	q->tau *= -q->s_new;
	s->inprodRp1 = creal(q->tau) * creal(q->tau) + cimag(q->tau) * cimag(q->tau);
	return OR_OK;
}

/* QMR_CS_2 (Freund & Nachtigal coupled two-term recurrences), src/iterative.c:1038-1132; v in v1, d in v2 */
typedef struct {
	double c_old, theta_old, ro_old;
	cplx eps, eta;
} qmr2_state;

static void qmr2_init(solver *s, qmr2_state *q)
{
	q->ro_old = sqrt(s->inprodR);
	memcpy(s->v1, s->r, sizeof(cplx) * s->n);
	q->c_old = 1;
	q->eps = 1;
	q->theta_old = 0;
	q->eta = -1;
}

static int qmr2_iter(solver *s, qmr2_state *q)
{
	const size_t n = s->n;
	cplx *v = s->v1, *d = s->v2;
	const double iro = 1 / q->ro_old;
	for (size_t i = 0; i < n; i++) v[i] *= iro;
	cplx delta = ndot_conj(v, v, n);
	if (cabs(delta) < 1e-10) return OR_EBREAKDOWN;
	if (s->niter == 1) memcpy(s->p, v, sizeof(cplx) * n);
	else {
		cplx t = -q->ro_old * delta / q->eps;
		for (size_t i = 0; i < n; i++) s->p[i] = t * s->p[i] + v[i];
	}
	if (s->niter == 1 && s->matvec_ready)
		for (size_t i = 0; i < n; i++) s->Av[i] *= iro;
	else mv(s, s->p, s->Av, NULL);
	q->eps = ndot_conj(s->p, s->Av, n);
	cplx beta = q->eps / delta;
	if (cabs(q->eps) < 1e-10) return OR_EBREAKDOWN;
	cplx mb = -beta;
	double dt = 0;
	for (size_t i = 0; i < n; i++) {
		v[i] = mb * v[i] + s->Av[i];
		dt += creal(v[i]) * creal(v[i]) + cimag(v[i]) * cimag(v[i]);
	}
	const double ro_new = sqrt(dt);
	const double theta_new = ro_new / (q->c_old * cabs(beta));
	const double th2 = theta_new * theta_new;
	const double c_new = 1 / sqrt(1 + th2);
	const double sabs2 = th2 / (1 + th2);
	const double cr = c_new / q->c_old;
	q->eta = -q->ro_old * cr * cr * q->eta / beta;
	if (s->niter == 1)
		for (size_t i = 0; i < n; i++) d[i] = q->eta * s->p[i];
	else {
		const double tc = q->theta_old * c_new, tc2 = tc * tc;
		for (size_t i = 0; i < n; i++) d[i] = tc2 * d[i] + q->eta * s->p[i];
	}
	for (size_t i = 0; i < n; i++) s->x[i] += d[i];
	cplx me = -q->eta;
	double sum = 0;
	for (size_t i = 0; i < n; i++) {
		s->r[i] = sabs2 * s->r[i] + me * v[i];
		sum += creal(s->r[i]) * creal(s->r[i]) + cimag(s->r[i]) * cimag(s->r[i]);
	}
	s->inprodRp1 = sum;
	q->ro_old = ro_new;
	q->theta_old = theta_new;
	q->c_old = c_new;
	return OR_OK;
}

/* BCGS2 = BiCGstab(l) with l = 2 (Fokkema's enhanced implementation without reliable updates),
 * src/iterative.c:340-487: r_0..2 in r, v1, v3; u_0..2 in v2, Av, v4; r~0 in p */
typedef struct {
	cplx rho0, alpha;
} bcgs2_state;

static int bcgs2_iter(solver *s, bcgs2_state *b)
{
	const size_t n = s->n;
	cplx *r[3] = {s->r, s->v1, s->v3}, *u[3] = {s->v2, s->Av, s->v4};
	const cplx *rt = s->p;
	cplx rho1, beta, sigma;
	for (int j = 0; j < 2; j++) {
		rho1 = ndot(r[j], rt, n);
		if (s->niter == 1 && j == 0) memcpy(u[0], r[0], sizeof(cplx) * n);
		else {
			if (cabs(b->rho0) / (cabs(rho1) * cabs(b->alpha)) < 1e-10) return OR_EBREAKDOWN;
			beta = b->alpha * rho1 / b->rho0;
			cplx mb = -beta;
			for (int i = 0; i <= j; i++)
				for (size_t k = 0; k < n; k++) u[i][k] = mb * u[i][k] + r[i][k];
		}
		b->rho0 = rho1;
		if (!(s->niter == 1 && j == 0 && s->matvec_ready)) mv(s, u[j], u[j + 1], NULL);
		sigma = ndot(u[j + 1], rt, n);
		if (cabs(sigma) / cabs(rho1) < 1e-10) return OR_EBREAKDOWN;
		b->alpha = rho1 / sigma;
		for (size_t k = 0; k < n; k++) s->x[k] += b->alpha * u[0][k];
		cplx ma = -b->alpha;
		for (int i = 0; i <= j; i++)
			for (size_t k = 0; k < n; k++) r[i][k] += ma * u[i + 1][k];
		mv(s, r[j], r[j + 1], NULL);
	}
	// convex polynomial part: Z = R'R (Z[i][j] = r_j . conj(r_i))
	cplx Z[3][3], y0[3], yl[3], zy0[3], zyl[3];
	for (int i = 0; i <= 2; i++)
		for (int j = 0; j <= i; j++) {
			Z[i][j] = ndot(r[j], r[i], n);
			if (i != j) Z[j][i] = conj(Z[i][j]);
		}
	y0[0] = -1; y0[1] = Z[1][0] / Z[1][1]; y0[2] = 0;
	yl[0] = 0; yl[1] = Z[1][2] / Z[1][1]; yl[2] = -1;
	for (int i = 0; i <= 2; i++) {
		zy0[i] = zyl[i] = 0;
		for (int j = 0; j <= 2; j++) {
			zy0[i] += Z[i][j] * y0[j];
			zyl[i] += Z[i][j] * yl[j];
		}
	}
	double d = 0;
	for (int i = 0; i <= 2; i++) d += creal(zy0[i] * conj(y0[i]));
	const double kappa0 = sqrt(d);
	d = 0;
	for (int i = 0; i <= 2; i++) d += creal(zyl[i] * conj(yl[i]));
	const double kappal = sqrt(d);
	cplx varrho = 0;
	for (int i = 0; i <= 2; i++) varrho += zy0[i] * conj(yl[i]);
	varrho /= kappa0 * kappal;
	d = cabs(varrho);
	cplx hatgamma = varrho * (d > 0.7 ? d : 0.7) / d;
	cplx t = -hatgamma * kappa0 / kappal;
	for (int i = 0; i <= 2; i++) y0[i] += t * yl[i];
	const cplx omega = y0[2];
	for (int i = 1; i <= 2; i++) {
		cplx m = -y0[i];
		for (size_t k = 0; k < n; k++) u[0][k] += m * u[i][k];
		for (size_t k = 0; k < n; k++) s->x[k] += y0[i] * r[i - 1][k];
		for (size_t k = 0; k < n; k++) r[0][k] += m * r[i][k];
	}
	for (int i = 0; i <= 2; i++) {
		zy0[i] = 0;
		for (int j = 0; j <= 2; j++) zy0[i] += Z[i][j] * y0[j];
	}
	s->inprodRp1 = 0;
	for (int i = 0; i <= 2; i++) s->inprodRp1 += creal(zy0[i] * conj(y0[i]));
	b->rho0 *= -omega;
	return OR_OK;
}

/* ---------------- checkpoints, src/iterative.c:165-278 ----------------
 * File layout (native byte order, fields back to back): int ind_m (index of the method in the reference's params
 * table, iterative.c:118-125), size_t local_nRows, int niter, int counter, double inprodR, double prev_err,
 * double resid_scale, the method's scalars, then xvec, rvec, pvec and the method's vectors (local_nRows complex
 * doubles each). The reference stores buffers, not roles: QMR_CS and CSYM swap their vector pointers every
 * iteration, so which buffer holds which vector follows from the parity of niter (the pointer swaps on load,
 * iterative.c:809-812,935-938). */
typedef struct {
	unsigned char *buf;
	size_t cap, len;
} chp_w;
typedef struct {
	const unsigned char *buf;
	size_t len, pos;
	int bad;
} chp_r;

static void chp_put(chp_w *w, const void *p, size_t n)
{
	if (w->buf && w->len + n <= w->cap) memcpy(w->buf + w->len, p, n);
	w->len += n;
}

static void chp_get(chp_r *r, void *p, size_t n)
{
	if (r->pos + n > r->len) {
		r->bad = 1;
		memset(p, 0, n);
	}
	else memcpy(p, r->buf + r->pos, n);
	r->pos += n;
}

// index in the reference's params table (alphabetical: BCGS2, BiCG_CS, BiCGStab, CGNR, CSYM, QMR_CS, QMR_CS_2)
static const int chp_ind[7] = {5, 2, 1, 3, 4, 6, 0};

typedef struct {
	cplx *rvec, *pvec, *vec[3];
	int nvec;
} chp_roles;

/* buffers in the reference's order for the state before iteration niter */
static chp_roles chp_layout(solver *S, int method, qmr_state *q, bcgs_state *bs, csym_state *cs)
{
	chp_roles L;
	memset(&L, 0, sizeof(L));
	L.rvec = S->r;
	L.pvec = S->p;
	const int odd = S->niter & 1;
	switch (method) {
		case OR_QMR_CS: // v=vec1, vtilda=vec2 for odd niter, swapped for even; p_new=vec3, p_old=pvec for odd
			L.pvec = odd ? q->po : q->pn;
			L.vec[0] = odd ? q->v : q->vt;
			L.vec[1] = odd ? q->vt : q->v;
			L.vec[2] = odd ? q->pn : q->po;
			L.nvec = 3;
			break;
		case OR_BICGSTAB:
			L.vec[0] = bs->v;
			L.vec[1] = bs->sv;
			L.vec[2] = bs->rt;
			L.nvec = 3;
			break;
		case OR_CSYM: // q_new=rvec, q_old=vec1 for odd niter, swapped for even; p_new=vec2, p_old=pvec for odd
			L.rvec = odd ? cs->q_new : cs->q_old;
			L.vec[0] = odd ? cs->q_old : cs->q_new;
			L.pvec = odd ? cs->p_old : cs->p_new;
			L.vec[1] = odd ? cs->p_new : cs->p_old;
			L.nvec = 2;
			break;
		case OR_QMR_CS_2:
			L.vec[0] = S->v1; // v
			L.vec[1] = S->v2; // d
			L.nvec = 2;
			break;
		case OR_BCGS2:
			L.vec[0] = S->v2; // u[0]; pvec holds r~0
			L.nvec = 1;
			break;
		default: break; // BiCG_CS, CGNR: p in pvec only
	}
	return L;
}

/* the method's scalars in the order of its PHASE_VARS (iterative.c:383-386,520-521,661-664,741-742,796-803,
 * 919-928,1060-1066); dir = 0 writes, 1 reads */
static void chp_scalars(void *io, int dir, int method, qmr_state *q, bcgs_state *bs, csym_state *cs,
	qmr2_state *q2, bcgs2_state *b2, cplx *ro_c, double *ro_d)
{
#define CHP_IO(v) (dir ? chp_get((chp_r *)io, &(v), sizeof(v)) : chp_put((chp_w *)io, &(v), sizeof(v)))
	switch (method) {
		case OR_QMR_CS:
			CHP_IO(q->om_old); CHP_IO(q->om_new); CHP_IO(q->c_old); CHP_IO(q->c_new);
			CHP_IO(q->beta); CHP_IO(q->tautilda); CHP_IO(q->s_old); CHP_IO(q->s_new);
			break;
		case OR_BICGSTAB: CHP_IO(bs->ro_old); CHP_IO(bs->omega); CHP_IO(bs->alpha); break;
		case OR_BICG_CS: CHP_IO(*ro_c); break;
		case OR_CGNR: CHP_IO(*ro_d); break;
		case OR_CSYM:
			CHP_IO(cs->beta); CHP_IO(cs->c_old); CHP_IO(cs->c_new); CHP_IO(cs->tau); CHP_IO(cs->s_old);
			CHP_IO(cs->s_new);
			break;
		case OR_QMR_CS_2:
			CHP_IO(q2->c_old); CHP_IO(q2->theta_old); CHP_IO(q2->ro_old); CHP_IO(q2->eps); CHP_IO(q2->eta);
			break;
		default: CHP_IO(b2->rho0); CHP_IO(b2->alpha); break;
	}
#undef CHP_IO
}

/* IterativeSolver, src/iterative.c:1398-1530 with CalcInitField (:1342-1394) and ProgressReport (:282-318).
 * einc: incident field [N][3]; xvec receives x, pvec the polarisations S.x; resid_hist[0..] the relative residuals
 * RE_000, RE_001, ... (at most hist_cap values). Returns a status code; *niter_out = iterations performed. */
int or_solve(or_ctx *c, int method, const double *einc, double eps, int maxiter, int init_field,
	double *xvec, double *pvec, double *resid_hist, int hist_cap, int *niter_out)
{
	return or_solve_chp(c, method, einc, eps, maxiter, init_field, xvec, pvec, resid_hist, hist_cap, niter_out, NULL,
		0, NULL, NULL);
}

int or_solve_chp(or_ctx *c, int method, const double *einc, double eps, int maxiter, int init_field,
	double *xvec, double *pvec, double *resid_hist, int hist_cap, int *niter_out, const void *chp_in,
	size_t chp_in_len, void *chp_out, size_t *chp_out_len)
{
	solver S;
	memset(&S, 0, sizeof(S));
	S.c = c;
	S.n = 3 * c->n;
	const size_t n = S.n;
	const cplx *E = (const cplx *)einc;
	S.x = (cplx *)xvec;
	cplx *b = (cplx *)pvec;
	S.r = malloc(sizeof(cplx) * n);
	S.p = malloc(sizeof(cplx) * n);
	S.Av = malloc(sizeof(cplx) * n);
	S.v1 = malloc(sizeof(cplx) * n);
	S.v2 = malloc(sizeof(cplx) * n);
	S.v3 = malloc(sizeof(cplx) * n);
	S.v4 = malloc(sizeof(cplx) * n);
	S.full = chp_out != NULL;
	// b = S.Einc (nMult_mat)
	for (size_t i = 0; i < c->n; i++)
		for (int a = 0; a < 3; a++) b[3 * i + a] = ccs_of(c, i, a) * E[3 * i + a];
	double temp = nnorm2(b, n);
	double resid_scale = 1 / temp;
	S.epsB = eps * eps * temp;
	if (chp_in) {
		/* LoadIterChpoint replaces CalcInitField and the method's PHASE_INIT */
	}
	else if (init_field == OR_IF_ZERO) {
		memset(S.x, 0, sizeof(cplx) * n);
		memcpy(S.r, b, sizeof(cplx) * n);
		S.inprodR = temp;
	}
	else if (init_field == OR_IF_X0) { // x_0 from the caller: InitFieldfromE, iterative.c:1335-1337
		mv(&S, S.x, S.Av, NULL);
		double ip = 0;
		for (size_t i = 0; i < n; i++) {
			S.r[i] = b[i] - S.Av[i];
			ip += creal(S.r[i]) * creal(S.r[i]) + cimag(S.r[i]) * cimag(S.r[i]);
		}
		S.inprodR = ip;
	}
	else {
		mv(&S, b, S.Av, NULL);
		double ip = 0;
		for (size_t i = 0; i < n; i++) {
			S.r[i] = b[i] - S.Av[i];
			ip += creal(S.r[i]) * creal(S.r[i]) + cimag(S.r[i]) * cimag(S.r[i]);
		}
		S.inprodR = ip;
		if (init_field == OR_IF_AUTO && temp < S.inprodR) {
			memset(S.x, 0, sizeof(cplx) * n);
			memcpy(S.r, b, sizeof(cplx) * n);
			S.inprodR = temp;
			S.matvec_ready = 1;
		}
		else memcpy(S.x, b, sizeof(cplx) * n);
	}
	int nh = 0;
	double prev_err = sqrt(resid_scale * S.inprodR);
	S.niter = 1;
	S.counter = 0;
	// stagnation limits per method (iterative.c:118-125)
	const int mcm = (method == OR_BICGSTAB) ? 30000 : (method == OR_CGNR || method == OR_CSYM) ? 10
		: (method == OR_BCGS2) ? 15000 : 50000;
	qmr_state q;
	bcgs_state bs;
	csym_state cs;
	qmr2_state q2;
	bcgs2_state b2 = {-1, 0};
	cplx ro_c = 0;
	double ro_d = 0;
	bs.v = S.v1; bs.sv = S.v2; bs.rt = S.v3;
	q.v = S.v1; q.vt = S.v2; q.pn = S.p; q.po = S.v3;
	cs.q_new = S.r; cs.q_old = S.v1; cs.p_new = S.p; cs.p_old = S.v2;
	if (chp_in) {
		chp_r R = {chp_in, chp_in_len, 0, 0};
		int ind;
		size_t rows;
		chp_get(&R, &ind, sizeof(ind));
		chp_get(&R, &rows, sizeof(rows));
		if (R.bad || ind != chp_ind[method] || rows != n) {
			free(S.r); free(S.p); free(S.Av); free(S.v1); free(S.v2); free(S.v3); free(S.v4);
			return -1; // "is for different iterative method" / "different vector size" (iterative.c:238-241)
		}
		chp_get(&R, &S.niter, sizeof(int));
		chp_get(&R, &S.counter, sizeof(int));
		chp_get(&R, &S.inprodR, sizeof(double));
		chp_get(&R, &prev_err, sizeof(double));
		chp_get(&R, &resid_scale, sizeof(double));
		chp_scalars(&R, 1, method, &q, &bs, &cs, &q2, &b2, &ro_c, &ro_d);
		S.epsB = eps * eps / resid_scale;
		chp_roles L = chp_layout(&S, method, &q, &bs, &cs);
		chp_get(&R, S.x, sizeof(cplx) * n);
		chp_get(&R, L.rvec, sizeof(cplx) * n);
		chp_get(&R, L.pvec, sizeof(cplx) * n);
		for (int v = 0; v < L.nvec; v++) chp_get(&R, L.vec[v], sizeof(cplx) * n);
		if (R.bad || R.pos != R.len) { // "Failed reading" / "is too long" (iterative.c:258-266)
			free(S.r); free(S.p); free(S.Av); free(S.v1); free(S.v2); free(S.v3); free(S.v4);
			return -1;
		}
	}
	else if (method == OR_QMR_CS) qmr_init(&S, &q);
	else if (method == OR_BICGSTAB) memcpy(bs.rt, S.r, sizeof(cplx) * n);
	else if (method == OR_CSYM) csym_init(&S, &cs);
	else if (method == OR_QMR_CS_2) qmr2_init(&S, &q2);
	else if (method == OR_BCGS2) memcpy(S.p, S.r, sizeof(cplx) * n); // r~0 = r_0, rho0 = -1
	if (nh < hist_cap) resid_hist[nh++] = prev_err;
	int status = OR_OK;
	while (S.inprodR > S.epsB && S.niter <= maxiter && S.counter <= mcm) {
		S.complete = 1;
		switch (method) {
			case OR_QMR_CS: status = qmr_iter(&S, &q); break;
			case OR_BICGSTAB: status = bcgs_iter(&S, &bs); break;
			case OR_BICG_CS: status = bicg_iter(&S, &ro_c); break;
			case OR_CGNR: status = cgnr_iter(&S, &ro_d); break;
			case OR_QMR_CS_2: status = qmr2_iter(&S, &q2); break;
			case OR_BCGS2: status = bcgs2_iter(&S, &b2); break;
			default: status = csym_iter(&S, &cs); break;
		}
		if (status != OR_OK) break;
		if (S.inprodRp1 <= S.inprodR) {
			S.inprodR = S.inprodRp1;
			S.counter = 0;
		}
		else S.counter++;
		prev_err = sqrt(resid_scale * S.inprodRp1);
		if (nh < hist_cap) resid_hist[nh++] = prev_err;
		S.niter++;
	}
	if (chp_out_len && status == OR_OK) { // SaveIterChpoint after the loop (-chp_type always, iterative.c:1498)
		chp_w W = {chp_out, *chp_out_len, 0};
		int ind = chp_ind[method];
		size_t rows = n;
		chp_put(&W, &ind, sizeof(ind));
		chp_put(&W, &rows, sizeof(rows));
		chp_put(&W, &S.niter, sizeof(int));
		chp_put(&W, &S.counter, sizeof(int));
		chp_put(&W, &S.inprodR, sizeof(double));
		chp_put(&W, &prev_err, sizeof(double));
		chp_put(&W, &resid_scale, sizeof(double));
		chp_scalars(&W, 0, method, &q, &bs, &cs, &q2, &b2, &ro_c, &ro_d);
		chp_roles L = chp_layout(&S, method, &q, &bs, &cs);
		chp_put(&W, S.x, sizeof(cplx) * n);
		chp_put(&W, L.rvec, sizeof(cplx) * n);
		chp_put(&W, L.pvec, sizeof(cplx) * n);
		for (int v = 0; v < L.nvec; v++) chp_put(&W, L.vec[v], sizeof(cplx) * n);
		*chp_out_len = W.len;
	}
	if (status == OR_OK && S.inprodR > S.epsB) status = (S.niter > maxiter) ? OR_EMAXITER : OR_ESTAGNATION;
	for (size_t i = 0; i < c->n; i++)
		for (int a = 0; a < 3; a++) b[3 * i + a] = ccs_of(c, i, a) * S.x[3 * i + a];
	if (niter_out) *niter_out = S.niter - 1;
	free(S.r); free(S.p); free(S.Av); free(S.v1); free(S.v2); free(S.v3); free(S.v4);
	return status;
}

/* ExtCross (plane wave, free space) via CalcFieldFree, src/crosssec.c:506-596, 811-822; AbsCross (Draine),
 * src/crosssec.c:852-917. Positions are taken relative to the first dipole of the box, whose centre is at
 * box_origin = -gridspace*((boxX-1)/2, (boxY-1)/2, (boxZ-1)/2) (make_particle.c:2305-2308). */
/* CalcFieldFree, src/crosssec.c:506-596: scattering amplitude ebuff = (-i k^3) exp(-ik r0.n) (I - nn).sum_j P_j
 * exp(-i kd n.pos_j) for the direction n (unit vector), with r0 the box origin (make_particle.c:2305-2308) */
void or_field(const or_ctx *c, const double *pvec, const double n[3], double *ebuff)
{
	const cplx *P = (const cplx *)pvec;
	const double kd = c->k * c->gridspace;
	cplx sum[3] = {0, 0, 0};
	for (size_t j = 0; j < c->n; j++) {
		double ph = -kd * (n[0] * c->pos[3 * j] + n[1] * c->pos[3 * j + 1] + n[2] * c->pos[3 * j + 2]);
		cplx a = cos(ph) + I * sin(ph);
		for (int i = 0; i < 3; i++) sum[i] += P[3 * j + i] * a;
	}
	cplx dpr = sum[0] * n[0] + sum[1] * n[1] + sum[2] * n[2];
	double r0[3] = {-c->gridspace * (c->bX - 1) / 2.0, -c->gridspace * (c->bY - 1) / 2.0,
		-c->gridspace * (c->bZ - 1) / 2.0};
	double ph0 = -c->k * (r0[0] * n[0] + r0[1] * n[1] + r0[2] * n[2]);
	cplx amp = -I * (cos(ph0) + I * sin(ph0)) * (c->k * c->k * c->k);
	cplx *e = (cplx *)ebuff;
	for (int i = 0; i < 3; i++) e[i] = amp * (sum[i] - dpr * n[i]);
}

/* ExtCross (plane wave, free space) via CalcField in the propagation direction, src/crosssec.c:811-822; AbsCross
 * (Draine), src/crosssec.c:852-917 */
void or_cross(or_ctx *c, const double *pvec, const double prop[3], const double incpol[3], double *cext,
	double *cabs)
{
	const cplx *P = (const cplx *)pvec;
	cplx e[3];
	or_field(c, pvec, prop, (double *)e);
	double s = 0;
	for (int i = 0; i < 3; i++) s += creal(e[i] * incpol[i]);
	*cext = s * 4 * M_PI / (c->k * c->k);
	const double t1 = 2 * c->k * c->k * c->k / 3;
	double sa = 0;
	for (size_t j = 0; j < c->n; j++)
		for (int i = 0; i < 3; i++) {
			double mult = -cimag(1 / cc_of(c, j, i)) - t1;
			cplx p = P[3 * j + i];
			sa += mult * (creal(p) * creal(p) + cimag(p) * cimag(p));
		}
	*cabs = 4 * M_PI * c->k * sa;
}

/* ExtCross for a general incident field (the branch taken in surface mode), src/crosssec.c:823-845:
 * Cext = 4 pi k sum_j Im(P_j . conj(Einc_j)), times inc_scale (1/Re(msub) for a beam from the substrate, 1 otherwise,
 * GenerateB.c:104,117); AbsCross (Draine) times the same factor, src/crosssec.c:852-917 */
void or_cross_beam(or_ctx *c, const double *pvec, const double *einc, double inc_scale, double *cext, double *cabs)
{
	const cplx *P = (const cplx *)pvec, *E = (const cplx *)einc;
	double s = 0;
	for (size_t j = 0; j < 3 * c->n; j++) s += cimag(P[j]) * creal(E[j]) - creal(P[j]) * cimag(E[j]);
	*cext = s * 4 * M_PI * c->k * inc_scale;
	const double t1 = 2 * c->k * c->k * c->k / 3;
	double sa = 0;
	for (size_t j = 0; j < c->n; j++)
		for (int i = 0; i < 3; i++) {
			double mult = -cimag(1 / cc_of(c, j, i)) - t1;
			cplx p = P[3 * j + i];
			sa += mult * (creal(p) * creal(p) + cimag(p) * cimag(p));
		}
	*cabs = 4 * M_PI * c->k * sa * inc_scale;
}
