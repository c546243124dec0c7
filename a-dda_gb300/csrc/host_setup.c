/* host_setup.c - host-side inputs of the DDA hot path: particle lattice, incident plane wave, polarisabilities.
 *
 * These are the data the reference's C host hands to the FFT matvec and the iterative solver. They are restated here
 * so that a caller without the reference host (the tests, bench.py, other front ends) can build the same inputs:
 *   adda_gb300_fit_box          <- FitBox / FitBox_yz + InitShape sizing    src/make_particle.c:1283-1308, 1912-1919
 *   adda_gb300_make_particle    <- MakeParticle box loop                    src/make_particle.c:1984-2230
 *   adda_gb300_rotation         <- InitRotation (zyz Euler angles)          src/crosssec.c:82-139
 *   adda_gb300_plane_wave       <- GenerateB, free-space plane wave         src/GenerateB.c:324-328
 *   adda_gb300_plane_wave_surf  <- GenerateB, plane wave near a substrate   src/GenerateB.c:96-140, 257-323
 *   adda_gb300_polarizability   <- CoupleConstant (CM, LDR, RRC, DGF)        src/calculator.c:100-262
 *   adda_gb300_read_int_tables  <- ReadTables / ReadTableFile                src/interaction.c:1004-1063
 * All functions are pure host code: no GPU is touched.
 */
#include "adda_gb300.h"

#include <complex.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define TWO_PI_D 6.283185307179586476925286766559
#define FOUR_PI_D 12.566370614359172953850573533118

int adda_gb300_fit_box(int shape, const double *pars, int boxX, int *boxY, int *boxZ)
{
	double yx = 1, zx = 1;
	switch (shape) {
		case ADDA_SHAPE_SPHERE: break;
		case ADDA_SHAPE_ELLIPSOID:
		case ADDA_SHAPE_BOX:
			if (pars) { yx = pars[0]; zx = pars[1]; }
			break;
		default: return ADDA_GB300_EINVAL;
	}
	if (boxX < 1 || boxX % 2) return ADDA_GB300_EINVAL;
	/* FitBox_yz with jagged=1: 2*floor((size+1)/2) */
	*boxY = 2 * (int)floor((yx * boxX + 1) / 2);
	*boxZ = 2 * (int)floor((zx * boxX + 1) / 2);
	if (*boxY < 2) *boxY = 2;
	if (*boxZ < 2) *boxZ = 2;
	return ADDA_GB300_OK;
}

size_t adda_gb300_make_particle(int shape, const double *pars, int boxX, int boxY, int boxZ, uint16_t *position,
	uint8_t *material)
{
	double invsqY = 1, invsqZ = 1, haspY = 0.5, haspZ = 0.5;
	if (shape == ADDA_SHAPE_ELLIPSOID && pars) {
		invsqY = 1 / (pars[0] * pars[0]);
		invsqZ = 1 / (pars[1] * pars[1]);
	}
	if (shape == ADDA_SHAPE_BOX && pars) {
		haspY = pars[0] / 2;
		haspZ = pars[1] / 2;
	}
	size_t idx = 0;
	/* loop order z, y, x (x fastest), as in the reference: dipoles on one x-line are consecutive */
	for (int k = 0; k < boxZ; k++)
		for (int j = 0; j < boxY; j++)
			for (int i = 0; i < boxX; i++) {
				/* jagged=1: centre of cell relative to the box centre, scaled by boxX */
				double xr = (i - boxX / 2 + 0.5) / boxX;
				double yr = (j - boxY / 2 + 0.5) / boxX;
				double zr = (k - boxZ / 2 + 0.5) / boxX;
				int in = 0;
				switch (shape) {
					case ADDA_SHAPE_SPHERE: in = (xr * xr + yr * yr + zr * zr <= 0.25); break;
					case ADDA_SHAPE_ELLIPSOID: in = (xr * xr + yr * yr * invsqY + zr * zr * invsqZ <= 0.25); break;
					case ADDA_SHAPE_BOX: in = (fabs(yr) <= haspY && fabs(zr) <= haspZ); break;
					default: return 0;
				}
				if (!in) continue;
				if (position) {
					position[3 * idx] = (uint16_t)i;
					position[3 * idx + 1] = (uint16_t)j;
					position[3 * idx + 2] = (uint16_t)k;
				}
				if (material) material[idx] = 0;
				idx++;
			}
	return idx;
}

void adda_gb300_rotation(const double prop0_in[3], double alpha_deg, double beta_deg, double gamma_deg,
	double prop[3], double incPolY[3], double incPolX[3])
{
	/* laboratory frame (param.c:1988-1989, 2116-2131): prop_0 = (0,0,1) unless given (-prop, normalised), and the
	 * two incident polarisations derived from it */
	double p0[3] = {0, 0, 1}, y0[3], x0[3];
	if (prop0_in) {
		double nn = prop0_in[0] * prop0_in[0] + prop0_in[1] * prop0_in[1] + prop0_in[2] * prop0_in[2];
		for (int i = 0; i < 3; i++) p0[i] = prop0_in[i] / sqrt(nn);
	}
	if (fabs(p0[0]) < 1e-15 && fabs(p0[1]) < 1e-15) { // along z (vAlongZ, cmplx.h:501-505; ROUND_ERR)
		x0[0] = copysign(1.0, p0[2]);
		x0[1] = x0[2] = 0;
		y0[0] = y0[2] = 0;
		y0[1] = 1;
	}
	else {
		double t = sqrt(1 - p0[2] * p0[2]);
		x0[0] = p0[0] * p0[2] / t;
		x0[1] = p0[1] * p0[2] / t;
		x0[2] = -t;
		y0[0] = -p0[1] / t;
		y0[1] = p0[0] / t;
		y0[2] = 0;
	}
	/* InitRotation: zyz Euler matrix applied to prop_0, incPolY_0, incPolX_0 */
	const double d2r = TWO_PI_D / 360;
	double a = alpha_deg * d2r, b = beta_deg * d2r, g = gamma_deg * d2r;
	double ca = cos(a), sa = sin(a), cb = cos(b), sb = sin(b), cg = cos(g), sg = sin(g);
	double m[3][3] = {
		{ca * cb * cg - sa * sg, sa * cb * cg + ca * sg, -sb * cg},
		{-ca * cb * sg - sa * cg, -sa * cb * sg + ca * cg, sb * sg},
		{ca * sb, sa * sb, cb}};
	for (int i = 0; i < 3; i++) {
		prop[i] = m[i][0] * p0[0] + m[i][1] * p0[1] + m[i][2] * p0[2];
		incPolY[i] = m[i][0] * y0[0] + m[i][1] * y0[1] + m[i][2] * y0[2];
		incPolX[i] = m[i][0] * x0[0] + m[i][1] * x0[1] + m[i][2] * x0[2];
	}
}

void adda_gb300_plane_wave(size_t ndip, const uint16_t *position, int boxX, int boxY, int boxZ, double gridspace,
	double wavenum, const double prop[3], const double pol[3], double *einc)
{
	const double cX = (boxX - 1) / 2.0, cY = (boxY - 1) / 2.0, cZ = (boxZ - 1) / 2.0;
	for (size_t i = 0; i < ndip; i++) {
		double r0 = (position[3 * i] - cX) * gridspace;
		double r1 = (position[3 * i + 1] - cY) * gridspace;
		double r2 = (position[3 * i + 2] - cZ) * gridspace;
		double ph = wavenum * (r0 * prop[0] + r1 * prop[1] + r2 * prop[2]);
		double c = cos(ph), s = sin(ph);
		for (int a = 0; a < 3; a++) {
			einc[6 * i + 2 * a] = c * pol[a];
			einc[6 * i + 2 * a + 1] = s * pol[a];
		}
	}
}

/* normal component of the transmitted wavevector with the branch cut on the negative real axis handled explicitly
 * (cSqrtCut, src/cmplx.h:58-80) */
static double complex sqrt_cut(double complex a)
{
	if (cimag(a) == 0) return creal(a) >= 0 ? sqrt(creal(a)) : I * sqrt(-creal(a));
	return csqrt(a);
}

int adda_gb300_plane_wave_surf(size_t ndip, const uint16_t *position, int boxX, int boxY, int boxZ,
	double gridspace, double wavenum, const double prop[3], const double incPolY[3], const double incPolX[3],
	int which, double hsub, double msub_re, double msub_im, int msub_inf, double *einc, double *inc_scale)
{
	const double round_err = 1e-15, sqrt_rnd_err = 3e-8; // const.h:337-338
	if (prop[2] == 0 || (msub_inf && prop[2] > 0) || (which != 0 && which != 1)) return ADDA_GB300_EINVAL;
	const double complex msub = msub_re + I * msub_im;
	const double cX = (boxX - 1) / 2.0, cY = (boxY - 1) / 2.0, cZ = (boxZ - 1) / 2.0;
	const double k = wavenum;
	// beam frame: ex = the incident polarisation, ey completes it (GenerateB.c:245-252)
	double ex[3], ey[3];
	for (int a = 0; a < 3; a++) {
		ex[a] = which == 0 ? incPolY[a] : incPolX[a];
		ey[a] = which == 0 ? -incPolX[a] : incPolY[a];
	}
	const double tr2 = prop[0] * prop[0] + prop[1] * prop[1];
	double complex eRefl[3], eTran[3], ktVec[3] = {0, 0, 0}, ki, kt = 0;
	if (prop[2] > 0) { // from the substrate (below): only the transmitted wave reaches the particle
		*inc_scale = 1 / msub_re;
		ki = msub * prop[2];
		kt = (cabs(msub - 1) < round_err && cabs(ki) < sqrt_rnd_err) ? ki : sqrt_cut(1 - msub * msub * tr2);
		ktVec[0] = msub * prop[0];
		ktVec[1] = msub * prop[1];
		ktVec[2] = kt;
		double complex tc;
		if (which == 0) { // s-polarised: FresnelTS
			for (int a = 0; a < 3; a++) eTran[a] = ex[a];
			tc = 2 * ki / (ki + kt);
		}
		else { // p-polarised: eTran = ey x ktVec, FresnelTP with mr = 1/msub
			eTran[0] = ey[1] * ktVec[2] - ey[2] * ktVec[1];
			eTran[1] = ey[2] * ktVec[0] - ey[0] * ktVec[2];
			eTran[2] = ey[0] * ktVec[1] - ey[1] * ktVec[0];
			const double complex mr = 1 / msub;
			tc = 2 * mr * ki / (mr * mr * ki + kt);
		}
		const double complex f = tc * cexp(I * k * (kt - ki) * hsub);
		for (int a = 0; a < 3; a++) eTran[a] *= f;
		for (size_t i = 0; i < ndip; i++) {
			const double r[3] = {(position[3 * i] - cX) * gridspace, (position[3 * i + 1] - cY) * gridspace,
				(position[3 * i + 2] - cZ) * gridspace};
			const double complex ph = cexp(I * k * (ktVec[0] * r[0] + ktVec[1] * r[1] + ktVec[2] * r[2]));
			for (int a = 0; a < 3; a++) {
				const double complex v = ph * eTran[a];
				einc[6 * i + 2 * a] = creal(v);
				einc[6 * i + 2 * a + 1] = cimag(v);
			}
		}
		return ADDA_GB300_OK;
	}
	// from above: the incident wave plus the wave reflected by the substrate
	*inc_scale = 1;
	const double prRefl[3] = {prop[0], prop[1], -prop[2]};
	ki = -prop[2];
	if (!msub_inf) kt = (cabs(msub - 1) < round_err && fabs(creal(ki)) < sqrt_rnd_err) ? ki
		: sqrt_cut(msub * msub - tr2);
	double complex rc;
	if (which == 0) { // s-polarised: FresnelRS
		for (int a = 0; a < 3; a++) eRefl[a] = ex[a];
		rc = msub_inf ? -1 : (ki - kt) / (ki + kt);
	}
	else { // p-polarised: ex reflected about the z axis, FresnelRP with mr = msub
		eRefl[0] = -ex[0];
		eRefl[1] = -ex[1];
		eRefl[2] = ex[2];
		rc = msub_inf ? 1 : (msub * msub * ki - kt) / (msub * msub * ki + kt);
	}
	const double ph2 = 2 * k * creal(ki) * hsub;
	const double complex f = rc * (cos(ph2) + I * sin(ph2));
	for (int a = 0; a < 3; a++) eRefl[a] *= f;
	for (size_t i = 0; i < ndip; i++) {
		const double r[3] = {(position[3 * i] - cX) * gridspace, (position[3 * i + 1] - cY) * gridspace,
			(position[3 * i + 2] - cZ) * gridspace};
		const double p1 = k * (r[0] * prop[0] + r[1] * prop[1] + r[2] * prop[2]);
		const double p2 = k * (r[0] * prRefl[0] + r[1] * prRefl[1] + r[2] * prRefl[2]);
		const double complex e1 = cos(p1) + I * sin(p1), e2 = cos(p2) + I * sin(p2);
		for (int a = 0; a < 3; a++) {
			const double complex v = e1 * ex[a] + e2 * eRefl[a];
			einc[6 * i + 2 * a] = creal(v);
			einc[6 * i + 2 * a + 1] = cimag(v);
		}
	}
	return ADDA_GB300_OK;
}

/* polCM, polM, polMplusRR, pol3coef: src/calculator.c:100-132 */
static double complex pol_cm(double complex m, double dipvol)
{
	double complex m2 = m * m;
	return (3 / FOUR_PI_D) * dipvol * (m2 - 1) / (m2 + 2);
}

static double complex pol_m(double complex M, double complex m, double dipvol)
{
	double complex cm = pol_cm(m, dipvol);
	return cm / (1 - (cm / dipvol) * M);
}

static double complex pol_rr(double complex M, double complex m, double kd, double dipvol)
{
	return pol_m(M + I * 2 * kd * kd * kd / 3, m, dipvol);
}

/* coefficients of the lattice-dispersion-type prescriptions, M = (b1 + (b2 + b3 S) m^2) kd^2 (const.h:234-241):
 * LDR (Draine & Goodman) and the second-order (SO) formulation of Gutkowicz-Krusin & Draine */
#define LDR_B1 1.8915316
#define LDR_B2 (-0.1648469)
#define LDR_B3 1.7700004
#define SO_B1 1.5867182426530356710958782335228
#define SO_B2 0.13488017286410948123541594310740
#define SO_B3 0.11895825700597042937085940122438
#define DGF_B1 1.6119919540164696407169668466385 /* (4pi/3)^(1/3) */
#define LAK_C 0.62035049089940001666800681204778  /* (4pi/3)^(-1/3) */

/* sum_i prop_i^2 e_i^2 (LDR's S, calculator.c:214-222), or its orientation average */
static double ldr_s(const double prop[3], const double incPol[3], int avgpol)
{
	if (avgpol)
		return 0.5 * (1 - (prop[0] * prop[0] * prop[0] * prop[0] + prop[1] * prop[1] * prop[1] * prop[1] +
						  prop[2] * prop[2] * prop[2] * prop[2]));
	return prop[0] * prop[0] * incPol[0] * incPol[0] + prop[1] * prop[1] * incPol[1] * incPol[1] +
		prop[2] * prop[2] * incPol[2] * incPol[2];
}

int adda_gb300_polarizability(int relation, double m_re, double m_im, double kd, double gridspace,
	const double prop[3], const double incPol[3], int avgpol, double cc[6])
{
	const double dipvol = gridspace * gridspace * gridspace;
	const double complex m = m_re + I * m_im;
	const double kd2 = kd * kd;
	double complex r[3];
	switch (relation) {
		case ADDA_POL_CM: r[0] = pol_cm(m, dipvol); break;
		case ADDA_POL_RRC: r[0] = pol_rr(0, m, kd, dipvol); break;
		case ADDA_POL_DGF: r[0] = pol_rr(DGF_B1 * kd2, m, kd, dipvol); break;
		case ADDA_POL_LDR:
			r[0] = pol_rr((LDR_B1 + (LDR_B2 + LDR_B3 * ldr_s(prop, incPol, avgpol)) * m * m) * kd2, m, kd, dipvol);
			break;
		case ADDA_POL_FCD: /* M0 = (4/3)kd^2 + (2/(3pi)) log((pi-kd)/(pi+kd)) kd^3 (calculator.c:206-208) */
			r[0] = pol_rr(2.0 / 3 * kd2 * (2 + kd / M_PI * log((M_PI - kd) / (M_PI + kd))), m, kd, dipvol);
			break;
		case ADDA_POL_IGT_SO: r[0] = pol_rr(SO_B1 * kd2, m, kd, dipvol); break;
		case ADDA_POL_LAK: { /* M = (8pi/3)[(1-ika)exp(ika)-1], a = (4pi/3)^(-1/3) d (calculator.c:210-213) */
			const double ka = LAK_C * kd;
			r[0] = pol_m(2 * FOUR_PI_D / 3 * ((1 - I * ka) * cexp(I * ka) - 1), m, dipvol);
			break;
		}
		case ADDA_POL_CLDR: /* per component, S_i = prop_i^2 (calculator.c:196) */
			for (int a = 0; a < 3; a++)
				r[a] = pol_rr((LDR_B1 + (LDR_B2 + LDR_B3 * prop[a] * prop[a]) * m * m) * kd2, m, kd, dipvol);
			break;
		case ADDA_POL_SO: /* orientation-averaged S = 1/3 (calculator.c:197) */
			r[0] = pol_rr((SO_B1 + (SO_B2 + SO_B3 / 3) * m * m) * kd2, m, kd, dipvol);
			break;
		default: return ADDA_GB300_EINVAL;
	}
	if (relation != ADDA_POL_CLDR) r[1] = r[2] = r[0];
	for (int a = 0; a < 3; a++) {
		cc[2 * a] = creal(r[a]);
		cc[2 * a + 1] = cimag(r[a]);
	}
	return ADDA_GB300_OK;
}

/* ellTheta(a) = a^3 (theta_3(0, exp(-pi a^2))^3 - 1) (calculator.c:137-166): the lattice sum of a normalised Gaussian
 * over the cubic lattice minus its value at 0, scaled. theta_3(0, q) = 1 + 2 sum_k q^(k^2); for a >= 1 three terms
 * reach double precision, for a < 1 the Jacobi identity theta_3(0, exp(-pi a^2)) = theta_3(0, exp(-pi/a^2))/a is
 * used first */
static double ell_theta(double a)
{
	const double a2 = a * a, a3 = a * a2;
	if (a >= 1) {
		const double q = exp(-M_PI * a2);
		const double t = 2 * (q + pow(q, 4) + pow(q, 9)); /* theta_3 - 1 */
		return a3 * t * (3 + t * (3 + t));                 /* a^3 ((1+t)^3 - 1) */
	}
	const double q = exp(-M_PI / a2);
	const double th = 1 + 2 * (q + pow(q, 4) + pow(q, 9)); /* a theta_3(0, exp(-pi a^2)) */
	return th * th * th - a3;
}

int adda_gb300_polarizability_nloc(int relation, double m_re, double m_im, double gridspace, double rp, double cc[6])
{
	if ((relation != ADDA_POL_NLOC && relation != ADDA_POL_NLOC_AV) || !(rp >= 0) || !(gridspace > 0))
		return ADDA_GB300_EINVAL;
	const double dipvol = gridspace * gridspace * gridspace;
	const double complex m = m_re + I * m_im;
	double complex r;
	if (rp == 0) r = pol_cm(m, dipvol);
	else if (relation == ADDA_POL_NLOC) r = pol_m(FOUR_PI_D / 3 * ell_theta(gridspace / (sqrt(2 * M_PI) * rp)), m, dipvol);
	else {
		/* 1 - erf(x)^3, through erfc for x >= 1 to keep the digits */
		const double x = gridspace / (2 * M_SQRT2 * rp);
		double g0;
		if (x < 1) {
			const double t = erf(x);
			g0 = 1 - t * t * t;
		}
		else {
			const double t = erfc(x);
			g0 = t * (3 - 3 * t + t * t);
		}
		r = pol_m(FOUR_PI_D / 3 * g0, m, dipvol);
	}
	for (int a = 0; a < 3; a++) {
		cc[2 * a] = creal(r);
		cc[2 * a + 1] = cimag(r);
	}
	return ADDA_GB300_OK;
}

int adda_gb300_polarizability_dchi(int relation, double m_re, double m_im, double kd, double gridspace,
	const double prop[3], const double incPol[3], int avgpol, double out[2])
{
	/* 1/alpha = 1/alpha_CM - M/d^3 with 1/alpha_CM = 4pi/(3d^3) + 1/(d^3 chi), chi = (m^2-1)/(4pi), and for LDR
	 * M = (b1 + (b2 + b3 S) m^2) kd^2 + 2i kd^3/3 (calculator.c:100-132, 214-222); CM, RRC and DGF have M independent
	 * of m, so d(1/alpha)/dchi = -1/(d^3 chi^2) - 4pi (b2 + b3 S) kd^2/d^3 [LDR only] */
	const double dipvol = gridspace * gridspace * gridspace;
	const double complex m = m_re + I * m_im;
	const double complex chi = (m * m - 1) / FOUR_PI_D;
	double complex r = -1 / (dipvol * chi * chi);
	switch (relation) {
		case ADDA_POL_CM:
		case ADDA_POL_RRC:
		case ADDA_POL_DGF:
		case ADDA_POL_FCD:
		case ADDA_POL_IGT_SO:
		case ADDA_POL_LAK: break;
		case ADDA_POL_LDR: r -= FOUR_PI_D * (LDR_B2 + LDR_B3 * ldr_s(prop, incPol, avgpol)) * kd * kd / dipvol; break;
		case ADDA_POL_SO: r -= FOUR_PI_D * (SO_B2 + SO_B3 / 3) * kd * kd / dipvol; break;
		default: return ADDA_GB300_EINVAL; /* CLDR is anisotropic: no scalar derivative */
	}
	out[0] = creal(r);
	out[1] = cimag(r);
	return ADDA_GB300_OK;
}

int adda_gb300_wkb_field(int boxX, int boxY, int boxZ, size_t ndip, const uint16_t *position, const uint8_t *material,
	int nmat, const double *ref_index, double kd, const double *einc, double *field)
{
	if (boxX < 1 || boxY < 1 || boxZ < 1 || nmat < 1 || nmat > 255 || !position || !ref_index || !einc || !field)
		return ADDA_GB300_EINVAL;
	const size_t plane = (size_t)boxX * boxY, cells = plane * boxZ;
	unsigned char *mg = malloc(cells);
	double complex *arg = malloc(sizeof(double complex) * cells);
	double complex *top = malloc(sizeof(double complex) * plane);
	double complex vals[256];
	if (!mg || !arg || !top) {
		free(mg); free(arg); free(top);
		return ADDA_GB300_ENOMEM;
	}
	for (int i = 0; i < nmat; i++) vals[i] = I * (ref_index[2 * i] - 1 + I * ref_index[2 * i + 1]) * kd / 2;
	vals[nmat] = 0;
	memset(mg, nmat, cells);
	for (size_t d = 0; d < ndip; d++) {
		const size_t cell = ((size_t)position[3 * d + 2] * boxY + position[3 * d + 1]) * boxX + position[3 * d];
		mg[cell] = material ? material[d] : 0;
	}
	for (size_t i = 0; i < plane; i++) top[i] = 0;
	/* arg(z) = arg(z-1) + v(z-1) + v(z): half a cell of phase on each side of every cell boundary */
	for (int z = 0; z < boxZ; z++)
		for (size_t i = 0; i < plane; i++) {
			const size_t cell = (size_t)z * plane + i;
			arg[cell] = top[i] + vals[mg[cell]];
			top[i] = arg[cell] + vals[mg[cell]];
		}
	for (size_t d = 0; d < ndip; d++) {
		const size_t cell = ((size_t)position[3 * d + 2] * boxY + position[3 * d + 1]) * boxX + position[3 * d];
		const double complex f = cexp(arg[cell]);
		for (int a = 0; a < 3; a++) {
			const double complex e = (einc[6 * d + 2 * a] + I * einc[6 * d + 2 * a + 1]) * f;
			field[6 * d + 2 * a] = creal(e);
			field[6 * d + 2 * a + 1] = cimag(e);
		}
	}
	free(mg);
	free(arg);
	free(top);
	return ADDA_GB300_OK;
}

int adda_gb300_fft_fit(int x, int divis)
{
	if (x < 1 || divis < 1) return ADDA_GB300_EINVAL;
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

/* the integral tables of -int igt_so / so: files t1f.dat .. t10f.dat of dir, each TAB_SIZE = 142 entries times 1, 6,
 * 3, 18, 6, 36, 1, 6, 1, 6 values (src/const.h:274-277), read as whitespace-separated doubles like ReadTableFile;
 * extra values after the expected count are ignored */
int adda_gb300_read_int_tables(const char *dir, double *tables)
{
	static const int mult[10] = {1, 6, 3, 18, 6, 36, 1, 6, 1, 6};
	if (!dir || !tables) return ADDA_GB300_EINVAL;
	size_t off = 0;
	for (int t = 0; t < 10; t++) {
		char fname[4096];
		if (snprintf(fname, sizeof(fname), "%s/t%df.dat", dir, t + 1) >= (int)sizeof(fname)) return ADDA_GB300_EINVAL;
		FILE *f = fopen(fname, "r");
		if (!f) return ADDA_GB300_EINVAL;
		const int n = 142 * mult[t];
		for (int i = 0; i < n; i++)
			if (fscanf(f, "%lf", tables + off + i) != 1) {
				fclose(f);
				return ADDA_GB300_EINVAL;
			}
		fclose(f);
		off += (size_t)n;
	}
	return off == ADDA_GB300_INT_TABLES ? ADDA_GB300_OK : ADDA_GB300_EINVAL;
}
