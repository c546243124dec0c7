/* integrate.c - integrals over the scattering directions on the host: the angle grids of the reference's
 * alldir_params.dat (ScanIntegrParms, src/crosssec.c:233-307) and the two-level Romberg integration (Romberg2D,
 * src/Romberg.c:175-533) used for Csca and the asymmetry vector (ScaCross, AsymParm_x/y/z, crosssec.c:1116-1260).
 *
 * The Romberg scheme is the "bracketing" form of Davis & Rabinowitz, Methods of Numerical Integration (1975), 6.3: at
 * level m the trapezoid value T and the midpoint value M on 2^m intervals are both extrapolated by Richardson's
 * rule, M_k <- (4^j M_(k+1) - M_k)/(4^j - 1), and the result is their mean, the error half their difference. A periodic
 * variable uses the plain trapezoid rule (Davis & Rabinowitz 2.9). Values are precalculated on the full grid (the
 * directions' fields come from the GPU in one batch); with eps > 0 the integration stops as soon as the error estimate
 * allows, so some values are not used. Results are averages over the grid (the caller scales them).
 */
#include "adda_gb300.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define MAXJ 30
#define DEG2RAD 0.017453292519943295769236907684886 /* pi/180 */
#define RAD2DEG 57.295779513082320876798154814105   /* 180/pi */

int adda_gb300_integr_points(const adda_gb300_integr_parms *p, int in_cos, double *val)
{
	if (!p) return -1;
	if (p->min == p->max) {
		if (val) val[0] = p->min;
		return 1;
	}
	if (p->min > p->max || p->Jmax < p->Jmin || p->Jmin < 1 || p->eps < 0 || p->Jmax >= MAXJ) return -1;
	if (in_cos && (p->min < 0 || p->max > 180)) return -1;
	const int G = (1 << p->Jmax) + 1;
	const int n = p->equiv ? G - 1 : G;
	if (val) {
		if (in_cos) { /* equal steps in cos(angle), from cos(max) up to cos(min) */
			double lo = cos(DEG2RAD * p->max), hi = cos(DEG2RAD * p->min);
			if (fabs(lo) < 1e-15) lo = 0;
			if (fabs(hi) < 1e-15) hi = 0;
			const double unit = (hi - lo) / (G - 1);
			for (int i = 0; i < n; i++) val[i] = RAD2DEG * acos(lo + unit * i);
		}
		else {
			const double unit = (p->max - p->min) / (G - 1);
			for (int i = 0; i < n; i++) val[i] = p->min + unit * i;
		}
	}
	return n;
}

/* one Romberg level structure over a variable with G = 2^Jmax + 1 grid points (or 1); get(i) yields the dim values
 * at point i and an absolute error estimate of them (0 for plain values, the inner integral's error in the outer
 * variable). Returns the result's absolute error; *rel gets the relative one. */
typedef double (*get_fn)(void *ctx, int i, double *out);

typedef struct {
	double t1[MAXJ], t2[MAXJ], t3[MAXJ]; /* 4^i, 1/(4^i - 1), 2*4^i - 1 */
} coefs;

static void set_coefs(coefs *c, int J)
{
	c->t1[0] = 1;
	c->t2[0] = 0;
	for (int i = 1; i < J; i++) {
		c->t1[i] = c->t1[i - 1] * 4;
		c->t2[i] = 1 / (c->t1[i] - 1);
		c->t3[i - 1] = 2 * c->t1[i - 1] - 1;
	}
}

static double romberg_1d(const adda_gb300_integr_parms *p, int G, const coefs *cf, int dim, get_fn get, void *ctx,
	double *res, double *rel)
{
	double *T = calloc((size_t)dim * (MAXJ + 3), sizeof(double));
	double *M = T + dim;                    /* M[k][comp], k <= Jmax */
	double *tmp = M + (size_t)dim * (MAXJ + 1);
	double abs_err = 0, err = 0, int_err = 0;
	if (G == 1) {
		int_err = get(ctx, 0, res);
		*rel = (res[0] == 0) ? 0 : int_err / fabs(res[0]);
		free(T);
		return int_err;
	}
	int m0 = 0;
	for (int m = 0; m < p->Jmax; m++) {
		if (m == 0) { /* trapezoid on one interval */
			int_err = get(ctx, 0, T);
			if (!p->equiv) {
				int_err = 0.5 * (int_err + get(ctx, G - 1, tmp));
				for (int c = 0; c < dim; c++) T[c] = 0.5 * (tmp[c] + T[c]);
			}
		}
		else if (p->periodic) for (int c = 0; c < dim; c++) T[c] = 0.5 * (T[c] + M[c]);
		else {
			for (int c = 0; c < dim; c++) T[c] = cf->t3[m - 1] * cf->t2[m] * (T[c] - M[c]) + M[c];
			m0 = m;
		}
		/* midpoint sum on 2^m intervals */
		const int step = (G - 1) >> m;
		double *Mm = M + (size_t)m0 * dim, e = 0;
		for (int c = 0; c < dim; c++) Mm[c] = 0;
		for (int j = step >> 1; j < G; j += step) {
			e += get(ctx, j, tmp);
			for (int c = 0; c < dim; c++) Mm[c] += tmp[c];
		}
		const double sc = pow(2, -m);
		for (int c = 0; c < dim; c++) Mm[c] *= sc;
		int_err = 0.5 * (int_err + e * sc);
		/* Richardson extrapolation of the midpoint column */
		if (m0 != 0)
			for (int k = m - 1; k >= 0; k--)
				for (int c = 0; c < dim; c++)
					M[k * dim + c] = cf->t2[m - k] * (cf->t1[m - k] * M[(k + 1) * dim + c] - M[k * dim + c]);
		if (m >= p->Jmin - 1) {
			const double abs_res = 0.5 * fabs(M[0] + T[0]);
			abs_err = 0.5 * fabs(M[0] - T[0]) + int_err;
			err = (abs_res == 0) ? 0 : abs_err / abs_res;
			if (err < p->eps) break;
		}
	}
	for (int c = 0; c < dim; c++) res[c] = 0.5 * (M[c] + T[c]);
	*rel = err;
	free(T);
	return abs_err;
}

typedef struct {
	const adda_gb300_integr_parms *p;
	int Gt, Gp, nphi, dim;
	const double *values;
	const coefs *cf;
	int theta;              /* row of the inner integration */
	int pole_lo, pole_hi;   /* the first / last outer point is a pole: its inner integral is its first value */
} r2d;

static double get_value(void *ctx, int j, double *out)
{
	r2d *s = ctx;
	/* the last phi point of an "equivalent" range is the first one */
	const int jj = (j >= s->nphi) ? j - s->nphi : j;
	memcpy(out, s->values + ((size_t)s->theta * s->nphi + jj) * s->dim, sizeof(double) * s->dim);
	return 0;
}

static double get_inner(void *ctx, int i, double *out)
{
	r2d *s = ctx;
	s->theta = i;
	double rel;
	if ((i == 0 && s->pole_lo) || (i == s->Gt - 1 && s->pole_hi)) return get_value(s, 0, out); /* onepoint */
	return romberg_1d(&s->p[1], s->Gp, s->cf, s->dim, get_value, s, out, &rel);
}

double adda_gb300_romberg2d(const adda_gb300_integr_parms p[2], int dim, const double *values, double *res)
{
	return adda_gb300_romberg2d_ex(p, dim, values, res, 0);
}

double adda_gb300_romberg2d_ex(const adda_gb300_integr_parms p[2], int dim, const double *values, double *res,
	int poles)
{
	const int nth = adda_gb300_integr_points(&p[0], 1, NULL), nph = adda_gb300_integr_points(&p[1], 0, NULL);
	if (nth < 1 || nph < 1 || dim < 1 || !values || !res) return -1;
	coefs cf;
	const int Jt = (p[0].min == p[0].max) ? 1 : p[0].Jmax, Jp = (p[1].min == p[1].max) ? 1 : p[1].Jmax;
	set_coefs(&cf, (Jt > Jp ? Jt : Jp) + 1);
	r2d s = {p, (p[0].min == p[0].max) ? 1 : (1 << p[0].Jmax) + 1, (p[1].min == p[1].max) ? 1 : (1 << p[1].Jmax) + 1,
		nph, dim, values, &cf, 0, 0, 0};
	/* the outer grid starts at cos(max) and ends at cos(min): a pole where that angle is 180 or 0 degrees */
	s.pole_lo = poles && p[0].max == 180 && p[0].min != p[0].max;
	s.pole_hi = poles && p[0].min == 0 && p[0].min != p[0].max;
	adda_gb300_integr_parms outer = p[0], inner = p[1];
	if (p[0].min == p[0].max) outer.Jmax = 1;
	if (p[1].min == p[1].max) inner.Jmax = 1;
	adda_gb300_integr_parms pp[2] = {outer, inner};
	s.p = pp;
	double rel;
	romberg_1d(&pp[0], s.Gt, &cf, dim, get_inner, &s, res, &rel);
	return rel;
}
