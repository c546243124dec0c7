/* cfft.c - mixed-radix Stockham FFT (double complex) for the oracle; see cfft.h.
 *
 * TEST INFRASTRUCTURE (oracle) only.
 */
#include "cfft.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* exp(-2*pi*i*t/n) with octant reduction so that sin/cos only see arguments in [0, pi/4] */
static double complex unit_root(long t, long n)
{
	t %= n;
	if (t < 0) t += n;
	/* angle = 2*pi*t/n; work with 8*t relative to n to find the octant */
	long e = 8 * t;
	int oct = (int)(e / n);
	double c, s;
	/* residual angle within the octant, in radians */
	double frac = (double)(e - (long)oct * n) / (double)n; // in [0,1)
	double a = frac * (M_PI / 4);
	double ca = cos(a), sa = sin(a), cb = cos(M_PI / 4 - a), sb = sin(M_PI / 4 - a);
	switch (oct) {
		case 0: c = ca; s = sa; break;
		case 1: c = sb; s = cb; break;
		case 2: c = -sa; s = ca; break;
		case 3: c = -cb; s = sb; break;
		case 4: c = -ca; s = -sa; break;
		case 5: c = -sb; s = -cb; break;
		case 6: c = sa; s = -ca; break;
		default: c = cb; s = -sb; break;
	}
	return c - I * s; // exp(-i*angle)
}

int cfft_plan_init(cfft_plan *p, int n)
{
	memset(p, 0, sizeof(*p));
	if (n < 1) return -1;
	p->n = n;
	int m = n;
	/* radix-4 first (fewest passes), then the remaining primes in increasing order */
	while (m % 4 == 0) { p->fac[p->nf++] = 4; m /= 4; }
	while (m % 2 == 0) { p->fac[p->nf++] = 2; m /= 2; }
	for (int q = 3; m > 1; q += 2) {
		while (m % q == 0) {
			if (p->nf >= CFFT_MAXF || q > 61) return -1; // generic butterfly holds at most 64 points
			p->fac[p->nf++] = q;
			m /= q;
		}
	}
	p->tw = malloc(sizeof(double complex) * (size_t)n);
	if (!p->tw) return -1;
	for (int t = 0; t < n; t++) p->tw[t] = unit_root(t, n);
	return 0;
}

void cfft_plan_free(cfft_plan *p)
{
	free(p->tw);
	p->tw = NULL;
}

/* one Stockham pass: radix r, span m (product of earlier radices); x -> y */
static void pass(const cfft_plan *p, int r, int m, const double complex *x, double complex *y, int sign)
{
	const int n = p->n;
	const int nr = n / r;
	const int tstep = n / (m * r); // twiddle stride in the n-th root table
	double complex a[64];
	double complex wr[64];
	if (r > 4) { // roots of unity for the generic butterfly
		for (int q = 0; q < r; q++) {
			double complex w = p->tw[(long)q * nr % n];
			wr[q] = (sign < 0) ? w : conj(w);
		}
	}
	for (int j = 0; j < nr; j++) {
		const int k = j % m;
		for (int q = 0; q < r; q++) {
			double complex v = x[j + q * nr];
			if (q && k) {
				double complex w = p->tw[(long)q * k * tstep % n];
				v *= (sign < 0) ? w : conj(w);
			}
			a[q] = v;
		}
		double complex *out = y + (j / m) * m * r + k;
		switch (r) {
			case 2:
				out[0] = a[0] + a[1];
				out[m] = a[0] - a[1];
				break;
			case 4: {
				double complex t0 = a[0] + a[2], t1 = a[0] - a[2];
				double complex t2 = a[1] + a[3], t3 = a[1] - a[3];
				// multiply t3 by -i*sign... forward (sign=-1): exp(-i pi/2) = -i
				double complex t3r = (sign < 0) ? -I * t3 : I * t3;
				out[0] = t0 + t2;
				out[m] = t1 + t3r;
				out[2 * m] = t0 - t2;
				out[3 * m] = t1 - t3r;
				break;
			}
			case 3: {
				const double c = -0.5, s = (sign < 0 ? -1.0 : 1.0) * 0.86602540378443864676;
				double complex t1 = a[1] + a[2], t2 = a[1] - a[2];
				double complex m1 = a[0] + c * t1;
				double complex m2 = I * s * t2;
				out[0] = a[0] + t1;
				out[m] = m1 + m2;
				out[2 * m] = m1 - m2;
				break;
			}
			default: // generic prime radix
				for (int q = 0; q < r; q++) {
					double complex sacc = 0;
					for (int qq = 0; qq < r; qq++) sacc += a[qq] * wr[(q * qq) % r];
					out[q * m] = sacc;
				}
				break;
		}
	}
}

void cfft_exec(const cfft_plan *p, double complex *data, double complex *work, int sign)
{
	double complex *x = data, *y = work;
	int m = 1;
	for (int f = 0; f < p->nf; f++) {
		pass(p, p->fac[f], m, x, y, sign);
		m *= p->fac[f];
		double complex *t = x;
		x = y;
		y = t;
	}
	if (x != data) memcpy(data, x, sizeof(double complex) * (size_t)p->n);
}

void cfft_exec_strided(const cfft_plan *p, double complex *data, ptrdiff_t stride, ptrdiff_t dist, size_t howmany,
	int sign)
{
	const int n = p->n;
	double complex *buf = malloc(sizeof(double complex) * 2 * (size_t)n);
	for (size_t l = 0; l < howmany; l++) {
		double complex *base = data + (ptrdiff_t)l * dist;
		if (stride == 1) cfft_exec(p, base, buf, sign);
		else {
			for (int j = 0; j < n; j++) buf[n + j] = base[j * stride];
			cfft_exec(p, buf + n, buf, sign);
			for (int j = 0; j < n; j++) base[j * stride] = buf[n + j];
		}
	}
	free(buf);
}
