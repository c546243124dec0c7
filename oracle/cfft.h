/* cfft.h - mixed-radix complex FFT on the CPU, double precision.
 *
 * TEST INFRASTRUCTURE (oracle): this FFT backs the CPU restatement of the ADDA hot path (adda_oracle.c) and the
 * FFTW-subset shim (fftw_shim.c) that lets the reference's sequential build link without FFTW. It is never part of
 * the shipped GPU product.
 *
 * Semantics follow FFTW's unnormalised DFT, which is what the reference calls (fft.c:574-604, 750-787):
 *   out[k] = sum_j in[j] * exp(sign * 2*pi*i * j*k / n),  sign = -1 (forward) or +1 (backward).
 * Algorithm: self-sorting Stockham passes over the prime factorisation of n (radices 4,2,3,5 hand-written, any other
 * prime through a generic O(p^2) butterfly), twiddles from one table of n-th roots of unity.
 */
#ifndef ADDA_ORACLE_CFFT_H
#define ADDA_ORACLE_CFFT_H

#include <complex.h>
#include <stddef.h>

#define CFFT_MAXF 64

typedef struct {
	int n;
	int nf;                 // number of passes
	int fac[CFFT_MAXF];     // radix of each pass
	double complex *tw;     // tw[t] = exp(-2*pi*i*t/n), t=0..n-1
} cfft_plan;

int cfft_plan_init(cfft_plan *p, int n);   // returns 0 on success
void cfft_plan_free(cfft_plan *p);
/* transform one contiguous line in place; work must hold n elements */
void cfft_exec(const cfft_plan *p, double complex *data, double complex *work, int sign);
/* transform 'howmany' lines of a strided layout: element j of line l is at data[l*dist + j*stride] */
void cfft_exec_strided(const cfft_plan *p, double complex *data, ptrdiff_t stride, ptrdiff_t dist, size_t howmany,
	int sign);

#endif
