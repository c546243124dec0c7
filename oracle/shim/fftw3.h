/* fftw3.h - minimal FFTW3 API subset for linking the reference's sequential ADDA build without FFTW.
 *
 * TEST INFRASTRUCTURE (oracle). Only the seven entry points and the types the reference uses are declared
 * (fft.c:566-604, fft.c:739-815, memory.c:65,270). The names and argument meanings must match FFTW3's public API
 * because the unmodified reference sources call them; the implementation (fftw_shim.c) is this project's own FFT.
 */
#ifndef ADDA_ORACLE_FFTW3_SHIM_H
#define ADDA_ORACLE_FFTW3_SHIM_H

#include <stddef.h>
#include <complex.h>

typedef double _Complex fftw_complex;
typedef struct fftw_plan_s *fftw_plan;
typedef struct { int n, is, os; } fftw_iodim;

#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_MEASURE (0U)
#define FFTW_ESTIMATE (1U << 6)

extern const char fftw_version[], fftw_cc[], fftw_codelet_optim[];

fftw_plan fftw_plan_many_dft(int rank, const int *n, int howmany, fftw_complex *in, const int *inembed, int istride,
	int idist, fftw_complex *out, const int *onembed, int ostride, int odist, int sign, unsigned flags);
fftw_plan fftw_plan_guru_dft(int rank, const fftw_iodim *dims, int howmany_rank, const fftw_iodim *howmany_dims,
	fftw_complex *in, fftw_complex *out, int sign, unsigned flags);
void fftw_execute(const fftw_plan p);
void fftw_destroy_plan(fftw_plan p);
void fftw_cleanup(void);
void *fftw_malloc(size_t n);
void fftw_free(void *p);

#endif
