/* fftw_shim.c - the FFTW3 subset declared in shim/fftw3.h, implemented on top of this project's cfft.c.
 *
 * TEST INFRASTRUCTURE (oracle): linked only into the reference's sequential build under oracle/_ref/, so that the
 * unmodified reference can run here as a pinned CPU oracle and CPU baseline. Supports what the reference plans:
 * rank-1 in-place transforms with one (plan_many, fft.c:574-577,751-757) or two (plan_guru, fft.c:761-787) batch
 * dimensions.
 */
#include "shim/fftw3.h"
#include "cfft.h"

#include <stdio.h>
#include <stdlib.h>

const char fftw_version[] = "oracle-shim", fftw_cc[] = "gcc", fftw_codelet_optim[] = "";

struct fftw_plan_s {
	cfft_plan p;
	double complex *data;
	int stride;        // element stride
	int nb;            // number of batch dims (1 or 2)
	int bn[2], bs[2];  // batch counts and strides
	int sign;
};

static void die(const char *msg)
{
	fprintf(stderr, "fftw shim: %s\n", msg);
	exit(1);
}

fftw_plan fftw_plan_many_dft(int rank, const int *n, int howmany, fftw_complex *in, const int *inembed, int istride,
	int idist, fftw_complex *out, const int *onembed, int ostride, int odist, int sign, unsigned flags)
{
	(void)inembed; (void)onembed; (void)flags;
	if (rank != 1 || in != out || istride != ostride || idist != odist) die("unsupported plan_many_dft");
	struct fftw_plan_s *pl = calloc(1, sizeof(*pl));
	if (cfft_plan_init(&pl->p, n[0])) die("bad size");
	pl->data = in;
	pl->stride = istride;
	pl->nb = 1;
	pl->bn[0] = howmany;
	pl->bs[0] = idist;
	pl->sign = sign;
	return pl;
}

fftw_plan fftw_plan_guru_dft(int rank, const fftw_iodim *dims, int howmany_rank, const fftw_iodim *howmany_dims,
	fftw_complex *in, fftw_complex *out, int sign, unsigned flags)
{
	(void)flags;
	if (rank != 1 || in != out || howmany_rank < 1 || howmany_rank > 2 || dims[0].is != dims[0].os)
		die("unsupported plan_guru_dft");
	struct fftw_plan_s *pl = calloc(1, sizeof(*pl));
	if (cfft_plan_init(&pl->p, dims[0].n)) die("bad size");
	pl->data = in;
	pl->stride = dims[0].is;
	pl->nb = howmany_rank;
	for (int i = 0; i < howmany_rank; i++) {
		if (howmany_dims[i].is != howmany_dims[i].os) die("unsupported guru strides");
		pl->bn[i] = howmany_dims[i].n;
		pl->bs[i] = howmany_dims[i].is;
	}
	pl->sign = sign;
	return pl;
}

void fftw_execute(const fftw_plan pl)
{
	if (pl->nb == 1) cfft_exec_strided(&pl->p, pl->data, pl->stride, pl->bs[0], (size_t)pl->bn[0], pl->sign);
	else for (int i = 0; i < pl->bn[0]; i++)
		cfft_exec_strided(&pl->p, pl->data + (ptrdiff_t)i * pl->bs[0], pl->stride, pl->bs[1], (size_t)pl->bn[1],
			pl->sign);
}

void fftw_destroy_plan(fftw_plan pl)
{
	if (!pl) return;
	cfft_plan_free(&pl->p);
	free(pl);
}

void fftw_cleanup(void) {}

void *fftw_malloc(size_t n)
{
	void *p = NULL;
	if (posix_memalign(&p, 64, n ? n : 1)) return NULL;
	return p;
}

void fftw_free(void *p) { free(p); }
