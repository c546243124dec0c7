/* fftw_alloc.c - the two FFTW allocation helpers the reference's memory.c calls (memory.c:65,270). The GPU build
 * performs no host FFT, so aligned malloc/free stand in for them. */
#include <stdlib.h>

void *fftw_malloc(size_t n)
{
	void *p = NULL;
	return posix_memalign(&p, 64, n ? n : 1) ? NULL : p;
}

void fftw_free(void *p) { free(p); }
