/* fftw3.h - the part of FFTW3's header that the reference's memory.c needs when it is compiled into the drop-in
 * build (memory.c:30,65,270: fftw_malloc/fftw_free for its aligned vectors). The drop-in performs no host FFT;
 * fftw_alloc.c defines the two helpers. Only the names and signatures follow FFTW3's public API. */
#ifndef ADDA_DROPIN_FFTW3_H
#define ADDA_DROPIN_FFTW3_H

#include <stddef.h>

void *fftw_malloc(size_t n);
void fftw_free(void *p);

#endif
