/* mock_crosssec.c - stand-in for the reference's crosssec.c in the drop-in test: its CPU CalcField must never be
 * reached, because the drop-in wraps CalcField (-Wl,--wrap=CalcField) and serves it on the GPU. */
#include <stdio.h>
#include <stdlib.h>

#include "adda_dropin.h"

void CalcField(doublecomplex ebuff[3], const double n[3])
{
	(void)ebuff;
	(void)n;
	fprintf(stderr, "mock host: the CPU CalcField was called\n");
	exit(3);
}
