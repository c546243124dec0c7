/* mock_crosssec.c - stand-in for the reference's crosssec.c in the drop-in test: its CPU CalcField and CalcAlldir
 * must never be reached, because the drop-in wraps them (-Wl,--wrap=CalcField,--wrap=CalcAlldir) and serves them on
 * the GPU. SetScatPlane follows the reference's beam-frame definition (crosssec.c:944-990, no surface). */
#include <math.h>
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

void CalcScatGrid(enum incpol which)
{
	(void)which;
	fprintf(stderr, "mock host: the CPU CalcScatGrid was called\n");
	exit(3);
}

void CalcAlldir(void)
{
	fprintf(stderr, "mock host: the CPU CalcAlldir was called\n");
	exit(3);
}

extern double prop[3], incPolX[3], incPolY[3];

void SetScatPlane(const double ct, const double st, const double phi, double robs[3], double polPer[3])
{
	const double cphi = cos(phi), sphi = sin(phi);
	for (int a = 0; a < 3; a++) robs[a] = ct * prop[a] + st * (cphi * incPolX[a] + sphi * incPolY[a]);
	if (fabs(st) < 1e-15)
		for (int a = 0; a < 3; a++) polPer[a] = sphi * incPolX[a] - cphi * incPolY[a];
	else {
		polPer[0] = robs[1] * prop[2] - robs[2] * prop[1];
		polPer[1] = robs[2] * prop[0] - robs[0] * prop[2];
		polPer[2] = robs[0] * prop[1] - robs[1] * prop[0];
		const double nn = sqrt(polPer[0] * polPer[0] + polPer[1] * polPer[1] + polPer[2] * polPer[2]);
		for (int a = 0; a < 3; a++) polPer[a] /= nn;
	}
}
